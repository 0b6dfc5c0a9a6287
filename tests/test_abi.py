"""The C-ABI library builds, loads and exports every entry point that
include/diffstir.h declares (no compute calls: this runs without a GPU)."""

import ctypes
import os
import re

from diffstir_gb300 import _abi
from diffstir_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'diffstir.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'^\s*(?:int|void|const char\s*\*)\s*(dstir_\w+)\s*\(', src, flags=re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert 'dstir_create' in syms and 'dstir_backward' in syms and len(syms) >= 15


def test_library_exports_all_declared_symbols():
    lib = ctypes.CDLL(build())
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_python_prototypes_cover_header():
    assert set(declared_symbols()) == set(_abi.PROTOTYPES)


def test_scene_desc_layout_matches_header():
    # 10 int32 + 12 float32
    assert ctypes.sizeof(_abi.DstirSceneDesc) == 10 * 4 + 12 * 4


def test_red_rate_probe_rejects_bad_arguments_before_any_cuda_call():
    lib = _abi.bind(ctypes.CDLL(build()))
    rate = ctypes.c_double(0.0)
    assert lib.dstir_measure_red_rate(16, 8, ctypes.byref(rate), None) == -1
    assert lib.dstir_measure_red_rate(1 << 18, 0, ctypes.byref(rate), None) == -1
    assert lib.dstir_measure_red_rate(1 << 18, 8, None, None) == -1


def test_fp32_rate_probe_rejects_bad_arguments_before_any_cuda_call():
    lib = _abi.bind(ctypes.CDLL(build()))
    rate = ctypes.c_double(0.0)
    assert lib.dstir_measure_fp32_rate(0, ctypes.byref(rate), None) == -1
    assert lib.dstir_measure_fp32_rate(16, None, None) == -1


def _desc(n_grid, n_liquid=1000):
    d = _abi.DstirSceneDesc()
    d.n_grid, d.bound, d.n_liquid = n_grid, 3, n_liquid
    d.model, d.rod_mode, d.j_mode = 2, 1, 0
    d.dt = 2e-4
    return d


def test_static_substep_rejects_huge_grids_before_any_cuda_call():
    # n_grid = 2^21 and 2^22: n_grid^3 overflows 64 bits (2^22 wraps to 0), so
    # the per-axis bound must be checked first; nothing is queued, and the
    # pointers (host dummies here) are never dereferenced
    lib = _abi.bind(ctypes.CDLL(build()))
    dummy = (ctypes.c_float * 32)()
    p = ctypes.cast(dummy, ctypes.c_void_p)
    for n in (1 << 21, 1 << 22, 65):
        d = _desc(n)
        assert lib.dstir_substep_static(ctypes.byref(d), p, p, p, p, p, None) == _abi.DSTIR_ERANGE, n


def test_create_rejects_batches_beyond_32bit_node_keys_before_any_cuda_call():
    # three 1024^3 scenes hold 3 * 2^30 nodes, beyond the 32-bit cell keys of
    # the re-sort; the handle is refused before anything is built or allocated
    lib = _abi.bind(ctypes.CDLL(build()))
    descs = (_abi.DstirSceneDesc * 3)(*[_desc(1024) for _ in range(3)])
    h = ctypes.c_void_p(1)
    assert lib.dstir_create(descs, 3, 10, ctypes.byref(h)) == _abi.DSTIR_ERANGE
    assert not h.value
