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
