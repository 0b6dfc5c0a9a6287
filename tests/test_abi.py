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
