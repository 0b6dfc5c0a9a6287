"""Loads libdiffstir.so (the CUDA extension) and binds the C ABI."""

import ctypes
import os

from . import _abi
from .build import LIB, build, up_to_date

_lib = None


class DstirError(RuntimeError):
    """A C-ABI call returned a negative DSTIR_E* code."""

    def __init__(self, code, msg):
        super().__init__('%s: %s' % (_abi.errname(code), msg))
        self.code = code


def lib(auto_build=True):
    """The bound library.  Builds it in-tree when it is missing or stale and
    ``auto_build`` is set; raises if it cannot be loaded (there is no CPU
    fallback)."""
    global _lib
    if _lib is None:
        if not up_to_date():
            if not auto_build:
                raise RuntimeError('libdiffstir.so is missing or stale; run diffstir_gb300.build.build()')
            build()
        _lib = _abi.bind(ctypes.CDLL(LIB))
    return _lib


def lib_path():
    return os.path.abspath(LIB)


def check(rc, handle=None, what=''):
    if rc < 0:
        msg = ''
        if handle is not None:
            msg = lib().dstir_last_error(handle).decode(errors='replace')
        raise DstirError(rc, (what + ': ' if what else '') + msg)
    return rc
