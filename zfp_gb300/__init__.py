"""GB300-native zfp block codec.

The product is libzfp_gb300.so (zfp_gb300/csrc, built in-tree by
zfp_gb300/build.py): the reference's zfp.h C API with zfp_compress /
zfp_decompress running hand-written sm_103a CUDA kernels.  This package
only loads it (ctypes) and adds synthetic inputs for tests and benchmarks.
There is no CPU fallback: `load()` raises if the library is not built.
"""
from __future__ import annotations

import ctypes as C
import os

from . import capi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libzfp_gb300.so")

_EXT = [
    ("zfp_gb300_stream_set_cuda_stream", C.c_int, [capi.PZ, C.c_void_p]),
    ("zfp_gb300_stream_set_async", C.c_int, [capi.PZ, C.c_int]),
    ("zfp_gb300_stream_synchronize", C.c_int, [capi.PZ]),
    ("zfp_gb300_last_error", C.c_char_p, []),
    ("zfp_gb300_last_staged_bytes", C.c_size_t, []),
]

_lib = None


def load() -> capi.ZfpLib:
    """The product library, bound with ctypes (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with zfp_gb300.build.build()")
        lib = capi.ZfpLib(LIB_PATH)
        for name, res, args in _EXT:
            fn = getattr(lib.lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
            setattr(lib, name, fn)
        _lib = lib
    return _lib


def last_error() -> str:
    msg = load().zfp_gb300_last_error()
    return msg.decode() if msg else ""
