"""ctypes binding of zfp's high-level C API.

The struct layouts and prototypes are those of the reference's public
header (include/zfp.h:60-136 for the types, include/zfp.h:151-613 for the
functions, include/zfp/bitstream.h:27-100 for the bit stream).  Any shared
library exporting that ABI can be bound: libzfp_gb300.so (this package's
GPU codec) or, in the test suite, a reference build.  Each library is
opened with RTLD_LOCAL so two libraries exporting the same zfp_* names can
live in one process.
"""
from __future__ import annotations

import ctypes as C
import os

# zfp_type (include/zfp.h:122-128)
TYPE_NONE, TYPE_INT32, TYPE_INT64, TYPE_FLOAT, TYPE_DOUBLE = 0, 1, 2, 3, 4
# zfp_exec_policy (include/zfp.h:68-72)
EXEC_SERIAL, EXEC_OMP, EXEC_CUDA = 0, 1, 2
# zfp_mode (include/zfp.h:96-103)
MODE_NULL, MODE_EXPERT, MODE_FIXED_RATE, MODE_FIXED_PRECISION, MODE_FIXED_ACCURACY, MODE_REVERSIBLE = range(6)
# header masks (include/zfp.h:24-28)
HEADER_NONE, HEADER_MAGIC, HEADER_META, HEADER_MODE, HEADER_FULL = 0, 1, 2, 4, 7

MIN_BITS, MAX_BITS, MAX_PREC, MIN_EXP = 1, 16658, 64, -1074


class zfp_execution(C.Structure):
    _fields_ = [("policy", C.c_int), ("params", C.c_void_p)]


class zfp_stream(C.Structure):
    _fields_ = [
        ("minbits", C.c_uint),
        ("maxbits", C.c_uint),
        ("maxprec", C.c_uint),
        ("minexp", C.c_int),
        ("stream", C.c_void_p),
        ("exec", zfp_execution),
    ]


class zfp_field(C.Structure):
    _fields_ = [
        ("type", C.c_int),
        ("nx", C.c_size_t), ("ny", C.c_size_t), ("nz", C.c_size_t), ("nw", C.c_size_t),
        ("sx", C.c_ssize_t), ("sy", C.c_ssize_t), ("sz", C.c_ssize_t), ("sw", C.c_ssize_t),
        ("data", C.c_void_p),
    ]


PZ = C.POINTER(zfp_stream)
PF = C.POINTER(zfp_field)

# (name, restype, argtypes)
_PROTOS = [
    ("stream_open", C.c_void_p, [C.c_void_p, C.c_size_t]),
    ("stream_close", None, [C.c_void_p]),
    ("stream_rewind", None, [C.c_void_p]),
    ("stream_size", C.c_size_t, [C.c_void_p]),
    ("stream_capacity", C.c_size_t, [C.c_void_p]),
    ("stream_data", C.c_void_p, [C.c_void_p]),
    ("stream_wtell", C.c_uint64, [C.c_void_p]),
    ("stream_rtell", C.c_uint64, [C.c_void_p]),
    ("stream_wseek", None, [C.c_void_p, C.c_uint64]),
    ("stream_rseek", None, [C.c_void_p, C.c_uint64]),
    ("stream_write_bits", C.c_uint64, [C.c_void_p, C.c_uint64, C.c_size_t]),
    ("stream_read_bits", C.c_uint64, [C.c_void_p, C.c_size_t]),
    ("stream_write_bit", C.c_uint, [C.c_void_p, C.c_uint]),
    ("stream_read_bit", C.c_uint, [C.c_void_p]),
    ("stream_pad", None, [C.c_void_p, C.c_uint64]),
    ("stream_skip", None, [C.c_void_p, C.c_uint64]),
    ("stream_flush", C.c_size_t, [C.c_void_p]),
    ("stream_align", C.c_size_t, [C.c_void_p]),
    ("stream_copy", None, [C.c_void_p, C.c_void_p, C.c_uint64]),
    ("zfp_type_size", C.c_size_t, [C.c_int]),
    ("zfp_stream_open", PZ, [C.c_void_p]),
    ("zfp_stream_close", None, [PZ]),
    ("zfp_stream_bit_stream", C.c_void_p, [PZ]),
    ("zfp_stream_set_bit_stream", None, [PZ, C.c_void_p]),
    ("zfp_stream_compression_mode", C.c_int, [PZ]),
    ("zfp_stream_mode", C.c_uint64, [PZ]),
    ("zfp_stream_params", None, [PZ, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_int)]),
    ("zfp_stream_compressed_size", C.c_size_t, [PZ]),
    ("zfp_stream_maximum_size", C.c_size_t, [PZ, PF]),
    ("zfp_stream_rewind", None, [PZ]),
    ("zfp_stream_set_reversible", None, [PZ]),
    ("zfp_stream_set_rate", C.c_double, [PZ, C.c_double, C.c_int, C.c_uint, C.c_int]),
    ("zfp_stream_set_precision", C.c_uint, [PZ, C.c_uint]),
    ("zfp_stream_set_accuracy", C.c_double, [PZ, C.c_double]),
    ("zfp_stream_set_mode", C.c_int, [PZ, C.c_uint64]),
    ("zfp_stream_set_params", C.c_int, [PZ, C.c_uint, C.c_uint, C.c_uint, C.c_int]),
    ("zfp_stream_execution", C.c_int, [PZ]),
    ("zfp_stream_set_execution", C.c_int, [PZ, C.c_int]),
    ("zfp_stream_set_omp_threads", C.c_int, [PZ, C.c_uint]),
    ("zfp_stream_rate", C.c_double, [PZ, C.c_uint]),
    ("zfp_stream_precision", C.c_uint, [PZ]),
    ("zfp_stream_accuracy", C.c_double, [PZ]),
    ("zfp_stream_flush", C.c_size_t, [PZ]),
    ("zfp_stream_align", C.c_size_t, [PZ]),
    ("zfp_field_alloc", PF, []),
    ("zfp_field_1d", PF, [C.c_void_p, C.c_int, C.c_size_t]),
    ("zfp_field_2d", PF, [C.c_void_p, C.c_int, C.c_size_t, C.c_size_t]),
    ("zfp_field_3d", PF, [C.c_void_p, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t]),
    ("zfp_field_4d", PF, [C.c_void_p, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t]),
    ("zfp_field_free", None, [PF]),
    ("zfp_field_pointer", C.c_void_p, [PF]),
    ("zfp_field_begin", C.c_void_p, [PF]),
    ("zfp_field_type", C.c_int, [PF]),
    ("zfp_field_precision", C.c_uint, [PF]),
    ("zfp_field_dimensionality", C.c_uint, [PF]),
    ("zfp_field_size", C.c_size_t, [PF, C.POINTER(C.c_size_t)]),
    ("zfp_field_size_bytes", C.c_size_t, [PF]),
    ("zfp_field_blocks", C.c_size_t, [PF]),
    ("zfp_field_stride", C.c_int, [PF, C.POINTER(C.c_ssize_t)]),
    ("zfp_field_is_contiguous", C.c_int, [PF]),
    ("zfp_field_metadata", C.c_uint64, [PF]),
    ("zfp_field_set_pointer", None, [PF, C.c_void_p]),
    ("zfp_field_set_type", C.c_int, [PF, C.c_int]),
    ("zfp_field_set_size_1d", None, [PF, C.c_size_t]),
    ("zfp_field_set_size_2d", None, [PF, C.c_size_t, C.c_size_t]),
    ("zfp_field_set_size_3d", None, [PF, C.c_size_t, C.c_size_t, C.c_size_t]),
    ("zfp_field_set_size_4d", None, [PF, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t]),
    ("zfp_field_set_stride_1d", None, [PF, C.c_ssize_t]),
    ("zfp_field_set_stride_2d", None, [PF, C.c_ssize_t, C.c_ssize_t]),
    ("zfp_field_set_stride_3d", None, [PF, C.c_ssize_t, C.c_ssize_t, C.c_ssize_t]),
    ("zfp_field_set_stride_4d", None, [PF, C.c_ssize_t, C.c_ssize_t, C.c_ssize_t, C.c_ssize_t]),
    ("zfp_field_set_metadata", C.c_int, [PF, C.c_uint64]),
    ("zfp_compress", C.c_size_t, [PZ, PF]),
    ("zfp_decompress", C.c_size_t, [PZ, PF]),
    ("zfp_write_header", C.c_size_t, [PZ, PF, C.c_uint]),
    ("zfp_read_header", C.c_size_t, [PZ, PF, C.c_uint]),
]


class ZfpLib:
    """The zfp C API of one shared library, bound with ctypes."""

    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.path = path
        self.lib = C.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        for name, res, args in _PROTOS:
            fn = getattr(self.lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
            setattr(self, name, fn)

    def has(self, name: str) -> bool:
        return hasattr(self.lib, name)

    def params(self, zfp) -> tuple:
        a, b, c, d = C.c_uint(), C.c_uint(), C.c_uint(), C.c_int()
        self.zfp_stream_params(zfp, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return (a.value, b.value, c.value, d.value)


def field_args(n, s):
    """Normalise extents/strides (fastest axis first) to 4-tuples."""
    n = tuple(int(v) for v in n) + (0,) * (4 - len(n))
    s = tuple(int(v) for v in s) + (0,) * (4 - len(s))
    return n, s


def make_field(lib: ZfpLib, ptr: int, ztype: int, n, s=()):
    """Allocate a zfp_field through `lib` for data at `ptr`."""
    n, s = field_args(n, s)
    dims = sum(1 for v in n if v)
    if dims == 1:
        f = lib.zfp_field_1d(ptr, ztype, n[0])
    elif dims == 2:
        f = lib.zfp_field_2d(ptr, ztype, n[0], n[1])
    elif dims == 3:
        f = lib.zfp_field_3d(ptr, ztype, n[0], n[1], n[2])
    else:
        f = lib.zfp_field_4d(ptr, ztype, n[0], n[1], n[2], n[3])
    if any(s):
        f.contents.sx, f.contents.sy, f.contents.sz, f.contents.sw = s
    return f


def set_mode(lib: ZfpLib, zfp, mode: str, arg=None, ztype: int = TYPE_FLOAT, dims: int = 3):
    """Configure a zfp_stream like the reference's setters (src/zfp.c:751-811)."""
    if mode == "rate":
        return lib.zfp_stream_set_rate(zfp, float(arg), ztype, dims, 0)
    if mode == "precision":
        return lib.zfp_stream_set_precision(zfp, int(arg))
    if mode == "accuracy":
        return lib.zfp_stream_set_accuracy(zfp, float(arg))
    if mode == "reversible":
        lib.zfp_stream_set_reversible(zfp)
        return None
    if mode == "expert":
        return lib.zfp_stream_set_params(zfp, *arg)
    raise ValueError(mode)
