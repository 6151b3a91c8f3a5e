"""zfpy-compatible front end running on the GPU.

The reference's Python binding (python/zfpy.pyx) drives zfp's C API with the
default serial policy; this module makes the same calls on libzfp_gb300.so
with `zfp_stream_set_execution(stream, zfp_exec_cuda)` added, so its bytes
and arrays equal zfpy's.  Same functions, arguments and errors:

    compress_numpy(arr, tolerance=-1, rate=-1, precision=-1, write_header=True) -> bytes
    decompress_numpy(compressed) -> numpy.ndarray          (needs a full header)
    header(compressed) -> dict
    _decompress(compressed, ztype, shape, out=None, tolerance=-1, rate=-1, precision=-1)

Arrays are numpy arrays in host memory (any strides, up to 4 dimensions,
float32/float64/int32/int64); the library stages them through device
memory, or reads them in place when they are page-locked.
"""
from __future__ import annotations

import ctypes as C
from itertools import zip_longest

import numpy as np

from . import capi, load

_DTYPE_TO_ZTYPE = {np.dtype(np.int32): capi.TYPE_INT32, np.dtype(np.int64): capi.TYPE_INT64,
                   np.dtype(np.float32): capi.TYPE_FLOAT, np.dtype(np.float64): capi.TYPE_DOUBLE}
_ZTYPE_TO_DTYPE = {v: k for k, v in _DTYPE_TO_ZTYPE.items()}
_MODE_NAMES = {capi.MODE_NULL: "null", capi.MODE_EXPERT: "expert", capi.MODE_FIXED_RATE: "rate",
               capi.MODE_FIXED_PRECISION: "precision", capi.MODE_FIXED_ACCURACY: "tolerance",
               capi.MODE_REVERSIBLE: "reversible"}


def dtype_to_ztype(dtype) -> int:
    """zfp scalar type of a numpy dtype (python/zfpy.pyx:39-49)."""
    try:
        return _DTYPE_TO_ZTYPE[np.dtype(dtype)]
    except KeyError:
        raise TypeError("Unknown dtype: {}".format(dtype)) from None


def ztype_to_dtype(ztype: int):
    """numpy dtype of a zfp scalar type (python/zfpy.pyx:71-79)."""
    try:
        return _ZTYPE_TO_DTYPE[ztype]
    except KeyError:
        raise ValueError("Unsupported zfp_type {}".format(ztype)) from None


def _lib():
    lib = load()
    if not hasattr(lib.lib, "_zfpy_bound"):
        L = lib.lib
        L.zfp_field_alloc.restype = capi.PF
        L.zfp_field_alloc.argtypes = []
        L.zfp_field_set_type.restype = C.c_int
        L.zfp_field_set_type.argtypes = [capi.PF, C.c_int]
        L.zfp_field_set_pointer.restype = None
        L.zfp_field_set_pointer.argtypes = [capi.PF, C.c_void_p]
        L.zfp_stream_compression_mode.restype = C.c_int
        L.zfp_stream_compression_mode.argtypes = [capi.PZ]
        L.zfp_stream_params.restype = None
        L.zfp_stream_params.argtypes = [capi.PZ, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                        C.POINTER(C.c_int)]
        L.zfp_stream_accuracy.restype = C.c_double
        L.zfp_stream_accuracy.argtypes = [capi.PZ]
        L.zfp_stream_rate.restype = C.c_double
        L.zfp_stream_rate.argtypes = [capi.PZ, C.c_uint]
        L.zfp_stream_precision.restype = C.c_uint
        L.zfp_stream_precision.argtypes = [capi.PZ]
        L._zfpy_bound = True
    return lib


def _set_compression_mode(lib, stream, ztype, ndim, tolerance=-1.0, rate=-1.0, precision=-1):
    """python/zfpy.pyx:224-239, including its call of the rate setter with the
    type the caller passes (zfp_type_none from compress_numpy)."""
    if tolerance >= 0:
        lib.zfp_stream_set_accuracy(stream, tolerance)
    elif rate >= 0:
        lib.zfp_stream_set_rate(stream, rate, ztype, ndim, 0)
    elif precision >= 0:
        lib.zfp_stream_set_precision(stream, precision)
    else:
        lib.zfp_stream_set_reversible(stream)


def _init_field(lib, arr: np.ndarray):
    """python/zfpy.pyx:92-115: extents and element strides, fastest axis first."""
    ztype = dtype_to_ztype(arr.dtype)
    if arr.ndim < 1 or arr.ndim > 4:
        raise RuntimeError("Greater than 4 dimensions not supported")
    n = tuple(reversed(arr.shape))
    s = tuple(st // arr.itemsize for st in reversed(arr.strides))
    f = capi.make_field(lib, arr.ctypes.data, ztype, n)
    f.contents.sx, f.contents.sy, f.contents.sz, f.contents.sw = capi.field_args(n, s)[1]
    return f


def _word_buffer(nbytes: int) -> np.ndarray:
    """Zeroed bytes on a 64-bit word boundary (bit streams are read and
    written in 64-bit words)."""
    return np.zeros((nbytes + 7) // 8, dtype=np.uint64).view(np.uint8)


def compress_numpy(arr, tolerance=-1.0, rate=-1.0, precision=-1, write_header=True) -> bytes:
    """Compress a numpy array on the GPU (python/zfpy.pyx:140-186)."""
    if arr is None:
        raise TypeError("Input array cannot be None")
    if sum(1 for x in (tolerance, rate, precision) if x >= 0) > 1:
        raise ValueError("Only one of tolerance, rate, or precision can be set")
    arr = np.asarray(arr)
    lib = _lib()
    field = _init_field(lib, arr)
    stream = lib.zfp_stream_open(None)
    bstream = None
    try:
        _set_compression_mode(lib, stream, capi.TYPE_NONE, arr.ndim, float(tolerance), float(rate), int(precision))
        maxsize = lib.zfp_stream_maximum_size(stream, field)
        data = _word_buffer(maxsize)
        bstream = lib.stream_open(data.ctypes.data, maxsize)
        lib.zfp_stream_set_bit_stream(stream, bstream)
        lib.zfp_stream_rewind(stream)
        if not lib.zfp_stream_set_execution(stream, capi.EXEC_CUDA):
            raise RuntimeError("CUDA execution not available")
        if write_header and lib.zfp_write_header(stream, field, capi.HEADER_FULL) == 0:
            raise RuntimeError("Failed to write header to stream")
        size = lib.zfp_compress(stream, field)
        if size == 0:
            raise RuntimeError("Failed to write to stream")
        return data[:size].tobytes()
    finally:
        lib.zfp_field_free(field)
        lib.zfp_stream_close(stream)
        if bstream:
            lib.stream_close(bstream)


def _open_compressed(lib, compressed):
    """A bit stream over a word-aligned copy of `compressed`."""
    if compressed is None:
        raise TypeError("compressed_data cannot be None")
    raw = np.frombuffer(compressed, dtype=np.uint8)
    data = _word_buffer(len(raw))
    data[: len(raw)] = raw
    return data, lib.stream_open(data.ctypes.data, len(data))


def _decompress_into(lib, stream, field, out: np.ndarray):
    lib.zfp_field_set_pointer(field, out.ctypes.data)
    if not lib.zfp_stream_set_execution(stream, capi.EXEC_CUDA):
        raise RuntimeError("CUDA execution not available")
    if lib.zfp_decompress(stream, field) == 0:
        raise RuntimeError("error during zfp decompression")


def decompress_numpy(compressed) -> np.ndarray:
    """Decompress bytes written with a full header (python/zfpy.pyx:343-366)."""
    lib = _lib()
    data, bstream = _open_compressed(lib, compressed)
    field = lib.lib.zfp_field_alloc()
    stream = lib.zfp_stream_open(bstream)
    try:
        if lib.zfp_read_header(stream, field, capi.HEADER_FULL) == 0:
            raise ValueError("Failed to read required zfp header")
        fc = field.contents
        shape = tuple(x for x in (fc.nw, fc.nz, fc.ny, fc.nx) if x > 0)
        out = np.empty(shape, dtype=ztype_to_dtype(fc.type))
        _decompress_into(lib, stream, field, out)
        return out
    finally:
        lib.zfp_field_free(field)
        lib.zfp_stream_close(stream)
        lib.stream_close(bstream)


def _decompress(compressed, ztype, shape, out=None, tolerance=-1.0, rate=-1.0, precision=-1) -> np.ndarray:
    """Decompress a header-less stream of known type and shape
    (python/zfpy.pyx:260-341)."""
    if compressed is None:
        raise TypeError("compressed_data cannot be None")
    if compressed is out:
        raise ValueError("Cannot decompress in-place")
    shape = list(shape)
    if len(shape) > 4:
        raise ValueError("User-provided shape has too many dimensions (up to 4 supported)")
    if len(shape) <= 0:
        raise ValueError("User-provided shape needs at least one dimension")
    lib = _lib()
    data, bstream = _open_compressed(lib, compressed)
    field = lib.lib.zfp_field_alloc()
    stream = lib.zfp_stream_open(bstream)
    try:
        lib.zfp_stream_rewind(stream)
        zshape = (list(reversed(shape)) + [0, 0, 0, 0])[:4]
        fc = field.contents
        fc.nx, fc.ny, fc.nz, fc.nw = zshape
        lib.lib.zfp_field_set_type(field, ztype)
        ndim = sum(1 for x in zshape if x > 0)
        _set_compression_mode(lib, stream, ztype, ndim, float(tolerance), float(rate), int(precision))
        dtype = ztype_to_dtype(ztype)
        if out is None:
            output = np.empty([x for x in shape if x > 0], dtype=dtype)
        elif isinstance(out, np.ndarray):
            if out.dtype != dtype:
                raise ValueError("Out ndarray has dtype {} but decompression is using {}. "
                                 "Use out=ndarray.data to avoid this check.".format(out.dtype, dtype))
            user_shape = [x for x in shape if x > 0]
            if not all(x == y for x, y in zip_longest(out.shape, user_shape)):
                raise ValueError("Out ndarray has shape {} but decompression is using {}.  "
                                 "Use out=ndarray.data to avoid this check.".format(out.shape, user_shape))
            output = out
        else:
            output = np.frombuffer(out, dtype=dtype).reshape(shape)
        _decompress_into(lib, stream, field, output)
        return output
    finally:
        lib.zfp_field_free(field)
        lib.zfp_stream_close(stream)
        lib.stream_close(bstream)


def header(compressed) -> dict:
    """Stream header as a dict (python/zfpy.pyx:369-423)."""
    lib = _lib()
    data, bstream = _open_compressed(lib, compressed)
    field = lib.lib.zfp_field_alloc()
    stream = lib.zfp_stream_open(bstream)
    try:
        if lib.zfp_read_header(stream, field, capi.HEADER_FULL) == 0:
            raise ValueError("Failed to read required zfp header")
        L = lib.lib
        mode = L.zfp_stream_compression_mode(stream)
        fc = field.contents
        ndim = sum(1 for x in (fc.nx, fc.ny, fc.nz, fc.nw) if x > 0)
        minbits, maxbits, maxprec, minexp = C.c_uint(), C.c_uint(), C.c_uint(), C.c_int()
        L.zfp_stream_params(stream, C.byref(minbits), C.byref(maxbits), C.byref(maxprec), C.byref(minexp))
        return {
            "nx": int(fc.nx), "ny": int(fc.ny), "nz": int(fc.nz), "nw": int(fc.nw),
            "type": ztype_to_dtype(fc.type),
            "mode": _MODE_NAMES.get(mode, "null"),
            "config": {
                "mode": int(mode),
                "tolerance": float(L.zfp_stream_accuracy(stream)),
                "rate": float(L.zfp_stream_rate(stream, ndim)),
                "precision": int(L.zfp_stream_precision(stream)),
                # the reference reports minbits under "maxbits" too (python/zfpy.pyx:414)
                "expert": {"minbits": int(minbits.value), "maxbits": int(minbits.value),
                           "maxprec": int(maxprec.value), "minexp": int(minexp.value)},
            },
        }
    finally:
        lib.zfp_field_free(field)
        lib.zfp_stream_close(stream)
        lib.stream_close(bstream)
