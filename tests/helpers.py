"""Client-side helpers: drive a zfp C library (the GB300 one or the
reference) the way the reference's own end-to-end tests do
(tests/src/endtoend/zfpEndtoendBase.c): open a bit stream over a buffer,
set the mode, describe the field, compress, hash/compare."""
from __future__ import annotations

import ctypes as C

import numpy as np

from oracle.pyoracle import ZTYPE, mode_params
from zfp_gb300 import capi


def geometry(a):
    """zfp extents/strides (fastest axis first) of a numpy array or torch tensor."""
    shape = tuple(a.shape)
    if hasattr(a, "stride") and callable(a.stride):
        strides = tuple(a.stride())
    else:
        strides = tuple(s // a.itemsize for s in a.strides)
    return tuple(reversed(shape)), tuple(reversed(strides))


def ztype_of(a) -> int:
    name = str(a.dtype).replace("torch.", "")
    return {"int32": 1, "int64": 2, "float32": 3, "float64": 4}[name]


def ptr_of(a) -> int:
    return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data


def zfp_run(lib, direction, data_ptr, ztype, n, s, mode, arg, buf_ptr, buf_bytes, prefix=None,
            policy=capi.EXEC_CUDA, cuda_stream=None, async_=False):
    """One zfp_compress / zfp_decompress call.  `prefix` = (word, value, nbits)
    positions the stream at bit 64*word + nbits with `value` as the bits
    already written there (for decompression of a device buffer nbits must
    be 0: a mid-word seek reads the buffer from the host).  Returns
    (return value, stream offset after)."""
    dims = sum(1 for v in n if v)
    bs = lib.stream_open(buf_ptr, buf_bytes)
    z = lib.zfp_stream_open(bs)
    try:
        capi.set_mode(lib, z, mode, arg, ztype, dims)
        if policy is not None:
            assert lib.zfp_stream_set_execution(z, policy)
        if cuda_stream is not None:
            assert lib.zfp_gb300_stream_set_cuda_stream(z, cuda_stream)
        if async_:
            assert lib.zfp_gb300_stream_set_async(z, 1)
        if prefix:
            word, value, nbits = prefix
            if direction == "compress":
                lib.stream_wseek(bs, 64 * word)
                if nbits:
                    lib.stream_write_bits(bs, value, nbits)
            else:
                lib.stream_rseek(bs, 64 * word + nbits)
        f = capi.make_field(lib, data_ptr, ztype, n, s)
        try:
            if direction == "compress":
                r = lib.zfp_compress(z, f)
                pos = lib.stream_wtell(bs)
            else:
                r = lib.zfp_decompress(z, f)
                pos = lib.stream_rtell(bs)
        finally:
            lib.zfp_field_free(f)
        return r, pos
    finally:
        lib.zfp_stream_close(z)
        lib.stream_close(bs)


def oracle_stream(oracle, view, mode, arg, prefix=None, room=0):
    """Oracle stream words for a numpy view (with the same prefix bits).
    `room`: words to provide at least, for budgets below the block header
    size, where the reference's bit budget wraps around and blocks run past
    what zfp_stream_maximum_size allows for."""
    n, s = geometry(view)
    prm = mode_params(mode, arg, view.dtype, len(n))
    bit0 = 0
    words = np.zeros(max(room, oracle.max_words(n, view.dtype, prm)) + 8 + (prefix[0] if prefix else 0),
                     dtype=np.uint64)
    if prefix:
        word, value, nbits = prefix
        bit0 = 64 * word + nbits
        if nbits:
            words[word] = np.uint64(value & ((1 << nbits) - 1))
    words, end = oracle.compress(view, prm, bit0=bit0, words=words)
    return words[: (end + 63) // 64].copy(), end, prm
