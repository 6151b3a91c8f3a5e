"""zfp's low-level block codec (zfp_encode_block_* / zfp_decode_block_*,
reference include/zfp.h:636-775) against the reference library itself:
the same sequence of per-block calls on the same stream must write the same
bits and return the same bit counts, and so must one batched call
(zfp_gb300_encode_blocks) for a run of blocks; decoding must give the
reference's arrays.  Full, strided and partial blocks, every scalar type and
dimensionality, fixed rate / precision / accuracy / reversible.  Needs the
reference's sources (its library is compiled from them)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from zfp_gb300 import capi

pytestmark = pytest.mark.gpu

TYPES = {np.int32: ("int32", capi.TYPE_INT32), np.int64: ("int64", capi.TYPE_INT64),
         np.float32: ("float", capi.TYPE_FLOAT), np.float64: ("double", capi.TYPE_DOUBLE)}


def fn(lib, name):
    f = getattr(lib.lib, name)
    f.restype = C.c_size_t
    return f


def blocks_of(dtype, dims, count, rng):
    shape = (count,) + (4,) * dims
    if np.dtype(dtype).kind == "f":
        base = np.cumsum(rng.standard_normal(shape), axis=-1) * 10.0 ** rng.uniform(-3, 3)
        return base.astype(dtype)
    bits = 24 if dtype == np.int32 else 50
    return rng.integers(-(1 << bits), 1 << bits, size=shape, dtype=dtype)


def open_stream(lib, buf, mode, arg, ztype, dims):
    bs = lib.stream_open(buf.ctypes.data if isinstance(buf, np.ndarray) else buf.data_ptr(),
                         buf.nbytes if isinstance(buf, np.ndarray) else buf.numel() * 8)
    z = lib.zfp_stream_open(bs)
    capi.set_mode(lib, z, mode, arg, ztype, dims)
    return bs, z


MODES = [("rate", 12.0), ("precision", 20), ("accuracy", 1e-3), ("reversible", None)]


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64], ids=lambda d: np.dtype(d).name)
def test_block_calls_match_reference(lib, ref, cuda, dims, dtype):
    rng = np.random.default_rng(dims * 7 + np.dtype(dtype).itemsize)
    name, ztype = TYPES[dtype]
    count = 23
    blk = blocks_of(dtype, dims, count, rng)
    step = blk[0].nbytes
    for mode, arg in MODES:
        if mode == "accuracy" and np.dtype(dtype).kind == "i":
            continue
        words = count * (64 * (4 ** dims) + 64) // 64 + 16
        out = {}
        for who, L in (("ref", ref), ("gpu", lib)):
            buf = np.zeros(words, dtype=np.uint64)
            bs, z = open_stream(L, buf, mode, arg, ztype, dims)
            enc = fn(L, f"zfp_encode_block_{name}_{dims}")
            sizes = [enc(z, C.c_void_p(blk.ctypes.data + i * step)) for i in range(count)]
            L.stream_flush(bs)
            out[who] = (buf.copy(), sizes)
            # decode the same way
            L.zfp_stream_rewind(z)
            dec = fn(L, f"zfp_decode_block_{name}_{dims}")
            back = np.zeros_like(blk)
            dsizes = [dec(z, C.c_void_p(back.ctypes.data + i * step)) for i in range(count)]
            out[who] += (back, dsizes)
            L.zfp_stream_close(z)
            L.stream_close(bs)
        assert out["gpu"][1] == out["ref"][1], (mode, "bit counts differ")
        assert np.array_equal(out["gpu"][0], out["ref"][0]), (mode, "streams differ")
        assert out["gpu"][3] == out["ref"][3], (mode, "decode bit counts differ")
        assert np.array_equal(out["gpu"][2].view(np.uint8), out["ref"][2].view(np.uint8)), (mode, "decode differs")
        # one batched call, host buffers, then device buffers
        ref_words, ref_sizes, ref_back = out["ref"][0], out["ref"][1], out["ref"][2]
        total = sum(ref_sizes)
        for device in (False, True):
            torch = cuda
            buf = torch.zeros(words, dtype=torch.int64, device="cuda") if device else np.zeros(words, dtype=np.uint64)
            data = torch.from_numpy(blk).cuda() if device else blk
            ptr = data.data_ptr() if device else data.ctypes.data
            bs, z = open_stream(lib, buf, mode, arg, ztype, dims)
            bits = fn(lib, "zfp_gb300_encode_blocks")(z, ztype, dims, C.c_void_p(ptr), count)
            assert bits == total, (mode, device, bits, total, lib.zfp_gb300_last_error())
            assert lib.stream_wtell(bs) == total
            nw = (total + 63) // 64
            got = (buf.cpu().numpy().view(np.uint64) if device else buf)[:nw].copy()
            if total % 64:   # the last word's bits past the end are the caller's to pad
                got[-1] &= np.uint64((1 << (total % 64)) - 1)
            assert np.array_equal(got, ref_words[:nw]), (mode, device, "batched stream differs")
            lib.zfp_stream_rewind(z)
            back = torch.zeros_like(data) if device else np.zeros_like(blk)
            bptr = back.data_ptr() if device else back.ctypes.data
            assert fn(lib, "zfp_gb300_decode_blocks")(z, ztype, dims, C.c_void_p(bptr), count) == total
            assert lib.stream_rtell(bs) == total
            b = back.cpu().numpy() if device else back
            assert np.array_equal(b.view(np.uint8), ref_back.view(np.uint8)), (mode, device, "batched decode differs")
            lib.zfp_stream_close(z)
            lib.stream_close(bs)


def test_strided_and_partial_blocks_match_reference(lib, ref, cuda):
    """Strided full blocks and partial blocks (padded on encode, scattered on
    decode) of a larger array, in 2D, 3D and 4D."""
    rng = np.random.default_rng(5)
    a = (np.cumsum(rng.standard_normal((9, 10, 11, 12)), axis=-1)).astype(np.float64)
    cases = [  # (function suffix, dims, extents or None, numpy view)
        ("block_strided_double_2", 2, None, a[0, 0, 2:10:2, 1:5]),
        ("partial_block_strided_double_2", 2, (3, 2), a[0, 0, 3:5, 1:4]),
        ("block_strided_double_3", 3, None, a[1, 4:8, 2:6, 0:12:3]),
        ("partial_block_strided_double_3", 3, (2, 3, 1), a[2, 5:6, 1:4, 7:9]),
        ("partial_block_strided_double_4", 4, (1, 4, 2, 3), a[6:9, 2:4, 5:9, 10:11]),
        ("block_strided_double_1", 1, None, a[3, 3, 3, 0:12:3]),
        ("partial_block_strided_double_1", 1, (3,), a[3, 3, 3, 4:7]),
    ]
    for suffix, dims, ext, view in cases:
        strides = [s // 8 for s in reversed(view.strides)]
        out = {}
        for who, L in (("ref", ref), ("gpu", lib)):
            buf = np.zeros(256, dtype=np.uint64)
            bs, z = open_stream(L, buf, "precision", 30, capi.TYPE_DOUBLE, dims)
            args = [C.c_void_p(view.ctypes.data)] + [C.c_size_t(e) for e in (ext or ())] + \
                   [C.c_ssize_t(s) for s in strides]
            bits = fn(L, f"zfp_encode_{suffix}")(z, *args)
            L.stream_flush(bs)
            L.zfp_stream_rewind(z)
            dst = np.zeros((13, 13, 13, 13), dtype=np.float64)
            dview = dst[tuple(slice(0, n) for n in view.shape)]
            dstr = [s // 8 for s in reversed(dview.strides)]
            dargs = [C.c_void_p(dview.ctypes.data)] + [C.c_size_t(e) for e in (ext or ())] + \
                    [C.c_ssize_t(s) for s in dstr]
            dbits = fn(L, f"zfp_decode_{suffix}")(z, *dargs)
            out[who] = (bits, buf.copy(), dbits, dst)
            L.zfp_stream_close(z)
            L.stream_close(bs)
        assert out["gpu"][0] == out["ref"][0] and out["gpu"][0] > 0, (suffix, lib.zfp_gb300_last_error())
        assert np.array_equal(out["gpu"][1], out["ref"][1]), suffix
        assert out["gpu"][2] == out["ref"][2], suffix
        assert np.array_equal(out["gpu"][3], out["ref"][3]), suffix
