"""zfp's block-index formats (include/zfp/index.hpp) as a side channel:
zfp_gb300_index_pack / _unpack against golden vectors written by the
reference's own index classes (tests/golden/index_golden.*, made by
make_index_golden.py), and export / import around the GPU codec."""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np
import pytest

import zfp_gb300
from zfp_gb300 import capi
from tests.helpers import geometry, oracle_stream, zfp_run, ztype_of

HERE = os.path.dirname(os.path.abspath(__file__))
VERBATIM, HYBRID4, HYBRID8 = 1, 2, 3


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "index_golden.json")) as f:
        cases = json.load(f)["cases"]
    return cases, np.load(os.path.join(HERE, "golden", "index_golden.npz"))


def bind(lib):
    L = lib.lib
    L.zfp_gb300_index_bytes.restype = C.c_size_t
    L.zfp_gb300_index_bytes.argtypes = [C.c_int, C.c_size_t]
    L.zfp_gb300_index_pack.restype = C.c_size_t
    L.zfp_gb300_index_pack.argtypes = [C.c_int, C.c_uint, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]
    L.zfp_gb300_index_unpack.restype = C.c_int
    L.zfp_gb300_index_unpack.argtypes = [C.c_int, C.c_uint, C.c_void_p, C.c_size_t, C.c_size_t, C.c_uint64,
                                         C.c_void_p]
    L.zfp_gb300_index_export.restype = C.c_size_t
    L.zfp_gb300_index_export.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t,
                                         C.POINTER(C.c_uint64)]
    L.zfp_gb300_index_import.restype = C.c_int
    L.zfp_gb300_index_import.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_uint64]
    return L


def open_stream(lib, data_ptr, ztype, n, s, mode, arg, buf_ptr, buf_bytes):
    """A zfp_stream (CUDA policy) over the buffer, rewound, and a field."""
    bs = lib.stream_open(buf_ptr, buf_bytes)
    z = lib.zfp_stream_open(bs)
    capi.set_mode(lib, z, mode, arg, ztype, sum(1 for v in n if v))
    assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
    lib.zfp_stream_rewind(z)
    return z, capi.make_field(lib, data_ptr, ztype, n, s), bs


def close_stream(lib, z, f, bs):
    lib.zfp_field_free(f)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)


def pack(L, fmt, dims, offsets):
    n = len(offsets) - 1
    out = np.zeros(L.zfp_gb300_index_bytes(fmt, n), dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    r = L.zfp_gb300_index_pack(fmt, dims, off.ctypes.data, n, out.ctypes.data, len(out))
    return out if r == len(out) else None


def unpack(L, fmt, dims, packed, n, rng):
    off = np.zeros(n + 1, dtype=np.uint64)
    ok = L.zfp_gb300_index_unpack(fmt, dims, packed.ctypes.data, len(packed), n, rng, off.ctypes.data)
    return off if ok else None


def test_pack_unpack_match_reference_index_classes(lib, golden):
    """Packed bytes equal what index.hpp's verbatim / hybrid4 / hybrid8<d>
    build from the same block sizes; unpacking gives its block offsets."""
    L = bind(lib)
    cases, data = golden
    for c in cases:
        sizes = data["sizes_" + c["key"]]
        offsets = np.concatenate([[0], np.cumsum(sizes, dtype=np.uint64)]).astype(np.uint64)
        assert int(offsets[-1]) == c["range"], c
        got = pack(L, c["format"], c["dims"], offsets)
        assert got is not None, (c, zfp_gb300.last_error())
        assert np.array_equal(got, data["packed_" + c["key"]]), c
        back = unpack(L, c["format"], c["dims"], data["packed_" + c["key"]], c["nblocks"], c["range"])
        assert back is not None, (c, zfp_gb300.last_error())
        assert np.array_equal(back[:-1], data["offsets_" + c["key"]]) and int(back[-1]) == c["range"], c


def test_pack_rejects_what_the_formats_cannot_hold(lib):
    L = bind(lib)
    assert pack(L, HYBRID4, 3, np.array([0, 16658, 16658 + 16659], dtype=np.uint64)) is None   # > ZFP_MAX_BITS
    assert pack(L, HYBRID8, 3, np.array([0, 4095, 4095 + 4096], dtype=np.uint64)) is None     # > 12 bits
    assert pack(L, HYBRID8, 3, np.array([0, 4095, 8190], dtype=np.uint64)) is not None
    assert pack(L, VERBATIM, 2, np.array([0, 5, 3], dtype=np.uint64)) is None                 # decreasing
    off = np.array([0, 5], dtype=np.uint64)
    out = np.zeros(64, dtype=np.uint8)
    assert L.zfp_gb300_index_bytes(7, 1) == 0                                                  # unknown format
    assert L.zfp_gb300_index_pack(7, 2, off.ctypes.data, 1, out.ctypes.data, len(out)) == 0
    assert L.zfp_gb300_index_pack(HYBRID4, 3, off.ctypes.data, 1, out.ctypes.data, 4) == 0     # buffer too small
    assert L.zfp_gb300_index_bytes(HYBRID4, 5) == 24 and L.zfp_gb300_index_bytes(HYBRID8, 9) == 32
    assert L.zfp_gb300_index_bytes(VERBATIM, 5) == 48


@pytest.mark.gpu
def test_export_import_around_the_gpu_codec(lib, oracle, cuda):
    """Export after compression gives the oracle's block offsets in every
    format; importing one lets a copy of the stream (which the library never
    saw) decode to the oracle's array, and a wrong index still decodes right
    (the decoder checks every block and parses instead)."""
    L = bind(lib)
    torch = cuda
    rng = np.random.default_rng(31)
    shape = (20, 36, 44)
    vals = np.cumsum(rng.standard_normal(shape), axis=-1).astype(np.float32)
    words, end, prm = oracle_stream(oracle, vals, "accuracy", 1e-3)
    _, _, ends = oracle.compress(vals, prm, block_ends=True)
    offsets = np.concatenate([[0], np.asarray(ends, dtype=np.uint64)]).astype(np.uint64)
    ref_out = np.zeros(shape, dtype=np.float32)
    oracle.decompress(words, ref_out, prm, 0)
    n, s = geometry(vals)
    zt = ztype_of(vals)
    nwords = len(words) + 8
    dx = torch.from_numpy(vals).cuda()
    dbuf = torch.zeros(nwords, dtype=torch.int64, device="cuda")
    r, _ = zfp_run(lib, "compress", dx.data_ptr(), zt, n, s, "accuracy", 1e-3, dbuf.data_ptr(), nwords * 8)
    assert r == len(words) * 8, zfp_gb300.last_error()

    # export: reopen the stream at its start
    z, f, bs = open_stream(lib, dx.data_ptr(), zt, n, s, "accuracy", 1e-3, dbuf.data_ptr(), nwords * 8)
    try:
        for fmt, dims in [(VERBATIM, 3), (HYBRID4, 3), (HYBRID8, 3)]:
            size = L.zfp_gb300_index_bytes(fmt, len(offsets) - 1)
            buf = np.zeros(size, dtype=np.uint8)
            rng_bits = C.c_uint64()
            got = L.zfp_gb300_index_export(C.cast(z, C.c_void_p), C.cast(f, C.c_void_p), fmt, buf.ctypes.data,
                                           size, C.byref(rng_bits))
            assert got == size, zfp_gb300.last_error()
            assert rng_bits.value == int(offsets[-1])
            assert np.array_equal(buf, pack(L, fmt, dims, offsets)), fmt
    finally:
        close_stream(lib, z, f, bs)

    # import into a copy of the stream the library has never seen
    for fmt, corrupt in [(HYBRID4, False), (HYBRID8, False), (VERBATIM, True)]:
        other = dbuf.clone()
        idx_off = offsets.copy()
        if corrupt:
            idx_off[1:-1] += 1
        packed = pack(L, fmt, 3, idx_off)
        out = torch.zeros_like(dx)
        z, f, bs = open_stream(lib, out.data_ptr(), zt, n, s, "accuracy", 1e-3, other.data_ptr(), nwords * 8)
        try:
            ok = L.zfp_gb300_index_import(C.cast(z, C.c_void_p), C.cast(f, C.c_void_p), fmt, packed.ctypes.data,
                                          len(packed), int(idx_off[-1]))
            assert ok, zfp_gb300.last_error()
            assert lib.zfp_decompress(z, f) == r, zfp_gb300.last_error()
        finally:
            close_stream(lib, z, f, bs)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), ref_out.view(np.uint32)), (fmt, corrupt)
