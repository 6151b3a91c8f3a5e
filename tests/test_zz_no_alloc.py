"""zfp_gb300_compress_noalloc: compression for callers that cannot let the
library allocate device memory (their memory belongs to another allocator,
or their loop must not trigger an allocation).  Its scratch is a fixed
device array inside the library, shared by all calls, so every case runs
twice in a row: the second call must not see the first call's leftovers.
The streams must equal zfp_compress's bit for bit.  This file is collected
last on purpose; it also passes alone in a fresh process."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from zfp_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def bind(lib):
    fn = lib.lib.zfp_gb300_compress_noalloc
    fn.restype = C.c_size_t
    fn.argtypes = [capi.PZ, capi.PF]
    return fn


def compress(lib, fn, field_ptr, ztype, n, mode, arg, buf, prefix_bits=0):
    bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
    z = lib.zfp_stream_open(bs)
    capi.set_mode(lib, z, mode, arg, ztype, len(n))
    assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
    if prefix_bits:   # bits still held in the bit stream, as after a header
        lib.stream_write_bits(bs, 0x5a5a5, prefix_bits)
    f = capi.make_field(lib, field_ptr, ztype, n)
    size = fn(z, f)
    pos = lib.stream_wtell(bs)
    lib.zfp_field_free(f)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)
    return size, pos


CASES = [  # shape (numpy order), dtype, mode, arg, prefix bits
    ((40, 48, 56), np.float32, "rate", 8.0, 0),
    ((40, 48, 56), np.float32, "accuracy", 1e-3, 0),
    ((33, 65, 70), np.float64, "reversible", None, 0),
    ((17, 29, 23), np.float32, "precision", 16, 11),
    ((300, 257), np.float64, "rate", 12.5, 5),
    ((64, 64, 64, 8), np.float32, "accuracy", 1e-2, 0),
    # 4D 64-bit reversible: tiles far larger than shared memory, coded straight into the stream
    ((12, 10, 9, 11), np.float64, "reversible", None, 3),
]


@pytest.mark.parametrize("shape,dtype,mode,arg,prefix", CASES, ids=lambda v: str(v))
def test_noalloc_matches_zfp_compress_twice(lib, cuda, shape, dtype, mode, arg, prefix):
    torch = cuda
    fn = bind(lib)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    ztype = capi.TYPE_FLOAT if dtype == np.float32 else capi.TYPE_DOUBLE
    x = synth.smooth_field_torch(shape, tdt, seed=7, noise=1e-2)
    n = tuple(reversed(shape))
    words = x.numel() * x.element_size() // 8 * 2 + 256
    ref = torch.zeros(words, dtype=torch.int64, device="cuda")
    size, pos = compress(lib, lib.zfp_compress, x.data_ptr(), ztype, n, mode, arg, ref, prefix)
    assert size > 0, lib.zfp_gb300_last_error()
    for attempt in range(2):
        out = torch.full((words,), -1, dtype=torch.int64, device="cuda")
        size2, pos2 = compress(lib, fn, x.data_ptr(), ztype, n, mode, arg, out, prefix)
        assert size2 == size and pos2 == pos, (attempt, size2, size, lib.zfp_gb300_last_error())
        assert torch.equal(out[: size // 8], ref[: size // 8]), f"stream differs on call {attempt + 1}"


def test_noalloc_refuses_what_it_cannot_do_without_allocating(lib, cuda):
    torch = cuda
    fn = bind(lib)
    # host-resident field: would need a staging copy
    h = np.ones((16, 16, 16), dtype=np.float32)
    buf = torch.zeros(4096, dtype=torch.int64, device="cuda")
    size, pos = compress(lib, fn, h.ctypes.data, capi.TYPE_FLOAT, (16, 16, 16), "rate", 8.0, buf)
    assert size == 0 and pos == 0
    assert "device memory" in lib.zfp_gb300_last_error().decode()
    # more blocks than the fixed scratch covers
    big = torch.zeros(4 * 4194304 + 4, dtype=torch.float32, device="cuda")
    buf = torch.zeros(big.numel() // 8 + 64, dtype=torch.int64, device="cuda")
    size, pos = compress(lib, fn, big.data_ptr(), capi.TYPE_FLOAT, (big.numel(),), "rate", 8.0, buf)
    assert size == 0 and "4194304" in lib.zfp_gb300_last_error().decode()


# Driver-level view of device memory, so the test sees allocations made by
# the library itself (its stream-ordered allocations come from the device's
# default memory pool; torch's caching allocator does not use that pool).
_USED_CURRENT, _USED_HIGH, _RESERVED_CURRENT = 7, 8, 5   # CUmemPool_attribute


def _driver():
    d = C.CDLL("libcuda.so.1")
    assert d.cuInit(0) == 0
    dev = C.c_int()
    assert d.cuCtxGetDevice(C.byref(dev)) == 0
    pool = C.c_void_p()
    assert d.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    return d, pool


def _pool_attr(d, pool, attr):
    v = C.c_uint64()
    assert d.cuMemPoolGetAttribute(pool, attr, C.byref(v)) == 0
    return v.value


def _free_bytes(d):
    free, total = C.c_size_t(), C.c_size_t()
    assert d.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    return free.value


def test_noalloc_allocates_no_device_memory(lib, cuda):
    """The point of the entry point: after its set-up (first call), calls
    take no memory from the device's pool and none from the driver."""
    torch = cuda
    fn = bind(lib)
    x = synth.smooth_field_torch((48, 40, 56), torch.float32, seed=5, noise=1e-2)
    n = tuple(reversed(x.shape))
    buf = torch.zeros(x.numel() // 2 + 256, dtype=torch.int64, device="cuda")
    assert compress(lib, fn, x.data_ptr(), capi.TYPE_FLOAT, n, "accuracy", 1e-3, buf)[0] > 0
    torch.cuda.synchronize()
    d, pool = _driver()
    zero = C.c_uint64(0)
    assert d.cuMemPoolSetAttribute(pool, _USED_HIGH, C.byref(zero)) == 0   # high-water mark := current use
    used0 = _pool_attr(d, pool, _USED_CURRENT)
    reserved0 = _pool_attr(d, pool, _RESERVED_CURRENT)
    free0 = _free_bytes(d)
    for mode, arg in (("rate", 8.0), ("accuracy", 1e-3), ("reversible", None), ("rate", 8.0)):
        assert compress(lib, fn, x.data_ptr(), capi.TYPE_FLOAT, n, mode, arg, buf)[0] > 0, \
            lib.zfp_gb300_last_error()
    torch.cuda.synchronize()
    assert _pool_attr(d, pool, _USED_HIGH) <= used0, "a call took memory from the device pool"
    assert _pool_attr(d, pool, _RESERVED_CURRENT) == reserved0
    assert _free_bytes(d) == free0, "device memory changed across the calls"


def test_noalloc_stream_replaces_an_indexed_one_and_decodes(lib, cuda):
    """A variable-rate stream written by zfp_compress leaves a block index
    behind; writing another stream at the same place with the no-alloc call
    must drop it (zfp_gb300_index_export then reports no index), and the new
    stream must decode -- by parsing, as it carries no index -- to exactly
    what zfp_compress's stream of the same field decodes to."""
    torch = cuda
    fn = bind(lib)
    L = lib.lib
    L.zfp_gb300_index_export.restype = C.c_size_t
    L.zfp_gb300_index_export.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t,
                                         C.POINTER(C.c_uint64)]
    shape = (36, 44, 52)
    a = synth.smooth_field_torch(shape, torch.float64, seed=11, noise=1e-2)
    b = synth.smooth_field_torch(shape, torch.float64, seed=12, noise=1e-2) * 3.0
    n = tuple(reversed(shape))
    words = a.numel() * 2 + 256
    buf = torch.zeros(words, dtype=torch.int64, device="cuda")
    ref = torch.zeros(words, dtype=torch.int64, device="cuda")
    assert compress(lib, lib.zfp_compress, a.data_ptr(), capi.TYPE_DOUBLE, n, "accuracy", 1e-3, buf)[0] > 0
    size_b, _ = compress(lib, fn, b.data_ptr(), capi.TYPE_DOUBLE, n, "accuracy", 1e-3, buf)
    assert size_b > 0, lib.zfp_gb300_last_error()
    assert compress(lib, lib.zfp_compress, b.data_ptr(), capi.TYPE_DOUBLE, n, "accuracy", 1e-3, ref)[0] == size_b

    def open_stream(buffer):
        bs = lib.stream_open(buffer.data_ptr(), buffer.numel() * 8)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, "accuracy", 1e-3, capi.TYPE_DOUBLE, 3)
        assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        return bs, z

    bs, z = open_stream(buf)
    f = capi.make_field(lib, b.data_ptr(), capi.TYPE_DOUBLE, n)
    out = np.zeros(8 * (a.numel() // 64 + 8), dtype=np.uint8)
    rng = C.c_uint64()
    got = L.zfp_gb300_index_export(C.cast(z, C.c_void_p), C.cast(f, C.c_void_p), 1, out.ctypes.data, out.nbytes,
                                   C.byref(rng))
    assert got == 0 and "no index" in lib.zfp_gb300_last_error().decode()
    lib.zfp_field_free(f)

    outs = []
    for buffer in (buf, ref):
        bs2, z2 = open_stream(buffer)
        y = torch.empty_like(b)
        f2 = capi.make_field(lib, y.data_ptr(), capi.TYPE_DOUBLE, n)
        assert lib.zfp_decompress(z2, f2) == size_b, lib.zfp_gb300_last_error()
        outs.append(y)
        lib.zfp_field_free(f2)
        lib.zfp_stream_close(z2)
        lib.stream_close(bs2)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)
    torch.cuda.synchronize()
    assert torch.equal(outs[0].view(torch.int64), outs[1].view(torch.int64))
    assert (outs[0] - b).abs().max().item() <= 1e-3
