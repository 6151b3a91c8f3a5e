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
