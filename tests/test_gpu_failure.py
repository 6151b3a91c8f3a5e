"""Failure detection without a GPU fault: a variable-rate encoder tile whose
predecessor never publishes its bit count must give up after its bounded
wait, the call must fail cleanly ("GPU wait timed out"), and the next call
on the same GPU must succeed and match the oracle.  The failure is made on
the host (zfp_gb300_test_skip_first_tile: the first tile is never handed
out), with a short wait bound (zfp_gb300_set_wait_limit)."""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import pytest

from zfp_gb300 import capi, synth
from tests.helpers import oracle_stream

pytestmark = pytest.mark.gpu


def test_lost_predecessor_times_out_and_gpu_stays_usable(lib, oracle, cuda):
    torch = cuda
    L = lib.lib
    L.zfp_gb300_set_wait_limit.restype = C.c_ulonglong
    L.zfp_gb300_set_wait_limit.argtypes = [C.c_ulonglong]
    L.zfp_gb300_test_skip_first_tile.argtypes = [C.c_int]
    a = synth.smooth_field((48, 64, 80), np.float32, seed=9, noise=1e-2)   # 3840 blocks: 30 tiles
    x = torch.from_numpy(a).cuda()
    n = tuple(reversed(a.shape))
    buf = torch.zeros(a.size, dtype=torch.int64, device="cuda")

    def compress():
        bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, "accuracy", 1e-3, capi.TYPE_FLOAT, 3)
        assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        f = capi.make_field(lib, x.data_ptr(), capi.TYPE_FLOAT, n)
        size = lib.zfp_compress(z, f)
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
        return size

    prev = L.zfp_gb300_set_wait_limit(200000)   # about 0.1 ms
    try:
        L.zfp_gb300_test_skip_first_tile(1)
        t0 = time.perf_counter()
        assert compress() == 0
        elapsed = time.perf_counter() - t0
        assert "timed out" in lib.zfp_gb300_last_error().decode()
        assert elapsed < 5.0
    finally:
        L.zfp_gb300_test_skip_first_tile(0)
        L.zfp_gb300_set_wait_limit(prev)
    # the same GPU, context and library go on working
    size = compress()
    assert size > 0, lib.zfp_gb300_last_error()
    words, _, _ = oracle_stream(oracle, a, "accuracy", 1e-3)
    assert size == len(words) * 8
    assert np.array_equal(buf[: len(words)].cpu().numpy().view(np.uint64), words)
