"""Serving (zfp_gb300_server_*): requests submitted while others run are
batched continuously under an HBM budget on several CUDA streams.  Every
result must be the same as the request run alone through zfp_compress /
zfp_decompress (bit for bit), and the budget must be honoured."""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np
import pytest

from zfp_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def bind(lib):
    L = lib.lib
    L.zfp_gb300_server_create.restype = C.c_void_p
    L.zfp_gb300_server_create.argtypes = [C.c_size_t, C.c_int]
    L.zfp_gb300_server_submit.restype = C.c_uint64
    L.zfp_gb300_server_submit.argtypes = [C.c_void_p, capi.PZ, capi.PF, C.c_int]
    L.zfp_gb300_server_wait.restype = C.c_size_t
    L.zfp_gb300_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]
    L.zfp_gb300_server_free.argtypes = [C.c_void_p]
    L.zfp_gb300_server_stats.restype = C.c_int
    L.zfp_gb300_server_stats.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_uint64)]
    return L


class Req:
    def __init__(self, lib, torch, rng, i):
        self.lib = lib
        kind = i % 4
        dims = 2 if kind in (1, 3) else 3
        self.dtype = torch.float64 if kind >= 2 else torch.float32
        self.ztype = capi.TYPE_DOUBLE if kind >= 2 else capi.TYPE_FLOAT
        n = int(np.exp(rng.uniform(np.log(6), np.log(64 if dims == 3 else 400))))
        self.shape = (n,) * dims
        self.x = synth.smooth_field_torch(self.shape, self.dtype, seed=i, noise=1e-2)
        rangev = float(self.x.max() - self.x.min())
        self.mode, self.arg = [("accuracy", 1e-4 * rangev), ("rate", 12.0), ("precision", 22),
                               ("reversible", None)][i % 4]
        self.cap = self.x.numel() * self.x.element_size() // 8 * 2 + 64
        self.buf = torch.zeros(self.cap, dtype=torch.int64, device="cuda")
        self.out = torch.zeros_like(self.x)
        self.objs = []

    def open(self, direction):
        lib = self.lib
        bs = lib.stream_open(self.buf.data_ptr(), self.cap * 8)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, self.mode, self.arg, self.ztype, len(self.shape))
        lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        ptr = self.x.data_ptr() if direction == 0 else self.out.data_ptr()
        f = capi.make_field(lib, ptr, self.ztype, tuple(reversed(self.shape)))
        self.objs.append((bs, z, f))
        return z, f

    def close(self):
        for bs, z, f in self.objs:
            self.lib.zfp_field_free(f)
            self.lib.zfp_stream_close(z)
            self.lib.stream_close(bs)
        self.objs = []


def test_server_results_equal_alone(lib, cuda):
    """Compress and decompress requests interleaved in the same batches."""
    torch = cuda
    L = bind(lib)
    rng = np.random.default_rng(3)
    reqs = [Req(lib, torch, rng, i) for i in range(160)]
    # alone: each request through zfp_compress / zfp_decompress
    alone, alone_out = [], []
    for r in reqs:
        z, f = r.open(0)
        size = lib.zfp_compress(z, f)
        assert size, lib.zfp_gb300_last_error()
        alone.append((size, r.buf[: size // 8].clone()))
        r.close()
        z, f = r.open(1)
        assert lib.zfp_decompress(z, f) == size
        r.close()
        alone_out.append(r.out.clone())
    # odd requests will be decompressed from the streams written above; even
    # ones compressed again from scratch, all through one server
    for i, r in enumerate(reqs):
        r.out.zero_()
        if i % 2 == 0:
            r.buf.zero_()
    server = L.zfp_gb300_server_create(64 << 20, 3)   # small budget: admission has to wait
    assert server
    tickets = []

    def submitter():
        for i, r in enumerate(reqs):
            direction = i % 2
            z, f = r.open(direction)
            t = L.zfp_gb300_server_submit(server, z, f, direction)
            assert t, lib.zfp_gb300_last_error()
            tickets.append(t)
            time.sleep(float(rng.exponential(2e-4)))

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    lat = C.c_double()
    for i, (r, t, (size, words)) in enumerate(zip(reqs, tickets, alone)):
        got = L.zfp_gb300_server_wait(server, t, C.byref(lat))
        assert got == size, (i, lib.zfp_gb300_last_error())
        assert lat.value > 0
        if i % 2 == 0:
            assert torch.equal(r.buf[: size // 8], words), f"request {i}: stream differs"
        else:
            assert torch.equal(r.out.view(torch.int8), alone_out[i].view(torch.int8)), f"request {i}: decode differs"
    for r in reqs:
        r.close()
    # every even request's new stream decodes to the same array as alone
    tickets = []
    for i, r in enumerate(reqs):
        if i % 2 == 0:
            r.out.zero_()
            z, f = r.open(1)
            tickets.append((i, L.zfp_gb300_server_submit(server, z, f, 1)))
    for i, t in tickets:
        assert t and L.zfp_gb300_server_wait(server, t, None) == alone[i][0]
        assert torch.equal(reqs[i].out.view(torch.int8), alone_out[i].view(torch.int8))
    for r in reqs:
        r.close()
    # the budget was honoured: admitted bytes never exceeded it, and it did
    # bind (more than one batch was needed for what was queued)
    peak, batches, served = C.c_size_t(), C.c_uint64(), C.c_uint64()
    assert L.zfp_gb300_server_stats(server, C.byref(peak), C.byref(batches), C.byref(served))
    assert 0 < peak.value <= (64 << 20)
    assert served.value == len(reqs) + len(tickets)
    assert batches.value > 1
    L.zfp_gb300_server_free(server)


def test_server_refuses_oversized_and_host(lib, cuda):
    torch = cuda
    L = bind(lib)
    server = L.zfp_gb300_server_create(1 << 20, 1)
    x = torch.zeros((64, 64, 64), dtype=torch.float32, device="cuda")   # 1 MiB field + stream > budget
    buf = torch.zeros(1 << 17, dtype=torch.int64, device="cuda")
    bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
    z = lib.zfp_stream_open(bs)
    lib.zfp_stream_set_rate(z, 8, capi.TYPE_FLOAT, 3, 0)
    lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
    f = capi.make_field(lib, x.data_ptr(), capi.TYPE_FLOAT, (64, 64, 64))
    assert L.zfp_gb300_server_submit(server, z, f, 0) == 0
    assert "budget" in lib.zfp_gb300_last_error().decode()
    h = np.zeros((8, 8), dtype=np.float32)
    g = capi.make_field(lib, h.ctypes.data, capi.TYPE_FLOAT, (8, 8))
    assert L.zfp_gb300_server_submit(server, z, g, 0) == 0
    for x_ in (f, g):
        lib.zfp_field_free(x_)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)
    L.zfp_gb300_server_free(server)
