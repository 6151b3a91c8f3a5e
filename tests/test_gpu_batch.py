"""Batched launch (zfp_gb300_batch_*): many uneven fields of mixed modes,
types and dimensionalities in one persistent launch per group, replayed as
a CUDA graph.  Every stream must equal the oracle's (and hence the
per-field zfp_compress output) and decode to the oracle's arrays."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle.pyoracle import mode_params
from zfp_gb300 import capi, synth
from tests.helpers import oracle_stream

pytestmark = pytest.mark.gpu


def bind_batch(lib):
    L = lib.lib
    L.zfp_gb300_batch_create.restype = C.c_void_p
    L.zfp_gb300_batch_create.argtypes = [C.POINTER(capi.PZ), C.POINTER(capi.PF), C.c_size_t, C.c_int]
    L.zfp_gb300_batch_run.restype = C.c_int
    L.zfp_gb300_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    L.zfp_gb300_batch_finish.restype = C.c_int
    L.zfp_gb300_batch_finish.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
    L.zfp_gb300_batch_free.argtypes = [C.c_void_p]
    L.zfp_gb300_batch_set_ctas_per_sm.restype = C.c_int
    L.zfp_gb300_batch_set_ctas_per_sm.argtypes = [C.c_void_p, C.c_int]
    return L


def make_jobs(torch, rng, count):
    jobs = []
    for i in range(count):
        kind = i % 5
        if kind == 4:
            dtype, dims = (np.float64, 2)
        elif kind == 3:
            dtype, dims = (np.int32, 3)
        else:
            dtype, dims = (np.float32, 3)
        shape = tuple(int(v) for v in np.exp(rng.uniform(np.log(3), np.log(40), size=dims)).astype(int))
        if np.dtype(dtype).kind == "f":
            x = synth.smooth_field(shape, dtype, seed=int(rng.integers(1 << 30)), noise=1e-2,
                                   scale=10.0 ** rng.uniform(-3, 3))
            if i % 2:
                mode, arg = "rate", float(rng.choice([4, 8, 12, 16, 24, 32]))
            else:
                mode, arg = "accuracy", 10.0 ** rng.uniform(-5, -2)
        else:
            x = rng.integers(-(1 << 20), 1 << 20, size=shape, dtype=np.int32)
            mode, arg = ("reversible", None) if i % 2 else ("precision", 18)
        jobs.append(dict(x=x, mode=mode, arg=arg, dims=dims))
    return jobs


def run_batch(lib, L, torch, jobs, direction, bufs, fields_ptrs, ctas=0):
    streams, fields, keep = [], [], []
    for j, buf, fptr in zip(jobs, bufs, fields_ptrs):
        bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
        z = lib.zfp_stream_open(bs)
        zt = {"float32": 3, "float64": 4, "int32": 1}[j["x"].dtype.name]
        capi.set_mode(lib, z, j["mode"], j["arg"], zt, j["dims"])
        lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        f = capi.make_field(lib, fptr, zt, tuple(reversed(j["x"].shape)))
        streams.append(z)
        fields.append(f)
        keep.append(bs)
    zs = (capi.PZ * len(streams))(*streams)
    fs = (capi.PF * len(fields))(*fields)
    b = L.zfp_gb300_batch_create(zs, fs, len(jobs), direction)
    assert b, lib.zfp_gb300_last_error()
    if ctas:
        assert L.zfp_gb300_batch_set_ctas_per_sm(b, ctas)
    sizes = (C.c_size_t * len(jobs))()
    for _ in range(2):                     # the second run replays the captured graph
        assert L.zfp_gb300_batch_run(b, None)
        assert L.zfp_gb300_batch_finish(b, sizes), lib.zfp_gb300_last_error()
        for z in streams:
            lib.zfp_stream_rewind(z)
    L.zfp_gb300_batch_free(b)
    for z, f, bs in zip(streams, fields, keep):
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
    return list(sizes)


@pytest.mark.parametrize("ctas", [0, 1])
def test_batch_matches_oracle(lib, oracle, cuda, ctas):
    torch = cuda
    L = bind_batch(lib)
    rng = np.random.default_rng(2 + ctas)
    jobs = make_jobs(torch, rng, 150)
    expect = [oracle_stream(oracle, j["x"], j["mode"], j["arg"]) for j in jobs]
    bufs = [torch.zeros(len(e[0]) + 64, dtype=torch.int64, device="cuda") for e in expect]
    dev = [torch.from_numpy(j["x"]).cuda() for j in jobs]
    sizes = run_batch(lib, L, torch, jobs, 0, bufs, [d.data_ptr() for d in dev], ctas)
    for j, e, buf, size in zip(jobs, expect, bufs, sizes):
        words = e[0]
        assert size == len(words) * 8, (j["mode"], j["arg"], j["x"].shape)
        assert np.array_equal(buf[: len(words)].cpu().numpy().view(np.uint64), words), (j["mode"], j["x"].shape)
    # decompress as a batch (variable-rate jobs use the index recorded at compress time)
    outs = [torch.zeros_like(d) for d in dev]
    dsizes = run_batch(lib, L, torch, jobs, 1, bufs, [o.data_ptr() for o in outs], ctas)
    assert dsizes == sizes
    for j, e, o in zip(jobs, expect, outs):
        ref = np.zeros_like(j["x"])
        oracle.decompress(e[0], ref, e[2])
        assert np.array_equal(o.cpu().numpy().view(np.uint8), ref.view(np.uint8)), (j["mode"], j["x"].shape)


def test_batch_rejects_host_memory(lib, cuda):
    L = bind_batch(lib)
    x = np.ones((8, 8, 8), dtype=np.float32)
    buf = np.zeros(1024, dtype=np.uint64)
    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
    z = lib.zfp_stream_open(bs)
    lib.zfp_stream_set_rate(z, 8, capi.TYPE_FLOAT, 3, 0)
    f = capi.make_field(lib, x.ctypes.data, capi.TYPE_FLOAT, (8, 8, 8))
    zs = (capi.PZ * 1)(z)
    fs = (capi.PF * 1)(f)
    assert not L.zfp_gb300_batch_create(zs, fs, 1, 0)
    assert "device memory" in lib.zfp_gb300_last_error().decode()
    lib.zfp_field_free(f)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)
