"""The batched and serving benchmark workloads at their real size and mix,
against the oracle (the C restatement of the reference's serial codec, run
in parallel on the host cores).

* Batch: the benchmark's 4096 uneven 3D float32 arrays (seed 2; half fixed
  rate, half fixed accuracy), compressed in one batched launch and decoded
  in another: every stream must equal the oracle's and every decoded array
  the oracle's decoding of it.
* Serving: the first 200 requests of the benchmark's request stream (seed 3:
  70% compress, 30% decompress; 2D/3D float32/float64 views of resident
  fields, 16 KiB to 256 MiB; tolerance 1e-4 x the field's range) through the
  continuous-batching server: compress results equal the oracle's streams,
  decompress results equal the oracle's decoding of the request's stream
  and lie within the tolerance of the original.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np
import pytest

from oracle.pyoracle import mode_params
from zfp_gb300 import capi, workloads

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


def oracle_code(oracle, a, mode, arg):
    """(stream words, end bit, params, block starts) of the oracle's compression of a."""
    prm = mode_params(mode, arg, a.dtype, a.ndim)
    words, end, ends = oracle.compress(a, prm, threads=THREADS, block_ends=True)
    starts = np.concatenate([[0], ends[:-1]]).astype(np.uint64)
    return words[: (end + 63) // 64], end, prm, starts


def oracle_decode(oracle, code, shape, dtype):
    words, end, prm, starts = code
    out = np.zeros(shape, dtype=dtype)
    fixed = prm[0] == prm[1] and prm[3] >= -1074
    oracle.decompress_par(words, out, prm, THREADS, block_start=None if fixed else starts)
    return out


def bind_batch(lib):
    L = lib.lib
    L.zfp_gb300_batch_create.restype = C.c_void_p
    L.zfp_gb300_batch_create.argtypes = [C.POINTER(capi.PZ), C.POINTER(capi.PF), C.c_size_t, C.c_int]
    L.zfp_gb300_batch_run.restype = C.c_int
    L.zfp_gb300_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    L.zfp_gb300_batch_finish.restype = C.c_int
    L.zfp_gb300_batch_finish.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
    L.zfp_gb300_batch_free.argtypes = [C.c_void_p]
    return L


def batch_pass(lib, L, arrays, bufs, ptrs, direction):
    zs, fs, keep = [], [], []
    for (x, mode, arg), buf, ptr in zip(arrays, bufs, ptrs):
        bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, mode, arg, capi.TYPE_FLOAT, 3)
        assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        fs.append(capi.make_field(lib, ptr, capi.TYPE_FLOAT, tuple(reversed(x.shape))))
        zs.append(z)
        keep.append(bs)
    b = L.zfp_gb300_batch_create((capi.PZ * len(zs))(*zs), (capi.PF * len(fs))(*fs), len(zs), direction)
    assert b, lib.zfp_gb300_last_error()
    sizes = (C.c_size_t * len(zs))()
    assert L.zfp_gb300_batch_run(b, None)
    assert L.zfp_gb300_batch_finish(b, sizes), lib.zfp_gb300_last_error()
    L.zfp_gb300_batch_free(b)
    for z, f, bs in zip(zs, fs, keep):
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
    return list(sizes)


def test_batch_workload_matches_oracle(lib, oracle, cuda):
    torch = cuda
    L = bind_batch(lib)
    arrays = workloads.batch_arrays(torch, 4096)
    host = [x.cpu().numpy() for x, _, _ in arrays]
    codes = [oracle_code(oracle, a, mode, arg) for a, (_, mode, arg) in zip(host, arrays)]
    bufs = [torch.zeros(len(c[0]) + 64, dtype=torch.int64, device="cuda") for c in codes]
    sizes = batch_pass(lib, L, arrays, bufs, [x.data_ptr() for x, _, _ in arrays], 0)
    for i, (code, buf, size) in enumerate(zip(codes, bufs, sizes)):
        words = code[0]
        assert size == len(words) * 8, (i, arrays[i][1:], tuple(arrays[i][0].shape))
        assert np.array_equal(buf[: len(words)].cpu().numpy().view(np.uint64), words), (i, arrays[i][1:])
    outs = [torch.empty_like(x) for x, _, _ in arrays]
    dsizes = batch_pass(lib, L, arrays, bufs, [o.data_ptr() for o in outs], 1)
    assert dsizes == sizes
    for i, (a, code, o) in enumerate(zip(host, codes, outs)):
        ref = oracle_decode(oracle, code, a.shape, a.dtype)
        assert np.array_equal(o.cpu().numpy().view(np.uint32), ref.view(np.uint32)), (i, arrays[i][1:])


def bind_server(lib):
    L = lib.lib
    L.zfp_gb300_server_create.restype = C.c_void_p
    L.zfp_gb300_server_create.argtypes = [C.c_size_t, C.c_int]
    L.zfp_gb300_server_submit.restype = C.c_uint64
    L.zfp_gb300_server_submit.argtypes = [C.c_void_p, capi.PZ, capi.PF, C.c_int]
    L.zfp_gb300_server_wait.restype = C.c_size_t
    L.zfp_gb300_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]
    L.zfp_gb300_server_free.argtypes = [C.c_void_p]
    return L


def test_serving_workload_sample_matches_oracle(lib, oracle, cuda):
    torch = cuda
    L = bind_server(lib)
    mix = workloads.ServingMix(torch, 200)
    host_bases = {k: v.cpu().numpy() for k, v in mix.bases.items()}

    def host_view(r):
        return host_bases[(r["esz"], r["dims"])][(slice(0, r["n"]),) * r["dims"]]

    def objects(r, buf, out_ptr=None):
        bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
        z = lib.zfp_stream_open(bs)
        zt = capi.TYPE_FLOAT if r["esz"] == 4 else capi.TYPE_DOUBLE
        assert lib.zfp_stream_set_accuracy(z, r["tol"]) > 0
        assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        v = r["view"]
        if out_ptr is None:
            f = capi.make_field(lib, v.data_ptr(), zt, tuple(reversed(v.shape)), tuple(reversed(v.stride())))
        else:
            f = capi.make_field(lib, out_ptr, zt, tuple(reversed(v.shape)))
        return bs, z, f

    # templates of the decompress requests: written by zfp_compress, checked against the oracle
    used = {r["template"] for r in mix.requests if r["direction"] == 1}
    tcode, tbuf = {}, {}
    for t in sorted(used):
        r = mix.templates[t]
        code = oracle_code(oracle, host_view(r), "accuracy", r["tol"])
        buf = torch.zeros(len(code[0]) + 64, dtype=torch.int64, device="cuda")
        bs, z, f = objects(r, buf)
        size = lib.zfp_compress(z, f)
        assert size == len(code[0]) * 8, lib.zfp_gb300_last_error()
        assert np.array_equal(buf[: len(code[0])].cpu().numpy().view(np.uint64), code[0])
        for obj, fn in ((f, lib.zfp_field_free), (z, lib.zfp_stream_close), (bs, lib.stream_close)):
            fn(obj)
        tcode[t], tbuf[t] = code, buf

    # the sample through one server, submitted on the benchmark's arrival schedule
    expect, objs, outs = [], [], []
    for r in mix.requests:
        if r["direction"] == 0:
            code = oracle_code(oracle, host_view(r), "accuracy", r["tol"])
            buf = torch.zeros(len(code[0]) + 64, dtype=torch.int64, device="cuda")
            objs.append(objects(r, buf))
            outs.append(buf)
            expect.append(code)
        else:
            out = torch.empty(tuple(r["view"].shape), dtype=r["view"].dtype, device="cuda")
            objs.append(objects(r, tbuf[r["template"]], out.data_ptr()))
            outs.append(out)
            expect.append(tcode[r["template"]])
    torch.cuda.synchronize()
    server = L.zfp_gb300_server_create(64 << 30, 4)
    assert server
    t0 = time.perf_counter()
    tickets = []
    for i, (r, (bs, z, f)) in enumerate(zip(mix.requests, objs)):
        delay = t0 + mix.arrivals[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        t = L.zfp_gb300_server_submit(server, z, f, r["direction"])
        assert t, lib.zfp_gb300_last_error()
        tickets.append(t)
    for i, (r, t, code, out) in enumerate(zip(mix.requests, tickets, expect, outs)):
        size = L.zfp_gb300_server_wait(server, t, None)
        assert size == len(code[0]) * 8, (i, r["direction"], lib.zfp_gb300_last_error())
        if r["direction"] == 0:
            assert np.array_equal(out[: len(code[0])].cpu().numpy().view(np.uint64), code[0]), f"request {i}"
        else:
            view = host_view(r)
            ref = oracle_decode(oracle, code, view.shape, view.dtype)
            got = out.cpu().numpy()
            bits = np.uint32 if view.dtype == np.float32 else np.uint64
            assert np.array_equal(got.view(bits), ref.view(bits)), f"request {i}: decode differs"
            assert np.max(np.abs(got.astype(np.float64) - view.astype(np.float64))) <= r["tol"], f"request {i}"
    L.zfp_gb300_server_free(server)
    for bs, z, f in objs:
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
