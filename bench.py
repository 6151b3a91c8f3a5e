#!/usr/bin/env python
"""Benchmark of the GB300 zfp block codec (libzfp_gb300.so) on the
configuration the reference's headline metric is quoted on: a 3D float32
512^3 smooth field (seed 1, N(0,1e-2) noise) in four modes -- fixed-rate 8,
fixed-precision 20, fixed-accuracy 1e-3, reversible -- and the same sweep on
a 3D float64 384^3 field.

One step = compress then decompress of both fields in all four modes,
device-resident, through the C ABI (zfp_compress / zfp_decompress,
zfp_exec_cuda).  value = raw bytes coded per second (both directions).
e2e = the same sweep with host (pinned) field and stream buffers, so the
host<->device copies are inside the timed region.  `--impl reference` times
the reference's own CPU codec (its library compiled from its sources:
OpenMP compress on all host cores, serial decompress -- the reference has
no OpenMP decompressor -- plus serial compress on one core) on a bounded
sample; `reference_cuda` times the reference's own CUDA backend on the same
fields at fixed rate 8 beside this library's kernels.
"""
from __future__ import annotations

import argparse
import ctypes as C
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

MODES = [("rate", 8.0), ("precision", 20), ("accuracy", 1e-3), ("reversible", None)]
FIELDS = [("f32", (512, 512, 512), 1), ("f64", (384, 384, 384), 1)]  # name, shape (z,y,x), seed
METRIC = "raw GB/s compress+decompress (bit-exact), 3D fp32 512^3 + fp64 384^3, 4 modes"
SMI_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--small", action="store_true", help="shrink the fields (smoke runs only)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-serve", action="store_true")
    p.add_argument("--no-refcuda", action="store_true")
    p.add_argument("--no-config3", action="store_true")
    p.add_argument("--only", default=None,
                   help="profiling: run one kernel, FIELD:MODE:DIR (e.g. f32:rate:c), --steps times")
    p.add_argument("--shape", default=None, help="profiling: field shape Z,Y,X for --only")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def job_ms(ms_local: float, world: int, device: str) -> float:
    """Length of the timed region of the whole job: the slowest rank's
    milliseconds (all-reduce MAX, then a barrier so no rank leaves early)."""
    if world <= 1:
        return ms_local
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_local], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_gbs(raw_bytes_per_step: int, steps: int, world: int, ms: float) -> float:
    """Whole-job throughput: every rank codes the same bytes per step (weak
    scaling), so the job moved world x steps x bytes in the slowest rank's time."""
    return world * raw_bytes_per_step * steps / (ms / 1e3) / 1e9


def field_shapes(small: bool):
    if not small:
        return FIELDS
    return [("f32", (64, 96, 128), 1), ("f64", (48, 64, 80), 1)]


# ---------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={SMI_QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """dram bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    out = {}
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith("#") or ":" not in ln:
                    continue
                k, v = ln.split(":", 1)
                out[k.strip()] = float(v.split()[0])
    except (OSError, ValueError):
        pass
    return out


# ---------------------------------------------------------------------------
# GPU arm

class GpuCodec:
    """Reusable zfp_stream/bitstream/field objects over fixed buffers."""

    def __init__(self, lib, torch, stream_handle):
        from zfp_gb300 import capi
        self.lib, self.torch, self.capi = lib, torch, capi
        self.stream_handle = stream_handle

    def run(self, direction, field_ptr, ztype, n, mode, arg, buf_ptr, buf_bytes, async_=True):
        lib, capi = self.lib, self.capi
        bs = lib.stream_open(buf_ptr, buf_bytes)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, mode, arg, ztype, 3)
        lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        lib.zfp_gb300_stream_set_cuda_stream(z, self.stream_handle)
        lib.zfp_gb300_stream_set_async(z, 1 if async_ else 0)
        f = capi.make_field(lib, field_ptr, ztype, n)
        r = lib.zfp_compress(z, f) if direction == "c" else lib.zfp_decompress(z, f)
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
        return r


def gpu_arm(args):
    import torch
    import torch.distributed as dist

    import zfp_gb300
    from zfp_gb300 import capi, synth

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = zfp_gb300.load()
    stream = torch.cuda.current_stream()
    codec = GpuCodec(lib, torch, stream.cuda_stream)

    fields = []
    for name, shape, seed in field_shapes(args.small):
        dt = torch.float32 if name == "f32" else torch.float64
        x = synth.smooth_field_torch(shape, dt, seed=seed, noise=1e-2)
        ztype = capi.TYPE_FLOAT if name == "f32" else capi.TYPE_DOUBLE
        n = tuple(reversed(shape))
        raw = x.numel() * x.element_size()
        # worst case stream (reversible) plus a little
        cap_words = (raw + 4096 * 64) // 8 + x.numel() // 8 + 1024
        bufs = {m: torch.zeros(cap_words, dtype=torch.int64, device="cuda") for m, _ in MODES}
        out = torch.empty_like(x)
        fields.append(dict(name=name, shape=shape, x=x, out=out, ztype=ztype, n=n, raw=raw, bufs=bufs,
                           cap=cap_words * 8, sizes={}))
    torch.cuda.synchronize()

    def one(fd, mode, arg, direction):
        buf = fd["bufs"][mode]
        ptr = fd["x"].data_ptr() if direction == "c" else fd["out"].data_ptr()
        r = codec.run(direction, ptr, fd["ztype"], fd["n"], mode, arg, buf.data_ptr(), fd["cap"])
        if not r:
            raise RuntimeError(f"{fd['name']} {mode} {direction} failed: {zfp_gb300.last_error()}")
        if direction == "c":
            fd["sizes"][mode] = r
        return r

    def step():
        for fd in fields:
            for mode, arg in MODES:
                one(fd, mode, arg, "c")
                one(fd, mode, arg, "d")

    # correctness gates on the full fields before timing
    step()
    torch.cuda.synchronize()
    checks = {}
    for fd in fields:
        for mode, arg in MODES:
            one(fd, mode, arg, "c")
            one(fd, mode, arg, "d")
            torch.cuda.synchronize()
            if mode == "reversible":
                ok = torch.equal(fd["x"].view(torch.int32 if fd["name"] == "f32" else torch.int64),
                                 fd["out"].view(torch.int32 if fd["name"] == "f32" else torch.int64))
                checks[f"{fd['name']}_reversible_bitwise"] = bool(ok)
            elif mode == "accuracy":
                err = (fd["x"].double() - fd["out"].double()).abs().max().item()
                checks[f"{fd['name']}_accuracy_maxerr"] = err
                checks[f"{fd['name']}_accuracy_ok"] = bool(err <= arg)
            elif mode == "rate":
                nblocks = np.prod([(s + 3) // 4 for s in fd["shape"]])
                bits = int(np.floor(64 * arg + 0.5))
                checks[f"{fd['name']}_rate_size_ok"] = bool(fd["sizes"][mode] == ((int(nblocks) * bits + 63) // 64) * 8)

    # per-kernel timing (roofline), each direction/mode alone
    per = []
    reps = max(3, args.steps)
    for fd in fields:
        for mode, arg in MODES:
            for direction in ("c", "d"):
                one(fd, mode, arg, direction)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    one(fd, mode, arg, direction)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                comp = fd["sizes"][mode]
                per.append(dict(field=fd["name"], mode=mode, dir="compress" if direction == "c" else "decompress",
                                ms=ms, raw_bytes=fd["raw"], stream_bytes=comp,
                                raw_gbs=fd["raw"] / ms / 1e6, hbm_gbs=(fd["raw"] + comp) / ms / 1e6))

    # timed steps
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms_total = job_ms(e0.elapsed_time(e1), world, "cuda")
    raw_step = sum(2 * fd["raw"] * len(MODES) for fd in fields)
    value = job_gbs(raw_step, args.steps, world, ms_total)
    launches = 2 * len(MODES) * len(fields) * args.steps

    # roofline of the dominant kernel
    peak, peak_kind = peak_hbm()
    dom = max(per, key=lambda r: r["ms"])
    traffic = ncu_traffic()
    key = f"{dom['field']}_{dom['mode']}_{dom['dir']}"
    roofline = {"bound": "hbm", "kernel": key, "achieved": round(dom["hbm_gbs"], 1), "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": round(dom["hbm_gbs"] / peak, 4),
                "traffic": traffic.get(key),
                "traffic_source": "profiles/traffic.txt: an earlier ncu capture of this kernel on the same field "
                                  "(dram__bytes_read.sum + dram__bytes_write.sum), not measured in this run"}
    fixed = [r for r in per if r["mode"] == "rate"]

    # the reference's own CUDA backend on the same fields (fixed rate 8)
    ref_cuda = None
    if not args.no_refcuda:
        ref_cuda = reference_cuda_column(fields, one, torch, reps)

    # the edge-shape configuration at full size
    cfg3 = None
    if not args.no_config3:
        torch.cuda.empty_cache()
        cfg3 = config3_timings(lib, torch, max(3, min(args.steps, 10)), stream.cuda_stream)

    # end to end: host pinned buffers through the same C API (synchronous calls)
    ratios = {f"{fd['name']}_{m}": round(fd["raw"] / fd["sizes"][m], 3) for fd in fields for m, _ in MODES}
    shapes = [list(fd["shape"]) for fd in fields]
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(lib, torch, codec, fields, args)
        link = e2e["host_link"] = host_link(torch)
        # each call against the link: its bytes at the copy engines' one-way
        # rates, overlapped, and at their rate both ways at once
        for c in e2e["per_call"]:
            one_way = max(c["h2d_bytes"] / link["h2d_gbs"], c["d2h_bytes"] / link["d2h_gbs"]) / 1e6
            both = (c["h2d_bytes"] + c["d2h_bytes"]) / link["bidirectional_gbs"] / 1e6
            c["link_bound_ms"] = round(max(one_way, both), 3)
            c["frac_of_link"] = round(c["link_bound_ms"] / c["ms"], 3) if c["ms"] else None

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(fields, args)

    batch = None
    if not args.no_batch:
        del fields
        torch.cuda.empty_cache()
        batch = batch_compare(lib, torch, stream, args)

    serving = None
    if not args.no_serve:
        torch.cuda.empty_cache()
        serving = {"at_6000_per_s": serve_compare(lib, torch, args, 20000, 6000.0)}
        torch.cuda.empty_cache()
        serving["saturating"] = serve_compare(lib, torch, args, 8000, 40000.0)

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_total / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 in, u64 stream", "data": "synthetic",
            "config": {"workload": "3D float32 512^3 + float64 384^3 smooth fields (8 sinusoids + N(0,1e-2)), "
                                   "modes rate 8 / precision 20 / accuracy 1e-3 / reversible, compress+decompress, "
                                   "device-resident", "l2": "inputs larger than L2 (no flush)",
                       "fields": shapes},
            "impl": "gb300", "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": launches,
            "fixed_rate": {f"{r['field']}_{r['dir']}": {"raw_gbs": round(r["raw_gbs"], 1),
                                                         "hbm_frac": round(r["hbm_gbs"] / peak, 4)} for r in fixed},
            "per_kernel": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()} for r in per],
            "reference_cuda": ref_cuda,
            "config3": cfg3,
            "checks": checks,
            "compression_ratio": ratios,
            "batch": batch,
            "serving": serving,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def bind_batch(lib):
    from zfp_gb300 import capi
    L = lib.lib
    L.zfp_gb300_batch_create.restype = C.c_void_p
    L.zfp_gb300_batch_create.argtypes = [C.POINTER(capi.PZ), C.POINTER(capi.PF), C.c_size_t, C.c_int]
    L.zfp_gb300_batch_run.restype = C.c_int
    L.zfp_gb300_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    L.zfp_gb300_batch_finish.restype = C.c_int
    L.zfp_gb300_batch_finish.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
    L.zfp_gb300_batch_free.argtypes = [C.c_void_p]
    L.zfp_gb300_batch_get_tuning.restype = C.c_int
    L.zfp_gb300_batch_get_tuning.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    return L


def batch_compare(lib, torch, stream, args):
    """4096 independent 3D float32 arrays, extents log-uniform in [8,128]
    (seed 2), amplitude scale 10^U(-3,3); half fixed-rate (rate in
    {4,8,12,16,24,32}), half fixed-accuracy (tolerance 10^U(-5,-2)).  One
    batched launch against one zfp_compress / zfp_decompress per array."""
    from zfp_gb300 import capi, workloads
    L = bind_batch(lib)
    count = 4096 if not args.small else 256
    arrays = workloads.batch_arrays(torch, count)
    from zfp_gb300 import build as zbuild
    loop = C.CDLL(zbuild.LOOP_LIB).zfp_gb300_loop_calls
    loop.restype = C.c_size_t
    loop.argtypes = [C.POINTER(capi.PZ), C.POINTER(capi.PF), C.c_size_t, C.c_int, C.c_int]
    raw = sum(x.numel() * 4 for x, _, _ in arrays)

    def objects(outs, bufs, use_out):
        zs, fs, keep = [], [], []
        for (x, mode, arg), o, buf in zip(arrays, outs, bufs):
            bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
            z = lib.zfp_stream_open(bs)
            capi.set_mode(lib, z, mode, arg, capi.TYPE_FLOAT, 3)
            lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
            lib.zfp_gb300_stream_set_cuda_stream(z, stream.cuda_stream)
            lib.zfp_gb300_stream_set_async(z, 1)
            f = capi.make_field(lib, (o if use_out else x).data_ptr(), capi.TYPE_FLOAT, tuple(reversed(x.shape)))
            zs.append(z)
            fs.append(f)
            keep.append(bs)
        return zs, fs, keep

    def close(zs, fs, keep):
        for z, f, bs in zip(zs, fs, keep):
            lib.zfp_field_free(f)
            lib.zfp_stream_close(z)
            lib.stream_close(bs)

    def buffers():
        out = []
        for x, mode, arg in arrays:
            z = lib.zfp_stream_open(None)
            capi.set_mode(lib, z, mode, arg, capi.TYPE_FLOAT, 3)
            f = capi.make_field(lib, 0, capi.TYPE_FLOAT, tuple(reversed(x.shape)))
            nbytes = lib.zfp_stream_maximum_size(z, f)
            lib.zfp_field_free(f)
            lib.zfp_stream_close(z)
            out.append(torch.zeros(nbytes // 8 + 8, dtype=torch.int64, device="cuda"))
        return out

    per_bufs, bat_bufs = buffers(), buffers()
    per_out = [torch.empty_like(x) for x, _, _ in arrays]
    bat_out = [torch.empty_like(x) for x, _, _ in arrays]
    reps = max(2, min(args.steps, 5))
    result = {"arrays": count, "raw_bytes": raw}
    for direction, name in ((0, "compress"), (1, "decompress")):
        # one zfp_compress / zfp_decompress call per array, from a C loop
        # over prebuilt objects (zfp_gb300/csrc/percall_loop.c)
        zs, fs, keep = objects(per_out, per_bufs, direction == 1)
        za, fa = (capi.PZ * count)(*zs), (capi.PF * count)(*fs)
        assert loop(za, fa, count, direction, 1) == 0, lib.zfp_gb300_last_error()   # warm-up, index lookups
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        failed = loop(za, fa, count, direction, reps)
        torch.cuda.synchronize()
        per_s = (time.perf_counter() - t0) / reps
        assert failed == 0
        close(zs, fs, keep)
        # one batched launch
        zs, fs, keep = objects(bat_out, bat_bufs, direction == 1)
        b = L.zfp_gb300_batch_create((capi.PZ * count)(*zs), (capi.PF * count)(*fs), count, direction)
        assert b, lib.zfp_gb300_last_error()
        sizes = (C.c_size_t * count)()
        assert L.zfp_gb300_batch_run(b, stream.cuda_stream)   # autotune + graph capture
        assert L.zfp_gb300_batch_finish(b, sizes)
        tc, tsp = C.c_int(), C.c_int()
        assert L.zfp_gb300_batch_get_tuning(b, C.byref(tc), C.byref(tsp))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            L.zfp_gb300_batch_run(b, stream.cuda_stream)
        torch.cuda.synchronize()
        bat_s = (time.perf_counter() - t0) / reps
        assert L.zfp_gb300_batch_finish(b, sizes)
        L.zfp_gb300_batch_free(b)
        close(zs, fs, keep)
        same = all(torch.equal(p, q) for p, q in zip(per_bufs, bat_bufs)) if direction == 0 else \
            all(torch.equal(p.view(torch.int32), q.view(torch.int32)) for p, q in zip(per_out, bat_out))
        result[name] = {"per_array_gbs": round(raw / per_s / 1e9, 2), "batched_gbs": round(raw / bat_s / 1e9, 2),
                        "speedup": round(per_s / bat_s, 2), "bit_identical": bool(same),
                        "tuned": {"ctas_per_sm": tc.value, "staging_pct": tsp.value},
                        "per_array_ms": round(per_s * 1e3, 3), "batched_ms": round(bat_s * 1e3, 3)}
    return result


def serve_compare(lib, torch, args, count=20000, rate=6000.0):
    """Configuration 5: a Poisson stream of requests (70% compress, 30%
    decompress), each a 2D or 3D float32/float64 field whose raw size is
    log-uniform in [16 KiB, 256 MiB] (smooth-field generator, seed 3),
    fixed-accuracy tolerance 1e-4 x the field's range.  Served by the
    continuous-batching server under a 64 GiB HBM budget, and by one worker
    calling zfp_compress / zfp_decompress per request on the same arrival
    schedule.  Fields are views of resident generated fields; decompress
    requests read streams compressed before the timed run."""
    import queue

    from zfp_gb300 import capi, workloads
    L = lib.lib
    L.zfp_gb300_server_create.restype = C.c_void_p
    L.zfp_gb300_server_create.argtypes = [C.c_size_t, C.c_int]
    L.zfp_gb300_server_submit.restype = C.c_uint64
    L.zfp_gb300_server_submit.argtypes = [C.c_void_p, capi.PZ, capi.PF, C.c_int]
    L.zfp_gb300_server_wait.restype = C.c_size_t
    L.zfp_gb300_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]
    L.zfp_gb300_server_free.argtypes = [C.c_void_p]
    if args.small:
        count, rate = min(count, 600), rate / 3
    smax = (256 << 20) if not args.small else (8 << 20)
    mix = workloads.ServingMix(torch, count, smax=smax, rate=rate)
    bases, templates, reqs, arrivals = mix.bases, mix.templates, mix.requests, mix.arrivals
    total_raw = sum(r["raw"] for r in reqs)

    def make_objects(r, buf_ptr, nbytes, out_ptr=None):
        bs = lib.stream_open(buf_ptr, nbytes)
        z = lib.zfp_stream_open(bs)
        zt = capi.TYPE_FLOAT if r["esz"] == 4 else capi.TYPE_DOUBLE
        lib.zfp_stream_set_accuracy(z, r["tol"])
        lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        v = r["view"]
        n = tuple(reversed(v.shape))
        st = tuple(reversed(v.stride()))
        f = capi.make_field(lib, out_ptr if out_ptr is not None else v.data_ptr(), zt, n,
                            st if out_ptr is None else ())
        return bs, z, f

    def max_bytes(r):
        bs, z, f = make_objects(r, 0, 0)
        m = lib.zfp_stream_maximum_size(z, f)
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
        return m

    # output buffers: a ring per direction (requests that share a slot overwrite each other's
    # output; only the timing of this experiment is measured, the parity test is separate)
    ring = 48 if not args.small else 16
    worst = max_bytes(max(reqs, key=lambda r: r["raw"])) + 4096
    cbufs = [torch.empty(worst // 8 + 8, dtype=torch.int64, device="cuda") for _ in range(ring)]
    outs = {k: [torch.empty_like(v) for _ in range(4)] for k, v in bases.items()}
    dstreams = []
    for r in templates:
        m = max_bytes(r)
        buf = torch.empty(m // 8 + 8, dtype=torch.int64, device="cuda")
        bs, z, f = make_objects(r, buf.data_ptr(), m)
        assert lib.zfp_compress(z, f)
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
        dstreams.append((buf, m))
    objs = []
    for i, r in enumerate(reqs):
        if r["direction"] == 0:
            buf = cbufs[i % ring]
            objs.append(make_objects(r, buf.data_ptr(), max_bytes(r)))
        else:
            buf, m = dstreams[r["template"]]
            out = outs[(r["esz"], r["dims"])][i % 4]
            objs.append(make_objects(r, buf.data_ptr(), m, out_ptr=out.data_ptr()))
    torch.cuda.synchronize()

    def run(submit_fn, wait_fn):
        lat = [0.0] * count
        q = queue.Queue()
        t0 = time.perf_counter() + 0.05

        def waiter():
            for _ in range(count):
                i, tk = q.get()
                lat[i] = wait_fn(i, tk)
        th = threading.Thread(target=waiter)
        th.start()
        for i in range(count):
            delay = t0 + arrivals[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            q.put((i, submit_fn(i)))
        th.join()
        return lat, time.perf_counter() - t0

    # continuous batching server
    server = L.zfp_gb300_server_create(64 << 30, 4)
    secs = C.c_double()

    def s_submit(i):
        bs, z, f = objs[i]
        lib.zfp_stream_rewind(z)
        return L.zfp_gb300_server_submit(server, z, f, reqs[i]["direction"])

    failed = []

    def s_wait(i, tk):
        if not tk or not L.zfp_gb300_server_wait(server, tk, C.byref(secs)):
            failed.append((i, zfp_gb300_last()))
            return float("nan")
        return secs.value

    # warm-up outside the schedule: one of every kind of request (direction,
    # type, dimensionality) through the server, so kernel loading and pool
    # growth are not timed
    kinds = {}
    for i, r in enumerate(reqs):
        kinds.setdefault((r["direction"], r["esz"], r["dims"]), i)
    for i in kinds.values():
        tk = s_submit(i)
        assert tk and L.zfp_gb300_server_wait(server, tk, C.byref(secs)), zfp_gb300_last()
        bs, z, f = objs[i]
        lib.zfp_stream_rewind(z)
        assert (lib.zfp_compress if reqs[i]["direction"] == 0 else lib.zfp_decompress)(z, f)
    torch.cuda.synchronize()

    lat_s, wall_s = run(s_submit, s_wait)
    L.zfp_gb300_server_stats.restype = C.c_int
    L.zfp_gb300_server_stats.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_uint64), C.c_void_p]
    pk, nb = C.c_size_t(), C.c_uint64()
    L.zfp_gb300_server_stats(server, C.byref(pk), C.byref(nb), None)
    server_peak, server_batches = pk.value, nb.value
    L.zfp_gb300_server_free(server)

    # per-request GPU path on the same schedule: one worker, one call per request
    work = queue.Queue()
    done_at = [0.0] * count

    def worker():
        while True:
            item = work.get()
            if item is None:
                return
            i = item
            bs, z, f = objs[i]
            lib.zfp_stream_rewind(z)
            fn = lib.zfp_compress if reqs[i]["direction"] == 0 else lib.zfp_decompress
            assert fn(z, f)
            done_at[i] = time.perf_counter()

    wth = threading.Thread(target=worker)
    wth.start()
    sub_at = [0.0] * count

    def p_submit(i):
        sub_at[i] = time.perf_counter()
        work.put(i)
        return i

    def p_wait(i, tk):
        while not done_at[i]:
            time.sleep(5e-5)
        return done_at[i] - sub_at[i]

    lat_p, wall_p = run(p_submit, p_wait)
    work.put(None)
    wth.join()
    for bs, z, f in objs:
        lib.zfp_field_free(f)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)

    def pct(a, q):
        return round(float(np.nanpercentile(np.array(a) * 1e3, q)), 3)
    return {"requests": count, "mean_rate_per_s": rate, "offered_gbs": round(total_raw / arrivals[-1] / 1e9, 1),
            "hbm_budget_gib": 64, "lanes": 4, "raw_bytes": total_raw,
            "latency": "arrival to result ready on the host: server, submission to the end of the request's GPU work "
                       "(host callback); per request, submission to the return of the synchronous call",
            "server_batches": server_batches, "server_peak_admitted_bytes": server_peak,
            "server": {"p50_ms": pct(lat_s, 50), "p99_ms": pct(lat_s, 99), "sustained_gbs": round(total_raw / wall_s / 1e9, 2),
                       "wall_s": round(wall_s, 3), "failed": len(failed),
                       "first_failure": failed[0][1] if failed else None},
            "per_request": {"p50_ms": pct(lat_p, 50), "p99_ms": pct(lat_p, 99),
                            "sustained_gbs": round(total_raw / wall_p / 1e9, 2), "wall_s": round(wall_p, 3)}}


def zfp_gb300_last():
    import zfp_gb300
    return zfp_gb300.last_error()


def config3_timings(lib, torch, reps, stream_handle):
    """The edge-shape configuration at full size, each case compressed and
    decompressed alone on the device (CUDA events, `reps` calls): (a) 2D
    float64 16384^2, (b) 4D float32 64^4, (c) 3D float32 383x257x129, (d) the
    transposed strided view of (c) with strides (257*129, 1, 257), in fixed
    rate 12 and fixed precision 24; (e) 3D int32 256^3 uniform in
    [-2^20, 2^20), reversible.  Raw GB/s and (raw + stream) bytes per second
    against the HBM peak."""
    from zfp_gb300 import capi, synth
    peak, _ = peak_hbm()
    stream = torch.cuda.current_stream()
    cases = []
    c = synth.smooth_field_torch((129, 257, 383), torch.float32, seed=4, noise=1e-2)
    mem = c.permute(2, 0, 1).contiguous()          # memory order x (slowest), z, y (fastest)
    view = mem.as_strided((129, 257, 383), (257, 1, 257 * 129))
    for mode, arg in (("rate", 12), ("precision", 24)):
        cases.append(("b_4d_f32_64^4", lambda: synth.smooth_field_torch((64, 64, 64, 64), torch.float32, seed=3,
                                                                         noise=1e-2), mode, arg))
        cases.append(("c_3d_f32_383x257x129", lambda: c, mode, arg))
        cases.append(("d_strided_view_of_c", lambda: view, mode, arg))
        cases.append(("a_2d_f64_16384^2", lambda: synth.smooth_field_torch((16384, 16384), torch.float64, seed=5,
                                                                            noise=1e-2), mode, arg))
    cases.append(("e_3d_i32_256^3", lambda: torch.randint(-(1 << 20), 1 << 20, (256, 256, 256), dtype=torch.int32,
                                                           device="cuda", generator=torch.Generator(device="cuda")
                                                           .manual_seed(3)), "reversible", None))
    out = []
    for name, make, mode, arg in cases:
        x = make()
        ztype = {torch.float32: capi.TYPE_FLOAT, torch.float64: capi.TYPE_DOUBLE, torch.int32: capi.TYPE_INT32}[x.dtype]
        n, st = tuple(reversed(x.shape)), tuple(reversed(x.stride()))
        raw = x.numel() * x.element_size()
        y = torch.empty(x.shape, dtype=x.dtype, device="cuda")
        cap = raw * 2 + (1 << 20)
        buf = torch.zeros(cap // 8, dtype=torch.int64, device="cuda")
        bs = lib.stream_open(buf.data_ptr(), cap)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, mode, arg, ztype, x.dim())
        lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
        lib.zfp_gb300_stream_set_cuda_stream(z, stream_handle)
        fc = capi.make_field(lib, x.data_ptr(), ztype, n, st)
        fd = capi.make_field(lib, y.data_ptr(), ztype, n, st)   # same strides: the decoded view lands the same way
        row = {"case": name, "mode": mode, "arg": arg, "raw_bytes": raw}
        size = 0
        for direction, f in (("compress", fc), ("decompress", fd)):
            fn = lib.zfp_compress if direction == "compress" else lib.zfp_decompress
            lib.zfp_stream_rewind(z)
            size = fn(z, f)
            assert size, f"{name} {mode} {direction}: {zfp_gb300_last()}"
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                lib.zfp_stream_rewind(z)
                fn(z, f)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            row[direction] = {"ms": round(ms, 4), "raw_gbs": round(raw / ms / 1e6, 1),
                              "hbm_frac": round((raw + size) / ms / 1e6 / peak, 4)}
        row["stream_bytes"] = size
        if mode == "reversible":
            row["lossless"] = bool(torch.equal(x, y))
        lib.zfp_field_free(fc)
        lib.zfp_field_free(fd)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
        out.append(row)
        del x, y, buf
    return out


def host_link(torch, nbytes=1 << 30, reps=5):
    """Copy-engine bandwidth between pinned host memory and HBM (the ceiling
    of the e2e measurement, whose calls read and write pinned buffers over
    the same link): host-to-device, device-to-host, and both at once on two
    CUDA streams.  CUDA events, best of `reps`."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn):
        best = 1e30
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    def both():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    t_h2d = timed(lambda: d.copy_(h, non_blocking=True))
    t_d2h = timed(lambda: h2.copy_(d2, non_blocking=True))
    t_both = timed(both)
    return {"bytes": nbytes, "h2d_gbs": round(nbytes / t_h2d / 1e9, 1), "d2h_gbs": round(nbytes / t_d2h / 1e9, 1),
            "bidirectional_gbs": round(2 * nbytes / t_both / 1e9, 1),
            "how": "pinned host <-> device copies of 1 GiB (torch copy_ on the copy engines), best of 5"}


def e2e_run(lib, torch, codec, fields, args):
    """Same sweep, host pinned field and stream buffers: every call uploads
    its input and downloads its result inside the timed region."""
    hosts = []
    for fd in fields:
        hx = torch.empty(fd["x"].shape, dtype=fd["x"].dtype, pin_memory=True)
        hx.copy_(fd["x"])
        hout = torch.empty_like(hx, pin_memory=True)
        hbuf = torch.zeros(fd["cap"] // 8, dtype=torch.int64, pin_memory=True)
        hosts.append((fd, hx, hout, hbuf))
    h2d = d2h = 0
    sizes = {}
    staged = [0]
    calls = {}   # (field, mode, direction) -> fastest call in seconds (the calls are synchronous)

    def call(fd, direction, ptr, mode, arg, hbuf):
        t0 = time.perf_counter()
        r = codec.run(direction, ptr, fd["ztype"], fd["n"], mode, arg, hbuf.data_ptr(), fd["cap"], async_=False)
        dt = time.perf_counter() - t0
        key = (fd["name"], mode, direction)
        calls[key] = min(calls.get(key, 1e30), dt)
        staged[0] += lib.zfp_gb300_last_staged_bytes()
        return r

    def step():
        staged[0] = 0
        for fd, hx, hout, hbuf in hosts:
            for mode, arg in MODES:
                r = call(fd, "c", hx.data_ptr(), mode, arg, hbuf)
                r2 = call(fd, "d", hout.data_ptr(), mode, arg, hbuf)
                if not r or r2 != r:
                    raise RuntimeError(f"e2e {fd['name']} {mode} failed")
                sizes[(fd["name"], mode)] = r

    step()
    torch.cuda.synchronize()
    calls.clear()
    n = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(n):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    raw_step = sum(2 * fd["raw"] * len(MODES) for fd in fields)
    for fd in fields:
        for mode, _ in MODES:
            h2d += fd["raw"] + sizes[(fd["name"], mode)]
            d2h += fd["raw"] + sizes[(fd["name"], mode)]
    _, world, _ = dist_info()
    per_call = []
    for fd in fields:
        for mode, _ in MODES:
            size = sizes[(fd["name"], mode)]
            for direction in ("c", "d"):
                per_call.append({"field": fd["name"], "mode": mode, "dir": direction,
                                 "ms": round(calls[(fd["name"], mode, direction)] * 1e3, 3),
                                 "h2d_bytes": fd["raw"] if direction == "c" else size,
                                 "d2h_bytes": size if direction == "c" else fd["raw"]})
    return {"value": round(world * raw_step * n / dt / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": n, "per_call": per_call,
            "buffers": "pinned host field and stream, read and written in place by the kernels over the host link, "
                       "except streams whose decode tiles outgrow shared memory, uploaded once (staged_bytes_per_step); "
                       "h2d/d2h = bytes crossing the link", "staged_bytes_per_step": staged[0]}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's own CPU codec (the library compiled from its
# sources by oracle/Makefile), driven through its public C API; the oracle
# port of it only where the reference could not be compiled

REF_CPU_LIB = os.path.join(ROOT, "oracle", "_ref", "libzfp_ref.so")
REF_CUDA_LIB = os.path.join(ROOT, "baseline", "_ref", "libzfp_refcuda.so")
CPU_SAMPLE_PLANES = {"f32": 16, "f64": 12}


def cpu_sample(fields_spec, small):
    """A bounded sample of each field: its first z-planes (same generator, same seed)."""
    from zfp_gb300 import synth
    out = []
    for name, shape, seed in fields_spec:
        dt = np.float32 if name == "f32" else np.float64
        planes = min(shape[0], CPU_SAMPLE_PLANES[name] if not small else 8)
        sub = (planes, shape[1], shape[2])
        out.append((name, sub, synth.smooth_field(sub, dt, seed=seed, noise=1e-2)))
    return out


def ref_cpu_lib():
    """The reference library, built from its own sources (None if it could not be built here)."""
    if not os.path.exists(REF_CPU_LIB):
        return None
    from zfp_gb300 import capi
    return capi.ZfpLib(REF_CPU_LIB)


def ref_cpu_measure(lib, samples, threads, reps=1):
    """Per mode and sample field, through the reference's zfp_compress /
    zfp_decompress: serial compress (1 core), OpenMP compress (`threads`
    cores; its stream must equal the serial one) and serial decompress (the
    reference has no OpenMP decompressor, src/zfp.c:1137-1138).  Returns raw
    bytes per direction and the three times in seconds."""
    from zfp_gb300 import capi
    raw = 0
    t_ser = t_omp = t_dec = 0.0
    for _ in range(reps):
        for name, sub, a in samples:
            ztype = capi.TYPE_FLOAT if a.dtype == np.float32 else capi.TYPE_DOUBLE
            n = tuple(reversed(a.shape))
            for mode, arg in MODES:
                z = lib.zfp_stream_open(None)
                capi.set_mode(lib, z, mode, arg, ztype, 3)
                f = capi.make_field(lib, a.ctypes.data, ztype, n)
                cap = lib.zfp_stream_maximum_size(z, f)
                streams = []
                for policy in (capi.EXEC_SERIAL, capi.EXEC_OMP):
                    buf = np.zeros(cap // 8 + 1, dtype=np.uint64)
                    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
                    lib.zfp_stream_set_bit_stream(z, bs)
                    if policy == capi.EXEC_OMP:
                        assert lib.zfp_stream_set_omp_threads(z, threads)
                    else:
                        assert lib.zfp_stream_set_execution(z, capi.EXEC_SERIAL)
                    lib.zfp_stream_rewind(z)
                    t0 = time.perf_counter()
                    size = lib.zfp_compress(z, f)
                    dt = time.perf_counter() - t0
                    assert size, f"reference compress failed ({name} {mode})"
                    if policy == capi.EXEC_OMP:
                        t_omp += dt
                    else:
                        t_ser += dt
                    streams.append((buf, size, bs))
                (b0, s0, bs0), (b1, s1, bs1) = streams
                assert s0 == s1 and np.array_equal(b0[: s0 // 8], b1[: s1 // 8]), "OpenMP stream differs from serial"
                out = np.empty_like(a)
                lib.zfp_field_set_pointer(f, out.ctypes.data)
                assert lib.zfp_stream_set_execution(z, capi.EXEC_SERIAL)
                lib.zfp_stream_set_bit_stream(z, bs0)
                lib.zfp_stream_rewind(z)
                t0 = time.perf_counter()
                assert lib.zfp_decompress(z, f) == s0
                t_dec += time.perf_counter() - t0
                raw += a.nbytes
                lib.zfp_field_free(f)
                lib.zfp_stream_close(z)
                lib.stream_close(bs0)
                lib.stream_close(bs1)
    return raw, t_ser, t_omp, t_dec


def port_measure(samples, threads, reps=1):
    """The oracle port (a C restatement of the reference's serial codec), only
    where the reference itself could not be compiled."""
    from oracle.pyoracle import Oracle, mode_params
    orc = Oracle()
    raw = 0
    t_c = t_d = 0.0
    for _ in range(reps):
        for name, sub, a in samples:
            for mode, arg in MODES:
                prm = mode_params(mode, arg, a.dtype, 3)
                t0 = time.perf_counter()
                words, end = orc.compress(a, prm, threads=threads)
                t1 = time.perf_counter()
                out = np.empty_like(a)
                orc.decompress(words[: (end + 63) // 64], out, prm)
                t2 = time.perf_counter()
                t_c += t1 - t0
                t_d += t2 - t1
                raw += a.nbytes
    return raw, t_c, t_d


def sample_text(samples):
    return ", ".join(f"{n} {list(s)}" for n, s, _ in samples)


def cpu_columns(samples, threads, reps, warm=True):
    """The baseline's value (GB/s of raw bytes, compress + decompress, each
    direction on the reference's fastest CPU path: OpenMP compress, serial
    decompress) and its columns."""
    lib = ref_cpu_lib()
    if lib is not None:
        if warm:
            ref_cpu_measure(lib, samples, threads)
        raw, t_ser, t_omp, t_dec = ref_cpu_measure(lib, samples, threads, reps)
        return {"value": round(2 * raw / (t_omp + t_dec) / 1e9, 4), "unit": "GB/s", "cores": threads,
                "kind": "reference",
                "sample": "the reference library (its own sources, compiled by oracle/Makefile) through "
                          "zfp_compress / zfp_decompress, 4 modes, over the first z-planes of each field: "
                          + sample_text(samples),
                "serial_compress_gbs_1core": round(raw / t_ser / 1e9, 4),
                "omp_compress_gbs": round(raw / t_omp / 1e9, 4), "omp_threads": threads,
                "serial_decompress_gbs_1core": round(raw / t_dec / 1e9, 4),
                "omp_decompress": "none in the reference (src/zfp.c:1137-1138)"}, (t_omp + t_dec)
    if warm:
        port_measure(samples, threads)
    raw, t_c, t_d = port_measure(samples, threads, reps)
    return {"value": round(2 * raw / (t_c + t_d) / 1e9, 4), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "oracle port (the reference library could not be compiled here): OpenMP compress, serial "
                      "decompress, over the first z-planes of each field: " + sample_text(samples),
            "compress_gbs": round(raw / t_c / 1e9, 4), "decompress_gbs": round(raw / t_d / 1e9, 4)}, (t_c + t_d)


def cpu_baseline(fields, args):
    spec = [(fd["name"], fd["shape"], 1) for fd in fields]
    samples = cpu_sample(spec, args.small)
    threads = os.cpu_count() or 1
    cols, _ = cpu_columns(samples, threads, reps=12 if not args.small else 1)
    return cols


def reference_arm(args):
    """The reference's own CPU implementation of the path on this host's
    cores, on the same fields and modes (a bounded sample per step)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    samples = cpu_sample(field_shapes(args.small), args.small)
    threads = os.cpu_count() or 1
    for _ in range(max(0, args.warmup - 1)):
        cpu_columns(samples, threads, 1, warm=False)
    cols, secs = cpu_columns(samples, threads, args.steps)
    value = cols["value"]
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(secs * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 in, u64 stream",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "same fields and modes, bounded sample per step (first z-planes): "
                                   + sample_text(samples)},
            "cpu_baseline": cols,
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def reference_cuda_column(fields, codec_one, torch, reps):
    """The reference's own CUDA backend (src/cuda_zfp, compiled for sm_103a by
    oracle/Makefile into baseline/_ref) on the same fields at fixed rate 8,
    the only mode and dimensionality range it supports (1-3D, fixed rate),
    through zfp_compress / zfp_decompress with device-resident field and
    stream, timed with CUDA events on the stream it uses (the legacy
    default stream) like this library's kernels.  Its streams and decoded
    arrays are checked against this library's."""
    if not os.path.exists(REF_CUDA_LIB):
        return {"unavailable": "the reference's CUDA backend was not built (no reference sources here)"}
    from zfp_gb300 import capi
    lib = capi.ZfpLib(REF_CUDA_LIB)
    out = {}
    legacy = torch.cuda.default_stream()
    for fd in fields:
        ztype, n = fd["ztype"], fd["n"]
        z = lib.zfp_stream_open(None)
        capi.set_mode(lib, z, "rate", 8.0, ztype, 3)
        if not lib.zfp_stream_set_execution(z, capi.EXEC_CUDA):
            return {"unavailable": "the reference library was built without its CUDA backend"}
        f = capi.make_field(lib, fd["x"].data_ptr(), ztype, n)
        cap = lib.zfp_stream_maximum_size(z, f)
        buf = torch.zeros(cap // 8 + 8, dtype=torch.int64, device="cuda")
        bs = lib.stream_open(buf.data_ptr(), buf.numel() * 8)
        lib.zfp_stream_set_bit_stream(z, bs)
        size = lib.zfp_compress(z, f)
        torch.cuda.synchronize()
        mine = codec_one(fd, "rate", 8.0, "c")
        torch.cuda.synchronize()
        same_stream = size == mine and torch.equal(buf[: size // 8], fd["bufs"]["rate"][: size // 8])
        # decode both streams; the arrays must agree
        codec_one(fd, "rate", 8.0, "d")
        torch.cuda.synchronize()
        my_out = fd["out"].clone()
        rout = torch.empty_like(fd["x"])
        fo = capi.make_field(lib, rout.data_ptr(), ztype, n)
        lib.zfp_stream_rewind(z)
        dsize = lib.zfp_decompress(z, fo)
        torch.cuda.synchronize()
        bits = torch.int32 if fd["name"] == "f32" else torch.int64
        same_out = dsize == size and torch.equal(rout.view(bits), my_out.view(bits))
        res = {"stream_bytes": int(size), "stream_equal": bool(same_stream), "decoded_equal": bool(same_out)}
        for direction, fld in (("compress", f), ("decompress", fo)):
            fn = lib.zfp_compress if direction == "compress" else lib.zfp_decompress
            for _ in range(2):
                lib.zfp_stream_rewind(z)
                fn(z, fld)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(legacy)
            for _ in range(reps):
                lib.zfp_stream_rewind(z)
                fn(z, fld)
            e1.record(legacy)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            res[direction] = {"ms": round(ms, 4), "raw_gbs": round(fd["raw"] / ms / 1e6, 1),
                              "hbm_gbs": round((fd["raw"] + size) / ms / 1e6, 1)}
        lib.zfp_field_free(f)
        lib.zfp_field_free(fo)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)
        out[f"{fd['name']}_rate8"] = res
    return out


def profile_one(args):
    """One kernel on one field, for ncu: field and stream stay on the device."""
    import torch

    import zfp_gb300
    from zfp_gb300 import capi, synth

    name, mode, direction = args.only.split(":")
    arg = dict(MODES)[mode]
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else dict(
        (f, s) for f, s, _ in FIELDS)[name]
    torch.cuda.set_device(0)
    lib = zfp_gb300.load()
    codec = GpuCodec(lib, torch, torch.cuda.current_stream().cuda_stream)
    dt = torch.float32 if name == "f32" else torch.float64
    x = synth.smooth_field_torch(shape, dt, seed=1, noise=1e-2)
    out = torch.empty_like(x)
    ztype = capi.TYPE_FLOAT if name == "f32" else capi.TYPE_DOUBLE
    n = tuple(reversed(shape))
    cap = x.numel() * x.element_size() * 5 // 4 + (1 << 20)
    buf = torch.zeros(cap // 8, dtype=torch.int64, device="cuda")
    size = codec.run("c", x.data_ptr(), ztype, n, mode, arg, buf.data_ptr(), cap, async_=False)
    assert size, zfp_gb300.last_error()
    for _ in range(args.steps):
        ptr = x.data_ptr() if direction == "c" else out.data_ptr()
        assert codec.run(direction, ptr, ztype, n, mode, arg, buf.data_ptr(), cap, async_=False)
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.only, "shape": list(shape), "stream_bytes": size,
                      "raw_bytes": x.numel() * x.element_size()}))


def main():
    faulthandler.enable()
    args = parse_args()
    if args.only:
        profile_one(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
