"""The GPU block codec (zfp_gb300/csrc/codec.cuh) compiled for the host and
run block by block on the CPU, compared with the oracle.  This checks the
per-block logic of the kernels -- transforms, bit-plane transpose, group
testing, budgets, reversible mode, special values -- without a GPU."""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle.pyoracle import ZTYPE, mode_params

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "host_codec.cu")
OUT = os.path.join(HERE, "native", "_build", "libhostcodec.so")


@pytest.fixture(scope="module")
def host():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    deps = [SRC] + [os.path.join(HERE, "..", "zfp_gb300", "csrc", f) for f in ("codec.cuh", "kernels.cuh", "launch.h", "job.h")]
    if not os.path.exists(OUT) or any(os.path.getmtime(d) > os.path.getmtime(OUT) for d in deps):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        subprocess.run([nvcc, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC", "-o", OUT, SRC], check=True)
    lib = C.CDLL(OUT)
    lib.zgh_compress.restype = C.c_uint64
    lib.zgh_decompress.restype = C.c_uint64
    return lib


def _geom(a):
    n = list(reversed(a.shape))
    s = [st // a.itemsize for st in reversed(a.strides)]
    d = len(n)
    return d, (C.c_size_t * 4)(*(n + [0] * (4 - d))), (C.c_ssize_t * 4)(*(s + [0] * (4 - d)))


def host_compress(h, oracle, a, prm, bit0=0):
    d, n, s = _geom(a)
    words = np.zeros(oracle.max_words(tuple(reversed(a.shape)), a.dtype, prm) + 8 + (bit0 >> 6), dtype=np.uint64)
    p = (C.c_uint * 4)(*[v & 0xffffffff for v in prm])
    end = h.zgh_compress(ZTYPE[a.dtype], d, n, s, C.c_void_p(a.ctypes.data), p, C.c_void_p(words.ctypes.data),
                         C.c_uint64(bit0))
    return words, end


def host_decompress(h, words, out, prm, bit0=0):
    d, n, s = _geom(out)
    p = (C.c_uint * 4)(*[v & 0xffffffff for v in prm])
    return h.zgh_decompress(ZTYPE[out.dtype], d, n, s, C.c_void_p(out.ctypes.data), p,
                            C.c_void_p(words.ctypes.data), C.c_uint64(len(words)), C.c_uint64(bit0))


SPECIAL = {np.float32: np.array([0.0, -0.0, 1e-45, -1e-45, 1e-40, 3.4e38, -3.4e38, np.inf, -np.inf, np.nan, 1.0,
                                 -2.5, 1e-30, 1e-39], dtype=np.float32),
           np.float64: np.array([0.0, -0.0, 5e-324, -5e-324, 1e-310, 1.7e308, -1.7e308, np.inf, -np.inf, np.nan,
                                 1.0, -2.5, 1e-300, 1e-290])}


@pytest.mark.parametrize("coder", ["per_event", "table"])
@pytest.mark.parametrize("dims", [1, 2, 3, 4])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64], ids=lambda d: np.dtype(d).name)
def test_device_codec_on_host_matches_oracle(host, oracle, dims, dtype, coder):
    """Both plane coders of codec.cuh: emit_block (one put per significance
    event) and emit_block_seq (group-test codes a byte at a time from a
    table, used by the encoder kernel for 1-3D blocks)."""
    host.zgh_set_coder(1 if coder == "table" else 0)
    rng = np.random.default_rng(dims * 10 + ZTYPE[np.dtype(dtype)])
    modes = [("rate", 4), ("rate", 12.5), ("rate", 1), ("precision", 7), ("precision", 20), ("accuracy", 1e-3),
             ("accuracy", 1e-9), ("reversible", None), ("rate", 32), ("precision", 64), ("expert", (30, 70, 33, -5))]
    for mode, arg in modes:
        if mode == "accuracy" and np.dtype(dtype).kind == "i":
            continue
        for trial in range(4):
            shape = tuple(int(v) for v in rng.integers(1, {1: 40, 2: 14, 3: 9, 4: 7}[dims], size=dims))
            if np.dtype(dtype).kind == "f":
                a = (np.cumsum(rng.standard_normal(shape), axis=-1) * 10.0 ** rng.uniform(-5, 5)).astype(dtype)
                if trial == 3:
                    a = rng.choice(SPECIAL[dtype], size=shape).astype(dtype)
            else:
                bits = 30 if dtype == np.int32 else 60
                a = rng.integers(-(1 << bits), 1 << bits, size=shape, dtype=dtype)
            view = a[(slice(None, None, -1),) * dims] if trial == 1 else (
                np.swapaxes(a, 0, dims - 1) if trial == 2 and dims >= 2 else a)
            prm = mode_params(mode, arg, dtype, dims)
            bit0 = int(rng.integers(0, 200)) if trial == 2 else 0
            w0, e0 = oracle.compress(view, prm, bit0=bit0)
            w1, e1 = host_compress(host, oracle, view, prm, bit0)
            nw = (e0 + 63) // 64
            assert e0 == e1 and np.array_equal(w0[:nw], w1[:nw]), (mode, arg, shape, trial)
            assert not host.zgh_unclean_put(), ("a sink received bits above its length", mode, arg, shape)
            assert not host.zgh_or_overrun(), ("bits written past the block's length", mode, arg, shape)
            assert not host.zgh_floor_touched(), ("a plane below P - maxprec was written", mode, arg, shape)
            d0 = np.zeros(view.shape, dtype=dtype)
            d1 = np.zeros(view.shape, dtype=dtype)
            x0 = oracle.decompress(w0[: nw + 2], d0, prm, bit0)
            x1 = host_decompress(host, w0[: nw + 2].copy(), d1, prm, bit0)
            assert x0 == x1 and np.array_equal(d0.view(np.uint8), d1.view(np.uint8)), (mode, arg, shape, trial)
            assert not host.zgh_floor_touched(), ("a plane below P - maxprec was written", mode, arg, shape)


def test_integer_casts_match_fp64_arithmetic(host):
    """int_scale / scale_trunc (the double-precision casts done on integer
    pipes) against numpy's IEEE multiply, over their whole valid range."""
    rng = np.random.default_rng(11)
    host.zgh_int_scale.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p]
    host.zgh_scale_trunc.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p]
    n = 20000
    for e in [-1022, -1000, -500, -62, -1, 0, 7, 500, 960]:
        bits = rng.integers(0, 64, size=n)
        v = (rng.integers(0, 2**62, size=n, dtype=np.int64) >> (62 - np.minimum(bits, 62))).astype(np.int64)
        v = np.where(rng.random(n) < 0.5, -v, v)
        v[:8] = [0, 1, -1, 2**53 + 1, -(2**53 + 3), 2**62 + 1023, -(2**63), 2**63 - 1]
        out = np.zeros(n, dtype=np.uint64)
        host.zgh_int_scale(v.ctypes.data, n, e, out.ctypes.data)
        want = (v.astype(np.float64) * np.ldexp(1.0, e)).view(np.uint64)
        assert np.array_equal(out, want), e
    for emax in [-960, -900, -1, 0, 1, 100, 1023, 1024]:
        se = 62 - emax
        with np.errstate(over="ignore"):
            x = np.ldexp(rng.uniform(-1, 1, size=n), emax)
            x[:6] = [0.0, -0.0, np.ldexp(1.0, emax - 1), -np.ldexp(0.75, emax), 5e-324, -2.2e-308]
            x = np.where(np.abs(x) < np.ldexp(1.0, emax), x, 0.0)
        out = np.zeros(n, dtype=np.int64)
        host.zgh_scale_trunc(x.ctypes.data, n, se, out.ctypes.data)
        with np.errstate(over="ignore"):
            want = np.trunc(x * np.ldexp(1.0, se)).astype(np.int64)
        assert np.array_equal(out, want), emax


def test_bfp_exactness_shortcut(host):
    """bfp_exact's integer test agrees with casting each value and back."""
    rng = np.random.default_rng(12)
    host.zgh_bfp_exact64.argtypes = [C.c_void_p, C.c_int, C.c_int]
    host.zgh_bfp_exact32.argtypes = [C.c_void_p, C.c_int, C.c_int]
    for dtype, fn, P, I in [(np.float64, host.zgh_bfp_exact64, 64, np.int64),
                            (np.float32, host.zgh_bfp_exact32, 32, np.int32)]:
        seen = set()
        for trial in range(3000):
            emax = int(rng.integers(-1000 if dtype == np.float64 else -140, 60))
            k = int(rng.integers(0, P + 4))
            vals = np.ldexp(np.floor(rng.uniform(-1, 1, 64) * 2.0 ** k), emax - k).astype(dtype)
            if trial % 5 == 0:
                vals[rng.integers(0, 64)] = -0.0
            vals[0] = np.ldexp(0.5, emax) if trial % 3 else vals[0]
            vals = np.where(np.abs(vals) < np.ldexp(1.0, emax), vals, 0).astype(dtype)
            if not vals.any():
                continue
            em = int(np.max(np.frexp(vals.astype(np.float64))[1]))
            raw = vals.view(np.uint64 if dtype == np.float64 else np.uint32).copy()
            with np.errstate(over="ignore", under="ignore", invalid="ignore"):
                s = np.ldexp(dtype(1), P - 2 - em) if P - 2 - em <= (1023 if P == 64 else 127) else dtype(np.inf)
                prod = (vals * s).astype(dtype)
                ok = np.abs(prod) < 2.0 ** (P - 1)
                iv = np.where(ok, np.trunc(np.where(ok, prod, 0)), -(2.0 ** (P - 1))).astype(I)
                back = (iv.astype(dtype) * dtype(np.ldexp(1.0, em - (P - 2)))).astype(dtype)
            want = bool(np.array_equal(back.view(raw.dtype), raw))
            got = bool(fn(raw.ctypes.data, em, 0))
            assert got == want, (dtype, em, trial)
            seen.add(want)
        assert seen == {True, False}


def test_shared_memory_image_layout(host):
    """Tile images keep a spare word after every 16 (bank spreading); a buffer
    sized for L logical words holds them all, and nothing maps past its end."""
    assert host.zgh_image_layout_ok(C.c_uint32(200000))


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64], ids=lambda d: np.dtype(d).name)
def test_length_only_parse_matches_oracle_block_ends(host, oracle, dims, dtype):
    """skip_block (the GPU parse of streams without an index) ends every
    block exactly where the oracle's encoder ended it, in every mode."""
    rng = np.random.default_rng(100 + dims)
    modes = [("rate", 4), ("rate", 12.5), ("precision", 9), ("precision", 40), ("accuracy", 1e-3),
             ("accuracy", 1e-9), ("reversible", None), ("expert", (30, 70, 33, -5)), ("expert", (64, 900, 64, -30))]
    for mode, arg in modes:
        if mode == "accuracy" and np.dtype(dtype).kind == "i":
            continue
        shape = tuple(int(v) for v in rng.integers(1, {1: 60, 2: 17, 3: 10, 4: 7}[dims], size=dims))
        if np.dtype(dtype).kind == "f":
            a = (np.cumsum(rng.standard_normal(shape), axis=-1) * 10.0 ** rng.uniform(-5, 5)).astype(dtype)
            a.flat[:: max(1, a.size // 7)] = 0
        else:
            a = rng.integers(-(1 << 20), 1 << 20, size=shape, dtype=dtype)
        prm = mode_params(mode, arg, dtype, dims)
        bit0 = int(rng.integers(0, 100))
        words, end, be = oracle.compress(a, prm, bit0=bit0, block_ends=True)
        n = (C.c_size_t * 4)(*(list(reversed(a.shape)) + [0] * (4 - dims)))
        p = (C.c_uint * 4)(*[v & 0xffffffff for v in prm])
        ends = np.zeros(len(be), dtype=np.uint64)
        host.zgh_parse.restype = C.c_uint64
        got = host.zgh_parse(ZTYPE[np.dtype(dtype)], dims, n, p, C.c_void_p(words.ctypes.data),
                             C.c_uint64(len(words)), C.c_uint64(bit0), C.c_void_p(ends.ctypes.data))
        assert got == end and np.array_equal(ends, be), (mode, arg, shape)


@pytest.mark.parametrize("dims", [1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64], ids=lambda d: np.dtype(d).name)
def test_decoder_on_random_words_matches_oracle(host, oracle, dims, dtype):
    """Any bit string is a stream: decoding random words drives the plane
    decoder (windowed group tests, budget and last-coefficient limits)
    through code patterns an encoder rarely writes."""
    rng = np.random.default_rng(300 + dims * 7 + ZTYPE[np.dtype(dtype)])
    modes = [("rate", 4), ("rate", 12.5), ("rate", 40), ("precision", 20), ("precision", 64),
             ("reversible", None), ("expert", (30, 70, 33, -5)), ("expert", (0, 4000, 64, -1074))]
    for mode, arg in modes:
        for density in (0.5, 0.9, 0.1):
            shape = tuple(int(v) for v in rng.integers(1, {1: 60, 2: 17, 3: 9}[dims], size=dims))
            prm = mode_params(mode, arg, dtype, dims)
            nw = oracle.max_words(tuple(reversed(shape)), np.dtype(dtype), prm) + 8
            words = np.zeros(nw, dtype=np.uint64)
            for b in range(64):
                words |= (rng.random(nw) < density).astype(np.uint64) << np.uint64(b)
            d0 = np.zeros(shape, dtype=dtype)
            d1 = np.zeros(shape, dtype=dtype)
            x0 = oracle.decompress(words, d0, prm, 0)
            x1 = host_decompress(host, words.copy(), d1, prm, 0)
            assert x0 == x1 and np.array_equal(d0.view(np.uint8), d1.view(np.uint8)), (mode, arg, shape, density)
            # the length-only parse ends where the decoder ended
            n = (C.c_size_t * 4)(*(list(reversed(shape)) + [0] * (4 - dims)))
            p = (C.c_uint * 4)(*[v & 0xffffffff for v in prm])
            nb = int(np.prod([(v + 3) // 4 for v in shape]))
            ends = np.zeros(nb, dtype=np.uint64)
            host.zgh_parse.restype = C.c_uint64
            got = host.zgh_parse(ZTYPE[np.dtype(dtype)], dims, n, p, C.c_void_p(words.ctypes.data),
                                 C.c_uint64(len(words)), C.c_uint64(0), C.c_void_p(ends.ctypes.data))
            assert got == x0, (mode, arg, shape, density)
