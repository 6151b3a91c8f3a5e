"""The oracle pinned against the reference: golden fixtures written by the
reference library (tests/golden/), and, where the reference's sources are
present, the reference library itself on random and special-value inputs."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from oracle.pyoracle import mode_params
from zfp_gb300 import capi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden_cases.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, "golden_streams.npz"))
    return meta, arrays


def view_of(a, layout):
    if layout == "rev":
        return a[(slice(None, None, -1),) * a.ndim]
    if layout == "perm" and a.ndim > 1:
        return np.swapaxes(a, 0, a.ndim - 1)
    return a


def test_oracle_reproduces_golden_streams(oracle, golden):
    meta, arrays = golden
    checked = 0
    for case in meta["cases"]:
        base = arrays[case["input"]]
        view = view_of(base, case["layout"])
        prm = tuple(case["params"])
        expect = arrays["s_" + case["key"]]
        hb = case["header_bits"]
        words = np.zeros(len(expect) + 8, dtype=np.uint64)
        if hb:  # the header bits the reference wrote come first, then the blocks
            words[: (hb + 63) // 64] = expect[: (hb + 63) // 64]
            words[hb // 64] &= np.uint64((1 << (hb % 64)) - 1)
            words[hb // 64 + 1:] = 0
        words, end = oracle.compress(view, prm, bit0=hb, words=words)
        nw = (end + 63) // 64
        assert nw == len(expect) and np.array_equal(words[:nw], expect), case["key"]
        out = np.zeros(view.shape, dtype=view.dtype)
        oracle.decompress(expect, out, prm, bit0=hb)
        assert hashlib.sha256(out.tobytes()).hexdigest() == case["decoded_sha256"], case["key"]
        checked += 1
    assert checked == len(meta["cases"]) > 500


def test_oracle_parallel_matches_serial(oracle):
    from zfp_gb300 import synth
    a = synth.smooth_field((30, 41, 52), np.float64, seed=5, noise=1e-3)
    for mode, arg in (("rate", 12), ("precision", 18), ("accuracy", 1e-5), ("reversible", None)):
        prm = mode_params(mode, arg, a.dtype, 3)
        w1, e1, be1 = oracle.compress(a, prm, block_ends=True)
        w2, e2, be2 = oracle.compress(a, prm, threads=4, block_ends=True)
        nw = (e1 + 63) // 64
        assert e1 == e2 and np.array_equal(w1[:nw], w2[:nw]) and np.array_equal(be1, be2)
        starts = np.concatenate([[0], be1[:-1]]).astype(np.uint64)
        d1 = np.zeros_like(a)
        d2 = np.zeros_like(a)
        oracle.decompress(w1[:nw], d1, prm)
        oracle.decompress_par(w1[:nw], d2, prm, 4, starts)
        assert np.array_equal(d1.view(np.uint64), d2.view(np.uint64))


def _ref_roundtrip(ref, view, mode, arg):
    zt = {"int32": 1, "int64": 2, "float32": 3, "float64": 4}[view.dtype.name]
    n = tuple(reversed(view.shape))
    s = tuple(st // view.itemsize for st in reversed(view.strides))
    buf = np.zeros(1 << 18, dtype=np.uint64)
    bs = ref.stream_open(buf.ctypes.data, buf.nbytes)
    z = ref.zfp_stream_open(bs)
    capi.set_mode(ref, z, mode, arg, zt, len(n))
    prm = ref.params(z)
    f = capi.make_field(ref, view.ctypes.data, zt, n, s)
    size = ref.zfp_compress(z, f)
    out = np.zeros(view.shape, dtype=view.dtype)
    fo = capi.make_field(ref, out.ctypes.data, zt, tuple(reversed(out.shape)))
    ref.zfp_stream_rewind(z)
    ref.zfp_decompress(z, fo)
    for x in (f, fo):
        ref.zfp_field_free(x)
    ref.zfp_stream_close(z)
    ref.stream_close(bs)
    return buf[: size // 8].copy(), out, prm


def test_oracle_matches_reference_random(oracle, ref):
    rng = np.random.default_rng(77)
    special = {np.float32: np.array([0.0, -0.0, 1e-45, 1e-40, 3.4e38, np.inf, -np.inf, np.nan, 1.0, 1e-30],
                                    dtype=np.float32),
               np.float64: np.array([0.0, -0.0, 5e-324, 1e-310, 1.7e308, np.inf, -np.inf, np.nan, 1.0, 1e-300])}
    n = 0
    for dims in (1, 2, 3, 4):
        for dtype in (np.float32, np.float64, np.int32, np.int64):
            for mode, arg in (("rate", 3), ("rate", 9.75), ("precision", 5), ("precision", 33),
                              ("accuracy", 2e-4), ("reversible", None), ("expert", (20, 90, 40, -8))):
                if mode == "accuracy" and np.dtype(dtype).kind == "i":
                    continue
                for trial in range(3):
                    shape = tuple(int(v) for v in rng.integers(1, {1: 50, 2: 15, 3: 9, 4: 6}[dims], size=dims))
                    if np.dtype(dtype).kind == "f":
                        a = (np.cumsum(rng.standard_normal(shape), axis=-1) * 10.0 ** rng.uniform(-6, 6)).astype(dtype)
                        if trial == 2:
                            a = rng.choice(special[dtype], size=shape).astype(dtype)
                    else:
                        a = rng.integers(-(1 << 30), 1 << 30, size=shape).astype(dtype)
                    view = view_of(a, ("c", "rev", "perm")[trial])
                    expect, ref_out, prm = _ref_roundtrip(ref, view, mode, arg)
                    words, end = oracle.compress(view, prm)
                    nw = (end + 63) // 64
                    assert nw == len(expect) and np.array_equal(words[:nw], expect), (dims, dtype, mode, shape)
                    out = np.zeros(view.shape, dtype=view.dtype)
                    oracle.decompress(expect, out, prm)
                    assert np.array_equal(out.view(np.uint8), np.ascontiguousarray(ref_out).view(np.uint8))
                    n += 1
    assert n > 250


def test_oracle_matches_reference_tiny_budgets(oracle, ref):
    """Expert budgets of a few bits per block, as the GPU tests use them: the
    oracle must write and read what the reference does, including integer
    blocks of no bits (maxbits 0) and float budgets below the block header,
    where the reference's remaining budget wraps around and its blocks are
    coded in full (the stream then runs past zfp_stream_maximum_size, so the
    buffers here are sized for full blocks)."""
    rng = np.random.default_rng(78)
    params = [(0, 0, 64, -1074), (0, 1, 64, -1074), (1, 1, 64, -1074), (0, 3, 1, -1074), (2, 2, 64, -1074),
              (0, 9, 64, -1074), (12, 12, 64, -1074), (0, 20, 3, 0)]
    n = 0
    for dims in (1, 2, 3, 4):
        for dtype in (np.float32, np.float64, np.int32, np.int64):
            for prm_arg in params:
                if np.dtype(dtype).kind == "f" and prm_arg[1] < 1:
                    continue   # a float block codes at least one bit
                shape = tuple(int(v) for v in rng.integers(1, {1: 40, 2: 12, 3: 7, 4: 5}[dims], size=dims))
                if np.dtype(dtype).kind == "f":
                    a = (np.cumsum(rng.standard_normal(shape), axis=-1) * 10.0 ** rng.uniform(-3, 3)).astype(dtype)
                else:
                    a = rng.integers(-(1 << 20), 1 << 20, size=shape).astype(dtype)
                expect, ref_out, prm = _ref_roundtrip(ref, a, "expert", prm_arg)
                blocks = int(np.prod([(v + 3) // 4 for v in shape]))
                room = blocks * (4 ** dims * 65 + 64) // 64 + 16
                words, end = oracle.compress(a, prm, words=np.zeros(room, dtype=np.uint64))
                nw = (end + 63) // 64
                assert nw == len(expect) and np.array_equal(words[:nw], expect), (dims, dtype, prm_arg, shape)
                out = np.zeros(a.shape, dtype=a.dtype)
                oracle.decompress(expect, out, prm)
                assert np.array_equal(out.view(np.uint8), ref_out.view(np.uint8)), (dims, dtype, prm_arg, shape)
                n += 1
    assert n >= 100
