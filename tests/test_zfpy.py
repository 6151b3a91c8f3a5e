"""zfp_gb300.zfpy, the zfpy-compatible front end (python/zfpy.pyx), against
the reference's own streams: every golden stream that the reference wrote
with a full header (tests/golden) for a mode zfpy can set must come back
byte for byte from compress_numpy, and decompress_numpy must return the
reference's decoded array."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from zfp_gb300 import zfpy

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "golden_cases.json")) as f:
        cases = json.load(f)["cases"]
    data = np.load(os.path.join(HERE, "golden", "golden_streams.npz"))
    picked = [c for c in cases if c["header"] and c["layout"] == "c" and c["mode"] != "expert"]
    return picked, data


def kwargs_of(case):
    return {"rate": {"rate": case["arg"]}, "precision": {"precision": case["arg"]},
            "accuracy": {"tolerance": case["arg"]}, "reversible": {}}[case["mode"]]


def stream_bytes(data, case):
    return data["s_" + case["key"]].tobytes()


def test_header_of_reference_streams(lib, golden):
    """header() reads the reference's full headers (host code, no GPU)."""
    cases, data = golden
    for c in cases:
        h = zfpy.header(stream_bytes(data, c))
        a = data[c["input"]]
        assert [h["nx"], h["ny"], h["nz"], h["nw"]] == list(reversed(a.shape)) + [0] * (4 - a.ndim), c["key"]
        assert h["type"] == a.dtype, c["key"]
        want = {"rate": "rate", "precision": "precision", "accuracy": "tolerance", "reversible": "reversible"}
        assert h["mode"] == want[c["mode"]], c["key"]


def test_argument_errors(lib):
    with pytest.raises(ValueError):
        zfpy.compress_numpy(np.zeros(8, np.float32), tolerance=1e-3, rate=8)
    with pytest.raises(TypeError):
        zfpy.compress_numpy(None)
    with pytest.raises(TypeError):
        zfpy.compress_numpy(np.zeros(8, np.float16), rate=8)
    with pytest.raises(ValueError):
        zfpy.header(np.zeros(64, np.uint8).tobytes())


@pytest.mark.gpu
def test_compress_numpy_equals_reference_bytes(lib, cuda, golden):
    cases, data = golden
    checked = 0
    for c in cases:
        a = data[c["input"]]
        if c["mode"] == "rate":
            # zfpy hands the rate setter zfp_type_none: no minimum block size,
            # so only rates above the header size write what the C API wrote
            ebits = {np.dtype(np.float32): 9, np.dtype(np.float64): 12}.get(a.dtype, 0)
            if int(np.floor(4 ** a.ndim * c["arg"] + 0.5)) < ebits:
                continue
        got = zfpy.compress_numpy(a, **kwargs_of(c))
        assert got == stream_bytes(data, c), c["key"]
        out = zfpy.decompress_numpy(got)
        assert out.shape == a.shape and out.dtype == a.dtype
        assert hashlib.sha256(np.ascontiguousarray(out).tobytes()).hexdigest() == c["decoded_sha256"], c["key"]
        checked += 1
    assert checked >= 100


@pytest.mark.gpu
def test_headerless_decompress_and_out_checks(lib, cuda):
    rng = np.random.default_rng(7)
    a = np.cumsum(rng.standard_normal((20, 30, 40)), axis=2).astype(np.float64)
    b = zfpy.compress_numpy(a, precision=30, write_header=False)
    full = zfpy.decompress_numpy(zfpy.compress_numpy(a, precision=30))
    out = zfpy._decompress(b, zfpy.dtype_to_ztype(a.dtype), a.shape, precision=30)
    assert np.array_equal(out.view(np.uint8), full.view(np.uint8))
    buf = np.empty_like(a)
    zfpy._decompress(b, zfpy.dtype_to_ztype(a.dtype), a.shape, out=buf, precision=30)
    assert np.array_equal(buf.view(np.uint8), full.view(np.uint8))
    with pytest.raises(ValueError):
        zfpy._decompress(b, zfpy.dtype_to_ztype(a.dtype), a.shape, out=np.empty(a.shape, np.float32), precision=30)
    # reversible round trip of a strided view
    v = a[::-1, :, ::2]
    r = zfpy.decompress_numpy(zfpy.compress_numpy(v))
    assert np.array_equal(r, v)
