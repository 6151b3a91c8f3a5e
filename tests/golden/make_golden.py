"""Generate golden fixtures from the reference library itself.

Run in a container where the reference's sources exist: the library is
compiled from them by oracle/Makefile (`make -C oracle ref`) and driven
through its own public API (stream_open, zfp_stream_set_*, zfp_field_*,
zfp_write_header, zfp_compress, zfp_decompress) with the serial policy.
The inputs, the streams it wrote and SHA-256 digests of the arrays it
decoded (C order) are stored here,
so the GPU machine (which has no reference sources) can check against them.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from zfp_gb300 import capi, synth  # noqa: E402

MODES = [("rate", 8), ("rate", 16), ("rate", 12.5), ("precision", 16), ("precision", 24), ("accuracy", 1e-3),
         ("accuracy", 1e-6), ("reversible", None), ("expert", [150, 400, 30, -20])]
DTYPES = ["float32", "float64", "int32", "int64"]
SHAPES = {1: (37,), 2: (13, 18), 3: (9, 10, 7), 4: (5, 6, 7, 5)}


def values(rng, dtype, shape):
    if dtype.startswith("float"):
        x = np.cumsum(rng.standard_normal(shape), axis=-1) * 10.0 ** rng.uniform(-3, 3)
        return x.astype(dtype)
    return np.cumsum(rng.integers(-(1 << 16), 1 << 16, size=shape), axis=-1).astype(dtype)


def view_of(a, layout):
    if layout == "rev":
        return a[(slice(None, None, -1),) * a.ndim]
    if layout == "perm" and a.ndim > 1:
        return np.swapaxes(a, 0, a.ndim - 1)
    return a


def geometry(v):
    return tuple(reversed(v.shape)), tuple(s // v.itemsize for s in reversed(v.strides))


def ref_run(ref, view, mode, arg, header):
    """Compress with the reference (serial), optionally after a full header;
    decompress the stream back.  Returns (stream bytes, decoded array, params)."""
    zt = {"int32": 1, "int64": 2, "float32": 3, "float64": 4}[view.dtype.name]
    n, s = geometry(view)
    dims = len(n)
    buf = np.zeros(1 << 20, dtype=np.uint64)
    bs = ref.stream_open(buf.ctypes.data, buf.nbytes)
    z = ref.zfp_stream_open(bs)
    capi.set_mode(ref, z, mode, arg if mode != "expert" else tuple(arg), zt, dims)
    prm = ref.params(z)
    f = capi.make_field(ref, view.ctypes.data, zt, n, s)
    hbits = ref.zfp_write_header(z, f, capi.HEADER_FULL) if header else 0
    size = ref.zfp_compress(z, f)
    assert size > 0
    stream = buf[: size // 8].copy()
    out = np.zeros(view.shape, dtype=view.dtype)
    fo = capi.make_field(ref, out.ctypes.data, zt, tuple(reversed(out.shape)))
    ref.zfp_stream_rewind(z)
    if header:
        assert ref.zfp_read_header(z, fo, capi.HEADER_FULL) == hbits
    dsize = ref.zfp_decompress(z, fo)
    assert dsize == size
    ref.zfp_field_free(f)
    ref.zfp_field_free(fo)
    ref.zfp_stream_close(z)
    ref.stream_close(bs)
    return stream, out, prm, hbits


def host_api_cases(ref):
    """Expected results of the host-side API functions (mode setters, mode
    words, maximum size, metadata)."""
    out = []
    buf = np.zeros(16, dtype=np.uint64)
    bs = ref.stream_open(buf.ctypes.data, buf.nbytes)
    z = ref.zfp_stream_open(bs)
    for zt in (1, 2, 3, 4):
        for dims in (1, 2, 3, 4):
            for rate in (0.5, 1, 4, 7.3, 8, 12, 16, 31.9, 64):
                for align in (0, 1):
                    r = ref.zfp_stream_set_rate(z, rate, zt, dims, align)
                    out.append({"fn": "set_rate", "args": [rate, zt, dims, align], "ret": r,
                                "params": list(ref.params(z)), "mode": ref.zfp_stream_mode(z),
                                "cmode": ref.zfp_stream_compression_mode(z)})
    for prec in (0, 1, 7, 20, 64, 65, 100):
        r = ref.zfp_stream_set_precision(z, prec)
        out.append({"fn": "set_precision", "args": [prec], "ret": r, "params": list(ref.params(z)),
                    "mode": ref.zfp_stream_mode(z), "cmode": ref.zfp_stream_compression_mode(z)})
    for tol in (0.0, 1e-300, 1e-9, 1e-3, 0.1, 0.75, 1.0, 3.0, 1e10, 2.0 ** 900):
        r = ref.zfp_stream_set_accuracy(z, tol)
        out.append({"fn": "set_accuracy", "args": [tol], "ret": r, "params": list(ref.params(z)),
                    "mode": ref.zfp_stream_mode(z), "cmode": ref.zfp_stream_compression_mode(z)})
    ref.zfp_stream_set_reversible(z)
    out.append({"fn": "set_reversible", "args": [], "ret": None, "params": list(ref.params(z)),
                "mode": ref.zfp_stream_mode(z), "cmode": ref.zfp_stream_compression_mode(z)})
    for ex in ((1, 16658, 64, -1074), (100, 200, 30, -40), (5, 3, 10, 0), (8, 8, 0, 0), (1, 100000, 12, 7),
               (40000, 40000, 64, -1074), (1, 16658, 64, -2000)):
        r = ref.zfp_stream_set_params(z, *ex)
        out.append({"fn": "set_params", "args": list(ex), "ret": r, "params": list(ref.params(z)),
                    "mode": ref.zfp_stream_mode(z), "cmode": ref.zfp_stream_compression_mode(z)})
    # maximum size
    for mode, arg in MODES:
        for zt in (1, 2, 3, 4):
            for n in ((100,), (33, 17), (9, 10, 7), (5, 6, 7, 5)):
                capi.set_mode(ref, z, mode, arg if mode != "expert" else tuple(arg), zt, len(n))
                f = capi.make_field(ref, 0, zt, n)
                out.append({"fn": "maximum_size", "args": [mode, arg, zt, list(n)],
                            "ret": ref.zfp_stream_maximum_size(z, f), "meta": ref.zfp_field_metadata(f)})
                ref.zfp_field_free(f)
    # mode words round trip
    for m in (0, 7, 511, 2047, 2048, 2100, 2175, 2176, 2177, 3000, 4094, 0x1234567890abcfff):
        r = ref.zfp_stream_set_mode(z, m)
        out.append({"fn": "set_mode", "args": [m], "ret": r, "params": list(ref.params(z)),
                    "mode": ref.zfp_stream_mode(z)})
    ref.zfp_stream_close(z)
    ref.stream_close(bs)
    return out


def main():
    path = pyoracle.build_ref()
    if not path:
        raise SystemExit("reference sources are not available here")
    ref = capi.ZfpLib(path)
    rng = np.random.default_rng(20261203)
    arrays = {}
    cases = []
    for dims, shape in SHAPES.items():
        for dtype in DTYPES:
            base = values(rng, dtype, shape)
            arrays[f"in_{dims}d_{dtype}"] = base
            for mode, arg in MODES:
                if mode == "accuracy" and dtype.startswith("int"):
                    continue
                for layout in ("c", "rev", "perm"):
                    for header in (False, True):
                        if header and layout != "c":
                            continue
                        v = view_of(base, layout)
                        stream, out, prm, hbits = ref_run(ref, v, mode, arg, header)
                        key = f"{dims}d_{dtype}_{mode}_{arg}_{layout}_{int(header)}"
                        arrays["s_" + key] = stream
                        cases.append({"key": key, "input": f"in_{dims}d_{dtype}", "dims": dims, "dtype": dtype,
                                      "mode": mode, "arg": arg, "layout": layout, "header": header,
                                      "header_bits": int(hbits), "params": list(prm),
                                      "decoded_sha256": hashlib.sha256(out.tobytes()).hexdigest()})
    # plain-codec configuration: 3D float64 64^3 smooth field, seed 0, N(0,1e-3), fixed rate 16
    c1 = synth.smooth_field((64, 64, 64), np.float64, seed=0, noise=1e-3)
    arrays["in_config1"] = c1
    stream, out, prm, _ = ref_run(ref, c1, "rate", 16, False)
    arrays["s_config1"] = stream
    cases.append({"key": "config1", "input": "in_config1", "dims": 3, "dtype": "float64", "mode": "rate",
                  "arg": 16, "layout": "c", "header": False, "header_bits": 0, "params": list(prm),
                  "decoded_sha256": hashlib.sha256(out.tobytes()).hexdigest()})
    np.savez_compressed(os.path.join(HERE, "golden_streams.npz"), **arrays)
    with open(os.path.join(HERE, "golden_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "library": "reference zfp 1.0.1, serial policy",
                   "cases": cases, "host_api": host_api_cases(ref)}, f, indent=0)
    print(len(cases), "stream cases")


if __name__ == "__main__":
    main()
