"""The drop-in boundary without a GPU: libzfp_gb300.so loads, exports every
entry point the headers in include/ declare, and its host-side API (mode
setters, mode words, maximum size, field metadata, headers, bit streams)
returns exactly what the reference returns (golden values recorded from the
reference library, and the live reference where its sources exist)."""
from __future__ import annotations

import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from zfp_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(INCLUDE):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith(("zfp_", "stream_")) and not name.startswith("zfp_bool"):
                names.add(name)
        for m in re.finditer(r"extern\s+const\s+[^;]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*;", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) > 90
    missing = [n for n in names if not hasattr(lib.lib, n)]
    assert not missing, missing


def test_identity_data(lib):
    assert C.c_uint.in_dll(lib.lib, "zfp_codec_version").value == 5
    assert C.c_size_t.in_dll(lib.lib, "stream_word_bits").value == 64


@pytest.fixture(scope="module")
def host_cases():
    with open(os.path.join(ROOT, "tests", "golden", "golden_cases.json")) as f:
        return json.load(f)["host_api"]


def test_host_api_matches_reference_values(lib, host_cases):
    buf = np.zeros(16, dtype=np.uint64)
    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
    z = lib.zfp_stream_open(bs)
    for c in host_cases:
        fn, args = c["fn"], c["args"]
        if fn == "set_rate":
            r = lib.zfp_stream_set_rate(z, *args)
        elif fn == "set_precision":
            r = lib.zfp_stream_set_precision(z, *args)
        elif fn == "set_accuracy":
            r = lib.zfp_stream_set_accuracy(z, *args)
        elif fn == "set_reversible":
            r = lib.zfp_stream_set_reversible(z)
        elif fn == "set_params":
            r = lib.zfp_stream_set_params(z, *args)
        elif fn == "set_mode":
            r = lib.zfp_stream_set_mode(z, args[0])
        elif fn == "maximum_size":
            mode, arg, zt, n = args
            capi.set_mode(lib, z, mode, tuple(arg) if mode == "expert" else arg, zt, len(n))
            f = capi.make_field(lib, 0, zt, n)
            assert lib.zfp_stream_maximum_size(z, f) == c["ret"], c
            assert lib.zfp_field_metadata(f) == c["meta"], c
            lib.zfp_field_free(f)
            continue
        else:
            raise AssertionError(fn)
        assert r == c["ret"], c
        assert list(lib.params(z)) == c["params"], c
        assert lib.zfp_stream_mode(z) == c["mode"], c
        if "cmode" in c:
            assert lib.zfp_stream_compression_mode(z) == c["cmode"], c
    lib.zfp_stream_close(z)
    lib.stream_close(bs)


def test_header_bits_match_reference(lib):
    """zfp_write_header output equals the leading bits of the reference's
    streams that were written with a full header (tests/golden)."""
    with open(os.path.join(ROOT, "tests", "golden", "golden_cases.json")) as f:
        cases = [c for c in json.load(f)["cases"] if c["header"]]
    arrays = np.load(os.path.join(ROOT, "tests", "golden", "golden_streams.npz"))
    for c in cases:
        base = arrays[c["input"]]
        zt = {"int32": 1, "int64": 2, "float32": 3, "float64": 4}[c["dtype"]]
        buf = np.zeros(8, dtype=np.uint64)
        bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
        z = lib.zfp_stream_open(bs)
        capi.set_mode(lib, z, c["mode"], tuple(c["arg"]) if c["mode"] == "expert" else c["arg"], zt, c["dims"])
        f = capi.make_field(lib, base.ctypes.data, zt, tuple(reversed(base.shape)))
        hb = lib.zfp_write_header(z, f, capi.HEADER_FULL)
        assert hb == c["header_bits"]
        lib.stream_flush(bs)
        expect = arrays["s_" + c["key"]].copy()
        nfull = hb // 64
        assert np.array_equal(buf[:nfull], expect[:nfull])
        mask = np.uint64((1 << (hb % 64)) - 1)
        assert (buf[nfull] & mask) == (expect[nfull] & mask)
        # and read back: the field and mode are recovered
        lib.stream_rewind(bs)
        g = lib.zfp_field_alloc()
        assert lib.zfp_read_header(z, g, capi.HEADER_FULL) == hb
        assert (g.contents.type, g.contents.nx) == (zt, base.shape[-1])
        for x in (f, g):
            lib.zfp_field_free(x)
        lib.zfp_stream_close(z)
        lib.stream_close(bs)


def _bit_ops(lib, seed):
    """A random sequence of bit-stream operations; returns the buffer and a
    trace of every return value."""
    rng = np.random.default_rng(seed)
    buf = np.zeros(64, dtype=np.uint64)
    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
    trace = []
    for _ in range(300):
        op = int(rng.integers(0, 4))
        if op == 0:
            n = int(rng.integers(0, 65))
            v = int(rng.integers(0, 1 << 63)) * 2 + int(rng.integers(0, 2))
            trace.append(int(lib.stream_write_bits(bs, v, n)))
        elif op == 1:
            trace.append(int(lib.stream_write_bit(bs, int(rng.integers(0, 2)))))
        elif op == 2:
            lib.stream_pad(bs, int(rng.integers(0, 90)))
        else:
            trace.append(int(lib.stream_flush(bs)))
        trace.append(int(lib.stream_wtell(bs)))
        if lib.stream_wtell(bs) > 64 * 50:
            break
    lib.stream_flush(bs)
    size = lib.stream_size(bs)
    lib.stream_rewind(bs)
    for _ in range(200):
        op = int(rng.integers(0, 3))
        if op == 0:
            trace.append(int(lib.stream_read_bits(bs, int(rng.integers(0, 65)))))
        elif op == 1:
            trace.append(int(lib.stream_read_bit(bs)))
        else:
            lib.stream_skip(bs, int(rng.integers(0, 70)))
        trace.append(int(lib.stream_rtell(bs)))
        if lib.stream_rtell(bs) > 64 * 45:
            break
    trace.append(int(lib.stream_align(bs)))
    trace.append(size)
    lib.stream_close(bs)
    return buf, trace


def test_bitstream_known_answers(lib):
    buf = np.zeros(4, dtype=np.uint64)
    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
    assert lib.stream_write_bits(bs, 0b1011, 3) == 1   # returns the bits above n
    lib.stream_write_bits(bs, 0xffffffffffffffff, 64)
    lib.stream_write_bit(bs, 1)
    assert lib.stream_wtell(bs) == 68
    assert lib.stream_flush(bs) == 60
    assert buf[0] == 0xfffffffffffffffb and buf[1] == 0xf
    lib.stream_rewind(bs)
    assert lib.stream_read_bits(bs, 3) == 3
    assert lib.stream_read_bits(bs, 64) == 0xffffffffffffffff
    lib.stream_close(bs)


def test_bitstream_matches_reference(lib, ref):
    for seed in range(20):
        b1, t1 = _bit_ops(lib, seed)
        b2, t2 = _bit_ops(ref, seed)
        assert t1 == t2 and np.array_equal(b1, b2), seed


def test_no_cpu_codec(lib):
    """Only zfp_exec_cuda compresses; serial returns 0 before any GPU call."""
    a = np.ones((8, 8), dtype=np.float32)
    buf = np.zeros(256, dtype=np.uint64)
    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
    z = lib.zfp_stream_open(bs)
    lib.zfp_stream_set_rate(z, 8, capi.TYPE_FLOAT, 2, 0)
    f = capi.make_field(lib, a.ctypes.data, capi.TYPE_FLOAT, (8, 8))
    assert lib.zfp_stream_execution(z) == capi.EXEC_SERIAL
    assert lib.zfp_compress(z, f) == 0 and lib.zfp_decompress(z, f) == 0
    assert lib.stream_wtell(bs) == 0
    assert not lib.zfp_stream_set_execution(z, capi.EXEC_OMP)
    assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
    assert lib.zfp_stream_execution(z) == capi.EXEC_CUDA
    lib.zfp_field_free(f)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)
