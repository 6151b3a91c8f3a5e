"""GPU streams and decoded arrays against the reference library's own
outputs (tests/golden, written by tests/golden/make_golden.py), including
streams that follow a full zfp header and the plain-codec configuration
(3D float64 64^3, fixed rate 16)."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from zfp_gb300 import capi
from tests.helpers import geometry

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden_cases.json")) as f:
        meta = json.load(f)
    return meta["cases"], np.load(os.path.join(GOLDEN, "golden_streams.npz"))


def view_of(a, layout):
    if layout == "rev":
        return a[(slice(None, None, -1),) * a.ndim]
    if layout == "perm" and a.ndim > 1:
        return np.swapaxes(a, 0, a.ndim - 1)
    return a


def gpu_roundtrip(lib, torch, view, case, device):
    zt = {"int32": 1, "int64": 2, "float32": 3, "float64": 4}[case["dtype"]]
    n, s = geometry(view)
    mode, arg = case["mode"], case["arg"]
    arg = tuple(arg) if mode == "expert" else arg
    expect_words = len(case["_expect"])
    cap = expect_words + 32
    hbuf = np.zeros(cap, dtype=np.uint64)
    if device:   # contiguous layouts only: the field is moved as a dense tensor
        fdev = torch.from_numpy(np.ascontiguousarray(view)).cuda()
        fptr = fdev.data_ptr()
        sbuf = torch.zeros(cap, dtype=torch.int64, device="cuda")
        sptr = sbuf.data_ptr()
    else:
        fptr = view.ctypes.data
        sptr = hbuf.ctypes.data
    bs = lib.stream_open(sptr, cap * 8)
    z = lib.zfp_stream_open(bs)
    capi.set_mode(lib, z, mode, arg, zt, case["dims"])
    assert lib.zfp_stream_set_execution(z, capi.EXEC_CUDA)
    f = capi.make_field(lib, fptr, zt, n, s)
    if case["header"]:
        assert lib.zfp_write_header(z, f, capi.HEADER_FULL) == case["header_bits"]
    size = lib.zfp_compress(z, f)
    assert size == expect_words * 8, (case["key"], size)
    got = sbuf[:expect_words].cpu().numpy().view(np.uint64) if device else hbuf[:expect_words]
    assert np.array_equal(got, case["_expect"]), case["key"]
    # decode
    out = np.zeros(view.shape, dtype=view.dtype)
    if device:
        odev = torch.zeros(out.shape, dtype=fdev.dtype, device="cuda")
        optr = odev.data_ptr()
    else:
        optr = out.ctypes.data
    fo = capi.make_field(lib, optr, zt, tuple(reversed(out.shape)))
    lib.zfp_stream_rewind(z)
    if case["header"]:
        assert lib.zfp_read_header(z, fo, capi.HEADER_FULL) == case["header_bits"]
        lib.zfp_field_set_pointer(fo, optr)
    assert lib.zfp_decompress(z, fo) == size
    if device:
        out = odev.cpu().numpy()
    assert hashlib.sha256(out.tobytes()).hexdigest() == case["decoded_sha256"], case["key"]
    for x in (f, fo):
        lib.zfp_field_free(x)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)


def test_golden_streams_host_buffers(lib, cuda, golden):
    cases, arrays = golden
    for case in cases:
        case["_expect"] = arrays["s_" + case["key"]]
        view = view_of(arrays[case["input"]], case["layout"])
        gpu_roundtrip(lib, cuda, view, case, device=False)


def test_golden_streams_device_buffers(lib, cuda, golden):
    cases, arrays = golden
    n = 0
    for case in cases:
        if case["layout"] != "c" or case["header"]:
            continue
        case["_expect"] = arrays["s_" + case["key"]]
        gpu_roundtrip(lib, cuda, arrays[case["input"]], case, device=True)
        n += 1
    assert n > 100
