"""GPU codec parity through the C ABI (zfp_compress / zfp_decompress with
zfp_exec_cuda) against the oracle, bit for bit.

Covers the reference's end-to-end matrix (tests/src/endtoend/zfpEndtoendBase.c:
1-4D x int32/int64/float/double x fixed rate/precision/accuracy/reversible x
AS_IS/REVERSED/PERMUTED/INTERLEAVED strides) plus what the GPU path adds:
host or device field and stream buffers, streams that start mid-word,
variable-rate streams written elsewhere (no index), and error returns."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle.pyoracle import mode_params
from zfp_gb300 import capi
from tests.helpers import geometry, oracle_stream, zfp_run, ztype_of

pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(1234)

MODES = [("rate", 4), ("rate", 8), ("rate", 12.5), ("rate", 1.5), ("precision", 12), ("precision", 24),
         ("accuracy", 1e-3), ("accuracy", 1e-7), ("reversible", None), ("expert", (100, 300, 20, -30))]


def make_values(dtype, shape, kind="smooth"):
    if np.dtype(dtype).kind == "f":
        if kind == "special":
            sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -2.5, 1e-30, 1e-40, 3e38], dtype=np.float64)
            if dtype == np.float64:
                sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -2.5, 1e-300, 5e-324, 1.7e308])
            return RNG.choice(sp, size=shape).astype(dtype)
        x = np.cumsum(RNG.standard_normal(shape), axis=-1)
        if len(shape) > 1:
            x = np.cumsum(x, axis=0)
        if kind == "patchy":   # runs of two zero blocks between runs of two coded ones
            x[..., (np.arange(shape[-1]) // 8) % 2 == 0] = 0
        return (x * 10.0 ** RNG.uniform(-4, 4)).astype(dtype)
    bits = 28 if dtype == np.int32 else 58
    x = np.cumsum(RNG.integers(-(1 << 20), 1 << 20, size=shape), axis=-1).clip(-(1 << bits), 1 << bits)
    if kind == "patchy":
        x[..., (np.arange(shape[-1]) // 8) % 2 == 0] = 0
    return x.astype(dtype)


def make_view(base, layout):
    d = base.ndim
    if layout == "rev":
        return base[(slice(None, None, -1),) * d]
    if layout == "perm" and d >= 2:
        return np.swapaxes(base, 0, d - 1)
    if layout == "gap":
        return base[..., ::2]
    return base


def base_shape(shape, layout):
    if layout == "gap":
        return shape[:-1] + (2 * shape[-1],)
    if layout == "perm" and len(shape) >= 2:
        s = list(shape)
        s[0], s[-1] = s[-1], s[0]
        return tuple(s)
    return shape


class DevSpan:
    """Device copy of the memory span of a numpy view, addressed like the view."""

    def __init__(self, torch, view, upload=True):
        n, s = geometry(view)
        lo = sum(min(0, st * (nn - 1)) for nn, st in zip(n, s))
        hi = sum(max(0, st * (nn - 1)) for nn, st in zip(n, s))
        self.isz = view.itemsize
        self.nbytes = (hi - lo + 1) * self.isz
        self.host_begin = view.ctypes.data + lo * self.isz
        self.dev = torch.zeros(self.nbytes, dtype=torch.uint8, device="cuda")
        if upload:
            raw = np.ctypeslib.as_array((C.c_uint8 * self.nbytes).from_address(self.host_begin))
            self.dev.copy_(torch.from_numpy(raw.copy()))
        self.ptr = self.dev.data_ptr() + (view.ctypes.data - self.host_begin)

    def download_into(self, view):
        raw = np.ctypeslib.as_array((C.c_uint8 * self.nbytes).from_address(self.host_begin))
        raw[:] = self.dev.cpu().numpy()


def run_case(lib, oracle, torch, dtype, shape, mode, arg, layout="c", field_dev=False, stream_dev=False,
             prefix=None, kind="smooth", async_=False, room=0):
    base = make_values(dtype, base_shape(shape, layout), kind)
    view = make_view(base, layout)
    n, s = geometry(view)
    zt = ztype_of(view)
    exp_words, exp_end, prm = oracle_stream(oracle, view, mode, arg, prefix, room)
    nwords = len(exp_words) + 16

    fspan = DevSpan(torch, view) if field_dev else None
    fptr = fspan.ptr if field_dev else view.ctypes.data
    if stream_dev:
        sbuf = torch.zeros(nwords, dtype=torch.int64, device="cuda")
        sptr = sbuf.data_ptr()
    else:
        sbuf = np.zeros(nwords, dtype=np.uint64)
        sptr = sbuf.ctypes.data
    r, pos = zfp_run(lib, "compress", fptr, zt, n, s, mode, arg, sptr, nwords * 8, prefix, async_=async_)
    if async_:
        torch.cuda.synchronize()
    msg = f"{np.dtype(dtype).name} {shape} {mode}={arg} {layout} fdev={field_dev} sdev={stream_dev} prefix={prefix}"
    assert r == len(exp_words) * 8, f"size {r} != {len(exp_words) * 8}: {msg}; {lib.zfp_gb300_last_error()}"
    assert pos == len(exp_words) * 64
    got = sbuf[: len(exp_words)].cpu().numpy().view(np.uint64) if stream_dev else sbuf[: len(exp_words)]
    bad = np.nonzero(got != exp_words)[0]
    assert bad.size == 0, f"stream differs at words {bad[:8]} of {len(exp_words)}: {msg}"

    # decompress into a fresh view of the same layout.  Positioning a stream
    # mid-word (stream_rseek) reads the buffer from the host, as in the
    # reference, so a device stream that starts mid-word is read back from a
    # host copy.
    if stream_dev and prefix and prefix[2]:
        hcopy = sbuf.cpu().numpy().view(np.uint64).copy()
        sptr = hcopy.ctypes.data
    out_base = np.zeros(base.shape, dtype=dtype)
    out_view = make_view(out_base, layout)
    ospan = DevSpan(torch, out_view) if field_dev else None
    optr = ospan.ptr if field_dev else out_view.ctypes.data
    r2, pos2 = zfp_run(lib, "decompress", optr, zt, n, s, mode, arg, sptr, nwords * 8, prefix, async_=async_)
    if async_:
        torch.cuda.synchronize()
    assert r2 == len(exp_words) * 8, f"decompress returned {r2}: {msg}; {lib.zfp_gb300_last_error()}"
    if field_dev:
        ospan.download_into(out_view)
    ref_out = np.zeros(view.shape, dtype=dtype)
    bit0 = 64 * prefix[0] + prefix[2] if prefix else 0
    oracle.decompress(exp_words, ref_out, prm, bit0)
    got_out = np.ascontiguousarray(out_view).view(np.uint8)
    assert np.array_equal(got_out, ref_out.view(np.uint8)), f"decoded values differ: {msg}"


SHAPES = {1: [(1,), (7,), (64,), (1001,)], 2: [(1, 1), (5, 7), (16, 16), (37, 61)],
          3: [(1, 1, 1), (3, 5, 7), (8, 8, 8), (13, 21, 30)], 4: [(2, 3, 5, 6), (4, 4, 4, 4), (5, 9, 7, 6)]}
DTYPES = [np.float32, np.float64, np.int32, np.int64]


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
@pytest.mark.parametrize("dtype", DTYPES, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("mode,arg", MODES, ids=lambda v: str(v))
def test_matrix_host(lib, oracle, cuda, dims, dtype, mode, arg):
    if mode == "accuracy" and np.dtype(dtype).kind == "i":
        pytest.skip("accuracy mode is for floating point")
    for shape in SHAPES[dims]:
        for layout in ("c", "rev", "perm", "gap"):
            run_case(lib, oracle, cuda, dtype, shape, mode, arg, layout)


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
@pytest.mark.parametrize("dtype", DTYPES, ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("mode,arg", [("rate", 8), ("precision", 16), ("accuracy", 1e-4), ("reversible", None)],
                         ids=lambda v: str(v))
def test_matrix_device(lib, oracle, cuda, dims, dtype, mode, arg):
    if mode == "accuracy" and np.dtype(dtype).kind == "i":
        pytest.skip("accuracy mode is for floating point")
    shape = SHAPES[dims][-1]
    for layout in ("c", "rev", "perm"):
        for fdev, sdev in ((True, True), (True, False), (False, True)):
            run_case(lib, oracle, cuda, dtype, shape, mode, arg, layout, field_dev=fdev, stream_dev=sdev)


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("mode,arg", [("rate", 16), ("precision", 30), ("accuracy", 1e-3), ("accuracy", 0.0),
                                      ("reversible", None)], ids=lambda v: str(v))
def test_special_values(lib, oracle, cuda, dtype, mode, arg):
    for dims in (1, 2, 3):
        run_case(lib, oracle, cuda, dtype, SHAPES[dims][-1], mode, arg, kind="special")


@pytest.mark.parametrize("mode,arg", [("rate", 8), ("rate", 5.5), ("accuracy", 1e-3), ("reversible", None)],
                         ids=lambda v: str(v))
def test_stream_offsets(lib, oracle, cuda, mode, arg):
    """Streams that start mid-word, as after zfp_write_header (src/zfp.c:1183)."""
    for prefix in ((0, 0x5, 3), (2, 0x1234567, 29), (1, (1 << 63) - 5, 63), (3, 0, 0)):
        run_case(lib, oracle, cuda, np.float32, (9, 10, 11), mode, arg, prefix=prefix)
        run_case(lib, oracle, cuda, np.float64, (33, 17), mode, arg, prefix=prefix)
    # device streams: word-aligned start plus bits still held in the stream buffer
    for prefix in ((1, 0x2b, 7), (0, 0, 0)):
        run_case(lib, oracle, cuda, np.float32, (9, 10, 11), mode, arg, prefix=prefix, field_dev=True,
                 stream_dev=True)


def test_many_tiles(lib, oracle, cuda):
    """Fields spanning many CTA tiles: exercises look-back and tile seams."""
    for mode, arg in (("accuracy", 1e-2), ("precision", 10), ("rate", 3.25), ("reversible", None)):
        run_case(lib, oracle, cuda, np.float32, (40, 64, 90), mode, arg, field_dev=True, stream_dev=True)
        run_case(lib, oracle, cuda, np.float64, (40, 64, 90), mode, arg, field_dev=True, stream_dev=True,
                 prefix=(0, 0x3, 2))
        run_case(lib, oracle, cuda, np.float32, (257, 129), mode, arg, layout="perm")


@pytest.mark.parametrize("dtype,mode,arg", [(np.float64, "accuracy", 1e-3), (np.float64, "reversible", None),
                                            (np.float64, "precision", 40), (np.float32, "accuracy", 1e-6),
                                            (np.float32, "precision", 32), (np.int64, "reversible", None)],
                         ids=lambda v: str(v))
def test_direct_tiles_with_short_blocks(lib, oracle, cuda, dtype, mode, arg):
    """Tiles too large for the encoder's shared-memory image are coded
    straight into the stream.  Zero blocks code in a bit or a few, so several
    block boundaries share one stream word; they alternate here with coded
    blocks over many tiles, on and off word boundaries, host and device."""
    shape = (40, 64, 90)
    for prefix in (None, (1, 0x2b, 7), (0, 0x5, 3)):
        run_case(lib, oracle, cuda, dtype, shape, mode, arg, prefix=prefix, kind="patchy")
    run_case(lib, oracle, cuda, dtype, shape, mode, arg, field_dev=True, stream_dev=True, kind="patchy")


@pytest.mark.parametrize("dtype", DTYPES, ids=lambda d: np.dtype(d).name)
def test_tiny_budgets(lib, oracle, cuda, dtype):
    """Expert-mode budgets of a few bits per block over many tiles, streams
    starting on and off a word: integer blocks of no bits at all (maxbits 0)
    leave only the bits ahead of the stream; a float budget below the block
    header makes the reference's remaining budget wrap around, so its blocks
    code in full (zfp_stream_maximum_size does not hold for them)."""
    shape = (40, 64, 90)
    room = 10 * 16 * 23 * (64 * 65 + 64) // 64
    params = [(0, 0, 64, -1074), (0, 1, 64, -1074), (1, 1, 64, -1074), (0, 3, 1, -1074), (2, 2, 64, -1074),
              (0, 9, 64, -1074), (12, 12, 64, -1074), (0, 20, 3, 0)]
    for prm in params:
        if np.dtype(dtype).kind == "f" and prm[1] < 1:
            continue   # a float block codes at least one bit
        for prefix in (None, (1, 0x2b, 7), (0, 0x5, 3)):
            run_case(lib, oracle, cuda, dtype, shape, "expert", prm, prefix=prefix, room=room)
        run_case(lib, oracle, cuda, dtype, shape, "expert", prm, field_dev=True, stream_dev=True, room=room)


def test_async_fixed_rate(lib, oracle, cuda):
    run_case(lib, oracle, cuda, np.float32, (32, 48, 64), "rate", 8, field_dev=True, stream_dev=True, async_=True)


def test_foreign_variable_stream(lib, oracle, cuda):
    """A variable-rate stream this library did not write (no index): the
    decoder must recover block offsets itself."""
    torch = cuda
    for dtype, mode, arg in ((np.float32, "accuracy", 1e-3), (np.float64, "reversible", None),
                             (np.int32, "precision", 20)):
        a = make_values(dtype, (19, 23, 17))
        words, end, prm = oracle_stream(oracle, a, mode, arg)
        n, s = geometry(a)
        for sdev in (False, True):
            if sdev:
                buf = torch.from_numpy(words.view(np.int64).copy()).cuda()
                ptr = buf.data_ptr()
            else:
                buf = words.copy()
                ptr = buf.ctypes.data
            out = np.zeros_like(a)
            r, _ = zfp_run(lib, "decompress", out.ctypes.data, ztype_of(a), n, s, mode, arg, ptr, words.nbytes)
            assert r == words.nbytes, lib.zfp_gb300_last_error()
            ref = np.zeros_like(a)
            oracle.decompress(words, ref, prm)
            assert np.array_equal(out.view(np.uint8), ref.view(np.uint8))


def test_stale_index_is_detected(lib, oracle, cuda):
    """Compress field A into a device buffer (the library keeps its block
    index), overwrite the buffer with a different stream B of the same shape
    and mode, decompress: the result must be B's, not A's."""
    torch = cuda
    a = make_values(np.float32, (16, 24, 20))
    b = make_values(np.float32, (16, 24, 20)) * 7
    wb, endb, prm = oracle_stream(oracle, b, "accuracy", 1e-4)
    n, s = geometry(a)
    cap = max(len(wb), oracle.max_words(n, np.float32, prm)) + 8
    buf = torch.zeros(cap, dtype=torch.int64, device="cuda")
    r, _ = zfp_run(lib, "compress", a.ctypes.data, 3, n, s, "accuracy", 1e-4, buf.data_ptr(), cap * 8)
    assert r > 0
    buf.zero_()
    buf[: len(wb)] = torch.from_numpy(wb.view(np.int64).copy()).cuda()
    out = np.zeros_like(a)
    r, _ = zfp_run(lib, "decompress", out.ctypes.data, 3, n, s, "accuracy", 1e-4, buf.data_ptr(), cap * 8)
    assert r == len(wb) * 8, lib.zfp_gb300_last_error()
    ref = np.zeros_like(b)
    oracle.decompress(wb, ref, prm)
    assert np.array_equal(out, ref)


def test_errors_return_zero(lib, cuda):
    a = make_values(np.float32, (8, 8, 8))
    n, s = geometry(a)
    buf = np.zeros(1024, dtype=np.uint64)
    # serial policy: no CPU codec in this library
    r, pos = zfp_run(lib, "compress", a.ctypes.data, 3, n, s, "rate", 8, buf.ctypes.data, buf.nbytes,
                     policy=capi.EXEC_SERIAL)
    assert r == 0 and pos == 0
    # OpenMP cannot be selected
    bs = lib.stream_open(buf.ctypes.data, buf.nbytes)
    z = lib.zfp_stream_open(bs)
    assert not lib.zfp_stream_set_execution(z, capi.EXEC_OMP)
    lib.zfp_stream_close(z)
    lib.stream_close(bs)
    # fixed-rate stream that does not fit: refused up front, stream untouched
    r, pos = zfp_run(lib, "compress", a.ctypes.data, 3, n, s, "rate", 8, buf.ctypes.data, 32 * 8)
    assert r == 0 and pos == 0
    # variable-rate overflow detected on the GPU
    b = make_values(np.float32, (8, 8, 8)) + np.float32(1.0)
    r, pos = zfp_run(lib, "compress", b.ctypes.data, 3, n, s, "reversible", None, buf.ctypes.data, 16 * 8)
    assert r == 0 and pos == 0
    assert "small" in lib.zfp_gb300_last_error().decode()
    # the same for tiles too large for shared memory, written straight into a
    # device stream: the blocks past its end are dropped and the call fails
    torch = cuda
    c = np.random.default_rng(8).standard_normal((40, 64, 90)) * 1e3
    dc = torch.from_numpy(c).cuda()
    dbuf = torch.zeros(1 << 16, dtype=torch.int64, device="cuda")
    n3, s3 = geometry(c)
    r, pos = zfp_run(lib, "compress", dc.data_ptr(), 4, n3, s3, "reversible", None, dbuf.data_ptr(), dbuf.numel() * 8)
    assert r == 0 and pos == 0
    assert "small" in lib.zfp_gb300_last_error().decode()
    big = torch.zeros(1 << 21, dtype=torch.int64, device="cuda")   # and a buffer that holds it works
    r, _ = zfp_run(lib, "compress", dc.data_ptr(), 4, n3, s3, "reversible", None, big.data_ptr(), big.numel() * 8)
    assert r > 0, lib.zfp_gb300_last_error()


def test_pinned_host_buffers_zero_copy(lib, oracle, cuda):
    """Page-locked host fields and streams are read and written in place by
    the kernels (nothing is staged through device memory) with the same bits
    as the oracle; pageable host buffers are still staged."""
    torch = cuda
    tdt = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.int64: torch.int64}
    # (64-bit accuracy tiles can outgrow the decoder's shared memory, and
    # such streams are uploaded instead: see the test below)
    cases = [(np.float32, (37, 45, 66), "rate", 8), (np.float64, (21, 30, 47), "precision", 24),
             (np.int32, (300, 301), "precision", 20), (np.float32, (40, 64, 90), "reversible", None),
             (np.int64, (9, 10, 11, 12), "rate", 12)]
    for dtype, shape, mode, arg in cases:
        vals = make_values(dtype, shape)
        exp_words, _, prm = oracle_stream(oracle, vals, mode, arg)
        nwords = len(exp_words) + 16
        hx = torch.empty(shape, dtype=tdt[dtype], pin_memory=True)
        hx.numpy()[...] = vals
        hs = torch.zeros(nwords + 8, dtype=torch.int64, pin_memory=True)
        sptr = hs.data_ptr() + 64            # the stream starts inside the pinned block
        n, s = geometry(vals)
        zt = ztype_of(vals)
        msg = f"{np.dtype(dtype).name} {shape} {mode}={arg}"
        r, _ = zfp_run(lib, "compress", hx.data_ptr(), zt, n, s, mode, arg, sptr, nwords * 8)
        assert r == len(exp_words) * 8, (msg, lib.zfp_gb300_last_error())
        assert lib.zfp_gb300_last_staged_bytes() == 0, msg
        assert np.array_equal(hs.numpy().view(np.uint64)[8: 8 + len(exp_words)], exp_words), msg
        hout = torch.zeros(shape, dtype=tdt[dtype], pin_memory=True)
        r2, _ = zfp_run(lib, "decompress", hout.data_ptr(), zt, n, s, mode, arg, sptr, nwords * 8)
        assert r2 == r and lib.zfp_gb300_last_staged_bytes() == 0, msg
        ref_out = np.zeros(shape, dtype=dtype)
        oracle.decompress(exp_words, ref_out, prm, 0)
        assert np.array_equal(hout.numpy().view(np.uint8), ref_out.view(np.uint8)), msg
        # the same stream from pageable memory goes through staging
        page = np.zeros(nwords, dtype=np.uint64)
        page[: len(exp_words)] = exp_words
        out2 = np.zeros(shape, dtype=dtype)
        r3, _ = zfp_run(lib, "decompress", out2.ctypes.data, zt, n, s, mode, arg, page.ctypes.data, nwords * 8)
        assert r3 == r and lib.zfp_gb300_last_staged_bytes() > 0, msg
        assert np.array_equal(out2.view(np.uint8), ref_out.view(np.uint8)), msg


def test_pinned_stream_offsets(lib, oracle, cuda):
    """Page-locked streams starting inside a word, written in place: tiles are
    staged in shared memory (fixed rate too) and the caller's bits ahead of
    the stream survive."""
    torch = cuda
    for dtype, shape, mode, arg in [(np.float32, (40, 64, 90), "rate", 8), (np.float32, (40, 64, 90), "rate", 5.5),
                                    (np.float64, (33, 40, 50), "accuracy", 1e-3),
                                    (np.float64, (33, 40, 50), "reversible", None)]:
        vals = make_values(dtype, shape)
        for prefix in ((1, 0x2b, 7), (0, 0x5, 3)):
            exp_words, _, prm = oracle_stream(oracle, vals, mode, arg, prefix)
            nwords = len(exp_words) + 16
            hs = torch.zeros(nwords, dtype=torch.int64, pin_memory=True)
            hx = torch.from_numpy(vals.copy()).pin_memory()
            n, s = geometry(vals)
            r, _ = zfp_run(lib, "compress", hx.data_ptr(), ztype_of(vals), n, s, mode, arg, hs.data_ptr(),
                           nwords * 8, prefix)
            msg = f"{np.dtype(dtype).name} {shape} {mode}={arg} prefix={prefix}"
            assert r == len(exp_words) * 8, (msg, lib.zfp_gb300_last_error())
            assert lib.zfp_gb300_last_staged_bytes() == 0, msg
            got = hs.numpy().view(np.uint64)[: len(exp_words)]
            bad = np.nonzero(got != exp_words)[0]
            assert bad.size == 0, (msg, bad[:8])


def test_pinned_stream_uploaded_when_tiles_exceed_shared_memory(lib, oracle, cuda):
    """A page-locked stream whose decode tiles do not fit the decoder's shared
    memory (4D 64-bit reversible noise: about 270 KB a tile of 128 blocks,
    more than a CTA's shared memory) is uploaded once instead of being read
    word by word across the host link; 32-byte row stores write the 64-bit
    field.  Same bits as the oracle either way."""
    torch = cuda
    shape = (16, 16, 16, 16)
    vals = np.random.default_rng(5).standard_normal(shape) * 1e3   # about 64 bits a value
    exp_words, _, prm = oracle_stream(oracle, vals, "reversible", None)
    nwords = len(exp_words) + 16
    hx = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    hx.numpy()[...] = vals
    hs = torch.zeros(nwords, dtype=torch.int64, pin_memory=True)
    n, s = geometry(vals)
    zt = ztype_of(vals)
    r, _ = zfp_run(lib, "compress", hx.data_ptr(), zt, n, s, "reversible", None, hs.data_ptr(), nwords * 8)
    assert r == len(exp_words) * 8, lib.zfp_gb300_last_error()
    assert lib.zfp_gb300_last_staged_bytes() == 0
    assert np.array_equal(hs.numpy().view(np.uint64)[: len(exp_words)], exp_words)
    hout = torch.zeros(shape, dtype=torch.float64, pin_memory=True)
    r2, _ = zfp_run(lib, "decompress", hout.data_ptr(), zt, n, s, "reversible", None, hs.data_ptr(), nwords * 8)
    assert r2 == r and lib.zfp_gb300_last_staged_bytes() == r
    assert np.array_equal(hout.numpy().view(np.uint64), vals.view(np.uint64))


def test_foreign_stream_long_parallel_parse(lib, cuda):
    """A long variable-rate stream with no index (more than 32,768 blocks)
    takes the speculative parallel parse; the decoded arrays must equal the
    ones decoded with the encoder's own index, bit for bit."""
    torch = cuda
    from zfp_gb300 import synth
    for dtype, ztype, shape, mode, arg in [(torch.float32, capi.TYPE_FLOAT, (64, 256, 256), "accuracy", 1e-3),
                                           (torch.float32, capi.TYPE_FLOAT, (48, 200, 320), "reversible", None),
                                           (torch.float64, capi.TYPE_DOUBLE, (64, 192, 192), "precision", 30)]:
        x = synth.smooth_field_torch(shape, dtype, seed=5, noise=1e-2)
        n, s = tuple(reversed(shape)), (0, 0, 0)
        cap = x.numel() * x.element_size() * 2 + 4096
        buf = torch.zeros(cap // 8, dtype=torch.int64, device="cuda")
        size, _ = zfp_run(lib, "compress", x.data_ptr(), ztype, n, s, mode, arg, buf.data_ptr(), cap)
        assert size, lib.zfp_gb300_last_error()
        out_idx = torch.zeros_like(x)
        assert zfp_run(lib, "decompress", out_idx.data_ptr(), ztype, n, s, mode, arg, buf.data_ptr(), cap)[0] == size
        foreign = buf.clone()     # another buffer: no recorded index, offsets come from the parse
        out = torch.zeros_like(x)
        r, _ = zfp_run(lib, "decompress", out.data_ptr(), ztype, n, s, mode, arg, foreign.data_ptr(), cap)
        assert r == size, (mode, lib.zfp_gb300_last_error())
        assert torch.equal(out.view(torch.int8), out_idx.view(torch.int8)), mode
