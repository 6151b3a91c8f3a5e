"""Benchmark configurations at full size, bit for bit against the oracle
(parallel compress/decompress of the oracle on the host cores).

Configuration 2: 3D float32 512^3 and float64 384^3 smooth fields (seed 1,
N(0,1e-2) noise) in fixed-rate 8, fixed-precision 20, fixed-accuracy 1e-3
and reversible mode.  Configuration 3: fixed-rate 12 and fixed-precision 24
on 2D float64 16384^2, 4D float32 64^4, 3D float32 383x257x129 (partial
blocks), its transposed strided view (strides 257*129, 1, 257), and 3D int32
256^3 uniform in [-2^20, 2^20) in reversible mode.  Size-independent
properties are checked too: reversible is lossless, fixed-accuracy error is
within the tolerance, fixed-rate size is exact."""
from __future__ import annotations

import os

import numpy as np
import pytest

from oracle.pyoracle import mode_params
from zfp_gb300 import capi, synth
from tests.helpers import geometry, zfp_run, ztype_of

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def check_full(lib, oracle, torch, host_view, mode, arg, dev_field_ptr=None):
    """Compress on the GPU (device buffers), compare with the oracle's stream;
    decompress on the GPU, compare with the oracle's decode."""
    n, s = geometry(host_view)
    zt = ztype_of(host_view)
    prm = mode_params(mode, arg, host_view.dtype, len(n))
    words, end, be = oracle.compress(host_view, prm, threads=THREADS, block_ends=True)
    nw = (end + 63) // 64
    words = words[:nw]
    cap = nw + 64
    sbuf = torch.zeros(cap, dtype=torch.int64, device="cuda")
    if dev_field_ptr is None:
        dev = torch.from_numpy(np.ascontiguousarray(host_view)).cuda()
        fptr = dev.data_ptr()
        fn, fs = tuple(reversed(dev.shape)), ()
    else:
        fptr, fn, fs = dev_field_ptr, n, s
    r, _ = zfp_run(lib, "compress", fptr, zt, fn, fs, mode, arg, sbuf.data_ptr(), cap * 8)
    assert r == nw * 8, (mode, arg, r, nw * 8, lib.zfp_gb300_last_error())
    got = sbuf[:nw].cpu().numpy().view(np.uint64)
    bad = np.nonzero(got != words)[0]
    assert bad.size == 0, f"{mode}={arg}: {bad.size} words differ, first {bad[:4]}"
    # GPU decode vs oracle decode of the same stream
    out = torch.empty(host_view.shape, dtype=getattr(torch, host_view.dtype.name), device="cuda")
    r2, _ = zfp_run(lib, "decompress", out.data_ptr(), zt, tuple(reversed(out.shape)), (), mode, arg,
                    sbuf.data_ptr(), cap * 8)
    assert r2 == r, lib.zfp_gb300_last_error()
    ref = np.empty(host_view.shape, dtype=host_view.dtype)
    starts = None if prm[0] == prm[1] and mode == "rate" else np.concatenate([[0], be[:-1]]).astype(np.uint64)
    oracle.decompress_par(words, ref, prm, THREADS, starts)
    got_out = out.cpu().numpy()
    assert np.array_equal(got_out.view(np.uint8), ref.view(np.uint8)), f"{mode}={arg}: decode differs"
    return got_out, nw * 8


@pytest.mark.parametrize("name,shape", [("f32", (512, 512, 512)), ("f64", (384, 384, 384))])
def test_config2_four_modes(lib, oracle, cuda, name, shape):
    torch = cuda
    dt = torch.float32 if name == "f32" else torch.float64
    x = synth.smooth_field_torch(shape, dt, seed=1, noise=1e-2).cpu().numpy()
    for mode, arg in (("rate", 8), ("precision", 20), ("accuracy", 1e-3), ("reversible", None)):
        out, size = check_full(lib, oracle, torch, x, mode, arg)
        if mode == "reversible":
            assert np.array_equal(out.view(np.uint8), x.view(np.uint8))
        if mode == "accuracy":
            assert np.abs(out.astype(np.float64) - x.astype(np.float64)).max() <= 1e-3
        if mode == "rate":
            assert size == x.size * 8 // 8   # 8 bits per value, whole words


def test_config3_edge_shapes(lib, oracle, cuda):
    torch = cuda
    rng = np.random.default_rng(3)
    for mode, arg in (("rate", 12), ("precision", 24)):
        # (b) 4D float32 64^4
        b = synth.smooth_field_torch((64, 64, 64, 64), torch.float32, seed=3, noise=1e-2).cpu().numpy()
        check_full(lib, oracle, torch, b, mode, arg)
        # (c) 3D float32 383x257x129 (numpy shape z, y, x)
        c = synth.smooth_field_torch((129, 257, 383), torch.float32, seed=4, noise=1e-2).cpu().numpy()
        check_full(lib, oracle, torch, c, mode, arg)
        # (d) the transposed strided view of (c): strides (257*129, 1, 257)
        mem = np.ascontiguousarray(c.transpose(2, 0, 1))          # memory order x (slowest), z, y (fastest)
        view = np.lib.stride_tricks.as_strided(mem, shape=(129, 257, 383), strides=(257 * 4, 4, 257 * 129 * 4))
        assert geometry(view) == ((383, 257, 129), (257 * 129, 1, 257))
        dev = torch.from_numpy(mem).cuda()
        check_full(lib, oracle, torch, view, mode, arg, dev_field_ptr=dev.data_ptr())
    # (a) 2D float64 16384^2
    a = synth.smooth_field_torch((16384, 16384), torch.float64, seed=5, noise=1e-2).cpu().numpy()
    for mode, arg in (("rate", 12), ("precision", 24)):
        check_full(lib, oracle, torch, a, mode, arg)
    del a
    # (e) 3D int32 256^3 uniform in [-2^20, 2^20), reversible
    e = rng.integers(-(1 << 20), 1 << 20, size=(256, 256, 256), dtype=np.int32)
    out, _ = check_full(lib, oracle, torch, e, "reversible", None)
    assert np.array_equal(out, e)


def test_field_beyond_32_bit_offsets(lib, oracle, cuda):
    """A field of more than 2^32 values (float32 2048 x 2048 x 1040, 17 GB) at
    fixed rate 1 (one 64-bit word per block): element offsets and stream bit
    positions pass 32 bits.  Spot blocks -- the first, the last, and those
    around the 2^32-th element -- must hold the oracle's code for their 64
    values, and decompress to the oracle's decoding of it."""
    torch = cuda
    from tests.helpers import oracle_stream
    nz, ny, nx = 1040, 2048, 2048
    if torch.cuda.mem_get_info()[0] < 40 * 2**30:
        pytest.skip("needs 40 GB of free device memory")
    assert nz * ny * nx > 2**32
    g = torch.Generator(device="cuda").manual_seed(9)
    x = torch.randn((nz, ny, nx), dtype=torch.float32, device="cuda", generator=g)
    nblocks = (nz // 4) * (ny // 4) * (nx // 4)
    buf = torch.zeros(nblocks + 16, dtype=torch.int64, device="cuda")
    n = (nx, ny, nz)
    r, pos = zfp_run(lib, "compress", x.data_ptr(), capi.TYPE_FLOAT, n, (), "rate", 1, buf.data_ptr(), buf.numel() * 8)
    assert r == nblocks * 8 and pos == nblocks * 64, lib.zfp_gb300_last_error()
    out = torch.empty_like(x)
    r2, _ = zfp_run(lib, "decompress", out.data_ptr(), capi.TYPE_FLOAT, n, (), "rate", 1, buf.data_ptr(),
                    buf.numel() * 8)
    assert r2 == r, lib.zfp_gb300_last_error()
    nbx, nby = nx // 4, ny // 4
    edge = 2**32 // (ny * nx) // 4          # the block row holding element 2^32
    spots = [(0, 0, 0), (nbx - 1, nby - 1, nz // 4 - 1), (nbx - 1, nby - 1, edge - 1), (0, 0, edge),
             (17, 301, edge), (nbx - 1, 0, edge + 1)]
    for bx, by, bz in spots:
        blk = x[4 * bz:4 * bz + 4, 4 * by:4 * by + 4, 4 * bx:4 * bx + 4].cpu().numpy()
        exp, _, prm = oracle_stream(oracle, blk, "rate", 1)
        b = bx + nbx * (by + nby * bz)
        got = int(buf[b].item()) & (2**64 - 1)
        assert got == int(exp[0]), (bx, by, bz)
        ref = np.zeros_like(blk)
        oracle.decompress(exp, ref, prm, 0)
        dec = out[4 * bz:4 * bz + 4, 4 * by:4 * by + 4, 4 * bx:4 * bx + 4].cpu().numpy()
        assert np.array_equal(dec.view(np.uint32), ref.view(np.uint32)), (bx, by, bz)
    del x, out, buf
    torch.cuda.empty_cache()
