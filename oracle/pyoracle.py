"""Python front end of the test oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker.  The product never imports it.

Also holds `mode_params`, a restatement of the reference's mode setters
(src/zfp.c:751-811) that maps a mode to (minbits, maxbits, maxprec, minexp).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libzfp_ref.so")

ZTYPE = {np.dtype(np.int32): 1, np.dtype(np.int64): 2,
         np.dtype(np.float32): 3, np.dtype(np.float64): 4}
DTYPE = {v: k for k, v in ZTYPE.items()}
MIN_BITS, MAX_BITS, MAX_PREC, MIN_EXP = 1, 16658, 64, -1074


class _Field(C.Structure):
    _fields_ = [("type", C.c_int), ("n", C.c_size_t * 4), ("s", C.c_ssize_t * 4), ("data", C.c_void_p)]


class _Params(C.Structure):
    _fields_ = [("minbits", C.c_uint), ("maxbits", C.c_uint), ("maxprec", C.c_uint), ("minexp", C.c_int)]


def build(quiet: bool = True) -> str:
    """Compile liboracle.so (and the reference library when its sources exist)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + (out.stdout or "") + (out.stderr or ""))
    return LIB_PATH


REF_CUDA_LIB_PATH = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "libzfp_refcuda.so")
STAGED = os.path.join(HERE, "_ref", "src")


def reference_checkout() -> str | None:
    """The reference's source checkout on this machine: $ZFP_REFERENCE, else
    the recipe's default location (absent on the GPU host)."""
    for d in (os.environ.get("ZFP_REFERENCE"), "/root/reference"):
        if d and os.path.isfile(os.path.join(d, "src", "zfp.c")):
            return d
    return None


def reference_sources() -> str | None:
    """Where the reference's sources can be compiled from: the checkout, or
    the copy `make stage` put under oracle/_ref/src (git-ignored)."""
    d = reference_checkout()
    if d:
        return d
    return STAGED if os.path.isfile(os.path.join(STAGED, "src", "zfp.c")) else None


def stage_ref(quiet: bool = True) -> bool:
    """Copy the reference sources the recipe compiles into oracle/_ref/src, so
    that they travel with the working tree to a machine without a checkout."""
    if not reference_checkout():
        return False
    out = subprocess.run(["make", "-C", HERE, "stage"], capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("staging the reference sources failed:\n" + (out.stdout or "") + (out.stderr or ""))
    return True


def _make(target: str, path: str, quiet: bool) -> str | None:
    src = reference_sources()
    if not src:
        return path if os.path.exists(path) else None
    jobs = str(min(32, os.cpu_count() or 4))
    out = subprocess.run(["make", "-j", jobs, "-C", HERE, target, f"ZFP_REFERENCE={src}"],
                         capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"reference build ({target}) failed:\n" + (out.stdout or "") + (out.stderr or ""))
    return path


def build_ref(quiet: bool = True) -> str | None:
    """Compile the reference library (serial + OpenMP codecs) from its sources, where they are present."""
    return _make("ref", REF_LIB_PATH, quiet)


def build_ref_cuda(quiet: bool = True) -> str | None:
    """Compile the reference library with its own CUDA backend (src/cuda_zfp) for
    sm_103a into baseline/_ref: the benchmark's comparison column (it is not
    part of the checker)."""
    return _make("refcuda", REF_CUDA_LIB_PATH, quiet)


def mode_params(mode: str, arg=None, dtype=np.float32, dims: int = 3, align: bool = False):
    """(minbits, maxbits, maxprec, minexp) as the reference's setters produce them."""
    ztype = ZTYPE[np.dtype(dtype)]
    if mode == "rate":
        n = 1 << (2 * dims)
        bits = int(math.floor(n * float(arg) + 0.5))
        if ztype == 3:
            bits = max(bits, 1 + 8)
        elif ztype == 4:
            bits = max(bits, 1 + 11)
        if align:
            bits = (bits + 63) & ~63
        return (bits, bits, MAX_PREC, MIN_EXP)
    if mode == "precision":
        p = int(arg)
        return (MIN_BITS, MAX_BITS, min(p, MAX_PREC) if p else MAX_PREC, MIN_EXP)
    if mode == "accuracy":
        tol = float(arg)
        emin = MIN_EXP
        if tol > 0:
            emin = math.frexp(tol)[1] - 1
        return (MIN_BITS, MAX_BITS, MAX_PREC, emin)
    if mode == "reversible":
        return (MIN_BITS, MAX_BITS, MAX_PREC, MIN_EXP - 1)
    if mode == "expert":
        return tuple(arg)
    raise ValueError(mode)


class Oracle:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        pf, pp, pu = C.POINTER(_Field), C.POINTER(_Params), C.POINTER(C.c_uint64)
        self.lib.orc_compress.restype = C.c_uint64
        self.lib.orc_compress.argtypes = [pf, pp, pu, C.c_uint64, pu]
        self.lib.orc_compress_par.restype = C.c_uint64
        self.lib.orc_compress_par.argtypes = [pf, pp, pu, C.c_uint64, C.c_int, pu]
        self.lib.orc_decompress_par.restype = C.c_uint64
        self.lib.orc_decompress_par.argtypes = [pf, pp, pu, C.c_uint64, pu, C.c_int]
        self.lib.orc_decompress.restype = C.c_uint64
        self.lib.orc_decompress.argtypes = [pf, pp, pu, C.c_uint64]
        self.lib.orc_blocks.restype = C.c_size_t
        self.lib.orc_blocks.argtypes = [pf]
        self.lib.orc_block_maxbits.restype = C.c_uint
        self.lib.orc_block_maxbits.argtypes = [pf, pp]

    @staticmethod
    def _field(ptr: int, ztype: int, n, s) -> _Field:
        f = _Field()
        f.type = ztype
        for i in range(4):
            f.n[i] = int(n[i]) if i < len(n) else 0
            f.s[i] = int(s[i]) if i < len(s) else 0
        f.data = ptr
        return f

    @staticmethod
    def array_geometry(a: np.ndarray):
        """zfp extents/strides (fastest axis first) of a numpy array or view."""
        n = tuple(reversed(a.shape))
        s = tuple(st // a.itemsize for st in reversed(a.strides))
        return n, s

    def max_words(self, n, dtype, params) -> int:
        f = self._field(0, ZTYPE[np.dtype(dtype)], n, ())
        p = _Params(*params)
        blocks = self.lib.orc_blocks(C.byref(f))
        return (blocks * self.lib.orc_block_maxbits(C.byref(f), C.byref(p)) + 148 + 63) // 64 + 2

    def compress(self, a: np.ndarray, params, bit0: int = 0, words: np.ndarray | None = None,
                 n=None, s=None, threads: int = 0, block_ends: bool = False):
        """Compress array (or view) `a`; returns (words, end_bit[, block_end_offsets])."""
        if n is None:
            n, s = self.array_geometry(a)
        f = self._field(a.ctypes.data, ZTYPE[a.dtype], n, s)
        p = _Params(*params)
        if words is None:
            words = np.zeros(self.max_words(n, a.dtype, params) + (bit0 >> 6) + 1, dtype=np.uint64)
        wp = words.ctypes.data_as(C.POINTER(C.c_uint64))
        if threads:
            if block_ends:
                be = np.zeros(self.lib.orc_blocks(C.byref(f)), dtype=np.uint64)
                end = self.lib.orc_compress_par(C.byref(f), C.byref(p), wp, bit0, threads,
                                                be.ctypes.data_as(C.POINTER(C.c_uint64)))
                return words, int(end), be
            end = self.lib.orc_compress_par(C.byref(f), C.byref(p), wp, bit0, threads, None)
            return words, int(end)
        if block_ends:
            be = np.zeros(self.lib.orc_blocks(C.byref(f)), dtype=np.uint64)
            end = self.lib.orc_compress(C.byref(f), C.byref(p), wp, bit0,
                                        be.ctypes.data_as(C.POINTER(C.c_uint64)))
            return words, int(end), be
        end = self.lib.orc_compress(C.byref(f), C.byref(p), wp, bit0, None)
        return words, int(end)

    def decompress_par(self, words: np.ndarray, out: np.ndarray, params, threads: int, block_start=None,
                       bit0: int = 0, n=None, s=None) -> int:
        """Parallel decode; block_start = per-block start bits (None: fixed rate)."""
        if n is None:
            n, s = self.array_geometry(out)
        f = self._field(out.ctypes.data, ZTYPE[out.dtype], n, s)
        p = _Params(*params)
        w = np.ascontiguousarray(words, dtype=np.uint64)
        w = np.concatenate([w, np.zeros(2, dtype=np.uint64)])
        bs = None
        if block_start is not None:
            block_start = np.ascontiguousarray(block_start, dtype=np.uint64)
            bs = block_start.ctypes.data_as(C.POINTER(C.c_uint64))
        end = self.lib.orc_decompress_par(C.byref(f), C.byref(p), w.ctypes.data_as(C.POINTER(C.c_uint64)),
                                          bit0, bs, threads)
        return int(end)

    def decompress(self, words: np.ndarray, out: np.ndarray, params, bit0: int = 0, n=None, s=None) -> int:
        if n is None:
            n, s = self.array_geometry(out)
        f = self._field(out.ctypes.data, ZTYPE[out.dtype], n, s)
        p = _Params(*params)
        w = np.ascontiguousarray(words, dtype=np.uint64)
        # one spare word: the reader may look one word ahead
        w = np.concatenate([w, np.zeros(2, dtype=np.uint64)])
        end = self.lib.orc_decompress(C.byref(f), C.byref(p), w.ctypes.data_as(C.POINTER(C.c_uint64)), bit0)
        return int(end)
