"""The oracle against the known-answer checksums the reference ships for its
end-to-end tests (tests/constants/checksums/{1..4}d{Int32,Int64,Float,Double}.h).

The reference's own generator (tests/utils/genSmoothRandNums.c) makes the
inputs and its hashes (tests/utils/zfpHash.c) digest the results, both
compiled from the reference's sources by `make -C oracle kat`; the keys
follow tests/utils/zfpChecksums.c:73-135 and the mode parameters
tests/utils/zfpCompressionParams.c and tests/src/endtoend/zfpEndtoendBase.c:
fixed precision 2^(p+3), fixed rate 2^(p+3) (unaligned), fixed accuracy
2^-(2^p) for p = 0, 1, 2, and reversible.  For every table entry of an
end-to-end array test, the oracle's stream (its flushed bytes) and decoded
array must hash to the recorded value.  CPU only; needs the reference's
sources (its checkout, or the copy staged from it; skipped where neither exists)."""
from __future__ import annotations

import ctypes as C
import math
import os
import re
import subprocess

import numpy as np
import pytest

from oracle.pyoracle import mode_params, reference_sources

REF = reference_sources() or ""
HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), "oracle")
KAT_LIB = os.path.join(ORACLE, "_ref", "libzfpkat.so")

TYPES = {1: ("Int32", np.int32), 2: ("Int64", np.int64), 3: ("Float", np.float32), 4: ("Double", np.float64)}
ARRAY_TEST, ORIGINAL, COMPRESSED, DECOMPRESSED = 2, 0, 1, 2
MODES = {"rate": 2, "precision": 3, "accuracy": 4, "reversible": 5}   # zfp_mode values (include/zfp.h)


@pytest.fixture(scope="module")
def kat():
    if not REF or not os.path.isdir(os.path.join(REF, "tests", "utils")):
        pytest.skip("reference sources not available here")
    r = subprocess.run(["make", "-C", ORACLE, "kat", f"ZFP_REFERENCE={REF}"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("reference test utilities do not build here: " + r.stderr[-300:])
    lib = C.CDLL(KAT_LIB)
    lib.kat_generate.restype = C.c_void_p
    lib.kat_generate.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    lib.kat_free.argtypes = [C.c_void_p]
    lib.kat_hash_stream.restype = C.c_uint64
    lib.kat_hash_stream.argtypes = [C.c_void_p, C.c_size_t]
    lib.kat_hash_array.restype = C.c_uint64
    lib.kat_hash_array.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_ssize_t]
    return lib


def table(dims, tname):
    path = os.path.join(REF, "tests", "constants", "checksums", f"{dims}d{tname}.h")
    rows = re.findall(r"\{UINT64C\((0x[0-9a-f]+)\),\s*UINT64C\((0x[0-9a-f]+)\),\s*UINT64C\((0x[0-9a-f]+)\)\}",
                      open(path).read())
    return {(int(a, 16), int(b, 16)): int(c, 16) for a, b, c in rows}


def key1(subject, mode, param):
    return ((((ARRAY_TEST << 2) + subject) << 3) + mode << 4) + param


def key2(n):
    """zfpChecksums.c:104-132: n = extents, fastest first."""
    n = [v for v in n if v]
    if len(n) == 1:
        return n[0] - 1
    if len(n) == 2:
        return ((n[0] - 1) << 24) + n[1] - 1
    if len(n) == 3:
        return ((((n[0] - 1) << 16) + n[1] - 1) << 16) + n[2] - 1
    return ((((((n[0] - 1) << 12) + n[1] - 1) << 12) + n[2] - 1) << 12) + n[3] - 1


def params(mode, p):
    if mode == "precision":
        return 1 << (p + 3)
    if mode == "rate":
        return float(1 << (p + 3))
    if mode == "accuracy":
        return math.ldexp(1.0, -(1 << p))
    return None


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
@pytest.mark.parametrize("ztype", [1, 2, 3, 4], ids=lambda t: TYPES[t][0])
def test_oracle_matches_reference_checksums(kat, oracle, dims, ztype):
    tname, dtype = TYPES[ztype]
    tab = table(dims, tname)
    side, total = C.c_size_t(), C.c_size_t()
    ptr = kat.kat_generate(ztype, dims, C.byref(side), C.byref(total))
    try:
        bits = np.dtype(dtype).itemsize * 8
        arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(total.value * bits // 8,))
        vals = arr.view(dtype).reshape((side.value,) * dims).copy()
    finally:
        kat.kat_free(ptr)
    n = [side.value] * dims
    k2 = key2(n)
    # the generated input is the reference's
    assert kat.kat_hash_array(bits, vals.ctypes.data, vals.size, 1) == tab[(key1(ORIGINAL, 0, 0), k2)]
    seen = {(key1(ORIGINAL, 0, 0), k2)}
    for mode, mval in MODES.items():
        if mode == "accuracy" and np.dtype(dtype).kind == "i":
            continue
        for p in range(1 if mode == "reversible" else 3):
            want_s = tab.get((key1(COMPRESSED, mval, p), k2))
            want_d = tab.get((key1(DECOMPRESSED, mval, p), k2))
            if want_s is None and want_d is None:
                continue
            prm = mode_params(mode, params(mode, p), dtype, dims)
            words, end = oracle.compress(vals, prm)
            nbytes = (end + 63) // 64 * 8
            if want_s is not None:
                assert kat.kat_hash_stream(words.ctypes.data, nbytes) == want_s, (mode, p)
                seen.add((key1(COMPRESSED, mval, p), k2))
            if want_d is not None:
                out = np.zeros_like(vals)
                oracle.decompress(words, out, prm, 0)
                assert kat.kat_hash_array(bits, out.ctypes.data, out.size, 1) == want_d, (mode, p)
                seen.add((key1(DECOMPRESSED, mval, p), k2))
    # every end-to-end array entry of the table was checked
    assert seen == {k for k in tab if k[0] >> 9 == ARRAY_TEST}
