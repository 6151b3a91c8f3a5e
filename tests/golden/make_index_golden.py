"""Golden vectors for zfp's block index formats (include/zfp/index.hpp).

Run in a container where the reference's headers exist: index_gen.cpp is
compiled against them (the index classes are header-only) into oracle/_ref/,
fed seeded block sizes, and the packed index bytes, the range and every
block offset it reports are stored in index_golden.npz, so the library's own
packer and unpacker (zfp_gb300_index_pack / _unpack) can be checked against
the reference anywhere.

    python tests/golden/make_index_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("ZFP_REFERENCE", "/root/reference")
BIN = os.path.join(ROOT, "oracle", "_ref", "index_gen")

MAX_BITS = 16658  # ZFP_MAX_BITS, include/zfp.h


def build():
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++11", "-I", os.path.join(REF, "include"),
                    os.path.join(HERE, "index_gen.cpp"), "-o", BIN], check=True)


def run(fmt, dims, sizes):
    inp = f"{fmt} {dims} {len(sizes)} " + " ".join(str(int(s)) for s in sizes)
    out = subprocess.run([BIN], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    nbytes = int(out[0])
    packed = np.frombuffer(bytes.fromhex(out[1]), dtype=np.uint8) if nbytes else np.zeros(0, np.uint8)
    assert len(packed) == nbytes
    rng_bits = int(out[2])
    offsets = np.array([int(v) for v in out[3].split()], dtype=np.uint64)
    return packed, rng_bits, offsets


def main():
    build()
    rng = np.random.default_rng(2024)
    cases, arrays = [], {}
    specs = [(1, 3, 1000, MAX_BITS), (1, 2, 1, MAX_BITS), (2, 3, 1001, MAX_BITS), (2, 3, 4, MAX_BITS),
             (2, 2, 1003, 300)]
    for dims in (1, 2, 3, 4):
        hbits = 2 * (dims - 1)
        specs.append((3, dims, 1003, (1 << (hbits + 8)) - 1))
        specs.append((3, dims, 16, (1 << (hbits + 8)) - 1))
    for i, (fmt, dims, n, hi) in enumerate(specs):
        sizes = rng.integers(0 if fmt != 3 else 1, hi + 1, size=n).astype(np.uint64)
        packed, rng_bits, offsets = run(fmt, dims, sizes)
        key = f"c{i}"
        arrays[f"sizes_{key}"] = sizes
        arrays[f"packed_{key}"] = packed
        arrays[f"offsets_{key}"] = offsets
        cases.append({"key": key, "format": fmt, "dims": dims, "nblocks": n, "range": rng_bits})
    np.savez_compressed(os.path.join(HERE, "index_golden.npz"), **arrays)
    with open(os.path.join(HERE, "index_golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/index_gen.cpp over include/zfp/index.hpp", "cases": cases}, f,
                  indent=1)
    print(f"{len(cases)} index cases")


if __name__ == "__main__":
    sys.exit(main())
