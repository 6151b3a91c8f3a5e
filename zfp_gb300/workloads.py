"""Synthetic workloads of the batched and serving benchmarks, shared by
bench.py and the tests so that both see exactly the same inputs.

batch_arrays: 4096 independent 3D float32 arrays, each extent log-uniform in
[8, 128] (seed 2), smooth-field generator with amplitude scale 10^U(-3,3);
every other array fixed-rate with rate in {4, 8, 12, 16, 24, 32}, the others
fixed-accuracy with tolerance 10^U(-5,-2).

ServingMix: a stream of requests, 70% compress and 30% decompress, each a
2D or 3D float32/float64 field of raw size log-uniform in [16 KiB, 256 MiB]
(seed 3), fixed-accuracy tolerance 1e-4 x the field's range.  Fields are
views (leading sub-squares / sub-cubes) of four resident generated fields,
one per (type, dimensionality); decompress requests draw from 64 template
requests of the same distribution.
"""
from __future__ import annotations

import numpy as np

from . import synth


def batch_arrays(torch, count: int = 4096, seed: int = 2):
    """[(tensor on cuda, mode, arg)] in generation order."""
    rng = np.random.default_rng(seed)
    arrays = []
    for i in range(count):
        shape = tuple(int(v) for v in np.exp(rng.uniform(np.log(8), np.log(128), size=3)).astype(int))
        scale = float(10.0 ** rng.uniform(-3, 3))
        x = synth.smooth_field_torch(shape, torch.float32, seed=int(rng.integers(1 << 31)), noise=1e-2, scale=scale)
        if i % 2 == 0:
            mode, arg = "rate", float(rng.choice([4, 8, 12, 16, 24, 32]))
        else:
            mode, arg = "accuracy", float(10.0 ** rng.uniform(-5, -2))
        arrays.append((x, mode, arg))
    return arrays


class ServingMix:
    """The request stream of the serving benchmark (see the module docstring)."""

    TEMPLATES = 64

    def __init__(self, torch, count: int, smax: int = 256 << 20, rate: float = 6000.0, seed: int = 3):
        self.torch = torch
        self.rng = np.random.default_rng(seed)
        self.smax = smax
        self.bases = {}
        for dt, esz in ((torch.float32, 4), (torch.float64, 8)):
            for dims in (2, 3):
                side = int((smax / esz) ** (1.0 / dims)) + 1
                self.bases[(esz, dims)] = synth.smooth_field_torch((side,) * dims, dt, seed=seed + esz + dims,
                                                                   noise=1e-2)
        self.templates = [self._field() for _ in range(self.TEMPLATES)]
        self.requests = []
        for _ in range(count):
            if self.rng.random() < 0.7:
                self.requests.append(dict(self._field(), direction=0))
            else:
                t = int(self.rng.integers(len(self.templates)))
                self.requests.append(dict(self.templates[t], direction=1, template=t))
        gaps = self.rng.exponential(1.0 / rate, size=count)
        self.arrivals = np.cumsum(gaps) - gaps[0]

    def _field(self):
        esz = 4 if self.rng.random() < 0.5 else 8
        dims = 2 if self.rng.random() < 0.5 else 3
        size = float(np.exp(self.rng.uniform(np.log(16 << 10), np.log(self.smax))))
        base = self.bases[(esz, dims)]
        n = max(4, min(base.shape[0], int(round((size / esz) ** (1.0 / dims)))))
        view = base[(slice(0, n),) * dims]
        lo, hi = self.torch.aminmax(view)
        return dict(view=view, esz=esz, dims=dims, n=n, tol=1e-4 * float(hi - lo), raw=view.numel() * esz)
