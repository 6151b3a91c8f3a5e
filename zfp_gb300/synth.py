"""Synthetic fields for tests and benchmarks (no dataset is involved).

smooth_field: sum of 8 sinusoids sin(2*pi*(k.x)/64 + phi) with integer
wavevector components uniform in 1..4, amplitudes N(0,1), phases U[0,2pi),
plus N(0, noise^2) noise -- the generator the benchmark configurations name.
Shapes are numpy order (slowest axis first); x is the zfp index vector.
"""
from __future__ import annotations

import math

import numpy as np


def _terms(seed: int, dims: int, terms: int = 8):
    rng = np.random.default_rng(seed)
    k = rng.integers(1, 5, size=(terms, dims))
    amp = rng.standard_normal(terms)
    phase = rng.uniform(0.0, 2.0 * math.pi, size=terms)
    return rng, k, amp, phase


def smooth_field(shape, dtype=np.float32, seed: int = 0, noise: float = 1e-3, scale: float = 1.0) -> np.ndarray:
    """numpy version (CPU), for small and medium fields."""
    dims = len(shape)
    rng, k, amp, phase = _terms(seed, dims)
    axes = [np.arange(n, dtype=np.float64) for n in reversed(shape)]  # x, y, z, w
    out = np.zeros(shape, dtype=np.float64)
    for j in range(len(amp)):
        arg = np.zeros(shape, dtype=np.float64) + phase[j]
        for a in range(dims):
            view = [1] * dims
            view[dims - 1 - a] = shape[dims - 1 - a]
            arg = arg + (2.0 * math.pi * k[j, a] / 64.0) * axes[a].reshape(view)
        out += amp[j] * np.sin(arg)
    if noise:
        out += noise * rng.standard_normal(shape)
    return (scale * out).astype(dtype)


def smooth_field_torch(shape, dtype, seed: int = 0, noise: float = 1e-3, scale: float = 1.0, device="cuda"):
    """torch version (generated on the GPU), for full-size benchmark fields."""
    import torch

    dims = len(shape)
    _, k, amp, phase = _terms(seed, dims)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = torch.zeros(shape, dtype=torch.float64 if dtype == torch.float64 else torch.float32, device=device)
    axes = [torch.arange(n, device=device, dtype=out.dtype) for n in reversed(shape)]
    for j in range(len(amp)):
        arg = torch.full(shape, float(phase[j]), dtype=out.dtype, device=device)
        for a in range(dims):
            view = [1] * dims
            view[dims - 1 - a] = shape[dims - 1 - a]
            arg += (2.0 * math.pi * float(k[j, a]) / 64.0) * axes[a].reshape(view)
        out += float(amp[j]) * torch.sin(arg)
        del arg
    if noise:
        out += noise * torch.randn(shape, generator=g, device=device, dtype=out.dtype)
    if scale != 1.0:
        out *= scale
    return out.to(dtype)
