"""Host-side input generators: Gaussian and Hermite-Gauss modes at the waist
(src/modes/gaussian_modes.jl:22-33, :116-233, :288-478).  Arrays are (ny, nx)."""

from __future__ import annotations

import math

import numpy as np


def gaussian(w0, x, y):
    c = math.sqrt(math.sqrt(2.0 / math.pi) / w0)
    return (c * np.exp(-(np.asarray(y) / w0) ** 2))[:, None] * (c * np.exp(-(np.asarray(x) / w0) ** 2))[None, :]


def _hermite(n, x):
    h0 = np.ones_like(x)
    if n == 0:
        return h0
    h1 = 2.0 * x
    for k in range(1, n):
        h0, h1 = h1, 2.0 * x * h1 - 2.0 * k * h0
    return h1


def hermite_gaussian(w0, m, n, x, y):
    def one(k, s):
        s = np.asarray(s, dtype=np.float64)
        c = math.sqrt(math.sqrt(2.0 / math.pi) / w0) / math.sqrt(2.0 ** k * math.factorial(k))
        return c * _hermite(k, math.sqrt(2.0) * s / w0) * np.exp(-(s / w0) ** 2)
    return one(n, y)[:, None] * one(m, x)[None, :]


def hermite_gaussian_groups(n_groups):
    """Orders (m, n) with m + n < n_groups in the reference's order."""
    return [(m, n) for m in range(n_groups) for n in range(n_groups - m)]
