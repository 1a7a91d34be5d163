"""Host-side input generators: Gaussian, Hermite-Gauss and Laguerre-Gauss modes, at the
waist or propagated to a distance z (src/modes/gaussian_modes.jl).

The mode objects mirror the reference's constructors by their positional arguments:

    Gaussian(w0) | Gaussian(w0x, w0y) | Gaussian(w0, lam, z) | Gaussian(w0x, w0y, lam, z)
    HermiteGaussian(w0, m, n) | HermiteGaussian(w0x, w0y, m, n)
    HermiteGaussian(w0, m, n, lam, z) | HermiteGaussian(w0x, w0y, m, n, lam, z)
    LaguerreGaussian(w0, p, l; kind) | LaguerreGaussian(w0, p, l, lam, z; kind)

and are evaluated on grid vectors: ``mode(x, y)`` returns the (ny, nx) complex128 array
whose element [j, i] is the mode at (x[i], y[j]) -- the memory layout of the reference's
nx x ny Julia array -- and ``mode(x, y, out=a)`` fills ``a`` in place.  Everything is
computed in float64."""

from __future__ import annotations

import cmath
import math

import numpy as np


def _gaussian_norm(w0):
    # gaussian_normalization_constant (gaussian_modes.jl:22-24)
    return math.sqrt(math.sqrt(2.0 / math.pi) / w0)


def _hg_norm(m):
    # hg_normalization_constant (gaussian_modes.jl:26-28)
    return 1.0 / math.sqrt(2.0 ** m * math.factorial(m))


def _hermite(n, x):
    """Physicists' Hermite polynomial H_n(x) by its three-term recurrence."""
    x = np.asarray(x)
    h0 = np.ones_like(x)
    if n == 0:
        return h0
    h1 = 2.0 * x
    for k in range(1, n):
        h0, h1 = h1, 2.0 * x * h1 - 2.0 * k * h0
    return h1


class Gaussian1D:
    """One-dimensional Gaussian mode at the waist, or propagated to z with wavelength
    lam (gaussian_modes.jl:80-127): C exp(i k x^2 / (2 q(z))) exp(i k z), with
    q(z) = z - i zR, zR = pi w0^2 / lam and C = N sqrt(q(0) / q(z)).  ``norm_constant``
    sets the peak intensity instead of unit power."""

    def __init__(self, w0, lam=None, z=None, constant_phase=True, norm_constant=None):
        if (lam is None) != (z is None):
            raise TypeError("Gaussian1D takes both lam and z, or neither")
        self.w0 = float(w0)
        nc = _gaussian_norm(self.w0) if norm_constant is None else math.sqrt(norm_constant)
        self.propagated = lam is not None
        if not self.propagated:
            self.C = complex(nc)
            self.e_arg = -1.0 / self.w0 ** 2
            self.wz = self.w0
            self.eikz = 1.0 + 0j
            return
        lam, z = float(lam), float(z)
        zr = math.pi * self.w0 ** 2 / lam
        q0, qz = complex(0.0, -zr), complex(z, -zr)
        k = 2.0 * math.pi / lam
        self.lam, self.z, self.qz = lam, z, qz
        self.wz = self.w0 * math.sqrt(1.0 + (z / zr) ** 2)
        self.eikz = cmath.exp(1j * k * z) if constant_phase else 1.0 + 0j
        self.C = nc * cmath.sqrt(q0 / qz)
        self.e_arg = 1j * k / (2.0 * qz)

    def exp_arg(self, x):
        return self.e_arg * np.asarray(x, dtype=np.float64) ** 2

    def __call__(self, x):
        return self.C * np.exp(self.exp_arg(x)) * self.eikz


class HermiteGaussian1D:
    """HG_n in one dimension (gaussian_modes.jl:253-326): C H_n(sqrt(2) x / w(z)) g(x),
    with C = (2^n n!)^(-1/2) (-conj(q) / q)^(n/2) for the propagated mode."""

    def __init__(self, w0, n, lam=None, z=None, constant_phase=True):
        if int(n) != n or n < 0:
            raise ValueError("the mode number must be a non-negative integer")
        self.n = int(n)
        self.g = Gaussian1D(w0, lam, z, constant_phase=constant_phase)
        self.C = complex(_hg_norm(self.n))
        if self.g.propagated:
            qz = self.g.qz
            self.C *= (-qz.conjugate() / qz) ** (self.n / 2.0)

    def hermite(self, x):
        return _hermite(self.n, math.sqrt(2.0) * np.asarray(x, dtype=np.float64) / self.g.wz)

    def __call__(self, x):
        return self.C * self.hermite(x) * self.g(x)


class _Mode2D:
    def _eval(self, x, y):
        raise NotImplementedError

    def __call__(self, x, y, out=None):
        v = self._eval(np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64))
        if out is None:
            return v
        if out.shape != v.shape:
            raise ValueError(f"out has shape {out.shape}, the grid gives {v.shape}")
        out[...] = v
        return out


class Gaussian(_Mode2D):
    """Two-dimensional Gaussian mode (gaussian_modes.jl:130-233), circular or
    elliptical, at the waist or propagated: Gaussian(w0), Gaussian(w0x, w0y),
    Gaussian(w0, lam, z), Gaussian(w0x, w0y, lam, z)."""

    def __init__(self, *args, constant_phase=True, norm_constant=None):
        if len(args) == 1:
            wx = wy = args[0]
            lam = z = None
        elif len(args) == 2:
            wx, wy = args
            lam = z = None
        elif len(args) == 3:
            wx = wy = args[0]
            lam, z = args[1:]
        elif len(args) == 4:
            wx, wy, lam, z = args
        else:
            raise TypeError("Gaussian takes (w0), (w0x, w0y), (w0, lam, z) or (w0x, w0y, lam, z)")
        self.gx = Gaussian1D(wx, lam, z, constant_phase=constant_phase, norm_constant=norm_constant)
        # the peak intensity and the constant phase are counted once, in gx
        self.gy = Gaussian1D(wy, lam, z, constant_phase=False, norm_constant=None if norm_constant is None else 1.0)

    def _eval(self, x, y):
        c = self.gx.C * self.gy.C * self.gx.eikz
        return c * np.exp(self.gy.exp_arg(y)[:, None] + self.gx.exp_arg(x)[None, :])


class HermiteGaussian(_Mode2D):
    """HG_{m,n} (gaussian_modes.jl:329-426): HermiteGaussian(w0, m, n),
    HermiteGaussian(w0x, w0y, m, n), HermiteGaussian(w0, m, n, lam, z),
    HermiteGaussian(w0x, w0y, m, n, lam, z); m is the order along x, n along y."""

    def __init__(self, *args, constant_phase=True):
        if len(args) == 3:
            wx = wy = args[0]
            m, n = args[1:]
            lam = z = None
        elif len(args) == 4:
            wx, wy, m, n = args
            lam = z = None
        elif len(args) == 5:
            wx = wy = args[0]
            m, n, lam, z = args[1:]
        elif len(args) == 6:
            wx, wy, m, n, lam, z = args
        else:
            raise TypeError("HermiteGaussian takes (w0, m, n), (w0x, w0y, m, n), (w0, m, n, lam, z) "
                            "or (w0x, w0y, m, n, lam, z)")
        self.m, self.n = int(m), int(n)
        self.hgx = HermiteGaussian1D(wx, m, lam, z, constant_phase=constant_phase)
        self.hgy = HermiteGaussian1D(wy, n, lam, z, constant_phase=False)

    def _eval(self, x, y):
        mx, my = self.hgx, self.hgy
        c = mx.C * mx.g.C * my.C * my.g.C * mx.g.eikz
        fx = mx.hermite(x) * np.exp(mx.g.exp_arg(x))
        fy = my.hermite(y) * np.exp(my.g.exp_arg(y))
        return c * (fy[:, None] * fx[None, :])


def _laguerre(p, l, x):
    """Generalised Laguerre polynomial L_p^l(x) by its three-term recurrence."""
    x = np.asarray(x)
    if p == 0:
        return np.ones_like(x)
    a, b = np.ones_like(x), 1.0 + l - x
    for k in range(2, p + 1):
        a, b = b, ((2 * k + l - 1 - x) * b - (k + l - 1) * a) / k
    return b


class LaguerreGaussian(_Mode2D):
    """LG_{p,l} (gaussian_modes.jl:480-640): LaguerreGaussian(w0, p, l) at the waist or
    LaguerreGaussian(w0, p, l, lam, z) propagated, with the azimuthal factor
    exp(i l phi) (kind "vortex"), sqrt(2) cos(l phi) ("even") or sqrt(2) sin(l phi)
    ("odd")."""

    def __init__(self, *args, constant_phase=True, kind="vortex"):
        if len(args) == 3:
            w0, p, l = args
            lam = z = None
        elif len(args) == 5:
            w0, p, l, lam, z = args
        else:
            raise TypeError("LaguerreGaussian takes (w0, p, l) or (w0, p, l, lam, z)")
        if int(p) != p or p < 0 or int(l) != l:
            raise ValueError("p must be a non-negative integer and l an integer")
        kind = str(kind).lstrip(":")
        if kind not in ("vortex", "even", "odd"):
            raise ValueError("kind must be vortex, even or odd")
        self.w0, self.p, self.l, self.kind = float(w0), int(p), int(l), kind
        al = abs(self.l)
        norm = math.sqrt(2.0 * math.factorial(self.p) / (math.pi * math.factorial(self.p + al))) / self.w0
        self.propagated = lam is not None
        if not self.propagated:
            self.C = complex(norm)
            return
        lam, z = float(lam), float(z)
        zr = math.pi * self.w0 ** 2 / lam
        q0, qz = complex(0.0, -zr), complex(z, -zr)
        k = 2.0 * math.pi / lam
        self.wz = self.w0 * math.sqrt(1.0 + (z / zr) ** 2)
        self.eikz = cmath.exp(1j * k * z) if constant_phase else 1.0 + 0j
        self.e_arg = 1j * k / (2.0 * qz)
        self.C = norm * (q0 / qz) * (-qz.conjugate() / qz) ** (self.p + al / 2.0)

    def _angular(self, x, y):
        phi = np.arctan2(y[:, None], x[None, :])
        if self.kind == "vortex":
            return np.exp(1j * self.l * phi)
        return math.sqrt(2.0) * (np.cos(self.l * phi) if self.kind == "even" else np.sin(self.l * phi))

    def _eval(self, x, y):
        al = abs(self.l)
        r2 = y[:, None] ** 2 + x[None, :] ** 2
        if not self.propagated:
            s = r2 / self.w0 ** 2
            v = self.C * (math.sqrt(2.0) * np.sqrt(s)) ** al * _laguerre(self.p, al, 2.0 * s) * np.exp(-s)
            return v * self._angular(x, y)
        rl = (math.sqrt(2.0) * np.sqrt(r2) / self.wz) ** al
        v = self.C * rl * _laguerre(self.p, al, 2.0 * r2 / self.wz ** 2) * np.exp(self.e_arg * r2)
        return v * self._angular(x, y) * self.eikz


def gaussian(w0, x, y):
    """Gaussian(w0) at the waist evaluated on (x, y): array of shape (ny, nx)."""
    return Gaussian(w0)(x, y)


def hermite_gaussian(w0, m, n, x, y):
    """HermiteGaussian(w0, m, n) at the waist evaluated on (x, y)."""
    return HermiteGaussian(w0, m, n)(x, y)


def hermite_gaussian_groups(w0, n_groups=None):
    """All HG_{m,n} with m + n < n_groups, m outer and n inner, as the reference builds
    them (gaussian_modes.jl:469-478): ``hermite_gaussian_groups(w0, n_groups)`` returns the
    HermiteGaussian modes; ``hermite_gaussian_groups(n_groups)`` returns their (m, n)
    orders."""
    if n_groups is None:
        n_groups, w0 = w0, None
    if int(n_groups) != n_groups or n_groups <= 0:
        raise ValueError("n_groups must be a positive integer")
    orders = [(m, n) for m in range(int(n_groups)) for n in range(int(n_groups) - m)]
    return orders if w0 is None else [HermiteGaussian(w0, m, n) for m, n in orders]
