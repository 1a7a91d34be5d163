"""FP64 CPU oracle for FluxOptics.jl's scalar-propagation hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path may import this module:
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use it, and only as the checker / the timed CPU restatement.

This is a numpy/scipy (pocketfft, complex128) restatement of the reference's
algorithm.  The reference is Julia (FluxOptics.jl v0.1.0) and cannot be run in
this environment (no Julia toolchain), so the restatement is pinned by the
reference's own property and known-answer tests (AS/RS unitarity, AS energy
conservation, SquaredIntensityDifference closed form, HG00 == Gaussian, Fista
convergence, Phase angle checks), by the analytic paraxial Gaussian beam, and
by central finite differences of every gradient.  No reference test fixes the
values of a propagated field or a gradient, so field-level parity is
"partially pinned" (properties + analytic beams), not golden-vector pinned.

Array layout (matches the GPU path): a field batch is a C-ordered array of
shape ``(..., ny, nx)``; the last axis is the reference's first (fastest,
column-major) Julia dimension ``x``.  Trailing Julia dims (wavelengths x modes)
become the leading numpy axes, flattened to ``B`` fields.

Third-party arithmetic the reference relies on and which is restated here:
FFTW.jl 1.9.0 / FFTW_jll 3.3.11 (unnormalised forward FFT, 1/N-normalised
inverse, ``plan_fft!``/``plan_ifft!`` in ``src/FFTutils.jl:13-28``) and
AbstractFFTs 1.5.0 ``fftfreq``.
"""

from __future__ import annotations

import math
import os

import numpy as np
import scipy.fft as sfft

FORWARD = 1
BACKWARD = -1

_WORKERS = int(os.environ.get("FO_ORACLE_WORKERS", "1"))


def set_workers(n: int) -> None:
    """Number of pocketfft threads used by the oracle (the CPU baseline sets it)."""
    global _WORKERS
    _WORKERS = max(1, int(n))


def fft2(u):
    # src/FFTutils.jl:20-23 -- unnormalised forward transform over the two spatial dims
    return sfft.fft2(u, axes=(-2, -1), workers=_WORKERS)


def ifft2(u):
    # src/FFTutils.jl:25-28 -- inverse transform with 1/(nx*ny)
    return sfft.ifft2(u, axes=(-2, -1), workers=_WORKERS)


# ---------------------------------------------------------------------------
# Grids, modes, field utilities
# ---------------------------------------------------------------------------

def spatial_vectors(ns, ds, offset=None):
    """Centred grid ``((0:n-1) - (n-1)/2)*d - c`` (src/GridUtils.jl:56-60).

    ``ns``/``ds`` are given in Julia order (x first)."""
    if offset is None:
        offset = (0.0,) * len(ns)
    return tuple((np.arange(n) - (n - 1) / 2.0) * d - c for n, d, c in zip(ns, ds, offset))


def gaussian(w0, x, y):
    """Gaussian(w0) at the waist: sqrt(2/pi)/w0 * exp(-(x^2+y^2)/w0^2).

    src/modes/gaussian_modes.jl:22-24 (normalisation), :116-127 (eval), :216-233 (2-D).
    Returns an array of shape (ny, nx)."""
    c = math.sqrt(math.sqrt(2.0 / math.pi) / w0)
    gx = c * np.exp(-(x / w0) ** 2)
    gy = c * np.exp(-(y / w0) ** 2)
    return (gy[:, None] * gx[None, :]).astype(np.complex128)


def _hermite(n, x):
    # physicists' Hermite polynomial (src/modes/gaussian_modes.jl:238-250)
    h0 = np.ones_like(x)
    if n == 0:
        return h0
    h1 = 2.0 * x
    for k in range(1, n):
        h0, h1 = h1, 2.0 * x * h1 - 2.0 * k * h0
    return h1


def hermite_gaussian(w0, m, n, x, y):
    """HG_{m,n} at the waist (src/modes/gaussian_modes.jl:288-426)."""
    def one(w, k, s):
        c = math.sqrt(math.sqrt(2.0 / math.pi) / w) / math.sqrt(2.0 ** k * math.factorial(k))
        return c * _hermite(k, math.sqrt(2.0) * s / w) * np.exp(-(s / w) ** 2)
    return (one(w0, n, y)[:, None] * one(w0, m, x)[None, :]).astype(np.complex128)


def hermite_gaussian_groups(n_groups):
    """Mode orders (m, n) with m + n < n_groups, in the reference's order
    (src/modes/gaussian_modes.jl:469-478)."""
    out = []
    for m in range(n_groups):
        for n in range(n_groups - m):
            out.append((m, n))
    return out


def power(u, ds):
    """sum |u|^2 * prod(ds) per field (src/Fields.jl:843-846)."""
    return np.sum(np.abs(u) ** 2, axis=(-2, -1)) * float(np.prod(ds))


def normalize_power(u, ds, target=1.0):
    """In-place power normalisation per field (src/Fields.jl:889-892)."""
    p = power(u, ds)
    u *= np.sqrt(target / p)[..., None, None]
    return u


def coupling_efficiency(u, v):
    """|<u,v>|^2/(|u|^2 |v|^2) per field (src/Fields.jl:748-756)."""
    num = np.abs(np.sum(np.conj(u) * v, axis=(-2, -1))) ** 2
    den = np.sum(np.abs(u) ** 2, axis=(-2, -1)) * np.sum(np.abs(v) ** 2, axis=(-2, -1))
    return num / den


def rel_l2(a, b):
    """Relative L2 error ||a-b|| / ||b|| (b is the reference)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


# ---------------------------------------------------------------------------
# Transfer functions
# ---------------------------------------------------------------------------

def fftfreqs(nx, ny, dx, dy):
    """Frequency vectors in FFT order (src/optical_components/freespace_propagators/
    fourier_kernel.jl:17-18)."""
    return np.fft.fftfreq(nx, dx), np.fft.fftfreq(ny, dy)


def as_kernel(nx, ny, dx, dy, lam, z, n0=1.0):
    """On-axis angular-spectrum transfer function, shape (ny, nx).

    H = cis(2 pi z sqrt(complex(n0^2/lam^2) - fx^2 - fy^2)); for z < 0 the kernel
    is conj(H(-z)), so evanescent waves decay both ways
    (src/optical_components/freespace_propagators/angular_spectrum.jl:1-12)."""
    fx, fy = fftfreqs(nx, ny, dx, dy)
    lam_m = lam / n0
    f2 = 1.0 / lam_m ** 2
    arg = (f2 - fx[None, :] ** 2 - fy[:, None] ** 2).astype(np.complex128)
    za = abs(z)
    h = np.exp(1j * 2.0 * np.pi * za * np.sqrt(arg))
    return h if z >= 0 else np.conj(h)


def as_kernel_general(nx, ny, dx, dy, lam, z, n0=1.0, paraxial=False, theta=(0.0, 0.0), track_tilts=False,
                      filt=None):
    """Paraxial and tilted angular-spectrum transfer functions, shape (ny, nx)
    (angular_spectrum.jl:27-76); lm = lam / n0, f0 = sin(theta) / lm.

    paraxial: cis(-pi lm z ((fx+f0x)^2 + (fy+f0y)^2) - off + 2 pi z / lm),
              off = track_tilts ? 2 (f0x fx + f0y fy) : 0, filter(fx, fy);
    tilted  : cis(2 pi z (sqrt(1/lm^2 - (fx+f0x)^2 - (fy+f0y)^2) + off)),
              off = track_tilts ? (f0x fx + f0y fy) lm : 0, filter(fx+f0x, fy+f0y),
              conj(H(-z)) for z < 0;
    neither : the on-axis kernel times filter(fx, fy)."""
    fx, fy = fftfreqs(nx, ny, dx, dy)
    FX, FY = fx[None, :] + 0 * fy[:, None], fy[:, None] + 0 * fx[None, :]
    lm = lam / n0
    f0x, f0y = np.sin(theta[0]) / lm, np.sin(theta[1]) / lm
    if paraxial:
        off = 2 * (f0x * FX + f0y * FY) if track_tilts else 0.0
        h = np.exp(1j * (-np.pi * lm * z * ((FX + f0x) ** 2 + (FY + f0y) ** 2) - off + 2 * np.pi * z / lm))
        if filt is not None:
            h = h * filt(FX, FY)
        return h
    tilted = theta[0] != 0.0 or theta[1] != 0.0
    gx, gy = (FX + f0x, FY + f0y) if tilted else (FX, FY)
    off = (f0x * FX + f0y * FY) * lm if (tilted and track_tilts) else 0.0
    za = abs(z)
    h = np.exp(1j * 2 * np.pi * za * (np.sqrt((1 / lm ** 2 - gx ** 2 - gy ** 2).astype(np.complex128)) + off))
    if filt is not None:
        h = h * filt(gx, gy)
    # z < 0: conj of the z > 0 kernel, filter value included (angular_spectrum.jl:9-12, 55-60)
    return np.conj(h) if z < 0 else h


def rs_kernel_spatial(n_x, n_y, dx, dy, lam, z, m_x=None, m_y=None):
    """Rayleigh-Sommerfeld impulse response sampled on offsets in FFT order.

    h = nrm * cis(k r)/r * (z/r) * (1/r - i k), nrm = dx*dy/(2 pi), k = 2 pi/lam
    (rayleigh_sommerfeld.jl:1-12, :660).  Offsets are circshift((1-n):(n-1), n)*d
    on a grid of length 2n-1 (convolution_kernel.jl:492); with ``m_x``/``m_y``
    larger than 2n-1 the same samples are placed on an m-point circular grid
    (0..n-1 at the start, -(n-1)..-1 at the end, zeros between)."""
    def offsets(n, m):
        if m is None:
            m = 2 * n - 1
        o = np.zeros(m)
        valid = np.zeros(m, dtype=bool)
        o[:n] = np.arange(n)
        valid[:n] = True
        o[m - (n - 1):] = np.arange(-(n - 1), 0)
        valid[m - (n - 1):] = True
        return o, valid
    ox, vx = offsets(n_x, m_x)
    oy, vy = offsets(n_y, m_y)
    x = ox[None, :] * dx
    y = oy[:, None] * dy
    za = abs(z)
    k = 2.0 * np.pi / lam
    r = np.sqrt(x ** 2 + y ** 2 + za ** 2)
    nrm = dx * dy / (2.0 * np.pi)
    h = nrm * (np.exp(1j * k * r) / r) * (za / r) * (1.0 / r - 1j * k)
    h = h * (vy[:, None] & vx[None, :])
    return h if z >= 0 else np.conj(h)


def rs_kernel(n_x, n_y, dx, dy, lam, z, m_x=None, m_y=None):
    """FFT of the sampled RS kernel (convolution_kernel.jl:47-55, unnormalised fft!)."""
    return fft2(rs_kernel_spatial(n_x, n_y, dx, dy, lam, z, m_x, m_y))


def rs_valid_distance(nx, ny, dx, dy, lam):
    """Critical distance below which RSProp warns (rayleigh_sommerfeld.jl:29-36)."""
    if dx < lam / 2 and dy < lam / 2:
        return 0.0
    zx = 0.0 if dx < lam / 2 else (nx * dx / 2) * math.sqrt(4 * dx ** 2 / lam ** 2 - 1)
    zy = 0.0 if dy < lam / 2 else (ny * dy / 2) * math.sqrt(4 * dy ** 2 / lam ** 2 - 1)
    return max(zx, zy)


def _lams(lambdas, nb):
    lam = np.broadcast_to(np.asarray(lambdas, dtype=np.float64).ravel(), (nb,)) \
        if np.ndim(lambdas) else np.full(nb, float(lambdas))
    return np.asarray(lam)


# ---------------------------------------------------------------------------
# Free-space propagators
# ---------------------------------------------------------------------------

def asprop(u, dx, dy, lambdas, z, direction=FORWARD, n0=1.0, paraxial=False, tilts=None, track_tilts=False,
           filt=None):
    """ASProp: u <- IFFT2(conj_direction(H) * FFT2(u)) per field.

    Sequence (ft, ASKernelProp, ift) of angular_spectrum.jl:193-234; Backward
    applies conj(H) (abstract_kernel.jl:36,45 with OpticalComponents.jl:919-925).
    ``u`` has shape (..., ny, nx); ``lambdas`` is a scalar or one value per field;
    ``tilts`` is None or one (theta_x, theta_y) pair (shared) or one per field;
    ``paraxial``, ``track_tilts`` and ``filt`` (a function of (fx, fy)) select
    as_kernel_general."""
    u = np.asarray(u, dtype=np.complex128)
    shp = u.shape
    ny, nx = shp[-2:]
    v = u.reshape(-1, ny, nx)
    lam = _lams(lambdas, v.shape[0])
    th = np.zeros((v.shape[0], 2))
    if tilts is not None:
        th[:] = np.asarray(tilts, dtype=np.float64).reshape(-1, 2)
    general = paraxial or filt is not None or bool(np.any(th != 0.0))
    out = np.empty_like(v)
    cache = {}
    for b in range(v.shape[0]):
        key = (float(lam[b]), float(th[b, 0]), float(th[b, 1]))
        if key not in cache:
            if general:
                cache[key] = as_kernel_general(nx, ny, dx, dy, key[0], z, n0, paraxial, key[1:], track_tilts, filt)
            else:
                cache[key] = as_kernel(nx, ny, dx, dy, key[0], z, n0)
        h = cache[key] if direction == FORWARD else np.conj(cache[key])
        out[b] = ifft2(fft2(v[b]) * h)
    return out.reshape(shp)


def asprop_z_gradient(u_in, du, dx, dy, lambdas, z, direction=FORWARD, n0=1.0, paraxial=False, tilts=None,
                      track_tilts=False, filt=None, return_scale=False):
    """d loss / d z of ASPropZ as Zygote computes it through
    ifft(fft(u) .* conj_direction(kernel)) (angular_spectrum.jl:325-344): with
    U = FFT2(u_in), G = FFT2(du) (du the adjoint at the output) and dH/dz = i R H,
    dz = Re sum_b sum_k U conj(G) conj_direction(dH/dz) / (nx ny).  R is the derivative
    in z of the kernel's phase (lm = lambda / n0, g = f + f0, f0 = sin(theta) / lm;
    angular_spectrum.jl:1-76): on axis and tilted, R = 2 pi (sqrt(complex(1/lm^2 - g^2))
    + off) with off = track_tilts ? (f0x fx + f0y fy) lm : 0, conjugated for z < 0;
    paraxial, R = -pi lm g^2 + 2 pi / lm.  The filter is constant in z.

    With ``return_scale`` also returns the sum of the magnitudes of the summed terms,
    sum |U conj(G) dH| / (nx ny): the sum nearly cancels for intensity losses (the
    constant part of R is a global phase), and a float32 evaluation of it is accurate
    to a few ulps of that scale, not of the result."""
    u = np.asarray(u_in, dtype=np.complex128)
    g = np.asarray(du, dtype=np.complex128)
    ny, nx = u.shape[-2:]
    u = u.reshape(-1, ny, nx)
    g = g.reshape(-1, ny, nx)
    lam = _lams(lambdas, u.shape[0])
    th = np.zeros((u.shape[0], 2))
    if tilts is not None:
        th[:] = np.asarray(tilts, dtype=np.float64).reshape(-1, 2)
    general = paraxial or filt is not None or bool(np.any(th != 0.0))
    fx, fy = fftfreqs(nx, ny, dx, dy)
    FX, FY = fx[None, :] + 0 * fy[:, None], fy[:, None] + 0 * fx[None, :]
    tot = 0.0
    scale = 0.0
    for b in range(u.shape[0]):
        lm = lam[b] / n0
        tilted = th[b, 0] != 0.0 or th[b, 1] != 0.0
        f0x, f0y = (np.sin(th[b, 0]) / lm, np.sin(th[b, 1]) / lm) if (tilted or paraxial) else (0.0, 0.0)
        gx, gy = FX + f0x, FY + f0y
        if paraxial:
            rate = -np.pi * lm * (gx ** 2 + gy ** 2) + 2 * np.pi / lm + 0j
        else:
            kz = np.sqrt((1.0 / lm ** 2 - gx ** 2 - gy ** 2).astype(np.complex128))
            off = (f0x * FX + f0y * FY) * lm if (tilted and track_tilts) else 0.0
            rate = 2 * np.pi * (kz + off)
            if z < 0:
                rate = np.conj(rate)
        if general:
            h = as_kernel_general(nx, ny, dx, dy, lam[b], z, n0, paraxial, tuple(th[b]), track_tilts, filt)
        else:
            h = as_kernel(nx, ny, dx, dy, lam[b], z, n0)
        dh = 1j * rate * h
        if direction != FORWARD:
            dh = np.conj(dh)
        terms = fft2(u[b]) * np.conj(fft2(g[b])) * dh
        tot += float(np.real(np.sum(terms))) / (nx * ny)
        scale += float(np.sum(np.abs(terms))) / (nx * ny)
    return (tot, scale) if return_scale else tot


def rsprop(u, dx, dy, lambdas, z, direction=FORWARD, pad=None):
    """RSProp: pad to (2n-1) (or ``pad``) at offset 0, FFT, * H_RS (conj for
    Backward), IFFT, crop the top-left n x n (rayleigh_sommerfeld.jl:128-169,
    pad_crop_operators.jl:1-16,61-79,291-356)."""
    u = np.asarray(u, dtype=np.complex128)
    shp = u.shape
    ny, nx = shp[-2:]
    v = u.reshape(-1, ny, nx)
    mx = (2 * nx - 1) if pad is None else pad[0]
    my = (2 * ny - 1) if pad is None else pad[1]
    lam = _lams(lambdas, v.shape[0])
    out = np.empty_like(v)
    cache = {}
    for b in range(v.shape[0]):
        key = float(lam[b])
        if key not in cache:
            cache[key] = rs_kernel(nx, ny, dx, dy, key, z, mx, my)
        h = cache[key] if direction == FORWARD else np.conj(cache[key])
        up = np.zeros((my, mx), dtype=np.complex128)
        up[:ny, :nx] = v[b]
        out[b] = ifft2(fft2(up) * h)[:ny, :nx]
    return out.reshape(shp)


# ---------------------------------------------------------------------------
# Modulators
# ---------------------------------------------------------------------------

def phase_forward(u, phi, direction=FORWARD):
    """u * cis(s*phi), phi broadcast over the batch (phasemask.jl:90-94)."""
    return np.asarray(u) * np.exp(1j * direction * np.asarray(phi, dtype=np.float64))


def phase_backward(dv, phi, u_saved, direction=FORWARD):
    """Adjoint of Phase with its gradient (phasemask.jl:96-98, :115-150).

    du = cis(-s*phi) dv;  dphi = s * sum_batch Im(du * conj(u_saved))."""
    du = np.asarray(dv) * np.exp(-1j * direction * np.asarray(phi, dtype=np.float64))
    g = direction * np.imag(du * np.conj(u_saved))
    dphi = g.reshape(-1, *g.shape[-2:]).sum(axis=0)
    return du, dphi


def tea_coefs(lambdas, dn, r=1.0):
    """Per-field (k_b, r_b) of TeaDOE: k = 2π dn(λ)/λ and r(λ) (tea_doe.jl:54-76);
    dn and r are numbers or functions of λ."""
    lams = np.atleast_1d(np.asarray(lambdas, dtype=np.float64))
    dnf = dn if callable(dn) else (lambda lam: dn)
    rf = r if callable(r) else (lambda lam: r)
    k = np.array([2 * np.pi * dnf(l) / l for l in lams])
    rv = np.array([complex(rf(l)) for l in lams])
    return k, rv


def tea_forward(u, h, k, r, direction=FORWARD):
    """u_b * r_b cis(s k_b h), conj(r_b) for s < 0 (tea_doe.jl:150-156); u is
    (batch, ny, nx), k and r hold one value per field."""
    u = np.asarray(u)
    rr = r if direction > 0 else np.conj(r)
    t = rr[:, None, None] * np.exp(1j * direction * k[:, None, None] * np.asarray(h, dtype=np.float64))
    return u * t


def tea_backward(dv, h, k, r, u_saved, direction=FORWARD):
    """Adjoint of TeaDOE and the height gradient (tea_doe.jl:180-215):
    du_b = conj(r_b cis(s k_b h)) dv_b;  dh = sum_b s k_b Im(du_b conj(u_saved_b))."""
    dv = np.asarray(dv)
    rr = np.conj(r) if direction > 0 else r
    du = dv * rr[:, None, None] * np.exp(-1j * direction * k[:, None, None] * np.asarray(h, dtype=np.float64))
    g = direction * k[:, None, None] * np.imag(du * np.conj(u_saved))
    return du, g.sum(axis=0)


def fourier_forward(u, w, direction=FORWARD):
    """FourierPhase / FourierMask forward: IFFT2(w FFT2(u)), conj(w) for Backward
    (fourier/fourier_wrapper.jl:1-5 with fourier_operator.jl:37-83); w = cis(phi) or m
    on the FFT-ordered frequency grid."""
    u = np.asarray(u, dtype=np.complex128)
    ww = w if direction > 0 else np.conj(w)
    return ifft2(fft2(u) * ww)


def fourier_phase_backward(dv, phi, u_saved, direction=FORWARD):
    """Adjoint of FourierPhase and its gradient: the Backward sequence is FFT (the
    ift operator reversed), Phase's backpropagate_with_gradient! on the spectra, IFFT
    (the ft operator reversed):  dU = cis(-s phi) FFT2(dv),
    dphi = s sum_b Im(dU_b conj(FFT2(u_saved)_b)),  du = IFFT2(dU)."""
    s = direction
    dU = fft2(np.asarray(dv, dtype=np.complex128)) * np.exp(-1j * s * np.asarray(phi, dtype=np.float64))
    U = fft2(np.asarray(u_saved, dtype=np.complex128))
    g = s * np.imag(dU * np.conj(U))
    return ifft2(dU), g.reshape(-1, *g.shape[-2:]).sum(axis=0)


def fourier_mask_backward(dv, m, u_saved, direction=FORWARD):
    """Adjoint of FourierMask and its gradient (Mask's rules, mask.jl:263-291, on the
    spectra): A = FFT2(dv), dm = sum_b conj_s(A_b conj(FFT2(u_saved)_b)),
    du = IFFT2(conj_s(m)... ) with the adjoint multiplier conj(m) (m for s < 0)."""
    s = direction
    A = fft2(np.asarray(dv, dtype=np.complex128))
    U = fft2(np.asarray(u_saved, dtype=np.complex128))
    g = A * np.conj(U)
    if s < 0:
        g = np.conj(g)
    m = np.asarray(m, dtype=np.complex128)
    madj = np.conj(m) if s > 0 else m
    return ifft2(A * madj), g.reshape(-1, *g.shape[-2:]).sum(axis=0)


def mask_forward(u, m, direction=FORWARD):
    """u * conj_direction(m) (mask.jl:241-248)."""
    m = np.asarray(m, dtype=np.complex128)
    return np.asarray(u) * (m if direction == FORWARD else np.conj(m))


def mask_backward(dv, m, u_saved, direction=FORWARD):
    """Adjoint of Mask with its gradient (mask.jl:263-291).

    dm = sum_batch conj_direction(dv * conj(u_saved)), taken before
    du = conj_direction(m, reverse(direction)) * dv."""
    m = np.asarray(m, dtype=np.complex128)
    g = np.asarray(dv) * np.conj(u_saved)
    if direction == BACKWARD:
        g = np.conj(g)
    dm = g.reshape(-1, *g.shape[-2:]).sum(axis=0)
    du = np.asarray(dv) * (np.conj(m) if direction == FORWARD else m)
    return du, dm


# ---------------------------------------------------------------------------
# AS_BPM
# ---------------------------------------------------------------------------

def _bpm_kdz(nb, dz, tilts):
    """kdz per field: 2 pi dz / (cos theta_x cos theta_y) (bpm.jl:3-6, :67-70)."""
    th = np.zeros((nb, 2))
    if tilts is not None:
        th[:] = np.asarray(tilts, dtype=np.float64).reshape(-1, 2)
    return (2.0 * np.pi * dz / (np.cos(th[:, 0]) * np.cos(th[:, 1])))[:, None, None]


def bpm_forward(u, dx, dy, lambdas, thickness, n0, dn, direction=FORWARD, save=False, paraxial=False, tilts=None):
    """Symmetric split-step AS_BPM march (bpm.jl:54-74, :130-142, :235-260).

    dn has shape (n_slices, ny, nx).  dz = thickness/n_slices, props ASProp(dz; n0,
    paraxial) and ASProp(dz/2; n0, paraxial) -- the tilted kernel for fields with
    ``tilts`` -- and kdz = 2 pi dz / (cos theta_x cos theta_y) per field.  Returns the
    output field and, when ``save``, the list of slice inputs u_k (taken before the dn
    phase)."""
    u = np.array(u, dtype=np.complex128)
    shp = u.shape
    ny, nx = shp[-2:]
    v = u.reshape(-1, ny, nx)
    lam = _lams(lambdas, v.shape[0])[:, None, None]
    n_slices = dn.shape[0]
    dz = thickness / n_slices
    kdz = _bpm_kdz(v.shape[0], dz, tilts)
    prop = lambda w, zz: asprop(w, dx, dy, lam.ravel(), zz, direction, n0, paraxial, tilts)
    saves = []
    v = prop(v, dz / 2)
    for k in range(n_slices - 1):
        if save:
            saves.append(v.copy())
        v = v * np.exp(1j * direction * kdz / lam * dn[k][None])
        v = prop(v, dz)
    if save:
        saves.append(v.copy())
    v = v * np.exp(1j * direction * kdz / lam * dn[-1][None])
    v = prop(v, dz / 2)
    return v.reshape(shp), saves


def bpm_backward(dv, dx, dy, lambdas, thickness, n0, dn, saves, direction=FORWARD, paraxial=False, tilts=None):
    """Adjoint march with the dn gradient (bpm.jl:262-321).

    d_dn_k = s * kdz/lam * sum_batch Im(du * conj(u_k)), taken after the
    conjugate dn phase of slice k."""
    du = np.array(dv, dtype=np.complex128)
    shp = du.shape
    ny, nx = shp[-2:]
    du = du.reshape(-1, ny, nx)
    lam = _lams(lambdas, du.shape[0])[:, None, None]
    n_slices = dn.shape[0]
    dz = thickness / n_slices
    kdz = _bpm_kdz(du.shape[0], dz, tilts)
    rev = -direction
    prop = lambda w, zz: asprop(w, dx, dy, lam.ravel(), zz, rev, n0, paraxial, tilts)
    ddn = np.zeros_like(dn, dtype=np.float64)
    du = prop(du, dz / 2)
    for k in range(n_slices - 1, 0, -1):
        du = du * np.exp(1j * rev * kdz / lam * dn[k][None])
        ddn[k] = (direction * kdz / lam * np.imag(du * np.conj(saves[k].reshape(du.shape)))).sum(0)
        du = prop(du, dz)
    du = du * np.exp(1j * rev * kdz / lam * dn[0][None])
    ddn[0] = (direction * kdz / lam * np.imag(du * np.conj(saves[0].reshape(du.shape)))).sum(0)
    du = prop(du, dz / 2)
    return du.reshape(shp), ddn


# ---------------------------------------------------------------------------
# Metric
# ---------------------------------------------------------------------------

def sid_value(u, target, target_index=None):
    """SquaredIntensityDifference (squared_intensity_difference.jl:58-83).

    I_t = sum over the fields mapped to target slice t of |u|^2; returns the
    per-slice losses c_t = sum (I_t - target_t)^2 and the residuals I - target.
    ``u`` has shape (B, ny, nx), ``target`` (T, ny, nx) and ``target_index[b]``
    gives the slice of field b (default: all fields to slice 0 when T == 1, else
    b % T -- the broadcast of a (nx, ny, T) target over (nx, ny, T, M) fields)."""
    u = np.asarray(u).reshape(-1, *np.shape(u)[-2:])
    t = np.asarray(target, dtype=np.float64)
    if t.ndim == 2:
        t = t[None]
    nb, nt = u.shape[0], t.shape[0]
    if target_index is None:
        target_index = np.arange(nb) % nt
    inten = np.zeros_like(t)
    for b in range(nb):
        inten[target_index[b]] += np.abs(u[b]) ** 2
    r = inten - t
    return np.sum(r ** 2, axis=(-2, -1)), r


def sid_backward(u, target, dc=1.0, target_index=None):
    """du = 4 * dc * (I - target) * u (squared_intensity_difference.jl:85-90)."""
    u2 = np.asarray(u).reshape(-1, *np.shape(u)[-2:])
    _, r = sid_value(u2, target, target_index)
    nt = r.shape[0]
    if target_index is None:
        target_index = np.arange(u2.shape[0]) % nt
    dc = np.broadcast_to(np.asarray(dc, dtype=np.float64).ravel(), (nt,)) \
        if np.ndim(dc) else np.full(nt, float(dc))
    du = np.empty_like(u2)
    for b in range(u2.shape[0]):
        ti = target_index[b]
        du[b] = 4.0 * dc[ti] * r[ti] * u2[b]
    return du.reshape(np.shape(u))


# ---------------------------------------------------------------------------
# Optimiser and proximal operators
# ---------------------------------------------------------------------------

class FistaState:
    """State (t_k, x_k, newdx) of Optimisers.init(::Fista) (OptimisersExt.jl:41-43)."""

    def __init__(self, x):
        self.t = 1.0
        # FP64 copy of the parameter, complex for a complex parameter (a source field)
        self.xk = np.array(x, dtype=np.result_type(np.asarray(x).dtype, np.float64), copy=True)
        self.newdx = np.zeros_like(self.xk)


def dot_product(u, v, ds, mode_selective=True):
    """DotProduct metric (metrics/dot_product.jl:70-87): per field
    c_b = sum u_b conj(v_b) dx dy, or with mode_selective=False the matrix
    c[i, j] = sum conj(v_i) u_j dx dy (v' u of the (npix, n) views).  u, v: (batch, ny, nx)."""
    u = np.asarray(u, dtype=np.complex128).reshape(-1, *np.shape(u)[-2:])
    v = np.asarray(v, dtype=np.complex128).reshape(-1, *np.shape(v)[-2:])
    a = ds[0] * ds[1]
    if mode_selective:
        return (u * np.conj(v)).reshape(len(u), -1).sum(axis=1) * a
    U = u.reshape(len(u), -1).T
    V = v.reshape(len(v), -1).T
    return (V.conj().T @ U) * a


def dot_product_backward(v, dc, mode_selective=True):
    """Pull-back of DotProduct (dot_product.jl:89-100): du_b = v_b dc_b, or
    du = V dc for the matrix form (columns of V are the fields)."""
    v = np.asarray(v, dtype=np.complex128).reshape(-1, *np.shape(v)[-2:])
    if mode_selective:
        return v * np.asarray(dc)[:, None, None]
    V = v.reshape(len(v), -1).T
    return (V @ np.asarray(dc)).T.reshape(v.shape)


def power_coupling(u, v, ds, mode_selective=True):
    """PowerCoupling (metrics/power_coupling.jl:48-66): |DotProduct(u, v_hat)|^2 with
    v_hat the unit-power copies of v.  Returns (values, dot products, v_hat)."""
    v = np.asarray(v, dtype=np.complex128).reshape(-1, *np.shape(v)[-2:])
    vh = np.stack([normalize_power(x, ds) for x in v])
    c = dot_product(u, vh, ds, mode_selective)
    return np.abs(c) ** 2, c, vh


def power_coupling_backward(vh, c_dot, dc, mode_selective=True):
    """Pull-back of PowerCoupling: DotProduct's with dc' = 2 dc c_dot (power_coupling.jl:63-66)."""
    return dot_product_backward(vh, 2 * np.asarray(dc) * c_dot, mode_selective)


def fista_apply(eta, state, x, dx):
    """One Fista step, in place on x; the rule stores eta^2 (OptimisersExt.jl:33-54).

    t' = (1+sqrt(1+4t^2))/2, beta = (t-1)/t', newdx = eta^2 dx - beta (x - x_k),
    x_k <- x, then Optimisers subtracts newdx from x."""
    e = eta * eta
    tkn = (1.0 + math.sqrt(1.0 + 4.0 * state.t * state.t)) / 2.0
    beta = (state.t - 1.0) / tkn
    state.newdx = e * dx - beta * (x - state.xk)
    state.xk = x.copy()
    state.t = tkn
    x -= state.newdx
    return x


def rule_step(rule, x, v, dx, eta, rho=0.0):
    """One step of Descent / Momentum / Nesterov as Optimisers.jl 0.4 defines them (a
    third-party dependency of the reference, pinned in its Project.toml and re-exported
    by OptimisersExt.jl:9), in place on x (and the velocity v), in the arrays' own
    precision with the rules' operation order:
    Descent newdx = eta dx; Momentum v = rho v + eta dx, newdx = v;
    Nesterov newdx = (-rho^2) v + ((1 + rho) eta) dx, v = rho v - eta dx; x -= newdx."""
    t = x.dtype.type
    eta, rho = t(eta), t(rho)
    if rule == "descent":
        nd = eta * dx
    elif rule == "momentum":
        v[...] = rho * v + eta * dx
        nd = v.copy()
    elif rule == "nesterov":
        nd = (-(rho * rho)) * v + ((t(1) + rho) * eta) * dx
        v[...] = rho * v - eta * dx
    else:
        raise ValueError(rule)
    x -= nd
    return x


def clamp_prox(x, lo, hi):
    """ClampProx (clamp_prox.jl:35-37)."""
    np.clip(x, lo, hi, out=x)
    return x


def positive_prox(x):
    """PositiveProx (positive_prox.jl:1-12)."""
    x[x < 0] = 0
    return x


def ista_prox(x, s, c=0.0):
    """IstaProx soft threshold towards c (ista_prox.jl:1-19); a complex array has its
    real and imaginary parts shrunk separately, each towards the real c
    (ista_prox.jl:13-15)."""
    if np.iscomplexobj(x):
        x.real = ista_prox(x.real.copy(), s, c)
        x.imag = ista_prox(x.imag.copy(), s, c)
        return x
    xc = x - c
    out = np.where(np.abs(xc) <= s, c, np.where(xc > s, x - s, x + s))
    x[...] = out
    return x


def pad(u, ns, offset=(0, 0), pad_val=0.0):
    """pad (utilities/pad_crop_operators.jl:1-16, :55-59): an array of size ns = (px, py)
    (Julia order) filled with pad_val, u copied to the 0-based offset (ox, oy)."""
    u = np.asarray(u)
    out = np.full(u.shape[:-2] + (ns[1], ns[0]), pad_val, dtype=np.result_type(u, np.complex128))
    ny, nx = u.shape[-2:]
    out[..., offset[1]:offset[1] + ny, offset[0]:offset[0] + nx] = u
    return out


def crop(u, ns, offset=(0, 0)):
    """crop (pad_crop_operators.jl:61-79, :114-120): the ns = (nx, ny) block at offset."""
    u = np.asarray(u)
    return u[..., offset[1]:offset[1] + ns[1], offset[0]:offset[0] + ns[0]].copy()


def sfd_value(u, v):
    """SquaredFieldDifference per field: sum over the last two axes of |u - v|^2, with
    no dx dy factor (metrics/squared_field_difference.jl:50-54)."""
    d = np.asarray(u) - np.asarray(v)
    return np.sum(d.real ** 2 + d.imag ** 2, axis=(-2, -1))


def sfd_backward(u, v, dc=1.0):
    """du = 2 dc_b (u_b - v_b) (metrics/squared_field_difference.jl:56-61)."""
    dc = np.asarray(dc, dtype=np.float64)
    return 2.0 * dc[..., None, None] * (np.asarray(u) - np.asarray(v))


def _d(p_out, a):
    # D! (tv_prox.jl:30-41): forward differences per dim, written into slice i
    # over 1:n-1 along that dim; the last index along dim i is not written.
    # numpy axis order: Julia dim 1 (x) is axis -1, dim 2 (y) is axis -2.
    nd = a.ndim
    for i in range(nd):
        ax = nd - 1 - i
        sl_hi = [slice(None)] * nd
        sl_lo = [slice(None)] * nd
        sl_hi[ax] = slice(1, None)
        sl_lo[ax] = slice(0, -1)
        p_out[i][tuple(sl_lo)] = a[tuple(sl_hi)] - a[tuple(sl_lo)]
    return p_out


def _dt(a, p):
    # Dt! (tv_prox.jl:43-59), including the boundary overwrite A[1 along dim i] = -p_i[1]
    nd = a.ndim
    for i in range(nd):
        ax = nd - 1 - i
        hi = [slice(None)] * nd
        lo = [slice(None)] * nd
        hi[ax] = slice(1, None)
        lo[ax] = slice(0, -1)
        val = p[i][tuple(lo)] - p[i][tuple(hi)]
        if i == 0:
            a[tuple(hi)] = val
        else:
            a[tuple(hi)] += val
    for i in range(nd):
        ax = nd - 1 - i
        first = [slice(None)] * nd
        first[ax] = 0
        a[tuple(first)] = -p[i][tuple(first)]
    return a


def tv_prox(y0, lam, n_iter=50, isotropic=True, eta=None, tol=None):
    """TVProx: dual FISTA on p (tv_prox.jl:94-195), in place on y0.

    Default inner rule Fista(0.25) (isotropic) / Fista(2.5) (anisotropic); the
    isotropic projection divides each dual slice by its global norm when > 1;
    anisotropic uses lam/100 and clamps to [-1, 1].  With ``tol`` the loop stops,
    before the dual update, once max |y - y_prev| < tol, y_prev starting at zero
    (tv_prox.jl:150-166).  A complex y0 has its real and imaginary parts denoised
    separately (tv_prox.jl:177-195)."""
    y0 = np.asarray(y0)
    if np.iscomplexobj(y0):
        re, im = y0.real.copy(), y0.imag.copy()
        tv_prox(re, lam, n_iter, isotropic, eta, tol)
        tv_prox(im, lam, n_iter, isotropic, eta, tol)
        y0[...] = re + 1j * im
        return y0
    if eta is None:
        eta = 0.25 if isotropic else 2.5
    nd = y0.ndim
    lam_eff = lam if isotropic else lam / 100.0
    p = np.zeros((nd,) + y0.shape)
    dp = np.zeros_like(p)
    y = np.zeros_like(y0, dtype=np.float64)
    y_prev = np.zeros_like(y)
    st = FistaState(p)
    for _ in range(n_iter):
        _dt(y, p)
        y = lam_eff * y - y0
        if tol is not None:
            if np.max(np.abs(y_prev - y)) < tol:
                break
            y_prev = y.copy()
        _d(dp, y)
        fista_apply(eta, st, p, dp)
        for i in range(nd):
            if isotropic:
                nrm = np.linalg.norm(p[i])
                if nrm > 1:
                    p[i] /= nrm
            else:
                np.clip(p[i], -1, 1, out=p[i])
    _dt(y, p)
    y0 -= lam_eff * y
    return y0
