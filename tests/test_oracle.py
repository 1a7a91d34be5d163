"""Pins the FP64 oracle to the reference's own tests (CPU only).

Each test restates a property or known answer from FluxOptics.jl's test suite
(test/*.jl) or source (analytic beams), plus central finite differences of every
hand-written adjoint.
"""

import math

import numpy as np
import pytest

from oracle import fluxoptics_oracle as orc


def gauss_field(n, ds, w0):
    x, y = orc.spatial_vectors((n, n), ds)
    return orc.gaussian(w0, x, y)


# --- test/optical_components_test.jl:85-112 -----------------------------------
def test_as_rs_unitarity():
    ds, lam, z = (1.0, 1.0), 1.064, 1000.0
    u = gauss_field(128, ds, 20.0)
    v = orc.asprop(u, ds[0], ds[1], lam, z)
    w = orc.asprop(v, ds[0], ds[1], lam, z, orc.BACKWARD)
    assert orc.coupling_efficiency(u, w) > 0.9999
    v = orc.rsprop(u, ds[0], ds[1], lam, z)
    w = orc.rsprop(v, ds[0], ds[1], lam, z, orc.BACKWARD)
    assert orc.coupling_efficiency(u, w) > 0.999


# --- test/optical_components_test.jl:114-133 ----------------------------------
def test_as_energy_conservation():
    ds = (0.5, 0.5)
    u = gauss_field(128, ds, 15.0)
    orc.normalize_power(u, ds, 1.0)
    v = orc.asprop(u, ds[0], ds[1], 1.064, 500.0)
    assert np.isclose(orc.power(v, ds), orc.power(u, ds), rtol=1e-6)


# --- test/optical_components_test.jl:22-44 ------------------------------------
def test_phase_angles():
    n, ds = 64, (1.0, 1.0)
    u = np.ones((n, n), dtype=complex)
    r = orc.phase_forward(u, np.full((n, n), np.pi / 2))
    assert np.allclose(np.angle(r), np.pi / 2)
    x, y = orc.spatial_vectors((n, n), ds)
    phi = x[None, :] + y[:, None]
    r = orc.phase_forward(u, phi)
    assert np.allclose(np.angle(r), np.angle(np.exp(1j * phi)))


# --- test/optical_components_test.jl:46-65 ------------------------------------
def test_mask_aperture():
    n, ds = 64, (1.0, 1.0)
    x, y = orc.spatial_vectors((n, n), ds)
    m = ((x[None, :] ** 2 + y[:, None] ** 2) < 20.0 ** 2).astype(float)
    r = orc.mask_forward(np.ones((n, n), dtype=complex), m)
    c = n // 2 - 1  # Julia's center_idx = 32 (1-based)
    assert abs(r[c, c]) == pytest.approx(1.0)
    assert abs(r[0, 0]) < 0.1


# --- test/metrics_test.jl:52-75 ------------------------------------------------
def test_sid_closed_form():
    n = 32
    u = np.ones((n, n), dtype=complex)
    c, _ = orc.sid_value(u, 2.0 * np.ones((n, n)))
    assert c[0] == pytest.approx(n * n * 1.0 * 1.0, rel=1e-6)
    c, _ = orc.sid_value(math.sqrt(2.0) * u, 2.0 * np.ones((n, n)))
    assert c[0] < 1e-10


# --- test/modes_test.jl:21-43 and the hermite_gaussian_groups doctest -------------
def test_hermite_gauss_modes():
    x, y = orc.spatial_vectors((129, 129), (1.0, 1.0))
    assert np.max(np.abs(orc.hermite_gaussian(15.0, 0, 0, x, y) - orc.gaussian(15.0, x, y))) < 1e-10
    hg10 = orc.hermite_gaussian(15.0, 1, 0, x, y)
    assert abs(hg10[64, 64]) < 1e-10
    hg20 = orc.hermite_gaussian(15.0, 2, 0, x, y)
    assert abs(hg20[64, 69]) == pytest.approx(abs(hg20[64, 59]), abs=1e-10)
    assert len(orc.hermite_gaussian_groups(3)) == 6
    assert len(orc.hermite_gaussian_groups(4)) == 10
    assert len(orc.hermite_gaussian_groups(5)) == 15
    x, y = orc.spatial_vectors((64, 64), (2.0, 2.0))
    for m, n in orc.hermite_gaussian_groups(3):
        f = orc.hermite_gaussian(10.0, m, n, x, y)
        assert abs(np.sum(np.abs(f) ** 2) * 4.0 - 1.0) < 1e-10


# --- test/fields_test.jl:49-72 --------------------------------------------------
def test_power_normalisation():
    ds = (0.5, 0.5)
    u = gauss_field(128, ds, 20.0)
    orc.normalize_power(u, ds, 1.0)
    assert orc.power(u, ds) == pytest.approx(1.0, rel=1e-6)
    orc.normalize_power(u, ds, 2.5)
    assert orc.power(u, ds) == pytest.approx(2.5, rel=1e-6)


# --- test/optimisers_test.jl:50-66 ------------------------------------------------
def test_fista_quadratic():
    x = np.array([0.0])
    st = orc.FistaState(x)
    for _ in range(50):
        g = np.array([2 * (x[0] - 3.0)])
        orc.fista_apply(0.9, st, x, g)
    assert x[0] == pytest.approx(3.0, abs=1e-3)


# --- test/optimisers_test.jl:30-47 (IstaProx / ClampProx doctests) -----------------
def test_pointwise_prox():
    x = np.array([-1.0, -0.2, 0.0, 0.4, 1.5])
    orc.ista_prox(x, 0.5)
    assert np.allclose(x, [-0.5, 0.0, 0.0, 0.0, 1.0])
    x = np.array([-0.5, 0.3, 1.2, 0.8])
    orc.clamp_prox(x, 0.0, 1.0)
    assert np.allclose(x, [0.0, 0.3, 1.0, 0.8])


def test_prox_docstring_known_answers():
    """The values printed in the reference's docstrings: IstaProx(0.01, 0.0)
    (ista_prox.jl:35-49) and PositiveProx (positive_prox.jl:19-33)."""
    x = np.array([-0.5, -0.005, 0.0, 0.003, 0.2])
    orc.ista_prox(x, 0.01, 0.0)
    assert np.allclose(x, [-0.49, 0.0, 0.0, 0.0, 0.19], rtol=0, atol=1e-15)
    x = np.array([-0.1, 0.0, 0.5, -0.3, 1.2])
    orc.positive_prox(x)
    assert np.array_equal(x, [0.0, 0.0, 0.5, 0.0, 1.2])
    # complex values: real and imaginary parts shrink separately towards the real centre
    z = np.array([1.0 + 0.05j, 0.25 - 1.0j, 0.31 + 0.29j])
    orc.ista_prox(z, 0.1, 0.3)
    assert np.allclose(z, [0.9 + 0.15j, 0.3 - 0.9j, 0.3 + 0.3j])


def test_plain_rules_known_answers():
    """Two steps of Descent(0.1), Momentum(0.1, 0.9) and Nesterov(0.1, 0.9) on x = 1 with
    dx = 1, worked by hand from Optimisers.jl 0.4's update rules."""
    expect = {"descent": [0.9, 0.8], "momentum": [0.9, 0.71], "nesterov": [0.81, 0.539]}
    for rule, xs in expect.items():
        x, v = np.array([1.0]), np.zeros(1)
        for k in range(2):
            orc.rule_step(rule, x, v, np.array([1.0]), 0.1, 0.0 if rule == "descent" else 0.9)
            assert abs(x[0] - xs[k]) < 1e-12, (rule, k, x[0])


def test_sfd_known_answer_and_pullback():
    """SquaredFieldDifference: the docstring's 16.0 for 4 x 4 ones against zeros
    (squared_field_difference.jl:16-31), and its pull-back 2 dc (u - v) against
    central differences of the real loss sum(w c)."""
    assert orc.sfd_value(np.ones((4, 4), complex), np.zeros((4, 4), complex)) == 16.0
    rng = np.random.default_rng(5)
    u = rng.standard_normal((3, 6, 5)) + 1j * rng.standard_normal((3, 6, 5))
    v = rng.standard_normal((3, 6, 5)) + 1j * rng.standard_normal((3, 6, 5))
    w = rng.standard_normal(3)
    loss = lambda uu: float(np.sum(w * orc.sfd_value(uu, v)))
    g = orc.sfd_backward(u, v, w)
    eps = 1e-6
    for (b, i, j) in [(0, 0, 0), (2, 3, 4), (1, 5, 2)]:
        for part, unit in (("re", 1.0), ("im", 1j)):
            up, um = u.copy(), u.copy()
            up[b, i, j] += eps * unit
            um[b, i, j] -= eps * unit
            fd = (loss(up) - loss(um)) / (2 * eps)
            ref = g[b, i, j].real if part == "re" else g[b, i, j].imag
            assert abs(fd - ref) < 1e-6 * max(1.0, abs(fd)), (part, fd, ref)


# --- analytic paraxial Gaussian beam (src/modes/gaussian_modes.jl:87-104) -----------
def test_as_matches_paraxial_gaussian_beam():
    n, ds, lam, w0, z = 512, (1.0, 1.0), 1.064, 30.0, 1500.0
    x, y = orc.spatial_vectors((n, n), ds)
    u = orc.gaussian(w0, x, y)
    v = orc.asprop(u, ds[0], ds[1], lam, z)
    k = 2 * np.pi / lam
    zr = np.pi * w0 ** 2 / lam
    q0, qz = -1j * zr, z - 1j * zr
    r2 = x[None, :] ** 2 + y[:, None] ** 2
    ana = (math.sqrt(2 / np.pi) / w0) * (q0 / qz) * np.exp(1j * k * r2 / (2 * qz)) * np.exp(1j * k * z)
    assert orc.rel_l2(v, ana) < 1e-3


# --- AS_BPM with dn = 0 is one ASProp over the thickness (bpm.jl:244-260) ------------
def test_bpm_zero_dn_is_asprop():
    n, ds, lam, n0, L = 64, (1.0, 1.0), 1.064, 1.5, 100.0
    u = gauss_field(n, ds, 10.0)
    dn = np.zeros((20, n, n))
    v, _ = orc.bpm_forward(u, ds[0], ds[1], lam, L, n0, dn)
    w = orc.asprop(u, ds[0], ds[1], lam, L, orc.FORWARD, n0)
    assert orc.rel_l2(v, w) < 1e-12
    assert v.shape == (n, n)


# --- padding RSProp to a power of two >= 2n-1 is exact on the cropped block ----------
def test_rs_pow2_padding_is_exact():
    n, ds, lam, z = 40, (1.0, 1.0), 1.064, 300.0
    rng = np.random.default_rng(1)
    u = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a = orc.rsprop(u, ds[0], ds[1], lam, z)
    b = orc.rsprop(u, ds[0], ds[1], lam, z, pad=(128, 128))
    assert orc.rel_l2(b, a) < 1e-12


# --- adjoints against central finite differences ------------------------------------
def _fd_check(loss, grad_dot, x, d, eps=1e-6):
    fd = (loss(x + eps * d) - loss(x - eps * d)) / (2 * eps)
    an = grad_dot(d)
    assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-12) + 1e-9, (fd, an)


def _chain_setup(n=32, kind="as"):
    ds, lam = (1.0, 1.0), 1.064
    rng = np.random.default_rng(7)
    u0 = gauss_field(n, ds, 6.0) * (1 + 0.1 * rng.standard_normal((n, n)))
    phi1 = rng.uniform(0, 2 * np.pi, (n, n))
    phi2 = rng.uniform(0, 2 * np.pi, (n, n))
    target = np.abs(gauss_field(n, ds, 5.0)) ** 2
    prop = (lambda u, d=orc.FORWARD: orc.asprop(u, ds[0], ds[1], lam, 150.0, d)) if kind == "as" else \
        (lambda u, d=orc.FORWARD: orc.rsprop(u, ds[0], ds[1], lam, 150.0, d))
    return u0, phi1, phi2, target, prop


@pytest.mark.parametrize("kind", ["as", "rs"])
def test_fd_phase_chain(kind):
    u0, phi1, phi2, target, prop = _chain_setup(kind=kind)

    def fwd(p1, p2):
        v1 = prop(orc.phase_forward(u0, p1))
        v2 = prop(orc.phase_forward(v1, p2))
        return v1, v2

    def loss(p1):
        return orc.sid_value(fwd(p1, phi2)[1], target)[0].sum()

    v1, v2 = fwd(phi1, phi2)
    dv = prop(orc.sid_backward(v2, target), orc.BACKWARD)
    dv, g2 = orc.phase_backward(dv, phi2, v1)
    dv = prop(dv, orc.BACKWARD)
    _, g1 = orc.phase_backward(dv, phi1, u0)
    d = np.random.default_rng(3).standard_normal(phi1.shape)
    _fd_check(loss, lambda dd: np.sum(g1 * dd), phi1, d)
    loss2 = lambda p2: orc.sid_value(fwd(phi1, p2)[1], target)[0].sum()  # noqa: E731
    _fd_check(loss2, lambda dd: np.sum(g2 * dd), phi2, d)


@pytest.mark.parametrize("direction", [1, -1])
def test_fd_mask(direction):
    u0, _, _, target, prop = _chain_setup()
    rng = np.random.default_rng(5)
    m = rng.standard_normal(u0.shape) + 1j * rng.standard_normal(u0.shape)

    def loss(mm):
        return orc.sid_value(prop(orc.mask_forward(u0, mm, direction)), target)[0].sum()

    v = prop(orc.mask_forward(u0, m, direction))
    dv = prop(orc.sid_backward(v, target), orc.BACKWARD)
    _, gm = orc.mask_backward(dv, m, u0, direction)
    d = rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)
    _fd_check(loss, lambda dd: np.real(np.sum(np.conj(gm) * dd)), m, d)


@pytest.mark.parametrize("direction,paraxial,tilted", [(1, False, False), (-1, False, False), (1, True, False),
                                                       (1, False, True), (-1, True, True)])
def test_fd_bpm(direction, paraxial, tilted):
    """The AS_BPM adjoint's d(dn) against central differences, on axis and for the
    paraxial and tilted propagators with the per-field cos correction of kdz
    (bpm.jl:3-6)."""
    n, ds, lam, n0, L = 32, (0.5, 0.5), 1.064, 1.45, 12.0
    rng = np.random.default_rng(11)
    u0 = np.stack([gauss_field(n, ds, 4.0).astype(complex)] * 2)
    tilts = [(0.05, -0.03), (-0.02, 0.04)] if tilted else None
    lams = [lam, 0.8]
    dn = 5e-3 * rng.standard_normal((6, n, n))
    target = np.abs(gauss_field(n, ds, 3.0)) ** 2

    def loss(d):
        v, _ = orc.bpm_forward(u0, ds[0], ds[1], lams, L, n0, d, direction, paraxial=paraxial, tilts=tilts)
        return orc.sid_value(v, target)[0].sum()

    v, saves = orc.bpm_forward(u0, ds[0], ds[1], lams, L, n0, dn, direction, save=True, paraxial=paraxial,
                               tilts=tilts)
    _, g = orc.bpm_backward(orc.sid_backward(v, target), ds[0], ds[1], lams, L, n0, dn, saves, direction,
                            paraxial=paraxial, tilts=tilts)
    d = rng.standard_normal(dn.shape)
    _fd_check(loss, lambda dd: np.sum(g * dd), dn, d, eps=1e-7)
    if tilted:
        # the tilted march differs from the on-axis one through both the kernel and kdz
        v0, _ = orc.bpm_forward(u0, ds[0], ds[1], lams, L, n0, dn, direction, paraxial=paraxial)
        assert orc.rel_l2(v, v0) > 1e-3


# --- TVProx against a loop-by-loop restatement of tv_prox.jl:1-59 ---------------------
def _loop_tv(y0, lam, n_iter, eta=0.25):
    ny, nx = y0.shape
    y0 = y0.copy()
    p = np.zeros((2, ny, nx))
    dp = np.zeros_like(p)
    xk = p.copy()
    t = 1.0

    def dt(p):
        a = np.zeros((ny, nx))
        for j in range(ny):
            for i in range(1, nx):
                a[j, i] = p[0, j, i - 1] - p[0, j, i]
        for j in range(1, ny):
            for i in range(nx):
                a[j, i] += p[1, j - 1, i] - p[1, j, i]
        for j in range(ny):
            a[j, 0] = -p[0, j, 0]
        for i in range(nx):
            a[0, i] = -p[1, 0, i]
        return a

    for _ in range(n_iter):
        y = lam * dt(p) - y0
        for j in range(ny):
            for i in range(nx - 1):
                dp[0, j, i] = y[j, i + 1] - y[j, i]
        for j in range(ny - 1):
            for i in range(nx):
                dp[1, j, i] = y[j + 1, i] - y[j, i]
        tn = (1 + math.sqrt(1 + 4 * t * t)) / 2
        beta = (t - 1) / tn
        newdx = eta * eta * dp - beta * (p - xk)
        xk = p.copy()
        p = p - newdx
        t = tn
        for k in range(2):
            nr = np.linalg.norm(p[k])
            if nr > 1:
                p[k] /= nr
    return y0 - lam * dt(p)


def test_tv_prox_matches_loops():
    rng = np.random.default_rng(2)
    y0 = rng.standard_normal((9, 11))
    ref = _loop_tv(y0, 0.3, 7)
    got = orc.tv_prox(y0.copy(), 0.3, 7)
    assert np.max(np.abs(got - ref)) < 1e-12


def test_tv_prox_tolerance_and_complex():
    """TVProx's tol stops the dual iterations before their update once the primal
    iterate changes by less than tol (tv_prox.jl:150-166): here after two updates, the
    same as n_iter = 2 (changes 3.3, 0.32, then 7.8e-3 < 1e-2).  A complex array is
    denoised as its real and imaginary parts (tv_prox.jl:177-195)."""
    rng = np.random.default_rng(3)
    y0 = rng.standard_normal((40, 30))
    a = orc.tv_prox(y0.copy(), 1.0, 25, tol=1e-2)
    assert np.array_equal(a, orc.tv_prox(y0.copy(), 1.0, 2))
    assert orc.rel_l2(a, orc.tv_prox(y0.copy(), 1.0, 25)) > 1e-4
    z0 = y0 + 1j * rng.standard_normal((40, 30))
    z = orc.tv_prox(z0.copy(), 0.2, 10)
    assert np.array_equal(z.real, orc.tv_prox(z0.real.copy(), 0.2, 10))
    assert np.array_equal(z.imag, orc.tv_prox(z0.imag.copy(), 0.2, 10))


def test_tv_prox_smooths():
    rng = np.random.default_rng(4)
    x = np.outer(np.sin(0.1 * np.arange(64)), np.sin(0.1 * np.arange(64))) * 5 + rng.standard_normal((64, 64))
    v0 = np.var(x)
    orc.tv_prox(x, 0.1, 100)
    assert np.var(x) < v0


def test_tea_doe_reduces_to_phase_and_matches_finite_differences(orc):
    """TeaDOE with r = 1 and constant dn is Phase(2π dn h / λ) field by field, and
    its height gradient matches central finite differences of a real loss."""
    rng = np.random.default_rng(8)
    lams = np.array([0.5, 0.8, 1.1])
    u = rng.standard_normal((3, 12, 10)) + 1j * rng.standard_normal((3, 12, 10))
    h = rng.uniform(0, 0.5, (12, 10))
    k, r = orc.tea_coefs(lams, 0.45)
    v = orc.tea_forward(u, h, k, r)
    for b in range(3):
        assert np.allclose(v[b], orc.phase_forward(u[b], 2 * np.pi * 0.45 * h / lams[b]))
    k, r = orc.tea_coefs(lams, lambda l: 0.4 + 0.02 / l, r=lambda l: 0.9 * np.exp(0.3j * l))
    w = rng.standard_normal((3, 12, 10)) + 1j * rng.standard_normal((3, 12, 10))

    def loss(hh):
        return float(np.real(np.vdot(w, orc.tea_forward(u, hh, k, r))))

    _, g = orc.tea_backward(w, h, k, r, u)
    eps = 1e-6
    for (i, j) in [(0, 0), (5, 7), (11, 9)]:
        hp, hm = h.copy(), h.copy()
        hp[i, j] += eps
        hm[i, j] -= eps
        fd = (loss(hp) - loss(hm)) / (2 * eps)
        assert abs(fd - g[i, j]) < 1e-6 * max(1.0, abs(fd))


def test_tilted_and_paraxial_kernels(orc):
    """Tilted kernel with zero tilts is the on-axis kernel; a tilted kernel without
    carrier tracking propagates a tilted plane wave as a plane wave (intensity
    unchanged); the paraxial kernel approaches the exact one for small angles."""
    n, d, lam, z = 64, 1.0, 1.0, 200.0
    h0 = orc.as_kernel(n, n, d, d, lam, z)
    assert np.allclose(orc.as_kernel_general(n, n, d, d, lam, z, theta=(0.0, 0.0)), h0)
    hz = orc.as_kernel_general(n, n, d, d, lam, -z, theta=(0.05, -0.02), track_tilts=True)
    assert np.allclose(hz, np.conj(orc.as_kernel_general(n, n, d, d, lam, z, theta=(0.05, -0.02),
                                                         track_tilts=True)))
    x, y = orc.spatial_vectors((n, n), (d, d))
    u = orc.gaussian(12.0, x, y)
    exact = orc.asprop(u, d, d, lam, 50.0)
    parax = orc.asprop(u, d, d, lam, 50.0, paraxial=True)
    # same up to the global phase convention of the Fresnel kernel's carrier term
    c = np.vdot(exact, parax)
    assert orc.rel_l2(parax * np.conj(c) / abs(c), exact) < 2e-3
    filt = lambda fx, fy: (np.hypot(fx, fy) < 0.2).astype(np.float64)
    hf = orc.as_kernel_general(n, n, d, d, lam, z, filt=filt)
    assert np.allclose(hf, h0 * filt(*np.meshgrid(np.fft.fftfreq(n, d), np.fft.fftfreq(n, d))))


def _kat_field():
    # the docstring example of dot_product.jl / power_coupling.jl: ones(4, 4, 2) with
    # data[3:end, :, 2] = -1 (Julia x-fastest), power-normalised field by field
    d = np.ones((2, 4, 4), dtype=np.complex128)
    d[1, :, 2:] = -1
    return np.stack([f for f in d])


def test_dot_product_and_power_coupling_known_answers(orc):
    """Known answers printed in the reference's docstrings (dot_product.jl:29-41,
    power_coupling.jl:28-40): selective [1, 1]; non-selective identity 2x2."""
    u = np.stack([orc.normalize_power(f, (1.0, 1.0)) for f in _kat_field()])
    assert np.allclose(orc.dot_product(u, u, (1.0, 1.0)), [1.0, 1.0])
    assert np.allclose(orc.dot_product(u, u, (1.0, 1.0), mode_selective=False), np.eye(2))
    p, _, _ = orc.power_coupling(u, u, (1.0, 1.0))
    assert np.allclose(p, [1.0, 1.0])
    p, _, _ = orc.power_coupling(u, u, (1.0, 1.0), mode_selective=False)
    assert np.allclose(p, np.eye(2))


def test_overlap_pullbacks_match_finite_differences(orc):
    """Real losses Re(w . c) of the DotProduct and PowerCoupling outputs: the
    pull-backs give the gradient (dL/dRe u + i dL/dIm u) up to the reference's
    convention, checked by central differences on a few pixels."""
    rng = np.random.default_rng(4)
    u = rng.standard_normal((3, 6, 5)) + 1j * rng.standard_normal((3, 6, 5))
    v = rng.standard_normal((3, 6, 5)) + 1j * rng.standard_normal((3, 6, 5))
    ds = (0.5, 0.7)
    for sel in (True, False):
        w = rng.standard_normal((3,) if sel else (3, 3))
        p, c, vh = orc.power_coupling(u, v, ds, sel)
        loss = lambda uu: float(np.sum(w * orc.power_coupling(uu, v, ds, sel)[0]))
        g = orc.power_coupling_backward(vh, c, w, sel)
        eps = 1e-6
        for (b, i, j) in [(0, 0, 0), (2, 3, 4), (1, 5, 2)]:
            for part, unit in (("re", 1.0), ("im", 1j)):
                up, um = u.copy(), u.copy()
                up[b, i, j] += eps * unit
                um[b, i, j] -= eps * unit
                fd = (loss(up) - loss(um)) / (2 * eps)
                # the reference's pull-back is the conjugate Wirtinger form times dx dy
                ref = (g[b, i, j].real if part == "re" else g[b, i, j].imag) * ds[0] * ds[1]
                assert abs(fd - ref) < 1e-5 * max(1.0, abs(fd)), (sel, part, fd, ref)


def test_fourier_phase_gradient_matches_finite_differences(orc):
    """FourierPhase: the spectral-domain phase gradient of a real loss Re<w, out>
    matches central differences; FourierMask with m = cis(phi) gives the same field."""
    rng = np.random.default_rng(6)
    u = rng.standard_normal((2, 8, 8)) + 1j * rng.standard_normal((2, 8, 8))
    w = rng.standard_normal((2, 8, 8)) + 1j * rng.standard_normal((2, 8, 8))
    phi = rng.uniform(0, 2 * np.pi, (8, 8))
    out = orc.fourier_forward(u, np.exp(1j * phi))
    assert np.allclose(out, orc.fourier_forward(u, np.exp(1j * phi), 1))
    loss = lambda p: float(np.real(np.vdot(w, orc.fourier_forward(u, np.exp(1j * p)))))
    _, g = orc.fourier_phase_backward(w, phi, u)
    eps = 1e-6
    for (i, j) in [(0, 0), (3, 5), (7, 2)]:
        pp, pm = phi.copy(), phi.copy()
        pp[i, j] += eps
        pm[i, j] -= eps
        fd = (loss(pp) - loss(pm)) / (2 * eps)
        # the reference's spectra are unnormalised: its gradient is N times the
        # derivative of the normalised-IFFT loss
        assert abs(fd * u.shape[-1] * u.shape[-2] - g[i, j]) < 1e-6 * max(1.0, abs(g[i, j]))


def test_asprop_z_gradient_matches_finite_differences(orc):
    """dL/dz of ASPropZ for L = Re<w, asprop(u, z)> against central differences in z,
    both directions and both signs of z (evanescent components included)."""
    rng = np.random.default_rng(3)
    u = rng.standard_normal((2, 16, 16)) + 1j * rng.standard_normal((2, 16, 16))
    w = rng.standard_normal((2, 16, 16)) + 1j * rng.standard_normal((2, 16, 16))
    lams = np.array([0.9, 1.3])
    for z in (37.0, -22.0):
        for d in (orc.FORWARD, orc.BACKWARD):
            loss = lambda zz: float(np.real(np.vdot(w, orc.asprop(u, 0.5, 0.5, lams, zz, d))))
            eps = 1e-5
            fd = (loss(z + eps) - loss(z - eps)) / (2 * eps)
            g = orc.asprop_z_gradient(u, w, 0.5, 0.5, lams, z, d)
            assert abs(fd - g) < 1e-6 * max(1.0, abs(fd)), (z, d, fd, g)


def test_asprop_z_gradient_general_kernels(orc):
    """dL/dz of ASPropZ with the paraxial kernel, the tilted kernel (per-field tilts,
    with and without tilt tracking) and a complex frequency filter, against central
    differences in z, both directions and both signs of z."""
    rng = np.random.default_rng(4)
    u = rng.standard_normal((2, 16, 16)) + 1j * rng.standard_normal((2, 16, 16))
    w = rng.standard_normal((2, 16, 16)) + 1j * rng.standard_normal((2, 16, 16))
    lams = np.array([0.9, 1.3])
    tilts = np.array([[0.05, -0.02], [0.01, 0.03]])
    filt = lambda fx, fy: np.exp(-(fx ** 2 + fy ** 2) / 0.3) * np.exp(0.4j * fx)
    cases = [dict(paraxial=True), dict(paraxial=True, tilts=tilts, track_tilts=True),
             dict(tilts=tilts), dict(tilts=tilts, track_tilts=True), dict(filt=filt),
             dict(tilts=tilts, filt=filt), dict(paraxial=True, filt=filt)]
    for kw in cases:
        for z in (37.0, -22.0):
            for d in (orc.FORWARD, orc.BACKWARD):
                loss = lambda zz: float(np.real(np.vdot(w, orc.asprop(u, 0.5, 0.5, lams, zz, d, n0=1.2, **kw))))
                eps = 1e-5
                fd = (loss(z + eps) - loss(z - eps)) / (2 * eps)
                g = orc.asprop_z_gradient(u, w, 0.5, 0.5, lams, z, d, n0=1.2, **kw)
                assert abs(fd - g) < 1e-6 * max(1.0, abs(fd)), (kw.keys(), z, d, fd, g)


def test_filtered_kernel_is_conjugated_for_negative_z(orc):
    """For z < 0 the reference takes conj of the z > 0 kernel with its filter value
    (angular_spectrum.jl:9-12, 55-60): a complex filter is conjugated too."""
    filt = lambda fx, fy: np.exp(0.7j * fx) * (1 + 0 * fy)
    for theta in ((0.0, 0.0), (0.03, -0.01)):
        hp = orc.as_kernel_general(8, 8, 0.5, 0.5, 0.8, 30.0, 1.0, False, theta, False, filt)
        hm = orc.as_kernel_general(8, 8, 0.5, 0.5, 0.8, -30.0, 1.0, False, theta, False, filt)
        assert np.allclose(hm, np.conj(hp))


# --- pad / crop (utilities/pad_crop_operators.jl:1-120; test/optical_components_test.jl:171-189) ---
def test_pad_crop_restatement():
    u = np.ones((32, 32), dtype=np.complex128)
    p = orc.pad(u, (64, 64))
    assert p.shape == (64, 64) and p[16, 16] == 1.0 and p[40, 40] == 0.0
    assert np.array_equal(orc.crop(p, (32, 32)), u)
    rng = np.random.default_rng(3)
    a = rng.standard_normal((2, 5, 7)) + 1j * rng.standard_normal((2, 5, 7))
    q = orc.pad(a, (11, 9), offset=(3, 2), pad_val=0.5)
    assert q.shape == (2, 9, 11)
    assert np.array_equal(q[:, 2:7, 3:10], a) and np.all(q[:, :2] == 0.5) and np.all(q[:, :, :3] == 0.5)
    assert np.array_equal(orc.crop(q, (7, 5), offset=(3, 2)), a)


# --- tilted kernels against the on-axis one (angular_spectrum.jl:27-76) ----------------------
# A field u carried as the envelope e = u exp(-i 2 pi f0.r) with f0 = sin(theta)/lambda on the
# frequency grid: the tilted kernel H(f + f0) propagates e exactly as the on-axis kernel
# propagates u (for a band-limited u, whose spectrum does not wrap at Nyquist); with
# track_tilts the envelope also follows the beam's walk-off, e'(r) = u'(r + z sin(theta)) x
# exp(-i 2 pi f0.(r + z sin(theta))).  Both pin the tilted kernels physically.
def _tilt_case():
    N, d, lam = 64, 1.0, 1.0
    x = (np.arange(N) - (N - 1) / 2) * d
    u = orc.gaussian(6.0, x, x) * np.exp(1j * 0.02 * (x[None, :] ** 2 - 0.5 * x[:, None] ** 2))
    f0 = np.array([3 / (N * d), -2 / (N * d)])
    carrier = np.exp(2j * np.pi * (f0[0] * x[None, :] + f0[1] * x[:, None]))
    return N, d, lam, u, f0, tuple(np.arcsin(f0 * lam)), carrier


def test_tilted_kernel_propagates_the_envelope():
    N, d, lam, u, f0, th, carrier = _tilt_case()
    v = orc.asprop(u / carrier, d, d, lam, 40.0, tilts=th) * carrier
    assert orc.rel_l2(v, orc.asprop(u, d, d, lam, 40.0)) < 1e-12


def test_tracked_tilts_follow_the_walk_off():
    N, d, lam, u, f0, th, carrier = _tilt_case()
    z = 64.0  # z sin(theta) = (3, -2) pixels
    e = orc.asprop(u / carrier, d, d, lam, z, tilts=th, track_tilts=True)
    ref = np.roll(orc.asprop(u, d, d, lam, z), shift=(2, -3), axis=(0, 1))  # u'(r + (3, -2))
    ph = np.exp(2j * np.pi * (f0[0] * 3 + f0[1] * -2))
    assert orc.rel_l2(e * carrier * ph, ref) < 1e-12


# --- RSProp against ASProp (rayleigh_sommerfeld.jl:1-12 against angular_spectrum.jl:1-12) -----
# The RS impulse response is the inverse Fourier transform of the AS transfer function, so
# for a band-limited field the two propagators, each restated independently (one from a
# sampled impulse response, one from the analytic transfer function), agree; AS runs on a
# window padded so that its circular convolution is the linear one.
@pytest.mark.parametrize("n,lam,w0,z", [(256, 1.064, 12.0, 400.0), (256, 1.064, 12.0, 1500.0),
                                        (200, 0.8, 10.0, 600.0)])
def test_rs_and_as_agree_on_band_limited_fields(n, lam, w0, z):
    x = (np.arange(n) - (n - 1) / 2)
    u = orc.gaussian(w0, x, x)
    h = n // 2
    a = orc.asprop(np.pad(u, ((h, h), (h, h))), 1.0, 1.0, lam, z)[h:h + n, h:h + n]
    assert orc.rel_l2(orc.rsprop(u, 1.0, 1.0, lam, z), a) < 1e-11


# --- AS_BPM with a uniform index perturbation (bpm.jl:3-6, 235-260) -----------------------------
# A uniform dn = c commutes with every step of the march, so the split-step result is one
# ASProp over the thickness times cis(2 pi c L / (lambda cos(theta_x) cos(theta_y))): this
# pins the dn phase scale kdz / lambda, the slice count and the half steps.
@pytest.mark.parametrize("tilts", [None, (0.02, -0.03)])
def test_bpm_uniform_dn_is_a_constant_phase(tilts):
    n, lam, n0, L, ns, c = 64, 1.064, 1.5, 100.0, 20, 3e-3
    x = (np.arange(n) - (n - 1) / 2)
    u = orc.gaussian(8.0, x, x)
    v, _ = orc.bpm_forward(u, 1.0, 1.0, lam, L, n0, np.full((ns, n, n), c), tilts=tilts)
    th = (0.0, 0.0) if tilts is None else tilts
    w = orc.asprop(u, 1.0, 1.0, lam, L, orc.FORWARD, n0, tilts=tilts)
    w = w * np.exp(2j * np.pi * c * L / (lam * np.cos(th[0]) * np.cos(th[1])))
    assert orc.rel_l2(v, w) < 1e-12
