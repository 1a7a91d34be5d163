"""Input generators (Gaussian / HermiteGaussian modes, at the waist and propagated)
against the known answers of the reference's docstrings (src/modes/gaussian_modes.jl)
and against the FP64 angular-spectrum oracle for the propagated forms.  CPU only."""

import numpy as np
import pytest

from __graft_entry__ import load_package
from oracle import fluxoptics_oracle as orc


@pytest.fixture(scope="module")
def fo():
    return load_package()


def grid(n, d):
    return (np.arange(n) - (n - 1) / 2.0) * d


def test_gaussian1d_docstring(fo):
    # gaussian_modes.jl:53-73
    x, dx = grid(40, 4.0), 4.0
    assert np.isclose(np.sum(np.abs(fo.Gaussian1D(10.0)(x)) ** 2) * dx, 1.0)
    assert np.isclose(np.sum(np.abs(fo.Gaussian1D(10.0, 1.064, 1000.0)(x)) ** 2) * dx, 1.0, atol=1e-5)


def test_gaussian_docstring(fo):
    # gaussian_modes.jl:156-176: in-place evaluation, and the propagated elliptical beam
    n, d = 64, 4.0
    x = y = grid(n, d)
    field = np.zeros((n, n), dtype=np.complex128)
    fo.Gaussian(10.0)(x, y, out=field)
    assert np.isclose(np.sum(np.abs(field) ** 2) * d * d, 1.0)
    ell = fo.Gaussian(10.0, 20.0, 1.064, 1000.0)(x, y)
    assert np.isclose(np.sum(np.abs(ell) ** 2) * d * d, 1.0)
    # the waist form equals the oracle's restatement and the plain function
    assert np.max(np.abs(field - orc.gaussian(10.0, x, y))) < 1e-15
    assert np.array_equal(fo.gaussian(10.0, x, y), field)
    # elliptical: x is the fast (second) numpy axis, as x is Julia's first index
    e0 = fo.Gaussian(10.0, 20.0)(x, y)
    assert np.isclose(abs(e0[n // 2, n // 2 + 5]) / abs(e0[n // 2, n // 2]), np.exp(-((5.5 * d) ** 2 - (0.5 * d) ** 2) / 100.0))


def test_gaussian_peak_norm_constant(fo):
    # norm_constant sets the peak intensity, counted once for the two axes
    x = y = grid(33, 1.0)
    g = fo.Gaussian(5.0, norm_constant=2.5)(x, y)
    assert np.isclose(np.abs(g[16, 16]) ** 2, 2.5)


def test_hermite_gaussian_docstrings(fo):
    # HermiteGaussian1D (gaussian_modes.jl:271-291) and HermiteGaussian (:346-369)
    x, dx = grid(64, 2.0), 2.0
    f0, f1 = fo.HermiteGaussian1D(20.0, 0)(x), fo.HermiteGaussian1D(20.0, 1)(x)
    assert np.isclose(np.sum(np.abs(f0) ** 2) * dx, 1.0)
    assert abs(np.sum(f0 * np.conj(f1)) * dx) < 1e-15
    y = x
    h00, h10 = fo.HermiteGaussian(10.0, 0, 0)(x, y), fo.HermiteGaussian(10.0, 1, 0)(x, y)
    assert np.isclose(np.sum(np.abs(h00) ** 2) * dx * dx, 1.0)
    assert abs(np.sum(h00 * np.conj(h10)) * dx * dx) < 1e-15
    # HG00 is the Gaussian (test/modes_test.jl:21-43)
    assert np.max(np.abs(h00 - fo.Gaussian(10.0)(x, y))) < 1e-15
    # m is the order along x: HG10 changes sign across x = 0, not across y = 0
    assert h10[32, 40].real * h10[32, 23].real < 0
    assert h10[40, 40].real * h10[23, 40].real > 0
    # the waist form equals the oracle's restatement
    for m, n in [(0, 1), (2, 1), (3, 0)]:
        assert np.max(np.abs(fo.HermiteGaussian(10.0, m, n)(x, y) - orc.hermite_gaussian(10.0, m, n, x, y))) < 1e-15


def test_hermite_gaussian_groups_docstring(fo):
    # gaussian_modes.jl:440-468
    modes = fo.hermite_gaussian_groups(10.0, 3)
    assert len(modes) == 6
    assert [(m.m, m.n) for m in modes] == [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (2, 0)]
    x = y = grid(64, 2.0)
    assert all(abs(np.sum(np.abs(md(x, y)) ** 2) * 4.0 - 1.0) < 1e-10 for md in modes)
    assert len(fo.hermite_gaussian_groups(10.0, 4)) == 10
    assert fo.hermite_gaussian_groups(3) == [(m.m, m.n) for m in modes]
    with pytest.raises(ValueError):
        fo.hermite_gaussian_groups(10.0, 0)


@pytest.mark.parametrize("m,n", [(0, 0), (1, 2), (3, 1)])
def test_propagated_modes_match_the_angular_spectrum(fo, m, n):
    """The propagated (paraxial) HG mode at z against the FP64 angular-spectrum
    propagation of the waist mode: they differ only by the paraxial approximation."""
    N, d, lam, w0, z = 512, 1.0, 1.064, 40.0, 1500.0
    x = y = grid(N, d)
    u0 = fo.HermiteGaussian(w0, m, n)(x, y)
    v = orc.asprop(u0, d, d, lam, z)
    ana = fo.HermiteGaussian(w0, m, n, lam, z)(x, y)
    assert orc.rel_l2(v, ana) < 2e-4  # measured 7e-6 (HG00) to 7e-5 (HG31)
    # without the constant phase, the field differs by exp(i k z) alone
    bare = fo.HermiteGaussian(w0, m, n, lam, z, constant_phase=False)(x, y)
    assert np.allclose(bare * np.exp(2j * np.pi / lam * z), ana, rtol=0, atol=1e-14)


def test_elliptical_propagated_gaussian_matches_the_angular_spectrum(fo):
    N, d, lam, z = 512, 1.0, 1.064, 2000.0
    x = y = grid(N, d)
    v = orc.asprop(fo.Gaussian(30.0, 45.0)(x, y), d, d, lam, z)
    assert orc.rel_l2(v, fo.Gaussian(30.0, 45.0, lam, z)(x, y)) < 2e-4  # measured 1.8e-5


def test_constructor_forms(fo):
    with pytest.raises(TypeError):
        fo.Gaussian(1.0, 2.0, 3.0, 4.0, 5.0)
    with pytest.raises(TypeError):
        fo.HermiteGaussian(1.0, 2)
    with pytest.raises(TypeError):
        fo.Gaussian1D(10.0, 1.064)
    with pytest.raises(ValueError):
        fo.HermiteGaussian(10.0, -1, 0)
    with pytest.raises(ValueError):
        fo.Gaussian(10.0)(grid(8, 1.0), grid(8, 1.0), out=np.zeros((4, 4), np.complex128))


def test_laguerre_gaussian_docstring(fo):
    # gaussian_modes.jl:516-541
    n, d = 65, 2.0
    x = y = grid(n, d)
    f00 = fo.LaguerreGaussian(10.0, 0, 0)(x, y)
    f01 = fo.LaguerreGaussian(10.0, 0, 1)(x, y)
    assert np.isclose(np.sum(np.abs(f00) ** 2) * d * d, 1.0)
    assert abs(f01[n // 2, n // 2]) < 1e-10
    even = fo.LaguerreGaussian(10.0, 0, 2, kind="even")(x, y)
    assert np.all(even.imag == 0)
    # LG00 is the Gaussian; LG modes are orthonormal
    assert np.max(np.abs(f00 - fo.Gaussian(10.0)(x, y))) < 1e-15
    modes = [fo.LaguerreGaussian(10.0, p, l)(x, y) for p, l in [(0, 0), (0, 1), (1, 0), (1, -2), (2, 3)]]
    G = np.array([[np.sum(np.conj(a) * b) * d * d for b in modes] for a in modes])
    assert np.max(np.abs(G - np.eye(len(modes)))) < 1e-8
    # even and odd are the real combinations of the +l and -l vortices
    vp, vm = fo.LaguerreGaussian(10.0, 1, 2)(x, y), fo.LaguerreGaussian(10.0, 1, -2)(x, y)
    assert np.allclose(fo.LaguerreGaussian(10.0, 1, 2, kind="odd")(x, y), (vp - vm) / (np.sqrt(2) * 1j), atol=1e-14)


@pytest.mark.parametrize("p,l", [(0, 1), (1, -2), (2, 1)])
def test_propagated_laguerre_gaussian_matches_the_angular_spectrum(fo, p, l):
    N, d, lam, w0, z = 512, 1.0, 1.064, 40.0, 1500.0
    x = y = grid(N, d)
    v = orc.asprop(fo.LaguerreGaussian(w0, p, l)(x, y), d, d, lam, z)
    assert orc.rel_l2(v, fo.LaguerreGaussian(w0, p, l, lam, z)(x, y)) < 2e-4
