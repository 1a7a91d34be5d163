"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Tolerances (relative L2 against the FP64 oracle, inputs rounded to the GPU's
float32 first): fields 1e-5, gradients 1e-4, losses 1e-4.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5
GRAD_TOL = 1e-4


def c64(a):
    return np.asarray(a).astype(np.complex64).astype(np.complex128)


def f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def npy(t):
    return t.detach().cpu().numpy().astype(np.complex128 if t.is_complex() else np.float64)


def rand_field(rng, shape):
    return c64(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


# ---------------------------------------------------------------------------
# Free-space propagators
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
def test_asprop_sizes(fo, orc, n):
    rng = np.random.default_rng(n)
    ds, lam, z = (1.0, 1.0), 1.064, 700.0
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(orc.gaussian(n / 8, x, y) * (1 + 0.2 * rng.standard_normal((n, n))))
    u = fo.ScalarField(u0, ds, lam)
    p = fo.ASProp(u, z)
    for d in (fo.Forward, fo.Backward):
        v = p.propagate(u, d)
        ref = orc.asprop(u0, ds[0], ds[1], lam, z, d)
        assert orc.rel_l2(npy(v.electric), ref) < FIELD_TOL


@pytest.mark.parametrize("shape", [(64, 128), (256, 32), (16, 4096), (2048, 64)])
def test_asprop_rectangular(fo, orc, shape):
    ny, nx = shape
    rng = np.random.default_rng(1)
    u0 = rand_field(rng, (ny, nx))
    u = fo.ScalarField(u0, (0.7, 1.3), 0.8)
    v = fo.ASProp(u, 250.0).propagate(u)
    assert orc.rel_l2(npy(v.electric), orc.asprop(u0, 0.7, 1.3, 0.8, 250.0)) < FIELD_TOL


def test_asprop_batch_wavelengths_n0_negative_z(fo, orc):
    rng = np.random.default_rng(2)
    lams = np.array([0.640, 0.538, 0.455])
    u0 = rand_field(rng, (4, 3, 128, 128))  # Julia (128, 128, 3, 4): lambda along dim 3
    u = fo.ScalarField(u0, (0.5, 0.5), lams)
    for z, n0 in ((5000.0, 1.0), (-800.0, 1.45)):
        v = fo.ASProp(u, z, n0=n0).propagate(u)
        ref = orc.asprop(u0.reshape(12, 128, 128), 0.5, 0.5, np.tile(lams, 4), z, 1, n0).reshape(u0.shape)
        assert orc.rel_l2(npy(v.electric), ref) < FIELD_TOL


def test_asprop_evanescent(fo, orc):
    # ds < lambda/2: part of the spectrum is evanescent and must decay
    rng = np.random.default_rng(3)
    u0 = rand_field(rng, (64, 64))
    u = fo.ScalarField(u0, (0.2, 0.2), 1.064)
    for z in (3.0, -3.0):
        v = fo.ASProp(u, z).propagate(u)
        assert orc.rel_l2(npy(v.electric), orc.asprop(u0, 0.2, 0.2, 1.064, z)) < FIELD_TOL


@pytest.mark.parametrize("n", [16, 40, 64, 250, 512])
def test_rsprop(fo, orc, n):
    rng = np.random.default_rng(n)
    ds, lam, z = (1.0, 1.0), 1.064, 1500.0
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(orc.gaussian(n / 6, x, y) * (1 + 0.2 * rng.standard_normal((n, n))))
    u = fo.ScalarField(u0, ds, lam)
    p = fo.RSProp(u, z)
    for d in (fo.Forward, fo.Backward):
        v = p.propagate(u, d)
        ref = orc.rsprop(u0, ds[0], ds[1], lam, z, d)  # the reference's 2n-1 padding
        assert orc.rel_l2(npy(v.electric), ref) < FIELD_TOL


def test_rsprop_rect_batch(fo, orc):
    rng = np.random.default_rng(5)
    u0 = rand_field(rng, (2, 48, 100))
    u = fo.ScalarField(u0, (2.0, 1.5), [1.064, 0.532])
    v = fo.RSProp(u, 900.0).propagate(u)
    ref = orc.rsprop(u0, 2.0, 1.5, [1.064, 0.532], 900.0)
    assert orc.rel_l2(npy(v.electric), ref) < FIELD_TOL


# ---------------------------------------------------------------------------
# Modulators
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("d", [1, -1])
def test_phase_mask_standalone(fo, orc, d):
    rng = np.random.default_rng(6)
    ny, nx, B = 33, 47, 3
    u0 = rand_field(rng, (B, ny, nx))
    dv0 = rand_field(rng, (B, ny, nx))
    phi = f32(rng.uniform(0, 2 * np.pi, (ny, nx)))
    m = c64(rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx)))
    u = fo.ScalarField(u0, (1.0, 1.0), 1.0)
    ph = fo.Phase(u, phi, trainable=True)
    mk = fo.Mask(u, m, trainable=True)
    saved = torch.empty_like(u.electric)
    v = u.copy()
    ph.propagate_and_save_(v, saved, d)
    assert orc.rel_l2(npy(v.electric), orc.phase_forward(u0, phi, d)) < FIELD_TOL
    assert orc.rel_l2(npy(saved), u0) == 0.0
    dv = fo.ScalarField(dv0, (1.0, 1.0), 1.0)
    g = torch.empty_like(ph.phi)
    ph.backpropagate_with_gradient_(dv, saved, g, d)
    du_ref, g_ref = orc.phase_backward(dv0, phi, u0, d)
    assert orc.rel_l2(npy(dv.electric), du_ref) < FIELD_TOL
    assert orc.rel_l2(npy(g), g_ref) < GRAD_TOL
    v = u.copy()
    mk.propagate_and_save_(v, saved, d)
    assert orc.rel_l2(npy(v.electric), orc.mask_forward(u0, m, d)) < FIELD_TOL
    dv = fo.ScalarField(dv0, (1.0, 1.0), 1.0)
    gm = torch.empty_like(mk.m)
    mk.backpropagate_with_gradient_(dv, saved, gm, d)
    du_ref, gm_ref = orc.mask_backward(dv0, m, u0, d)
    assert orc.rel_l2(npy(dv.electric), du_ref) < FIELD_TOL
    assert orc.rel_l2(npy(gm), gm_ref) < GRAD_TOL


# ---------------------------------------------------------------------------
# Fused chains with gradients
# ---------------------------------------------------------------------------

def _oracle_chain(orc, kind, u0, mods, ds, lams, zs, d):
    """mods: list of (kind, param) or None, len(zs)+1; returns out, saves."""
    def prop(v, z, dd):
        if kind == "AS":
            return orc.asprop(v, ds[0], ds[1], lams, z, dd)
        return orc.rsprop(v, ds[0], ds[1], lams, z, dd)

    def apply(v, m):
        if m is None:
            return v
        return orc.phase_forward(v, m[1], d) if m[0] == "phase" else orc.mask_forward(v, m[1], d)

    saves = []
    v = u0
    for k, z in enumerate(zs):
        saves.append(v)
        v = prop(apply(v, mods[k]), z, d)
    saves.append(v)
    return apply(v, mods[-1]), saves, prop


@pytest.mark.parametrize("kind,d", [("AS", 1), ("RS", 1), ("AS", -1)])
def test_chain_gradients(fo, orc, kind, d):
    rng = np.random.default_rng(8)
    n, B = 64, 2
    ds, lams = (1.0, 1.0), np.array([1.064, 0.8])
    zs = [300.0, 450.0, 200.0]
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(9.0, x, y)] * B) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    phi0 = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    m1 = c64(0.5 + rng.uniform(0, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    m3 = c64(0.5 + rng.uniform(0, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    target = f32(np.abs(orc.gaussian(7.0, x - 5, y)) ** 2)

    u = fo.ScalarField(u0, ds, lams)
    P = fo.ASProp if kind == "AS" else fo.RSProp
    c0 = fo.Phase(u, phi0, trainable=True)
    c1 = fo.Mask(u, m1, trainable=True)
    # the last modulator is a Mask: a phase-only mask right before an intensity
    # loss has an identically zero gradient
    c3 = fo.Mask(u, m3, trainable=True)
    props = [P(u, z) for z in zs]
    system = fo.OpticalSystem(fo.ScalarSource(u), [c0, props[0], c1, props[1], props[2], c3], direction=d)
    segs = system.segments(u)
    assert len(segs) == 1  # one fused chain
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)

    mods = [("phase", phi0), ("mask", m1), None, ("mask", m3)]
    out, saves, prop = _oracle_chain(orc, kind, u0, mods, ds, lams, zs, d)
    got = npy(system()["out"].electric)
    assert orc.rel_l2(got, out) < FIELD_TOL
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.sid_backward(out, target)
    dv, g3 = orc.mask_backward(dv, m3, saves[3], d)
    dv = prop(dv, zs[2], -d)
    dv = prop(dv, zs[1], -d)
    dv, g1 = orc.mask_backward(dv, m1, saves[1], d)
    dv = prop(dv, zs[0], -d)
    _, g0 = orc.phase_backward(dv, phi0, saves[0], d)
    assert orc.rel_l2(npy(grads[c3]["m"]), g3) < GRAD_TOL
    assert orc.rel_l2(npy(grads[c1]["m"]), g1) < GRAD_TOL
    assert orc.rel_l2(npy(grads[c0]["phi"]), g0) < GRAD_TOL


def test_balanced_column_units(fo, orc, monkeypatch):
    """A 2048^2 batch whose column CTAs leave the last round partly empty: the TMA
    column pass runs over balanced work units (the last round's field runs cut
    short).  Each field-strip is transformed the same way whichever CTA takes it, so
    the result equals the plain 2-D launch bit for bit, and the oracle to FIELD_TOL."""
    import ctypes as C
    rng = np.random.default_rng(40)
    n, B = 2048, 16
    ds, lam, z = (0.5, 0.5), 0.64, 5000.0
    x, y = orc.spatial_vectors((n, n), ds)
    base = orc.gaussian(80.0, x, y)
    u0 = c64(np.stack([base * np.exp(1j * 0.3 * k * x / 80.0) for k in range(B)])
             * (1 + 0.05 * rng.standard_normal((1, n, n))))
    lib = fo.load_library()

    def run(units):
        monkeypatch.setenv("FO_COL_UNITS", "1" if units else "0")
        u = fo.ScalarField(u0, ds, lam)
        prop = fo.ASProp(u, z)
        plan = prop.plan_for(u)
        name = C.create_string_buffer(200)
        fo._capi.check(lib.fo_prop_variants(plan, None, None, None, name, 200))
        prop.propagate_(u)
        torch.cuda.synchronize()
        return npy(u.electric), name.value.decode()

    got, name = run(True)
    ref, name0 = run(False)
    if "balanced work units" not in name:
        pytest.skip(f"this launch shape fills its last round: {name}")
    assert "balanced" not in name0
    assert np.array_equal(got, ref)
    for b in (0, B - 1):
        assert orc.rel_l2(got[b], orc.asprop(u0[b], ds[0], ds[1], lam, z, 1)) < FIELD_TOL


@pytest.mark.parametrize("n", [16, 64, 256, 512])
@pytest.mark.parametrize("kind", ["AS", "RS"])
@pytest.mark.parametrize("uneven", [False, True])
def test_metric_fused_into_last_pass(fo, orc, n, kind, uneven):
    """SquaredIntensityDifference evaluated inside the chain's last pass (uniform
    target slices) or as its own pass (uneven slices), the first modulator reading
    its saved input from the source field, and the seeded adjoint after it."""
    rng = np.random.default_rng(30 + n)
    B = 6
    ds = (1.0, 1.0)
    lams = np.array([1.064, 0.8, 0.6, 1.064, 0.8, 0.6])
    zs = [0.2 * n * n / 8, 0.15 * n * n / 8]
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(n / 6, x, y)] * B) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    phi0 = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    m2 = c64(0.5 + rng.uniform(0, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    target = f32(rng.uniform(0, 2, (3, n, n)) * np.abs(orc.gaussian(n / 5, x, y)) ** 2)
    tix = [0, 0, 0, 1, 2, 2] if uneven else None

    u = fo.ScalarField(u0, ds, lams)
    P = fo.ASProp if kind == "AS" else fo.RSProp
    c0 = fo.Phase(u, phi0, trainable=True)
    c2 = fo.Mask(u, m2, trainable=True)
    props = [P(u, z) for z in zs]
    system = fo.OpticalSystem(fo.ScalarSource(u), [c0, props[0], props[1], c2])
    assert len(system.segments(u)) == 1
    metric = fo.SquaredIntensityDifference((u, target), target_index=tix)
    loss, grads = fo.withgradient(metric, system)

    # the fused forward leaves the same field as the plain forward, and the same
    # loss as the metric's own pass
    a, b = u.similar(), u.similar()
    system.forward(a, src=u, metric=metric)
    l_fused = npy(metric.loss).astype(np.float64)
    system.forward(b, src=u)
    l_sep = npy(metric(b)).astype(np.float64)
    assert np.array_equal(npy(a.electric), npy(b.electric))
    assert np.max(np.abs(l_fused - l_sep) / np.abs(l_sep)) < 1e-5

    out, saves, prop = _oracle_chain(orc, kind, u0, [("phase", phi0), None, ("mask", m2)], ds, lams, zs, 1)
    assert orc.rel_l2(npy(a.electric), out) < FIELD_TOL
    c_ref, _ = orc.sid_value(out, target, tix)
    assert np.max(np.abs(l_fused - c_ref) / np.abs(c_ref)) < 1e-4
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.sid_backward(out, target, target_index=tix)
    dv, g2 = orc.mask_backward(dv, m2, saves[2], 1)
    dv = prop(dv, zs[1], -1)
    dv = prop(dv, zs[0], -1)
    _, g0 = orc.phase_backward(dv, phi0, saves[0], 1)
    assert orc.rel_l2(npy(grads[c2]["m"]), g2) < GRAD_TOL
    assert orc.rel_l2(npy(grads[c0]["phi"]), g0) < GRAD_TOL


@pytest.mark.parametrize("mode", ["paraxial", "tilted", "tilted_track", "filtered", "paraxial_tilted_track"])
@pytest.mark.parametrize("d", [1, -1])
def test_asprop_paraxial_tilted_filtered(fo, orc, mode, d):
    """ASProp variants of angular_spectrum.jl:27-76 on a batch with per-field
    wavelengths and tilts: the paraxial (Fresnel) kernel, the tilted kernel with and
    without carrier tracking, and a frequency filter (evaluated by the library
    through the host callback at the frequencies the reference passes to it)."""
    rng = np.random.default_rng(12)
    n, B = 256, 4
    ds, lams = (0.5, 0.5), np.array([0.64, 0.455, 0.8, 0.64])
    z = 180.0 if d > 0 else -180.0
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(16.0, x - 3 * b, y) for b in range(B)])
             * (1 + 0.05 * rng.standard_normal((B, n, n))))
    tilted = "tilted" in mode
    tx = np.array([0.02, -0.01, 0.0, 0.03]) if tilted else 0.0
    ty = np.array([0.0, 0.015, -0.02, 0.01]) if tilted else 0.0
    track = "track" in mode
    paraxial = "paraxial" in mode
    filt = (lambda fx, fy: np.where(np.hypot(fx, fy) < 0.6, 1.0, 0.3) * np.exp(0.2j * fx)) \
        if mode == "filtered" else None
    u = fo.ScalarField(u0, ds, lams, tilts=(tx, ty))
    p = fo.ASProp(u, abs(z), paraxial=paraxial, track_tilts=track, filter=filt)
    v = u.copy()
    p.propagate_(v, d)
    tl = None if not tilted else np.stack([np.broadcast_to(tx, (B,)), np.broadcast_to(ty, (B,))], axis=1)
    ref = orc.asprop(u0, ds[0], ds[1], lams, abs(z), d, paraxial=paraxial, tilts=tl, track_tilts=track,
                     filt=filt)
    assert orc.rel_l2(npy(v.electric).reshape(B, n, n), ref) < FIELD_TOL


def test_fourier_operator_and_wrapper(fo, orc):
    """fo_fft2's four modes against numpy's FFTs (FFTW's conventions), FourierOperator
    with its direction swap, and FourierWrapper(u, Phase) inside a system: loss and
    phase gradient against the oracle, where the adjoint of the inverse transform is
    F / (nx ny) (fourier/fourier_operator.jl:37-83, fourier_wrapper.jl:1-42)."""
    rng = np.random.default_rng(45)
    B, ny, nx = 3, 64, 128
    u0 = rand_field(rng, (B, ny, nx))
    u = fo.ScalarField(u0, (0.5, 0.5), [0.64, 0.538, 0.455])
    op = fo.FourierOperator(u, True)
    N = nx * ny
    F = lambda a: np.fft.fft2(a)
    refs = {0: F(u0), 1: np.fft.ifft2(u0), 2: N * np.fft.ifft2(u0), 3: F(u0) / N}
    for mode, ref in refs.items():
        v = u.copy()
        fo._capi.call("fo_fft2", op._plan(v), C.c_void_p(v.electric.data_ptr()), mode,
                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert orc.rel_l2(npy(v.electric), ref) < 1e-6, mode
    # the Backward direction swaps the transforms; FFT then IFFT is the identity
    v = op.propagate(u, fo.Backward)
    assert orc.rel_l2(npy(v.electric), np.fft.ifft2(u0)) < 1e-6
    w = fo.FourierOperator(u, False).propagate(op.propagate(u))
    assert orc.rel_l2(npy(w.electric), u0) < 1e-6

    n = 128
    lams = [0.64, 0.538]
    v0 = rand_field(rng, (2, n, n))
    target = f32(rng.uniform(0, 2, (2, n, n)))
    phi = f32(rng.uniform(0, 6, (n, n)))
    uu = fo.ScalarField(v0, (0.5, 0.5), lams)
    ph = fo.Phase(uu, phi, trainable=True)
    system = fo.ScalarSource(uu) | fo.FourierWrapper(uu, ph) | fo.ASProp(uu, 200.0)
    metric = fo.SquaredIntensityDifference((uu, target))
    loss, grads = fo.withgradient(metric, system)
    U = np.fft.fft2(v0)
    a = np.fft.ifft2(orc.phase_forward(U, phi))
    out = orc.asprop(a, 0.5, 0.5, lams, 200.0)
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    g = orc.asprop(orc.sid_backward(out, target), 0.5, 0.5, lams, 200.0, orc.BACKWARD)
    G = np.fft.fft2(g) / (n * n)  # adjoint of the inverse transform
    _, gphi = orc.phase_backward(G, phi, U)
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL


def test_fourier_wrapper_backward_direction(fo, orc):
    """A sequence runs in reverse in the Backward direction, each part with its Backward
    form (optical_sequence.jl:54-70): FourierWrapper(u, Phase) in a Backward system is
    IFFT(cis(-phi) FFT(u)), with the phase gradient of that order.  Also get_sequence,
    a standalone sequence in both directions, and trainable(system) through it."""
    rng = np.random.default_rng(46)
    n = 64
    lams = [0.64, 0.538]
    v0 = rand_field(rng, (2, n, n))
    target = f32(rng.uniform(0, 2, (n, n)))
    phi = f32(rng.uniform(0, 6, (n, n)))
    uu = fo.ScalarField(v0, (0.5, 0.5), lams)
    ph = fo.Phase(uu, phi, trainable=True)
    fw = fo.FourierWrapper(uu, ph)
    assert len(fo.get_sequence(fw)) == 3 and fo.get_sequence(fw)[1] is ph
    system = fo.OpticalSystem(fo.ScalarSource(uu), [fw], direction=fo.Backward)
    assert list(fo.trainable(system)) == [ph]
    X = np.fft.fft2(v0)
    out = np.fft.ifft2(orc.phase_forward(X, phi, orc.BACKWARD))
    assert orc.rel_l2(npy(system()["out"].electric), out) < 1e-6
    metric = fo.SquaredIntensityDifference((uu, target))
    loss, grads = fo.withgradient(metric, system)
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dY = np.fft.fft2(orc.sid_backward(out, target)) / (n * n)  # adjoint of the inverse transform
    _, gphi = orc.phase_backward(dY, phi, X, orc.BACKWARD)
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL
    # standalone: Forward and Backward, and the sequence's adjoint
    seq = fo.OpticalSequence(fo.ASProp(uu, 100.0), fo.Phase(uu, phi))
    a = fo.propagate(uu, seq, fo.Forward)
    assert orc.rel_l2(npy(a.electric), orc.phase_forward(orc.asprop(v0, 0.5, 0.5, lams, 100.0), phi)) < FIELD_TOL
    b = fo.propagate(uu, seq, fo.Backward)
    ref_b = orc.asprop(orc.phase_forward(v0, phi, orc.BACKWARD), 0.5, 0.5, lams, 100.0, orc.BACKWARD)
    assert orc.rel_l2(npy(b.electric), ref_b) < FIELD_TOL
    g = fo.backpropagate(uu, seq, fo.Forward)
    ref_g = orc.asprop(orc.phase_forward(v0, phi, orc.BACKWARD), 0.5, 0.5, lams, 100.0, orc.BACKWARD)
    assert orc.rel_l2(npy(g.electric), ref_g) < FIELD_TOL


@pytest.mark.parametrize("selective", [True, False])
def test_dot_product_power_coupling(fo, orc, selective):
    """DotProduct and PowerCoupling (values and pull-backs) against the oracle, and
    the gradient of a phase mask through Phase -> ASProp -> PowerCoupling."""
    rng = np.random.default_rng(17)
    n, B = 256, 5
    ds, lams = (0.8, 0.8), np.array([0.64, 0.538, 0.455, 0.64, 0.538])
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.hermite_gaussian(20.0, b % 3, b // 3, x, y) for b in range(B)])
             * (1 + 0.1 * rng.standard_normal((B, n, n))))
    v0 = c64(np.stack([orc.hermite_gaussian(18.0, (b + 1) % 3, b // 2, x - 2, y + 1) for b in range(B)]))
    u = fo.ScalarField(u0, ds, lams)
    v = fo.ScalarField(v0, ds, lams)
    dp = fo.DotProduct(v, mode_selective=selective)
    c = dp(u).cpu().numpy()
    c_ref = orc.dot_product(u0, v0, ds, selective)
    got = c if selective else c.T  # out[j, i] = c[i, j]
    assert orc.rel_l2(got, c_ref) < 1e-5
    w = c64(rng.standard_normal(c.shape) + 1j * rng.standard_normal(c.shape))
    du = dp.backpropagate(u, torch.tensor(w, device="cuda"))
    du_ref = orc.dot_product_backward(v0, w if selective else w.T, selective)
    assert orc.rel_l2(npy(du.electric).reshape(B, n, n), du_ref) < FIELD_TOL

    pc = fo.PowerCoupling(v, mode_selective=selective)
    p = pc(u).cpu().numpy()
    p_ref, cd, vh = orc.power_coupling(u0, v0, ds, selective)
    assert orc.rel_l2(p if selective else p.T, p_ref) < 1e-5
    wr = f32(rng.standard_normal(p.shape))
    du = pc.backpropagate(u, torch.tensor(wr, device="cuda"))
    du_ref = orc.power_coupling_backward(vh, cd, wr if selective else wr.T, selective)
    assert orc.rel_l2(npy(du.electric).reshape(B, n, n), du_ref) < GRAD_TOL

    if selective:
        phi = f32(rng.uniform(0, 2 * np.pi, (n, n)))
        ph = fo.Phase(u, phi, trainable=True)
        system = fo.ScalarSource(u) | ph | fo.ASProp(u, 300.0)
        loss, grads = fo.withgradient(pc, system)
        a = orc.asprop(orc.phase_forward(u0, phi), ds[0], ds[1], lams, 300.0)
        pr, cdr, vh = orc.power_coupling(a, v0, ds, True)
        assert abs(float(loss) - pr.sum()) / pr.sum() < 1e-4
        g = orc.power_coupling_backward(vh, cdr, np.ones(B), True)
        g = orc.asprop(g, ds[0], ds[1], lams, 300.0, orc.BACKWARD)
        _, gphi = orc.phase_backward(g, phi, u0)
        assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL


@pytest.mark.parametrize("d", [1, -1])
def test_asprop_z_trainable_distance(fo, orc, d):
    """ASPropZ with a trainable distance in Phase -> ASPropZ -> Mask -> ASProp -> SID:
    the propagated field, dL/dz and the mask gradients against the oracle."""
    rng = np.random.default_rng(29)
    n, B = 256, 3
    ds, lams = (0.5, 0.5), np.array([0.64, 0.538, 0.455])
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(10.0, x, y + b) for b in range(B)]) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    phi = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    m1 = c64(0.5 + rng.uniform(0, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    target = f32(np.abs(orc.gaussian(8.0, x - 2, y)) ** 2)
    z0 = 250.0
    u = fo.ScalarField(u0, ds, lams)
    ph = fo.Phase(u, phi, trainable=True)
    pz = fo.ASPropZ(u, z0, trainable=True)
    mk = fo.Mask(u, m1, trainable=True)
    system = fo.OpticalSystem(fo.ScalarSource(u), [ph, pz, mk, fo.ASProp(u, 120.0)], direction=d)
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    a0 = orc.phase_forward(u0, phi, d)
    a1 = orc.asprop(a0, ds[0], ds[1], lams, z0, d)
    a2 = orc.mask_forward(a1, m1, d)
    out = orc.asprop(a2, ds[0], ds[1], lams, 120.0, d)
    assert orc.rel_l2(npy(system()["out"].electric).reshape(B, n, n), out) < FIELD_TOL
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.asprop(orc.sid_backward(out, target), ds[0], ds[1], lams, 120.0, -d)
    dv, gm = orc.mask_backward(dv, m1, a1, d)
    gz = orc.asprop_z_gradient(a0, dv, ds[0], ds[1], lams, z0, d)
    dv = orc.asprop(dv, ds[0], ds[1], lams, z0, -d)
    _, gphi = orc.phase_backward(dv, phi, u0, d)
    assert orc.rel_l2(npy(grads[mk]["m"]), gm) < GRAD_TOL
    assert abs(float(grads[pz]["z"].item()) - gz) < GRAD_TOL * abs(gz) + 1e-12, (float(grads[pz]["z"].item()), gz)
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL


@pytest.mark.parametrize("mode", ["paraxial", "tilted", "tilted_track", "filtered", "paraxial_track_filtered"])
@pytest.mark.parametrize("z0", [180.0, -140.0])
def test_asprop_z_general_kernels(fo, orc, mode, z0):
    """ASPropZ with the reference's other kernels (angular_spectrum.jl:274-344): the
    paraxial kernel, the tilted kernel on fields with per-field tilts (with and without
    tilt tracking) and a complex frequency filter, for both signs of z: the propagated
    field after the distance was rebuilt from device memory, and dL/dz, against the
    oracle; a later z set on the device moves the result accordingly.

    dL/dz of an intensity loss is a sum over the spectra that nearly cancels: the
    constant part of the kernel's phase rate, 2 pi n0 / lambda, is a global phase the
    loss does not see, and it dominates every term (the terms' magnitudes add up to
    1e3 - 1e5 times the result here).  Computed from float32 spectra, the sum is
    accurate to about one float32 ulp of that magnitude, so dL/dz is held to 1e-4 of
    its value plus float32 epsilon times the sum of magnitudes."""
    rng = np.random.default_rng(33)
    n, B = 128, 2
    ds, lams, n0 = (0.5, 0.5), np.array([0.64, 0.455]), 1.1
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(6.0, x, y + b) for b in range(B)]) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    target = f32(np.abs(orc.gaussian(5.0, x - 1, y)) ** 2)
    tilts = np.array([[0.04, -0.02], [0.01, 0.03]]) if "tilted" in mode or "track" in mode else None
    filt = (lambda fx, fy: np.exp(-(fx ** 2 + fy ** 2) / 1.5) * np.exp(0.3j * fx)) if "filtered" in mode else None
    kw = dict(paraxial="paraxial" in mode, track_tilts="track" in mode, filt=filt)
    u = fo.ScalarField(u0, ds, lams, tilts=None if tilts is None else (tilts[:, 0], tilts[:, 1]))
    pz = fo.ASPropZ(u, z0, n0=n0, trainable=True, paraxial=kw["paraxial"], track_tilts=kw["track_tilts"],
                    filter=filt)
    system = fo.ScalarSource(u) | pz
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    out = orc.asprop(u0, ds[0], ds[1], lams, z0, 1, n0=n0, tilts=tilts, **kw)
    assert orc.rel_l2(npy(system()["out"].electric).reshape(B, n, n), out) < FIELD_TOL
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    gz, scale = orc.asprop_z_gradient(u0, orc.sid_backward(out, target), ds[0], ds[1], lams, z0, 1, n0=n0,
                                      tilts=tilts, return_scale=True, **kw)
    tol = GRAD_TOL * abs(gz) + float(np.finfo(np.float32).eps) * scale
    assert abs(float(grads[pz]["z"].item()) - gz) < tol, (float(grads[pz]["z"].item()), gz, scale)
    # move z on the device: the next forward rebuilds every table from it
    pz.z.fill_(z0 + 30.0)
    out2 = orc.asprop(u0, ds[0], ds[1], lams, z0 + 30.0, 1, n0=n0, tilts=tilts, **kw)
    assert orc.rel_l2(npy(system()["out"].electric).reshape(B, n, n), out2) < FIELD_TOL


@pytest.mark.parametrize("d", [1, -1])
def test_fourier_phase_and_mask(fo, orc, d):
    """FourierPhase / FourierMask: a static Fourier filter fused into a chain as a
    propagator (AS -> FourierPhase -> Mask -> AS, one fused segment), and trainable
    FourierPhase / FourierMask with their spectral-domain gradients, against the
    oracle (the reference's conventions, unnormalised spectra included)."""
    rng = np.random.default_rng(23)
    n, B = 128, 3
    ds, lams = (1.0, 1.0), np.array([0.64, 0.8, 0.455])
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(11.0, x + 2 * b, y) for b in range(B)]) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    fphi = lambda fx, fy: 40.0 * (fx ** 2 + fy ** 2) + 3.0 * fx
    FX, FY = np.meshgrid(np.fft.fftfreq(n, ds[0]), np.fft.fftfreq(n, ds[1]))
    phiF = fphi(FX, FY)
    m1 = c64(0.5 + rng.uniform(0, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    target = f32(np.abs(orc.gaussian(9.0, x - 3, y)) ** 2)
    u = fo.ScalarField(u0, ds, lams)

    fp = fo.FourierPhase(u, fphi)
    c1 = fo.Mask(u, m1, trainable=True)
    system = fo.OpticalSystem(fo.ScalarSource(u), [fo.ASProp(u, 200.0), fp, c1, fo.ASProp(u, 150.0)], direction=d)
    assert len(system.segments(u)) == 1  # the Fourier phase rides in a column pass
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    a1 = orc.asprop(u0, 1.0, 1.0, lams, 200.0, d)
    a2 = orc.fourier_forward(a1, np.exp(1j * phiF), d)
    a3 = orc.mask_forward(a2, m1, d)
    out = orc.asprop(a3, 1.0, 1.0, lams, 150.0, d)
    assert orc.rel_l2(npy(system()["out"].electric).reshape(B, n, n), out) < FIELD_TOL
    dv = orc.asprop(orc.sid_backward(out, target), 1.0, 1.0, lams, 150.0, -d)
    _, gm = orc.mask_backward(dv, m1, a2, d)
    assert orc.rel_l2(npy(grads[c1]["m"]), gm) < GRAD_TOL

    for cls, param in ((fo.FourierPhase, f32(phiF)), (fo.FourierMask, m1)):
        comp = cls(u, param, trainable=True)
        system = fo.OpticalSystem(fo.ScalarSource(u), [fo.ASProp(u, 200.0), comp, fo.ASProp(u, 150.0)], direction=d)
        loss, grads = fo.withgradient(metric, system)
        w = np.exp(1j * np.asarray(param, dtype=np.float64)) if cls is fo.FourierPhase else param
        a2 = orc.fourier_forward(a1, w, d)
        out = orc.asprop(a2, 1.0, 1.0, lams, 150.0, d)
        c_ref, _ = orc.sid_value(out, target)
        assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
        dv = orc.asprop(orc.sid_backward(out, target), 1.0, 1.0, lams, 150.0, -d)
        if cls is fo.FourierPhase:
            _, g = orc.fourier_phase_backward(dv, param, a1, d)
        else:
            _, g = orc.fourier_mask_backward(dv, param, a1, d)
        assert orc.rel_l2(npy(grads[comp][comp.pname]), g) < GRAD_TOL


@pytest.mark.parametrize("d", [1, -1])
def test_tea_doe_standalone_and_fused(fo, orc, d):
    """TeaDOE with a dispersive dn(λ) and a complex r(λ) on a two-wavelength batch:
    the standalone kernels (forward, adjoint, height gradient) and the same element
    fused into a chain (Tea -> AS -> Mask -> AS -> SID) with its gradient."""
    rng = np.random.default_rng(31)
    n, B = 128, 4
    ds, lams = (1.0, 1.0), np.array([0.64, 0.455, 0.64, 0.455])
    dn = lambda lam: 0.45 + 0.01 / lam ** 2
    r = lambda lam: 0.95 * np.exp(0.2j * lam)
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(14.0, x, y)] * B) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    h = f32(rng.uniform(0, 1.2, (n, n)))
    k, rv = orc.tea_coefs(lams, dn, r)

    u = fo.ScalarField(u0, ds, lams)
    tea = fo.TeaDOE(u, dn, h, r=r, trainable=True)
    v = u.copy()
    saved = torch.empty_like(v.electric)
    tea.propagate_and_save_(v, saved, d)
    ref = orc.tea_forward(u0, h, k, rv, d)
    assert orc.rel_l2(npy(v.electric).reshape(B, n, n), ref) < FIELD_TOL
    w0 = c64(rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n)))
    dvf = fo.ScalarField(w0, ds, lams)
    g = torch.empty((n, n), dtype=torch.float32, device="cuda")
    tea.backpropagate_with_gradient_(dvf, saved, g, d)
    du_ref, g_ref = orc.tea_backward(w0, h, k, rv, u0, d)
    assert orc.rel_l2(npy(dvf.electric).reshape(B, n, n), du_ref) < FIELD_TOL
    assert orc.rel_l2(npy(g), g_ref) < GRAD_TOL

    m1 = c64(0.5 + rng.uniform(0, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    target = f32(np.abs(orc.gaussian(10.0, x - 4, y)) ** 2)
    c1 = fo.Mask(u, m1, trainable=True)
    zs = [350.0, 250.0]
    system = fo.OpticalSystem(fo.ScalarSource(u), [tea, fo.ASProp(u, zs[0]), c1, fo.ASProp(u, zs[1])],
                              direction=d)
    assert len(system.segments(u)) == 1  # fused: Tea -> AS -> Mask -> AS
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    a0 = orc.tea_forward(u0, h, k, rv, d)
    a1 = orc.asprop(a0, 1.0, 1.0, lams, zs[0], d)
    a2 = orc.mask_forward(a1, m1, d)
    out = orc.asprop(a2, 1.0, 1.0, lams, zs[1], d)
    assert orc.rel_l2(npy(system()["out"].electric).reshape(B, n, n), out) < FIELD_TOL
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.asprop(orc.sid_backward(out, target), 1.0, 1.0, lams, zs[1], -d)
    dv, gm = orc.mask_backward(dv, m1, a1, d)
    dv = orc.asprop(dv, 1.0, 1.0, lams, zs[0], -d)
    _, gh = orc.tea_backward(dv, h, k, rv, u0, d)
    assert orc.rel_l2(npy(grads[c1]["m"]), gm) < GRAD_TOL
    assert orc.rel_l2(npy(grads[tea]["h"]), gh) < GRAD_TOL


# ---------------------------------------------------------------------------
# AS_BPM
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("every", [1, 0, 3, 7])
def test_bpm_forward_and_gradient(fo, orc, every):
    rng = np.random.default_rng(9)
    n, ns, B = 64, 20, 2
    ds, lams, n0, L = (0.5, 0.5), np.array([1.064, 0.9]), 1.45, 40.0
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(6.0, x, y), orc.gaussian(5.0, x - 1, y)]))
    dn = f32(3e-3 * rng.standard_normal((ns, n, n)))
    target = f32(np.abs(orc.gaussian(5.0, x, y)) ** 2)
    u = fo.ScalarField(u0, ds, lams)
    bpm = fo.AS_BPM(u, L, n0, dn, trainable=True, checkpoint_every=every)
    system = fo.ScalarSource(u) | bpm
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    out, saves = orc.bpm_forward(u0, ds[0], ds[1], lams, L, n0, dn, 1, save=True)
    assert orc.rel_l2(npy(system()["out"].electric), out) < FIELD_TOL
    _, g = orc.bpm_backward(orc.sid_backward(out, target), ds[0], ds[1], lams, L, n0, dn, saves, 1)
    assert orc.rel_l2(npy(grads[bpm]["dn"]), g) < GRAD_TOL


def test_bpm_config_shape(fo, orc):
    """AS_BPM at the benchmark's grid (1024^2, ds = 0.25 um, n0 = 1.45, smooth dn of
    amplitude 5e-3), 16 slices with checkpoints every 4: field and d(dn) against the oracle."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(44)
    n, ns, ds, lam, n0 = 1024, 16, (0.25, 0.25), 1.064, 1.45
    dn = gaussian_filter(rng.standard_normal((ns, n, n)).astype(np.float32), (2.0, 4.0, 4.0))
    dn = f32(dn * (5e-3 / np.max(np.abs(dn))))
    x, y = orc.spatial_vectors((n, n), ds)
    tilt = 0.02
    u0 = c64(orc.gaussian(40.0, x, y) * np.exp(2j * np.pi * np.sin(tilt) / lam * x[None, :]))
    target = f32(np.abs(orc.gaussian(35.0, x - 3, y)) ** 2)
    u = fo.ScalarField(u0, ds, lam)
    bpm = fo.AS_BPM(u, float(ns), n0, dn, trainable=True, checkpoint_every=4)
    system = fo.ScalarSource(u) | bpm
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    out, saves = orc.bpm_forward(u0, ds[0], ds[1], lam, float(ns), n0, dn, 1, save=True)
    assert orc.rel_l2(npy(system()["out"].electric), out) < FIELD_TOL
    _, g = orc.bpm_backward(orc.sid_backward(out, target), ds[0], ds[1], lam, float(ns), n0, dn, saves, 1)
    assert orc.rel_l2(npy(grads[bpm]["dn"]), g) < GRAD_TOL


def test_rs_two_doe_config_shape(fo, orc):
    """The two-DOE RSProp chain at the benchmark's shape (512^2 padded to 1024^2,
    z = 1500 / 2000 / 1500 um): loss and both mask gradients against the oracle."""
    rng = np.random.default_rng(45)
    n, ds, lam = 512, (1.0, 1.0), 1.064
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = orc.gaussian(30.0, x, y)
    u0 = c64(u0 / np.sqrt(orc.power(u0, ds)))
    t = np.abs(orc.gaussian(30.0, x - 60.0, y) + orc.gaussian(30.0, x + 60.0, y)) ** 2
    t = f32(t / (t.sum() * ds[0] * ds[1]))
    p1 = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    p2 = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    u = fo.ScalarField(u0, ds, lam)
    m1 = fo.Phase(u, p1, trainable=True)
    m2 = fo.Phase(u, p2, trainable=True)
    system = fo.ScalarSource(u) | fo.RSProp(u, 1500.0) | m1 | fo.RSProp(u, 2000.0) | m2 | fo.RSProp(u, 1500.0)
    metric = fo.SquaredIntensityDifference((u, t))
    loss, grads = fo.withgradient(metric, system)
    a1 = orc.rsprop(u0, 1.0, 1.0, lam, 1500.0)
    a2 = orc.rsprop(orc.phase_forward(a1, p1), 1.0, 1.0, lam, 2000.0)
    out = orc.rsprop(orc.phase_forward(a2, p2), 1.0, 1.0, lam, 1500.0)
    c_ref, _ = orc.sid_value(out, t)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.rsprop(orc.sid_backward(out, t), 1.0, 1.0, lam, 1500.0, orc.BACKWARD)
    dv, g2 = orc.phase_backward(dv, p2, a2)
    dv = orc.rsprop(dv, 1.0, 1.0, lam, 2000.0, orc.BACKWARD)
    _, g1 = orc.phase_backward(dv, p1, a1)
    assert orc.rel_l2(npy(grads[m2]["phi"]), g2) < GRAD_TOL
    assert orc.rel_l2(npy(grads[m1]["phi"]), g1) < GRAD_TOL


def test_bpm_backward_direction(fo, orc):
    rng = np.random.default_rng(10)
    n, ns = 32, 6
    ds, lam, n0, L = (0.5, 0.5), 1.064, 1.45, 12.0
    u0 = rand_field(rng, (n, n))
    dv0 = rand_field(rng, (n, n))
    dn = f32(5e-3 * rng.standard_normal((ns, n, n)))
    u = fo.ScalarField(u0, ds, lam)
    bpm = fo.AS_BPM(u, L, n0, dn, trainable=True, checkpoint_every=2)
    v = u.copy()
    bpm.propagate_and_save_(v, None, fo.Backward)
    out, saves = orc.bpm_forward(u0, ds[0], ds[1], lam, L, n0, dn, -1, save=True)
    assert orc.rel_l2(npy(v.electric), out) < FIELD_TOL
    dv = fo.ScalarField(dv0, ds, lam)
    g = torch.empty_like(bpm.dn)
    bpm.backpropagate_with_gradient_(dv, None, g, fo.Backward)
    du_ref, g_ref = orc.bpm_backward(dv0, ds[0], ds[1], lam, L, n0, dn, saves, -1)
    assert orc.rel_l2(npy(dv.electric), du_ref) < FIELD_TOL
    assert orc.rel_l2(npy(g), g_ref) < GRAD_TOL


@pytest.mark.parametrize("paraxial,tilted,d", [(True, False, 1), (False, True, 1), (True, True, -1)])
def test_bpm_paraxial_and_tilted(fo, orc, paraxial, tilted, d):
    """AS_BPM with Fresnel steps and with tilted fields (tilted kernel and the per-field
    kdz = 2 pi dz / (cos theta_x cos theta_y), bpm.jl:3-6): output field and d(dn)
    against the oracle, with recomputed segments (checkpoint_every=3)."""
    rng = np.random.default_rng(12 if tilted else 13)
    n, ns = 64, 8
    ds, lams, n0, L = (0.5, 0.5), [1.064, 0.8], 1.45, 16.0
    u0 = rand_field(rng, (2, n, n))
    dv0 = rand_field(rng, (2, n, n))
    dn = f32(5e-3 * rng.standard_normal((ns, n, n)))
    tilts = ([0.05, -0.02], [-0.03, 0.04]) if tilted else None  # (theta_x per field, theta_y per field)
    u = fo.ScalarField(u0, ds, lams, tilts=tilts)
    bpm = fo.AS_BPM(u, L, n0, dn, paraxial=paraxial, trainable=True, checkpoint_every=3)
    v = u.copy()
    bpm.propagate_and_save_(v, None, d)
    th = None if tilts is None else np.stack(tilts, axis=1)  # one (theta_x, theta_y) pair per field
    out, saves = orc.bpm_forward(u0, ds[0], ds[1], lams, L, n0, dn, d, save=True, paraxial=paraxial, tilts=th)
    assert orc.rel_l2(npy(v.electric), out) < FIELD_TOL
    dv = fo.ScalarField(dv0, ds, lams, tilts=tilts)
    g = torch.empty_like(bpm.dn)
    bpm.backpropagate_with_gradient_(dv, None, g, d)
    du_ref, g_ref = orc.bpm_backward(dv0, ds[0], ds[1], lams, L, n0, dn, saves, d, paraxial=paraxial, tilts=th)
    assert orc.rel_l2(npy(dv.electric), du_ref) < FIELD_TOL
    assert orc.rel_l2(npy(g), g_ref) < GRAD_TOL


# ---------------------------------------------------------------------------
# Metric and optimiser
# ---------------------------------------------------------------------------

def test_sid_multi_target(fo, orc):
    rng = np.random.default_rng(12)
    u0 = rand_field(rng, (2, 3, 40, 24))  # Julia (24, 40, 3, 2): target (24, 40, 3)
    target = f32(rng.uniform(0, 4, (3, 40, 24)))
    u = fo.ScalarField(u0, (1.0, 1.0), 1.0)
    m = fo.SquaredIntensityDifference((u, target))
    loss = npy(m(u))
    ref, _ = orc.sid_value(u0.reshape(6, 40, 24), target)
    assert np.max(np.abs(loss - ref) / np.abs(ref)) < 1e-4
    du = m.backpropagate(u)
    du_ref = orc.sid_backward(u0.reshape(6, 40, 24), target).reshape(u0.shape)
    assert orc.rel_l2(npy(du.electric), du_ref) < 1e-5


def test_fista_clamp_tv(fo, orc):
    rng = np.random.default_rng(13)
    x0 = f32(rng.standard_normal((37, 53)))
    xs = torch.tensor(x0, dtype=torch.float32, device="cuda")
    rule = fo.ProxRule(fo.Fista(0.3), fo.ClampProx(-0.5, 0.7))
    st = rule.init(xs)
    xo = x0.copy()
    so = orc.FistaState(xo)
    for it in range(5):
        g = f32(rng.standard_normal(x0.shape))
        rule.apply_(st, xs, torch.tensor(g, dtype=torch.float32, device="cuda"))
        orc.fista_apply(0.3, so, xo, g)
        orc.clamp_prox(xo, -0.5, 0.7)
        assert orc.rel_l2(npy(xs), xo) < 1e-5
    # plain Fista (the float4 body and the scalar tail), and the clamp fused into the
    # Fista pass equal to Fista followed by ClampProx
    for shape in ((64, 48), (37, 53)):
        x1 = f32(rng.standard_normal(shape))
        a, b, c = (torch.tensor(x1, dtype=torch.float32, device="cuda") for _ in range(3))
        fa, fb = fo.Fista(0.2), fo.Fista(0.2)
        sa, sb = fa.init(a), fb.init(b)
        clamp = fo.ClampProx(-0.4, 0.6)
        fused = fo.ProxRule(fo.Fista(0.2), clamp)
        sc = fused.init(c)
        xo = x1.copy()
        so = orc.FistaState(xo)
        for it in range(4):
            g = f32(rng.standard_normal(shape))
            gt = torch.tensor(g, dtype=torch.float32, device="cuda")
            fa.apply_(sa, a, gt)
            orc.fista_apply(0.2, so, xo, g)
            assert orc.rel_l2(npy(a), xo) < 1e-5
            fb.apply_(sb, b, gt)
            clamp.apply_(None, b)
            fused.apply_(sc, c, gt)
            assert np.array_equal(npy(b), npy(c))
    for iso in (True, False):
        y0 = f32(rng.standard_normal((40, 30)))
        yt = torch.tensor(y0, dtype=torch.float32, device="cuda")
        tv = fo.TVProx(0.2, 25, isotropic=iso)
        tv.apply_(tv.init(yt), yt)
        ref = orc.tv_prox(y0.copy(), 0.2, 25, isotropic=iso)
        assert orc.rel_l2(npy(yt), ref) < 1e-5
    # tol: the device-side test stops after two dual updates here (changes 3.3, 0.32,
    # then 7.8e-3 < 1e-2), like the oracle; TV_denoise! and a complex parameter
    y0 = np.random.default_rng(3).standard_normal((40, 30))
    yt = torch.tensor(f32(y0), dtype=torch.float32, device="cuda")
    fo.tv_denoise_(yt, 1.0, 25, tol=1e-2)
    ref = orc.tv_prox(f32(y0), 1.0, 25, tol=1e-2)
    assert orc.rel_l2(npy(yt), ref) < 1e-5
    assert orc.rel_l2(ref, orc.tv_prox(f32(y0), 1.0, 25)) > 1e-4
    z0 = c64(rng.standard_normal((40, 30)) + 1j * rng.standard_normal((40, 30)))
    zt = torch.tensor(z0, dtype=torch.complex64, device="cuda")
    tvc = fo.TVProx(0.2, 25)
    tvc.apply_(tvc.init(zt), zt)
    assert orc.rel_l2(npy(zt), orc.tv_prox(z0.copy(), 0.2, 25)) < 1e-5
    # 1-D and 3-D parameters (a dn volume of AS_BPM is 3-D): the reference's n-D D / D^T
    for shape in ((50,), (6, 10, 12)):
        for iso in (True, False):
            a0 = f32(rng.standard_normal(shape))
            at = torch.tensor(a0, dtype=torch.float32, device="cuda")
            fo.tv_denoise_(at, 0.3, 20, isotropic=iso)
            assert orc.rel_l2(npy(at), orc.tv_prox(a0.copy(), 0.3, 20, isotropic=iso)) < 1e-5, (shape, iso)


def test_ista_positive_prox(fo, orc):
    """IstaProx on real and complex parameters and PositiveProx, bit-exact against the
    oracle evaluated in float32 (thresholds exactly representable in float32), and
    ProxRule(Fista, IstaProx) against Fista followed by the oracle's shrink."""
    rng = np.random.default_rng(31)
    x0 = rng.standard_normal((37, 53)).astype(np.float32)
    xs = torch.tensor(x0, device="cuda")
    fo.IstaProx(0.25, 0.125).apply_(None, xs)
    assert np.array_equal(npy(xs), orc.ista_prox(x0.copy(), 0.25, 0.125))
    z0 = (rng.standard_normal((3, 40, 24)) + 1j * rng.standard_normal((3, 40, 24))).astype(np.complex64)
    zs = torch.tensor(z0, device="cuda")
    fo.IstaProx(0.375, -0.5).apply_(None, zs)
    ref = orc.ista_prox(z0.copy(), 0.375, -0.5)
    assert ref.dtype == np.complex64 and np.array_equal(npy(zs), ref)
    xs = torch.tensor(x0, device="cuda")
    fo.PositiveProx().apply_(None, xs)
    assert np.array_equal(npy(xs), orc.positive_prox(x0.copy()))
    with pytest.raises(TypeError):
        fo.PositiveProx().apply_(None, zs)
    # PointwiseProx of a device expression equals the built-in operator it spells out
    xa, xb = (torch.tensor(x0, device="cuda") for _ in range(2))
    fo.PointwiseProx(lambda v: torch.clamp(v, min=0.0)).apply_(None, xa)
    fo.PositiveProx().apply_(None, xb)
    assert torch.equal(xa, xb)
    rule = fo.ProxRule(fo.Fista(0.3), fo.IstaProx(0.125))
    xs = torch.tensor(x0, device="cuda")
    st = rule.init(xs)
    xo = x0.astype(np.float64)
    so = orc.FistaState(xo)
    for it in range(4):
        g = rng.standard_normal(x0.shape).astype(np.float32)
        rule.apply_(st, xs, torch.tensor(g, device="cuda"))
        orc.fista_apply(0.3, so, xo, g.astype(np.float64))
        orc.ista_prox(xo, 0.125)
        assert orc.rel_l2(npy(xs), xo) < 1e-5


def test_trainable_source(fo, orc):
    """A trainable ScalarSource (sources/scalar_source.jl:39-106): withgradient returns
    the input-field gradient as its "u0" gradient, through the shared metric + seed
    pass and through the separate sweeps (a DotProduct loss), and one Fista step
    updates the complex source field like the oracle's Fista on complex values."""
    rng = np.random.default_rng(46)
    n = 128
    lams = [0.64, 0.538]
    u0 = rand_field(rng, (2, n, n))
    target = f32(rng.uniform(0, 2, (2, n, n)))
    phi = f32(rng.uniform(0, 6, (n, n)))
    u = fo.ScalarField(u0, (0.5, 0.5), lams)
    src = fo.ScalarSource(u, trainable=True)
    ph = fo.Phase(u, phi, trainable=True)
    system = src | ph | fo.ASProp(u, 200.0)
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    out = orc.asprop(orc.phase_forward(u0, phi), 0.5, 0.5, lams, 200.0)
    g = orc.asprop(orc.sid_backward(out, target), 0.5, 0.5, lams, 200.0, orc.BACKWARD)
    du_ref, gphi = orc.phase_backward(g, phi, u0)
    assert orc.rel_l2(npy(grads[src]["u0"]), du_ref) < GRAD_TOL
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL

    # two Fista steps, so that the momentum term (x - x_k) of the complex field counts
    opt = fo.setup(fo.Fista(0.1), system)
    so = orc.FistaState(u0.copy())
    x_ref = u0.copy()
    for it in range(2):
        g_src = npy(grads[src]["u0"])
        fo.update_(opt, system, grads)
        orc.fista_apply(0.1, so, x_ref, g_src)
        assert orc.rel_l2(npy(src.u0.electric), x_ref) < 1e-6, it
        if it == 0:
            _, grads = fo.withgradient(metric, system)

    v0 = rand_field(rng, (2, n, n))
    dp = fo.DotProduct(fo.ScalarField(v0, (0.5, 0.5), lams))
    _, grads = fo.withgradient(dp, system)
    uu = npy(src.u0.electric)
    out = orc.asprop(orc.phase_forward(uu, npy(ph.phi)), 0.5, 0.5, lams, 200.0)
    g = orc.dot_product_backward(v0, np.ones(2))
    g = orc.asprop(g, 0.5, 0.5, lams, 200.0, orc.BACKWARD)
    du_ref, _ = orc.phase_backward(g, npy(ph.phi), uu)
    assert orc.rel_l2(npy(grads[src]["u0"]), du_ref) < GRAD_TOL


def test_plain_rules(fo, orc):
    """Descent / Momentum / Nesterov (Optimisers.jl 0.4, re-exported by the reference):
    three steps on a float32 parameter and on a complex64 one, bit-exact against the
    oracle evaluated in float32 with the rules' operation order, and ProxRule(Momentum,
    ClampProx)."""
    rng = np.random.default_rng(47)
    cases = [(fo.Descent(0.1), "descent", 0.1, 0.0), (fo.Momentum(0.05, 0.9), "momentum", 0.05, 0.9),
             (fo.Nesterov(0.01, 0.8), "nesterov", 0.01, 0.8)]
    for rule, name, eta, rho in cases:
        for cplx in (False, True):
            shape = (37, 53)
            x0 = rng.standard_normal(shape).astype(np.float32)
            if cplx:
                x0 = (x0 + 1j * rng.standard_normal(shape)).astype(np.complex64)
            xs = torch.tensor(x0, device="cuda")
            st = rule.init(xs)
            xo = x0.view(np.float32).copy() if cplx else x0.copy()
            vo = np.zeros_like(xo)
            for it in range(3):
                g = rng.standard_normal(shape).astype(np.float32)
                if cplx:
                    g = (g + 1j * rng.standard_normal(shape)).astype(np.complex64)
                rule.apply_(st, xs, torch.tensor(g, device="cuda"))
                orc.rule_step(name, xo, vo, g.view(np.float32) if cplx else g, eta, rho)
                got = xs.detach().cpu().numpy()
                got = got.view(np.float32) if cplx else got
                assert np.array_equal(got, xo), (name, cplx, it)
    pr = fo.ProxRule(fo.Momentum(0.05, 0.9), fo.ClampProx(-0.5, 0.5))
    x0 = rng.standard_normal((16, 24)).astype(np.float32)
    xs = torch.tensor(x0, device="cuda")
    st = pr.init(xs)
    xo, vo = x0.copy(), np.zeros_like(x0)
    for it in range(2):
        g = rng.standard_normal(x0.shape).astype(np.float32)
        pr.apply_(st, xs, torch.tensor(g, device="cuda"))
        orc.clamp_prox(orc.rule_step("momentum", xo, vo, g, 0.05, 0.9), -0.5, 0.5)
        assert np.array_equal(xs.cpu().numpy(), xo)


def test_merge_rules(fo, orc):
    """The reference's merge rules (system/merge_rules.jl:1-80) on adjacent static
    components: ASProp(300) | ASProp(200) becomes one ASProp(500), Phase | Phase | Mask
    one Mask, so the system runs as one fused chain of two propagators; the output
    matches the oracle applying every component, and the unmerged system."""
    rng = np.random.default_rng(48)
    n = 128
    lams = [0.64, 0.538]
    u0 = rand_field(rng, (2, n, n))
    phi1, phi2 = (f32(rng.uniform(0, 6, (n, n))) for _ in range(2))
    m = c64(rng.uniform(0.5, 1.0, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    u = fo.ScalarField(u0, (0.5, 0.5), lams)
    comps = [fo.ASProp(u, 300.0), fo.ASProp(u, 200.0), fo.Phase(u, phi1), fo.Phase(u, phi2), fo.Mask(u, m),
             fo.ASProp(u, 250.0), fo.ASProp(u, -100.0)]
    system = fo.OpticalSystem(fo.ScalarSource(u), comps)
    merged = system.merged_components(u)
    assert [type(c).__name__ for c in merged] == ["ASProp", "Mask", "ASProp", "ASProp"]
    assert merged[0].z == 500.0 and merged[2].z == 250.0  # opposite signs stay apart
    segs = system.segments(u)
    assert len(segs) == 1 and len(segs[0].props) == 3
    out = npy(system()["out"].electric)
    P = lambda v, z: orc.asprop(v, 0.5, 0.5, lams, z)
    ref = P(P(u0, 300.0), 200.0)
    ref = orc.mask_forward(orc.phase_forward(orc.phase_forward(ref, phi1), phi2), m)
    ref = P(P(ref, 250.0), -100.0)
    assert orc.rel_l2(out, ref) < FIELD_TOL
    plain = fo.OpticalSystem(fo.ScalarSource(u), comps, merge_components=False)
    assert orc.rel_l2(npy(plain()["out"].electric), ref) < FIELD_TOL


def test_squared_field_difference(fo, orc):
    """SquaredFieldDifference values and pull-back against the oracle, the docstring's
    16.0, and the gradient of a phase mask through Phase -> ASProp -> the metric."""
    one = fo.ScalarField(np.ones((4, 4), np.complex64), (1.0, 1.0), 1.064)
    zero = fo.ScalarField(np.zeros((4, 4), np.complex64), (1.0, 1.0), 1.064)
    assert npy(fo.SquaredFieldDifference(one)(zero)).tolist() == [16.0]
    rng = np.random.default_rng(32)
    n, B = 256, 5
    ds, lams = (0.8, 0.8), np.array([0.64, 0.538, 0.455, 0.64, 0.538])
    u0 = rand_field(rng, (B, n, n))
    v0 = rand_field(rng, (B, n, n))
    u = fo.ScalarField(u0, ds, lams)
    v = fo.ScalarField(v0, ds, lams)
    m = fo.SquaredFieldDifference(v)
    c = npy(m(u))
    c_ref = orc.sfd_value(u0.astype(np.complex128), v0.astype(np.complex128))
    assert np.max(np.abs(c - c_ref) / c_ref) < 1e-5
    # repeated evaluation is bit-identical (fixed-order sums)
    assert np.array_equal(npy(m(u)), c)
    w = f32(rng.standard_normal(B))
    du = m.backpropagate(u, torch.tensor(w, device="cuda"))
    assert orc.rel_l2(npy(du.electric), orc.sfd_backward(u0, v0, w)) < 1e-6
    du = m.backpropagate(u)
    assert orc.rel_l2(npy(du.electric), orc.sfd_backward(u0, v0)) < 1e-6
    with pytest.raises(ValueError):
        m(fo.ScalarField(u0[:2], ds, lams[:2]))

    phi = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    ph = fo.Phase(u, phi, trainable=True)
    system = fo.ScalarSource(u) | ph | fo.ASProp(u, 300.0)
    loss, grads = fo.withgradient(m, system)
    a = orc.asprop(orc.phase_forward(u0, phi), ds[0], ds[1], lams, 300.0)
    lr = orc.sfd_value(a, v0).sum()
    assert abs(float(loss) - lr) / lr < 1e-5
    g = orc.asprop(orc.sfd_backward(a, v0), ds[0], ds[1], lams, 300.0, orc.BACKWARD)
    _, gphi = orc.phase_backward(g, phi, u0)
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL


# ---------------------------------------------------------------------------
# Full-size properties (sizes where the FP64 oracle is too slow)
# ---------------------------------------------------------------------------

def test_fullsize_unitarity_and_power(fo):
    torch.manual_seed(0)
    n = 2048
    u0 = torch.randn(2, 3, n, n, dtype=torch.complex64, device="cuda")  # Julia (n, n, 3, 2)
    u = fo.ScalarField(u0, (0.5, 0.5), [0.640, 0.538, 0.455])
    p = fo.ASProp(u, 5000.0)
    v = p.propagate(u)
    # power is conserved up to the evanescent part, which is empty at ds = 0.5 > lambda/2... check ratio
    pw0 = (u0.abs() ** 2).sum(dim=(-2, -1))
    pw1 = (v.electric.abs() ** 2).sum(dim=(-2, -1))
    assert torch.all(pw1 <= pw0 * (1 + 1e-5))
    w = p.propagate(v, fo.Backward)
    # propagating the result back recovers the propagating part of the input exactly
    v2 = p.propagate(w)
    rel = torch.linalg.vector_norm(v2.electric - v.electric) / torch.linalg.vector_norm(v.electric)
    assert rel.item() < 1e-5
    # linearity
    a = p.propagate(fo.ScalarField(u0 * (2 - 1j), (0.5, 0.5), [0.640, 0.538, 0.455]))
    rel = torch.linalg.vector_norm(a.electric - v.electric * (2 - 1j)) / torch.linalg.vector_norm(a.electric)
    assert rel.item() < 1e-6


def test_graph_capture_replays_iteration(fo, orc):
    rng = np.random.default_rng(14)
    n = 128
    u0 = rand_field(rng, (2, n, n))
    u = fo.ScalarField(u0, (1.0, 1.0), [1.0, 0.7])
    ph = fo.Phase(u, f32(rng.uniform(0, 6, (n, n))), trainable=True, buffered=True)
    system = fo.ScalarSource(u) | ph | fo.ASProp(u, 300.0) | fo.Phase(u, f32(rng.uniform(0, 6, (n, n)))) \
        | fo.ASProp(u, 100.0)
    metric = fo.SquaredIntensityDifference((u, f32(rng.uniform(0, 1, (n, n)))))
    opt = fo.setup(fo.Fista(0.01), system)
    phi_start = ph.phi.clone()
    losses_eager = []
    for _ in range(3):
        loss, g = fo.withgradient(metric, system)
        fo.update_(opt, system, g)
        losses_eager.append(float(loss))
    phi_eager = ph.phi.clone()
    # same iterations, captured once and replayed
    ph.phi.copy_(phi_start)
    opt = fo.setup(fo.Fista(0.01), system)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        lib = fo.load_library()
        x = system.source.propagate()  # allocations happen outside the capture
        tape = []
        system.forward(x, tape)
        torch.cuda.synchronize()
        ph.phi.copy_(phi_start)
        opt = fo.setup(fo.Fista(0.01), system)
        torch.cuda.synchronize()
        du = x.similar()
        h = C.c_void_p()
        assert lib.fo_graph_begin(C.c_void_p(s.cuda_stream)) == 0
        x.electric.copy_(system.source.u0.electric)
        tape = []
        system.forward(x, tape)
        loss_t = metric(x)
        grads = system.backward(du, tape, seed=(metric, x))
        fo.update_(opt, system, grads)
        assert lib.fo_graph_end(C.c_void_p(s.cuda_stream), C.byref(h)) == 0
        losses = []
        for _ in range(3):
            assert lib.fo_graph_launch(h, C.c_void_p(s.cuda_stream)) == 0
            s.synchronize()
            losses.append(float(loss_t.sum()))
        lib.fo_graph_destroy(h)
    torch.cuda.synchronize()
    assert np.allclose(losses, losses_eager, rtol=1e-5)
    assert torch.allclose(ph.phi, phi_eager, rtol=1e-5, atol=1e-6)


# ---------------------------------------------------------------------------
# Every launch-shape variant of the passes (forced through the environment)
# ---------------------------------------------------------------------------

_VARIANTS = {512: (3, 9), 1024: (4, 10), 2048: (4, 9), 4096: (2, 6)}


@pytest.mark.parametrize("n", sorted(_VARIANTS))
def test_every_pass_variant(fo, orc, n, monkeypatch):
    rng = np.random.default_rng(n + 7)
    lams = np.array([0.9, 0.7])
    B = 4 if n <= 2048 else 2
    u0 = rand_field(rng, (B // 2, 2, n, n))
    phi = f32(rng.uniform(0, 2 * np.pi, (n, n)))
    ref = orc.asprop(orc.phase_forward(u0.reshape(B, n, n), phi), 1.0, 1.0, np.tile(lams, B // 2), 400.0)
    n_row, n_col = _VARIANTS[n]
    combos = [(r, 0) for r in range(n_row)] + [(0, c) for c in range(1, n_col)]
    for rv, cv in combos:
        for pf in ("0", "1", "2"):  # row staging: none, cp.async, register prefetch
            monkeypatch.setenv("FO_ROW_VARIANT", str(rv))
            monkeypatch.setenv("FO_COL_VARIANT", str(cv))
            monkeypatch.setenv("FO_PREFETCH", "0" if pf == "0" else "1")
            monkeypatch.setenv("FO_ROW_PF", pf)
            monkeypatch.setenv("FO_AUTOTUNE", "0")
            u = fo.ScalarField(u0, (1.0, 1.0), lams)
            system = fo.ScalarSource(u) | fo.Phase(u, phi) | fo.ASProp(u, 400.0)
            got = npy(system()["out"].electric).reshape(B, n, n)
            err = orc.rel_l2(got, ref)
            assert err < FIELD_TOL, (rv, cv, pf, err)


def test_ragged_batch_per_problem(fo, orc):
    """Ragged batch (sizes, wavelengths, distances, waists, offsets drawn per
    problem, as in the benchmark's ragged configuration): every problem's loss and
    mask gradient against the FP64 oracle."""
    import bench
    probs = bench.ragged_problems(seed=99, count=6, sizes=(64, 128, 256))
    systems = bench.build_ragged(fo, probs)
    for pr, (system, metric, ph, src, x_, du) in zip(probs, systems):
        loss, grads = fo.withgradient(metric, system)
        u0 = npy(src.electric)
        phi = npy(ph.phi)
        t = npy(metric.target)[0]
        v = orc.asprop(orc.phase_forward(u0, phi), 1.0, 1.0, pr["lam"], pr["z"])
        c, _ = orc.sid_value(v, t)
        dv = orc.asprop(orc.sid_backward(v, t), 1.0, 1.0, pr["lam"], pr["z"], orc.BACKWARD)
        _, g = orc.phase_backward(dv, phi, u0)
        assert abs(float(loss) - c.sum()) / c.sum() < 1e-4
        assert orc.rel_l2(npy(grads[ph]["phi"]), g) < GRAD_TOL


def test_ragged_persistent_launch(fo, orc):
    """fo_ragged_batch: problems of different sizes (256..1024, with sizes,
    wavelengths, distances, waists, offsets and masks drawn per problem) run forward
    + adjoint in one persistent cooperative launch; every problem's propagated field,
    loss and mask gradient against the FP64 oracle, on two consecutive runs (the
    launch resets its own counters)."""
    import bench
    probs = bench.ragged_problems(seed=123, count=7, sizes=(256, 512, 1024))
    specs, refs = [], []
    for pr in probs:
        n = pr["n"]
        rng = np.random.default_rng(pr["seed"])
        x, y = fo.spatial_vectors((n, n), (1.0, 1.0))
        u0 = fo.gaussian(pr["w0"], x - pr["off"][0], y - pr["off"][1]).astype(np.complex64)
        u0 = (u0 / np.sqrt(np.sum(np.abs(u0) ** 2))).astype(np.complex64)
        phi = rng.uniform(0, 2 * np.pi, (n, n)).astype(np.float32)
        t = (np.abs(fo.gaussian(pr["w0"], x, y)) ** 2).astype(np.float32)
        t = (t / t.sum()).astype(np.float32)
        u = fo.ScalarField(u0, (1.0, 1.0), pr["lam"])
        specs.append({"u": u, "phase": phi, "target": t, "z": pr["z"]})
        v = orc.asprop(orc.phase_forward(u0, phi), 1.0, 1.0, pr["lam"], pr["z"])
        c, _ = orc.sid_value(v, t)
        dv = orc.asprop(orc.sid_backward(v, t), 1.0, 1.0, pr["lam"], pr["z"], orc.BACKWARD)
        _, g = orc.phase_backward(dv, phi, u0)
        refs.append((v, float(c.sum()), g))
    rb = fo.RaggedBatch(specs)
    assert rb.info()["grid_ctas"] >= 1
    for _ in range(2):
        losses, outs, grads = rb.run()
        torch.cuda.synchronize()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        assert fo._capi.load().fo_device_status(stream) == 0
        for k, (v, c, g) in enumerate(refs):
            assert orc.rel_l2(npy(outs[k]), v) < FIELD_TOL, (k, probs[k]["n"])
            assert abs(float(losses[k]) - c) / c < 1e-4, (k, float(losses[k]), c)
            assert orc.rel_l2(npy(grads[k]), g) < GRAD_TOL, (k, probs[k]["n"])


def test_bounded_wait_reports_timeout(fo, orc, monkeypatch):
    """Failure detection without a GPU fault: a TMA column pass whose barrier is
    armed but whose copy is never issued must give up after its bounded wait (20 ms
    here), report FO_ERR_TIMEOUT through fo_device_status, and leave the context
    usable (the next, normal call is correct)."""
    capi = fo._capi
    lib = capi.load()
    n = 512
    rng = np.random.default_rng(77)
    u0 = rand_field(rng, (n, n))
    monkeypatch.setenv("FO_AUTOTUNE", "0")
    monkeypatch.setenv("FO_COL_VARIANT", "4")  # a TMA variant for 512
    monkeypatch.setenv("FO_WAIT_NS", "20000000")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.fo_device_status(stream) == 0
    u = fo.ScalarField(u0, (1.0, 1.0), 1.064)
    p = fo.ASProp(u, 300.0)
    monkeypatch.setenv("FO_TEST_SKIP_COPY", "1")
    v = u.copy()
    p.propagate_(v)
    rc = lib.fo_device_status(stream)
    assert rc == 5, rc  # FO_ERR_TIMEOUT
    assert "bounded device wait" in lib.fo_last_error().decode()
    monkeypatch.setenv("FO_TEST_SKIP_COPY", "0")
    v = p.propagate(u)
    assert lib.fo_device_status(stream) == 0
    assert orc.rel_l2(npy(v.electric), orc.asprop(u0, 1.0, 1.0, 1.064, 300.0)) < FIELD_TOL


# ---------------------------------------------------------------------------
# Field probes
# ---------------------------------------------------------------------------

def test_field_probes_in_fused_chain(fo, orc):
    """FieldProbe (system/field_probe.jl:31-43, collected by optical_system.jl:194-214)
    at every kind of plane of a fused chain -- the input, after a modulator, between
    two propagators, before and after the last modulator -- against the oracle's
    planes; the output matches the same system without probes, where the merge rules
    join the two propagators into one."""
    rng = np.random.default_rng(31)
    n, ds, lams = 128, (1.0, 1.0), [1.064, 0.8]
    u0 = rand_field(rng, (2, n, n))
    phi1, phi2 = f32(rng.uniform(0, 6, (n, n))), f32(rng.uniform(0, 6, (n, n)))
    u = fo.ScalarField(u0, ds, lams)
    m1, m2 = fo.Phase(u, phi1), fo.Phase(u, phi2)
    pa, pb = fo.ASProp(u, 300.0), fo.ASProp(u, 150.0)
    pr = [fo.FieldProbe() for _ in range(6)]
    system = fo.ScalarSource(u) | pr[0] | m1 | pr[1] | pa | pr[2] | pb | pr[3] | m2 | pr[4] | pr[5]
    plain = fo.ScalarSource(u) | m1 | pa | pb | m2
    segs = system.segments(u)
    assert len(segs) == 1 and len(segs[0].probes) == 6  # one fused chain, probes inside it
    res = system()
    a1 = orc.phase_forward(u0, phi1)
    a2 = orc.asprop(a1, 1.0, 1.0, lams, 300.0)
    a3 = orc.asprop(a2, 1.0, 1.0, lams, 150.0)
    a4 = orc.phase_forward(a3, phi2)
    refs = [u0, a1, a2, a3, a4, a4]
    for k, ref in enumerate(refs):
        assert pr[k] in res["probes"], k
        assert orc.rel_l2(npy(res["probes"][pr[k]].electric), ref) < FIELD_TOL, k
    assert orc.rel_l2(npy(res["out"].electric), a4) < FIELD_TOL
    assert orc.rel_l2(npy(res["out"].electric), npy(plain()["out"].electric)) < FIELD_TOL
    # a later call without probes leaves earlier probe copies alone
    keep = res["probes"][pr[2]].electric.clone()
    system.forward(system.source.u0.similar(), src=system.source.u0)
    assert torch.equal(keep, res["probes"][pr[2]].electric)


def test_field_probes_standalone(fo):
    """The reference's own probe test (test/optical_components_test.jl:212-236):
    probes around a constant pi/2 Phase with no propagator capture the input and
    the phase-shifted field."""
    n = 64
    u0 = np.ones((n, n), dtype=np.complex64)
    u = fo.ScalarField(u0, (1.0, 1.0), 1.0)
    p1, p2 = fo.FieldProbe(), fo.FieldProbe()
    system = fo.ScalarSource(u) | p1 | fo.Phase(u, np.full((n, n), np.pi / 2, dtype=np.float32)) | p2
    res = system()
    assert torch.allclose(res["probes"][p1].electric, torch.tensor(u0, device="cuda"))
    ang = torch.angle(res["probes"][p2].electric)
    assert torch.allclose(ang, torch.full_like(ang, np.pi / 2), atol=1e-6)


# ---------------------------------------------------------------------------
# Forward, metric and adjoint in one call (shared metric + seed pass)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("kind,d,with_out,last_mod", [("AS", 1, False, False), ("AS", -1, True, False),
                                                     ("RS", 1, True, False), ("AS", 1, False, True)])
def test_withgradient_sid_shared_pass(fo, orc, kind, d, with_out, last_mod):
    """fo_chain_withgradient_sid: the chain's last forward row pass and the adjoint's
    first row pass run as one pass (or, with a modulator in the last slot, as the two
    separate sweeps).  Losses, output field and every gradient equal the separate
    fo_chain_forward_sid + fo_chain_backward_ex calls bit for bit, and the oracle."""
    rng = np.random.default_rng(41 if kind == "AS" else 42)
    n = 256 if kind == "AS" else 200
    lams = [0.64, 0.538, 0.455]
    u0 = rand_field(rng, (2, 3, n, n))  # Julia (n, n, 3, 2): 3 target slices of 2 fields
    target = f32(rng.uniform(0, 2, (3, n, n)))
    phis = [f32(rng.uniform(0, 6, (n, n))) for _ in range(3)]
    m_last = c64(rng.uniform(0.5, 1.0, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))

    def build():
        u = fo.ScalarField(u0, (0.5, 0.5) if kind == "AS" else (1.0, 1.0), lams)
        P = (lambda zz: fo.ASProp(u, zz)) if kind == "AS" else (lambda zz: fo.RSProp(u, zz))
        ph = [fo.Phase(u, p, trainable=True, buffered=True) for p in phis]
        comps = [ph[0], P(300.0), ph[1], P(200.0), ph[2], P(250.0)]
        mk = None
        if last_mod:
            mk = fo.Mask(u, m_last, trainable=True, buffered=True)
            comps.append(mk)
        system = fo.OpticalSystem(fo.ScalarSource(u), comps, direction=d)
        return u, system, ph, mk

    # separate sweeps
    u, system, ph, mk = build()
    metric = fo.SquaredIntensityDifference((u, target))
    src = system.source.u0
    x, du = src.similar(), src.similar()
    tape = []
    system.forward(x, tape, src=src, metric=metric)
    grads = system.backward(du, tape, seed=(metric, x), input_grad=True)
    torch.cuda.synchronize()
    ref_loss = metric.loss.clone()
    ref_out = x.electric.clone()
    ref_du = du.electric.clone()
    ref_g = {i: grads[p]["phi"].clone() for i, p in enumerate(ph)}
    ref_gm = grads[mk]["m"].clone() if mk is not None else None

    # one call
    u2, system2, ph2, mk2 = build()
    metric2 = fo.SquaredIntensityDifference((u2, target))
    src2 = system2.source.u0
    x2, du2 = src2.similar(), src2.similar()
    x2.electric.zero_()
    segs = system2.segments(src2)
    n_ch = len(segs)
    if last_mod:
        assert segs[0].mods[-1] is not None
    g2 = system2.forward_backward_sid(du2, src2, metric2, u_out=x2 if with_out else None, input_grad=True)
    assert g2 is not None and n_ch == 1
    torch.cuda.synchronize()
    assert torch.equal(metric2.loss, ref_loss)
    assert torch.equal(du2.electric, ref_du)
    for i, p in enumerate(ph2):
        assert torch.equal(g2[p]["phi"], ref_g[i]), i
    if mk2 is not None:
        assert torch.equal(g2[mk2]["m"], ref_gm)
    if with_out:
        assert torch.equal(x2.electric, ref_out)
    else:
        assert not torch.any(x2.electric != 0)  # the output field is not written

    # and the oracle, for the phase of the first slot
    prop = (lambda v, zz, dd: orc.asprop(v, 0.5, 0.5, np.tile(lams, 2), zz, dd)) if kind == "AS" else \
        (lambda v, zz, dd: orc.rsprop(v, 1.0, 1.0, np.tile(lams, 2), zz, dd))
    U = u0.reshape(6, n, n)
    a0 = U
    a1 = prop(orc.phase_forward(a0, phis[0], d), 300.0, d)
    a2 = prop(orc.phase_forward(a1, phis[1], d), 200.0, d)
    out = prop(orc.phase_forward(a2, phis[2], d), 250.0, d)
    if last_mod:
        a3 = out
        out = orc.mask_forward(a3, m_last, d)
    tidx = np.arange(6) % 3
    c_ref, _ = orc.sid_value(out, target, tidx)
    assert np.max(np.abs(npy(metric2.loss) - c_ref) / c_ref) < 1e-4
    dv = orc.sid_backward(out, target, 1.0, tidx)
    if last_mod:
        dv, _ = orc.mask_backward(dv, m_last, a3, d)
    dv = prop(dv, 250.0, -d)
    dv, _ = orc.phase_backward(dv, phis[2], a2, d)
    dv = prop(dv, 200.0, -d)
    dv, _ = orc.phase_backward(dv, phis[1], a1, d)
    dv = prop(dv, 300.0, -d)
    dv, g0 = orc.phase_backward(dv, phis[0], a0, d)
    assert orc.rel_l2(npy(g2[ph2[0]]["phi"]), g0) < GRAD_TOL
    assert orc.rel_l2(npy(du2.electric).reshape(6, n, n), dv) < 1e-4


@pytest.mark.parametrize("kind,n,d,with_out,weighted,last_mod", [
    ("AS", 256, 1, False, False, False), ("AS", 256, -1, True, True, False), ("RS", 200, 1, True, True, False),
    ("AS", 256, 1, True, False, True), ("AS", 32, 1, True, True, False), ("AS", 2048, -1, False, True, False)])
def test_withgradient_sfd_shared_pass(fo, orc, kind, n, d, with_out, weighted, last_mod):
    """fo_chain_withgradient_sfd: the chain's last forward row pass, SquaredFieldDifference,
    its pull-back and the adjoint's first row pass as one pass (or, with a modulator in
    the last slot, as the separate calls).  Gradients and the output field equal the
    separate forward + fo_sfd_forward + fo_sfd_backward + backward calls bit for bit;
    the values c differ only in the order of the sums; both match the oracle."""
    rng = np.random.default_rng(51 if kind == "AS" else 52)
    lams = [0.64, 0.538, 0.455, 0.64]
    B = len(lams)
    ds = (0.5, 0.5) if kind == "AS" else (1.0, 1.0)
    u0 = rand_field(rng, (B, n, n))
    v0 = rand_field(rng, (B, n, n))
    phis = [f32(rng.uniform(0, 6, (n, n))) for _ in range(2)]
    m_last = c64(rng.uniform(0.5, 1.0, (n, n)) * np.exp(1j * rng.uniform(0, 6, (n, n))))
    w = f32(rng.uniform(0.5, 2.0, B)) if weighted else None

    def build():
        u = fo.ScalarField(u0, ds, lams)
        P = (lambda zz: fo.ASProp(u, zz)) if kind == "AS" else (lambda zz: fo.RSProp(u, zz))
        ph = [fo.Phase(u, p, trainable=True, buffered=True) for p in phis]
        comps = [ph[0], P(300.0), ph[1], P(200.0)]
        mk = None
        if last_mod:
            mk = fo.Mask(u, m_last, trainable=True, buffered=True)
            comps.append(mk)
        system = fo.OpticalSystem(fo.ScalarSource(u), comps, direction=d)
        return u, system, ph, mk

    dc = torch.tensor(w, dtype=torch.float32, device="cuda") if weighted else None
    # separate calls
    u, system, ph, mk = build()
    metric = fo.SquaredFieldDifference(fo.ScalarField(v0, ds, lams))
    src = system.source.u0
    x, du = src.similar(), src.similar()
    tape = []
    system.forward(x, tape, src=src)
    c_sep = metric(x).clone()
    metric.backpropagate_into(x, du, dc)
    grads = system.backward(du, tape, input_grad=True)
    torch.cuda.synchronize()
    ref_out, ref_du = x.electric.clone(), du.electric.clone()
    ref_g = [grads[p]["phi"].clone() for p in ph]
    ref_gm = grads[mk]["m"].clone() if mk is not None else None

    # one call
    u2, system2, ph2, mk2 = build()
    metric2 = fo.SquaredFieldDifference(fo.ScalarField(v0, ds, lams))
    src2 = system2.source.u0
    x2, du2 = src2.similar(), src2.similar()
    x2.electric.zero_()
    g2 = system2.forward_backward_sfd(du2, src2, metric2, dc=dc, u_out=x2 if with_out else None, input_grad=True)
    assert g2 is not None
    torch.cuda.synchronize()
    c2 = metric2.out.clone()
    assert torch.max(torch.abs(c2 - c_sep) / c_sep).item() < 1e-5
    assert torch.equal(du2.electric, ref_du)
    for i, p in enumerate(ph2):
        assert torch.equal(g2[p]["phi"], ref_g[i]), i
    if mk2 is not None:
        assert torch.equal(g2[mk2]["m"], ref_gm)
    if with_out:
        assert torch.equal(x2.electric, ref_out)
    elif not last_mod:
        assert not torch.any(x2.electric != 0)  # the output field is not written
    # the fused values are fixed-order too
    system2.forward_backward_sfd(du2, src2, metric2, dc=dc, input_grad=True)
    assert torch.equal(metric2.out, c2)

    # withgradient dispatches to the fused call and returns sum(dc * c); dc of another
    # dtype is converted
    loss, g3 = fo.withgradient(metric2, system2, dc=None if dc is None else dc.double())
    wsum = (c2 if dc is None else dc * c2).sum()
    assert torch.equal(loss, wsum)
    assert torch.equal(g3[ph2[0]]["phi"], ref_g[0])

    # the oracle
    prop = (lambda a, zz, dd: orc.asprop(a, ds[0], ds[1], lams, zz, dd)) if kind == "AS" else \
        (lambda a, zz, dd: orc.rsprop(a, ds[0], ds[1], lams, zz, dd))
    a0 = u0
    a1 = prop(orc.phase_forward(a0, phis[0], d), 300.0, d)
    out = prop(orc.phase_forward(a1, phis[1], d), 200.0, d)
    a2 = out
    if last_mod:
        out = orc.mask_forward(a2, m_last, d)
    c_ref = orc.sfd_value(out, v0)
    assert np.max(np.abs(npy(c2) - c_ref) / c_ref) < 1e-4
    dv = orc.sfd_backward(out, v0, 1.0 if w is None else w)
    if last_mod:
        dv, _ = orc.mask_backward(dv, m_last, a2, d)
    dv = prop(dv, 200.0, -d)
    dv, _ = orc.phase_backward(dv, phis[1], a1, d)
    dv = prop(dv, 300.0, -d)
    dv, g0 = orc.phase_backward(dv, phis[0], a0, d)
    assert orc.rel_l2(npy(g2[ph2[0]]["phi"]), g0) < GRAD_TOL
    assert orc.rel_l2(npy(du2.electric), dv) < 1e-4


def test_component_accessors(fo, orc):
    """trainable / istrainable / isbuffered / get_data / get_source / get_components and
    the out-of-place backpropagate (OpticalComponents.jl:277-340)."""
    rng = np.random.default_rng(61)
    n = 64
    u0 = rand_field(rng, (2, n, n))
    u = fo.ScalarField(u0, (1.0, 1.0), [0.64, 0.455])
    phi = f32(rng.uniform(0, 6, (n, n)))
    ph = fo.Phase(u, phi, trainable=True, buffered=True)
    mk = fo.Mask(u, c64(np.ones((n, n))))
    p = fo.ASProp(u, 300.0)
    src = fo.ScalarSource(u)
    system = src | ph | p | mk
    assert fo.istrainable(ph) and fo.isbuffered(ph) and not fo.istrainable(mk) and not fo.isbuffered(p)
    assert set(fo.trainable(ph)) == {"phi"} and fo.trainable(mk) == {}
    tr = fo.trainable(system)
    assert list(tr) == [ph] and tr[ph]["phi"] is fo.get_data(ph)
    assert fo.get_source(system) is src and fo.get_components(system) == [ph, p, mk]
    assert np.allclose(npy(fo.get_data(ph)), phi)
    # out-of-place adjoint leaves its input alone and equals the in-place one
    dv = fo.ScalarField(rand_field(rng, (2, n, n)), (1.0, 1.0), [0.64, 0.455])
    keep = dv.electric.clone()
    out = fo.backpropagate(dv, p)
    assert torch.equal(dv.electric, keep)
    fo.backpropagate_(dv, p)
    assert torch.equal(out.electric, dv.electric)
    ref = orc.asprop(npy(keep), 1.0, 1.0, [0.64, 0.455], 300.0, orc.BACKWARD)
    assert orc.rel_l2(npy(out.electric), ref) < FIELD_TOL


# ---------------------------------------------------------------------------
# PadCropOperator, pad, crop
# ---------------------------------------------------------------------------

def test_pad_crop_reference_case(fo, orc):
    """The reference's pad / crop test (test/optical_components_test.jl:171-189), and
    offsets, a fill value and a batch against the oracle (bit-exact: copies)."""
    u = fo.ScalarField(np.ones((32, 32), np.complex64), (1.0, 1.0), 1.064)
    up = fo.pad(u, (64, 64))
    assert (up.nx, up.ny) == (64, 64)
    uc = fo.crop(up, (32, 32))
    assert (uc.nx, uc.ny) == (32, 32) and torch.equal(uc.electric, u.electric)
    assert complex(up.electric[16, 16]) == 1.0
    rng = np.random.default_rng(71)
    a = rand_field(rng, (2, 3, 20, 24)).astype(np.complex64)
    t = torch.tensor(a, device="cuda")
    p = fo.pad(t, (40, 33), offset=(5, 9), pad_val=0.5 - 0.25j)
    assert np.array_equal(p.cpu().numpy(), orc.pad(a, (40, 33), (5, 9), 0.5 - 0.25j).astype(np.complex64))
    c = fo.crop(p, (24, 20), offset=(5, 9))
    assert torch.equal(c, t)
    c2 = fo.crop(p, (7, 4), offset=(30, 20))
    assert np.array_equal(c2.cpu().numpy(), orc.crop(p.cpu().numpy(), (7, 4), (30, 20)))
    with pytest.raises(fo.FluxOpticsError):
        fo.crop(p, (24, 20), offset=(20, 9))  # does not fit


@pytest.mark.parametrize("offset", [(0, 0), (32, 16)])
def test_padcrop_operator_in_a_system(fo, orc, offset):
    """ScalarSource | Phase | pad | ASProp | Phase (padded grid) | ASProp | crop, with
    SquaredIntensityDifference: output, loss and both phase gradients against the oracle
    (the reference's docstring pattern, pad_crop_operators.jl:276-287)."""
    rng = np.random.default_rng(72)
    n, npad, B = 64, 128, 2
    ds, lams = (1.0, 1.0), np.array([1.064, 0.8])
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(9.0, x, y)] * B) * (1 + 0.1 * rng.standard_normal((B, n, n))))
    phi1 = f32(rng.uniform(0, 6, (n, n)))
    phi2 = f32(rng.uniform(0, 6, (npad, npad)))
    target = f32(np.abs(orc.gaussian(12.0, x - 5, y)) ** 2)
    u = fo.ScalarField(u0, ds, lams)
    up = u.set_field_data(torch.zeros((B, npad, npad), dtype=torch.complex64, device="cuda"))
    pad_op = fo.PadCropOperator(u, up.electric, offset=offset)
    ph1 = fo.Phase(u, phi1, trainable=True)
    ph2 = fo.Phase(up, phi2, trainable=True)
    system = fo.ScalarSource(u) | ph1 | pad_op | fo.ASProp(up, 400.0) | ph2 | fo.ASProp(up, 300.0) | fo.adjoint(pad_op)
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    out = system()["out"]
    assert (out.nx, out.ny) == (n, n)

    a1 = orc.phase_forward(u0, phi1)
    b0 = orc.pad(a1, (npad, npad), offset)
    b1 = orc.asprop(b0, ds[0], ds[1], lams, 400.0)
    b2 = orc.asprop(orc.phase_forward(b1, phi2), ds[0], ds[1], lams, 300.0)
    ref = orc.crop(b2, (n, n), offset)
    assert orc.rel_l2(npy(out.electric), ref) < FIELD_TOL
    c_ref, _ = orc.sid_value(ref, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.pad(orc.sid_backward(ref, target), (npad, npad), offset)
    dv = orc.asprop(dv, ds[0], ds[1], lams, 300.0, orc.BACKWARD)
    dv, g2 = orc.phase_backward(dv, phi2, b1)
    dv = orc.asprop(dv, ds[0], ds[1], lams, 400.0, orc.BACKWARD)
    dv = orc.crop(dv, (n, n), offset)
    _, g1 = orc.phase_backward(dv, phi1, u0)
    assert orc.rel_l2(npy(grads[ph2]["phi"]), g2) < GRAD_TOL
    assert orc.rel_l2(npy(grads[ph1]["phi"]), g1) < GRAD_TOL
    # the padded span's result does not depend on where the field sits in the padded grid
    # for a translation-invariant propagator: compare with the centred placement
    if offset == (0, 0):
        pc = fo.PadCropOperator(u, (npad, npad), offset=(32, 32))
        sys_c = fo.ScalarSource(u) | ph1 | pc | fo.ASProp(up, 400.0) | fo.adjoint(pc)
        sys_0 = fo.ScalarSource(u) | ph1 | pad_op | fo.ASProp(up, 400.0) | fo.adjoint(pad_op)
        assert orc.rel_l2(npy(sys_c()["out"].electric), npy(sys_0()["out"].electric)) < FIELD_TOL


def test_padcrop_operator_backward_direction_and_errors(fo, orc):
    rng = np.random.default_rng(73)
    n, npad = 48, 64
    ds, lam = (1.0, 1.0), 0.9
    u0 = rand_field(rng, (n, n))
    u = fo.ScalarField(u0, ds, lam)
    up = fo.ScalarField(np.zeros((npad, npad), np.complex64), ds, lam)
    op = fo.PadCropOperator(u, up, offset=(3, 7), pad_val=0.0)
    # Backward: the adjoint operator pads, the operator crops
    system = fo.OpticalSystem(fo.ScalarSource(u), [fo.adjoint(op), fo.ASProp(up, 250.0), op], direction=fo.Backward)
    out = npy(system()["out"].electric)
    ref = orc.crop(orc.asprop(orc.pad(u0, (npad, npad), (3, 7)), 1.0, 1.0, lam, 250.0, orc.BACKWARD), (n, n), (3, 7))
    assert orc.rel_l2(out, ref) < FIELD_TOL
    # standalone propagate / backpropagate change the grid
    v = fo.propagate(u, op)
    assert (v.nx, v.ny) == (npad, npad)
    assert torch.equal(fo.backpropagate(v, op).electric, u.electric)
    with pytest.raises(TypeError):
        op.propagate_(u)
    with pytest.raises(ValueError):
        (fo.ScalarSource(u) | op | fo.ASProp(up, 100.0))()  # no cropping partner
    with pytest.raises(ValueError):
        (fo.ScalarSource(up) | fo.adjoint(op) | fo.ASProp(up, 100.0))()  # crops before any pad
    with pytest.raises(ValueError):
        fo.PadCropOperator(u, (40, 64))  # does not fit


def test_field_helpers(fo, orc):
    """ScalarField accessors, offset_tilts_, arithmetic, phase and dot (src/Fields.jl)."""
    rng = np.random.default_rng(81)
    n = 32
    u0 = rand_field(rng, (2, 3, n, n))  # Julia (n, n, 3, 2)
    lams = np.array([0.64, 0.538, 0.455])
    u = fo.ScalarField(u0, (0.5, 0.25), lams)
    assert fo.get_lambdas(u) is lams
    assert np.array_equal(fo.get_lambdas_collection(u), np.tile(lams, 2))
    assert fo.is_on_axis(u) and fo.get_tilts(u) == (0.0, 0.0)
    ut = fo.set_field_tilts(u, (0.01, np.array([0.0, -0.02, 0.03])))
    assert not fo.is_on_axis(ut) and ut.electric is u.electric
    tc = fo.get_tilts_collection(ut)
    assert np.allclose(tc[:, 0], 0.01) and np.allclose(tc[:, 1], np.tile([0.0, -0.02, 0.03], 2))
    sel = fo.select_lambdas(u)
    assert sel(False) is lams and np.array_equal(sel(True), np.tile(lams, 2))
    sx, sy = fo.select_tilts(ut)
    assert sx(False) == 0.01 and np.allclose(sy(True), np.tile([0.0, -0.02, 0.03], 2))
    fo.set_field_ds_(ut, (1.0, 2.0))
    assert ut.ds == (1.0, 2.0) and u.ds == (0.5, 0.25)
    # offset_tilts_: the carrier moves into the envelope, and back
    v = u.copy()
    fo.offset_tilts_(v, (0.01, -0.02))
    x = (np.arange(n) - (n - 1) / 2) * 0.5
    y = (np.arange(n) - (n - 1) / 2) * 0.25
    k = 2 * np.pi / np.tile(lams, 2)
    ref = u0.reshape(6, n, n) * np.exp(-1j * k[:, None, None] * (np.sin(0.01) * x[None, None, :]
                                                                  + np.sin(-0.02) * y[None, :, None]))
    assert orc.rel_l2(npy(v.electric).reshape(6, n, n), ref) < 1e-6
    assert np.allclose(v.tilts_per_field(), [[0.01, -0.02]] * 6)
    fo.offset_tilts_(v, (0.0, 0.0))
    assert orc.rel_l2(npy(v.electric), u0) < 1e-6 and fo.is_on_axis(v)
    # construction from a Julia size, ndims, copyto_
    z = fo.ScalarField((24, 16, 3), (1.0, 1.0), lams)
    assert z.size() == (24, 16, 3) and tuple(z.electric.shape) == (3, 16, 24) and not torch.any(z.electric != 0)
    assert z.ndims() == 3 and z.ndims(True) == 2
    z2 = fo.ScalarField((24, 16, 3), (1.0, 1.0), lams).fill_(2.0)
    assert torch.equal(z.copyto_(z2).electric, z2.electric)
    # arithmetic, conj, fill_
    w = fo.ScalarField(rand_field(rng, (2, 3, n, n)), (0.5, 0.25), lams)
    assert torch.equal((u + w).electric, u.electric + w.electric)
    assert torch.equal((u - w).electric, u.electric - w.electric)
    assert torch.equal((-u).electric, -u.electric)
    assert torch.equal((2.0 * u).electric, (u * 2.0).electric)
    assert torch.equal((u / 4.0).electric, u.electric / 4.0)
    assert np.array_equal(npy(u.conj().electric), np.conj(npy(u.electric)))
    f = u.copy().fill_(1.5 - 0.5j)
    assert torch.all(f.electric == complex(1.5, -0.5))
    # phase and dot (no dx dy factor)
    assert np.allclose(npy(fo.phase(u)), np.angle(npy(u.electric)), atol=1e-6)
    d = npy(fo.dot(u, w))
    ref = np.sum(np.conj(npy(u.electric)) * npy(w.electric), axis=(-2, -1)).reshape(-1)
    assert np.max(np.abs(d - ref) / np.abs(ref)) < 1e-5


def test_metric_free_functions(fo, orc):
    """compute_metric / backpropagate_metric (metrics/Metrics.jl) equal the callable
    form and the pull-back, for SquaredFieldDifference and DotProduct."""
    rng = np.random.default_rng(82)
    u0, v0 = rand_field(rng, (3, 32, 32)), rand_field(rng, (3, 32, 32))
    u = fo.ScalarField(u0, (1.0, 1.0), 0.64)
    v = fo.ScalarField(v0, (1.0, 1.0), 0.64)
    m = fo.SquaredFieldDifference(v)
    assert np.allclose(npy(fo.compute_metric(m, u)), orc.sfd_value(u0, v0), rtol=1e-5)
    w = torch.tensor([1.0, 2.0, 0.5], device="cuda")
    du = fo.backpropagate_metric(m, u, w)
    assert orc.rel_l2(npy(du.electric), orc.sfd_backward(u0, v0, [1.0, 2.0, 0.5])) < 1e-6
    d = fo.DotProduct(v)
    assert torch.equal(fo.compute_metric(d, u).clone(), d(u).clone())


def test_user_component_protocol(fo, orc):
    """A component written by a user against the component protocol (the reference's
    AbstractCustomComponent, OpticalComponents.jl:751-816) runs inside a system between
    fused chains, trainable and static: output, loss and both gradients against the
    oracle."""

    class Amplitude(fo.Component):
        def __init__(self, a, trainable=False):
            self.a = torch.tensor(a, dtype=torch.float32, device="cuda")
            self.trainable = trainable

        def params(self):
            return {"a": self.a} if self.trainable else {}

        def propagate_(self, u, direction=fo.Forward):
            u.electric.mul_(self.a)
            return u

        def backpropagate_(self, dv, direction=fo.Forward):
            dv.electric.mul_(self.a)
            return dv

        def get_saved_buffer(self, u):
            return torch.empty_like(u.electric)

        def propagate_and_save_(self, u, saved, direction=fo.Forward):
            saved.copy_(u.electric)
            return self.propagate_(u, direction)

        def get_gradient_buffer(self):
            return torch.empty_like(self.a)

        def backpropagate_with_gradient_(self, dv, saved, grad, direction=fo.Forward):
            grad.copy_((dv.electric.conj() * saved).real.reshape(-1, *self.a.shape).sum(0))
            return self.backpropagate_(dv, direction), {"a": grad}

    rng = np.random.default_rng(83)
    n, lams, ds = 64, np.array([0.64, 0.455]), (1.0, 1.0)
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(8.0, x, y)] * 2) * (1 + 0.1 * rng.standard_normal((2, n, n))))
    phi = f32(rng.uniform(0, 6, (n, n)))
    a = f32(rng.uniform(0.5, 1.5, (n, n)))
    target = f32(np.abs(orc.gaussian(10.0, x, y)) ** 2)
    u = fo.ScalarField(u0, ds, lams)
    for trainable in (True, False):
        ph = fo.Phase(u, phi, trainable=True)
        amp = Amplitude(a, trainable)
        system = fo.ScalarSource(u) | ph | fo.ASProp(u, 300.0) | amp | fo.ASProp(u, 200.0)
        metric = fo.SquaredIntensityDifference((u, target))
        loss, grads = fo.withgradient(metric, system)
        a1 = orc.asprop(orc.phase_forward(u0, phi), 1.0, 1.0, lams, 300.0)
        out = orc.asprop(a1 * a, 1.0, 1.0, lams, 200.0)
        assert orc.rel_l2(npy(system()["out"].electric), out) < FIELD_TOL
        c_ref, _ = orc.sid_value(out, target)
        assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
        dv = orc.asprop(orc.sid_backward(out, target), 1.0, 1.0, lams, 200.0, orc.BACKWARD)
        ga = np.sum(np.real(np.conj(dv) * a1), axis=0)
        dv = orc.asprop(dv * a, 1.0, 1.0, lams, 300.0, orc.BACKWARD)
        _, gphi = orc.phase_backward(dv, phi, u0)
        assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL
        if trainable:
            assert orc.rel_l2(npy(grads[amp]["a"]), ga) < GRAD_TOL
            assert list(fo.trainable(system)) == [ph, amp]
        else:
            assert amp not in grads


def test_tilt_anchor(fo, orc):
    """TiltAnchor (utilities/tilt_anchor.jl): a field on axis anchored to tilted
    coordinates, propagated with the tilted kernel through a trainable phase, and anchored
    back: output and phase gradient against the oracle, whose adjoint restores the entry
    tilts at each anchor."""
    rng = np.random.default_rng(84)
    n, lams, ds, th = 64, np.array([0.64, 0.455]), (1.0, 1.0), (0.02, -0.01)
    x, y = orc.spatial_vectors((n, n), ds)
    u0 = c64(np.stack([orc.gaussian(8.0, x, y)] * 2) * (1 + 0.1 * rng.standard_normal((2, n, n))))
    phi = f32(rng.uniform(0, 6, (n, n)))
    target = f32(np.abs(orc.gaussian(10.0, x, y)) ** 2)
    u = fo.ScalarField(u0, ds, lams)
    ut = fo.set_field_tilts(u, th)
    ph = fo.Phase(ut, phi, trainable=True)
    system = fo.ScalarSource(u) | fo.TiltAnchor(ut) | fo.ASProp(ut, 300.0) | ph | fo.ASProp(ut, 200.0) | fo.TiltAnchor(u)
    res = system()["out"]
    assert res.is_on_axis()
    k = 2 * np.pi / lams
    carrier = np.exp(1j * k[:, None, None] * (np.sin(th[0]) * x[None, None, :] + np.sin(th[1]) * y[None, :, None]))
    a0 = u0 / carrier
    a1 = orc.asprop(a0, 1.0, 1.0, lams, 300.0, tilts=th)
    a2 = orc.asprop(orc.phase_forward(a1, phi), 1.0, 1.0, lams, 200.0, tilts=th)
    out = a2 * carrier
    assert orc.rel_l2(npy(res.electric), out) < FIELD_TOL
    metric = fo.SquaredIntensityDifference((u, target))
    loss, grads = fo.withgradient(metric, system)
    c_ref, _ = orc.sid_value(out, target)
    assert abs(float(loss) - c_ref.sum()) / c_ref.sum() < 1e-4
    dv = orc.sid_backward(out, target) / carrier  # adjoint of the last anchor
    dv = orc.asprop(dv, 1.0, 1.0, lams, 200.0, orc.BACKWARD, tilts=th)
    _, gphi = orc.phase_backward(dv, phi, a1)
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL


def test_padded_span_with_rsprop_mask_and_sfd(fo, orc):
    """A padded span holding an RSProp (which pads again inside its own passes), a
    trainable Mask on the padded grid and an ASProp, with SquaredFieldDifference and
    per-field weights: values, input-side phase gradient and mask gradient against the
    oracle."""
    rng = np.random.default_rng(85)
    n, npad, lams, ds = 40, 64, np.array([1.064, 0.8]), (1.0, 1.0)
    u0 = rand_field(rng, (2, n, n))
    v0 = rand_field(rng, (2, n, n))
    phi = f32(rng.uniform(0, 6, (n, n)))
    m = c64(rng.uniform(0.5, 1.0, (npad, npad)) * np.exp(1j * rng.uniform(0, 6, (npad, npad))))
    w = np.array([0.5, 2.0])
    u = fo.ScalarField(u0, ds, lams)
    up = fo.ScalarField(np.zeros((2, npad, npad), np.complex64), ds, lams)
    op = fo.PadCropOperator(u, up, offset=(10, 6))
    ph = fo.Phase(u, phi, trainable=True)
    mk = fo.Mask(up, m, trainable=True)
    system = fo.ScalarSource(u) | ph | op | fo.RSProp(up, 150.0) | mk | fo.ASProp(up, 120.0) | fo.adjoint(op)
    metric = fo.SquaredFieldDifference(fo.ScalarField(v0, ds, lams))
    loss, grads = fo.withgradient(metric, system, dc=torch.tensor(w, device="cuda"))
    a1 = orc.phase_forward(u0, phi)
    b0 = orc.pad(a1, (npad, npad), (10, 6))
    b1 = orc.rsprop(b0, 1.0, 1.0, lams, 150.0)
    b2 = orc.asprop(orc.mask_forward(b1, m), 1.0, 1.0, lams, 120.0)
    out = orc.crop(b2, (n, n), (10, 6))
    c_ref = orc.sfd_value(out, v0)
    assert abs(float(loss) - np.sum(w * c_ref)) / np.sum(w * c_ref) < 1e-4
    dv = orc.pad(orc.sfd_backward(out, v0, w), (npad, npad), (10, 6))
    dv = orc.asprop(dv, 1.0, 1.0, lams, 120.0, orc.BACKWARD)
    dv, gm = orc.mask_backward(dv, m, b1)
    dv = orc.rsprop(dv, 1.0, 1.0, lams, 150.0, orc.BACKWARD)
    dv = orc.crop(dv, (n, n), (10, 6))
    _, gphi = orc.phase_backward(dv, phi, u0)
    assert orc.rel_l2(npy(grads[mk]["m"]), gm) < GRAD_TOL
    assert orc.rel_l2(npy(grads[ph]["phi"]), gphi) < GRAD_TOL


@pytest.mark.parametrize("track", [False, True])
def test_tilted_propagation_identities(fo, orc, track):
    """The GPU's tilted ASProp against its own on-axis ASProp through the physical
    identities of the tilted kernels: an envelope on a carrier of whole frequency bins
    propagates as the physical field (without track_tilts), or as the physical field
    followed along its walk-off z sin(theta) (with track_tilts)."""
    N, d, lam = 64, 1.0, 1.0
    x = (np.arange(N) - (N - 1) / 2) * d
    u = orc.gaussian(6.0, x, x) * np.exp(1j * 0.02 * (x[None, :] ** 2 - 0.5 * x[:, None] ** 2))
    f0 = np.array([3 / (N * d), -2 / (N * d)])
    th = tuple(np.arcsin(f0 * lam))
    carrier = np.exp(2j * np.pi * (f0[0] * x[None, :] + f0[1] * x[:, None]))
    z = 64.0 if track else 40.0
    uf = fo.ScalarField(u.astype(np.complex64), (d, d), lam)
    ef = fo.ScalarField((u / carrier).astype(np.complex64), (d, d), lam, tilts=th)
    out_u = npy(fo.propagate(uf, fo.ASProp(uf, z)).electric)
    out_e = npy(fo.propagate(ef, fo.ASProp(ef, z, track_tilts=track)).electric)
    if track:
        ref = np.roll(out_u, shift=(2, -3), axis=(0, 1))
        got = out_e * carrier * np.exp(2j * np.pi * (f0[0] * 3 + f0[1] * -2))
    else:
        ref, got = out_u, out_e * carrier
    assert orc.rel_l2(got, ref) < FIELD_TOL


def test_rsprop_equals_padded_asprop_on_band_limited_fields(fo, orc):
    """The GPU's RSProp against its own ASProp run inside a PadCropOperator span on a
    window of twice the size: the RS impulse response is the inverse transform of the AS
    transfer function, so for a band-limited field the two agree (the oracle's
    restatements agree to 1e-13)."""
    n, lam, z = 256, 0.8, 600.0  # the padded window (512) must be a power of two for ASProp
    x = (np.arange(n) - (n - 1) / 2)
    lams = [lam, 1.064]
    u0 = np.stack([orc.gaussian(10.0, x, x), orc.gaussian(14.0, x - 5, x + 3)]).astype(np.complex64)
    u = fo.ScalarField(u0, (1.0, 1.0), lams)
    up = fo.ScalarField(np.zeros((2, 2 * n, 2 * n), np.complex64), (1.0, 1.0), lams)
    op = fo.PadCropOperator(u, up, offset=(n // 2, n // 2))
    rs = npy(fo.propagate(u, fo.RSProp(u, z)).electric)
    as_ = npy((fo.ScalarSource(u) | op | fo.ASProp(up, z) | fo.adjoint(op))()["out"].electric)
    assert orc.rel_l2(rs, as_) < FIELD_TOL
