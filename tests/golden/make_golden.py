"""Generates the golden fixtures of tests/golden/ from the FP64 oracle.

    python tests/golden/make_golden.py

Small seeded cases of every hot-path operation; tests/test_golden.py checks that
the oracle still reproduces them (regression pin) and that the CUDA path matches
them within the parity tolerances.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import fluxoptics_oracle as orc  # noqa: E402


def c64(a):
    return np.asarray(a).astype(np.complex64).astype(np.complex128)


def f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def cases():
    rng = np.random.default_rng(2026)
    out = {}
    # ASProp, 64 x 64, two wavelengths, forward and backward
    x, y = orc.spatial_vectors((64, 64), (1.0, 1.0))
    u = c64(np.stack([orc.gaussian(8.0, x, y), orc.hermite_gaussian(6.0, 1, 2, x, y)]) *
            (1 + 0.1 * rng.standard_normal((2, 64, 64))))
    out["as_u"] = u
    out["as_fwd"] = orc.asprop(u, 1.0, 1.0, [1.064, 0.633], 450.0)
    out["as_bwd"] = orc.asprop(u, 1.0, 1.0, [1.064, 0.633], 450.0, orc.BACKWARD)
    # RSProp, 40 x 40 (reference padding 79 x 79)
    u = c64(orc.gaussian(5.0, *orc.spatial_vectors((40, 40), (1.0, 1.0))) * (1 + 0.1 * rng.standard_normal((40, 40))))
    out["rs_u"] = u
    out["rs_fwd"] = orc.rsprop(u, 1.0, 1.0, 1.064, 600.0)
    # Phase -> AS -> Phase -> AS with SID gradient, 32 x 32
    x, y = orc.spatial_vectors((32, 32), (1.0, 1.0))
    u0 = c64(orc.gaussian(6.0, x, y))
    p1 = f32(rng.uniform(0, 2 * np.pi, (32, 32)))
    p2 = f32(rng.uniform(0, 2 * np.pi, (32, 32)))
    t = f32(np.abs(orc.gaussian(5.0, x - 3, y)) ** 2)
    v1 = orc.asprop(orc.phase_forward(u0, p1), 1.0, 1.0, 1.064, 200.0)
    v2 = orc.asprop(orc.phase_forward(v1, p2), 1.0, 1.0, 1.064, 200.0)
    c, _ = orc.sid_value(v2, t)
    dv = orc.asprop(orc.sid_backward(v2, t), 1.0, 1.0, 1.064, 200.0, orc.BACKWARD)
    dv, g2 = orc.phase_backward(dv, p2, v1)
    dv = orc.asprop(dv, 1.0, 1.0, 1.064, 200.0, orc.BACKWARD)
    _, g1 = orc.phase_backward(dv, p1, u0)
    out.update(chain_u0=u0, chain_p1=p1, chain_p2=p2, chain_t=t, chain_out=v2, chain_loss=c, chain_g1=g1,
               chain_g2=g2)
    # AS_BPM 32 x 32 x 6 slices with the dn gradient
    u0 = c64(orc.gaussian(4.0, *orc.spatial_vectors((32, 32), (0.5, 0.5))))
    dn = f32(3e-3 * rng.standard_normal((6, 32, 32)))
    tb = f32(np.abs(orc.gaussian(3.0, *orc.spatial_vectors((32, 32), (0.5, 0.5)))) ** 2)
    vb, saves = orc.bpm_forward(u0, 0.5, 0.5, 1.064, 12.0, 1.45, dn, save=True)
    _, gdn = orc.bpm_backward(orc.sid_backward(vb, tb), 0.5, 0.5, 1.064, 12.0, 1.45, dn, saves)
    out.update(bpm_u0=u0, bpm_dn=dn, bpm_t=tb, bpm_out=vb, bpm_gdn=gdn)
    # TVProx 24 x 20
    y0 = f32(rng.standard_normal((20, 24)))
    out["tv_in"] = y0
    out["tv_out"] = orc.tv_prox(y0.copy(), 0.25, 30)
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "hotpath_small.npz"), **cases())
    print("wrote", os.path.join(HERE, "hotpath_small.npz"))
