"""Golden fixtures (tests/golden/hotpath_small.npz, made by make_golden.py).

CPU: the oracle still reproduces the fixtures (regression pin of the oracle).
GPU: the CUDA path matches them (fields 1e-5, gradients 1e-4 relative L2)."""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "hotpath_small.npz")))


def test_oracle_reproduces_fixtures(gold):
    import make_golden
    fresh = make_golden.cases()
    for k, v in gold.items():
        assert np.allclose(fresh[k], v, rtol=1e-12, atol=1e-14), k


@pytest.mark.gpu
def test_cuda_path_matches_fixtures(fo, orc, gold):
    g = gold
    u = fo.ScalarField(g["as_u"], (1.0, 1.0), [1.064, 0.633])
    p = fo.ASProp(u, 450.0)
    assert orc.rel_l2(p.propagate(u).electric.cpu().numpy(), g["as_fwd"]) < 1e-5
    assert orc.rel_l2(p.propagate(u, fo.Backward).electric.cpu().numpy(), g["as_bwd"]) < 1e-5
    u = fo.ScalarField(g["rs_u"], (1.0, 1.0), 1.064)
    assert orc.rel_l2(fo.RSProp(u, 600.0).propagate(u).electric.cpu().numpy(), g["rs_fwd"]) < 1e-5

    u = fo.ScalarField(g["chain_u0"], (1.0, 1.0), 1.064)
    ph1 = fo.Phase(u, g["chain_p1"], trainable=True)
    ph2 = fo.Phase(u, g["chain_p2"], trainable=True)
    prop = fo.ASProp(u, 200.0)
    system = fo.ScalarSource(u) | ph1 | prop | ph2 | prop
    loss, grads = fo.withgradient(fo.SquaredIntensityDifference((u, g["chain_t"])), system)
    assert orc.rel_l2(system()["out"].electric.cpu().numpy(), g["chain_out"]) < 1e-5
    assert abs(float(loss) - g["chain_loss"].sum()) / g["chain_loss"].sum() < 1e-4
    assert orc.rel_l2(grads[ph1]["phi"].cpu().numpy(), g["chain_g1"]) < 1e-4
    assert orc.rel_l2(grads[ph2]["phi"].cpu().numpy(), g["chain_g2"]) < 1e-4

    u = fo.ScalarField(g["bpm_u0"], (0.5, 0.5), 1.064)
    bpm = fo.AS_BPM(u, 12.0, 1.45, g["bpm_dn"], trainable=True)
    system = fo.ScalarSource(u) | bpm
    _, grads = fo.withgradient(fo.SquaredIntensityDifference((u, g["bpm_t"])), system)
    assert orc.rel_l2(system()["out"].electric.cpu().numpy(), g["bpm_out"]) < 1e-5
    assert orc.rel_l2(grads[bpm]["dn"].cpu().numpy(), g["bpm_gdn"]) < 1e-4

    import torch
    x = torch.tensor(g["tv_in"], dtype=torch.float32, device="cuda")
    tv = fo.TVProx(0.25, 30)
    tv.apply_(tv.init(x), x)
    assert orc.rel_l2(x.cpu().numpy(), g["tv_out"]) < 1e-5
