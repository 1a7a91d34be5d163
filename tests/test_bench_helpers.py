"""Host-side helpers of bench.py (no GPU): the traffic accounting behind the
reported bandwidths and the whole-job rate."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_pass_traffic_of_the_headline_iteration():
    n2, B = 2048 * 2048, 48
    fld = 8 * n2 * B
    # 6 column passes, 3 forward row passes, the shared metric + seed pass, 3 adjoint
    # row passes, Fista on 3 masks
    col = 6 * (2 * fld + 3 * 8 * n2)
    fwd = (2 * fld + 4 * n2) + 2 * (3 * fld + 4 * n2)
    shared = 2 * fld + 6 * 4 * n2
    adj = 2 * (3 * fld + 8 * n2) + (2 * fld + 8 * n2)
    assert bench.pass_bytes_per_step() == col + fwd + shared + adj + 3 * 24 * n2
    assert abs(bench.pass_bytes_per_step() / 1e9 - 49.48) < 0.01
    assert bench.col_pass_bytes() == 16 * n2 * B + 3 * 8 * n2


def test_job_rate_and_single_rank_max():
    assert bench.job_rate(288, 2, 10.0) == 2 * 288 / 0.010
    assert bench.max_over_ranks(12.5) == 12.5


def test_small_inputs_are_seeded_and_normalised():
    f1, m1, t1 = bench.make_inputs(n=64)
    f2, m2, t2 = bench.make_inputs(n=64)
    assert f1.shape == (bench.N_MODES, len(bench.LAMBDAS), 64, 64) and f1.dtype == np.complex64
    assert np.array_equal(f1, f2) and all(np.array_equal(a, b) for a, b in zip(m1, m2))
    # each target slice integrates to the number of modes (dx dy = 0.25)
    assert np.allclose(t1.sum(axis=(1, 2)) * bench.DS[0] * bench.DS[1], bench.N_MODES, rtol=1e-5)
