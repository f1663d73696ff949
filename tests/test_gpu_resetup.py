"""Re-setup of a preconditioner with a matrix of the same sparsity pattern.

sg_precond_setup keeps its host integer set-up when the pattern, partition
and options are unchanged and redoes only the device factorisation; the
result must be bit-identical to a fresh set-up on the new values, and a
changed pattern must rebuild everything.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["ras", "twolevel_ras"])
@pytest.mark.parametrize("dtypes", ["fp64", "mixed"])
def test_resetup_same_pattern_matches_fresh_setup(sg, kind, dtypes):
    N, NP = 24, 8
    part = sg.partition_boxes(N, N, N, NP, 0.08, 3)
    fd, sd = (sg.FP64, sg.FP64) if dtypes == "fp64" else (sg.BF16, sg.FP32)

    def make():
        if kind == "ras":
            return sg.RASPrecond(NP, 1, partition=part, factor_dtype=fd, sweep_dtype=sd)
        return sg.TwoLevelSchwarzPrecond(NP, 1, sg.FineLevelType.RAS, partition=part,
                                         factor_dtype=fd, sweep_dtype=sd)

    A1 = sg.make_varcoef_3d(N, N, N, 1.0, 3.0, 11)
    A2 = sg.make_varcoef_3d(N, N, N, 1.0, 3.0, 12)
    v = sg.uniform(A1.nrows, 5)
    reused = make()
    reused.setup(A1)
    y1 = reused.apply(v)
    reused.setup(A2)  # same pattern: host structures kept
    fresh = make()
    fresh.setup(A2)
    assert np.array_equal(reused.apply(v), fresh.apply(v))
    assert not np.array_equal(y1, fresh.apply(v))
    if kind == "twolevel_ras":
        assert np.array_equal(reused.coarse_a0(), fresh.coarse_a0())
    # a different pattern with the same n and partition rebuilds everything
    B = sg.make_poisson_2d(144, 96)
    assert B.nrows == A1.nrows
    reused.setup(B)
    fresh_b = make()
    fresh_b.setup(B)
    assert np.array_equal(reused.apply(v), fresh_b.apply(v))
    assert reused.decomposition()["sub"].tolist() == fresh_b.decomposition()["sub"].tolist()
