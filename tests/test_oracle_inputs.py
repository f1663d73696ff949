"""The oracle's restatement of the project's benchmark inputs (uniform
vectors, uneven box partitions, the variable-coefficient 3D operator) against
the package's generators, bit for bit.  The CPU baseline builds its problem
from the oracle side alone, so both arms must see the same matrix, partition
and right-hand side."""
from __future__ import annotations

import numpy as np
import pytest


def test_uniform_matches_package(sg, oracle):
    for seed, n in ((0, 1), (2, 1000), (123456789, 4097)):
        np.testing.assert_array_equal(oracle.uniform(n, seed), sg.uniform(n, seed=seed))
    np.testing.assert_array_equal(oracle.uniform(50, 7, 0.5, 2.0), sg.uniform(50, 7, 0.5, 2.0))


@pytest.mark.parametrize("dims,nparts,spread,seed", [
    ((128, 128, 128), 256, 0.08, 1),   # the 128^3 benchmark partition
    ((96, 96, 96), 108, 0.08, 1),      # the 96^3 learned-stage workload
    ((33, 17, 9), 13, 0.3, 5),         # odd sizes, odd part count
    ((8, 8, 8), 1, 0.0, 0),
])
def test_partition_boxes_matches_package(sg, oracle, dims, nparts, spread, seed):
    a = oracle.partition_boxes(*dims, nparts, spread, seed)
    b = sg.partition_boxes(*dims, nparts, spread, seed=seed)
    np.testing.assert_array_equal(a, b)
    assert a.min() == 0 and a.max() == nparts - 1


@pytest.mark.parametrize("dims,sigma,corr,seed", [
    ((24, 24, 24), 1.0, 8.0, 0),
    ((17, 11, 13), 1.0, 4.0, 3),
    ((40, 40, 40), 0.5, 2.0, 1234),
])
def test_varcoef3d_matches_package(sg, oracle, dims, sigma, corr, seed):
    H = oracle.varcoef3d(*dims, sigma, corr, seed)
    A = sg.make_varcoef_3d(*dims, sigma, corr, seed=seed)
    np.testing.assert_array_equal(H.row_ptr, A.row_ptr)
    np.testing.assert_array_equal(H.col_idx, A.col_idx)
    np.testing.assert_array_equal(H.vals, A.vals)
