"""The integer set-up on the device (setup_gpu.cu) against the host set-up
(setup.cpp): decomposition, owned-local map, local matrices and their global
entries, diagonal positions, widths, level schedules, level orders, slot
layouts and launch order must be the same arrays, bit for bit, and so must
the factors and an FP64 apply.  Cases: 3D box subdomains (the 128^3
workload's shape, smaller; overlap 1 and 2), the built-in graph partitioner
on the reference's Poisson matrices (overlap 0, 1, 2), a 2D anisotropic
batch with many small parts (more than 256 parts: a two-pass radix sort of
the owned lists), one ILU(0) block, and a matrix with duplicate diagonal
entries."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHED = range(13)


def _pair(sg, mk, A):
    out = []
    for where in ("device", "host"):
        pc = mk(where)
        pc.setup(A)
        assert pc.setup_on_device() == (where == "device"), where
        out.append(pc)
    return out


def _same(sg, dev, host, A):
    da, db = dev.decomposition(), host.decomposition()
    for k in da:
        assert np.array_equal(da[k], db[k]), ("decomposition", k)
    for s in range(len(da["sub_ptr"]) - 1):
        fa, fb = dev.factors(s), host.factors(s)
        for k in fa:
            assert np.array_equal(fa[k], fb[k]), ("factors", s, k)
    for w in SCHED:
        assert np.array_equal(dev.schedule(w), host.schedule(w)), ("schedule", w)
    x = sg.uniform(A.nrows, seed=5)
    ya, yb = dev.apply(x), host.apply(x)
    assert np.array_equal(ya, yb)  # same structure and schedule: the same bits in any precision


def test_box_subdomains(sg):
    A = sg.make_varcoef_3d(30, 26, 22, 1.0, 6.0, seed=3)
    part = sg.partition_boxes(30, 26, 22, 24, 0.1, seed=4)
    for ov in (1, 2):
        dev, host = _pair(sg, lambda where: sg.TwoLevelSchwarzPrecond(
            24, ov, sg.FineLevelType.RAS, part, setup=where), A)
        _same(sg, dev, host, A)
        assert np.array_equal(dev.coarse_a0(), host.coarse_a0())


@pytest.mark.parametrize("ov", [0, 1, 2])
def test_graph_partition_poisson(sg, ov):
    A = sg.make_poisson_3d(18, 17, 16)
    part = sg.partition_graph(A, 11)
    dev, host = _pair(sg, lambda where: sg.RASPrecond(11, ov, partition=part, setup=where), A)
    _same(sg, dev, host, A)
    A2 = sg.make_poisson_2d(40, 37)
    part2 = sg.partition_graph(A2, 7)
    dev, host = _pair(sg, lambda where: sg.ASMPrecond(7, ov, partition=part2, setup=where), A2)
    _same(sg, dev, host, A2)


def test_many_parts_two_radix_passes(sg):
    prob = sg.make_aniso_batch(40, seed=6, nmin=30, nmax=60, rows_per_part=64, min_parts=4,
                               max_parts=16)
    assert prob.nparts > 256
    dev, host = _pair(sg, lambda where: sg.RASPrecond(
        prob.nparts, 1, partition=prob.partition, factor_dtype=sg.BF16, sweep_dtype=sg.FP32,
        setup=where), prob.A)
    _same(sg, dev, host, prob.A)


def test_single_ilu0_block(sg):
    A = sg.make_poisson_2d(33, 29)
    dev, host = _pair(sg, lambda where: sg.ILU0Precond(setup=where), A)
    _same(sg, dev, host, A)


def test_duplicate_diagonal_entries(sg):
    """A repeated diagonal entry (the reference's MatrixMarket reader keeps
    duplicates): both set-ups read the same level for it."""
    A = sg.make_poisson_2d(12, 11)
    rp, ci, v = A.row_ptr.copy(), A.col_idx.copy(), A.vals.copy()
    rows = []
    for i in range(A.nrows):
        cols = list(ci[rp[i]:rp[i + 1]])
        vals = list(v[rp[i]:rp[i + 1]])
        if i % 5 == 0:  # a second diagonal entry after the first
            k = cols.index(i)
            cols.insert(k + 1, i)
            vals.insert(k + 1, 0.5)
        rows.append((cols, vals))
    nrp = np.zeros(A.nrows + 1, np.int32)
    for i, (c, _) in enumerate(rows):
        nrp[i + 1] = nrp[i] + len(c)
    nci = np.concatenate([np.array(c, np.int32) for c, _ in rows])
    nv = np.concatenate([np.array(x, np.float64) for _, x in rows])
    B = sg.CSRMatrix(A.nrows, A.ncols, nrp, nci, nv)
    part = sg.partition_graph(B, 3)
    dev, host = _pair(sg, lambda where: sg.RASPrecond(3, 1, partition=part, setup=where), B)
    _same(sg, dev, host, B)
