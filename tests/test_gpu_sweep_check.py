"""Checked mode of the TMA-fed sweep (the debug-build bounds checks of the
kernel, done on the host): after set-up, every level record's row and column
slots are inside the subdomain vector, every column a row reads was computed
by an earlier level of its sweep, and the ring schedule issues every record
group before it is waited for and never over bytes or an mbarrier still in
use.  Checked on 3D box subdomains (the 128^3 workload's shape, smaller),
2D anisotropic 9-point subdomains (the batched workload's shape) and the
reference's Poisson matrices, in every factor / sweep precision and for
forced record-group sizes; a corrupted host copy must be caught."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {"fp64": (0, 0), "fp32": (1, 1), "bf16": (2, 1)}  # (factor dtype, sweep dtype)


def _mk(sg, kind, p, ov, part, dt, **kw):
    fd, sd = DT[dt]
    if kind == "ras":
        return sg.RASPrecond(p, ov, partition=part, factor_dtype=fd, sweep_dtype=sd, **kw)
    return sg.TwoLevelSchwarzPrecond(p, ov, sg.FineLevelType.RAS, part, factor_dtype=fd,
                                     sweep_dtype=sd, **kw)


@pytest.mark.parametrize("dt", ["fp64", "fp32", "bf16"])
def test_records_and_ring_schedule_hold(sg, dt):
    cases = []
    A = sg.make_varcoef_3d(24, 26, 22, 1.0, 6.0, seed=3)
    cases.append((A, sg.partition_boxes(24, 26, 22, 20, 0.1, seed=4), 20, 1, "twolevel"))
    A2 = sg.make_aniso_2d(90, 70, 0.01, 0.7)
    cases.append((A2, sg.partition_graph(A2, 6), 6, 1, "ras"))
    A3 = sg.make_poisson_3d(20, 20, 20)
    cases.append((A3, sg.partition_graph(A3, 8), 8, 2, "ras"))
    for A, part, p, ov, kind in cases:
        pc = _mk(sg, kind, p, ov, part, dt)
        pc.setup(A)
        ch = pc.sweep_choice()
        assert ch["sweep"] == "tma" and ch["ring_bytes"] > 0 and ch["group_bytes"] > 0, ch
        assert pc.check() == 0
        pc.close()


def test_forced_group_sizes_keep_the_schedule_valid(sg):
    A = sg.make_varcoef_3d(24, 26, 22, 1.0, 6.0, seed=3)
    part = sg.partition_boxes(24, 26, 22, 20, 0.1, seed=4)
    x = sg.uniform(A.nrows, seed=5)
    ys = []
    for grp in (1024, 4096, 16384, 65536):
        pc = _mk(sg, "twolevel", 20, 1, part, "bf16", sweep_threads=256, group_bytes=grp)
        pc.setup(A)
        assert pc.check() == 0, grp
        ys.append(pc.apply(x))
        pc.close()
    for y in ys[1:]:
        assert np.array_equal(y, ys[0])  # the record schedule never changes the bits


def test_check_catches_a_planted_fault(sg):
    A = sg.make_poisson_3d(16, 16, 16)
    pc = _mk(sg, "ras", 4, 1, sg.partition_graph(A, 4), "fp32")
    pc.setup(A)
    assert pc.check() == 0
    assert pc.check(plant=True) > 0
