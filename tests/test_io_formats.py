"""Host-side file formats of the library against the reference's own code
(golden outputs of tests/golden/make_golden.py, produced by oracle/_ref):

* sg_read_matrix_market vs read_matrix_market (src/io/matrix_market.h:14-92)
  on committed .mtx fixtures: general, symmetric (mirrored), pattern (read as
  1.0), duplicates (kept, not summed).  Structure must match exactly; values
  too, except that the order of duplicates within a row is the reference's
  unstable sort's, so duplicates are compared as multisets;
* sg_convergence_metrics / sg_write_convergence_jsonl vs ConvergenceMetrics
  (src/analysis/convergence_analysis.h:15-93): the same metrics and the same
  record bytes in <output>.conv.jsonl."""
from __future__ import annotations

import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MTX = os.path.join(ROOT, "tests", "golden", "mtx")


@pytest.mark.parametrize("name", ["general", "symmetric", "pattern", "duplicates"])
def test_matrix_market_reader_matches_reference(sg, golden, name):
    A = sg.read_matrix_market(os.path.join(MTX, f"{name}.mtx"))
    nr, nc = golden[f"mm/{name}/shape"]
    assert (A.nrows, A.ncols) == (nr, nc)
    rp, ci, v = (golden[f"mm/{name}/{k}"] for k in ("row_ptr", "col_idx", "vals"))
    np.testing.assert_array_equal(A.row_ptr, rp)
    np.testing.assert_array_equal(A.col_idx, ci)
    for i in range(nr):
        lo, hi = rp[i], rp[i + 1]
        for c in np.unique(ci[lo:hi]):
            m = ci[lo:hi] == c
            assert sorted(A.vals[lo:hi][m]) == sorted(v[lo:hi][m])


def test_matrix_market_errors(sg, tmp_path):
    with pytest.raises(sg.SgError, match="cannot open"):
        sg.read_matrix_market(str(tmp_path / "missing.mtx"))
    p = tmp_path / "short.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 4\n1 1 1\n2 2 1\n")
    with pytest.raises(sg.SgError, match="ends after 2 of 4"):
        sg.read_matrix_market(str(p))
    p = tmp_path / "range.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n")
    with pytest.raises(sg.SgError, match="outside the declared size"):
        sg.read_matrix_market(str(p))


def test_matrix_market_round_trip(sg, tmp_path):
    A = sg.make_poisson_2d(7, 5)
    p = tmp_path / "p.mtx"
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{A.nrows} {A.ncols} {A.nnz()}\n")
        for i in range(A.nrows):
            for e in range(A.row_ptr[i], A.row_ptr[i + 1]):
                f.write(f"{i + 1} {A.col_idx[e] + 1} {float(A.vals[e])!r}\n")
    B = sg.read_matrix_market(str(p))
    np.testing.assert_array_equal(B.row_ptr, A.row_ptr)
    np.testing.assert_array_equal(B.col_idx, A.col_idx)
    np.testing.assert_array_equal(B.vals, A.vals)


@pytest.mark.parametrize("name", ["gmres", "stagnating", "single", "empty"])
def test_convergence_record_matches_reference(sg, golden, tmp_path, name):
    h = golden[f"conv/{name}/history"]
    conv = bool(golden[f"conv/{name}/converged"])
    m = sg.convergence_metrics(h, conv)
    gm = golden[f"conv/{name}/metrics"]
    gi = golden[f"conv/{name}/imetrics"]
    assert m["iterations"] == gi[0] and m["stagnation_start"] == gi[1]
    np.testing.assert_allclose([m["initial_residual"], m["final_residual"],
                                m["asymptotic_rate"]], gm, rtol=1e-15, atol=0)
    np.testing.assert_allclose(m["rates"], golden[f"conv/{name}/rates"], rtol=1e-15, atol=0)
    path = tmp_path / "out.conv.jsonl"
    sg.write_convergence_jsonl(str(path), "poisson_12", "ilu0", 4, 1, h, conv)
    assert path.read_bytes() == golden[f"conv/{name}/jsonl"].tobytes()
