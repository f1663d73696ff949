"""CPU tests of libsgmres: the shared library loads and exports every symbol
include/*.h declares, and the host-side integer work (generators,
partitioners, decomposition, local structures, level schedules) matches the
oracle bit for bit.  No call here touches a GPU."""
from __future__ import annotations

import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT, HostCSR, golden_matrix


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(sg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(sg):
    names = declared_symbols()
    assert len(names) >= 20
    lib = C.CDLL(os.path.join(ROOT, "schwarz_gmres_dashboard_gb300", "_build", "libsgmres.so"))
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    from schwarz_gmres_dashboard_gb300 import _lib
    assert names <= set(_lib.PROTOTYPES), names - set(_lib.PROTOTYPES)


def test_abi_version_and_status_strings(sg):
    from schwarz_gmres_dashboard_gb300 import _lib as L
    lib = L.load()
    assert lib.sg_abi_version() == 1
    for st in range(11):
        assert lib.sg_status_string(st)


@pytest.mark.parametrize("dims", [(1, 1), (5, 5), (12, 7), (128, 128)])
def test_poisson2d_matches_reference_generator(sg, oracle, dims):
    A = sg.make_poisson_2d(*dims)
    rp, ci, v = oracle.poisson2d(*dims)
    assert np.array_equal(A.row_ptr, rp) and np.array_equal(A.col_idx, ci)
    assert np.array_equal(A.vals, v)


@pytest.mark.parametrize("dims", [(1, 1, 1), (6, 7, 5), (16, 16, 16)])
def test_poisson3d_matches_reference_generator(sg, oracle, dims):
    A = sg.make_poisson_3d(*dims)
    rp, ci, v = oracle.poisson3d(*dims)
    assert np.array_equal(A.row_ptr, rp) and np.array_equal(A.col_idx, ci)
    assert np.array_equal(A.vals, v)


def test_varcoef_reduces_to_poisson_and_is_spd_like(sg, oracle):
    A = sg.make_varcoef_3d(10, 9, 8, sigma=0.0, corr_len=3.0, seed=4)
    rp, ci, v = oracle.poisson3d(10, 9, 8)
    assert np.array_equal(A.row_ptr, rp) and np.array_equal(A.col_idx, ci)
    assert np.allclose(A.vals, v, rtol=0, atol=1e-14)
    B = sg.make_varcoef_3d(12, 12, 12, sigma=1.0, corr_len=4.0, seed=9)
    import scipy.sparse as sp
    M = sp.csr_matrix((B.vals, B.col_idx, B.row_ptr), shape=(B.nrows, B.nrows))
    assert abs(M - M.T).max() < 1e-12
    d = M.diagonal()
    off = np.asarray(abs(M).sum(axis=1)).ravel() - d
    assert (d >= off - 1e-12).all() and (d > 0).all()
    # deterministic in the seed
    B2 = sg.make_varcoef_3d(12, 12, 12, sigma=1.0, corr_len=4.0, seed=9)
    assert np.array_equal(B.vals, B2.vals)


def test_uniform_generator(sg):
    u = sg.uniform(1000, seed=0)
    assert u.min() >= -1 and u.max() < 1 and abs(u.mean()) < 0.1
    assert np.array_equal(u, sg.uniform(1000, seed=0))
    assert not np.array_equal(u, sg.uniform(1000, seed=1))


@pytest.mark.parametrize("nparts", [1, 2, 7, 16])
def test_graph_partition_valid(sg, nparts):
    A = sg.make_poisson_3d(10, 11, 12)
    part = sg.partition_graph(A, nparts)
    cnt = np.bincount(part, minlength=nparts)
    assert len(cnt) == nparts and cnt.min() > 0
    assert cnt.max() - cnt.min() <= 1
    assert np.array_equal(part, sg.partition_graph(A, nparts))


def test_box_partition_spread(sg):
    part = sg.partition_boxes(128, 128, 128, 256, spread=0.08, seed=1)
    cnt = np.bincount(part, minlength=256)
    assert cnt.min() > 0
    assert 1.5 < cnt.max() / cnt.min() < 2.6
    part0 = sg.partition_boxes(32, 32, 32, 64, spread=0.0, seed=1)
    assert (np.bincount(part0) == 512).all()


def _oracle_local(oracle, A, st):
    """Local CSR of each subdomain from the oracle's extraction, for comparison."""
    return None


@pytest.mark.parametrize("case", ["p2d_blocks", "p2d_scatter", "p3d_slabs"])
@pytest.mark.parametrize("overlap", [0, 1, 2])
def test_host_structure_matches_oracle(sg, oracle, golden, case, overlap):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    Am = sg.CSRMatrix(A.nrows, A.nrows, A.row_ptr, A.col_idx, A.vals)
    st = sg.schwarz_structure(Am, part, nparts, overlap)
    # decomposition: bit-exact against the reference's golden data
    for k in ("owned_ptr", "owned", "sub_ptr", "sub", "ownloc_ptr", "ownloc"):
        assert np.array_equal(st[k], golden[f"{case}/dd{overlap}/{k}"]), k
    # local matrices, diagonal positions and level schedules against the oracle
    from oracle.oracle import ORACLE_SO  # noqa: F401
    rp_all, ci_all = st["local_row_ptr"], st["local_col_idx"]
    roff, zoff = 0, 0
    for s in range(nparts):
        dofs = st["sub"][st["sub_ptr"][s]:st["sub_ptr"][s + 1]]
        ns = len(dofs)
        lrp = rp_all[roff:roff + ns + 1]
        nz = int(lrp[-1])
        lci = ci_all[zoff:zoff + nz]
        roff += ns + 1
        zoff += nz
        # oracle extraction
        import ctypes
        ext_rp = np.empty(ns + 1, np.int32)
        nzo = oracle.lib.orc_extract  # noqa: F841
        sub_rp, sub_ci, sub_v = _extract(oracle, A, dofs)
        assert np.array_equal(lrp, sub_rp) and np.array_equal(lci, sub_ci)
        L = HostCSR(sub_rp, sub_ci, sub_v)
        _, dg = oracle.ilu0_factor(L)
        lo, up = oracle.levels(L, dg)
        off = st["sub_ptr"][s]
        assert np.array_equal(st["diag_ptr"][off:off + ns], dg)
        assert np.array_equal(st["level_lower"][off:off + ns], lo)
        assert np.array_equal(st["level_upper"][off:off + ns], up)


def _extract(oracle, A, idx):
    import ctypes as C
    L = oracle.lib
    L.orc_extract.restype = C.c_int
    L.orc_extract.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    idx = np.ascontiguousarray(idx, np.int32)
    nz = L.orc_extract(A.nrows, A.nrows, A.row_ptr.ctypes.data, A.col_idx.ctypes.data,
                       A.vals.ctypes.data, idx.ctypes.data, len(idx), None, None, None)
    rp = np.empty(len(idx) + 1, np.int32)
    ci = np.empty(max(nz, 1), np.int32)
    v = np.empty(max(nz, 1), np.float64)
    L.orc_extract(A.nrows, A.nrows, A.row_ptr.ctypes.data, A.col_idx.ctypes.data,
                  A.vals.ctypes.data, idx.ctypes.data, len(idx), rp.ctypes.data, ci.ctypes.data,
                  v.ctypes.data)
    return rp, ci[:nz], v[:nz]


def test_host_structure_rejects_bad_input(sg):
    A = sg.make_poisson_2d(4, 4)
    with pytest.raises(sg.SgError):
        sg.schwarz_structure(A, np.full(16, 3, np.int32), 2, 1)  # part id out of range
    with pytest.raises(sg.SgError):
        sg.schwarz_structure(A, np.zeros(16, np.int32), 2, 1)  # empty subdomain
    # missing diagonal
    B = sg.CSRMatrix(2, 2, [0, 1, 2], [1, 0], [1.0, 1.0])
    with pytest.raises(sg.SgError) as e:
        sg.schwarz_structure(B, np.zeros(2, np.int32), 1, 0)
    assert e.value.status == 4


def test_aniso2d_generator(sg):
    """9-point anisotropic stencil: symmetric, K = R diag(1, eps) R^T, and the
    eps = 1 case equals the 5-point Laplacian (its corner entries are zeros)."""
    import scipy.sparse as sp
    n, eps, th = 7, 0.01, 0.6
    A = sg.make_aniso_2d(n, n, eps, th)
    S = sp.csr_matrix((A.vals, A.col_idx, A.row_ptr), shape=(n * n, n * n))
    assert abs(S - S.T).max() == 0
    c, s = np.cos(th), np.sin(th)
    kxx, kyy, kxy = c * c + eps * s * s, s * s + eps * c * c, (1 - eps) * s * c
    i = 3 * n + 3  # interior point
    row = dict(zip(A.col_idx[A.row_ptr[i]:A.row_ptr[i + 1]], A.vals[A.row_ptr[i]:A.row_ptr[i + 1]]))
    assert np.isclose(row[i], 2 * kxx + 2 * kyy) and np.isclose(row[i - 1], -kxx)
    assert np.isclose(row[i - n], -kyy) and np.isclose(row[i + n + 1], -kxy / 2)
    assert np.isclose(row[i + n - 1], kxy / 2) and len(row) == 9
    assert np.all(np.diff(A.col_idx[A.row_ptr[i]:A.row_ptr[i + 1]]) > 0)
    iso = sg.make_aniso_2d(n, n, 1.0, 0.3)
    P = sg.make_poisson_2d(n, n)
    Si = sp.csr_matrix((iso.vals, iso.col_idx, iso.row_ptr), shape=(n * n, n * n))
    Sp = sp.csr_matrix((P.vals, P.col_idx, P.row_ptr), shape=(n * n, n * n))
    assert abs(Si - Sp).max() < 1e-15


def test_aniso_batch_layout(sg):
    prob = sg.make_aniso_batch(9, seed=4, nmin=20, nmax=40, rows_per_part=200)
    assert prob.sys_row_ptr[-1] == prob.n == int((prob.sizes ** 2).sum())
    assert np.all((prob.sizes >= 20) & (prob.sizes <= 40))
    assert np.all((prob.eps >= 1e-3) & (prob.eps <= 1.0))
    # block diagonal, every part inside one system
    for s in range(prob.nsys):
        lo, hi = prob.sys_row_ptr[s], prob.sys_row_ptr[s + 1]
        cols = prob.A.col_idx[prob.A.row_ptr[lo]:prob.A.row_ptr[hi]]
        assert cols.min() >= lo and cols.max() < hi
        ps = np.unique(prob.partition[lo:hi])
        assert len(ps) == prob.parts[s]
        others = np.concatenate([prob.partition[:lo], prob.partition[hi:]])
        assert not np.isin(ps, others).any()
