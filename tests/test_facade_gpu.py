"""include/schwarz_gmres.hpp as a drop-in for code written against the
reference's headers, with plug-ins of the caller's own: a Preconditioner
subclass applied on the host inside the GPU solve (src/precond/
preconditioner.h:7-20), fgmres_flex with a FlexApply, linear and nonlinear
(src/core/fgmres.h:37, :50-55), bicgstab, the analysis calls and
read_matrix_market.  tests/cpp/facade_plugins.cpp is compiled with g++
against the header and libsgmres.so and run; its printed results are checked
here."""
from __future__ import annotations

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "schwarz_gmres_dashboard_gb300", "_build")


@pytest.fixture(scope="module")
def results(sg, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("facade") / "facade_plugins")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_plugins.cpp"), "-o", exe,
                    "-L", BUILD, "-lsgmres", f"-Wl,-rpath,{BUILD}"], check=True)
    # three runs: the program releases its context from a static destructor
    # at exit, after the library's thread-local storage is gone -- a path
    # that once wrote into freed memory and aborted one run in four
    outs = [subprocess.run([exe, os.path.join(ROOT, "tests", "golden", "mtx", "symmetric.mtx")],
                           capture_output=True, text=True, timeout=300, check=True).stdout
            for _ in range(3)]
    out = outs[0]
    return {ln.split(" ", 1)[0]: ln.split(" ", 1)[1].split() for ln in out.splitlines() if ln}


@pytest.mark.gpu
def test_plugin_preconditioner_matches_device_one(results):
    pg, dg = results["plugin_gmres"], results["device_gmres"]
    assert pg[0] == "1" and dg[0] == "1"
    # the caller's host Jacobi and the GPU Jacobi: the same iteration count
    assert abs(int(pg[1]) - int(dg[1])) <= 1
    assert float(pg[2]) < 1e-6 and int(pg[3]) >= int(pg[1])


@pytest.mark.gpu
def test_flexible_apply(results):
    assert results["flex_fgmres"][0] == "1" and float(results["flex_fgmres"][2]) < 1e-6
    # the FlexApply (host Jacobi) and the GPU Jacobi in FGMRES: same iterations
    assert abs(int(results["flex_fgmres"][1]) - int(results["device_fgmres"][1])) <= 1
    # a nonlinear apply (the number of inner sweeps varies): FGMRES still converges
    assert results["flex_nonlinear"][0] == "1" and float(results["flex_nonlinear"][2]) < 1e-6


@pytest.mark.gpu
def test_bicgstab_and_analysis_through_the_facade(results):
    assert results["plugin_bicgstab"][0] == "1" and results["device_bicgstab"][0] == "1"
    assert float(results["device_bicgstab"][2]) < 1e-6
    lmin1, lmax1, lmin2, lmax2, steps = results["condition"]
    # host plug-in Jacobi and GPU Jacobi give the same Ritz values
    assert abs(float(lmin1) - float(lmin2)) <= 1e-9 * abs(float(lmin2))
    assert abs(float(lmax1) - float(lmax2)) <= 1e-9 * abs(float(lmax2))
    assert int(steps) == 80
    rho, iters, ok = results["spectral"]
    assert 0.0 < float(rho) < 1.0 and ok == "1"
    assert int(results["convergence"][0]) == int(results["plugin_gmres"][1])


@pytest.mark.gpu
def test_plugin_exception_is_rethrown(results):
    assert " ".join(results["throw"]) == "plug-in failure 42"


@pytest.mark.gpu
def test_read_matrix_market_through_the_facade(results):
    assert results["mtx"] == ["5", "5", "12"]
