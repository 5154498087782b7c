"""The lockstep GMRES and iterative refinement (gmres_core.h) on the CPU: the same template the
plans and scenes run, compiled host-only by nvcc over a column layout of dense complex systems
of unequal sizes (tests/cpu_solver/solver_check.cu).  Checks that every column reaches tol in
the FP64 residual, that the refinement over an FP32 operator does too, that a zero right-hand
side stays zero, and that columns which have converged are left out of the operator."""
import json
import math
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("solver") / "solver_check")
    src = os.path.join(HERE, "cpu_solver", "solver_check.cu")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-o", exe, src], check=True, capture_output=True, timeout=600)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout
    return {d["case"]: d for d in (json.loads(line) for line in out.splitlines() if line.strip())}


def test_fp64_columns_reach_tol_and_report_their_true_residual(results):
    d = results["fp64"]
    assert d["status"] == 0
    assert all(r <= 1e-10 for r in d["true_res"])
    assert all(abs(a - b) <= 1e-12 for a, b in zip(d["relres"], d["true_res"]))
    assert results["fp64_long_restart"]["status"] == 0
    assert all(r <= 1e-10 for r in results["fp64_long_restart"]["true_res"])


def test_refinement_over_an_fp32_operator_reaches_the_fp64_tolerance(results):
    d = results["mixed"]
    assert d["status"] == 0
    assert all(r <= 1e-9 for r in d["true_res"])


def test_zero_right_hand_side_stays_zero(results):
    d = results["mixed_zero_rhs"]
    assert d["iters"][-1] == 0 and d["true_res"][-1] == 0.0
    assert all(r <= 1e-8 for r in d["true_res"][:-1])


def test_converged_columns_leave_the_operator(results):
    """Columns converge after 17 to ~640 steps; with GMRES(10) applying every column every step
    would take R (max_it + restarts) column applications."""
    d = results["fp64"]
    R, m = len(d["iters"]), max(d["iters"])
    all_columns = R * (m + math.ceil(m / 10) + 1)
    assert d["col_matvecs"] <= 0.5 * all_columns
