"""Host logic of the library on the CPU, compiled host-only by nvcc (nothing runs on a GPU):
the lockstep GMRES and iterative refinement (gmres_core.h) over a column layout of dense
complex systems of unequal sizes (tests/cpu_solver/solver_check.cu), and the work-item builder
of the batched translation passes (tests/cpu_solver/items_check.cu).  The solver checks: every
column reaches tol in the FP64 residual, the refinement over an FP32 operator does too, a zero
right-hand side stays zero, converged columns are left out of the operator.  The item checks:
every column covered once, items within one direction, Morton ranges beyond the L2 budget."""
import json
import math
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    return nvcc


def _build_and_run(tmp_path_factory, name, flags=()):
    exe = str(tmp_path_factory.mktemp(name) / name)
    src = os.path.join(HERE, "cpu_solver", name + ".cu")
    subprocess.run([_nvcc(), "-std=c++17", "-O2", *flags, "-o", exe, src], check=True, capture_output=True, timeout=900)
    return subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    out = _build_and_run(tmp_path_factory, "solver_check")
    return {d["case"]: d for d in (json.loads(line) for line in out.splitlines() if line.strip())}


@pytest.fixture(scope="module")
def items(tmp_path_factory):
    # batched.cu's kernels use FP32 vector atomics: device code for the GB300 target, never launched
    out = _build_and_run(tmp_path_factory, "items_check", ("-gencode", "arch=compute_103a,code=sm_103a"))
    return json.loads(out)


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


def test_items_cover_every_column_once_within_one_direction(items):
    kb, rank, nd = items["key_beg"], items["dst_rank"], items["ndst"]
    T = kb[-1]
    key_of = [d for d in range(len(kb) - 1) for _ in range(kb[d + 1] - kb[d])]
    for c in items["cases"]:
        nrhs, width = c["nrhs"], c["width"]
        seen = [0] * (T * nrhs)
        for d, first, count, w in c["items"]:
            assert 1 <= count <= width
            assert w == (items["key_w"][d] if c["coax_w"] else 0)
            for e in range(first, first + count):
                seen[e] += 1
                assert key_of[e // nrhs] == d
        assert seen == [1] * (T * nrhs)


def test_items_follow_morton_ranges_beyond_the_l2_budget(items):
    kb, rank, nd = items["key_beg"], items["dst_rank"], items["ndst"]
    budget = 48 << 20
    for c in items["cases"]:
        nblk = min(nd, max(1, -(-c["ws"] // budget)))
        # range k holds the destination ranks [k nd / nblk, (k + 1) nd / nblk), rounded down
        lo = [k * nd // nblk for k in range(nblk)]
        block_of = [max(k for k in range(nblk) if lo[k] <= r) for r in range(nd)]
        blocks = []
        for d, first, count, w in c["items"]:
            b = {block_of[rank[e // c["nrhs"]]] for e in range(first, first + count)}
            assert len(b) == 1  # one destination range per item
            blocks.append(b.pop())
        assert blocks == sorted(blocks)  # range by range
        if nblk == 1:
            # without ranges: direction by direction, as the translations lie
            assert [it[0] for it in c["items"]] == sorted(it[0] for it in c["items"])
