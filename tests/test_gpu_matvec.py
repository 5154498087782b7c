"""GPU matvec parity: the CUDA library against the FP64 oracle (through the C ABI)."""
import json
import os

import numpy as np
import pytest

import meshes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
K1 = 2 * np.pi * 1000 / 343.0
K2 = 2 * np.pi * 8000 / 343.0
P2 = {2: 40, 3: 30, 4: 20, 5: 14, 6: 10}


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def sphere3(fm):
    return fm.icosphere(3, 0.1)


@pytest.fixture(scope="module")
def x3(sphere3):
    rng = np.random.default_rng(0)
    n = len(sphere3[1])
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


@pytest.mark.parametrize("abc,rule", [((0.5, 0.0, -1.0), 1), ((0.0, 1.0, 0.0), 0), ((0.3, 0.7 + 0.2j, -1.0), 0)])
def test_fp64_matvec_matches_oracle(fm, oracle, sphere3, x3, abc, rule):
    V, F = sphere3
    a, b, c = abc
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=rule, a=a, b=b, c=c)
    y = plan.matvec(x3, fm.FMM_FP64)
    T = oracle.tree_for_fmm(V, F, depth=3)
    yo = oracle.FMM(V, F, K1, T, [8, 8], a=a, b=b, c=c, rule=rule).apply(x3)
    assert rel(y, yo) < 1e-10
    ym = plan.matvec(x3, fm.FMM_MIXED)
    assert rel(ym, yo) < 1e-5
    plan.close()


def test_octree_counts_match_reference(fm, sphere3):
    """Box and M2L counts per level equal the reference's octree (golden fixtures)."""
    V, F = sphere3
    for case, depth in (("ico3_r0.1_d3", 3), ("ico3_r0.1_s5", 0)):
        g = np.load(os.path.join(GOLDEN, "octree_%s.npz" % case))
        plan = fm.Plan(V, F, k=K1, depth=depth, p_levels={l: 4 for l in range(2, 12)})
        info = plan.info
        assert info.lmax == int(g["lmax"])
        assert info.d == float(g["d"])
        for l in range(2, info.lmax + 1):
            assert info.num_box[l] == len(g["set_%d" % l])
            assert info.num_m2l[l] == int(g["srnum_%d" % l].sum())
        plan.close()


def test_full_size_mixed_vs_fp64_and_oracle(fm, oracle):
    """The 81,920-triangle workload: mixed within 1e-5 of FP64, FP64 equal to the oracle,
    and the operator linear."""
    import torch

    V, F = fm.icosphere(6, 0.3)
    plan = fm.Plan(V, F, k=K2, depth=6, p_levels=P2, rule=0, a=0.5, b=0.0, c=-1.0)
    info = plan.info
    meta = json.load(open(os.path.join(GOLDEN, "octree_meta.json")))["ico6_r0.3_d6"]
    for l in range(2, 7):
        assert info.num_m2l[l] == meta["sizes"]["sr_origin_%d" % l]
    rng = np.random.default_rng(0)
    n = plan.nf
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    xd = torch.from_numpy(x).cuda()
    y64 = plan.matvec(xd, fm.FMM_FP64).cpu().numpy()
    y32 = plan.matvec(xd, fm.FMM_MIXED).cpu().numpy()
    assert rel(y32, y64) < 1e-5
    yz = plan.matvec(z, fm.FMM_FP64)
    ylin = plan.matvec(2.0 * x + 3j * z, fm.FMM_FP64)
    assert rel(ylin, 2.0 * y64 + 3j * yz) < 1e-12
    T = oracle.tree_for_fmm(V, F, depth=6)
    yo = oracle.FMM(V, F, K2, T, [P2[l] for l in range(2, 7)], a=0.5, b=0.0, c=-1.0, rule=0).apply(x)
    assert rel(y64, yo) < 1e-10
    plan.close()


def test_host_device_pointers_and_multiple_rhs(fm, sphere3, x3):
    import torch

    V, F = sphere3
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=1, a=0.5, b=0.0, c=-1.0)
    yh = plan.matvec(x3, fm.FMM_FP64)
    yd = plan.matvec(torch.from_numpy(x3).cuda(), fm.FMM_FP64).cpu().numpy()
    assert np.array_equal(yh, yd)
    X = np.stack([x3, 1j * x3])
    Y = plan.matvec(X.reshape(-1), fm.FMM_FP64).reshape(2, -1)
    assert rel(Y[0], yh) < 1e-15 and rel(Y[1], 1j * yh) < 1e-14
    plan.close()


def test_mixed_batched_columns_match_single_column(fm, sphere3, x3):
    """Three columns in one batched mixed pass (device and host buffers) against one column
    at a time, and against FP64."""
    import torch

    V, F = sphere3
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=1, a=0.5, b=0.0, c=-1.0)
    rng = np.random.default_rng(5)
    X = np.stack([x3, rng.standard_normal(len(x3)) + 1j * rng.standard_normal(len(x3)), -2j * x3])
    Y = plan.matvec(X.reshape(-1), fm.FMM_MIXED).reshape(3, -1)
    Yd = plan.matvec(torch.from_numpy(X.reshape(-1)).cuda(), fm.FMM_MIXED).cpu().numpy().reshape(3, -1)
    for r in range(3):
        single = plan.matvec(X[r], fm.FMM_MIXED)
        assert rel(Y[r], single) < 1e-6 and rel(Yd[r], single) < 1e-6
        assert rel(Y[r], plan.matvec(X[r], fm.FMM_FP64)) < 1e-5
    # the adjoint takes the same batched path
    At = plan.matvec_adjoint(X.reshape(-1), fm.FMM_MIXED).reshape(3, -1)
    assert rel(At[1], plan.matvec_adjoint(X[1], fm.FMM_FP64)) < 1e-5
    plan.close()


def test_graph_replay_and_profiling_modes(fm, sphere3, x3):
    """The mixed translation passes replayed as a CUDA graph (profiling off or mode 2) give the
    direct launches' result (mode 1, one timer per pass)."""
    V, F = sphere3
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=1, a=0.5, b=0.0, c=-1.0)
    plan.set_profiling(1)
    direct = plan.matvec(x3, fm.FMM_MIXED)
    names = [n for n, _ in plan.timings()]
    assert names[0] == "p2m" and names[-2:] == ["translations", "matvec"]
    assert {"m2m_l3", "m2l_l2", "m2l_l3", "l2l_l3", "l2p_near"} <= set(names)
    plan.set_profiling(2)
    for _ in range(3):  # first call direct, second captures, third replays
        y = plan.matvec(x3, fm.FMM_MIXED)
        assert rel(y, direct) < 1e-6
    tm = plan.timings()
    assert [n for n, _ in tm] == ["matvec"] and tm[0][1] > 0
    plan.set_profiling(False)
    assert rel(plan.matvec(x3, fm.FMM_MIXED), direct) < 1e-6
    plan.close()


def test_repeated_matvec_is_reproducible(fm, sphere3, x3):
    """FP64: owner-computes accumulation without atomics, identical bits run to run.
    Mixed: FP32 atomics in the batched translation tiles, equal to rounding."""
    V, F = sphere3
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=1, a=0.5, b=0.0, c=-1.0)
    a = plan.matvec(x3, fm.FMM_FP64)
    b = plan.matvec(x3, fm.FMM_FP64)
    assert np.array_equal(a, b)
    a = plan.matvec(x3, fm.FMM_MIXED)
    b = plan.matvec(x3, fm.FMM_MIXED)
    assert rel(a, b) < 1e-6
    plan.close()


def test_invalid_arguments_fail_cleanly(fm, sphere3, x3):
    V, F = sphere3
    bad = np.array(F, copy=True)
    bad[5, 1] = len(V) + 3
    with pytest.raises(fm.FmmError) as e:
        fm.Plan(V, bad, k=K1, depth=3)
    assert e.value.status == 7
    degenerate = np.array(F, copy=True)
    degenerate[0] = [0, 0, 1]
    with pytest.raises(fm.FmmError):
        fm.Plan(V, degenerate, k=K1, depth=3)
    with pytest.raises(fm.FmmError):
        fm.Plan(V, F, k=-1.0, depth=3)
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, build_mixed=False)
    with pytest.raises(fm.FmmError):
        plan.matvec(x3, fm.FMM_MIXED)
    with pytest.raises(fm.FmmError):
        plan.matvec(x3, 7)
    # the plan stays usable after rejected calls
    assert np.isfinite(plan.matvec(x3, fm.FMM_FP64)).all()
    plan.close()
