"""Burton-Miller operator (alpha != 0) and locally reacting surfaces on the GPU: matvecs
against the oracle's FMM and dense operators, the right-hand side and far field, and solves
against Mie series at a fictitious frequency of the sphere."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def normals(V, F):
    n = np.cross(V[F[:, 0]] - V[F[:, 2]], V[F[:, 1]] - V[F[:, 2]])
    return n / np.linalg.norm(n, axis=1)[:, None]


def fib_points(n, r=1.0):
    i = np.arange(n) + 0.5
    z = 1 - 2 * i / n
    ph = np.pi * (1 + 5 ** 0.5) * i
    s = np.sqrt(1 - z * z)
    return r * np.stack([s * np.cos(ph), s * np.sin(ph), z], axis=1)


@pytest.mark.parametrize("beta,rule", [(0.0, 1), (0.5 - 0.3j, 0), (0.1 + 0.05j, 1)])
def test_bm_matvec_matches_oracle(fm, oracle, beta, rule):
    V, F = fm.icosphere(3, 0.1)
    k = K1
    b = 1j * k * beta
    alpha = 1j / k
    a = 0.5 * (1 + alpha * b)
    plan = fm.Plan(V, F, k=k, depth=3, p_levels={2: 8, 3: 8}, rule=rule, a=a, b=b, c=-1.0, alpha=alpha)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    T = oracle.tree_for_fmm(V, F, depth=3)
    orc = oracle.FMM(V, F, k, T, [8, 8], a=a, b=b, c=-1.0, rule=rule, alpha=alpha)
    yo = orc.apply(x)
    y64 = plan.matvec(x, fm.FMM_FP64)
    assert rel(y64, yo) < 1e-10
    assert rel(plan.matvec(x, fm.FMM_MIXED), yo) < 1e-5
    assert rel(plan.matvec_adjoint(y, fm.FMM_FP64), orc.apply(y, transpose=True)) < 1e-10
    # against the dense combined operator, to the FMM's truncation accuracy
    yd = oracle.dense_apply(V, F, k, x, a=a, b=b, c=-1.0, rule=rule, alpha=alpha)
    assert rel(y64, yd) < 5e-4
    plan.close()


def test_bm_right_hand_side_and_admittance_far_field(fm, oracle):
    V, F = fm.icosphere(3, 0.1)
    k, beta = K1, 0.5 - 0.3j
    b, alpha = 1j * k * beta, 1j / k
    plan = fm.Plan(V, F, k=k, depth=3, p_levels={2: 8, 3: 8}, rule=1, a=0.5 * (1 + alpha * b), b=b, c=-1.0,
                   alpha=alpha)
    d = np.array([0.3, -0.4, np.sqrt(0.75)])
    C, N = V[F].mean(axis=1), normals(V, F)
    ref = np.exp(1j * k * C @ d) * (1 + alpha * 1j * k * (N @ d))
    assert rel(plan.plane_wave(d), ref) < 1e-13
    rng = np.random.default_rng(3)
    p = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    pts = fib_points(30, 1.0)
    assert rel(plan.far_field(p, pts), oracle.far_field(V, F, k, p, pts, rule=1, b=b, c=-1.0)) < 1e-12
    plan.close()


def test_bm_solve_at_fictitious_frequency_matches_mie(fm, oracle):
    """ka = pi: the conventional rigid-body operator is nearly singular there; the combined
    operator's GMRES solution matches the Mie series."""
    V, F = fm.icosphere(3, 0.1)
    k = np.pi / 0.1
    pts = fib_points(60, 1.0)
    mie = oracle.mie_rigid(k, 0.1, pts)
    out = {}
    for name, alpha in (("cbie", 0.0), ("bm", 1j / k)):
        plan = fm.Plan(V, F, k=k, depth=3, p_levels={2: 12, 3: 12}, rule=1, a=0.5, b=0.0, c=-1.0, alpha=alpha)
        x, it, rr, ok = plan.gmres(plan.plane_wave(), tol=1e-8, maxit=2000, restart=100, precision=fm.FMM_MIXED)
        assert ok
        out[name] = (it, rel(plan.far_field(x, pts), mie))
        plan.close()
    assert out["bm"][1] < 0.015
    assert out["cbie"][1] > 2 * out["bm"][1]


def test_admittance_bm_solve_matches_impedance_mie(fm, oracle):
    V, F = fm.icosphere(4, 0.1)
    k, beta = 2 * K1, 0.5 - 0.3j
    b, alpha = 1j * k * beta, 1j / k
    plan = fm.Plan(V, F, k=k, depth=4, p_levels={2: 14, 3: 12, 4: 10}, rule=1, a=0.5 * (1 + alpha * b), b=b, c=-1.0,
                   alpha=alpha)
    x, it, rr, ok = plan.gmres(plan.plane_wave(), tol=1e-8, maxit=1000, restart=60, precision=fm.FMM_MIXED)
    assert ok
    pts = fib_points(60, 1.0)
    assert rel(plan.far_field(x, pts), oracle.mie_impedance(k, 0.1, beta, pts)) < 0.01
    plan.close()
