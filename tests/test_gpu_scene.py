"""Scenes (fmm_scene_*): many plans applied and solved in lockstep with one set of launches
per matvec (persistent work-queue translation kernels, CUDA graph), against the same plans
one at a time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_bodies(fm):
    """Uneven bodies: orders from 8 to 50, depths 2 to 4, one with scaled FP32 expansions
    (1 kHz, p = 16), one with 4-column tiles (p = 50), Burton-Miller and admittance."""
    plans = []
    V, F = fm.icosphere(3, 0.1)
    k = 2 * np.pi * 1000 / 343.0
    plans.append(fm.Plan(V, F, k=k, depth=3, p_levels={2: 16, 3: 16}, rule=1, a=0.5, b=0.0, c=-1.0))
    k = 2 * np.pi * 8000 / 343.0
    plans.append(fm.Plan(V, F, k=k, depth=3, p_levels={2: 50, 3: 36}, rule=1, a=0.5, b=0.0, c=-1.0, alpha=1j / k))
    V, F = fm.ellipsoid(8, (0.05, 0.07, 0.04), lmax=8, sigma=1e-3, seed=3)
    k = 2 * np.pi * 4000 / 343.0
    beta = 0.3 - 0.1j
    b, alpha = 1j * k * beta, 1j / k
    plans.append(fm.Plan(V, F, k=k, depth=-1, rule=1, a=0.5 * (1 + alpha * b), b=b, c=-1.0, alpha=alpha))
    V, F = fm.box(6, (0.03, 0.05, 0.08))
    k = 2 * np.pi * 6000 / 343.0
    plans.append(fm.Plan(V, F, k=k, depth=-1, rule=1, a=0.5, b=0.0, c=-1.0, alpha=1j / k))
    V, F = fm.geodesic_sphere(12, 0.08)
    k = 2 * np.pi * 9000 / 343.0
    plans.append(fm.Plan(V, F, k=k, depth=4, p_levels={2: 24, 3: 18, 4: 12}, rule=1, a=0.5, b=0.0, c=-1.0,
                         alpha=1j / k))
    return plans


@pytest.fixture(scope="module")
def bodies(fm):
    plans = make_bodies(fm)
    yield plans
    for p in plans:
        p.close()


def test_scene_matvec_matches_the_plans(fm, bodies):
    sc = fm.Scene(bodies)
    assert sc.n == sum(p.nf for p in bodies)
    assert list(np.diff(sc.offsets)) == [p.nf for p in bodies]
    rng = np.random.default_rng(21)
    xs = [rng.standard_normal(p.nf) + 1j * rng.standard_normal(p.nf) for p in bodies]
    x = sc.join(xs)
    y64 = sc.split(sc.matvec(x, fm.FMM_FP64))
    for p, xi, yi in zip(bodies, xs, y64):
        assert rel(yi, p.matvec(xi, fm.FMM_FP64)) < 1e-13
    # the first call runs the launches directly, the second captures them, later ones replay
    for rep in range(4):
        ym = sc.split(sc.matvec(x, fm.FMM_MIXED))
        for p, xi, yi, y6 in zip(bodies, xs, ym, y64):
            assert rel(yi, y6) < 1e-5, (rep, p.nf)
            assert rel(yi, p.matvec(xi, fm.FMM_MIXED)) < 1e-5
    sc.close()


def test_scene_matvec_on_a_subset_of_plans(fm, bodies):
    sc = fm.Scene(bodies)
    rng = np.random.default_rng(22)
    xs = [rng.standard_normal(p.nf) + 1j * rng.standard_normal(p.nf) for p in bodies]
    on = [True, False, True, False, True]
    sc.set_active(on)
    for rep in range(3):
        ys = sc.split(sc.matvec(sc.join(xs), fm.FMM_MIXED))
        for p, xi, yi, a in zip(bodies, xs, ys, on):
            if a:
                assert rel(yi, p.matvec(xi, fm.FMM_FP64)) < 1e-5
            else:
                assert not np.any(yi)
    sc.set_active(None)
    ys = sc.split(sc.matvec(sc.join(xs), fm.FMM_MIXED))
    assert all(rel(yi, p.matvec(xi, fm.FMM_FP64)) < 1e-5 for p, xi, yi in zip(bodies, xs, ys))
    sc.close()


def test_scene_solve_matches_the_plans(fm, bodies):
    sc = fm.Scene(bodies)
    bs = [p.plane_wave(np.array([0.0, 0.6, 0.8])) for p in bodies]
    x, it, rr, ok = sc.solve(bs, tol=1e-7, maxit=2000, restart=60, precision=fm.FMM_MIXED)
    assert ok and (rr <= 1e-7).all()
    for p, b, xi, n_it in zip(bodies, bs, sc.split(x), it):
        xp, itp, rrp, okp = p.gmres(b, tol=1e-7, maxit=2000, restart=60, precision=fm.FMM_MIXED)
        assert okp
        assert rel(xi, xp) < 1e-5
        assert n_it > 0
        # the FP64 residual of the scene's solution is the one it reports
        assert np.linalg.norm(p.matvec(xi, fm.FMM_FP64) - b) <= 1.01e-7 * np.linalg.norm(b)
    # plain FP64 lockstep solve too
    x64, it64, rr64, ok64 = sc.solve(bs, tol=1e-7, maxit=2000, restart=60, precision=fm.FMM_FP64)
    assert ok64 and rel(x64, x) < 1e-5
    sc.close()


def test_scene_refuses_plans_whose_buffers_moved(fm):
    V, F = fm.icosphere(2, 0.1)
    k = 2 * np.pi * 2000 / 343.0
    plans = [fm.Plan(V, F, k=k * (1 + i), depth=2, p_levels={2: 8}, rule=1, a=0.5, b=0.0, c=-1.0) for i in range(2)]
    sc = fm.Scene(plans)
    x = np.ones(sc.n, dtype=np.complex128)
    sc.matvec(x)
    # a 4-column matvec of plan 1 reallocates its FP32 expansions
    plans[1].matvec(np.ones(4 * plans[1].nf, dtype=np.complex128), fm.FMM_MIXED)
    with pytest.raises(fm.FmmError, match="create the scene again"):
        sc.matvec(x)
    # a plan is not destroyed while a scene uses it
    with pytest.raises(fm.FmmError, match="destroy them first"):
        plans[0].close()
    sc.close()
    sc = fm.Scene(plans)
    y = sc.split(sc.matvec(x))
    assert all(rel(yi, p.matvec(np.ones(p.nf, dtype=np.complex128), fm.FMM_FP64)) < 1e-5 for p, yi in zip(plans, y))
    sc.close()
    for p in plans:
        p.close()


def test_scene_rejects_unsuitable_plans(fm, bodies):
    V, F = fm.icosphere(2, 0.1)
    fp64_only = fm.Plan(V, F, k=10.0, depth=2, p_levels={2: 8}, rule=1, a=0.5, b=0.0, c=-1.0, build_mixed=False)
    with pytest.raises(fm.FmmError, match="no mixed-precision tables"):
        fm.Scene([bodies[0], fp64_only])
    with pytest.raises(fm.FmmError, match="appears twice"):
        fm.Scene([bodies[0], bodies[1], bodies[0]])
    fp64_only.close()


def test_scene_frequency_sweep_matches_mie(fm, oracle):
    """One mesh at four frequencies (one plan each, orders from the truncation rule): the
    lockstep solve of the Burton-Miller rigid problem against the Mie series."""
    V, F = fm.icosphere(4, 0.1)
    freqs = [500.0, 1000.0, 2000.0, 3000.0]
    plans = []
    for f in freqs:
        k = 2 * np.pi * f / 343.0
        plans.append(fm.Plan(V, F, k=k, depth=4, rule=1, a=0.5, b=0.0, c=-1.0, alpha=1j / k))
    sc = fm.Scene(plans)
    d = np.array([0.0, 0.0, 1.0])
    x, it, rr, ok = sc.solve([p.plane_wave(d) for p in plans], tol=1e-7, maxit=1000, restart=60, precision=fm.FMM_MIXED)
    assert ok
    i = np.arange(40) + 0.5
    z = 1 - 2 * i / 40
    ph = np.pi * (1 + 5 ** 0.5) * i
    pts = np.stack([np.sqrt(1 - z * z) * np.cos(ph), np.sqrt(1 - z * z) * np.sin(ph), z], axis=1)
    for p, f, xi in zip(plans, freqs, sc.split(x)):
        k = 2 * np.pi * f / 343.0
        assert rel(p.far_field(xi, pts), oracle.mie_rigid(k, 0.1, pts)) < 0.02, f
    sc.close()
    for p in plans:
        p.close()
