"""Many independent bodies solved concurrently (fmm_solve_many): spheres, bumped ellipsoids
and boxes of different sizes and frequencies, one plane wave each, against one solve after
another; the first sphere against the Mie series."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DIR = np.array([0.0, 0.6, 0.8])


def scene(fm, n=10, seed=5):
    rng = np.random.default_rng(seed)
    bodies = []
    for i in range(n):
        kind = i % 3
        if kind == 0:
            V, F = fm.geodesic_sphere(int(rng.integers(10, 16)), rng.uniform(0.03, 0.1))
        elif kind == 1:
            ax = rng.uniform(0.02, 0.1, 3)
            V, F = fm.ellipsoid(int(rng.integers(6, 14)), ax, lmax=8, sigma=0.03 * ax.min(),
                                seed=int(rng.integers(1 << 30)))
        else:
            V, F = fm.box(int(rng.integers(4, 12)), rng.uniform(0.01, 0.1, 3))
        bodies.append((V, F, 2 * np.pi * rng.uniform(500.0, 10000.0) / 343.0))
    return bodies


def test_solve_many_matches_sequential_solves(fm, oracle):
    bodies = scene(fm)
    plans, rhs = [], []
    for V, F, k in bodies:
        plan = fm.Plan(V, F, k=k, s=5, rule=fm.RULE_DUNAVANT7, a=0.5, b=0.0, c=-1.0)
        plans.append(plan)
        rhs.append(plan.plane_wave(DIR))
    t0 = time.perf_counter()
    xs, it, rr, st = fm.solve_many(plans, rhs, tol=1e-6, restart=60, precision=fm.FMM_MIXED, nthreads=4)
    t_conc = time.perf_counter() - t0
    assert (st == 0).all() and (rr <= 1e-6).all() and (it > 0).all()
    t0 = time.perf_counter()
    for i, plan in enumerate(plans):
        prec = fm.FMM_MIXED if max(plan.info.m2l_columns) > 0 else fm.FMM_FP64
        x, _, r, ok = plan.gmres(rhs[i], tol=1e-6, restart=60, precision=prec)
        assert ok and np.linalg.norm(x - xs[i]) <= 1e-5 * np.linalg.norm(x)
    t_seq = time.perf_counter() - t0
    print("bodies %d: concurrent %.3f s, sequential %.3f s" % (len(plans), t_conc, t_seq))
    # the first body is a sphere: its scattered field against the Mie series, evaluated in a
    # frame whose third axis is the incident direction (the series is for exp(ikz))
    V, F, k = bodies[0]
    r = np.linalg.norm(V, axis=1).mean()
    pts = fm.fibonacci_sphere(64, 1.0)
    ff = plans[0].far_field(xs[0], pts)
    e1 = np.array([1.0, 0.0, 0.0])
    e2 = np.cross(DIR, e1)
    local = np.stack([pts @ e1, pts @ e2, pts @ DIR], axis=1)
    assert np.linalg.norm(ff - oracle.mie_rigid(k, r, local)) / np.linalg.norm(ff) < 0.03
    for p in plans:
        p.close()


def test_solve_many_rejects_repeated_plans(fm):
    V, F = fm.geodesic_sphere(4, 0.05)
    plan = fm.Plan(V, F, k=10.0, depth=2, p_levels={2: 6}, a=0.5, b=0.0, c=-1.0)
    b = plan.plane_wave((0.0, 0.0, 1.0))
    with pytest.raises(fm.FmmError):
        fm.solve_many([plan, plan], [b, b])
    plan.close()
