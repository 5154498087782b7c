"""fmm_vjp: the vertex-position gradient of J = sum |p_scat|^2 at far points, against central
finite differences of the GPU pipeline (plan, solve, far field) and of the oracle's dense
operator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0
DIR = (0.0, 0.6, 0.8)


def generic_sphere(fm, subdiv):
    """An icosphere turned and shifted by a seeded rigid motion: on the symmetric mesh many
    centroids lie exactly on leaf-box faces (the coordinate planes of a centred bounding
    cube), and a +-h perturbation would move them between boxes and change the operator's
    near/far split between the two finite-difference evaluations."""
    V, F = fm.icosphere(subdiv, 0.1)
    q, _ = np.linalg.qr(np.random.default_rng(7).standard_normal((3, 3)))
    return V @ q.T + np.array([0.0123, -0.0071, 0.0045]), F


def pipeline(fm, V, F, pts, depth, p, b=0.0, k=K1, alpha=0.0):
    plan = fm.Plan(V, F, k=k, depth=depth, p_levels={l: p for l in range(2, depth + 1)}, rule=fm.RULE_DUNAVANT7,
                   a=0.5 * (1 + alpha * b), b=b, c=-1.0, build_mixed=False, alpha=alpha)
    b = plan.plane_wave(DIR)
    x, it, rr, ok = plan.gmres(b, tol=1e-13, restart=80, maxit=2000, precision=fm.FMM_FP64)
    assert ok
    pf = plan.far_field(x, pts)
    return plan, x, pf, float(np.sum(np.abs(pf) ** 2))


@pytest.mark.parametrize("subdiv,depth,p", [(2, 2, 16), (3, 3, 14)])
def test_vjp_matches_central_differences(fm, subdiv, depth, p):
    V, F = generic_sphere(fm, subdiv)
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = pipeline(fm, V, F, pts, depth, p)
    assert plan.info.num_m2l[2] > 0  # far pairs go through the FMM branch of the gradient
    grad, lam = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    plan.close()
    assert np.isfinite(grad).all() and np.abs(grad).max() > 0
    rng = np.random.default_rng(11)
    verts = rng.choice(len(V), 20, replace=False)
    h = 1e-6
    scale = np.abs(grad).max()
    for v in verts:
        e = rng.standard_normal(3)
        e /= np.linalg.norm(e)
        Vp, Vm = V.copy(), V.copy()
        Vp[v] += h * e
        Vm[v] -= h * e
        fd = (pipeline(fm, Vp, F, pts, depth, p)[3] - pipeline(fm, Vm, F, pts, depth, p)[3]) / (2 * h)
        # the gradient holds the box centres fixed while the differences move them with the
        # bounding cube; at these orders that leaves < 1e-6 of the largest component
        assert abs(grad[v] @ e - fd) <= 1e-4 * scale, (v, grad[v] @ e, fd)


def test_vjp_against_dense_oracle_differences(fm, oracle):
    """The same gradient against central differences of J computed with the oracle's dense
    operator and a dense FP64 solve (no FMM anywhere)."""
    V, F = generic_sphere(fm, 2)
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = pipeline(fm, V, F, pts, 2, 16)
    grad, _ = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    plan.close()
    d = np.array(DIR)

    def J_dense(Vx):
        A = oracle.dense_matrix(Vx, F, K1, a=0.5, b=0.0, c=-1.0, rule=1)
        tri = Vx[F]
        c = tri[:, 0] + (2.0 / 3.0) * (0.5 * (tri[:, 1] + tri[:, 2]) - tri[:, 0])
        xs = np.linalg.solve(A, np.exp(1j * K1 * (c @ d)))
        return float(np.sum(np.abs(oracle.far_field(Vx, F, K1, xs, pts, rule=1)) ** 2))

    assert abs(J_dense(V) - np.sum(np.abs(pf) ** 2)) < 1e-5 * np.sum(np.abs(pf) ** 2)
    rng = np.random.default_rng(3)
    h = 1e-6
    scale = np.abs(grad).max()
    for v in rng.choice(len(V), 6, replace=False):
        for a in range(3):
            Vp, Vm = V.copy(), V.copy()
            Vp[v, a] += h
            Vm[v, a] -= h
            fd = (J_dense(Vp) - J_dense(Vm)) / (2 * h)
            assert abs(grad[v, a] - fd) <= 1e-4 * scale, (v, a, grad[v, a], fd)


def test_vjp_with_admittance_boundary(fm):
    """An admittance (Robin) boundary beta = 0.1 + 0.05i on a bumped ellipsoid at 3 kHz: the
    operator gains the single layer, b = i k beta, so the gradient's single-layer branches
    (singular self terms, near G, the far phi J term) enter; against central differences."""
    k = 2 * np.pi * 3000 / 343.0
    b = 1j * k * (0.1 + 0.05j)
    V, F = fm.ellipsoid(6, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=1)
    V = V + np.array([0.0031, -0.0017, 0.0023])  # off the centred cube's symmetry planes
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = pipeline(fm, V, F, pts, 3, 16, b=b, k=k)
    assert plan.info.num_m2l[2] > 0
    grad, _ = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    plan.close()
    rng = np.random.default_rng(12)
    h = 1e-6
    scale = np.abs(grad).max()
    for v in rng.choice(len(V), 12, replace=False):
        e = rng.standard_normal(3)
        e /= np.linalg.norm(e)
        Vp, Vm = V.copy(), V.copy()
        Vp[v] += h * e
        Vm[v] -= h * e
        fd = (pipeline(fm, Vp, F, pts, 3, 16, b=b, k=k)[3] - pipeline(fm, Vm, F, pts, 3, 16, b=b, k=k)[3]) / (2 * h)
        assert abs(grad[v] @ e - fd) <= 1e-4 * scale, (v, grad[v] @ e, fd)


@pytest.mark.parametrize("beta", [0.0, 0.1 + 0.05j])
def test_vjp_with_burton_miller(fm, beta):
    """The Burton-Miller operator (alpha = i/k): the gradient gains the hypersingular and
    normal-derivative near terms (both elements' vertices), the target-side normal derivative
    of the far field and the alpha dp_inc/dn term of the right-hand side; against central
    differences of the GPU pipeline, rigid and with an admittance boundary."""
    k = 2 * np.pi * 2000 / 343.0
    b, alpha = 1j * k * beta, 1j / k
    V, F = generic_sphere(fm, 2)
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = pipeline(fm, V, F, pts, 2, 16, b=b, k=k, alpha=alpha)
    assert plan.info.num_m2l[2] > 0
    grad, _ = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    plan.close()
    assert np.isfinite(grad).all()
    rng = np.random.default_rng(21)
    h = 1e-6
    scale = np.abs(grad).max()
    for v in rng.choice(len(V), 12, replace=False):
        e = rng.standard_normal(3)
        e /= np.linalg.norm(e)
        Vp, Vm = V.copy(), V.copy()
        Vp[v] += h * e
        Vm[v] -= h * e
        fd = (pipeline(fm, Vp, F, pts, 2, 16, b=b, k=k, alpha=alpha)[3]
              - pipeline(fm, Vm, F, pts, 2, 16, b=b, k=k, alpha=alpha)[3]) / (2 * h)
        assert abs(grad[v] @ e - fd) <= 1e-4 * scale, (v, grad[v] @ e, fd)


def test_vjp_burton_miller_against_dense_oracle_differences(fm, oracle):
    """The Burton-Miller gradient against central differences of J with the oracle's dense
    combined operator and a dense FP64 solve."""
    k = 2 * np.pi * 2000 / 343.0
    alpha = 1j / k
    V, F = generic_sphere(fm, 2)
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = pipeline(fm, V, F, pts, 2, 16, k=k, alpha=alpha)
    grad, _ = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    plan.close()
    d = np.array(DIR)

    def J_dense(Vx):
        A = oracle.dense_matrix(Vx, F, k, a=0.5, b=0.0, c=-1.0, rule=1, alpha=alpha)
        tri = Vx[F]
        c = tri[:, 0] + (2.0 / 3.0) * (0.5 * (tri[:, 1] + tri[:, 2]) - tri[:, 0])
        n = np.cross(tri[:, 0] - tri[:, 2], tri[:, 1] - tri[:, 2])
        n /= np.linalg.norm(n, axis=1)[:, None]
        rhs = np.exp(1j * k * (c @ d)) * (1 + alpha * 1j * k * (n @ d))
        xs = np.linalg.solve(A, rhs)
        return float(np.sum(np.abs(oracle.far_field(Vx, F, k, xs, pts, rule=1)) ** 2))

    assert abs(J_dense(V) - J) < 1e-4 * J
    rng = np.random.default_rng(4)
    h = 1e-6
    scale = np.abs(grad).max()
    for v in rng.choice(len(V), 5, replace=False):
        for a in range(3):
            Vp, Vm = V.copy(), V.copy()
            Vp[v, a] += h
            Vm[v, a] -= h
            fd = (J_dense(Vp) - J_dense(Vm)) / (2 * h)
            assert abs(grad[v, a] - fd) <= 2e-4 * scale, (v, a, grad[v, a], fd)
