"""The admittance half of the adjoint path: fmm_vjp_admittance, the derivative of the far-field
objective J = sum |p_scat|^2 with respect to the surface admittance beta of a locally
reacting surface (b = i k beta, a = (1 + alpha b)/2), per element and for one admittance on the
whole surface; against central differences of the GPU pipeline and against a dense FP64
gradient (oracle operators, dense solves, beta varied per element).  Also the test-only
torch.autograd.Function that joins it with fmm_vjp, checked by torch.autograd.gradcheck."""
import numpy as np
import pytest

from test_gpu_vjp import DIR, generic_sphere

pytestmark = pytest.mark.gpu
BETA = 0.1 + 0.05j


def solve(fm, V, F, pts, k, beta, alpha, depth=2, p=16):
    b = 1j * k * beta
    plan = fm.Plan(V, F, k=k, depth=depth, p_levels={l: p for l in range(2, depth + 1)}, rule=fm.RULE_DUNAVANT7,
                   a=0.5 * (1 + alpha * b), b=b, c=-1.0, build_mixed=False, alpha=alpha)
    x, it, rr, ok = plan.gmres(plan.plane_wave(DIR), tol=1e-13, restart=80, maxit=2000, precision=fm.FMM_FP64)
    assert ok
    pf = plan.far_field(x, pts)
    return plan, x, pf, float(np.sum(np.abs(pf) ** 2))


@pytest.mark.parametrize("alpha_of_k", [0.0, 1.0])
def test_admittance_gradient_matches_central_differences(fm, alpha_of_k):
    k = 2 * np.pi * 2000 / 343.0
    alpha = alpha_of_k * 1j / k
    V, F = generic_sphere(fm, 2)
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = solve(fm, V, F, pts, k, BETA, alpha)
    _, lam = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    g, dj = plan.vjp_admittance(x, pts, pf, lam)
    plan.close()
    assert np.isfinite(g).all() and np.allclose(dj, [2 * g.sum().real, -2 * g.sum().imag])
    h = 1e-6
    fd = []
    for step in (h, 1j * h):
        Jp = solve(fm, V, F, pts, k, BETA + step, alpha)[3]
        Jm = solve(fm, V, F, pts, k, BETA - step, alpha)[3]
        fd.append((Jp - Jm) / (2 * h))
    scale = np.abs(fd).max()
    assert scale > 0
    assert np.abs(dj - np.array(fd)).max() <= 1e-4 * scale, (dj, fd)


def test_admittance_gradient_per_element_against_dense(fm, oracle):
    """Per element: the GPU gradient against the dense FP64 one of an admittance varied element
    by element, A(beta) = diag((1 + alpha b)/2) + S diag(b) - T, F(beta) = -L_far diag(b) + M_far
    (oracle matrices), and that dense gradient against central differences in three elements."""
    k = 2 * np.pi * 2000 / 343.0
    alpha = 1j / k
    V, F = generic_sphere(fm, 2)
    nf = len(F)
    pts = fm.fibonacci_sphere(32, 1.0)
    plan, x, pf, J = solve(fm, V, F, pts, k, BETA, alpha)
    _, lam = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
    g, _ = plan.vjp_admittance(x, pts, pf, lam)
    plan.close()

    S = oracle.dense_matrix(V, F, k, a=0.0, b=1.0, c=0.0, rule=1, alpha=alpha)
    T = oracle.dense_matrix(V, F, k, a=0.0, b=0.0, c=1.0, rule=1, alpha=alpha)
    eye = np.eye(nf)
    Lf = np.stack([oracle.far_field(V, F, k, eye[j], pts, rule=1, b=1.0, c=0.0) for j in range(nf)], axis=1)
    Mf = np.stack([oracle.far_field(V, F, k, eye[j], pts, rule=1, b=0.0, c=1.0) for j in range(nf)], axis=1)
    tri = V[F]
    c = tri[:, 0] + (2.0 / 3.0) * (0.5 * (tri[:, 1] + tri[:, 2]) - tri[:, 0])
    n = np.cross(tri[:, 0] - tri[:, 2], tri[:, 1] - tri[:, 2])
    n /= np.linalg.norm(n, axis=1)[:, None]
    d = np.array(DIR)
    rhs = np.exp(1j * k * (c @ d)) * (1 + alpha * 1j * k * (n @ d))

    def parts(beta_vec):
        b = 1j * k * beta_vec
        A = np.diag(0.5 * (1 + alpha * b)) + S * b[None, :] - T
        Fm = Lf * b[None, :] - Mf      # far field -(L (b p) + c M p) with c = -1
        return A, Fm

    def J_of(beta_vec):
        A, Fm = parts(beta_vec)
        return float(np.sum(np.abs(Fm @ np.linalg.solve(A, rhs)) ** 2))

    beta0 = np.full(nf, BETA)
    A, Fm = parts(beta0)
    xd = np.linalg.solve(A, rhs)
    pd = Fm @ xd
    assert np.linalg.norm(pd - pf) < 1e-4 * np.linalg.norm(pd)
    lamd = np.linalg.solve(A.conj().T, Fm.conj().T @ pd)
    # dJ = 2 Re[ pbar^H dF x - lambda^H dA x ], dF/db_j = Lf[:, j], dA/db_j = S[:, j] + alpha/2 e_j
    gb = xd * (Lf.T @ pd.conj()) - xd * (S.T @ lamd.conj()) - 0.5 * alpha * lamd.conj() * xd
    gd = 1j * k * gb
    assert np.abs(g - gd).max() <= 1e-4 * np.abs(gd).max()
    h = 1e-6
    for j in np.random.default_rng(9).choice(nf, 3, replace=False):
        for step, part in ((h, 0), (1j * h, 1)):
            bp, bm = beta0.copy(), beta0.copy()
            bp[j] += step
            bm[j] -= step
            fd = (J_of(bp) - J_of(bm)) / (2 * h)
            an = 2 * gd[j].real if part == 0 else -2 * gd[j].imag
            assert abs(an - fd) <= 1e-5 * 2 * np.abs(gd).max(), (j, part, an, fd)


def test_autograd_function_gradcheck(fm):
    """A torch.autograd.Function over the GPU pipeline (tests only): J(V, beta) forward; fmm_vjp
    and fmm_vjp_admittance backward.  torch.autograd.gradcheck on four parameters that move two
    seeded vertex fields and the real and imaginary admittance."""
    torch = pytest.importorskip("torch")
    k = 2 * np.pi * 2000 / 343.0
    alpha = 1j / k
    V0, F = generic_sphere(fm, 2)
    pts = fm.fibonacci_sphere(32, 1.0)

    class FarFieldObjective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, V, beta):
            bt = complex(beta[0].item(), beta[1].item())
            plan, x, pf, J = solve(fm, V.detach().cpu().numpy(), F, pts, k, bt, alpha)
            grad_v, lam = plan.vjp(x, pts, pf, direction=DIR, tol=1e-13)
            _, dj = plan.vjp_admittance(x, pts, pf, lam)
            plan.close()
            ctx.save_for_backward(torch.from_numpy(grad_v), torch.from_numpy(dj))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            grad_v, dj = ctx.saved_tensors
            return gJ * grad_v, gJ * dj

    rng = np.random.default_rng(17)
    # two vertex fields of unit size: a translation and a smooth bump; gradcheck's steps of 1e-6
    # move vertices by 1e-6 m, as the finite differences of the other gradient tests do
    e0, e1 = rng.standard_normal(3), rng.standard_normal(3)
    D0 = torch.from_numpy(np.tile(e0 / np.linalg.norm(e0), (len(V0), 1)))
    D1 = torch.from_numpy(np.outer(np.exp(-np.sum((V0 - V0[0]) ** 2, axis=1) / 0.05 ** 2), e1 / np.linalg.norm(e1)))
    V0t = torch.from_numpy(V0)

    def f(t):
        V = V0t + t[0] * D0 + t[1] * D1
        beta = torch.stack([BETA.real + t[2], BETA.imag + t[3]])
        return FarFieldObjective.apply(V, beta)

    t = torch.zeros(4, dtype=torch.float64, requires_grad=True)
    f(t).backward()
    scale = float(t.grad.abs().max())
    assert scale > 0
    # central differences at eps against the backward, within 1e-4 of the largest derivative (the
    # bound of the other gradient tests: the derivative holds the octree's box centres fixed while
    # the differences move them with the bounding cube)
    assert torch.autograd.gradcheck(f, (t,), eps=1e-6, atol=1e-4 * scale, rtol=0.0, check_undefined_grad=False)
