"""The oracle's Burton-Miller operator and locally reacting (admittance) surfaces: the
regularised hypersingular integrals against independent quadrature, the FMM oracle against
the dense operator, and dense solutions against Mie series.  CPU only."""
import os
import sys

import numpy as np
import pytest

import meshes

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_oracle_pins import _hyper_finite_part  # noqa: E402

K1 = 2 * np.pi * 1000 / 343.0


def _normals(V, F):
    n = np.cross(V[F[:, 0]] - V[F[:, 2]], V[F[:, 1]] - V[F[:, 2]])
    return n / np.linalg.norm(n, axis=1)[:, None]


def _fine_hyper(k, tri, x, nx, levels=6):
    """int_T d2G/dn_x dn_y at x off T by the 7-point rule on 4^levels sub-triangles."""
    from oracle import oracle_py

    Vt = tri.reshape(3, 3)
    bary, w = oracle_py.quad_rule(1)
    tris = [Vt]
    for _ in range(levels):
        new = []
        for t in tris:
            m01, m12, m20 = (t[0] + t[1]) / 2, (t[1] + t[2]) / 2, (t[2] + t[0]) / 2
            new += [np.array([t[0], m01, m20]), np.array([m01, t[1], m12]), np.array([m20, m12, t[2]]),
                    np.array([m01, m12, m20])]
        tris = new
    nT = np.cross(Vt[0] - Vt[2], Vt[1] - Vt[2])
    nT /= np.linalg.norm(nT)
    total = 0.0
    for t in tris:
        J = np.linalg.norm(np.cross(t[0] - t[2], t[1] - t[2]))
        d = bary @ t - x
        r = np.linalg.norm(d, axis=1)
        a1, a2 = (d @ nT) / r, -(d @ nx) / r
        e = np.exp(1j * k * r) / (4 * np.pi * r ** 3)
        total += J * (w @ (e * ((3 - k * k * r * r - 3j * k * r) * a1 * a2 + (1 - 1j * k * r) * (nT @ nx))))
    return total


def test_mie_impedance_reduces_to_rigid(oracle):
    pts = np.random.default_rng(0).standard_normal((20, 3))
    for k in (K1, 40.0):
        assert np.abs(oracle.mie_impedance(k, 0.1, 0.0, pts) - oracle.mie_rigid(k, 0.1, pts)).max() == 0.0


def test_regularised_hypersingular_integrals(oracle):
    """Self term: the polar finite part equals the independent polar quadrature.  Adjacent
    elements: the Maue form agrees with fine direct quadrature far better than the
    reference's 3x3 rule on the raw kernel does."""
    tri = np.array([0.05, 0.02, 0.01, -0.03, 0.06, 0.02, 0.01, -0.04, 0.07])
    V3 = tri.reshape(3, 3)
    c = V3.mean(axis=0)
    n = np.cross(V3[0] - V3[2], V3[1] - V3[2])
    n /= np.linalg.norm(n)
    for k in (0.01, 9.3, 146.55):
        fp = _hyper_finite_part(k, tri)
        assert abs(oracle.elem_hyper_maue(k, tri, c, n, sgl=True) - fp) < 1e-9 * abs(fp)
    V, F = meshes.icosphere(3, 0.1)
    N = _normals(V, F)
    C = V[F].mean(axis=1)
    adj = [j for j in range(1, len(F)) if set(F[j]) & set(F[0])]
    worst_maue = worst_raw = 0.0
    for j in adj:
        tri = V[F[j]].reshape(9)
        ref = _fine_hyper(K1, tri, C[0], N[0])
        worst_maue = max(worst_maue, abs(oracle.elem_hyper_maue(K1, tri, C[0], N[0], rule=1) - ref) / abs(ref))
        worst_raw = max(worst_raw, abs(oracle.elem_hyper(K1, tri, N[0], C[0]) - ref) / abs(ref))
    assert worst_maue < 3e-4
    assert worst_raw > 30 * worst_maue


@pytest.mark.parametrize("beta", [0.0, 0.5 - 0.3j])
def test_fmm_oracle_burton_miller_matches_dense(oracle, beta):
    V, F = meshes.roundtrip(*meshes.icosphere(3, 0.1))
    k = K1
    b = 1j * k * beta
    alpha = 1j / k
    a = 0.5 * (1 + alpha * b)
    T = oracle.tree_for_fmm(V, F, depth=3)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))
    y = rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))
    A = oracle.dense_matrix(V, F, k, a=a, b=b, c=-1.0, rule=1, alpha=alpha)
    assert np.allclose(A @ x, oracle.dense_apply(V, F, k, x, a=a, b=b, c=-1.0, rule=1, alpha=alpha), rtol=0, atol=1e-12)
    errs = []
    for p in (6, 14):
        f = oracle.FMM(V, F, k, T, [p, p], a=a, b=b, c=-1.0, rule=1, alpha=alpha)
        ax, aty = f.apply(x), f.apply(y, transpose=True)
        errs.append(np.linalg.norm(ax - A @ x) / np.linalg.norm(A @ x))
        assert np.linalg.norm(aty - A.T @ y) / np.linalg.norm(A.T @ y) < 3 * errs[-1]
        assert abs(y @ ax - x @ aty) < 1e-12 * np.linalg.norm(x) * np.linalg.norm(y) * np.linalg.norm(A, 2)
    assert errs[0] > errs[1] and errs[1] < 2e-6


def test_burton_miller_removes_the_fictitious_frequency(oracle):
    """At ka = pi (an interior Dirichlet eigenvalue of the sphere) the conventional operator
    is nearly singular; the combined one is not, and its solution matches Mie."""
    V, F = meshes.icosphere(3, 0.1)
    N = _normals(V, F)
    C = V[F].mean(axis=1)
    pts = np.random.default_rng(0).standard_normal((40, 3))
    pts /= np.linalg.norm(pts, axis=1)[:, None]
    k = np.pi / 0.1
    mie = oracle.mie_rigid(k, 0.1, pts)
    res = {}
    for name, alpha in (("cbie", 0.0), ("bm", 1j / k)):
        A = oracle.dense_matrix(V, F, k, a=0.5, b=0.0, c=-1.0, rule=1, alpha=alpha)
        rhs = np.exp(1j * k * C[:, 2]) * (1 + alpha * 1j * k * N[:, 2])
        x = np.linalg.solve(A, rhs)
        ff = oracle.far_field(V, F, k, x, pts, rule=1)
        res[name] = (np.linalg.svd(A, compute_uv=False)[-1], np.linalg.norm(ff - mie) / np.linalg.norm(mie))
    assert res["bm"][0] > 20 * res["cbie"][0]
    assert res["bm"][1] < 0.015 and res["cbie"][1] > 2 * res["bm"][1]


@pytest.mark.parametrize("alpha_scale", [0.0, 1.0])
def test_admittance_dense_solution_matches_mie(oracle, alpha_scale):
    """dp/dn = i k beta p: b = i k beta, the far field -(b L + c M) p against the impedance
    Mie series, with and without the Burton-Miller coupling."""
    V, F = meshes.icosphere(3, 0.1)
    N = _normals(V, F)
    C = V[F].mean(axis=1)
    pts = np.random.default_rng(1).standard_normal((40, 3))
    pts /= np.linalg.norm(pts, axis=1)[:, None]
    k, beta = K1, 0.5 - 0.3j
    b, alpha = 1j * k * beta, alpha_scale * 1j / K1
    A = oracle.dense_matrix(V, F, k, a=0.5 * (1 + alpha * b), b=b, c=-1.0, rule=1, alpha=alpha)
    x = np.linalg.solve(A, np.exp(1j * k * C[:, 2]) * (1 + alpha * 1j * k * N[:, 2]))
    ff = oracle.far_field(V, F, k, x, pts, rule=1, b=b, c=-1.0)
    mie = oracle.mie_impedance(k, 0.1, beta, pts)
    assert np.linalg.norm(ff - mie) / np.linalg.norm(mie) < 0.012
