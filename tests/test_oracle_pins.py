"""Pin the oracle against the reference's own outputs (tests/golden) and against analytic
identities.  CPU only."""
import hashlib
import json
import os
import warnings

import numpy as np
import pytest

import meshes
from oracle import octree_oracle as oo

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
META = json.load(open(os.path.join(GOLDEN, "octree_meta.json")))


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def _oracle_tree(case):
    m = META[case]
    V, F = meshes.roundtrip(*meshes.icosphere(m["subdiv"], m["radius"]))
    T = oo.build(V, F, s=m["s"], depth=m["depth"] or None)
    return V, F, T


@pytest.mark.parametrize("case", sorted(META))
def test_octree_matches_reference(case):
    """Level sets, interaction lists and element-to-box indices equal the reference's."""
    g = dict(np.load(os.path.join(GOLDEN, "octree_%s.npz" % case)))
    m = META[case]
    V, F, T = _oracle_tree(case)
    lmax = T["lmax"]
    assert lmax == int(g["lmax"])
    assert T["d"] == float(g["d"])
    assert np.array_equal(T["pt_min"], g["pt_min"])
    out = {"btm_idx": oo.btm_lvl_elem_idx(V, F, T["pt_min"], T["d"], T["level_sets"][-1], lmax).astype(np.int32)}
    for l in range(2, lmax + 1):
        assert np.array_equal(T["level_sets"][l - 2], g["set_%d" % l]), "level %d set" % l
    sr = oo.sr_lists(T["level_sets"], lmax)
    ss = oo.ss_rr_lists(T["level_sets"], lmax)
    for l in range(2, lmax + 1):
        num, org, dst = sr[l - 2]
        out["srnum_%d" % l] = num.astype(np.int32)
        out["sr_origin_%d" % l] = org.astype(np.int32)
        out["sr_dest_%d" % l] = dst.astype(np.int32)
        if l > 2:
            out["ss_dest_%d" % l] = ss[l].astype(np.int32)
            out["rr_origin_%d" % l] = ss[l].astype(np.int32)
    for key, val in out.items():
        if key in g:
            assert np.array_equal(val, g[key]), key
        else:
            assert digest(val) == m["sha256"][key], key


@pytest.mark.parametrize("case", ["ico2_r0.1_s5", "ico3_r0.1_s5", "ico3_r0.1_d3", "ico4_r0.3_s5", "ico5_r0.3_d5"])
def test_near_lists_match_reference(case):
    """Leaf near lists I2 ∩ leaf set, in I2's order (the box itself last), equal the reference's."""
    near = np.load(os.path.join(GOLDEN, "octree_near.npz"))
    nmeta = json.load(open(os.path.join(GOLDEN, "octree_near_meta.json")))
    V, F, T = _oracle_tree(case)
    nl = oo.near_lists(T["level_sets"], T["lmax"])
    beg = np.concatenate([[0], np.cumsum([len(x) for x in nl])]).astype(np.int32)
    idx = np.concatenate([np.asarray(x) for x in nl]).astype(np.int32)
    if case + "_beg" in near.files:
        assert np.array_equal(beg, near[case + "_beg"]) and np.array_equal(idx, near[case + "_idx"])
    else:
        assert digest(beg) == nmeta[case]["beg"] and digest(idx) == nmeta[case]["idx"]
    assert all(x[-1] == i for i, x in enumerate(nl))


def test_quadrature_and_green_vs_reference(oracle):
    """Element integrals of G and dG/dn (regular and singular) against the reference's FP32."""
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    tris, ys, ks = q["tris"].astype(np.float64), q["ys"].astype(np.float64), q["ks"]
    for a, k in enumerate(ks):
        kf = float(np.float32(k))
        for b in range(len(tris)):
            for sgl in (0, 1):
                for kind, ref in (("G", q["G"]), ("dG", q["dG"])):
                    mine = oracle.elem_integral(kind, kf, tris[b], ys[b], rule=0, sgl=bool(sgl))
                    r = complex(*ref[a, b, sgl])
                    scale = max(abs(r), abs(oracle.elem_integral("G", kf, tris[b], ys[b], rule=0, sgl=bool(sgl))))
                    # the reference's FP32 phase k*r carries ~ulp(k r) absolute error
                    kr = kf * (np.linalg.norm(tris[b].reshape(3, 3) - ys[b], axis=1).max())
                    tol = 3e-7 * max(30.0, kr)
                    if kind == "dG" and sgl:
                        # flat element: (x - y).n = 0, the self term vanishes; the
                        # reference returns FP32 rounding noise
                        assert abs(mine) < 1e-13 and abs(r) < 1e-5
                        continue
                    assert abs(mine - r) <= tol * scale + 1e-9, (kind, a, b, sgl, mine, r)


def test_p2m_moments_vs_reference(oracle):
    """P2M moments int R_n^{-m} and int dR_n^{-m}/dn (triElemIntegral_R / pRpn)."""
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    tris, mom = q["tris"].astype(np.float64), q["moments"]
    ctr = q["moment_ctr"].astype(np.float64)
    k = float(np.float32(q["moment_k"]))
    for b in range(1, len(tris)):
        for deriv in (0, 1):
            mine = oracle.elem_moments(k, tris[b], ctr, 6, rule=0, deriv=bool(deriv))
            ref = mom[b, deriv, :, 0] + 1j * mom[b, deriv, :, 1]
            assert np.linalg.norm(mine - ref) <= 1e-5 * np.linalg.norm(ref), (b, deriv)


def test_normal_y_and_hypersingular_integrals_vs_reference(oracle):
    """int dG/dn_y and int d2G/dn_x dn_y (triElemIntegral_pGp2n_* / p2Gp1np2n_*, regular and
    self term) and dirDev_R against the reference's FP32 outputs."""
    g = np.load(os.path.join(GOLDEN, "integral_ext.npz"))
    tris, ys, nr = g["tris"].astype(np.float64), g["ys"].astype(np.float64), g["nrmls"].astype(np.float64)
    for a, k in enumerate(g["ks"]):
        kf = float(np.float32(k))
        for b in range(len(tris)):
            kr = kf * np.linalg.norm(tris[b].reshape(3, 3) - ys[b], axis=1).max()
            tol = 3e-7 * max(30.0, kr)
            for sgl in (0, 1):
                r = complex(*g["hyper"][a, b, sgl])
                mine = oracle.elem_hyper(kf, tris[b], nr[b], ys[b], sgl=bool(sgl))
                assert abs(mine - r) <= tol * abs(r), (a, b, sgl, mine, r)
            r = complex(*g["dGdny"][a, b, 0])
            assert abs(oracle.elem_dGdny(kf, tris[b], nr[b], ys[b]) - r) <= tol * abs(r)
            # flat element: (y - x).n = 0 on every sub-triangle; the reference returns FP32 noise
            assert abs(oracle.elem_dGdny(kf, tris[b], sgl=True)) < 1e-13 and abs(complex(*g["dGdny"][a, b, 1])) < 1e-5
    kd = float(np.float32(g["dirdev_k"]))
    for i, x in enumerate(g["dirdev_x"].astype(np.float64)):
        ref = g["dirdev"][i, :, 0] + 1j * g["dirdev"][i, :, 1]
        mine = np.array([oracle.dirdev_R(kd, n, m, nr[i], x) for n in range(6) for m in range(-n, n + 1)])
        assert np.abs(mine - ref).max() <= 2e-6 * np.abs(ref).max()


def test_normal_derivative_integrals_are_derivatives(oracle):
    """The regular integrals of dG/dn_y and d2G/dn_x dn_y are the y-derivatives along n_y of the
    integrals of G and dG/dn_x with the same rule; dirDev_R is the derivative of R_n^m."""
    rng = np.random.default_rng(11)
    tri = np.array([0.1, 0.0, 0.0, 0.0, 0.12, 0.0, 0.0, 0.0, 0.09])
    y = np.array([0.3, 0.2, -0.1])
    n = rng.standard_normal(3)
    n /= np.linalg.norm(n)
    k, h = 18.32, 1e-5
    fd_G = (oracle.elem_integral("G", k, tri, y + h * n) - oracle.elem_integral("G", k, tri, y - h * n)) / (2 * h)
    assert abs(oracle.elem_dGdny(k, tri, n, y) - fd_G) < 1e-7 * abs(fd_G)
    fd_dG = (oracle.elem_integral("dG", k, tri, y + h * n) - oracle.elem_integral("dG", k, tri, y - h * n)) / (2 * h)
    assert abs(oracle.elem_hyper(k, tri, n, y) - fd_dG) < 1e-7 * abs(fd_dG)
    x = np.array([0.05, -0.02, 0.03])
    for nn in range(5):
        for m in range(-nn, nn + 1):
            f = lambda v: oracle.basis(nn + 1, k, v)[nn * nn + nn + m]
            fd = (f(x + h * n) - f(x - h * n)) / (2 * h)
            assert abs(oracle.dirdev_R(k, nn, m, n, x) - fd) < 1e-7 * max(1.0, abs(fd)), (nn, m)


def _hyper_finite_part(k, tri, off=0.0):
    """int_T d2G/dn_x dn_y at the centroid c (off = 0: Hadamard finite part) or at c + off n
    (n = n_y = n_x), by polar integration about c: adaptive in r, Gauss in theta between the
    vertex angles.  Independent of the oracle's code."""
    from scipy.integrate import quad

    V = tri.reshape(3, 3)
    nrm = np.cross(V[0] - V[2], V[1] - V[2])
    nrm /= np.linalg.norm(nrm)
    c = V.mean(axis=0)
    e1 = (V[0] - c) / np.linalg.norm(V[0] - c)
    e2 = np.cross(nrm, e1)
    P = [(np.dot(v - c, e1), np.dot(v - c, e2)) for v in V]
    ang = [np.arctan2(py, px) % (2 * np.pi) for px, py in P]
    ang[0] = 0.0
    cuts = sorted(ang) + [2 * np.pi]
    t, w = np.polynomial.legendre.leggauss(48)

    def rho(th):
        u = np.array([np.cos(th), np.sin(th)])
        best = np.inf
        for i in range(3):
            A, B = np.array(P[i]), np.array(P[(i + 1) % 3])
            d = B - A
            den = u[0] * d[1] - u[1] * d[0]
            if abs(den) < 1e-300:
                continue
            tt = (A[0] * d[1] - A[1] * d[0]) / den
            s = ((tt * u - A) @ d) / (d @ d)
            if tt > 0 and -1e-12 <= s <= 1 + 1e-12:
                best = min(best, tt)
        return best

    h = off

    def radial(R):
        if h == 0.0:
            # finite part of int_0^R e^{ikr}(1 - ikr)/(4 pi r^2) dr = [-e^{ikr}/(4 pi r)]: drop the 1/r pole
            return (-np.exp(1j * k * R) / R + 1j * k) / (4 * np.pi)
        top = np.sqrt(R * R + h * h)

        def f(r):
            return np.exp(1j * k * r) / (4 * np.pi * r * r) * ((1 - 1j * k * r) - (3 - 3j * k * r - k * k * r * r) * h * h / (r * r))
        with warnings.catch_warnings():
            # quad reports roundoff when it reaches 1e-12; that is far below what the test needs
            warnings.simplefilter("ignore")
            re = quad(lambda r: f(r).real, h, top, limit=200, epsabs=0, epsrel=1e-12, points=[min(10 * h, top)])[0]
            im = quad(lambda r: f(r).imag, h, top, limit=200, epsabs=0, epsrel=1e-12, points=[min(10 * h, top)])[0]
        return re + 1j * im

    total = 0.0
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        th = 0.5 * (hi - lo) * t + 0.5 * (hi + lo)
        total += 0.5 * (hi - lo) * sum(wi * radial(rho(x)) for wi, x in zip(w, th))
    return total


def test_hypersingular_self_term_is_the_finite_part(oracle):
    """The self term of d2G/dn_x dn_y is the limit of the regular integral as y approaches the
    centroid along the normal (the normal derivative of the double layer is continuous), and
    the oracle's polar rule converges to it."""
    pytest.importorskip("scipy")
    tri = np.array([0.05, 0.02, 0.01, -0.03, 0.06, 0.02, 0.01, -0.04, 0.07])
    for k in (9.3, 146.55):
        fp = _hyper_finite_part(k, tri)
        near = _hyper_finite_part(k, tri, off=1e-7)
        assert abs(near - fp) < 1e-4 * abs(fp), (k, near, fp)
        assert abs(oracle.elem_hyper(k, tri, sgl=True, nth=512) - fp) < 1e-4 * abs(fp)


def test_truncnum_vs_reference(oracle):
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    for k, eps, sig, a, p in q["truncnum"]:
        assert oracle.truncnum(k, eps, sig, a) == int(p)


def test_rotation_matrices_vs_reference(oracle):
    """Sparse rotation matrices (rotMatsInit + sparseRotMatGen, FP32) against the oracle's
    Wigner-based FP64 coefficients."""
    g = np.load(os.path.join(GOLDEN, "tables_rot.npz"))
    for key in g.files:
        a, b, c, p = key.split("_")
        a, b, c, p = float(np.float32(a)), float(np.float32(b)), float(np.float32(c)), int(p)
        ref = g[key][0::2] + 1j * g[key][1::2]
        mine = oracle.rot_matrix(a, b, c, p)
        if p <= 8:
            assert np.max(np.abs(mine - ref)) < 5e-5, key
        else:
            # the reference's FP32 recurrence has drifted by p = 12 (entries off by ~1e-3)
            assert np.max(np.abs(mine - ref)) > 1e-4, key


def _rot_blocks(H, p):
    off = 0
    for n in range(p):
        w = 2 * n + 1
        yield H[off:off + w * w].reshape(w, w, order="F")
        off += w * w


def test_reference_rotation_recurrence_is_unstable(oracle):
    """The reference's H recurrence (translation.cu:1179-1204) loses orthogonality as p grows
    even in FP64, while the Wigner-d evaluation stays orthogonal to rounding at p = 40."""
    beta = 0.9553166181245093
    worst = lambda H, p: max(np.max(np.abs(B @ B.T - np.eye(len(B)))) for B in _rot_blocks(H, p))
    assert worst(oracle.rot_H(beta, 40), 40) < 1e-12
    assert worst(oracle.rot_H(beta, 20, recur=True), 20) > 1e-8
    assert worst(oracle.rot_H(beta, 10, recur=True), 10) < 1e-11


def test_coaxial_matrices_vs_reference(oracle):
    """Sparse coaxial matrices (S|R), (R|R) against the reference's FP32 generator."""
    g = np.load(os.path.join(GOLDEN, "tables_coax.npz"))
    for key in g.files:
        k, t, p, sr = key.split("_")
        k, t, p, sr = float(np.float32(k)), float(np.float32(t)), int(p), int(sr)
        ref = g[key][0::2] + 1j * g[key][1::2]
        mine = oracle.coax(k, t, p, bool(sr))
        assert np.linalg.norm(mine - ref) <= 1e-4 * np.linalg.norm(ref), key


def test_wigner_rotation_equals_reference_recurrence(oracle):
    """Where the reference's H recurrence is accurate (p <= 10) the stable Wigner form agrees."""
    for beta in (0.1, 0.9553166181245093, 2.2, 3.0):
        a = oracle.rot_H(beta, 10)
        b = oracle.rot_H(beta, 10, recur=True)
        assert np.max(np.abs(a - b)) < 1e-11


@pytest.mark.parametrize("p,off,k,box", [(12, (2, 1, 0), 18.32, 0.05), (40, (3, 2, 1), 146.55, 0.15),
                                          (30, (2, 0, 2), 146.55, 0.075)])
def test_rcr_translation_addition_theorem(oracle, p, off, k, box):
    """Multipole of a point source, RCR-translated to a local expansion, equals G directly."""
    rng = np.random.default_rng(3)
    cs = np.zeros(3)
    cd = np.array(off, float) * box
    y0 = rng.uniform(-0.4, 0.4, 3) * box
    x = cd + rng.uniform(-0.4, 0.4, 3) * box
    R = oracle.basis(p, k, y0 - cs)
    C = np.zeros(p * p, complex)
    for n in range(p):
        for m in range(-n, n + 1):
            C[n * n + n + m] = 1j * k * R[n * n + n - m]
    D = oracle.rcr(k, cd - cs, p, True, C)
    loc = np.sum(D * oracle.basis(p, k, x - cd))
    r = np.linalg.norm(x - y0)
    direct = np.exp(1j * k * r) / (4 * np.pi * r)
    assert abs(loc - direct) < 1e-9 * abs(direct) + (1e-6 if p == 12 else 0)


def _coax_rr_mp(x, p, dps=60):
    """The coaxial (R|R) recurrence (translation.cu:678-771) in 60-digit arithmetic, entry
    (m, n', n) -> value; exact enough to check the FP64 tables in both triangles."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = dps

    def aC(n, m):
        return mp.sqrt(mp.mpf(n + 1 + m) * (n + 1 - m) / ((2 * n + 1) * (2 * n + 3))) if n >= abs(m) else mp.mpf(0)

    def bC(n, m):
        if 0 <= m <= n:
            return mp.sqrt(mp.mpf(n - m - 1) * (n - m) / ((2 * n - 1) * (2 * n + 1)))
        if -n <= m < 0:
            return -mp.sqrt(mp.mpf(n - m - 1) * (n - m) / ((2 * n - 1) * (2 * n + 1)))
        return mp.mpf(0)

    x = mp.mpf(x)
    E = {}
    for q in range(2 * p - 1):
        E[0, q, 0] = (-1) ** q * mp.sqrt(2 * q + 1) * mp.sqrt(mp.pi / (2 * x)) * mp.besselj(q + mp.mpf(1) / 2, x)
    for m in range(p - 1):
        for q in range(m + 1, 2 * p - 2 - m):
            E[m + 1, q, m + 1] = (bC(q, -m - 1) * E[m, q - 1, m] - bC(q + 1, m) * E[m, q + 1, m]) / bC(m + 1, -m - 1)
    for m in range(p - 1):
        for n in range(m, p - 1):
            for q in range(m, 2 * p - 2 - n):
                e0 = E[m, q - 1, n] if q - 1 >= m else 0
                e2 = E[m, q, n - 1] if n - 1 >= m else 0
                E[m, q, n + 1] = (aC(q - 1, m) * e0 - aC(q, m) * E[m, q + 1, n] + aC(n - 1, m) * e2) / aC(n, m)
    return E


@pytest.mark.parametrize("kt", [2.0, 0.05])
def test_rr_coaxial_tables_accurate_in_both_triangles(oracle, kt):
    """(R|R) at small k t: the entries below the diagonal come from the exact symmetry
    (R|R)_{n'n} = (-1)^{n+n'} (R|R)_{nn'}; the plain recurrence loses them (1e13 relative
    error at kt = 0.05), which broke L2L at low frequency."""
    p = 12
    E = _coax_rr_mp(kt, p)
    C = oracle.coax(kt, 1.0, p, False)
    worst = 0.0
    for m in range(p):
        off = m * (2 * m * m - (3 + 6 * p) * m + 1 + 6 * (p + p * p)) // 6
        for q in range(m, p):
            for n in range(m, p):
                ex = float(E[m, q, n])
                worst = max(worst, abs(C[off + (q - m) + (n - m) * (p - m)].real - ex) / abs(ex))
    assert worst < 1e-13


@pytest.mark.parametrize("k", [20.0, 1.0, 0.2])
def test_m2l_then_l2l_accurate_at_low_frequency(oracle, k):
    """A point source's multipole, (S|R) to a well-separated box, then (R|R) to a child box,
    evaluated at a target: equals G to 1e-9 down to k t = 0.009 (p = 14)."""
    p, box = 14, 0.02
    rng = np.random.default_rng(3)
    cs, cd = np.zeros(3), np.array([2.0, 1.0, 0.0]) * box
    y0 = rng.uniform(-0.4, 0.4, 3) * box
    x = cd + rng.uniform(-0.4, 0.4, 3) * box
    R = oracle.basis(p, k, y0 - cs)
    C = np.array([1j * k * R[n * n + n - m] for n in range(p) for m in range(-n, n + 1)])
    D = oracle.rcr(k, cd - cs, p, True, C)
    cc = cd + 0.25 * box * np.array([1, -1, 1])
    D2 = oracle.rcr(k, cc - cd, p, False, D)
    r = np.linalg.norm(x - y0)
    direct = np.exp(1j * k * r) / (4 * np.pi * r)
    assert abs(np.sum(D2 * oracle.basis(p, k, x - cc)) - direct) < 1e-9 * abs(direct)


def test_fmm_oracle_converges_to_dense(oracle):
    """FMM oracle vs the dense direct-quadrature operator on the 1280-triangle sphere."""
    V, F = meshes.roundtrip(*meshes.icosphere(3, 0.1))
    k = 2 * np.pi * 1000 / 343.0
    T = oracle.tree_for_fmm(V, F, depth=3)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))
    yd = oracle.dense_apply(V, F, k, x, a=0.5, c=-1.0, rule=1, b=0.0)
    errs = []
    for p in (6, 10, 14):
        y = oracle.FMM(V, F, k, T, [p, p], a=0.5, b=0.0, c=-1.0, rule=1).apply(x)
        errs.append(np.linalg.norm(y - yd) / np.linalg.norm(yd))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 2e-6


def test_transposed_fmm_oracle_matches_dense_transpose(oracle):
    """The oracle's transposed FMM (no reference counterpart) against the transpose of the
    dense operator, to the forward FMM's accuracy, and the bilinear identity."""
    V, F = meshes.roundtrip(*meshes.icosphere(3, 0.1))
    k = 2 * np.pi * 1000 / 343.0
    T = oracle.tree_for_fmm(V, F, depth=3)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))
    y = rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))
    A = oracle.dense_matrix(V, F, k, a=0.3, b=0.7 + 0.2j, c=-1.0, rule=0)
    assert np.allclose(A @ x, oracle.dense_apply(V, F, k, x, a=0.3, b=0.7 + 0.2j, c=-1.0, rule=0), rtol=0, atol=1e-13)
    f = oracle.FMM(V, F, k, T, [12, 12], a=0.3, b=0.7 + 0.2j, c=-1.0, rule=0)
    ax, aty = f.apply(x), f.apply(y, transpose=True)
    fwd = np.linalg.norm(ax - A @ x) / np.linalg.norm(A @ x)
    assert fwd < 1e-5
    assert np.linalg.norm(aty - A.T @ y) / np.linalg.norm(A.T @ y) < 3 * fwd
    assert abs(y @ ax - x @ aty) < 1e-9 * np.linalg.norm(x) * np.linalg.norm(y) * np.linalg.norm(A, 2)


def test_bem_dense_solution_matches_mie(oracle):
    """Rigid sphere (ka = 0.9): dense BEM solve of (1/2 - M) p = p_inc, far field vs Mie."""
    V, F = meshes.roundtrip(*meshes.icosphere(3, 0.1))
    k = 9.0
    n = len(F)
    A = np.zeros((n, n), complex)
    for j in range(n):
        e = np.zeros(n, complex)
        e[j] = 1.0
        A[:, j] = oracle.dense_apply(V, F, k, e, a=0.5, b=0.0, c=-1.0, rule=1)
    C = oo.tri_centroids(V, F)
    rhs = np.exp(1j * k * C[:, 2])
    p = np.linalg.solve(A, rhs)
    pts = meshes.fibonacci_sphere(50, 1.0)
    ff = oracle.far_field(V, F, k, p, pts, rule=1)
    mie = oracle.mie_rigid(k, 0.1, pts)
    assert np.linalg.norm(ff - mie) / np.linalg.norm(mie) < 0.03


def test_gsl_shim_against_scipy():
    """The project-written GSL stand-in used to build the reference oracle (only where built)."""
    import ctypes
    from scipy.special import lpmv, spherical_jn, spherical_yn
    from oracle import build as ob

    if not os.path.exists(ob.REF_LIB):
        pytest.skip("reference oracle not built on this machine")
    L = ctypes.CDLL(ob.REF_LIB)
    for name in ("gsl_sf_bessel_jl", "gsl_sf_bessel_yl"):
        getattr(L, name).restype = ctypes.c_double
        getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_double]
    L.gsl_sf_legendre_Plm.restype = ctypes.c_double
    L.gsl_sf_legendre_Plm.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double]
    for n in range(0, 60, 3):
        for x in (0.05, 0.7, 2.75, 19.0, 44.0, 114.0):
            a, b = L.gsl_sf_bessel_jl(n, x), spherical_jn(n, x)
            assert abs(a - b) <= 1e-11 * abs(b) + 1e-300
            a, b = L.gsl_sf_bessel_yl(n, x), spherical_yn(n, x)
            assert abs(a - b) <= 1e-11 * abs(b)
    for n in range(0, 30, 2):
        for m in range(0, n + 1, 3):
            for x in (-0.7, 0.1, 0.95):
                a, b = L.gsl_sf_legendre_Plm(n, m, x), lpmv(m, n, x)
                assert abs(a - b) <= 1e-11 * abs(b) + 1e-300
