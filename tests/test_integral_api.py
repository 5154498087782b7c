"""The boundary-integral entry points of libfmmbem.so (include/integral.h) against the
reference's own outputs (tests/golden/quadrature.npz, integral_ext.npz) and the oracle.
Host-only routines: no GPU needed."""
import ctypes
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INTORDER = 3


class Cart(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


class CplxF(ctypes.Structure):
    _fields_ = [("re", ctypes.c_float), ("im", ctypes.c_float)]


class TriElem(ctypes.Structure):
    _fields_ = [("node", ctypes.c_int * 3), ("_pad", ctypes.c_int), ("alpha", ctypes.c_float * 2),
                ("beta", ctypes.c_float * 2), ("gamma", ctypes.c_float * 2)]


FP = ctypes.POINTER(ctypes.c_float)
NOD = Cart * 3


@pytest.fixture(scope="module")
def L(fm):
    L = fm.lib()
    L.genGaussParams.argtypes = [ctypes.c_int, FP, FP]
    L.green.restype = CplxF
    L.green.argtypes = [ctypes.c_float, Cart, Cart]
    for f in ("triElemIntegral_G_nsgl", "triElemIntegral_pGp1n_nsgl"):
        getattr(L, f).restype = CplxF
        getattr(L, f).argtypes = [ctypes.c_float, NOD, Cart, FP, FP]
    for f in ("triElemIntegral_G_sgl", "triElemIntegral_pGp1n_sgl", "triElemIntegral_pGp2n_sgl",
              "triElemIntegral_p2Gp1np2n_sgl"):
        getattr(L, f).restype = CplxF
        getattr(L, f).argtypes = [ctypes.c_float, NOD, FP, FP]
    for f in ("triElemIntegral_pGp2n_nsgl", "triElemIntegral_p2Gp1np2n_nsgl"):
        getattr(L, f).restype = CplxF
        getattr(L, f).argtypes = [ctypes.c_float, NOD, Cart, Cart, FP, FP]
    for f in ("triElemIntegral_R", "triElemIntegral_pRpn"):
        getattr(L, f).restype = CplxF
        getattr(L, f).argtypes = [ctypes.c_float, NOD, ctypes.c_int, ctypes.c_int, Cart, FP, FP]
    L.dirDev_R.restype = CplxF
    L.dirDev_R.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int, Cart, Cart]
    L.cmptDiffCoeff.argtypes = [ctypes.c_float, ctypes.c_void_p, ctypes.c_int, Cart, ctypes.c_void_p]
    L.bottomLevelCoeff_L.argtypes = [ctypes.c_float, TriElem, CplxF, ctypes.POINTER(Cart), Cart, FP, FP,
                                     ctypes.c_void_p, ctypes.c_int]
    return L


@pytest.fixture(scope="module")
def rule(L):
    pt, wgt = (ctypes.c_float * INTORDER)(), (ctypes.c_float * INTORDER)()
    assert L.genGaussParams(INTORDER, pt, wgt) == 0
    return pt, wgt


def c3(v):
    return Cart(*[float(t) for t in v])


def nod(tri):
    t = np.asarray(tri, np.float64).reshape(3, 3)
    return NOD(*[c3(r) for r in t])


def z(c):
    return complex(c.re, c.im)


def test_gauss_params_and_green(L, rule):
    pt, wgt = rule
    x, w = np.polynomial.legendre.leggauss(INTORDER)
    assert np.allclose(list(pt), x, atol=1e-7) and np.allclose(list(wgt), w, atol=1e-7)
    xs, ys = np.array([0.1, -0.2, 0.3]), np.array([0.4, 0.1, -0.05])
    r = np.linalg.norm(np.float32(xs) - np.float32(ys))
    k = 18.32
    assert abs(z(L.green(k, c3(xs), c3(ys))) - np.exp(1j * k * r) / (4 * np.pi * r)) < 1e-6 / r


def _tol(k, tri, y):
    # the FP32 phase k r carries ~ulp(k r) absolute error in the reference's own values
    kr = k * np.linalg.norm(tri.reshape(3, 3) - y, axis=1).max()
    return 3e-7 * max(30.0, kr)


def test_G_and_dGdnx_vs_reference(L, rule):
    pt, wgt = rule
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    tris, ys = q["tris"].astype(np.float64), q["ys"].astype(np.float64)
    for a, k in enumerate(q["ks"]):
        kf = float(np.float32(k))
        for b in range(len(tris)):
            for sgl in (0, 1):
                for name, ref in (("G", q["G"]), ("pGp1n", q["dG"])):
                    fn = getattr(L, "triElemIntegral_%s_%s" % (name, "sgl" if sgl else "nsgl"))
                    got = z(fn(kf, nod(tris[b]), pt, wgt) if sgl else fn(kf, nod(tris[b]), c3(ys[b]), pt, wgt))
                    r = complex(*ref[a, b, sgl])
                    if name == "pGp1n" and sgl:
                        # flat element: (x - y).n = 0, both sides are FP32 rounding noise
                        assert abs(got) < 1e-5 and abs(r) < 1e-5
                        continue
                    scale = abs(complex(*q["G"][a, b, sgl]))
                    assert abs(got - r) <= _tol(kf, tris[b], ys[b]) * max(scale, abs(r)), (name, a, b, sgl, got, r)


def test_dGdny_and_hypersingular_vs_reference(L, rule, oracle):
    pt, wgt = rule
    g = np.load(os.path.join(GOLDEN, "integral_ext.npz"))
    tris, ys, nr = g["tris"].astype(np.float64), g["ys"].astype(np.float64), g["nrmls"].astype(np.float64)
    for a, k in enumerate(g["ks"]):
        kf = float(np.float32(k))
        for b in range(len(tris)):
            t = nod(tris[b])
            d_ns = z(L.triElemIntegral_pGp2n_nsgl(kf, t, c3(nr[b]), c3(ys[b]), pt, wgt))
            h_ns = z(L.triElemIntegral_p2Gp1np2n_nsgl(kf, t, c3(nr[b]), c3(ys[b]), pt, wgt))
            d_s = z(L.triElemIntegral_pGp2n_sgl(kf, t, pt, wgt))
            h_s = z(L.triElemIntegral_p2Gp1np2n_sgl(kf, t, pt, wgt))
            tol = _tol(kf, tris[b], ys[b])
            for got, ref in ((d_ns, g["dGdny"][a, b, 0]), (h_ns, g["hyper"][a, b, 0]), (h_s, g["hyper"][a, b, 1])):
                r = complex(*ref)
                assert abs(got - r) <= tol * abs(r), (a, b, got, r)
            # the self term of dG/dn_y vanishes on the flat element
            assert abs(d_s) < 1e-5 and abs(complex(*g["dGdny"][a, b, 1])) < 1e-5
            # and against the oracle's FP64 restatement
            for got, ref in ((d_ns, oracle.elem_dGdny(kf, tris[b], nr[b], ys[b])),
                             (h_ns, oracle.elem_hyper(kf, tris[b], nr[b], ys[b])),
                             (h_s, oracle.elem_hyper(kf, tris[b], sgl=True))):
                assert abs(got - ref) <= 2e-6 * abs(ref), (a, b, got, ref)


def test_moments_and_dirdev_vs_reference(L, rule):
    pt, wgt = rule
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    tris, mom = q["tris"].astype(np.float64), q["moments"]
    ctr = c3(q["moment_ctr"])
    k = float(np.float32(q["moment_k"]))
    for b in range(1, len(tris)):
        for deriv, fn in ((0, L.triElemIntegral_R), (1, L.triElemIntegral_pRpn)):
            got = np.array([z(fn(k, nod(tris[b]), n, -m, ctr, pt, wgt)) for n in range(6) for m in range(-n, n + 1)])
            ref = mom[b, deriv, :, 0] + 1j * mom[b, deriv, :, 1]
            assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref), (b, deriv)
    # |m| > n gives zero
    assert z(L.triElemIntegral_R(k, nod(tris[1]), 2, 3, ctr, pt, wgt)) == 0
    g = np.load(os.path.join(GOLDEN, "integral_ext.npz"))
    kd = float(np.float32(g["dirdev_k"]))
    for i, x in enumerate(g["dirdev_x"]):
        got = np.array([z(L.dirDev_R(kd, n, m, c3(g["nrmls"][i]), c3(x))) for n in range(6) for m in range(-n, n + 1)])
        ref = g["dirdev"][i, :, 0] + 1j * g["dirdev"][i, :, 1]
        assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max(), i


def _expansion(oracle, p, k, coeff, x):
    return np.sum(coeff[: p * p] * oracle.basis(p, k, x))


def test_cmptDiffCoeff_is_the_normal_derivative(L, oracle):
    """cmptDiffCoeff's coefficients reproduce d/dn of the expansion: against the oracle's
    restatement, and against a central difference of sum c R when c has no orders >= p-1."""
    rng = np.random.default_rng(7)
    k, p = float(np.float32(18.32)), 8
    nrml = rng.standard_normal(3)
    nrml = (nrml / np.linalg.norm(nrml)).astype(np.float32)
    c = (rng.standard_normal((p + 1) ** 2) + 1j * rng.standard_normal((p + 1) ** 2)).astype(np.complex64)
    out = np.zeros(p * p, np.complex64)
    L.cmptDiffCoeff(k, c.ctypes.data, p, c3(nrml), out.ctypes.data)
    ref = oracle.diff_coeff(k, c.astype(np.complex128), p, nrml.astype(np.float64))
    assert np.linalg.norm(out - ref) <= 1e-6 * np.linalg.norm(ref)
    # orders p-1 and p zero: the derivative of the expansion is exactly the order-p output
    c[(p - 1) ** 2:] = 0
    L.cmptDiffCoeff(k, c.ctypes.data, p, c3(nrml), out.ctypes.data)
    cd = c.astype(np.complex128)
    x = np.array([0.03, -0.05, 0.02])
    h = 1e-5
    n64 = nrml.astype(np.float64)
    fd = (_expansion(oracle, p + 1, k, cd, x + h * n64) - _expansion(oracle, p + 1, k, cd, x - h * n64)) / (2 * h)
    got = np.sum(out.astype(np.complex128) * oracle.basis(p, k, x))
    assert abs(got - fd) <= 1e-5 * abs(fd)


def test_bottomLevelCoeff_L_is_ik_q_times_the_moments(L, rule, oracle):
    pt, wgt = rule
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    tri = q["tris"][2]
    pts = (Cart * 5)(c3([9, 9, 9]), c3(tri[0:3]), c3([7, 7, 7]), c3(tri[3:6]), c3(tri[6:9]))
    elem = TriElem()
    elem.node[0], elem.node[1], elem.node[2] = 1, 3, 4
    k, p = float(np.float32(18.32)), 6
    qv = CplxF(0.7, -0.3)
    out = np.zeros(p * p, np.complex64)
    L.bottomLevelCoeff_L(k, elem, qv, pts, c3(q["moment_ctr"]), pt, wgt, out.ctypes.data, p)
    mom = oracle.elem_moments(k, np.float32(tri).astype(np.float64), np.float32(q["moment_ctr"]).astype(np.float64), p)
    ref = 1j * k * (0.7 - 0.3j) * mom
    assert np.linalg.norm(out - ref) <= 1e-6 * np.linalg.norm(ref)
    # the reference's own moments of the same element
    g = q["moments"][2, 0, :, 0] + 1j * q["moments"][2, 0, :, 1]
    assert np.linalg.norm(out - 1j * k * (0.7 - 0.3j) * g) <= 1e-5 * np.linalg.norm(out)
