"""ctypes front end of the FP64 C oracle (test infrastructure only).

Used by tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg to check
the GPU library.  See ``oracle/fmm_oracle.c`` for the reference file:line each routine
restates.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from . import octree_oracle as oo

_lib = None
c_dp = ctypes.POINTER(ctypes.c_double)
c_ip = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.orc_fmm_create.restype = ctypes.c_void_p
        L.orc_fmm_create.argtypes = [ctypes.c_int, c_dp, ctypes.c_int, c_ip, ctypes.c_double] + [ctypes.c_double] * 8 + [
            ctypes.c_int, ctypes.c_int, c_ip, ctypes.POINTER(ctypes.c_longlong), c_ip, c_ip, ctypes.c_double, c_dp, ctypes.c_int]
        L.orc_fmm_apply.argtypes = [ctypes.c_void_p, c_dp, c_dp]
        L.orc_fmm_apply2.argtypes = [ctypes.c_void_p, c_dp, c_dp, ctypes.c_int]
        L.orc_fmm_destroy.argtypes = [ctypes.c_void_p]
        L.orc_fmm_num_sr.restype = ctypes.c_longlong
        L.orc_fmm_num_sr.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_fmm_num_near.restype = ctypes.c_longlong
        L.orc_fmm_num_near.argtypes = [ctypes.c_void_p]
        L.orc_dense_apply.argtypes = [ctypes.c_int, c_dp, ctypes.c_int, c_ip, ctypes.c_double] + [ctypes.c_double] * 8 + [
            ctypes.c_int, c_dp, c_dp, ctypes.c_int]
        L.orc_dense_matrix.argtypes = L.orc_dense_apply.argtypes[:14] + [c_dp, ctypes.c_int]
        L.orc_far_field.argtypes = [ctypes.c_int, c_dp, ctypes.c_int, c_ip, ctypes.c_double] + [ctypes.c_double] * 4 + [
            ctypes.c_int, c_dp, ctypes.c_int, c_dp, c_dp, ctypes.c_int]
        L.orc_elem_hyper_maue.argtypes = [ctypes.c_double, c_dp, c_dp, c_dp, ctypes.c_int, ctypes.c_int, c_dp]
        L.orc_mie_rigid.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, c_dp, c_dp]
        L.orc_mie_impedance.argtypes = [ctypes.c_double] * 4 + [ctypes.c_int, c_dp, c_dp]
        for name in ("orc_rot_H", "orc_rot_H_recur"):
            getattr(L, name).argtypes = [ctypes.c_double, ctypes.c_int, c_dp]
        L.orc_coax.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, c_dp]
        L.orc_rcr.argtypes = [ctypes.c_double, c_dp, ctypes.c_int, ctypes.c_int, c_dp, c_dp]
        L.orc_rot_matrix.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int, c_dp]
        L.orc_sph_jn.argtypes = [ctypes.c_int, ctypes.c_double, c_dp]
        L.orc_sph_yn.argtypes = [ctypes.c_int, ctypes.c_double, c_dp]
        L.orc_basis_R.argtypes = [ctypes.c_int, ctypes.c_double, c_dp, c_dp]
        L.orc_basis_S.argtypes = [ctypes.c_int, ctypes.c_double, c_dp, c_dp]
        L.orc_elem_G.argtypes = [ctypes.c_double, c_dp, c_dp, ctypes.c_int, ctypes.c_int, c_dp]
        L.orc_elem_dG.argtypes = [ctypes.c_double, c_dp, c_dp, ctypes.c_int, ctypes.c_int, c_dp]
        L.orc_elem_R.argtypes = [ctypes.c_double, c_dp, c_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_dp]
        L.orc_dirdev_R.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, c_dp, c_dp, c_dp]
        L.orc_elem_dGdny.argtypes = [ctypes.c_double, c_dp, c_dp, c_dp, ctypes.c_int, c_dp]
        L.orc_elem_hyper.argtypes = [ctypes.c_double, c_dp, c_dp, c_dp, ctypes.c_int, ctypes.c_int, c_dp]
        L.orc_diff_coeff.argtypes = [ctypes.c_double, c_dp, ctypes.c_int, c_dp, c_dp]
        L.orc_rule.argtypes = [ctypes.c_int, c_dp, c_dp]
        L.orc_rule.restype = ctypes.c_int
        L.orc_port_octree.argtypes = [c_dp, c_ip, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_ip, c_ip,
                                      c_ip, c_ip, ctypes.c_longlong, c_dp]
        L.orc_rot_size.restype = ctypes.c_int
        L.orc_coax_size.restype = ctypes.c_int
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(c_dp)


def _i(a):
    return a.ctypes.data_as(c_ip)


def rot_size(p):
    return p * (4 * p * p - 1) // 3


def coax_size(p):
    return p * (2 * p * p + 3 * p + 1) // 6


def rot_H(beta, p, recur=False):
    out = np.zeros(rot_size(p))
    (lib().orc_rot_H_recur if recur else lib().orc_rot_H)(beta, p, _d(out))
    return out


def coax(k, t, p, sr=True):
    out = np.zeros(2 * coax_size(p))
    lib().orc_coax(k, t, p, 1 if sr else 0, _d(out))
    return out.view(np.complex128)


def rot_matrix(alpha, beta, gamma, p):
    out = np.zeros(2 * rot_size(p))
    lib().orc_rot_matrix(alpha, beta, gamma, p, _d(out))
    return out.view(np.complex128)


def rcr(k, t, p, sr, x):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    y = np.zeros(p * p, dtype=np.complex128)
    t = np.ascontiguousarray(t, dtype=np.float64)
    lib().orc_rcr(k, _d(t), p, 1 if sr else 0, _d(x.view(np.float64)), _d(y.view(np.float64)))
    return y


def basis(p, k, v, singular=False):
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = np.zeros(p * p, dtype=np.complex128)
    (lib().orc_basis_S if singular else lib().orc_basis_R)(p, k, _d(v), _d(out.view(np.float64)))
    return out


def sph_jn(N, x):
    out = np.zeros(N)
    lib().orc_sph_jn(N, x, _d(out))
    return out


def sph_yn(N, x):
    out = np.zeros(N)
    lib().orc_sph_yn(N, x, _d(out))
    return out


def elem_integral(kind, k, nod, y=None, rule=0, sgl=False):
    nod = np.ascontiguousarray(nod, dtype=np.float64).reshape(9)
    y = np.zeros(3) if y is None else np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros(2)
    fn = lib().orc_elem_G if kind == "G" else lib().orc_elem_dG
    fn(k, _d(nod), _d(y), rule, 1 if sgl else 0, _d(out))
    return complex(out[0], out[1])


def elem_moments(k, nod, c, p, rule=0, deriv=False):
    nod = np.ascontiguousarray(nod, dtype=np.float64).reshape(9)
    c = np.ascontiguousarray(c, dtype=np.float64)
    out = np.zeros(p * p, dtype=np.complex128)
    lib().orc_elem_R(k, _d(nod), _d(c), p, rule, 1 if deriv else 0, _d(out.view(np.float64)))
    return out


def elem_hyper_maue(k, nod, x, nx, rule=0, sgl=False):
    """int_T d2G/dn_x dn_y dS in the regularised (Maue) form: k^2 (nx.nT) int G - the line
    integral of (nx x grad G) around T; the finite part when x is T's centroid (sgl)."""
    out = np.zeros(2)
    lib().orc_elem_hyper_maue(k, _d(np.ascontiguousarray(nod, dtype=np.float64).reshape(9)),
                              _d(np.ascontiguousarray(x, dtype=np.float64)), _d(np.ascontiguousarray(nx, dtype=np.float64)),
                              rule, 1 if sgl else 0, _d(out))
    return complex(out[0], out[1])


def dirdev_R(k, n, m, nrml, x):
    """Directional derivative of R_n^m at x along nrml (``dirDev_R``, integral.cu:284-331)."""
    out = np.zeros(2)
    lib().orc_dirdev_R(k, n, m, _d(np.ascontiguousarray(nrml, dtype=np.float64)),
                       _d(np.ascontiguousarray(x, dtype=np.float64)), _d(out))
    return complex(out[0], out[1])


def elem_dGdny(k, nod, nrml=None, y=None, sgl=False):
    """int_T dG/dn_y dS_x (``triElemIntegral_pGp2n_nsgl`` / ``_sgl``, integral.cu:509-601)."""
    nod = np.ascontiguousarray(nod, dtype=np.float64).reshape(9)
    nrml = np.zeros(3) if nrml is None else np.ascontiguousarray(nrml, dtype=np.float64)
    y = np.zeros(3) if y is None else np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros(2)
    lib().orc_elem_dGdny(k, _d(nod), _d(nrml), _d(y), 1 if sgl else 0, _d(out))
    return complex(out[0], out[1])


def elem_hyper(k, nod, nrml=None, y=None, sgl=False, nth=3):
    """int_T d2G/dn_x dn_y dS_x (``triElemIntegral_p2Gp1np2n_nsgl`` / ``_sgl``,
    integral.cu:624-660, 738-751); the self term is the finite part with an nth-point rule
    in the polar angle."""
    nod = np.ascontiguousarray(nod, dtype=np.float64).reshape(9)
    nrml = np.zeros(3) if nrml is None else np.ascontiguousarray(nrml, dtype=np.float64)
    y = np.zeros(3) if y is None else np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros(2)
    lib().orc_elem_hyper(k, _d(nod), _d(nrml), _d(y), 1 if sgl else 0, nth, _d(out))
    return complex(out[0], out[1])


def diff_coeff(k, coeff, p, nrml):
    """Coefficients of the normal derivative of sum_{n<=p} c_n^m R_n^m (``cmptDiffCoeff``,
    integral.cu:753-823); coeff holds (p+1)^2 entries."""
    c = np.ascontiguousarray(coeff, dtype=np.complex128)
    assert c.size >= (p + 1) ** 2
    out = np.zeros(p * p, dtype=np.complex128)
    lib().orc_diff_coeff(k, _d(c.view(np.float64)), p, _d(np.ascontiguousarray(nrml, dtype=np.float64)),
                         _d(out.view(np.float64)))
    return out


def quad_rule(rule):
    bary = np.zeros(3 * 64)
    w = np.zeros(64)
    n = lib().orc_rule(rule, _d(bary), _d(w))
    return bary[: 3 * n].reshape(n, 3), w[:n]


def truncnum(k, eps, sigma, a):
    """``truncNum`` (octree.c:777-796)."""
    p_lo = 1 - np.log(eps * (1 - 1.0 / sigma) ** 1.5) / np.log(sigma)
    t0 = k * a
    t1 = (3 * np.log(1.0 / eps)) ** 1.5 / 2
    p_hi = t0 + t1 * t0 ** (1.0 / 3)
    return int(np.ceil((p_lo ** 4 + p_hi ** 4) ** 0.25))


def tree_for_fmm(V, F, depth=None, s=5):
    """Octree oracle output arranged for the FMM oracle: level sets, leaf index per
    element (double-precision centroid Morton key, consistent with the leaf set)."""
    T = oo.build(V, F, s=s, depth=depth)
    leaf = T["level_sets"][-1]
    pos = {int(b): i for i, b in enumerate(leaf)}
    elem_leaf = np.asarray([pos[int(k)] for k in T["elem_leaf_key"]], dtype=np.int32)
    T["elem_leaf"] = elem_leaf
    return T


class FMM:
    """FP64 CPU FMM operator  y = a x + b L x + c M x  (test oracle)."""

    def __init__(self, V, F, k, tree, p_levels, a=0.0, b=0.0, c=0.0, rule=0, nthreads=None, alpha=0.0):
        L = lib()
        self.V = np.ascontiguousarray(V, dtype=np.float64)
        self.F = np.ascontiguousarray(F, dtype=np.int32)
        self.nf = len(F)
        lmax = tree["lmax"]
        sets = tree["level_sets"]
        nbox = np.asarray([len(s) for s in sets], dtype=np.int32)
        boxes = np.ascontiguousarray(np.concatenate(sets).astype(np.int64))
        elem_leaf = np.ascontiguousarray(tree["elem_leaf"], dtype=np.int32)
        p = np.ascontiguousarray(p_levels, dtype=np.int32)
        pt_min = np.ascontiguousarray(tree["pt_min"], dtype=np.float64)
        nthreads = nthreads or os.cpu_count() or 1
        a, b, c, al = complex(a), complex(b), complex(c), complex(alpha)
        self.h = L.orc_fmm_create(len(self.V), _d(self.V), self.nf, _i(self.F), k, a.real, a.imag, b.real, b.imag,
                                  c.real, c.imag, al.real, al.imag, rule, lmax, _i(nbox), boxes.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                  _i(elem_leaf), _i(p), tree["d"], _d(pt_min), nthreads)
        self.lmax = lmax

    def num_sr(self, l):
        return lib().orc_fmm_num_sr(self.h, l)

    def num_near(self):
        return lib().orc_fmm_num_near(self.h)

    def apply(self, x, transpose=False):
        """y = A x, or y = A^T x with transpose=True."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.nf, dtype=np.complex128)
        lib().orc_fmm_apply2(self.h, _d(x.view(np.float64)), _d(y.view(np.float64)), 1 if transpose else 0)
        return y

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_fmm_destroy(self.h)
            self.h = None


def dense_apply(V, F, k, x, a=0.0, b=0.0, c=0.0, rule=0, nthreads=None, alpha=0.0):
    V = np.ascontiguousarray(V, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    x = np.ascontiguousarray(x, dtype=np.complex128)
    y = np.zeros(len(F), dtype=np.complex128)
    a, b, c, al = complex(a), complex(b), complex(c), complex(alpha)
    lib().orc_dense_apply(len(V), _d(V), len(F), _i(F), k, a.real, a.imag, b.real, b.imag, c.real, c.imag, al.real,
                          al.imag, rule,
                          _d(x.view(np.float64)), _d(y.view(np.float64)), nthreads or os.cpu_count() or 1)
    return y


def dense_matrix(V, F, k, a=0.0, b=0.0, c=0.0, rule=0, nthreads=None, alpha=0.0):
    """The dense operator of dense_apply as an explicit complex nf x nf matrix (small meshes)."""
    V = np.ascontiguousarray(V, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    A = np.zeros((len(F), len(F)), dtype=np.complex128)
    a, b, c, al = complex(a), complex(b), complex(c), complex(alpha)
    lib().orc_dense_matrix(len(V), _d(V), len(F), _i(F), k, a.real, a.imag, b.real, b.imag, c.real, c.imag, al.real,
                           al.imag, rule,
                           _d(A.view(np.float64)), nthreads or os.cpu_count() or 1)
    return A


def far_field(V, F, k, p_surf, pts, rule=0, nthreads=None, b=0.0, c=-1.0):
    """-(b L + c M) p at the points pts: the scattered pressure of the exterior problem
    (c = -1, b = dp/dn / p on the surface; the rigid body b = 0)."""
    V = np.ascontiguousarray(V, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    p_surf = np.ascontiguousarray(p_surf, dtype=np.complex128)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(len(pts), dtype=np.complex128)
    b, c = complex(b), complex(c)
    lib().orc_far_field(len(V), _d(V), len(F), _i(F), k, b.real, b.imag, c.real, c.imag, rule,
                        _d(p_surf.view(np.float64)), len(pts), _d(pts),
                        _d(out.view(np.float64)), nthreads or os.cpu_count() or 1)
    return out


def mie_rigid(k, a, pts):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(len(pts), dtype=np.complex128)
    lib().orc_mie_rigid(k, a, len(pts), _d(pts), _d(out.view(np.float64)))
    return out


def mie_impedance(k, a, beta, pts):
    """Scattered pressure of a sphere with dp/dn = i k beta p (n outward) for exp(ikz)."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(len(pts), dtype=np.complex128)
    beta = complex(beta)
    lib().orc_mie_impedance(k, a, beta.real, beta.imag, len(pts), _d(pts), _d(out.view(np.float64)))
    return out


def port_octree(V, F, s=5, depth=0, sr_sample=0):
    """The reference's CPU octree build (srcBoxes, FMMLevelSet, FMMLevelSetNumSR) restated in
    C with its own quadratic set algebra (oracle/octree_port.c), timed.  Returns lmax, the level
    sets and SR counts per level (-1 for boxes a sampled run left out), and the stage times
    (srcBoxes, FMMLevelSet, FMMLevelSetNumSR as run, FMMLevelSetNumSR scaled to all boxes)."""
    V = np.ascontiguousarray(V, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    cap = 16 * len(F) + 64
    sets = np.zeros(cap, np.int32)
    srnum = np.zeros(cap, np.int32)
    counts = np.zeros(16, np.int32)
    times = np.zeros(4)
    lmax = ctypes.c_int(0)
    rc = lib().orc_port_octree(_d(V), _i(F), len(F), s, depth, sr_sample, ctypes.byref(lmax), _i(counts), _i(sets),
                               _i(srnum), cap, _d(times))
    if rc != 0:
        raise RuntimeError("orc_port_octree failed (lmax %d)" % lmax.value)
    out = {"lmax": lmax.value, "times": {"src_boxes_s": times[0], "level_sets_s": times[1], "sr_lists_s_run": times[2],
                                         "sr_lists_s": times[3]}}
    pos = 0
    for l in range(2, lmax.value + 1):
        n = int(counts[l])
        out["set_%d" % l] = sets[pos:pos + n].copy()
        out["srnum_%d" % l] = srnum[pos:pos + n].copy()
        pos += n
    return out
