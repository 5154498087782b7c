"""GB300 FMM-BEM Helmholtz solver: Python front end over the C ABI of libfmmbem.so.

The library is the product; this module only binds its entry points (``include/fmmbem.h``)
with ctypes, mirroring the plan API one to one.  There is no CPU implementation behind it:
if the CUDA library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfmmbem.so")

FMM_FP64 = 0
FMM_MIXED = 1
FMM_FLOAT2 = 2  # FP64 matvec with the M2L in float-float (the mixed solvers' residuals)
RULE_GAUSS3 = 0
RULE_DUNAVANT7 = 1
MAX_LEVEL = 12

_STATUS = {0: "FMM_OK", 1: "FMM_ERR_ARG", 2: "FMM_ERR_CUDA", 3: "FMM_ERR_ALLOC", 4: "FMM_ERR_IO",
           5: "FMM_ERR_BREAKDOWN", 6: "FMM_ERR_NOT_CONVERGED", 7: "FMM_ERR_MESH"}


class FmmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_STATUS.get(status, status), msg))
        self.status = status


class Options(ctypes.Structure):
    _fields_ = [("k", ctypes.c_double), ("depth", ctypes.c_int), ("s", ctypes.c_int),
                ("p_level", ctypes.c_int * (MAX_LEVEL + 1)), ("eps", ctypes.c_double), ("rule", ctypes.c_int),
                ("a_re", ctypes.c_double), ("a_im", ctypes.c_double), ("b_re", ctypes.c_double),
                ("b_im", ctypes.c_double), ("c_re", ctypes.c_double), ("c_im", ctypes.c_double),
                ("build_mixed", ctypes.c_int), ("device", ctypes.c_int), ("alpha_re", ctypes.c_double),
                ("alpha_im", ctypes.c_double), ("deterministic", ctypes.c_int)]


class Info(ctypes.Structure):
    _fields_ = [("num_elem", ctypes.c_int), ("num_vert", ctypes.c_int), ("lmin", ctypes.c_int), ("lmax", ctypes.c_int),
                ("d", ctypes.c_double), ("pt_min", ctypes.c_double * 3), ("p_level", ctypes.c_int * (MAX_LEVEL + 1)),
                ("num_box", ctypes.c_int * (MAX_LEVEL + 1)), ("num_m2l", ctypes.c_longlong * (MAX_LEVEL + 1)),
                ("num_near", ctypes.c_longlong), ("device_bytes", ctypes.c_size_t), ("setup_seconds", ctypes.c_double),
                ("m2l_columns", ctypes.c_int * (MAX_LEVEL + 1)), ("m2l_tensor", ctypes.c_int * (MAX_LEVEL + 1)),
                ("expansions_scaled", ctypes.c_int), ("pass_tc3", ctypes.c_int * (MAX_LEVEL + 1)),
                ("pass_dense", ctypes.c_int * (MAX_LEVEL + 1)), ("pass_balanced", ctypes.c_int * (MAX_LEVEL + 1))]


_lib = None
c_vp = ctypes.c_void_p
c_dp = ctypes.POINTER(ctypes.c_double)
c_ip = ctypes.POINTER(ctypes.c_int)


def lib():
    """Load libfmmbem.so; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FmmError(2, "CUDA library %s not built (run __graft_entry__.build())" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        L.fmm_default_options.argtypes = [ctypes.POINTER(Options)]
        L.fmm_plan_create.argtypes = [c_dp, ctypes.c_int, c_ip, ctypes.c_int, ctypes.POINTER(Options), ctypes.POINTER(c_vp)]
        L.fmm_plan_create_obj.argtypes = [ctypes.c_char_p, ctypes.POINTER(Options), ctypes.POINTER(c_vp)]
        L.fmm_plan_destroy.argtypes = [c_vp]
        L.fmm_plan_info.argtypes = [c_vp, ctypes.POINTER(Info)]
        L.fmm_vjp_admittance.argtypes = [c_vp, c_vp, c_dp, ctypes.c_int, c_vp, c_vp, c_vp, c_dp]
        L.fmm_plan_lists.argtypes = [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp]
        L.fmm_plan_direction.argtypes = [c_vp, ctypes.c_int, c_ip]
        L.fmm_plan_near_lists.argtypes = [c_vp, c_vp, c_vp, ctypes.POINTER(ctypes.c_longlong), c_vp, c_vp,
                                          ctypes.POINTER(ctypes.c_longlong)]
        L.fmm_matvec.argtypes = [c_vp, c_vp, c_vp, ctypes.c_int, ctypes.c_int]
        L.fmm_matvec_adjoint.argtypes = [c_vp, c_vp, c_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.fmm_gmres.argtypes = [c_vp, c_vp, c_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                c_ip, c_dp]
        L.fmm_solve_batched.argtypes = [c_vp, c_vp, c_vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, c_ip, c_dp]
        L.fmm_solve_many.argtypes = [ctypes.POINTER(c_vp), ctypes.c_int, ctypes.POINTER(c_vp), ctypes.POINTER(c_vp),
                                     ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_ip, c_dp, c_ip]
        L.fmm_scene_create.argtypes = [ctypes.POINTER(c_vp), ctypes.c_int, ctypes.POINTER(c_vp)]
        L.fmm_scene_destroy.argtypes = [c_vp]
        L.fmm_scene_unknowns.argtypes = [c_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
        L.fmm_scene_matvec.argtypes = [c_vp, c_vp, c_vp, ctypes.c_int]
        L.fmm_scene_solve.argtypes = [c_vp, c_vp, c_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      c_ip, c_dp]
        L.fmm_scene_timings.argtypes = [c_vp, c_dp, c_dp, c_ip, c_dp, c_ip]
        L.fmm_selftest_bounded_wait.argtypes = [ctypes.c_int, c_ip, c_ip]
        L.fmm_scene_set_active.argtypes = [c_vp, c_ip]
        L.fmm_vjp.argtypes = [c_vp, c_vp, c_dp, c_dp, ctypes.c_int, c_vp, ctypes.c_double, ctypes.c_int, c_dp, c_vp]
        L.fmm_far_field.argtypes = [c_vp, c_vp, c_dp, ctypes.c_int, c_vp]
        L.fmm_plane_wave_rhs.argtypes = [c_vp, c_dp, c_vp]
        L.fmm_mesh_icosphere.argtypes = [ctypes.c_int, ctypes.c_double, c_dp, c_ip, c_ip, c_ip]
        L.fmm_mesh_geodesic.argtypes = [ctypes.c_int, ctypes.c_double, c_dp, c_ip, c_ip, c_ip]
        L.fmm_mesh_ellipsoid.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_ulonglong, c_dp, c_ip, c_ip, c_ip]
        L.fmm_mesh_box.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, c_dp, c_ip, c_ip, c_ip]
        L.fmm_last_error.restype = ctypes.c_char_p
        L.fmm_set_profiling.argtypes = [c_vp, ctypes.c_int]
        L.fmm_last_timings.argtypes = [c_vp, ctypes.POINTER(ctypes.c_char_p), c_dp, c_ip]
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        raise FmmError(status, lib().fmm_last_error().decode(errors="replace"))


def default_options():
    o = Options()
    lib().fmm_default_options(ctypes.byref(o))
    return o


def icosphere(subdiv, radius):
    """Library mesh generator (``fmm_mesh_icosphere``)."""
    nv, nf = ctypes.c_int(), ctypes.c_int()
    _check(lib().fmm_mesh_icosphere(subdiv, radius, None, ctypes.byref(nv), None, ctypes.byref(nf)))
    V = np.zeros((nv.value, 3))
    F = np.zeros((nf.value, 3), dtype=np.int32)
    _check(lib().fmm_mesh_icosphere(subdiv, radius, V.ctypes.data_as(c_dp), ctypes.byref(nv), F.ctypes.data_as(c_ip),
                                    ctypes.byref(nf)))
    return V, F


def _mesh(fn, *args):
    nv, nf = ctypes.c_int(), ctypes.c_int()
    _check(fn(*args, None, ctypes.byref(nv), None, ctypes.byref(nf)))
    V = np.zeros((nv.value, 3))
    F = np.zeros((nf.value, 3), dtype=np.int32)
    _check(fn(*args, V.ctypes.data_as(c_dp), ctypes.byref(nv), F.ctypes.data_as(c_ip), ctypes.byref(nf)))
    return V, F


def geodesic_sphere(freq, radius):
    """Geodesic sphere, 20 freq^2 triangles (``fmm_mesh_geodesic``)."""
    return _mesh(lib().fmm_mesh_geodesic, freq, radius)


def ellipsoid(freq, axes, lmax=-1, sigma=0.0, seed=0):
    """Ellipsoid with seeded radial spherical-harmonic bumps (``fmm_mesh_ellipsoid``)."""
    return _mesh(lib().fmm_mesh_ellipsoid, freq, float(axes[0]), float(axes[1]), float(axes[2]), lmax, sigma, seed)


def box(n, edges):
    """Box centred at the origin, 12 n^2 triangles (``fmm_mesh_box``)."""
    return _mesh(lib().fmm_mesh_box, n, float(edges[0]), float(edges[1]), float(edges[2]))


def _ptr(a):
    """Raw pointer of a numpy array or a torch tensor (host or device)."""
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)


def selftest_bounded_wait(device=0):
    """Run the tensor-core M2L's bounded barrier wait on a barrier nothing completes
    (``fmm_selftest_bounded_wait``).  Returns (gave_up, completed_after_arrival)."""
    g, c = ctypes.c_int(), ctypes.c_int()
    _check(lib().fmm_selftest_bounded_wait(device, ctypes.byref(g), ctypes.byref(c)))
    return bool(g.value), bool(c.value)


def solve_many(plans, rhs, tol=1e-6, maxit=500, restart=50, precision=FMM_FP64, nthreads=8, x0=None):
    """Solve plans[i] x_i = rhs[i] for all i concurrently (``fmm_solve_many``).
    Returns (xs, iters, relres, status)."""
    n = len(plans)
    bs = [np.ascontiguousarray(b, dtype=np.complex128) for b in rhs]
    xs = [np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0[i], dtype=np.complex128).copy()
          for i, b in enumerate(bs)]
    ph = (c_vp * n)(*[p.h.value for p in plans])
    bp = (c_vp * n)(*[b.ctypes.data for b in bs])
    xp = (c_vp * n)(*[x.ctypes.data for x in xs])
    it = np.zeros(n, dtype=np.int32)
    rr = np.zeros(n)
    stv = np.zeros(n, dtype=np.int32)
    st = lib().fmm_solve_many(ph, n, bp, xp, tol, maxit, restart, precision, nthreads, it.ctypes.data_as(c_ip),
                              rr.ctypes.data_as(c_dp), stv.ctypes.data_as(c_ip))
    if st not in (0, 6):
        _check(st)
    return xs, it, rr, stv


class Scene:
    """Plans solved in lockstep (``fmm_scene_create``): their unknowns form one vector, plan i
    at ``offsets[i]``; a mixed matvec applies all operators with one set of launches.  The
    plans must outlive the scene."""

    def __init__(self, plans):
        self.plans = list(plans)
        n = len(self.plans)
        ph = (c_vp * n)(*[p.h.value for p in self.plans])
        h = c_vp()
        _check(lib().fmm_scene_create(ph, n, ctypes.byref(h)))
        self.h = h
        tot = ctypes.c_longlong()
        offs = (ctypes.c_longlong * (n + 1))()
        _check(lib().fmm_scene_unknowns(self.h, ctypes.byref(tot), offs))
        self.n = int(tot.value)
        self.offsets = np.array(offs[:], dtype=np.int64)

    def split(self, v):
        """Per-plan views of a scene vector."""
        return [v[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.plans))]

    def join(self, vs):
        """One scene vector from per-plan vectors."""
        return np.concatenate([np.asarray(v, dtype=np.complex128) for v in vs])

    def matvec(self, x, precision=FMM_MIXED, out=None):
        if out is None:
            if hasattr(x, "data_ptr"):
                import torch
                out = torch.empty_like(x)
            else:
                x = np.ascontiguousarray(x, dtype=np.complex128)
                out = np.empty_like(x)
        _check(lib().fmm_scene_matvec(self.h, _ptr(x), _ptr(out), precision))
        return out

    def set_active(self, on=None):
        """Apply only the plans with on[i] true in later matvecs (None: all); the others get y = 0."""
        if on is None:
            _check(lib().fmm_scene_set_active(self.h, None))
            return
        a = np.ascontiguousarray(np.asarray(on, dtype=bool).astype(np.int32))
        _check(lib().fmm_scene_set_active(self.h, a.ctypes.data_as(c_ip)))

    def solve(self, b, tol=1e-6, maxit=500, restart=50, precision=FMM_MIXED, x0=None):
        """Lockstep GMRES over all plans (``fmm_scene_solve``); b is a scene vector or a list of
        per-plan vectors.  Returns (x, iters, relres, converged) with x a scene vector."""
        if isinstance(b, (list, tuple)):
            b = self.join(b)
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0, dtype=np.complex128).copy()
        it = np.zeros(len(self.plans), dtype=np.int32)
        rr = np.zeros(len(self.plans))
        st = lib().fmm_scene_solve(self.h, _ptr(b), _ptr(x), tol, maxit, restart, precision, it.ctypes.data_as(c_ip),
                                   rr.ctypes.data_as(c_dp))
        if st not in (0, 6):
            _check(st)
        return x, it, rr, st == 0

    def timings(self):
        """The last solve: wall seconds, device ms and count of its mixed and FP64 matvecs."""
        s, mm, fm_ = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        mc, fc = ctypes.c_int(), ctypes.c_int()
        _check(lib().fmm_scene_timings(self.h, ctypes.byref(s), ctypes.byref(mm), ctypes.byref(mc), ctypes.byref(fm_),
                                       ctypes.byref(fc)))
        return {"solve_s": s.value, "mixed_ms": mm.value, "mixed_calls": mc.value, "fp64_ms": fm_.value,
                "fp64_calls": fc.value}

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().fmm_scene_destroy(self.h)
            self.h = c_vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """A solver plan for one mesh and wavenumber (``fmm_plan_create``)."""

    def __init__(self, V=None, F=None, k=1.0, depth=0, s=5, p_levels=None, eps=0.05, rule=RULE_GAUSS3,
                 a=0.0, b=1.0, c=0.0, build_mixed=True, obj=None, device=0, alpha=0.0, deterministic=False):
        o = default_options()
        o.k, o.depth, o.s, o.eps, o.rule = k, depth, s, eps, rule
        a, b, c, alpha = complex(a), complex(b), complex(c), complex(alpha)
        o.a_re, o.a_im, o.b_re, o.b_im, o.c_re, o.c_im = a.real, a.imag, b.real, b.imag, c.real, c.imag
        o.alpha_re, o.alpha_im = alpha.real, alpha.imag
        o.build_mixed = 1 if build_mixed else 0
        o.deterministic = 1 if deterministic else 0
        o.device = device
        if p_levels is not None:
            for l, p in p_levels.items() if isinstance(p_levels, dict) else enumerate(p_levels):
                o.p_level[l] = int(p)
        h = c_vp()
        if obj is not None:
            _check(lib().fmm_plan_create_obj(obj.encode(), ctypes.byref(o), ctypes.byref(h)))
        else:
            V = np.ascontiguousarray(V, dtype=np.float64)
            F = np.ascontiguousarray(F, dtype=np.int32)
            _check(lib().fmm_plan_create(V.ctypes.data_as(c_dp), len(V), F.ctypes.data_as(c_ip), len(F),
                                         ctypes.byref(o), ctypes.byref(h)))
        self.h = h
        self.info = self._info()
        self.nf = self.info.num_elem
        self.nv = self.info.num_vert

    def _info(self):
        i = Info()
        _check(lib().fmm_plan_info(self.h, ctypes.byref(i)))
        return i

    def lists(self, level):
        """The M2L lists the matvecs read at `level` (fmm_plan_lists): (boxes, m2l_beg, m2l_src,
        m2l_dir, offsets) with offsets[d] the integer box offset of direction d."""
        nb, t = self.info.num_box[level], self.info.num_m2l[level]
        boxes = np.zeros(nb, np.int64)
        beg = np.zeros(nb + 1, np.int32)
        src = np.zeros(max(t, 1), np.int32)
        dr = np.zeros(max(t, 1), np.int32)
        _check(lib().fmm_plan_lists(self.h, level, boxes.ctypes.data, beg.ctypes.data, src.ctypes.data, dr.ctypes.data))
        off = np.zeros((316, 3), np.int32)
        for d in range(316):
            _check(lib().fmm_plan_direction(self.h, d, off[d].ctypes.data_as(c_ip)))
        return boxes, beg, src[:t], dr[:t], off

    def near_lists(self):
        """Leaf near lists (fmm_plan_near_lists): (box_beg, box_idx, elem_beg, elem_col)."""
        nbp, nep = ctypes.c_longlong(), ctypes.c_longlong()
        _check(lib().fmm_plan_near_lists(self.h, None, None, ctypes.byref(nbp), None, None, ctypes.byref(nep)))
        nb = self.info.num_box[self.info.lmax]
        bb, bi = np.zeros(nb + 1, np.int32), np.zeros(max(nbp.value, 1), np.int32)
        eb, ec = np.zeros(self.nf + 1, np.int32), np.zeros(max(nep.value, 1), np.int32)
        _check(lib().fmm_plan_near_lists(self.h, bb.ctypes.data, bi.ctypes.data, ctypes.byref(nbp), eb.ctypes.data,
                                         ec.ctypes.data, ctypes.byref(nep)))
        return bb, bi[:nbp.value], eb, ec[:nep.value]

    def matvec(self, x, precision=FMM_FP64, out=None):
        """y = A x.  x: complex128 numpy array (host) or torch tensor (host or CUDA)."""
        if out is None:
            if hasattr(x, "data_ptr"):
                import torch
                out = torch.empty_like(x)
            else:
                x = np.ascontiguousarray(x, dtype=np.complex128)
                out = np.empty_like(x)
        nrhs = (x.numel() if hasattr(x, "numel") else x.size) // self.nf
        _check(lib().fmm_matvec(self.h, _ptr(x), _ptr(out), nrhs, precision))
        return out

    def matvec_adjoint(self, x, precision=FMM_FP64, conjugate=False, out=None):
        """y = A^T x, or A^H x with conjugate=True (vector-Jacobian products, adjoint solves)."""
        if out is None:
            if hasattr(x, "data_ptr"):
                import torch
                out = torch.empty_like(x)
            else:
                x = np.ascontiguousarray(x, dtype=np.complex128)
                out = np.empty_like(x)
        nrhs = (x.numel() if hasattr(x, "numel") else x.size) // self.nf
        _check(lib().fmm_matvec_adjoint(self.h, _ptr(x), _ptr(out), nrhs, precision, 1 if conjugate else 0))
        return out

    def gmres(self, b, x0=None, tol=1e-6, maxit=500, restart=50, precision=FMM_FP64):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0, dtype=np.complex128).copy()
        it, rr = ctypes.c_int(), ctypes.c_double()
        st = lib().fmm_gmres(self.h, _ptr(b), _ptr(x), tol, maxit, restart, precision, ctypes.byref(it), ctypes.byref(rr))
        if st not in (0, 6):
            _check(st)
        return x, it.value, rr.value, st == 0

    def solve_batched(self, B, X0=None, tol=1e-6, maxit=500, restart=50, precision=FMM_FP64):
        """Solve A X = B for the rows of B (nrhs x nf) at once; returns (X, iters, relres, ok)."""
        B = np.ascontiguousarray(B, dtype=np.complex128)
        nrhs = B.shape[0]
        X = np.zeros_like(B) if X0 is None else np.ascontiguousarray(X0, dtype=np.complex128).copy()
        it = np.zeros(nrhs, dtype=np.int32)
        rr = np.zeros(nrhs, dtype=np.float64)
        st = lib().fmm_solve_batched(self.h, _ptr(B), _ptr(X), nrhs, tol, maxit, restart, precision,
                                     it.ctypes.data_as(c_ip), rr.ctypes.data_as(c_dp))
        if st not in (0, 6):
            _check(st)
        return X, it, rr, st == 0

    def vjp(self, x, pts, pbar, direction=(0.0, 0.0, 1.0), tol=1e-10, precision=FMM_FP64):
        """dJ/dV (nv x 3) for dJ = 2 Re(pbar^H dp), p = far_field(x, pts), x solving A x = plane_wave(direction)
        (direction None: a right-hand side that does not move with the mesh).  Returns (grad, lambda)."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        pbar = np.ascontiguousarray(pbar, dtype=np.complex128)
        grad = np.zeros((self.nv, 3), dtype=np.float64)
        lam = np.zeros(self.nf, dtype=np.complex128)
        d = None if direction is None else np.ascontiguousarray(direction, dtype=np.float64)
        _check(lib().fmm_vjp(self.h, _ptr(x), None if d is None else d.ctypes.data_as(c_dp), pts.ctypes.data_as(c_dp),
                             len(pts), _ptr(pbar), tol, precision, grad.ctypes.data_as(c_dp), _ptr(lam)))
        return grad, lam

    def vjp_admittance(self, x, pts, pbar, lam):
        """Admittance derivative (fmm_vjp_admittance) for b = i k beta, a = (1 + alpha b)/2:
        returns (g, dJ_dbeta) with dJ = 2 Re sum_j g_j dbeta_j per element and dJ_dbeta =
        (dJ/dRe beta, dJ/dIm beta) for one admittance on the whole surface.  lam: the adjoint
        solution fmm_vjp returned for the same x, pts, pbar."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        pbar = np.ascontiguousarray(pbar, dtype=np.complex128)
        lam = np.ascontiguousarray(lam, dtype=np.complex128)
        g = np.zeros(self.nf, dtype=np.complex128)
        dj = np.zeros(2)
        _check(lib().fmm_vjp_admittance(self.h, _ptr(x), pts.ctypes.data_as(c_dp), len(pts), _ptr(pbar), _ptr(lam),
                                        _ptr(g), dj.ctypes.data_as(c_dp)))
        return g, dj

    def far_field(self, p, pts):
        p = np.ascontiguousarray(p, dtype=np.complex128)
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        out = np.zeros(len(pts), dtype=np.complex128)
        _check(lib().fmm_far_field(self.h, _ptr(p), pts.ctypes.data_as(c_dp), len(pts), _ptr(out)))
        return out

    def plane_wave(self, direction=(0.0, 0.0, 1.0)):
        d = np.ascontiguousarray(direction, dtype=np.float64)
        out = np.zeros(self.nf, dtype=np.complex128)
        _check(lib().fmm_plane_wave_rhs(self.h, d.ctypes.data_as(c_dp), _ptr(out)))
        return out

    def set_profiling(self, on=True):
        """True or 1: per-kernel timers (direct launches); 2: whole-matvec timer only; False or 0: off."""
        _check(lib().fmm_set_profiling(self.h, int(on) if not isinstance(on, bool) else (1 if on else 0)))

    def timings(self):
        cap = 80
        n = ctypes.c_int(cap)
        names = (ctypes.c_char_p * cap)()
        ms = (ctypes.c_double * cap)()
        _check(lib().fmm_last_timings(self.h, names, ms, ctypes.byref(n)))
        return [(names[i].decode(), ms[i]) for i in range(min(n.value, cap))]

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            _check(lib().fmm_plan_destroy(self.h))  # refused while a scene uses the plan
            self.h = c_vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fibonacci_sphere(n, radius):
    """n points on a sphere of the given radius (Fibonacci lattice), for far-field checks."""
    i = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    theta = np.pi * (1 + 5 ** 0.5) * i
    return radius * np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], axis=1)
