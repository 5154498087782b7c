"""Generate golden fixtures from the reference project's own code (run where it is mounted).

The reference (ZiqiFrancisFan/FMBEM_GPU_C) has no tests or golden files of its own, so the
fixtures here are its outputs on inputs this project generates:

* octree fixtures: the reference's readOBJ/srcBoxes/FMMLevelSet/FMMLevelSetNumSR, the
  element-to-leaf index of genOctree (translation.cu:3062-3076), the angle and distance
  tables and the SS/SR/RR index arrays (translation.cu:2479-2969), run on icosphere meshes
  written by tests/meshes.py.  Small cases keep every array; large ones keep SHA-256
  digests of each array plus the level sets.
* table fixtures: sparse rotation matrices (rotMatsInit + sparseRotMatGen) and coaxial
  matrices (sr/rrCoaxTransMatsInit + sparseCoaxTransMatGen), FP32 as the reference computes.
* quadrature fixtures: element integrals of G and dG/dn (regular and singular) and the
  P2M moments triElemIntegral_R / triElemIntegral_pRpn on fixed triangles.
* truncNum values.
* extended integral fixtures: dirDev_R at fixed points, the element integrals of dG/dn_y
  (triElemIntegral_pGp2n_*) and of d2G/dn_x dn_y (triElemIntegral_p2Gp1np2n_*), regular and
  singular.

* near-list fixtures: the leaf near lists I2 ∩ leaf set (octree.c:497-505) of every octree
  case, as leaf-set indices (``make_golden.py near`` regenerates only these).

Usage:  python tests/golden/make_golden.py [near]   (needs oracle/build_ref.sh to have run)
"""
import ctypes
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import meshes  # noqa: E402
from oracle import build as obuild  # noqa: E402

OCTREE_CASES = [
    # name, subdiv, radius, s, depth, keep_full
    ("ico2_r0.1_s5", 2, 0.1, 5, 0, True),
    ("ico3_r0.1_s5", 3, 0.1, 5, 0, True),
    ("ico3_r0.1_d3", 3, 0.1, 5, 3, True),
    ("ico4_r0.3_s5", 4, 0.3, 5, 0, True),
    ("ico5_r0.3_d5", 5, 0.3, 5, 5, False),
    ("ico6_r0.3_d6", 6, 0.3, 5, 6, False),
]


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def load_ref():
    lib = obuild.build_reference()
    if lib is None:
        raise SystemExit("reference tree not mounted")
    L = ctypes.CDLL(lib)
    L.ref_octree_build.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    L.ref_d.restype = ctypes.c_double
    L.ref_sparse_rot.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int, ctypes.c_void_p]
    L.ref_sparse_coax.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    L.ref_truncnum.argtypes = [ctypes.c_double] * 4
    for f in ("ref_elem_G", "ref_elem_dGdn"):
        getattr(L, f).argtypes = [ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.ref_elem_R.argtypes = [ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                             ctypes.c_void_p]
    L.ref_dirdev_R.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p]
    for f in ("ref_elem_dGdny", "ref_elem_hyper"):
        getattr(L, f).argtypes = [ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                  ctypes.c_void_p]
    return L


def ip(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def octree_case(L, name, subdiv, radius, s, depth, keep_full):
    V, F = meshes.icosphere(subdiv, radius)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "mesh.obj")
        meshes.write_obj(path, V, F)
        L.ref_octree_build(path.encode(), s, depth)
    lmax = L.ref_lmax()
    out = {"lmax": np.int64(lmax), "d": np.float64(L.ref_d())}
    pm = np.zeros(3)
    L.ref_pt_min(ip(pm))
    out["pt_min"] = pm
    nf = L.ref_num_elem()
    btm = np.zeros(nf, np.int32)
    L.ref_btm_idx(ip(btm))
    out["btm_idx"] = btm
    na = L.ref_num_ang()
    ang = np.zeros(3 * na, np.float32)
    L.ref_angles(ip(ang))
    out["angles"] = ang.reshape(-1, 3)
    nsr = L.ref_num_sr_vec()
    srv = np.zeros(nsr, np.float32)
    L.ref_sr_vec(ip(srv))
    out["sr_vec"] = srv
    nrr = L.ref_num_rr_vec()
    rrv = np.zeros(nrr, np.float32)
    L.ref_rr_vec(ip(rrv))
    out["rr_vec"] = rrv
    for l in range(2, lmax + 1):
        n = L.ref_level_count(l)
        st = np.zeros(n, np.int32)
        L.ref_level_set(l, ip(st))
        out["set_%d" % l] = st
        num = np.zeros(n, np.int32)
        L.ref_sr_num(l, ip(num))
        out["srnum_%d" % l] = num
        t = L.ref_sr_total(l)
        o, d_, c, r = (np.zeros(t, np.int32) for _ in range(4))
        L.ref_sr_arrays(l, ip(o), ip(d_), ip(c), ip(r))
        out["sr_origin_%d" % l], out["sr_dest_%d" % l], out["sr_coax_%d" % l], out["sr_rot_%d" % l] = o, d_, c, r
        if l > 2:
            dd, cc, rr = (np.zeros(n, np.int32) for _ in range(3))
            L.ref_ss_arrays(l, ip(dd), ip(cc), ip(rr))
            out["ss_dest_%d" % l], out["ss_coax_%d" % l], out["ss_rot_%d" % l] = dd, cc, rr
            oo, cc2, rr2 = (np.zeros(n, np.int32) for _ in range(3))
            L.ref_rr_arrays(l, ip(oo), ip(cc2), ip(rr2))
            out["rr_origin_%d" % l], out["rr_coax_%d" % l], out["rr_rot_%d" % l] = oo, cc2, rr2
    meta = {"subdiv": subdiv, "radius": radius, "s": s, "depth": depth, "nf": int(nf)}
    if keep_full:
        np.savez_compressed(os.path.join(HERE, "octree_%s.npz" % name), **out)
    else:
        small = {k: v for k, v in out.items() if k.startswith("set_") or k in ("lmax", "d", "pt_min", "angles", "sr_vec", "rr_vec")}
        np.savez_compressed(os.path.join(HERE, "octree_%s.npz" % name), **small)
        meta["sha256"] = {k: digest(v) for k, v in out.items()}
        meta["sizes"] = {k: int(np.size(v)) for k, v in out.items()}
    return meta


def tables(L):
    rot = {}
    for (a, b, g, p) in [(0.3, 0.7, 0.0, 5), (2.1, 1.9, 0.0, 8), (0.0, 0.9553166, 0.785398, 8), (-1.2, 2.6, 0.0, 12)]:
        out = np.zeros(2 * (p * (4 * p * p - 1) // 3), np.float32)
        L.ref_sparse_rot(a, b, g, p, ip(out))
        rot["%g_%g_%g_%d" % (a, b, g, p)] = out
    coax = {}
    for (k, t, p, sr) in [(13.1, 2.3, 5, 1), (13.1, 2.3, 2, 1), (18.32, 0.05, 8, 1), (18.32, 0.0433, 8, 0),
                          (40.0, 0.6, 12, 1), (40.0, 0.2, 12, 0)]:
        out = np.zeros(2 * (p * (2 * p * p + 3 * p + 1) // 6), np.float32)
        L.ref_sparse_coax(k, t, p, sr, ip(out))
        coax["%g_%g_%d_%d" % (k, t, p, sr)] = out
    np.savez_compressed(os.path.join(HERE, "tables_rot.npz"), **rot)
    np.savez_compressed(os.path.join(HERE, "tables_coax.npz"), **coax)


def quadrature(L):
    tris = np.array([[2.3, 3.2, 0.9, -0.3, -0.9, -0.4, 0.0, 0.1, -0.1],
                     [0.1, 0.0, 0.0, 0.0, 0.12, 0.0, 0.0, 0.0, 0.09],
                     [0.05, 0.02, 0.01, -0.03, 0.06, 0.02, 0.01, -0.04, 0.07]], np.float32)
    ys = np.array([[4.0, 1.0, 2.0], [0.3, 0.2, -0.1], [0.2, -0.3, 0.4]], np.float32)
    ks = [9.3, 18.32, 146.55]
    res = {"tris": tris, "ys": ys, "ks": np.array(ks, np.float64)}
    G = np.zeros((len(ks), len(tris), 2, 2), np.float32)    # k, tri, (nsgl, sgl), (re, im)
    dG = np.zeros_like(G)
    for a, k in enumerate(ks):
        for b, tri in enumerate(tris):
            tri_c = np.ascontiguousarray(tri)
            y = np.ascontiguousarray(ys[b])
            for sgl in (0, 1):
                o = np.zeros(2, np.float32)
                L.ref_elem_G(k, ip(tri_c), ip(y), sgl, ip(o))
                G[a, b, sgl] = o
                L.ref_elem_dGdn(k, ip(tri_c), ip(y), sgl, ip(o))
                dG[a, b, sgl] = o
    res["G"], res["dG"] = G, dG
    p = 6
    mom = np.zeros((len(tris), 2, p * p, 2), np.float32)
    ctr = np.array([0.01, -0.02, 0.03], np.float32)
    for b, tri in enumerate(tris[1:], start=1):
        tri_c = np.ascontiguousarray(tri)
        for deriv in (0, 1):
            for n in range(p):
                for m in range(-n, n + 1):
                    o = np.zeros(2, np.float32)
                    # the reference integrates R_n^{m} for the given m; the P2M moment of
                    # (n, m) uses m -> -m (integral.cu:833)
                    L.ref_elem_R(18.32, ip(tri_c), n, -m, ip(ctr), deriv, ip(o))
                    mom[b, deriv, n * n + n + m] = o
    res["moments"], res["moment_ctr"], res["moment_k"] = mom, ctr, np.float64(18.32)
    tn = []
    for (k, eps, sig, a) in [(18.32, 0.05, 1.5, 0.05), (146.55, 0.05, 1.5, 0.15), (366.4, 0.05, 1.5, 0.055), (2.0, 0.05, 1.5, 0.01)]:
        tn.append([k, eps, sig, a, L.ref_truncnum(k, eps, sig, a)])
    res["truncnum"] = np.array(tn)
    np.savez_compressed(os.path.join(HERE, "quadrature.npz"), **res)


def integral_ext(L):
    q = np.load(os.path.join(HERE, "quadrature.npz"))
    tris = np.concatenate([q["tris"], np.array([[0.0, 0.0, 0.0, 0.2, 0.01, 0.03, 0.05, 0.13, -0.02]], np.float32)])
    ys = np.concatenate([q["ys"], np.array([[0.1, 0.05, 0.3]], np.float32)])
    nrmls = np.array([[0.3, -0.5, 0.8], [0.0, 0.0, 1.0], [-0.6, 0.0, 0.8], [0.48, 0.6, 0.64]], np.float64)
    nrmls = (nrmls / np.linalg.norm(nrmls, axis=1)[:, None]).astype(np.float32)
    ks = [9.3, 18.32, 146.55]
    res = {"tris": tris, "ys": ys, "nrmls": nrmls, "ks": np.array(ks, np.float64)}
    dGy = np.zeros((len(ks), len(tris), 2, 2), np.float32)    # k, tri, (nsgl, sgl), (re, im)
    hyp = np.zeros_like(dGy)
    for a, k in enumerate(ks):
        for b, tri in enumerate(tris):
            tri_c, y, nr = np.ascontiguousarray(tri), np.ascontiguousarray(ys[b]), np.ascontiguousarray(nrmls[b])
            for sgl in (0, 1):
                o = np.zeros(2, np.float32)
                L.ref_elem_dGdny(k, ip(tri_c), ip(nr), ip(y), sgl, ip(o))
                dGy[a, b, sgl] = o
                L.ref_elem_hyper(k, ip(tri_c), ip(nr), ip(y), sgl, ip(o))
                hyp[a, b, sgl] = o
    res["dGdny"], res["hyper"] = dGy, hyp
    # dirDev_R(k, n, m, nrml, x) for n < 6, |m| <= n at four points
    xs = np.array([[0.05, -0.02, 0.03], [0.0, 0.0, 0.04], [-0.1, 0.07, -0.02], [0.01, 0.2, 0.0]], np.float32)
    dd = np.zeros((len(xs), 36, 2), np.float32)
    for i, x in enumerate(xs):
        x_c, nr = np.ascontiguousarray(x), np.ascontiguousarray(nrmls[i])
        for n in range(6):
            for m in range(-n, n + 1):
                o = np.zeros(2, np.float32)
                L.ref_dirdev_R(18.32, n, m, ip(nr), ip(x_c), ip(o))
                dd[i, n * n + n + m] = o
    res["dirdev_x"], res["dirdev"], res["dirdev_k"] = xs, dd, np.float64(18.32)
    np.savez_compressed(os.path.join(HERE, "integral_ext.npz"), **res)


def near_lists(L):
    """Leaf near lists I2 ∩ leaf set of the reference's tree (ref_near_lists: I2, intersection
    and findSetInd of octree.c) for every octree case: full arrays for the small cases, SHA-256
    digests and sizes for the large ones (octree_near.npz, octree_near_meta.json)."""
    L.ref_near_lists.restype = ctypes.c_longlong
    L.ref_near_lists.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    full, meta = {}, {}
    for name, subdiv, radius, s, depth, keep_full in OCTREE_CASES:
        V, F = meshes.icosphere(subdiv, radius)
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "mesh.obj")
            meshes.write_obj(path, V, F)
            L.ref_octree_build(path.encode(), s, depth)
        nb = L.ref_level_count(L.ref_lmax())
        tot = L.ref_near_lists(None, None)
        beg = np.zeros(nb + 1, np.int32)
        idx = np.zeros(tot, np.int32)
        L.ref_near_lists(ip(beg), ip(idx))
        if keep_full:
            full["%s_beg" % name], full["%s_idx" % name] = beg, idx
        else:
            meta[name] = {"beg": digest(beg), "idx": digest(idx), "num_pairs": int(tot)}
        print("near", name, nb, tot, flush=True)
    np.savez_compressed(os.path.join(HERE, "octree_near.npz"), **full)
    with open(os.path.join(HERE, "octree_near_meta.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def main():
    L = load_ref()
    if sys.argv[1:] == ["near"]:
        near_lists(L)
        return
    meta = {}
    for case in OCTREE_CASES:
        meta[case[0]] = octree_case(L, *case)
        print("octree", case[0], meta[case[0]]["nf"], flush=True)
    tables(L)
    quadrature(L)
    integral_ext(L)
    with open(os.path.join(HERE, "octree_meta.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    near_lists(L)


if __name__ == "__main__":
    main()
