"""The reference-compatible C entry points of libfmmbem.so (octree.h / translation.h) against
the reference's own outputs.  Host-only routines: no GPU needed."""
import ctypes
import os
import tempfile

import numpy as np
import pytest

import meshes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [("ico2_r0.1_s5", 2, 0.1, 5, 0), ("ico3_r0.1_s5", 3, 0.1, 5, 0), ("ico3_r0.1_d3", 3, 0.1, 5, 3),
         ("ico4_r0.3_s5", 4, 0.3, 5, 0)]


class CartD(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double)]


class TriElem(ctypes.Structure):
    # cuFloatComplex is 8-byte aligned: 12 bytes of nodes, 4 of padding, 3 x 8 = 40 bytes
    _fields_ = [("node", ctypes.c_int * 3), ("_pad", ctypes.c_int), ("alpha", ctypes.c_float * 2),
                ("beta", ctypes.c_float * 2), ("gamma", ctypes.c_float * 2)]


assert ctypes.sizeof(TriElem) == 40


class RotAng(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_float), ("beta", ctypes.c_float), ("gamma", ctypes.c_float)]


class TransIdx(ctypes.Structure):
    _fields_ = [("coaxIdx", ctypes.c_int), ("rotIdx", ctypes.c_int)]


IPP = ctypes.POINTER(ctypes.POINTER(ctypes.c_int))


@pytest.fixture(scope="module")
def L(fm):
    L = fm.lib()
    L.srcBoxes.argtypes = [ctypes.POINTER(CartD), ctypes.POINTER(TriElem), ctypes.c_int, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(CartD)]
    L.findBoundingCube.argtypes = [ctypes.POINTER(CartD), ctypes.c_int, ctypes.c_double, ctypes.POINTER(CartD),
                                   ctypes.POINTER(ctypes.c_double)]
    L.pnts2numSet.argtypes = [ctypes.POINTER(CartD), ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.triCentroid_d.restype = CartD
    L.triCentroid_d.argtypes = [ctypes.POINTER(CartD)]
    L.scale.restype = CartD
    L.scale.argtypes = [CartD, CartD, ctypes.c_double]
    L.FMMLevelSet.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int, IPP]
    L.FMMLevelSetNumSR.argtypes = [IPP, ctypes.c_int, IPP]
    L.genSRCoaxTransVecsRotAngles.argtypes = [ctypes.c_int, ctypes.c_double, CartD, ctypes.POINTER(ctypes.POINTER(ctypes.c_float)),
                                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.POINTER(RotAng)),
                                              ctypes.POINTER(ctypes.c_int)]
    L.genSSCoaxTransVecsRotAngles.argtypes = L.genSRCoaxTransVecsRotAngles.argtypes
    L.genRRCoaxTransVecsRotAngles.argtypes = L.genSRCoaxTransVecsRotAngles.argtypes
    L.sortRotArray.argtypes = [ctypes.POINTER(RotAng), ctypes.c_int, ctypes.c_float]
    L.bubbleSort.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int]
    TIP = ctypes.POINTER(ctypes.POINTER(TransIdx))
    L.genSRIdxArrs.argtypes = [IPP, IPP, ctypes.c_int, CartD, ctypes.c_double, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                               ctypes.POINTER(RotAng), ctypes.c_int, TIP, IPP, IPP]
    L.genSSIdxArrs.argtypes = [IPP, ctypes.c_int, CartD, ctypes.c_double, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                               ctypes.POINTER(RotAng), ctypes.c_int, TIP, IPP]
    L.genRRIdxArrs.argtypes = L.genSSIdxArrs.argtypes
    L.I4.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.I2.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.truncNum.argtypes = [ctypes.c_double] * 4
    return L


def _merge(existing, new, eps):
    for v in new:
        if not any(abs(np.float32(v) - np.float32(e)) < eps for e in existing):
            existing.append(v)
    return existing


@pytest.mark.parametrize("case,subdiv,radius,s,depth", CASES)
def test_legacy_octree_and_tables_equal_reference(L, case, subdiv, radius, s, depth):
    g = dict(np.load(os.path.join(GOLDEN, "octree_%s.npz" % case)))
    V, F = meshes.icosphere(subdiv, radius)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "m.obj")
        meshes.write_obj(path, V, F)
        nv, ne = ctypes.c_int(), ctypes.c_int()
        L.findNum(path.encode(), ctypes.byref(nv), ctypes.byref(ne))
        pts = (CartD * nv.value)()
        els = (TriElem * ne.value)()
        L.readOBJ(path.encode(), pts, els)
    nf = ne.value
    src = (ctypes.c_int * (nf + 1))()
    lmax, d, pmin = ctypes.c_int(), ctypes.c_double(), CartD()
    if depth == 0:
        L.srcBoxes(pts, els, nf, s, src, ctypes.byref(lmax), ctypes.byref(d), ctypes.byref(pmin))
    else:
        ctr = (CartD * nf)()
        for e in range(nf):
            nod = (CartD * 3)(*[pts[els[e].node[t]] for t in range(3)])
            ctr[e] = L.triCentroid_d(nod)
        bnd = (CartD * 8)()
        L.findBoundingCube(ctr, nf, 0.01, bnd, ctypes.byref(d))
        pmin = bnd[0]
        sc = (CartD * nf)(*[L.scale(ctr[e], pmin, d.value) for e in range(nf)])
        L.pnts2numSet(sc, nf, depth, src)
        lmax.value = depth
    assert lmax.value == int(g["lmax"]) and d.value == float(g["d"])
    assert np.array_equal([pmin.x, pmin.y, pmin.z], g["pt_min"])
    lm = lmax.value
    sets = (ctypes.POINTER(ctypes.c_int) * (lm - 1))()
    L.FMMLevelSet(src, lm, sets)
    nums = (ctypes.POINTER(ctypes.c_int) * (lm - 1))()
    L.FMMLevelSetNumSR(sets, lm, nums)
    for l in range(2, lm + 1):
        n = sets[l - 2][0]
        assert np.array_equal(np.ctypeslib.as_array(sets[l - 2], (n + 1,))[1:], g["set_%d" % l])
        assert np.array_equal(np.ctypeslib.as_array(nums[l - 2], (n,)), g["srnum_%d" % l])
    # angle and distance tables as genOctree builds them (translation.cu:3090-3158, 3188-3292)
    eps9 = np.float32(0.000000001 * d.value)
    angles, srv = None, []
    for l in range(2, lm + 1):
        vp, nvec, ap, nang = ctypes.POINTER(ctypes.c_float)(), ctypes.c_int(), ctypes.POINTER(RotAng)(), ctypes.c_int()
        L.genSRCoaxTransVecsRotAngles(l, d.value, pmin, ctypes.byref(vp), ctypes.byref(nvec), ctypes.byref(ap), ctypes.byref(nang))
        if angles is None:
            angles = (RotAng * nang.value)(*[ap[i] for i in range(nang.value)])
        srv = _merge(srv, [vp[i] for i in range(nvec.value)], eps9)
    L.sortRotArray(angles, len(angles), np.float32(0.05))
    sr_arr = (ctypes.c_float * len(srv))(*srv)
    L.bubbleSort(sr_arr, len(srv))
    rrv = []
    passes = [(L.genSSCoaxTransVecsRotAngles, range(lm, 2, -1)), (L.genRRCoaxTransVecsRotAngles, range(3, lm + 1))]
    for fn, levels in passes:
        for l in levels:
            vp, nvec, ap, nang = ctypes.POINTER(ctypes.c_float)(), ctypes.c_int(), ctypes.POINTER(RotAng)(), ctypes.c_int()
            fn(l, d.value, pmin, ctypes.byref(vp), ctypes.byref(nvec), ctypes.byref(ap), ctypes.byref(nang))
            rrv = _merge(rrv, [vp[i] for i in range(nvec.value)], eps9)
    rr_arr = (ctypes.c_float * len(rrv))(*rrv)
    L.bubbleSort(rr_arr, len(rrv))
    got_ang = np.array([[a.alpha, a.beta, a.gamma] for a in angles], np.float32)
    assert np.array_equal(got_ang, g["angles"])
    assert np.array_equal(np.array(sr_arr[:], np.float32), g["sr_vec"])
    assert np.array_equal(np.array(rr_arr[:], np.float32), g["rr_vec"])
    # index arrays
    TI = ctypes.POINTER(TransIdx)
    sri = (TI * (lm - 1))()
    sro = (ctypes.POINTER(ctypes.c_int) * (lm - 1))()
    srd = (ctypes.POINTER(ctypes.c_int) * (lm - 1))()
    L.genSRIdxArrs(sets, nums, lm, pmin, d.value, sr_arr, len(srv), angles, len(angles), sri, sro, srd)
    ssi = (TI * max(1, lm - 2))()
    ssd = (ctypes.POINTER(ctypes.c_int) * max(1, lm - 2))()
    L.genSSIdxArrs(sets, lm, pmin, d.value, rr_arr, len(rrv), angles, len(angles), ssi, ssd)
    rri = (TI * max(1, lm - 2))()
    rro = (ctypes.POINTER(ctypes.c_int) * max(1, lm - 2))()
    L.genRRIdxArrs(sets, lm, pmin, d.value, rr_arr, len(rrv), angles, len(angles), rri, rro)
    for l in range(2, lm + 1):
        t = int(g["srnum_%d" % l].sum())
        assert np.array_equal(np.ctypeslib.as_array(sro[l - 2], (t,)), g["sr_origin_%d" % l])
        assert np.array_equal(np.ctypeslib.as_array(srd[l - 2], (t,)), g["sr_dest_%d" % l])
        assert [sri[l - 2][i].coaxIdx for i in range(t)] == list(g["sr_coax_%d" % l])
        assert [sri[l - 2][i].rotIdx for i in range(t)] == list(g["sr_rot_%d" % l])
        if l > 2:
            n = sets[l - 2][0]
            assert np.array_equal(np.ctypeslib.as_array(ssd[l - 3], (n,)), g["ss_dest_%d" % l])
            assert [ssi[l - 3][i].coaxIdx for i in range(n)] == list(g["ss_coax_%d" % l])
            assert [ssi[l - 3][i].rotIdx for i in range(n)] == list(g["ss_rot_%d" % l])
            assert np.array_equal(np.ctypeslib.as_array(rro[l - 3], (n,)), g["rr_origin_%d" % l])
            assert [rri[l - 3][i].coaxIdx for i in range(n)] == list(g["rr_coax_%d" % l])
            assert [rri[l - 3][i].rotIdx for i in range(n)] == list(g["rr_rot_%d" % l])


def test_legacy_i2_i4_order(L):
    """I2 / I4 in the reference's enumeration order (oracle restatement of octree.c)."""
    from oracle import octree_oracle as oo

    buf = (ctypes.c_int * 256)()
    for l in (2, 3, 5):
        for num in (0, 7, 63, 100, 8 ** l - 1):
            if num >= 8 ** l:
                continue
            L.I4(num, l, buf)
            assert list(buf[1:buf[0] + 1]) == oo.i4(num, l)
            L.I2(num, l, buf)
            assert list(buf[1:buf[0] + 1]) == oo.i2(num, l)


def test_legacy_truncnum(L):
    q = np.load(os.path.join(GOLDEN, "quadrature.npz"))
    for k, eps, sig, a, p in q["truncnum"]:
        assert L.truncNum(k, eps, sig, a) == int(p)
