"""The reference-compatible entry points that use the GPU: genOctree, OprL and the sparse
matrix generators, through the C ABI."""
import ctypes
import os
import re
import tempfile

import numpy as np
import pytest

import meshes
from test_legacy_api import RotAng, TriElem, TransIdx, CartD

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class CartF(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


IPP = ctypes.POINTER(ctypes.POINTER(ctypes.c_int))
TIP = ctypes.POINTER(ctypes.POINTER(TransIdx))
FC = ctypes.c_float * 2


class Octree(ctypes.Structure):
    _fields_ = [("pt", ctypes.POINTER(CartF)), ("elem", ctypes.POINTER(TriElem)), ("numPt", ctypes.c_int),
                ("numElem", ctypes.c_int), ("fmmLevelSet", IPP), ("lmax", ctypes.c_int), ("lmin", ctypes.c_int),
                ("d", ctypes.c_double), ("pt_min", CartD), ("rotMat1", ctypes.POINTER(FC)), ("rotMat2", ctypes.POINTER(FC)),
                ("srCoaxMat", ctypes.POINTER(FC)), ("rrCoaxMat", ctypes.POINTER(FC)),
                ("srCoaxTransVec", ctypes.POINTER(ctypes.c_float)), ("numSRCoaxTransVec", ctypes.c_int),
                ("rrCoaxTransVec", ctypes.POINTER(ctypes.c_float)), ("numRRCoaxTransVec", ctypes.c_int),
                ("ang", ctypes.POINTER(RotAng)), ("numRotAng", ctypes.c_int), ("eps", ctypes.c_float),
                ("maxWavNum", ctypes.c_float), ("pmax", ctypes.c_int), ("pmax_coax", ctypes.c_int),
                ("btmLvlElemIdx", ctypes.POINTER(ctypes.c_int)), ("ssTransIdx", TIP), ("srTransIdx", TIP),
                ("rrTransIdx", TIP), ("ssTransDestArr", IPP), ("srNumLevelArr", IPP), ("srTransOriginArr", IPP),
                ("srTransDestArr", IPP), ("rrTransOriginArr", IPP)]


def cplx(ptr, n):
    a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), (2 * n,))
    return a[0::2] + 1j * a[1::2]


def test_genoctree_and_oprl(fm, oracle):
    L = fm.lib()
    L.genOctree.argtypes = [ctypes.c_char_p, ctypes.c_float, ctypes.c_int, ctypes.POINTER(Octree)]
    L.initOctree.argtypes = [ctypes.POINTER(Octree)]
    L.destroyOctree.argtypes = [ctypes.POINTER(Octree)]
    L.OprL.argtypes = [ctypes.c_float, ctypes.POINTER(Octree), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    g = dict(np.load(os.path.join(GOLDEN, "octree_ico3_r0.1_s5.npz")))
    V, F = meshes.icosphere(3, 0.1)
    k = np.float32(18.32)
    oct_ = Octree()
    L.initOctree(ctypes.byref(oct_))
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "m.obj")
        meshes.write_obj(path, V, F)
        assert L.genOctree(path.encode(), k, 5, ctypes.byref(oct_)) == 0
    lm = oct_.lmax
    assert lm == int(g["lmax"]) and oct_.d == float(g["d"])
    assert np.array_equal(np.ctypeslib.as_array(oct_.btmLvlElemIdx, (oct_.numElem,)), g["btm_idx"])
    for l in range(2, lm + 1):
        n = oct_.fmmLevelSet[l - 2][0]
        assert np.array_equal(np.ctypeslib.as_array(oct_.fmmLevelSet[l - 2], (n + 1,))[1:], g["set_%d" % l])
        t = int(g["srnum_%d" % l].sum())
        assert np.array_equal(np.ctypeslib.as_array(oct_.srTransOriginArr[l - 2], (t,)), g["sr_origin_%d" % l])
        assert [oct_.srTransIdx[l - 2][i].rotIdx for i in range(t)] == list(g["sr_rot_%d" % l])
    ang = np.array([[oct_.ang[i].alpha, oct_.ang[i].beta, oct_.ang[i].gamma] for i in range(oct_.numRotAng)], np.float32)
    # float angles come from libm's acosf/atan2f, which may differ by an ulp between
    # platforms (exact equality is checked on the x86 host in test_legacy_api.py); every
    # integer array above is exact here too
    assert ang.shape == g["angles"].shape and np.max(np.abs(ang - g["angles"])) < 1e-6
    # rotation matrices at pmax against the oracle's FP64 Wigner coefficients
    p = oct_.pmax
    rs = p * (4 * p * p - 1) // 3
    R1 = cplx(oct_.rotMat1, oct_.numRotAng * rs).reshape(oct_.numRotAng, rs)
    R2 = cplx(oct_.rotMat2, oct_.numRotAng * rs).reshape(oct_.numRotAng, rs)
    for i in (0, 7, oct_.numRotAng - 1):
        a, b = float(ang[i, 0]), float(ang[i, 1])
        assert np.max(np.abs(R1[i] - oracle.rot_matrix(a, b, 0.0, p))) < 2e-6
        assert np.max(np.abs(R2[i] - oracle.rot_matrix(0.0, b, a, p))) < 2e-6
    pc = oct_.pmax_coax
    cs = pc * (2 * pc * pc + 3 * pc + 1) // 6
    Csr = cplx(oct_.srCoaxMat, oct_.numSRCoaxTransVec * cs).reshape(-1, cs)
    nsr = oct_.numSRCoaxTransVec
    for i in (0, nsr - 1):
        ref = oracle.coax(float(k), float(oct_.srCoaxTransVec[i]), pc, True)
        fits = np.abs(ref) < 1e37
        # the FP32 format of struct octree overflows where |h_n(kt)| exceeds the float range
        # (small kt at high order), as the reference's own FP32 matrices do
        assert np.all(np.isfinite(Csr[i][fits]))
        assert np.linalg.norm(Csr[i][fits] - ref[fits]) <= 1e-6 * np.linalg.norm(ref[fits])
    assert np.isfinite(Csr[nsr - 1]).all()
    # OprL: the complete single-layer operator against the oracle (same tree depth and p)
    rng = np.random.default_rng(1)
    q = (rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))).astype(np.complex64)
    prod = np.zeros_like(q)
    assert L.OprL(k, ctypes.byref(oct_), None, None, q.ctypes.data, prod.ctypes.data) == 0
    # the vertices genOctree holds: OBJ text ("%.9g") parsed to double, stored as float
    Vf = meshes.roundtrip(V, F)[0].astype(np.float32).astype(np.float64)
    T = oracle.tree_for_fmm(Vf, F, depth=lm)
    pl = [oracle.truncnum(float(k), 0.05, 1.5, T["d"] * 2.0 ** -l) for l in range(2, lm + 1)]
    yo = oracle.FMM(Vf, F, float(k), T, pl, a=0.0, b=1.0, c=0.0, rule=0).apply(q.astype(np.complex128))
    yd = oracle.dense_apply(Vf, F, float(k), q.astype(np.complex128), a=0.0, b=1.0, c=0.0, rule=0)
    # genOctree's depth rule (deterLmax, s = 5) makes leaf boxes smaller than the triangles
    # here: a triangle filed under its centroid's box reaches past the region its multipole
    # expansion assumes, so both FMMs sit ~4e-4 from the dense operator whatever p is (the
    # same mesh at depth 3 converges geometrically in p)
    assert np.linalg.norm(yo - yd) / np.linalg.norm(yd) < 2e-3
    assert np.linalg.norm(prod - yd) / np.linalg.norm(yd) < 3e-3
    assert np.linalg.norm(prod - yo) / np.linalg.norm(yo) < 3e-3
    L.destroyOctree(ctypes.byref(oct_))


def test_coaxial_truncation_like_reference_main(fm, oracle, capfd):
    """The calls of the reference's main.c (main.c:27-38), through the library: the p = 5 (S|R)
    matrix truncated to p = 2 equals the p = 2 matrix, and the two matrices main.c prints
    with printMat_cuFloatComplex agree."""
    L = fm.lib()
    L.genSRSparseCoaxTransMat.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    L.reduceSparseCoaxTransMat.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    t = ctypes.c_float(2.3)
    m5 = np.zeros(55, np.complex64)
    m2 = np.zeros(5, np.complex64)
    assert L.genSRSparseCoaxTransMat(13.1, ctypes.byref(t), 1, 5, m5.ctypes.data) == 0
    assert L.genSRSparseCoaxTransMat(13.1, ctypes.byref(t), 1, 2, m2.ctypes.data) == 0
    L.printMat_cuFloatComplex.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.printMat_cuFloatComplex(m2.ctypes.data, 1, 5, 1)
    red = np.zeros(5, np.complex64)
    L.reduceSparseCoaxTransMat(m5.ctypes.data, 5, red.ctypes.data, 2)
    L.printMat_cuFloatComplex(red.ctypes.data, 1, 5, 1)
    assert np.allclose(red, m2, rtol=1e-5, atol=1e-7)
    ctypes.CDLL(None).fflush(None)  # printf output is buffered when stdout is not a terminal
    rows = [ln for ln in capfd.readouterr().out.splitlines() if ln.startswith("(")]
    assert len(rows) == 2, rows
    a, b = (np.array([complex(float(u), float(v)) for u, v in re.findall(r"\(([^,]+),([^)]+)\)", r)]) for r in rows)
    assert len(a) == len(b) == 5 and np.allclose(a, b, rtol=1e-5, atol=1e-6)
    assert np.allclose(a, m2, rtol=1e-5, atol=1e-6)
    g = np.load(os.path.join(GOLDEN, "tables_coax.npz"))
    ref = g["13.1_2.3_5_1"][0::2] + 1j * g["13.1_2.3_5_1"][1::2]
    assert np.linalg.norm(m5 - ref) <= 1e-5 * np.linalg.norm(ref)
