"""fmm_coax_matrices_noalloc, the coaxial-matrix generator for callers that must not let the
library allocate device memory (an application that owns all device memory through its own
pool, or a loop that cannot take the device synchronisation of cudaMalloc/cudaFree).  Two
calls in a row through its shared fixed scratch must give the FP64 oracle's matrices and
those of the regular (allocating) generator genSR/genRRSparseCoaxTransMat, and sizes beyond
the scratch must be rejected.  The file name makes pytest collect it last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(fm):
    L = fm.lib()
    L.fmm_coax_matrices_noalloc.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p]
    L.genSRSparseCoaxTransMat.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p]
    L.genRRSparseCoaxTransMat.argtypes = L.genSRSparseCoaxTransMat.argtypes
    return L


def _coax_size(p):
    return p * (2 * p * p + 3 * p + 1) // 6


def _regular(L, k, t, p, sr):
    """The allocating generator with the reference's FP32 interface."""
    n = len(t)
    out = np.zeros(n * _coax_size(p), np.complex64)
    tf = (ctypes.c_float * n)(*t)
    fn = L.genSRSparseCoaxTransMat if sr else L.genRRSparseCoaxTransMat
    assert fn(k, tf, n, p, out.ctypes.data) == 0
    return out


def _noalloc(L, torch, k, t, p, sr):
    n = len(t)
    td = torch.tensor(np.asarray(t, np.float64), device="cuda")
    out = torch.full((n * _coax_size(p),), complex("nan"), dtype=torch.complex128, device="cuda")
    st = L.fmm_coax_matrices_noalloc(float(k), td.data_ptr(), n, p, 1 if sr else 0, out.data_ptr(), None)
    assert st == 0, L.fmm_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


# (S|R) at p = 30 on the 81,920-triangle workload's k, then (R|R) at p = 12 with small k t,
# where the library takes the entries below the diagonal from the coaxial symmetry
CASES = [(146.55, [0.3, 0.3354, 0.45, 0.7794], 30, True),
         (18.32, [0.0433, 0.05, 0.0612], 12, False)]


def test_noalloc_matches_fp64_oracle_twice(fm, oracle):
    """Two calls in a row through the shared scratch, each matrix against the FP64 oracle's
    coaxial recurrence (same relations, same symmetry rule) at 1e-12."""
    import torch

    L = _bind(fm)
    for k, t, p, sr in CASES:
        got = _noalloc(L, torch, k, t, p, sr).reshape(len(t), -1)
        assert np.isfinite(got).all()
        for i, ti in enumerate(t):
            ref = oracle.coax(k, ti, p, sr)
            assert np.linalg.norm(got[i] - ref) <= 1e-12 * np.linalg.norm(ref), (k, ti, p, sr)


def test_noalloc_matches_regular_generator_twice(fm):
    """The same two calls against the allocating generator of the reference's FP32 interface
    (genSR/genRRSparseCoaxTransMat), at its float inputs."""
    import torch

    L = _bind(fm)
    for k, t, p, sr in CASES:
        tf = [float(np.float32(v)) for v in t]
        ref = _regular(L, np.float32(k), tf, p, sr)
        got = _noalloc(L, torch, float(np.float32(k)), tf, p, sr)
        assert np.isfinite(got).all()
        # the same relative tolerance as the coaxial-matrix checks of the regular generator
        assert np.linalg.norm(got.astype(np.complex64) - ref) <= 1e-6 * np.linalg.norm(ref)


def test_noalloc_rejects_what_it_cannot_do(fm):
    import torch

    L = _bind(fm)
    p, n = 64, 8          # 8 * 64 * 127 * 64 entries > 2^19
    td = torch.ones(n, dtype=torch.float64, device="cuda")
    out = torch.zeros(n * _coax_size(p), dtype=torch.complex128, device="cuda")
    st = L.fmm_coax_matrices_noalloc(10.0, td.data_ptr(), n, p, 1, out.data_ptr(), None)
    assert st == 1 and b"exceeds the fixed scratch" in L.fmm_last_error()
    host = np.ones(2)
    assert L.fmm_coax_matrices_noalloc(10.0, host.ctypes.data, 2, 4, 1, out.data_ptr(), None) == 1
    # a zero length is outside (0, 1e5] for k t: that matrix comes out as NaN, the other one is computed
    td = torch.tensor([0.0, 0.5], dtype=torch.float64, device="cuda")
    out = torch.zeros(2 * _coax_size(4), dtype=torch.complex128, device="cuda")
    assert L.fmm_coax_matrices_noalloc(10.0, td.data_ptr(), 2, 4, 1, out.data_ptr(), None) == 0
    o = out.cpu().numpy()
    assert np.isnan(o[:_coax_size(4)]).all() and np.isfinite(o[_coax_size(4):]).all()
