"""Mesh front end (fmm_mesh_geodesic, fmm_mesh_ellipsoid, fmm_mesh_box): closed, consistently
outward-oriented surfaces with the expected counts, areas and volumes.  Host only."""
import numpy as np
import pytest


def closed_and_outward(V, F):
    # every edge used once in each direction: closed and consistently oriented
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    fwd = {tuple(x) for x in e}
    assert len(fwd) == len(e)
    assert all((b, a) in fwd for a, b in fwd)
    # Euler characteristic of a sphere
    assert len(V) - len(fwd) // 2 + len(F) == 2
    # divergence theorem: positive enclosed volume means outward normals
    n = np.cross(V[F[:, 0]] - V[F[:, 2]], V[F[:, 1]] - V[F[:, 2]])
    vol = np.einsum("ij,ij->", n, V[F].mean(axis=1)) / 6.0
    area = 0.5 * np.linalg.norm(n, axis=1)
    assert (area > 0).all()
    return vol, area.sum()


@pytest.mark.parametrize("freq", [1, 3, 10])
def test_geodesic_sphere(fm, freq):
    V, F = fm.geodesic_sphere(freq, 0.2)
    assert len(F) == 20 * freq * freq and len(V) == 10 * freq * freq + 2
    assert np.allclose(np.linalg.norm(V, axis=1), 0.2, atol=1e-9)
    vol, area = closed_and_outward(V, F)
    if freq == 10:
        assert abs(vol / (4 / 3 * np.pi * 0.2 ** 3) - 1) < 0.01 and abs(area / (4 * np.pi * 0.04) - 1) < 0.01


def test_ellipsoid_and_bumps(fm):
    V, F = fm.ellipsoid(20, (0.075, 0.09, 0.11))
    vol, _ = closed_and_outward(V, F)
    assert abs(vol / (4 / 3 * np.pi * 0.075 * 0.09 * 0.11) - 1) < 0.005
    r = V / np.array([0.075, 0.09, 0.11])
    assert np.allclose(np.linalg.norm(r, axis=1), 1.0, atol=1e-8)
    Vb, Fb = fm.ellipsoid(20, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=3)
    assert np.array_equal(Fb, F)
    d = np.linalg.norm(Vb, axis=1) - np.linalg.norm(V, axis=1)
    assert 0.5e-3 < d.std() < 10e-3
    Vc, _ = fm.ellipsoid(20, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=3)
    assert np.array_equal(Vb, Vc)  # seeded
    Vd, _ = fm.ellipsoid(20, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=4)
    assert not np.array_equal(Vb, Vd)
    closed_and_outward(Vb, Fb)


def test_box(fm):
    V, F = fm.box(4, (0.01, 0.02, 0.05))
    assert len(F) == 12 * 16 and len(V) == 6 * 16 + 2
    vol, area = closed_and_outward(V, F)
    assert abs(vol - 0.01 * 0.02 * 0.05) < 1e-12
    assert abs(area - 2 * (0.01 * 0.02 + 0.01 * 0.05 + 0.02 * 0.05)) < 1e-12
    assert np.allclose(np.abs(V).max(axis=0), [0.005, 0.01, 0.025])
