"""The port of the reference's CPU octree build (oracle/octree_port.c), which bench.py times
as the CPU baseline of the octree stage, gives the reference's own level sets and SR counts
(tests/golden, produced by the reference's octree.c), so its timing is that of the same
work.  Host only."""
import hashlib
import json
import os

import numpy as np
import pytest

import meshes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _digest(a):
    a = np.ascontiguousarray(np.asarray(a, np.int32))
    return hashlib.sha256(a.astype("<i4").tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["ico2_r0.1_s5", "ico3_r0.1_s5", "ico3_r0.1_d3", "ico4_r0.3_s5", "ico5_r0.3_d5"])
def test_port_matches_reference_octree(oracle, name):
    meta = json.load(open(os.path.join(GOLDEN, "octree_meta.json")))[name]
    g = np.load(os.path.join(GOLDEN, "octree_%s.npz" % name))
    # the vertices the reference read: OBJ text with 9 significant digits
    V, F = meshes.roundtrip(*meshes.icosphere(meta["subdiv"], meta["radius"]))
    T = oracle.port_octree(V, F, s=meta["s"], depth=meta["depth"])
    assert T["lmax"] == int(g["lmax"])
    for l in range(2, T["lmax"] + 1):
        assert np.array_equal(T["set_%d" % l], g["set_%d" % l]), l
        if "srnum_%d" % l in g.files:
            assert np.array_equal(T["srnum_%d" % l], g["srnum_%d" % l]), l
        else:
            assert _digest(T["srnum_%d" % l]) == meta["sha256"]["srnum_%d" % l], l


def test_port_sampled_run_scales_the_sr_stage(oracle):
    V, F = meshes.roundtrip(*meshes.icosphere(4, 0.3))
    full = oracle.port_octree(V, F, s=5)
    part = oracle.port_octree(V, F, s=5, sr_sample=200)
    lm = full["lmax"]
    ran = part["srnum_%d" % lm] >= 0
    assert 0 < ran.sum() < len(ran)
    assert np.array_equal(part["srnum_%d" % lm][ran], full["srnum_%d" % lm][ran])
    assert part["times"]["sr_lists_s"] >= part["times"]["sr_lists_s_run"]
