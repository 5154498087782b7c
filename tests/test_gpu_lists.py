"""The interaction lists every product matvec reads, element by element and in order, against
the reference's own (tests/golden: FMMLevelSet, FMMLevelSetNumSR and genSRIdxArrs of
octree.c/translation.cu, and I2 ∩ leaf set, run on the same meshes by the reference's code).

* level sets: the plan's box order is the reference's fmmLevelSet order;
* M2L lists (sr_lists_kernel): per destination box the count srNumLevelArr, the sources
  srTransOriginArr and the destinations srTransDestArr, in order; the direction index of each
  translation is the box offset destination - source, and maps to one reference (rotation,
  coaxial) index pair and back;
* leaf near lists (near_boxes_kernel): I2 ∩ leaf set in I2's order (neighbours in x-y-z order,
  the box itself last, octree.c:497-505); the near-field rows of every element are those boxes'
  elements, box after box.
Large cases compare SHA-256 digests of the reference's arrays."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["ico2_r0.1_s5", "ico3_r0.1_s5", "ico3_r0.1_d3", "ico4_r0.3_s5", "ico5_r0.3_d5", "ico6_r0.3_d6"]


def _digest(a):
    a = np.ascontiguousarray(np.asarray(a, np.int32))
    return hashlib.sha256(a.astype("<i4").tobytes()).hexdigest()


def _xyz(num, l):
    num = np.asarray(num, np.int64)
    x = np.zeros_like(num)
    y = np.zeros_like(num)
    z = np.zeros_like(num)
    for b in range(l):
        d = (num >> (3 * (l - 1 - b))) & 7
        x = 2 * x + ((d >> 2) & 1)
        y = 2 * y + ((d >> 1) & 1)
        z = 2 * z + (d & 1)
    return np.stack([x, y, z], axis=1)


class Golden:
    def __init__(self, name):
        self.meta = json.load(open(os.path.join(GOLDEN, "octree_meta.json")))[name]
        self.g = np.load(os.path.join(GOLDEN, "octree_%s.npz" % name))
        near = np.load(os.path.join(GOLDEN, "octree_near.npz"))
        self.near = {k[len(name) + 1:]: near[k] for k in near.files if k.startswith(name + "_")}
        self.near_meta = json.load(open(os.path.join(GOLDEN, "octree_near_meta.json"))).get(name)

    def same(self, key, arr):
        """arr equals the reference's array `key` (full fixture or its digest)."""
        if key in self.g.files:
            return np.array_equal(np.asarray(arr), self.g[key])
        return _digest(arr) == self.meta["sha256"][key]

    def same_near(self, key, arr):
        if key in self.near:
            return np.array_equal(np.asarray(arr), self.near[key])
        return _digest(arr) == self.near_meta[key]


@pytest.mark.parametrize("name", CASES)
def test_plan_lists_equal_reference(fm, oracle, name):
    G = Golden(name)
    m = G.meta
    V, F = fm.icosphere(m["subdiv"], m["radius"])
    plan = fm.Plan(V, F, k=10.0, depth=m["depth"], s=m["s"], p_levels={l: 4 for l in range(2, 13)},
                   build_mixed=False)
    info = plan.info
    lmax = info.lmax
    assert lmax == int(G.g["lmax"])
    for l in range(2, lmax + 1):
        boxes, beg, src, dr, off = plan.lists(l)
        assert G.same("set_%d" % l, boxes), ("level set", l)
        assert G.same("srnum_%d" % l, np.diff(beg)), ("SR counts", l)
        assert G.same("sr_origin_%d" % l, src), ("SR origins", l)
        dst = np.repeat(np.arange(len(boxes)), np.diff(beg))
        assert G.same("sr_dest_%d" % l, boxes[dst]), ("SR destinations", l)
        # the direction of each translation is its box offset
        assert np.array_equal(_xyz(boxes[dst], l) - _xyz(boxes[src], l), off[dr]), ("directions", l)
        if "sr_rot_%d" % l in G.g.files:
            # one reference (rotation, coaxial) pair per direction and one direction per pair
            pairs = G.g["sr_rot_%d" % l].astype(np.int64) * 1000 + G.g["sr_coax_%d" % l]
            fwd, back = {}, {}
            for d, q in zip(dr.tolist(), pairs.tolist()):
                assert fwd.setdefault(d, q) == q and back.setdefault(q, d) == d, ("direction tables", l)
    bb, bi, eb, ec = plan.near_lists()
    assert G.same_near("beg", bb) and G.same_near("idx", bi), "leaf near boxes"
    # near-field rows: the elements of the near boxes, box after box, each box's in increasing order
    T = oracle.tree_for_fmm(V, F, depth=m["depth"] or None, s=m["s"])
    leaf = np.asarray(T["elem_leaf"])
    order = np.argsort(leaf, kind="stable")
    lb = np.concatenate([[0], np.cumsum(np.bincount(leaf, minlength=len(bb) - 1))])
    box_rows = [np.concatenate([order[lb[q]:lb[q + 1]] for q in bi[bb[b]:bb[b + 1]]]) for b in range(len(bb) - 1)]
    exp_len = np.array([len(box_rows[b]) for b in leaf])
    assert np.array_equal(np.diff(eb), exp_len), "near-field row lengths"
    for e in range(0, len(F), max(1, len(F) // 4096)):
        assert np.array_equal(ec[eb[e]:eb[e + 1]], box_rows[leaf[e]]), ("near-field row", e)
    plan.close()
