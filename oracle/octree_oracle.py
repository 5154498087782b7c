"""Octree oracle: a NumPy restatement of the reference's octree and interaction lists.

TEST INFRASTRUCTURE ONLY.  The GPU octree build is tested against this module; it is
imported by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg,
never by the product library.

Every function restates one reference routine (paths are within the reference project):

* ``read_obj``            -- ``octree.c:563-619`` (``findNum``/``readOBJ``), including the
  48-character ``fgets`` chunking and the rule that any line starting with 'v' is a vertex.
* ``tri_centroids``       -- ``structs.cu:126-131`` (``triCentroid_d``), same operation order.
* ``bounding_cube``       -- ``octree.c:681-747`` (``findBoundingCube``) including the bug
  that seeds ``z_min``/``z_max`` from the *y* coordinate of the first point.
* ``morton``              -- ``octree.c:88-183`` (``dec2bin_frac``/``bitIntleave``/
  ``indArr2num``/``pnt2boxnum``).  Repeated doubling with exact subtraction produces the
  binary digits of ``s``, i.e. ``floor(s * 2**l)`` per axis, interleaved as 4x+2y+z.
* ``deter_lmax``          -- ``octree.c:635-679`` (``deterLmax``), returning 11 on a tie
  exactly as the reference does.
* ``first_occurrence_set``-- ``octree.c:393-410`` (``createSet``): dedupe preserving the
  order of first occurrence.
* ``fmm_level_sets``      -- ``octree.c:816-831``, ``890-906`` (``prntLevelSet``/
  ``FMMLevelSet``).
* ``neighbors``/``i2``/``i4`` -- ``octree.c:237-391``, ``497-543`` in the reference's
  enumeration order (x outer, then y, then z; the box itself appended last).
* ``sr_lists``            -- ``octree.c:908-919`` (``FMMLevelSetNumSR``) and
  ``translation.cu:2848-2922`` (``genSRIdxArrs`` origin/destination arrays).
* ``btm_lvl_elem_idx``    -- ``translation.cu:3062-3076``: the element-to-leaf index computed
  from *float* vertices and a float centroid (``integral.cu:659-664``).
* ``ss_rr_lists``         -- ``translation.cu:2797-2846``, ``2924-2969``.

Parity of this oracle is pinned against the reference's own ``octree.c`` compiled here
(``oracle/build_ref.sh``) through the fixtures in ``tests/golden``.
"""
from __future__ import annotations

import numpy as np

LMIN = 2


# ----------------------------------------------------------------------------- mesh input
def read_obj(path):
    """Parse an OBJ file the way ``readOBJ`` does (``octree.c:586-619``).

    ``fgets(line, 49, fp)`` reads at most 48 characters, so a longer line is split and each
    chunk is classified by its first character.  ``sscanf("%s %lf %lf %lf")`` parses the
    chunk; fields that fail to parse keep whatever the destination held (the reference reads
    into freshly malloc'd memory; we use 0.0, which only matters for malformed files).
    Faces are 1-based in the file and stored 0-based.
    """
    verts, faces = [], []
    with open(path, "rb") as fh:
        data = fh.read().decode("latin-1")
    for chunk in _fgets_chunks(data, 48):
        if not chunk:
            continue
        if chunk[0] == "v":
            toks = chunk.split()
            vals = []
            for t in toks[1:4]:
                try:
                    vals.append(float(_c_float_prefix(t)))
                except ValueError:
                    break
            while len(vals) < 3:
                vals.append(0.0)
            verts.append(vals)
        if chunk[0] == "f":
            toks = chunk.split()
            vals = []
            for t in toks[1:4]:
                pre = _c_int_prefix(t)
                if pre is None:
                    break
                vals.append(pre - 1)
            while len(vals) < 3:
                vals.append(-1)
            faces.append(vals)
    return np.asarray(verts, dtype=np.float64).reshape(-1, 3), np.asarray(faces, dtype=np.int64).reshape(-1, 3)


def _fgets_chunks(text, n):
    out = []
    for line in text.splitlines(keepends=True):
        while len(line) > n:
            out.append(line[:n])
            line = line[n:]
        if line:
            out.append(line)
    return out


def _c_int_prefix(tok):
    i = 0
    if i < len(tok) and tok[i] in "+-":
        i += 1
    j = i
    while j < len(tok) and tok[j].isdigit():
        j += 1
    if j == i:
        return None
    return int(tok[:j])


def _c_float_prefix(tok):
    # strtod accepts the longest valid prefix; OBJ files hold plain decimals.
    best = None
    for j in range(len(tok), 0, -1):
        try:
            float(tok[:j])
            best = tok[:j]
            break
        except ValueError:
            continue
    if best is None:
        raise ValueError(tok)
    return best


# ----------------------------------------------------------------------------- geometry
def tri_centroids(V, F):
    """``triCentroid_d`` (``structs.cu:126-131``): n0 + (2/3)*(0.5*(n1+n2) - n0)."""
    n0, n1, n2 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    c23 = 0.5 * (n1 + n2)
    return n0 + (2.0 / 3.0) * (c23 - n0)


def bounding_cube(P, eps=0.01):
    """``findBoundingCube`` (``octree.c:681-747``); returns (pt_min, d).

    The reference seeds z_min and z_max with P[0].y (bug kept for bit-exactness).
    """
    x_min = x_max = P[0, 0]
    y_min = y_max = P[0, 1]
    z_min = z_max = P[0, 1]
    if len(P) > 1:
        x_min = min(x_min, P[1:, 0].min())
        x_max = max(x_max, P[1:, 0].max())
        y_min = min(y_min, P[1:, 1].min())
        y_max = max(y_max, P[1:, 1].max())
        z_min = min(z_min, P[1:, 2].min())
        z_max = max(z_max, P[1:, 2].max())
    eps_d = 0.000001 * min(min(x_max - x_min, y_max - y_min), z_max - z_min)
    eps_d = min(eps, eps_d)
    x_max += eps_d; x_min -= eps_d
    y_max += eps_d; y_min -= eps_d
    z_max += eps_d; z_min -= eps_d
    d_x = x_max - x_min; d_y = y_max - y_min; d_z = z_max - z_min
    d_max = max(max(d_x, d_y), d_z)
    x_min -= (d_max - d_x) / 2
    y_min -= (d_max - d_y) / 2
    z_min -= (d_max - d_z) / 2
    return np.array([x_min, y_min, z_min], dtype=np.float64), float(d_max)


def scale(P, pt_min, d):
    """``scale`` (``octree.c:62-69``): (x - x_min)/d per axis."""
    return (P - pt_min[None, :]) / d


def morton(S, l):
    """``pnt2boxnum`` (``octree.c:158-183``) for an (n,3) array of scaled points."""
    f = float(2 ** l)
    ix = np.floor(S[:, 0] * f).astype(np.int64)
    iy = np.floor(S[:, 1] * f).astype(np.int64)
    iz = np.floor(S[:, 2] * f).astype(np.int64)
    key = np.zeros(len(S), dtype=np.int64)
    for b in range(l - 1, -1, -1):
        digit = 4 * ((ix >> b) & 1) + 2 * ((iy >> b) & 1) + ((iz >> b) & 1)
        key = key * 8 + digit
    return key


def box_coords(num, l):
    """Integer (x, y, z) of a Morton box number (inverse of the interleave)."""
    x = y = z = 0
    for b in range(l):
        digit = (num >> (3 * (l - 1 - b))) & 7
        x = (x << 1) | ((digit >> 2) & 1)
        y = (y << 1) | ((digit >> 1) & 1)
        z = (z << 1) | (digit & 1)
    return x, y, z


def box_number(x, y, z, l):
    key = 0
    for b in range(l - 1, -1, -1):
        key = key * 8 + 4 * ((x >> b) & 1) + 2 * ((y >> b) & 1) + ((z >> b) & 1)
    return key


def box_center(num, l):
    """``boxCenter`` (``octree.c:185-235``): 2^-l * t + 2^-(l+1) per axis (unit cube)."""
    x, y, z = box_coords(num, l)
    h = 2.0 ** (-l)
    return np.array([h * x + 2.0 ** (-l - 1), h * y + 2.0 ** (-l - 1), h * z + 2.0 ** (-l - 1)])


def deter_lmax(S, s):
    """``deterLmax`` (``octree.c:635-679``)."""
    keys = np.sort(morton(S, 10))
    n = len(keys)
    l_max = 0
    for i in range(0, n - s):
        a, b = int(keys[i]), int(keys[i + s])
        if a == b:
            return 11
        l = 10
        while a != b:
            l -= 1
            a //= 8
            b //= 8
        l_max = max(l_max, l + 1)
    return l_max


def first_occurrence_set(vals):
    """``createSet`` (``octree.c:393-410``): unique values in first-occurrence order."""
    vals = np.asarray(vals, dtype=np.int64)
    _, first = np.unique(vals, return_index=True)
    return vals[np.sort(first)]


def fmm_level_sets(leaf_set, lmax):
    """``FMMLevelSet`` (``octree.c:890-906``): list indexed by l-2, l = 2..lmax."""
    sets = [None] * (lmax - LMIN + 1)
    sets[lmax - LMIN] = np.asarray(leaf_set, dtype=np.int64)
    for l in range(lmax - 1, LMIN - 1, -1):
        sets[l - LMIN] = first_occurrence_set(sets[l + 1 - LMIN] // 8)
    return sets


def neighbors(num, l):
    """``neighbors`` (``octree.c:237-391``): up to 26 boxes, x outer / z inner, self excluded."""
    x, y, z = box_coords(num, l)
    top = 2 ** l - 1

    def rng(t):
        if t == 0:
            return [t, t + 1]
        if t == top:
            return [t - 1, t]
        return [t - 1, t, t + 1]

    out = []
    for xi in rng(x):
        for yi in rng(y):
            for zi in rng(z):
                t = box_number(xi, yi, zi, l)
                if t != num:
                    out.append(t)
    return out


def i2(num, l):
    """``I2`` (``octree.c:497-505``): neighbours then the box itself."""
    return neighbors(num, l) + [num]


def i4(num, l):
    """``I4`` (``octree.c:517-543``): children of the parent's neighbourhood (parent's
    neighbours in enumeration order, then the parent) minus the box's own neighbourhood."""
    near = set(neighbors(num, l) + [num])
    p = num // 8
    pn = neighbors(p, l - 1) + [p]
    out = []
    for q in pn:
        for c in range(8):
            ch = 8 * q + c
            if ch not in near:
                out.append(ch)
    return out


def sr_lists(level_sets, lmax):
    """``FMMLevelSetNumSR`` + ``genSRIdxArrs`` origin/destination arrays.

    Returns per level (l-2): (num_sr[B], origin_idx[T], dest_box[T]) where origin_idx is
    the index into the level set of the source box, and dest_box the destination's
    Morton number (the reference stores box numbers there, ``translation.cu:2890``).
    """
    out = []
    for l in range(LMIN, lmax + 1):
        s = level_sets[l - LMIN]
        pos = {int(b): i for i, b in enumerate(s)}
        num, org, dst = [], [], []
        for b in s:
            c = 0
            for q in i4(int(b), l):
                if q in pos:
                    org.append(pos[q])
                    dst.append(int(b))
                    c += 1
            num.append(c)
        out.append((np.asarray(num, np.int64), np.asarray(org, np.int64), np.asarray(dst, np.int64)))
    return out


def ss_rr_lists(level_sets, lmax):
    """``ssTransDestArr``/``rrTransOriginArr``: parent index of each box, levels lmax..3."""
    out = {}
    for l in range(LMIN + 1, lmax + 1):
        s = level_sets[l - LMIN]
        ps = level_sets[l - 1 - LMIN]
        pos = {int(b): i for i, b in enumerate(ps)}
        out[l] = np.asarray([pos[int(b) // 8] for b in s], dtype=np.int64)
    return out


def near_lists(level_sets, lmax):
    """Leaf-level near list per box: I2 ∩ leaf set, as indices into the leaf set."""
    s = level_sets[lmax - LMIN]
    pos = {int(b): i for i, b in enumerate(s)}
    return [[pos[q] for q in i2(int(b), lmax) if q in pos] for b in s]


def btm_lvl_elem_idx(V, F, pt_min, d, leaf_set, lmax):
    """``translation.cu:3062-3076``: leaf index of each element from a float centroid.

    Vertices are first cast to float (``genOctree`` stores ``cartCoord``), the centroid is
    computed in float by ``triCentroid`` (``integral.cu:659-664``, factor
    ``(float)(2.0/3.0)``), scaled in double, cast back to float, and located at ``lmax``.
    Elements whose float box is not in the leaf set get -1, as ``findSetInd`` returns.
    """
    Vf = V.astype(np.float32)
    n0, n1, n2 = Vf[F[:, 0]], Vf[F[:, 1]], Vf[F[:, 2]]
    c23 = np.float32(0.5) * (n1 + n2)
    ctr = n0 + np.float32(2.0 / 3.0) * (c23 - n0)
    sc = ((ctr.astype(np.float64) - pt_min[None, :]) / d).astype(np.float32).astype(np.float64)
    keys = morton(sc, lmax)
    pos = {int(b): i for i, b in enumerate(leaf_set)}
    return np.asarray([pos.get(int(k), -1) for k in keys], dtype=np.int64)


def build(V, F, s=5, depth=None):
    """The ``srcBoxes`` + ``FMMLevelSet`` pipeline (``octree.c:749-768``).

    With ``depth`` given, ``deterLmax`` is skipped and the leaf level is ``depth``.
    Returns a dict with the reference's octree fields.
    """
    C = tri_centroids(V, F)
    pt_min, d = bounding_cube(C, 0.01)
    S = scale(C, pt_min, d)
    lmax = deter_lmax(S, s) if depth is None else int(depth)
    leaf = first_occurrence_set(morton(S, lmax))
    sets = fmm_level_sets(leaf, lmax)
    return {
        "lmax": lmax,
        "d": d,
        "pt_min": pt_min,
        "level_sets": sets,
        "elem_leaf_key": morton(S, lmax),
    }
