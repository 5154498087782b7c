"""Synthetic test meshes (NumPy), written as OBJ text so both sides parse the same bytes.

The icosphere is built from the 12-vertex icosahedron by midpoint subdivision with every
new vertex projected to the sphere; faces are counter-clockwise seen from outside, so the
normal (n0-n2)x(n1-n2) points outward.  Coordinates are written with 9 significant digits,
keeping every OBJ line under the 48 characters that the reference's reader takes per
``fgets`` call.
"""
import numpy as np


def icosphere(subdiv, radius):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, dtype=np.float64) for v in V]
    V = [v / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) for v in V]
    for _ in range(subdiv):
        cache = {}
        newF = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = 0.5 * (V[a] + V[b])
                V.append(m / np.sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]))
                cache[key] = len(V) - 1
            return cache[key]

        for (a, b, c) in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            newF += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = newF
    V = np.asarray(V) * radius
    return V, np.asarray(F, dtype=np.int64)


def obj_text(V, F):
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in V]
    lines += ["f %d %d %d" % (f[0] + 1, f[1] + 1, f[2] + 1) for f in F]
    return "\n".join(lines) + "\n"


def write_obj(path, V, F):
    with open(path, "w") as fh:
        fh.write(obj_text(V, F))


def roundtrip(V, F):
    """Vertices as parsed back from the OBJ text (what every reader sees)."""
    Vr = np.array([[float("%.9g" % c) for c in v] for v in V], dtype=np.float64)
    return Vr, np.asarray(F, dtype=np.int64)


def fibonacci_sphere(n, radius):
    i = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    theta = np.pi * (1 + 5 ** 0.5) * i
    return radius * np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], axis=1)
