"""The C-ABI library builds, loads without a GPU, and exports every function declared in
include/*.h.  CPU only."""
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in sorted(os.listdir(INCLUDE)):
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", text)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name in ("if", "while", "for", "return", "sizeof", "typedef", "struct"):
                continue
            names.add(name)
    return names


def test_library_exports_every_declared_function(fm):
    from fmbem_gpu_c_gb300 import LIB_PATH

    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = declared_functions()
    assert len(declared) > 80
    missing = sorted(declared - exported)
    assert not missing, missing
    for var in ("INTPT_h", "INTWGT_h"):
        assert var in exported


def test_host_only_entry_points_work_without_gpu(fm):
    o = fm.default_options()
    assert o.s == 5 and abs(o.eps - 0.05) < 1e-12 and o.b_re == 1.0
    V, F = fm.icosphere(3, 0.1)
    assert V.shape == (642, 3) and F.shape == (1280, 3)
    n = np.cross(V[F[:, 0]] - V[F[:, 2]], V[F[:, 1]] - V[F[:, 2]])
    c = V[F].mean(axis=1)
    assert (np.einsum("ij,ij->i", n, c) > 0).all(), "faces must be counter-clockwise seen from outside"
