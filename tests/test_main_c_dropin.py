"""The reference's own driver program, main.c (main.c:18-45), builds unchanged against this
library's headers (include/) and links against libfmmbem.so alone, the way the reference's
makefile builds it (g++, makefile:199-200).  Host only: the reference tree is read where it
is mounted (the test skips elsewhere) and nothing is copied from it.

With LD_BIND_NOW every symbol the program uses is resolved when it loads, so a symbol that
libfmmbem.so lacks fails the run even before main().  Without a GPU the program then stops
at its first CUDA call (cudaDeviceReset) with the reference's own CUDA_CALL message; on a
GPU the calls it makes are checked by tests/test_gpu_legacy.py
(test_coaxial_truncation_like_reference_main)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAIN_C = "/root/reference/main.c"
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.mark.skipif(not os.path.exists(MAIN_C), reason="the reference tree is not mounted here")
def test_reference_main_c_builds_links_and_loads(fm, tmp_path):
    lib_dir = os.path.dirname(fm.lib()._name)
    exe = str(tmp_path / "main")
    # main.c is read from standard input, so that its quoted includes are not looked up beside
    # it, where the reference's own headers lie, but in this library's include/
    cmd = ["g++", "-x", "c++", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"), "-",
           "-L", lib_dir, "-lfmmbem", "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-o", exe]
    with open(MAIN_C) as src:
        res = subprocess.run(cmd, stdin=src, capture_output=True, text=True, cwd=str(tmp_path))
    assert res.returncode == 0, res.stdout + res.stderr
    env = dict(os.environ, LD_BIND_NOW="1",
               LD_LIBRARY_PATH=os.pathsep.join([lib_dir, os.path.join(CUDA, "lib64"), os.environ.get("LD_LIBRARY_PATH", "")]))
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True, env=env)
    assert "libfmmbem.so" in ldd.stdout and "not found" not in ldd.stdout, ldd.stdout
    run = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=120)
    out = run.stdout + run.stderr
    assert "symbol lookup error" not in out and "undefined symbol" not in out, out
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        # main.c prints the p = 2 matrix, then the p = 5 matrix truncated to p = 2: the same values
        assert run.returncode == 0, out
        rows = [ln for ln in run.stdout.splitlines() if ln.startswith("(")]
        assert len(rows) == 2, run.stdout
        a, b = (np.array([complex(float(u), float(v)) for u, v in re.findall(r"\(([^,]+),([^)]+)\)", r)]) for r in rows)
        assert len(a) == len(b) == 5 and np.allclose(a, b, rtol=1e-5, atol=1e-6), run.stdout
    else:
        # no device: the reference's CUDA_CALL(cudaDeviceReset()) reports and main returns EXIT_FAILURE
        assert run.returncode == 1 and "Error at" in run.stdout, out
