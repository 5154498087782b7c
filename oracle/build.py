"""Build the C oracle and the port of the reference's CPU octree build (test and baseline
infrastructure) into oracle/_build/liboracle.so.

Only the test suite, ``__graft_entry__`` and ``bench.py``'s CPU-baseline leg use the
oracle.  ``build_reference()`` compiles the reference project's own sources through
``oracle/build_ref.sh`` when the reference tree is mounted.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfmmref.so")


def build(force=False):
    srcs = [os.path.join(HERE, f) for f in ("fmm_oracle.c", "octree_port.c")]
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-std=gnu99"] + srcs + [
        "-o", LIB, "-lm"]
    subprocess.check_call(cmd)
    return LIB


def build_reference(ref_dir="/root/reference"):
    if not os.path.exists(os.path.join(ref_dir, "octree.c")):
        return None
    env = dict(os.environ, FMMBEM_REFERENCE_DIR=ref_dir)
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")], env=env)
    return REF_LIB
