"""Build recipe for the oracle shared library (test infrastructure only).

Compiles ``oracle/oracle.cpp`` (the C++ restatement of the Feel++ assembly
path) with g++ into ``oracle/_build/liboracle.so``. No reference sources are
compiled: the reference needs PETSc, Boost, Eigen, MPI and GiNaC, none of
which exist here, so it is unbuildable and the restatement stands in for it.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(HERE, "quad_tables.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(src), os.path.getmtime(hdr), os.path.getmtime(__file__))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-o", tmp, src]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
