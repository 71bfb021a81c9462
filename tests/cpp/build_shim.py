"""Compile tests/cpp/shim_poisson.cpp (a Feel++-style program on include/fgpu_feel.hpp) with g++
and link it against the in-tree libfgpu.so; the binary goes to tests/cpp/_build/."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIBDIR = os.path.join(ROOT, "feelpp_gb300", "_lib")


def build():
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "shim_poisson")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "shim_poisson.cpp"), "-o", exe, "-L", LIBDIR, "-lfgpu", "-Wl,-rpath," + LIBDIR]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


if __name__ == "__main__":
    print(build())
