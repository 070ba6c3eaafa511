"""Build recipe of the host build of the library's ExtendedMarchingCubes
passes (test infrastructure; see emc_host.cpp):

    python tests/emc_host/build.py   ->  tests/emc_host/_build/libemc_host.so
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "isosurface_gb300", "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libemc_host.so")
DEPS = [os.path.join(HERE, "emc_host.cpp")] + [os.path.join(CSRC, f) for f in
                                                ("emc.cuh", "emc_tables.h", "mc_tables.h", "qef.cuh", "qef_planes.cuh", "vm.cuh", "vm_math.cuh",
                                                 "internal.h")]
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in DEPS):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I", CUDA_INCLUDE, "-I", CSRC, "-I", os.path.join(ROOT, "include"),
           "-o", LIB + ".tmp", os.path.join(HERE, "emc_host.cpp")]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
