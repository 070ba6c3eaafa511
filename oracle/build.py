"""Build recipe of the oracle (test infrastructure; see iso_oracle.cpp's header).

    python oracle/build.py      ->  oracle/_build/libiso_oracle.so

-ffp-contract=off keeps gcc from fusing a*b+c (it does by default on aarch64),
because the reference's Rust arithmetic never fuses.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libiso_oracle.so")
SOURCES = [os.path.join(HERE, "iso_oracle.cpp")]
DEPS = SOURCES + [os.path.join(HERE, "program.h"), os.path.join(HERE, "ref_tables.h")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in DEPS)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-o", LIB + ".tmp"] + SOURCES + ["-lpthread"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
