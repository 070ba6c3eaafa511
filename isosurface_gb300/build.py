"""Build the CUDA library in-tree:  isosurface_gb300/_build/libisosurface_gpu.so

    python -m isosurface_gb300.build [--force]

One nvcc per translation unit, in parallel, for sm_103a only, then one link.
The translation units whose arithmetic must match the reference's f32 order
are compiled with -fmad=false (no a*b+c contraction; IEEE sqrt and division
are nvcc's defaults and stay on).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libisosurface_gpu.so")
# the FP32 FMA-rate probe the benchmark reports the sampler against (not part
# of the extraction library)
PEAK_SRC = os.path.join(CSRC, "fp32_peak.cu")
PEAK_LIB = os.path.join(OUT_DIR, "libiso_fp32_peak.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags
UNITS = {
    "ctx.cu": ["-fmad=false"],
    "sample.cu": ["-fmad=false"],
    "mc.cu": ["-fmad=false"],
    "dc.cu": ["-fmad=false"],
    "lhmc.cu": ["-fmad=false"],
    "batch.cu": ["-fmad=false"],
    "mlp.cu": [],
    "mlp_infer.cu": [],
    "surrogate.cu": ["-fmad=false"],
    "splat.cu": ["-fmad=false"],
    "emc.cu": ["-fmad=false"],
    "jit.cu": ["-fmad=false"],
}
HEADERS = ["internal.h", "vm.cuh", "vm_math.cuh", "bricks.cuh", "bricks_core.cuh", "mc_tables.h", "mc_chunk.cuh",
           "qef.cuh", "qef_planes.cuh", "dc_core.cuh", "mlp.h", "emc.cuh", "emc_tables.h"]
# sources the library compiles again at run time, for one program at a time
# (jit.cu): embedded as string literals in _build/jit_sources.inc
JIT_SOURCES = (("kJitVmMath", "vm_math.cuh"), ("kJitBricksCore", "bricks_core.cuh"),
               ("kJitQefPlanes", "qef_planes.cuh"), ("kJitDcCore", "dc_core.cuh"))
JIT_INC = os.path.join(OUT_DIR, "jit_sources.inc")


def _write_jit_sources():
    parts = ["// written by isosurface_gb300/build.py from csrc/" + ", ".join(f for _, f in JIT_SOURCES) + "\n"]
    for name, fname in JIT_SOURCES:
        text = open(os.path.join(CSRC, fname)).read()
        text = "".join(l for l in text.splitlines(True) if l.strip() != "#pragma once")
        assert ")ISOJIT\"" not in text
        parts.append("static const char %s[] = R\"ISOJIT(%s)ISOJIT\";\n" % (name, text))
    data = "".join(parts)
    if not os.path.exists(JIT_INC) or open(JIT_INC).read() != data:
        with open(JIT_INC, "w") as f:
            f.write(data)


def _deps():
    paths = [os.path.join(CSRC, u) for u in UNITS] + [os.path.join(CSRC, h) for h in HEADERS]
    paths.append(os.path.join(ROOT, "include", "isosurface_gpu.h"))
    paths.append(os.path.abspath(__file__))
    return [p for p in paths if os.path.exists(p)]


def _compile(unit, flags):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT_DIR, unit + ".o")
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "-I", os.path.join(ROOT, "include"), "-I", OUT_DIR, "-c", src, "-o", obj, *flags]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
    return obj


def _build_peak(force):
    if not force and os.path.exists(PEAK_LIB) and os.path.getmtime(PEAK_LIB) >= os.path.getmtime(PEAK_SRC):
        return
    cmd = [NVCC, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-cudart", "shared", PEAK_SRC,
           "-o", PEAK_LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for fp32_peak.cu:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(PEAK_LIB + ".tmp", PEAK_LIB)


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    _write_jit_sources()
    _build_peak(force)
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in _deps()):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(UNITS))) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    # -ldl: the NVTX ranges dlopen a profiler's injection library when one is
    # attached (dlopen is in libc from glibc 2.34, in libdl before)
    cmd = [NVCC, *ARCH, "-shared", "-cudart", "shared", "-o", LIB + ".tmp", *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
