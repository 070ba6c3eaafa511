"""Benchmark: cells/s meshed at 512^3 (MarchingCubes::new(513) on the seeded
64-sphere union over [-1,1]^3).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one MarchingCubes extraction of the whole 512 x 512 x 513-cell
grid (the reference's traversal visits 513 cell layers): sampling, cell
classification + scan, vertex/index emission.  `value` is timed with CUDA
events on the library's stream with the program already resident and the
mesh left on the device; `e2e` times the public C ABI with host buffers
(program upload H2D from host bytes, iso_mc_extract_host into page-locked
host buffers) on the host clock, from two host threads with a context each
(steps back to back; the mesh delivered by DMA, ISO_FLAG_HOST_COPY), and
`e2e.serial` the same from one thread.  L2 is flushed (a 256 MiB write)
before every timed step of `value` and `e2e.serial`; a step's working set
(540 MB) exceeds L2 in the two-thread run.

`roofline` covers the extraction pass (counting, scan, emission, resolve):
achieved = (4 B per sample for the field read once + 12 B per vertex + 12 B
per triangle) / that pass's event-timed duration, against the measured HBM
copy bandwidth; `traffic` is the DRAM bytes ncu measured for the same
kernels (profiles/traffic.json).

--impl reference times the oracle (the C++ restatement of the reference's
single-threaded Rust CPU path; Rust does not build here) on all host cores,
each step a bounded slab of the same grid.

Multi-GPU (torchrun, N > 1): the grid is split into N z-slabs, one per GPU,
with one all-gather of two counts per rank (run_sharded; strong scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZE = 513
CELLS = (SIZE - 1) * (SIZE - 1) * SIZE
METRIC = "cells/s meshed at 512^3"
WORKLOAD = {"workload": "MarchingCubes::new(513), hard-min union of 64 spheres (seed 1234), [-1,1]^3",
            "cells": CELLS, "samples": SIZE * SIZE * (SIZE + 1), "l2": "flushed (256 MiB write) before each step"}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# the kernels whose DRAM traffic profiles/traffic.json records; a capture
# counts only for the sources it was taken from
# every source of the translation units that hold the extraction's kernels
TRAFFIC_SOURCES = ["isosurface_gb300/csrc/" + f for f in
                   ("mc.cu", "mc_chunk.cuh", "mc_tables.h", "sample.cu", "bricks.cuh", "bricks_core.cuh", "vm.cuh",
                    "vm_math.cuh", "internal.h")] + ["include/isosurface_gpu.h"]


def kernel_sources_sha256():
    """Hash of the extraction kernels' sources with comments and blank lines
    removed (a comment edit leaves the captured kernels as they were)."""
    import hashlib
    import re
    h = hashlib.sha256()
    for rel in TRAFFIC_SOURCES:
        with open(os.path.join(ROOT, rel)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        lines = [l.rstrip() for l in text.splitlines() if l.strip()]
        h.update("\n".join(lines).encode())
    return h.hexdigest()


def measured_traffic():
    """DRAM bytes (read + write) per extraction of the extraction kernels,
    from the ncu capture recorded in profiles/traffic.json, or None when that
    capture was taken from other kernel sources than the ones built now."""
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tpath):
        return None, "no ncu capture recorded"
    t = json.load(open(tpath))
    if t.get("sources_sha256") != kernel_sources_sha256():
        return None, "the recorded ncu capture predates the current kernel sources"
    return t["classify_scan"] + t["emit"], "ncu capture of these kernel sources (profiles/traffic.json)"


def fp32_peak():
    """Measured FP32 rate (FMA chains on every SM, CUDA events): TFLOP/s."""
    import ctypes
    from isosurface_gb300 import build as gbuild
    L = ctypes.CDLL(gbuild.PEAK_LIB)
    L.iso_fp32_fma_peak.restype = ctypes.c_int
    L.iso_fp32_fma_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double)]
    tf, ms = ctypes.c_double(), ctypes.c_double()
    rc = L.iso_fp32_fma_peak(0, 10, ctypes.byref(tf), ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError("fp32 peak probe failed: CUDA error %d" % rc)
    return tf.value


# flops per sphere of a hard union as the reference evaluates it: p - c (3),
# |p - c| (3 mul, 2 add, 1 sqrt), minus r (1), min with the running value (1)
FLOPS_PER_SPHERE = 11


def sampler_fp32_workload(ctx, torch, timed):
    """The sampler against the FP32 rate: the same 64-sphere union written as
    nested Union(Translate(Sphere)) nodes, which the library samples with its
    general evaluator (every sphere at every sample, no culling), into the
    full f32 field of MarchingCubes::new(513): the program compiled for its
    own kernel, and beside it the interpreter; flops per sample = the domain
    map (3 mul + 3 add) + 64 x FLOPS_PER_SPHERE."""
    from isosurface_gb300 import scenes
    from isosurface_gb300 import source as S
    sph = scenes.random_spheres(1234, 64, 0.8, (0.05, 0.25))
    node = None
    for cx, cy, cz, r in sph:
        t = S.Translate(S.Sphere(float(r)), (float(cx), float(cy), float(cz)))
        node = t if node is None else S.Union(node, t)
    src = S.unit_to_cube(node)
    from isosurface_gb300._capi import lib
    field = torch.empty((SIZE + 1) * SIZE * SIZE, dtype=torch.float32, device="cuda")
    prog = ctx.program(src)
    samples = SIZE * SIZE * (SIZE + 1)
    flops = samples * (6 + 64 * FLOPS_PER_SPHERE)
    peak = fp32_peak()
    ms = {}
    # the program compiled for its own full-field kernel (what iso_sample_grid
    # runs; the warm-up compiles it), then the interpreter
    for enable in (1, 0):
        lib().iso_jit_enable(enable)
        try:
            for _ in range(2):
                ctx.sample_grid(prog, SIZE, field.data_ptr(), SIZE)
            ms[enable] = timed(lambda: ctx.sample_grid(prog, SIZE, field.data_ptr(), SIZE), 5)
        finally:
            lib().iso_jit_enable(1)
    del field
    achieved = flops / (ms[1] / 1e3) / 1e12
    interp = flops / (ms[0] / 1e3) / 1e12
    return {"bound": "fp32", "workload": "64-sphere union (seed 1234) as nested Union(Translate(Sphere)), general "
                                         "evaluator compiled for the program, full f32 field of MarchingCubes::new(513)",
            "ms": ms[1], "flops_per_sample": 6 + 64 * FLOPS_PER_SPHERE, "achieved_tflops": achieved,
            "peak_tflops": peak, "peak_source": "measured (FMA chains, libiso_fp32_peak)", "frac": achieved / peak,
            "interpreted": {"ms": ms[0], "achieved_tflops": interp, "frac": interp / peak}}


def mc_csg_workload(ctx, timed, steps):
    """A general program at the headline size: MarchingCubes::new(513) of the
    rigid-transformed CSG scene (box minus sphere, union torus), sampled by
    the culled sampler with the program's compiled evaluator (the first
    extraction compiles it: `first_ms`, host clock), device-resident, CUDA
    events; `interpreted_ms` is the same with compilation switched off."""
    import ctypes
    from isosurface_gb300 import scenes
    from isosurface_gb300._capi import lib
    src = scenes.csg()
    prog = ctx.program(src)
    t0 = time.perf_counter()
    info = ctx.mc_extract(prog, SIZE)
    first_ms = 1e3 * (time.perf_counter() - t0)
    for _ in range(2):
        info = ctx.mc_extract(prog, SIZE)
    ms = timed(lambda: ctx.mc_extract(prog, SIZE), max(5, min(steps, 30)))
    compiled = ctx.compiled(prog)
    lib().iso_jit_enable(0)
    try:
        for _ in range(2):
            ctx.mc_extract(prog, SIZE)
        interpreted_ms = timed(lambda: ctx.mc_extract(prog, SIZE), max(5, min(steps, 30)))
    finally:
        lib().iso_jit_enable(1)
    for _ in range(2):
        ctx.mc_extract(prog, SIZE)
    ms_buf = (ctypes.c_double * 8)()
    ln_buf = (ctypes.c_uint64 * 8)()
    lib().iso_ctx_stage_times(ctx.h, ms_buf, ln_buf)
    lib().iso_ctx_enable_stage_timing(ctx.h, 1)
    for _ in range(5):
        ctx.mc_extract(prog, SIZE)
    lib().iso_ctx_stage_times(ctx.h, ms_buf, ln_buf)
    lib().iso_ctx_enable_stage_timing(ctx.h, 0)
    stages = {name: ms_buf[i] / max(int(ln_buf[i]), 1) for name, i in (("sample", 0), ("classify_scan", 1),
                                                                          ("emit", 2))}
    return {"cells": CELLS, "ms": ms, "cells_per_s": CELLS / (ms / 1e3), "triangles": int(info.num_triangles),
            "vertices": int(info.num_vertices), "stage_ms": stages, "compiled": bool(compiled),
            "first_ms": first_ms, "interpreted_ms": interpreted_ms}


def cpu_baseline_port(src_bytes, budget_s=12.0, threads=1):
    """The oracle's MarchingCubes over a bounded middle slab of the same grid."""
    import oracle
    prog = oracle.Program(src_bytes)
    mid = SIZE // 2
    secs, cells, _ = prog.mc_timed(SIZE, mid, mid + 2 * threads, threads)
    per_layer = secs / (2 * threads)
    layers = max(threads, int(budget_s / max(per_layer, 1e-6)) * threads)
    layers = min(layers, SIZE - 1)
    z0 = max(0, mid - layers // 2)
    secs, cells, tris = prog.mc_timed(SIZE, z0, z0 + layers, threads)
    return {"value": cells / secs, "unit": "cells/s", "cores": threads, "kind": "port",
            "sample": "oracle MarchingCubes over cell layers [%d, %d) of the 512^3 grid (%d cells, %.1f s)"
                      % (z0, z0 + layers, cells, secs)}


def secondary_workloads(ctx, torch, steps, only=None, per_chunk=True):
    """The other workloads, timed with CUDA events on the library's stream:
    the sampler against the measured FP32 rate, MarchingCubes::new(513) of a
    general CSG program, the 4096-chunk batch (one CUDA graph vs one
    extraction per chunk),
    DualContouring at 256^3, LinearHashedMarchingCubes at depth 8, the
    reference's own benchmark shapes and the deferred point-splat frame
    (`only`: a set of names among refshapes, batch, dc, lhmc, splat to run
    just those; names: sampler, csg, refshapes, batch, dc, lhmc, splat, emc)."""
    from isosurface_gb300 import scenes
    stream = torch.cuda.ExternalStream(ctx.stream)

    def timed(fn, reps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        return min(a.elapsed_time(b) for a, b in ev)

    out = {}
    want = (lambda name: only is None or name in only)
    if want("sampler"):
        out["sampler_fp32_512"] = sampler_fp32_workload(ctx, torch, timed)
    if want("csg"):
        out["mc_512_csg"] = mc_csg_workload(ctx, timed, steps)
    if want("refshapes"):
        out["reference_bench_shapes"] = _reference_bench_shapes(ctx, timed, steps)
    if want("batch"):
        out.update(_batch_workload(ctx, timed, steps, per_chunk))
    src = scenes.csg()
    if want("dc"):
        for _ in range(2):
            info = ctx.dc_extract(src, 257)
        ms = timed(lambda: ctx.dc_extract(src, 257), max(3, min(steps, 20)))
        out["dc_256"] = {"cells": int(info.num_cells), "ms": ms, "cells_per_s": 256 * 256 * 257 / (ms / 1e3),
                         "triangles": int(info.num_triangles), "placer": "MinimiseQEF"}
    if want("lhmc"):
        for _ in range(2):
            info = ctx.lhmc_extract(src, 8)
        ms = timed(lambda: ctx.lhmc_extract(src, 8), max(3, min(steps, 20)))
        out["lhmc_depth8"] = {"dual_cubes": int(info.num_cells), "ms": ms, "triangles": int(info.num_triangles)}
    if want("splat"):
        out["point_splat_1024x768"] = _point_splat_frame(ctx, steps)
    if want("emc"):
        out["emc_128"] = _emc_workload(ctx, timed, steps)
    return out


def _emc_workload(ctx, timed, steps):
    """ExtendedMarchingCubes::new(128), the viewer's largest grid
    (examples/sampler.rs:100-118), of a CSG scene with the Directed metric
    (box minus sphere, union torus, centred in the sample frame); GPU time
    with CUDA events beside the single-threaded oracle's."""
    import oracle
    from isosurface_gb300 import source as S
    src = S.Translate(S.Union(S.Difference(S.Sphere(0.35), S.RectangularPrism((0.3, 0.3, 0.3))),
                              S.Torus(0.25, 0.06)), (0.5, 0.5, 0.5))
    for _ in range(3):
        info, flips = ctx.emc_extract(src, 128)
    gpu_ms = timed(lambda: ctx.emc_extract(src, 128), max(3, min(steps, 20)))
    t0 = time.time()
    m = oracle.Program(S.lower(src)).extended_marching_cubes(128)
    cpu_ms = 1e3 * (time.time() - t0)
    return {"cells": int(info.num_cells), "gpu_ms": gpu_ms, "cpu_baseline_ms": cpu_ms, "cpu_threads": 1,
            "vertices": int(info.num_vertices), "triangles": int(info.num_triangles), "flips": int(flips),
            "feature_vertices": int(m.features),
            "matches_oracle": bool(info.num_vertices == len(m.vertices) and 3 * info.num_triangles == len(m.indices))}


def _point_splat_frame(ctx, steps):
    """The deferred-rasterisation example's frame (examples/deferred_rasterisation.rs):
    PointCloud::new(64) of the centred torus with normals, splatted and
    gathered at 1024 x 768 into a host image; host-timed per frame,
    including the 12.6 MB image readback."""
    from isosurface_gb300 import scenes
    info = ctx.point_cloud_extract(scenes.demo_torus(), 64, normals=True)
    for _ in range(3):
        img = ctx.point_splat(1024, 768, 0.5 / 64)
    reps = max(5, min(steps, 50))
    t0 = time.perf_counter()
    for _ in range(reps):
        img = ctx.point_splat(1024, 768, 0.5 / 64)
    ms = 1e3 * (time.perf_counter() - t0) / reps
    return {"points": int(info.num_vertices), "ms_per_frame": ms, "lit_pixels": int((img[..., 3] == 1.0).sum())}


def _reference_bench_shapes(ctx, timed, steps):
    """The reference's own benchmark shapes (benches/isosurface.rs): Torus(0.25,
    0.1) at the origin, MarchingCubes::new(128) and LinearHashedMarchingCubes::
    new(7), on the GPU and with the single-threaded oracle beside them."""
    import oracle
    from isosurface_gb300 import scenes
    from isosurface_gb300 import source as S
    src = scenes.bench_torus()
    prog = ctx.program(src)
    o = oracle.Program(S.lower(src))
    out = {}
    for _ in range(3):
        info = ctx.mc_extract(prog, 128)
    gpu_ms = timed(lambda: ctx.mc_extract(prog, 128), max(5, min(steps, 20)))
    secs, cells, _ = o.mc_timed(128, 0, 128, 1)
    out["mc_128_torus"] = {"cells": int(info.num_cells), "gpu_ms": gpu_ms, "cpu_baseline_ms": 1e3 * secs,
                           "cpu_threads": 1, "triangles": int(info.num_triangles)}
    for _ in range(2):
        info = ctx.lhmc_extract(prog, 7)
    gpu_ms = timed(lambda: ctx.lhmc_extract(prog, 7), max(5, min(steps, 20)))
    t0 = time.time()
    o.lhmc(7)
    out["lhmc_7_torus"] = {"gpu_ms": gpu_ms, "cpu_baseline_ms": 1e3 * (time.time() - t0), "cpu_threads": 1,
                           "triangles": int(info.num_triangles)}
    return out


def _batch_workload(ctx, timed, steps, per_chunk=True):
    from isosurface_gb300 import scenes
    from isosurface_gb300.api import Batch
    out = {}
    chunks = scenes.chunks(seed=7, count=4096)
    batch = Batch(ctx, chunks)
    cache = os.path.join(ROOT, "isosurface_gb300", "_build", "autotune.txt")
    chosen = batch.autotune(cache)
    batch.run(graph=False)
    batch.run(graph=True)
    graph_ms = timed(lambda: batch.run(graph=True), max(3, min(steps, 20)))
    info = batch.run(graph=True)
    cells = info.num_cells
    out["batch_4096_chunks"] = {"cells": int(cells), "graph_ms": graph_ms, "cells_per_s": cells / (graph_ms / 1e3),
                                "triangles": int(info.num_triangles), "slab_depth_by_size": chosen}
    if per_chunk:
        per_ms = timed(batch.run_per_chunk, 2)
        batch.run_per_chunk_async()
        async_ms = timed(batch.run_per_chunk_async, 3)
        out["batch_4096_chunks"].update({"per_chunk_ms": per_ms, "per_chunk_no_sync_ms": async_ms,
                                         "speedup": per_ms / graph_ms, "speedup_vs_no_sync": async_ms / graph_ms})
    batch.close()
    return out


MLP_FLOPS_PER_POINT = 2 * (96 * 256 + 5 * 256 * 256 + 256)


def surrogate_workload(ctx, torch, train_steps):
    """The learned surrogate on the 4096-sphere smooth union (k = 0.05) at
    512^3: train the network (16M samples, Adam), then time the exact path
    (the brute O(4096)-per-point sampler, then marching cubes) against the
    surrogate path (network on every 4th lattice point, exact re-sampling of
    points within `band` cells of its surface, marching cubes), both with CUDA
    events on the library's stream, and score each surrogate mesh against the
    exact mesh (nearest-vertex Chamfer / Hausdorff in cells, fraction of cells
    whose corner signs differ)."""
    import ctypes
    from isosurface_gb300 import scenes
    from isosurface_gb300._capi import lib
    from isosurface_gb300.surrogate import Surrogate, case_disagreement, mesh_distance
    stream = torch.cuda.ExternalStream(ctx.stream)

    def timed(fn, reps):
        best = None
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r = fn()
            b.record(stream)
            torch.cuda.synchronize()
            best = a.elapsed_time(b) if best is None else min(best, a.elapsed_time(b))
        return best, r

    src = scenes.smooth_spheres()
    net = Surrogate(ctx, seed=5)
    t0 = time.time()
    net.make_dataset(src.source, 1 << 24, -1.0, 1.0, seed=9)
    hist = net.train(train_steps, batch=65536, lr=2e-3)
    train_s = time.time() - t0
    size, pitch = SIZE, SIZE
    nz = size + 1
    field = torch.empty((nz * size * pitch,), dtype=torch.float32, device="cuda")
    sfield = torch.empty_like(field)
    torch.cuda.synchronize()

    def exact_path():
        ctx.sample_grid(src, size, field.data_ptr(), pitch)
        return ctx.mc_extract_field(field.data_ptr(), size, size, nz, pitch)

    exact_ms, info = timed(exact_path, 2)
    exact = ctx.download(info)
    # the library's own exact extraction of the same program: the culled
    # sampler (every sample's sign, exact values only near the surface, the
    # set's 4096 spheres at every evaluated point), then marching cubes; the
    # same mesh as the full-field path
    ctx.mc_extract(src, size)
    exact_culled_ms, cinfo = timed(lambda: ctx.mc_extract(src, size), 2)
    culled = ctx.download(cinfo)
    culled_same = bool(np.array_equal(culled.vertices, exact.vertices) and np.array_equal(culled.indices, exact.indices))
    cell = 1.0 / (size - 1)
    out = {"workload": "MarchingCubes::new(513) of a smooth-min (k=0.05) union of 4096 spheres (seed 99), "
                       "exact sampler O(4096) per point",
           "train": {"samples": 1 << 24, "steps": train_steps, "batch": 65536, "seconds": train_s,
                     "loss_first": float(hist[0]), "loss_last": float(np.mean(hist[-20:]))},
           "exact_ms": exact_ms, "exact_triangles": int(info.num_triangles),
           "exact_culled_ms": exact_culled_ms, "exact_culled_same_mesh": culled_same, "bands": {}}
    # the least an exact mesh can re-sample: every end of a crossing edge lies
    # within one lattice step of the exact surface (the field is 1-Lipschitz),
    # and such points are this fraction of the grid, which bounds any
    # band-re-sampling surrogate's speed-up by its inverse
    near = int((field.view(nz, size, pitch)[:, :, :size].abs() <= 2.0 * cell).sum().item())
    out["exact_fraction_within_one_step"] = near / float(nz * size * size)
    out["speedup_bound"] = float(nz * size * size) / max(near, 1)
    ms_buf = (ctypes.c_double * 8)()
    ln_buf = (ctypes.c_uint64 * 8)()
    variants = [("%g" % b, b, False, False) for b in (1.0, 2.0)]
    variants += [("%g+witness" % b, b, False, True) for b in (1.5, 2.0, 3.0)]
    variants += [("%g+witness, exact coarse grid (no network)" % b, b, True, True) for b in (1.0, 2.0)]
    for name, band, exact_coarse, witness in variants:
        def surrogate_path():
            st = net.field_ex(src, size, sfield.data_ptr(), pitch, coarse_step=4, band_cells=band,
                              exact_coarse=exact_coarse, witness=witness)
            return st, ctx.mc_extract_field(sfield.data_ptr(), size, size, nz, pitch)

        surrogate_path()
        ms, (st, sinfo) = timed(surrogate_path, 3)
        lib().iso_ctx_stage_times(ctx.h, ms_buf, ln_buf)
        lib().iso_ctx_enable_stage_timing(ctx.h, 1)
        surrogate_path()
        lib().iso_ctx_stage_times(ctx.h, ms_buf, ln_buf)
        lib().iso_ctx_enable_stage_timing(ctx.h, 0)
        mlp_ms, band_ms = ms_buf[6], ms_buf[0]
        m = ctx.download(sinfo)
        d = mesh_distance(ctx, m.vertices, exact.vertices, 2 * cell, max_rings=64)
        dis = case_disagreement(ctx, field.data_ptr(), sfield.data_ptr(), size, size, nz, pitch)
        out["bands"][name] = {
            "ms": ms, "speedup_vs_exact": exact_ms / ms, "speedup_vs_exact_culled": exact_culled_ms / ms,
            "band_fraction": st["band_points"] / st["total_points"],
            "flagged_spheres": st["flagged"], "coarse_points": st["coarse_points"],
            "coarse_from": "exact source" if exact_coarse else "network", "network_ms": mlp_ms,
            "exact_resample_ms": band_ms,
            "network_tflops": (MLP_FLOPS_PER_POINT * st["coarse_points"] / (mlp_ms / 1e3) / 1e12
                               if not exact_coarse and mlp_ms > 0 else None),
            "chamfer_cells": d["chamfer"] / cell, "hausdorff_cells": d["hausdorff"] / cell,
            "distance_search_capped": d["capped"],
            "case_disagreement": dis / float((size - 1) * (size - 1) * size), "triangles": int(sinfo.num_triangles)}
    net.close()
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from isosurface_gb300 import scenes
    from isosurface_gb300 import source as S
    import oracle
    threads = os.cpu_count() or 1
    prog = oracle.Program(S.lower(scenes.sphere_union()))
    # size each step to a few seconds of work
    mid = SIZE // 2
    secs, _, _ = prog.mc_timed(SIZE, mid, mid + threads, threads)
    # each step a bounded sample: the whole run stays near the budget
    per_step = min(3.0, args.reference_budget / max(1, args.steps + args.warmup))
    layers = max(threads, int(per_step / max(secs, 1e-6)) * threads)
    layers = min(layers, SIZE - 1)
    z0 = max(0, mid - layers // 2)
    for _ in range(args.warmup):
        prog.mc_timed(SIZE, z0, z0 + layers, threads)
    total_s, total_cells = 0.0, 0
    for _ in range(args.steps):
        s, c, _ = prog.mc_timed(SIZE, z0, z0 + layers, threads)
        total_s += s
        total_cells += c
    value = total_cells / total_s
    out = {"metric": METRIC, "value": value, "unit": "cells/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": dict(WORKLOAD, sample_layers=[z0, z0 + layers]),
           "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                            "sample": "oracle (C++ restatement of the reference's CPU path) over cell layers "
                                      "[%d, %d) per step, split across %d threads" % (z0, z0 + layers, threads)},
           "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_sharded(args, torch, dist, world, rank, ctx, stream, src):
    """N > 1: the grid split into N z-slabs, one per GPU (isosurface_gb300/slabs.py):
    each rank samples and meshes its cell layers plus one halo layer, the
    ranks exchange their (vertices, triangles) counts with one NCCL
    all-gather, and each renumbers its triangles into the whole mesh.  Strong
    scaling: the whole 512^3 grid per step across the N GPUs.  `value` times
    the device extraction and the exchange with CUDA events (max over
    ranks); `e2e` adds the mesh's copy to host memory and the renumbering on
    the host.  Not measured on hardware: this pool lends one GPU per run."""
    from isosurface_gb300 import replicas, slabs
    z0, z1 = slabs.slab_bounds(SIZE, world)[rank]
    prog = ctx.program(src)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        info, hv, ht = ctx.mc_extract_slab(prog, SIZE, z0, z1, keys=True)
        slabs.all_gather_counts(info.num_vertices - hv, info.num_triangles - ht, dist)
        return info, hv, ht

    for _ in range(args.warmup):
        step()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    dist.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    launches0 = ctx.kernel_launches
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    ms = replicas.max_over_ranks(sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps, dist, "cuda")
    e2e_times = []
    for k in range(max(3, min(args.steps, 50))):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        v, i, base, tbase = slabs.extract_sharded(lambda a, b: slabs.extract_slab_device(ctx, prog, SIZE, a, b),
                                                  SIZE, rank, world, dist)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = replicas.max_over_ranks(sum(e2e_times) / len(e2e_times), dist, "cuda")
    batch_line = None if args.no_secondary else sharded_batch_workload(ctx, torch, dist, world, rank, stream)
    if rank == 0:
        out = {"metric": METRIC, "value": CELLS / (ms / 1e3), "unit": "cells/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": dict(WORKLOAD, parallelism="z-slabs x%d (one NCCL all-gather of 2 counts per rank)" % world),
               "e2e": {"value": CELLS / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 12 * len(v) + 4 * len(i), "ms_per_step": 1e3 * e2e_s,
                       "note": "rank 0's slab bytes"},
               "gpu_launches": int(launches), "clocks": clk, "roofline": None, "cpu_baseline": None}
        if batch_line:
            out["secondary"] = {"batch_4096_chunks_sharded": batch_line}
        print(json.dumps(out))
    ctx.close()
    dist.destroy_process_group()


def sharded_batch_workload(ctx, torch, dist, world, rank, stream):
    """N > 1: the 4096-chunk batch sharded over the ranks
    (isosurface_gb300/batch_shards.py: size-balanced round robin, each rank's
    chunks as one CUDA graph, one all-gather of four counts per rank at the
    end).  Strong scaling: the whole batch per step across the N GPUs, timed
    with CUDA events (max over ranks)."""
    from isosurface_gb300 import batch_shards, replicas, scenes
    chunks = scenes.chunks(seed=7, count=4096)
    mine, batch, info = batch_shards.run_shard(ctx, chunks, rank, world)
    for _ in range(2):
        batch.run(graph=True)
    reps = 10
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    torch.cuda.synchronize()
    dist.barrier()
    for a, b in ev:
        a.record(stream)
        info = batch.run(graph=True)
        b.record(stream)
    torch.cuda.synchronize()
    ms = replicas.max_over_ranks(sum(a.elapsed_time(b) for a, b in ev) / reps, dist, "cuda")
    counts = batch_shards.gather_counts(len(mine), info.num_cells, info.num_vertices, info.num_triangles, dist,
                                        "cuda")
    batch.close()
    cells = sum(c[1] for c in counts)
    return {"ms": ms, "cells": cells, "cells_per_s": cells / (ms / 1e3), "scaling": "strong",
            "chunks_per_rank": [c[0] for c in counts], "cells_per_rank": [c[1] for c in counts],
            "vertices": sum(c[2] for c in counts), "triangles": sum(c[3] for c in counts)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-budget", type=float, default=90.0,
                    help="--impl reference: seconds of oracle work across all steps (each step at most 3 s)")
    ap.add_argument("--no-secondary", action="store_true", help="skip the batch / DC / LHMC timings")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the learned-surrogate workload")
    ap.add_argument("--secondary-only", default=None,
                    help="comma list among sampler,csg,refshapes,batch,dc,lhmc,splat,surrogate,emc: run only these "
                         "secondary "
                         "workloads (emc runs only when named)")
    ap.add_argument("--surrogate-train-steps", type=int, default=4000)
    ap.add_argument("--no-per-chunk", action="store_true",
                    help="batch workload: time the batch graph only, not the one-extraction-per-chunk comparisons "
                         "(for profiling, where their 65 K launches are slow)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    from isosurface_gb300 import replicas
    world, rank, local = replicas.rank_env()
    torch.cuda.set_device(local)
    dist = replicas.init("nccl")

    from isosurface_gb300 import build as gbuild
    gbuild.build()
    from isosurface_gb300 import Context, scenes
    from isosurface_gb300 import source as S
    from isosurface_gb300._capi import lib

    src = scenes.sphere_union()
    src_bytes = S.lower(src)
    ctx = Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    if world > 1:
        run_sharded(args, torch, dist, world, rank, ctx, stream, src)
        return
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    prog = ctx.program(src)  # uploaded once, as a caller holding a program would
    for _ in range(args.warmup):
        info = ctx.mc_extract(prog, SIZE)
    import ctypes
    ms_buf = (ctypes.c_double * 8)()
    ln_buf = (ctypes.c_uint64 * 8)()

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.kernel_launches
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
        info = ctx.mc_extract(prog, SIZE)
        ends[k].record(stream)
    barrier()
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    # per-stage device times: a separate pass of the same extractions with the
    # library's stage events on (they run eagerly, kernel for kernel the same)
    lib().iso_ctx_stage_times(ctx.h, ms_buf, ln_buf)  # reset
    lib().iso_ctx_enable_stage_timing(ctx.h, 1)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        ctx.mc_extract(prog, SIZE)
    torch.cuda.synchronize()
    lib().iso_ctx_stage_times(ctx.h, ms_buf, ln_buf)
    lib().iso_ctx_enable_stage_timing(ctx.h, 0)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = replicas.max_over_ranks(sum(step_ms) / len(step_ms), dist, "cuda")
    value = replicas.whole_job_rate(CELLS, world, ms / 1e3)

    # per-stage device time (CUDA events on the launching stream) and the
    # roofline of the extraction pass (counting, scan, emission, resolve): the
    # unit the workload's bytes are defined for -- the field read once (4 B per
    # sample) plus the mesh written (12 B per vertex, 12 B per triangle).  The
    # library reads sign bits and near-surface values instead of the field, so
    # its measured traffic is below that figure.
    nv, nt = info.num_vertices, info.num_triangles
    samples = SIZE * SIZE * (SIZE + 1)
    words = (SIZE + 31) // 32
    stage_ix = {"sample": 0, "classify_scan": 1, "emit": 2}
    per_stage = {}
    total_ms = max(sum(ms_buf[i] for i in stage_ix.values()), 1e-9)
    for name, i in stage_ix.items():
        n = max(int(ln_buf[i]), 1)
        per_stage[name] = {"ms_per_launch": ms_buf[i] / n, "launches": int(ln_buf[i]), "share": ms_buf[i] / total_ms}
    extract_ms = per_stage["classify_scan"]["ms_per_launch"] + per_stage["emit"]["ms_per_launch"]
    algo = 4 * samples + 12 * nv + 12 * nt
    peak, peak_kind = peaks()
    achieved = algo / (extract_ms / 1e3) / 1e9
    traffic, traffic_note = measured_traffic()
    roofline = {"bound": "hbm", "kernel": "extraction (mc_chunk_count, mc_range_scan, mc_cell_emit, mc_resolve_ids)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic, "traffic_source": traffic_note, "algorithmic_bytes": algo,
                "ms_per_launch": extract_ms,
                "sampler": {"ms_per_launch": per_stage["sample"]["ms_per_launch"],
                            "bytes_written": 4 * words * SIZE * (SIZE + 1) + 8 * nv,
                            "note": "sign bits of every sample and exact values only near the surface"}}

    # e2e through the public C ABI with host buffers
    from isosurface_gb300._capi import MeshInfo, check
    vbuf = torch.empty((nv * 3 + 1024,), dtype=torch.float32, pin_memory=True)
    ibuf = torch.empty((nt * 3 + 1024,), dtype=torch.int32, pin_memory=True)
    f32p, u32p = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32)

    def e2e_step(c=ctx, vb=vbuf, ib=ibuf, flags=0):
        # a program uploaded from host bytes and the mesh delivered into the
        # caller's page-locked buffers, as a binding's extract() would do
        ph = ctypes.c_void_p()
        check(lib().iso_program_create(c.h, src_bytes, len(src_bytes), ctypes.byref(ph)), c.h)
        mi = MeshInfo()
        check(lib().iso_mc_extract_host(c.h, ph, SIZE, flags, ctypes.cast(vb.data_ptr(), f32p), vb.numel(),
                                        ctypes.cast(ib.data_ptr(), u32p), ib.numel(), ctypes.byref(mi)), c.h)
        lib().iso_program_destroy(ph)
        return mi

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mi = e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    barrier()
    e2e_s = replicas.max_over_ranks(sum(e2e_times) / len(e2e_times), dist, "cuda")
    serial_mesh = (vbuf[:3 * mi.num_vertices].clone(), ibuf[:3 * mi.num_triangles].clone())
    # the same calls from two host threads, each with its own context (and
    # stream) and page-locked buffers, steps back to back, with the mesh
    # delivered by the DMA engines after each extraction (ISO_FLAG_HOST_COPY):
    # one extraction's mesh crosses the CPU-GPU link while the other samples,
    # counts and emits on the SMs.  The working set of a step (540 MB of sign
    # bits and values, the 53 MB mesh) is larger than L2, so nothing carries
    # over between steps.
    ctx2 = Context(local)
    stream2 = torch.cuda.Stream()
    ctx2.set_stream(stream2.cuda_stream)
    lanes = [(ctx, vbuf, ibuf),
             (ctx2, torch.empty_like(vbuf).pin_memory(), torch.empty_like(ibuf).pin_memory())]
    HOST_COPY = 4  # ISO_FLAG_HOST_COPY
    for c, vb, ib in lanes:
        for _ in range(max(args.warmup, 2)):
            e2e_step(c, vb, ib, HOST_COPY)
    barrier()
    errors = []
    # both threads exist and wait at the gate before the clock starts, so the
    # timed region holds the steps and not the threads' start-up
    gate = threading.Barrier(len(lanes) + 1)

    def lane(c, vb, ib):
        gate.wait()
        try:
            for _ in range(args.steps):
                e2e_step(c, vb, ib, HOST_COPY)
        except Exception as exc:  # reported after the join
            errors.append(exc)

    threads = [threading.Thread(target=lane, args=l) for l in lanes]
    for t in threads:
        t.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gate.wait()
    for t in threads:
        t.join()
    pipe_s = (time.perf_counter() - t0) / (len(lanes) * args.steps)
    if errors:
        raise errors[0]
    same = all(torch.equal(vb[:3 * mi.num_vertices], serial_mesh[0]) and
               torch.equal(ib[:3 * mi.num_triangles], serial_mesh[1]) for _, vb, ib in lanes)
    pipe_s = replicas.max_over_ranks(pipe_s, dist, "cuda")
    ctx2.close()
    e2e = {"value": replicas.whole_job_rate(CELLS, world, pipe_s), "unit": "cells/s",
           "h2d_bytes_per_step": len(src_bytes), "d2h_bytes_per_step": 12 * mi.num_vertices + 12 * mi.num_triangles,
           "ms_per_step": 1e3 * pipe_s,
           "schedule": "two host threads, one context and stream each, steps back to back, "
                       "mesh delivered by DMA after each extraction (ISO_FLAG_HOST_COPY)",
           "meshes_equal_serial": bool(same),
           "serial": {"value": replicas.whole_job_rate(CELLS, world, e2e_s), "ms_per_step": 1e3 * e2e_s,
                      "l2": "flushed before each step",
                      "schedule": "one thread, mesh written to the host buffers by the extraction kernels"}}

    secondary = None
    if not args.no_secondary:
        only = set(args.secondary_only.split(",")) if args.secondary_only else None
        secondary = secondary_workloads(ctx, torch, args.steps, only, per_chunk=not args.no_per_chunk)
        if not args.no_surrogate and (only is None or "surrogate" in only):
            secondary["surrogate_512"] = surrogate_workload(ctx, torch, args.surrogate_train_steps)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_port(src_bytes)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": dict(WORKLOAD, parallelism="replicas" if world > 1 else "single", vertices=nv,
                              triangles=nt),
               "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "stages": per_stage,
               "cpu_baseline": cpu, "clocks": clk, "secondary": secondary}
        print(json.dumps(out))
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
