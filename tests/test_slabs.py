"""MarchingCubes sharded by z-slabs (isosurface_gb300/slabs.py).

On CPU the oracle's traversal of a slab (its cell layers plus the halo layer
below, which is what iso_mc_extract_slab leaves on a GPU) stands in for the
device, and the partition logic under test -- slab bounds, the halo-layer
drop, the renumbering, the one exchange of counts -- runs as written: in one
process for several world sizes, and as two gloo ranks.  The concatenated
per-rank buffers must equal the oracle's MarchingCubes of the whole grid byte
for byte.  The GPU tests run the same logic on iso_mc_extract_slab, and on
iso_dc_extract_slab (DualContouring's dual lattice, size - 1 as the size)
against iso_dc_extract and the oracle."""
import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from isosurface_gb300 import scenes, slabs
from isosurface_gb300 import source as S


def _oracle_slab(prog, size):
    """extract_slab(z0, z1) with the oracle: the layers [z0 - halo, z1) and
    the halo layer's vertex and triangle counts."""
    def extract(z0, z1):
        h = 1 if z0 > 0 else 0
        m = prog.marching_cubes_slab(size, z0 - h, z1)
        hv = ht = 0
        if h:
            hm = prog.marching_cubes_slab(size, z0 - 1, z0)
            hv, ht = len(hm.vertices), len(hm.indices) // 3
        return m.vertices, m.indices, m.keys, hv, ht
    return extract


def _concat(parts):
    v = np.concatenate([p[0] for p in parts]) if parts else np.zeros((0, 3), np.float32)
    i = np.concatenate([p[1] for p in parts])
    return v, i


def test_slab_bounds_cover_the_layers_once():
    for size in (2, 9, 65, 513):
        for world in (1, 2, 3, 8):
            if world > size:
                continue
            b = slabs.slab_bounds(size, world)
            assert b[0][0] == 0 and b[-1][1] == size
            assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
            assert max(z1 - z0 for z0, z1 in b) - min(z1 - z0 for z0, z1 in b) <= 1
    with pytest.raises(ValueError):
        slabs.slab_bounds(4, 5)


@pytest.mark.parametrize("name,size", [("sphere", 33), ("csg", 29), ("sphere_union", 41), ("bench_torus", 24)])
@pytest.mark.parametrize("world", [2, 3, 5])
def test_sharded_mesh_equals_whole_mesh(name, size, world):
    prog = oracle.Program(S.lower(getattr(scenes, name)()))
    want = prog.marching_cubes(size)
    extract = _oracle_slab(prog, size)
    # one process playing every rank: the counts the all-gather would bring
    counts = []
    for r, (z0, z1) in enumerate(slabs.slab_bounds(size, world)):
        v, i, k, hv, ht = extract(z0, z1)
        counts.append((len(v) - hv, len(i) // 3 - ht))
    bases = slabs.vertex_bases([c[0] for c in counts])
    out = []
    for r, (z0, z1) in enumerate(slabs.slab_bounds(size, world)):
        v, i, k, hv, ht = extract(z0, z1)
        out.append(slabs.assemble(v, i, k, hv, ht, z0, size, int(bases[r])))
    got_v, got_i = _concat(out)
    assert np.array_equal(got_v, want.vertices)
    assert np.array_equal(got_i, want.indices)
    # a single rank is the whole grid
    v, i, base, tbase = slabs.extract_sharded(extract, size, 0, 1)
    assert (base, tbase) == (0, 0)
    assert np.array_equal(v, want.vertices) and np.array_equal(i, want.indices)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


SIZE = 37


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    from isosurface_gb300 import replicas
    dist = replicas.init("gloo")
    try:
        prog = oracle.Program(S.lower(scenes.sphere_union(count=12, seed=5)))
        v, i, base, tbase = slabs.extract_sharded(_oracle_slab(prog, SIZE), SIZE, rank, world, dist)
        allparts = [None] * world
        dist.all_gather_object(allparts, (rank, v.tolist(), i.tolist(), base, tbase))
        if rank == 0:
            json.dump(allparts, open(os.path.join(out_dir, "parts.json"), "w"))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharded_mesh_equals_whole_mesh(tmp_path):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    parts = sorted(json.load(open(tmp_path / "parts.json")))
    want = oracle.Program(S.lower(scenes.sphere_union(count=12, seed=5))).marching_cubes(SIZE)
    got_v = np.concatenate([np.asarray(p[1], np.float32).reshape(-1, 3) for p in parts])
    got_i = np.concatenate([np.asarray(p[2], np.uint32) for p in parts])
    assert np.array_equal(got_v, want.vertices)
    assert np.array_equal(got_i, want.indices)
    # the exchanged counts place each rank's part
    assert parts[1][3] == len(parts[0][1]) and parts[1][4] == len(parts[0][2]) // 3


@pytest.mark.gpu
@pytest.mark.parametrize("name,size,worlds", [("sphere", 65, (2, 3, 7)), ("csg", 129, (2, 4)),
                                              ("sphere_union", 129, (3,))])
def test_device_slabs_equal_the_whole_extraction(ctx, name, size, worlds):
    """iso_mc_extract_slab on the device for every rank in turn, assembled by
    the same logic: the whole grid's buffers byte for byte (against the
    device's whole extraction and the oracle)."""
    src = getattr(scenes, name)()
    want = oracle.Program(S.lower(src)).marching_cubes(size)
    whole = ctx.download(ctx.mc_extract(src, size))
    assert np.array_equal(whole.vertices, want.vertices) and np.array_equal(whole.indices, want.indices)
    for world in worlds:
        counts, raw = [], []
        for z0, z1 in slabs.slab_bounds(size, world):
            v, i, k, hv, ht = slabs.extract_slab_device(ctx, src, size, z0, z1)
            raw.append((v, i, k, hv, ht, z0))
            counts.append(len(v) - hv)
        bases = slabs.vertex_bases(counts)
        out = [slabs.assemble(v, i, k, hv, ht, z0, size, int(b)) for (v, i, k, hv, ht, z0), b in zip(raw, bases)]
        got_v, got_i = _concat(out)
        assert np.array_equal(got_v, want.vertices), world
        assert np.array_equal(got_i, want.indices), world


@pytest.mark.gpu
def test_device_slabs_bench_grid(ctx):
    """The bench workload, MarchingCubes::new(513) of the 64-sphere union, in
    4 slabs: the whole device extraction's buffers byte for byte."""
    src = scenes.sphere_union()
    size = 513
    whole = ctx.download(ctx.mc_extract(src, size))
    counts, raw = [], []
    for z0, z1 in slabs.slab_bounds(size, 4):
        v, i, k, hv, ht = slabs.extract_slab_device(ctx, src, size, z0, z1)
        raw.append((v, i, k, hv, ht, z0))
        counts.append(len(v) - hv)
    bases = slabs.vertex_bases(counts)
    out = [slabs.assemble(v, i, k, hv, ht, z0, size, int(b)) for (v, i, k, hv, ht, z0), b in zip(raw, bases)]
    got_v, got_i = _concat(out)
    assert np.array_equal(got_v, whole.vertices)
    assert np.array_equal(got_i, whole.indices)


@pytest.mark.gpu
@pytest.mark.parametrize("name,size,worlds,placer", [("csg", 65, (2, 3, 7), 0), ("csg", 129, (2, 4), 0),
                                                     ("sphere", 65, (3,), 1), ("torus", 97, (2, 5), 0),
                                                     ("central_difference", 33, (2, 32), 1)])
def test_device_dc_slabs_equal_the_whole_extraction(ctx, name, size, worlds, placer):
    """iso_dc_extract_slab for every rank in turn (dual cube layers of the
    (size-1) x (size-1) x size dual lattice), assembled by the same logic
    with size - 1 as the size: iso_dc_extract's buffers byte for byte, and
    the oracle's DualContouring."""
    src = _dc_sources()[name]
    whole = ctx.download(ctx.dc_extract(src, size, placer))
    want = oracle.Program(S.lower(src)).dual_contouring(size, placer)
    assert np.array_equal(whole.vertices, want.vertices) and np.array_equal(whole.indices, want.indices)
    for world in worlds:
        counts, raw = [], []
        for z0, z1 in slabs.slab_bounds(size - 1, world):
            v, i, k, hv, ht = slabs.extract_dc_slab_device(ctx, src, size, z0, z1, placer)
            raw.append((v, i, k, hv, ht, z0))
            counts.append(len(v) - hv)
        bases = slabs.vertex_bases(counts)
        out = [slabs.assemble(v, i, k, hv, ht, z0, size - 1, int(b)) for (v, i, k, hv, ht, z0), b in zip(raw, bases)]
        got_v, got_i = _concat(out)
        assert np.array_equal(got_v, whole.vertices), world
        assert np.array_equal(got_i, whole.indices), world


def _dc_sources():
    return {"csg": scenes.csg(), "sphere": scenes.sphere(), "torus": S.unit_to_cube(S.Torus(0.5, 0.2)),
            "central_difference": S.unit_to_cube(S.CentralDifference(
                S.Intersection(S.Sphere(0.8), S.RectangularPrism((0.6, 0.6, 0.6)))))}


@pytest.mark.gpu
def test_device_dc_slab_arguments(ctx):
    from isosurface_gb300._capi import IsoError
    src = scenes.csg()
    for z0, z1 in ((0, 0), (3, 2), (0, 65)):  # empty, reversed, past the 64 dual cube layers of new(65)
        with pytest.raises(IsoError):
            ctx.dc_extract_slab(src, 65, z0, z1)
