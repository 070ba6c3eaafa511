"""Batched MarchingCubes over many uneven chunks (the 4096-chunk workload's
machinery): every chunk's mesh must equal the oracle's MarchingCubes on that
chunk byte for byte, for the eager run, the CUDA-graph replay, the autotuned
slab depths and the one-extraction-per-chunk path."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S
from isosurface_gb300.api import Batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chunk_set():
    return scenes.chunks(seed=7, count=48)


@pytest.fixture(scope="module")
def want(chunk_set):
    return [oracle.Program(S.lower(src)).marching_cubes(size) for size, src in chunk_set]


def _check(meshes, want):
    assert len(meshes) == len(want)
    for got, w in zip(meshes, want):
        assert np.array_equal(got.vertices, w.vertices)
        assert np.array_equal(got.indices, w.indices)


def test_batch_eager_graph_and_per_chunk(ctx, chunk_set, want):
    b = Batch(ctx, chunk_set)
    info = b.run(graph=False)
    _check(b.meshes(info), want)
    for _ in range(2):  # first graph run captures, the second replays
        info = b.run(graph=True)
        _check(b.meshes(info), want)
    info = b.run_per_chunk()
    _check(b.meshes(info), want)
    for _ in range(2):
        info = b.run_per_chunk_async()
        _check(b.meshes(info), want)
    b.close()


def test_batch_slab_depths_and_autotune(ctx, chunk_set, want, tmp_path):
    b = Batch(ctx, chunk_set)
    for depth in (1, 3, 0):
        b.set_slab(0, depth)
        _check(b.meshes(b.run(graph=False)), want)
    cache = str(tmp_path / "autotune.txt")
    chosen = b.autotune(cache)
    assert set(chosen) == {17, 33, 65} & set(size for size, _ in chunk_set)
    _check(b.meshes(b.run(graph=True)), want)
    _check(b.meshes(b.run(graph=True)), want)
    # a second tuner run reads the cache and picks the same depths
    b2 = Batch(ctx, chunk_set)
    assert b2.autotune(cache) == chosen
    b.close()
    b2.close()


def test_batch_same_program_many_sizes(ctx):
    src = scenes.sphere()
    chunks = [(s, src) for s in (2, 3, 17, 33, 40, 65)]
    b = Batch(ctx, chunks)
    meshes = b.meshes(b.run(graph=False))
    for (size, _), got in zip(chunks, meshes):
        w = oracle.Program(S.lower(src)).marching_cubes(size)
        assert np.array_equal(got.vertices, w.vertices) and np.array_equal(got.indices, w.indices)
    b.close()


def test_batch_graph_survives_mesh_buffer_regrowth(ctx, chunk_set, want):
    """The captured graph writes into the context's mesh buffers; a larger
    extraction in between regrows (reallocates) them, and the next replay must
    notice and capture again instead of writing to the freed buffers."""
    b = Batch(ctx, chunk_set)
    b.run(graph=False)
    b.run(graph=True)
    big = ctx.mc_extract(scenes.sphere_union(), 385)  # many more vertices than the batch
    assert big.num_vertices > 0
    info = b.run(graph=True)
    _check(b.meshes(info), want)
    b.close()


def test_batch_4096_chunk_workload(ctx):
    """The batch workload itself: the 4096 seeded chunks (50 % 16^3, 35 %
    32^3, 15 % 64^3 cells, 1-16 random primitives each) extracted in one
    CUDA graph replay; every chunk's mesh equals the oracle's MarchingCubes
    of that chunk byte for byte.  The oracle runs on all host cores."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    chunk_set = scenes.chunks(seed=7, count=4096)
    b = Batch(ctx, chunk_set)
    b.run(graph=True)               # eager run, sizes the graph
    meshes = b.meshes(b.run(graph=True))
    b.close()
    assert len(meshes) == 4096

    def check(i):
        size, src = chunk_set[i]
        w = oracle.Program(S.lower(src)).marching_cubes(size)
        return np.array_equal(meshes[i].vertices, w.vertices) and np.array_equal(meshes[i].indices, w.indices)

    with ThreadPoolExecutor(max(1, os.cpu_count() or 1)) as pool:
        ok = list(pool.map(check, range(len(chunk_set))))
    bad = [i for i, good in enumerate(ok) if not good]
    assert not bad, "chunks differing from the oracle: %s" % bad[:20]
    assert sum(len(m.indices) for m in meshes) // 3 > 20_000_000
