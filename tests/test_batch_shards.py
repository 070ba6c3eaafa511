"""The chunk batch sharded across ranks (isosurface_gb300/batch_shards.py), on
CPU: the size-balanced round-robin partition, and two `gloo` ranks that each
mesh their share of the chunks (the oracle stands in for the device: the
layout under test is the host-side one) and gather their counts, against a
single-process run over every chunk."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from isosurface_gb300 import batch_shards as B
from isosurface_gb300 import scenes


def _workload_sizes():
    return [size for size, _ in scenes.chunks(seed=7, count=4096)]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_each_chunk_once_and_balances(world):
    sizes = _workload_sizes()
    parts = B.partition(sizes, world)
    assert len(parts) == world
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(sizes)))
    assert all(p == sorted(p) for p in parts)
    counts = [len(p) for p in parts]
    assert max(counts) - min(counts) <= 1
    cells = B.rank_cells(sizes, parts)
    assert sum(cells) == sum(B.chunk_cells(s) for s in sizes)
    assert max(cells) - min(cells) <= max(B.chunk_cells(s) for s in sizes)
    if world > 1:  # the workload's 223.7 M cells split to within 1 % (one 65^3 chunk: 266 K cells)
        assert max(cells) / min(cells) < 1.01


def test_partition_balance_on_random_sizes():
    rng = np.random.default_rng(11)
    for _ in range(200):
        n = int(rng.integers(0, 300))
        world = int(rng.integers(1, 9))
        sizes = [int(s) for s in rng.choice([2, 5, 9, 17, 33, 65, 129], size=n)]
        parts = B.partition(sizes, world)
        assert sorted(i for p in parts for i in p) == list(range(n))
        counts = [len(p) for p in parts]
        assert max(counts) - min(counts) <= 1
        cells = B.rank_cells(sizes, parts)
        biggest = max((B.chunk_cells(s) for s in sizes), default=0)
        assert max(cells) - min(cells) <= biggest


def test_chunk_cells_and_bad_world():
    assert B.chunk_cells(513) == 512 * 512 * 513
    assert B.chunk_cells(17) == 16 * 16 * 17
    assert B.chunk_cells(1) == 0
    with pytest.raises(ValueError):
        B.partition([17], 0)


def test_assemble_restores_chunk_order():
    parts = [[0, 3, 4], [1, 2]]
    got = B.assemble(parts, [["a", "d", "e"], ["b", "c"]])
    assert got == ["a", "b", "c", "d", "e"]
    with pytest.raises(ValueError):
        B.assemble(parts, [["a"], ["b", "c"]])


def test_gather_counts_single_process():
    assert B.gather_counts(3, 100, 7, 9, None) == [[3, 100, 7, 9]]


CHUNKS = 24


def _chunks():
    # small chunks of the batch workload's scene kinds, uneven sizes
    rng = scenes.SplitMix64(5)
    sizes = [9, 17, 13, 9, 21, 17]
    return [(sizes[i % len(sizes)], scenes.chunk_scene(rng)) for i in range(CHUNKS)]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _mesh(size, src):
    import oracle
    from isosurface_gb300 import source as S
    m = oracle.Program(S.lower(src)).marching_cubes(size)
    return np.asarray(m.vertices, np.float32).reshape(-1), np.asarray(m.indices, np.uint32).reshape(-1)


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    from isosurface_gb300 import replicas
    dist = replicas.init("gloo")
    try:
        chunks = _chunks()
        parts = B.partition([s for s, _ in chunks], world)
        mine = parts[rank]
        meshes = [_mesh(*chunks[i]) for i in mine]
        nv = sum(len(v) // 3 for v, _ in meshes)
        nt = sum(len(i) // 3 for _, i in meshes)
        counts = B.gather_counts(len(mine), sum(B.chunk_cells(chunks[i][0]) for i in mine), nv, nt, dist)
        gathered = [None] * world
        dist.all_gather_object(gathered, [(v.tobytes(), i.tobytes()) for v, i in meshes])
        if rank == 0:
            import pickle
            whole = B.assemble(parts, gathered)
            with open(os.path.join(out_dir, "result.pkl"), "wb") as f:
                pickle.dump({"counts": counts, "meshes": whole}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_mesh_the_whole_batch(tmp_path):
    pytest.importorskip("oracle")
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    import pickle
    with open(os.path.join(str(tmp_path), "result.pkl"), "rb") as f:
        res = pickle.load(f)
    chunks = _chunks()
    want = [_mesh(*c) for c in chunks]
    assert len(res["meshes"]) == CHUNKS
    for (v, i), (wv, wi) in zip(res["meshes"], want):
        assert v == wv.tobytes() and i == wi.tobytes()
    counts = res["counts"]
    assert [c[0] for c in counts] == [len(p) for p in B.partition([s for s, _ in chunks], world)]
    assert sum(c[1] for c in counts) == sum(B.chunk_cells(s) for s, _ in chunks)
    assert sum(c[2] for c in counts) == sum(len(v) // 3 for v, _ in want)
    assert sum(c[3] for c in counts) == sum(len(i) // 3 for _, i in want)
