"""Replica layout across ranks, on CPU with the gloo backend (world size 2).

Each rank extracts its own share of independent volumes (the oracle stands in
for the device extractor here: the layout under test is the host-side one),
the per-rank time is reduced with a max, and the gathered per-volume triangle
counts must equal a single-process run over all volumes.
"""
import os
import socket
import time

import pytest
import torch.multiprocessing as mp

from isosurface_gb300 import replicas

SIZES = [8, 11, 16, 19, 24]  # independent volumes (one unit each)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene_bytes():
    from isosurface_gb300 import scenes
    from isosurface_gb300 import source as S
    return S.lower(scenes.sphere_union(count=8, seed=3))


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import oracle
    assert replicas.rank_env() == (world, rank, rank)
    dist = replicas.init("gloo")
    try:
        lo, hi = replicas.shard(len(SIZES), rank, world)
        prog = oracle.Program(_scene_bytes())
        t0 = time.perf_counter()
        counts = {SIZES[i]: len(prog.marching_cubes(SIZES[i]).triangles) for i in range(lo, hi)}
        mine = time.perf_counter() - t0
        slowest = replicas.max_over_ranks(mine, dist)
        allmine = [None] * world
        dist.all_gather_object(allmine, (rank, mine, counts))
        if rank == 0:
            import json
            merged = {}
            for _, _, c in allmine:
                merged.update(c)
            json.dump({"slowest": slowest, "times": [t for _, t, _ in allmine],
                       "counts": {str(k): v for k, v in merged.items()}},
                      open(os.path.join(out_dir, "result.json"), "w"))
    finally:
        dist.destroy_process_group()


def test_shard_covers_units_once():
    for n in (0, 1, 5, 4096, 4097):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = replicas.shard(n, r, world)
                assert 0 <= lo <= hi <= n
                assert hi - lo in (n // world, n // world + 1)
                seen.extend(range(lo, hi))
            assert seen == list(range(n))


def test_single_process_helpers():
    assert replicas.init("gloo") is None or os.environ.get("WORLD_SIZE", "1") != "1"
    assert replicas.max_over_ranks(2.5, None) == 2.5
    assert replicas.whole_job_rate(100, 4, 2.0) == 200.0


def test_two_rank_replicas_match_single_process(tmp_path):
    import json

    import oracle
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = json.load(open(tmp_path / "result.json"))
    assert res["slowest"] == pytest.approx(max(res["times"]))
    prog = oracle.Program(_scene_bytes())
    want = {str(s): len(prog.marching_cubes(s).triangles) for s in SIZES}
    assert res["counts"] == want
