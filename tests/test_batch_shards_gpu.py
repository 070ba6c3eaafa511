"""The chunk batch sharded across ranks, on one GPU: every rank's share
(isosurface_gb300/batch_shards.py) meshed in turn as its own batch, the
per-chunk meshes put back in chunk order, equal the unsharded batch's and
the oracle's byte for byte, and the ranks' counts add up to the whole
batch's."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import batch_shards as B
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S
from isosurface_gb300.api import Batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chunk_set():
    return scenes.chunks(seed=7, count=96)


@pytest.mark.parametrize("world", [2, 3, 8])
def test_sharded_batch_equals_whole_batch_and_oracle(ctx, chunk_set, world):
    whole = Batch(ctx, chunk_set)
    winfo = whole.run(graph=False)
    want = whole.meshes(winfo)
    whole.close()
    parts = B.partition([size for size, _ in chunk_set], world)
    per_rank, counts = [], []
    for rank in range(world):
        mine, batch, info = B.run_shard(ctx, chunk_set, rank, world)
        assert mine == parts[rank]
        per_rank.append(batch.meshes(info))
        counts.append((len(mine), int(info.num_cells), int(info.num_vertices), int(info.num_triangles)))
        batch.close()
    got = B.assemble(parts, per_rank)
    assert len(got) == len(chunk_set)
    for g, w in zip(got, want):
        assert np.array_equal(g.vertices, w.vertices)
        assert np.array_equal(g.indices, w.indices)
    assert sum(c[0] for c in counts) == len(chunk_set)
    assert sum(c[1] for c in counts) == int(winfo.num_cells)
    assert sum(c[2] for c in counts) == int(winfo.num_vertices)
    assert sum(c[3] for c in counts) == int(winfo.num_triangles)
    for i in (0, len(chunk_set) // 2, len(chunk_set) - 1):
        size, src = chunk_set[i]
        m = oracle.Program(S.lower(src)).marching_cubes(size)
        assert np.array_equal(got[i].vertices, m.vertices)
        assert np.array_equal(got[i].indices, m.indices)
