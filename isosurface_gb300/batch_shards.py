"""The chunk batch across GPUs: chunks are independent units, so each rank
meshes its own share of them and the ranks exchange nothing but a final
gather of their counts.

Partition: size-balanced round robin.  The chunks, largest first (cells of
MarchingCubes::new(size) = (size-1)^2 * size; ties by chunk index), are
dealt to the ranks in a snake order (0, 1, ..., N-1, N-1, ..., 1, 0, 0, ...),
so the ranks' chunk counts differ by at most one and their cells by at most
one largest chunk.  Each rank keeps
its chunks in chunk order and meshes them as one batch (`api.Batch`, one
CUDA graph); a chunk's mesh does not depend on the other chunks of its
batch, so the per-chunk meshes equal those of the unsharded batch.
"""


def chunk_cells(size):
    """Cells of MarchingCubes::new(size): (size-1) x (size-1) x size."""
    return (size - 1) * (size - 1) * size if size >= 2 else 0


def partition(sizes, world):
    """Chunk indices per rank (each list ascending) for chunk sizes `sizes`."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(sizes)), key=lambda i: (-chunk_cells(sizes[i]), i))
    parts = [[] for _ in range(world)]
    for k, i in enumerate(order):
        lap, pos = divmod(k, world)
        parts[pos if lap % 2 == 0 else world - 1 - pos].append(i)
    return [sorted(p) for p in parts]


def rank_cells(sizes, parts):
    """Cells each rank meshes."""
    return [sum(chunk_cells(sizes[i]) for i in p) for p in parts]


def gather_counts(chunks, cells, vertices, triangles, dist, device="cpu"):
    """The final count gather: every rank's (chunks, cells, vertices,
    triangles), as a list over ranks (one entry without a process group)."""
    local = [int(chunks), int(cells), int(vertices), int(triangles)]
    if dist is None:
        return [local]
    import torch
    t = torch.tensor(local, dtype=torch.int64, device=device)
    out = [torch.empty_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(out, t)
    return [[int(x) for x in o.tolist()] for o in out]


def run_shard(ctx, chunks, rank, world, graph=True):
    """Mesh rank `rank`'s share of `chunks` (a list of (size, source)) as one
    batch on `ctx`.  Returns (chunk indices, batch, mesh info); the caller
    closes the batch."""
    from .api import Batch
    mine = partition([size for size, _ in chunks], world)[rank]
    batch = Batch(ctx, [chunks[i] for i in mine])
    if graph:
        batch.run(graph=False)  # the eager run records the counts the graph replays
    info = batch.run(graph=graph)
    return mine, batch, info


def assemble(parts, per_rank_meshes):
    """The per-chunk meshes in chunk order from each rank's meshes (in its
    own chunk order)."""
    n = sum(len(p) for p in parts)
    out = [None] * n
    for p, meshes in zip(parts, per_rank_meshes):
        if len(p) != len(meshes):
            raise ValueError("a rank's meshes do not match its chunks")
        for i, m in zip(p, meshes):
            out[i] = m
    return out
