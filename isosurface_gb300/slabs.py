"""MarchingCubes sharded across GPUs by z-slabs.

The reference's PrimalGrid visits cells layer by layer in z
(src/traversal/primal_grid.rs:59-88) and numbers vertices in order of first
use (src/mesh.rs:225-260), so the whole mesh is the concatenation of
per-slab meshes in slab order, once each slab knows the number of vertices
the slabs below it own.  One GPU (rank) per slab of cell layers:

* the rank samples and meshes its layers plus one halo layer below them
  (iso_mc_extract_slab): no field data crosses GPUs;
* one exchange of the ranks' owned-vertex and triangle counts (an
  all-gather of two integers per rank) gives each rank its first vertex and
  triangle;
* ``assemble`` drops the halo layer's vertices and triangles and renumbers
  the rest: the rank's own vertices keep their order from its first vertex
  on; a triangle corner on a vertex of the halo layer (an edge in the slab's
  bottom plane, which the layer below owns) points to that vertex among the
  last vertices of the rank below, which are the halo layer's own vertices
  in the same order, less those on the halo layer's bottom plane.

The concatenated buffers are byte-identical to iso_mc_extract's.

DualContouring shards the same way: its mesh is marching cubes over the
dual lattice ((size-1) x (size-1) x size dual vertices, one per primal cell,
in the same z-major order), so iso_dc_extract_slab's slabs of dual cube
layers assemble with these functions given size - 1 as the size.
"""
import numpy as np


def slab_bounds(size, world):
    """Cell layers [z0, z1) of MarchingCubes::new(size) for each of `world`
    ranks: contiguous, sizes differing by at most one.  The grid has `size`
    cell layers (size + 1 sample layers, as the reference samples them)."""
    if world < 1 or world > size:
        raise ValueError("need 1 <= world <= size")
    return [(size * r // world, size * (r + 1) // world) for r in range(world)]


def halo_owned_below(keys, halo_vertices, z_begin, size):
    """Which of the halo layer's vertices the rank below numbers as well: all
    but the edges along x or y in the halo layer's own bottom plane
    z_begin - 1 (which the halo layer owns only because it is the bottom of
    this slab's lattice; in the whole grid the layer below it owns them).
    `keys` are the per-vertex lattice-edge keys ((lower end point) * 3 + axis)."""
    k = np.asarray(keys[:halo_vertices, 0], np.uint64)
    axis = k % np.uint64(3)
    z = (k // np.uint64(3)) // np.uint64(size * size)
    return ~((z == np.uint64(z_begin - 1)) & (axis != np.uint64(2)))


def halo_plane_vertices(keys, halo_vertices, z_begin, size):
    """Which of the halo layer's vertices lie on the slab's bottom plane
    z_begin (edges along x or y there): the only halo vertices that the
    slab's own triangles use."""
    k = np.asarray(keys[:halo_vertices, 0], np.uint64)
    axis = k % np.uint64(3)
    z = (k // np.uint64(3)) // np.uint64(size * size)
    return (z == np.uint64(z_begin)) & (axis != np.uint64(2))


def assemble(vertices, indices, keys, halo_vertices, halo_triangles, z_begin, size, vertex_base):
    """One slab's part of the whole grid's IndexedVertices buffers.

    vertices, indices, keys: the slab's mesh as iso_mc_extract_slab leaves it
    (halo layer first); vertex_base: the number of vertices the slabs below
    own.  Returns (vertices, indices) with indices into the whole mesh."""
    hv, ht = int(halo_vertices), int(halo_triangles)
    tri = np.asarray(indices, np.int64)[3 * ht:]
    out = tri - hv + vertex_base
    if hv:
        # the rank below numbers the halo layer's vertices (but those of the
        # halo layer's bottom plane) as its last `below.sum()`, in this order
        below = halo_owned_below(keys, hv, z_begin, size)
        rank = np.cumsum(below) - below
        low = tri < hv
        if not halo_plane_vertices(keys, hv, z_begin, size)[tri[low]].all():
            raise ValueError("a slab triangle uses a halo vertex off the slab's bottom plane")
        out[low] = vertex_base - int(below.sum()) + rank[tri[low]]
    if out.size and (out.min() < 0 or out.max() >= 1 << 32):
        raise ValueError("vertex ids out of range: wrong vertex_base")
    return np.asarray(vertices)[hv:], out.astype(np.uint32)


def vertex_bases(counts):
    """Exclusive prefix of the ranks' owned-vertex counts."""
    return np.concatenate([[0], np.cumsum(np.asarray(counts, np.int64))[:-1]]).astype(np.int64)


def all_gather_counts(vertices, triangles, dist):
    """Every rank's (owned vertices, triangles): the one exchange of the
    sharded extraction, two integers per rank.  `dist` is torch.distributed
    (or None for a single process)."""
    if dist is None:
        return [(int(vertices), int(triangles))]
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    mine = torch.tensor([int(vertices), int(triangles)], dtype=torch.int64, device=device)
    got = [torch.zeros_like(mine) for _ in range(dist.get_world_size())]
    dist.all_gather(got, mine)
    return [(int(t[0].item()), int(t[1].item())) for t in got]


def extract_slab_device(ctx, source, size, z_begin, z_end):
    """The slab on this rank's GPU: (vertices, indices, keys, halo vertices,
    halo triangles)."""
    info, hv, ht = ctx.mc_extract_slab(source, size, z_begin, z_end, keys=True)
    m = ctx.download(info, keys=True)
    return m.vertices, m.indices, m.keys, hv, ht


def extract_dc_slab_device(ctx, source, size, z_begin, z_end, placer=0):
    """A DualContouring slab on this rank's GPU, in the form extract_sharded
    takes with the dual lattice's size - 1 as its size."""
    info, hv, ht = ctx.dc_extract_slab(source, size, z_begin, z_end, placer, keys=True)
    m = ctx.download(info, keys=True)
    return m.vertices, m.indices, m.keys, hv, ht


def extract_sharded(extract_slab, size, rank, world, dist=None):
    """This rank's part of MarchingCubes::new(size) of the whole grid.

    extract_slab(z_begin, z_end) -> (vertices, indices, keys, halo vertices,
    halo triangles) meshes one slab (extract_slab_device on a GPU).  Returns
    (vertices, indices, first vertex, first triangle) of this rank's part."""
    z0, z1 = slab_bounds(size, world)[rank]
    v, i, k, hv, ht = extract_slab(z0, z1)
    counts = all_gather_counts(len(v) - hv, len(i) // 3 - ht, dist)
    base = int(vertex_bases([c[0] for c in counts])[rank])
    tbase = int(vertex_bases([c[1] for c in counts])[rank])
    verts, idx = assemble(v, i, k, hv, ht, z0, size, base)
    return verts, idx, base, tbase
