"""Write the marching-cubes table headers used by the CUDA library and by the oracle.

    python isosurface_gb300/csrc/gen_mc_tables.py [tests/golden/mc_tables.json]

Input is the JSON copy of the reference's tables (marching_cubes_tables.rs:16-331
of swiftcoder/isosurface, Apache-2.0) that tests/golden/make_golden.py extracts.
The tables are data that must match the reference entry for entry, so they are
carried over unchanged; everything else in the headers is derived here:

* ``iso_tri_count[case]``      number of triangles of a case (<= 5)
* ``iso_tri_edges[case]``      the case's triangle edge list, 4 bits per edge,
                               edge k of the list in bits [4k, 4k+4)
* ``iso_edge_order[case]``     the case's distinct edges in order of first use
                               by the triangle list (again 4 bits each)
* ``iso_edge_mask[case]``      12-bit mask of the edges whose corners differ in
                               sign; equal to EDGE_CROSSING_MASK (checked here)

The generator also checks that every crossing edge of a case is used by one of
its triangles and that no triangle uses a non-crossing edge: the GPU's
vertex-ownership rule relies on it.

EDGE_LOOPS (ExtendedMarchingCubes' triangle fans, marching_cubes_tables.rs:
333-594: loop count, the length of each loop, then the loops' edges) goes to
the oracle's header as declared.  Checked here: every loop has at least three
edges, all of them crossing edges, and the loops of a case together use
exactly its crossing edges.  Rows 167, 181 and 229 hold stray entries after
their last loop; the reference reads each row only as far as its loop lengths
reach, so those entries are never used.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

LICENSE = """// Marching-cubes tables of swiftcoder/isosurface (src/marching_cubes_tables.rs),
// Copyright 2021 Tristam MacDonald, licensed under the Apache License, Version 2.0
// (http://www.apache.org/licenses/LICENSE-2.0).  Carried over entry for entry
// because the extracted meshes must match the reference's; the derived tables
// below them are generated.  Generated by isosurface_gb300/csrc/gen_mc_tables.py
// -- do not edit.
"""


def derive(t):
    ec = t["EDGE_CONNECTION"]
    tri = t["TRIANGLE_CONNECTION"]
    counts, packed, order, nord, masks = [], [], [], [], []
    for case in range(256):
        row = tri[case]
        n = 0
        while n < 5 and row[3 * n] >= 0:
            n += 1
        edges = row[: 3 * n]
        assert all(0 <= e < 12 for e in edges)
        assert all(v == -1 for v in row[3 * n:]), case
        mask = 0
        for e, (u, v) in enumerate(ec):
            if ((case >> u) & 1) != ((case >> v) & 1):
                mask |= 1 << e
        assert mask == t["EDGE_CROSSING_MASK"][case], case
        used = 0
        for e in edges:
            used |= 1 << e
        assert used == mask, (case, used, mask)
        w = 0
        for k, e in enumerate(edges):
            w |= e << (4 * k)
        firsts = []
        for e in edges:
            if e not in firsts:
                firsts.append(e)
        o = 0
        for k, e in enumerate(firsts):
            o |= e << (4 * k)
        counts.append(n)
        packed.append(w)
        order.append(o)
        nord.append(len(firsts))
        masks.append(mask)
    return counts, packed, order, nord, masks


def owned_mask(t, cls):
    """Edges a cell of boundary class cls ((x==0) | (y==0)<<1 | (z==0)<<2) is the
    first visitor of: an edge whose lower endpoint sits at offset 0 on an
    off-axis is first visited by the neighbour below on that axis, unless the
    cell is on the grid's low face there."""
    corners, ec = t["CORNERS"], t["EDGE_CONNECTION"]
    m = 0
    for e, (u, v) in enumerate(ec):
        lo = [min(corners[u][a], corners[v][a]) for a in range(3)]
        axis = [a for a in range(3) if corners[u][a] != corners[v][a]][0]
        own = all(lo[a] == 1 or (cls >> a) & 1 for a in range(3) if a != axis)
        if own:
            m |= 1 << e
    return m


def derive_ranks(t):
    """rank[cls][case]: 4 bits per edge e, the number of edges owned by class
    cls that precede e in the case's first-use order; slot[case]: 4 bits per
    triangle vertex, the index of its edge in the first-use order."""
    counts, packed, order, nord, masks = derive(t)
    rank = []
    for cls in range(8):
        om = owned_mask(t, cls)
        row = []
        for case in range(256):
            firsts = [(order[case] >> (4 * k)) & 15 for k in range(nord[case])]
            w, r = 0, 0
            for e in firsts:
                w |= r << (4 * e)
                r += (om >> e) & 1
            row.append(w)
        rank.append(row)
    slot = []
    for case in range(256):
        firsts = [(order[case] >> (4 * k)) & 15 for k in range(nord[case])]
        w = 0
        for k in range(3 * counts[case]):
            e = (packed[case] >> (4 * k)) & 15
            w |= firsts.index(e) << (4 * k)
        slot.append(w)
    return rank, slot


def fmt_rows(vals, per, fmt):
    lines = []
    for i in range(0, len(vals), per):
        lines.append("    " + ", ".join(fmt(v) for v in vals[i: i + per]) + ",")
    return "\n".join(lines)


def write_device_header(t, path):
    counts, packed, order, nord, masks = derive(t)
    s = [LICENSE, "#pragma once", "#include <stdint.h>", "",
         "// Storage class of the tables; a CUDA translation unit defines it as",
         "// `static __device__ const` (or __constant__) before including this header.",
         "#ifndef ISO_TABLE",
         "#define ISO_TABLE static const",
         "#endif", "",
         "// Corner offsets of a cell (CORNERS, marching_cubes_tables.rs:16-25).",
         "ISO_TABLE uint8_t iso_corners[8][3] = {" + ", ".join("{%d, %d, %d}" % tuple(c) for c in t["CORNERS"]) + "};",
         "// Corners joined by each cell edge (EDGE_CONNECTION, marching_cubes_tables.rs:32-45).",
         "ISO_TABLE uint8_t iso_edge_connection[12][2] = {" + ", ".join("{%d, %d}" % tuple(e) for e in t["EDGE_CONNECTION"]) + "};",
         "// Morton-cube to marching-cubes corner remap (REMAP_CUBE, marching_cubes_tables.rs:29).",
         "ISO_TABLE uint8_t iso_remap_cube[8] = {" + ", ".join(str(v) for v in t["REMAP_CUBE"]) + "};",
         "",
         "// Triangles per case.",
         "ISO_TABLE uint8_t iso_tri_count[256] = {",
         fmt_rows(counts, 32, str),
         "};",
         "// Triangle edge lists (TRIANGLE_CONNECTION, marching_cubes_tables.rs:74-331), 4 bits per edge.",
         "ISO_TABLE uint64_t iso_tri_edges[256] = {",
         fmt_rows(packed, 4, lambda v: "0x%015xull" % v),
         "};",
         "// Distinct edges of each case in order of first use, 4 bits per edge.",
         "ISO_TABLE uint64_t iso_edge_order[256] = {",
         fmt_rows(order, 4, lambda v: "0x%012xull" % v),
         "};",
         "// Number of distinct edges of each case.",
         "ISO_TABLE uint8_t iso_edge_count[256] = {",
         fmt_rows(nord, 32, str),
         "};",
         "// Crossing-edge masks (equal to EDGE_CROSSING_MASK, marching_cubes_tables.rs:49-70).",
         "ISO_TABLE uint16_t iso_edge_mask[256] = {",
         fmt_rows(masks, 16, lambda v: "0x%03x" % v),
         "};"]
    rank, slot = derive_ranks(t)
    s += ["// Edges each boundary class (x==0) | (y==0)<<1 | (z==0)<<2 is the first visitor of.",
          "ISO_TABLE uint16_t iso_owned_mask[8] = {" + ", ".join("0x%03x" % owned_mask(t, c) for c in range(8)) + "};",
          "// Per class and case, 4 bits per edge: owned edges of that class before the edge in first-use order.",
          "ISO_TABLE uint64_t iso_owned_rank[8][256] = {"]
    for cls in range(8):
        s.append("  {")
        s.append(fmt_rows(rank[cls], 4, lambda v: "0x%012xull" % v))
        s.append("  },")
    s += ["};",
          "// Per case, 4 bits per triangle vertex: index of its edge in the first-use order.",
          "ISO_TABLE uint64_t iso_tri_slot[256] = {",
          fmt_rows(slot, 4, lambda v: "0x%015xull" % v),
          "};"]
    # what an interior cell needs, in one 16-byte entry: the triangle edge
    # list, then crossing mask | triangle count << 12 | first-use rank of owned
    # edges 5, 6 and 10 (class 0) at bits 16, 20, 24
    pack = []
    for c in range(256):
        r = rank[0][c]
        info = masks[c] | (counts[c] << 12) | (((r >> 20) & 15) << 16) | (((r >> 24) & 15) << 20) | (((r >> 40) & 15) << 24)
        pack.append((packed[c] & 0xFFFFFFFF, packed[c] >> 32, info, 0))
    s += ["// Per case, for interior cells: {triangle edges low, high, crossing mask | triangle count << 12 |",
          "// rank of owned edge 5 << 16 | of edge 6 << 20 | of edge 10 << 24, 0}, one 16-byte load.",
          "struct alignas(16) IsoCasePack {",
          "    uint32_t w[4];",
          "};",
          "ISO_TABLE IsoCasePack iso_case_pack[256] = {",
          fmt_rows(pack, 2, lambda v: "{{0x%08x, 0x%08x, 0x%08x, 0}}" % v[:3]),
          "};", ""]
    open(path, "w").write("\n".join(s))


def check_edge_loops(t):
    """The structure the fans of ExtendedMarchingCubes rely on; returns the
    cases whose rows hold entries after their last loop."""
    stray = []
    for case in range(256):
        row = t["EDGE_LOOPS"][case]
        n = row[0]
        lengths = row[1:1 + n]
        at = 1 + n
        used = 0
        for k in lengths:
            assert k >= 3, case
            for e in row[at:at + k]:
                assert 0 <= e < 12 and (t["EDGE_CROSSING_MASK"][case] >> e) & 1, (case, e)
                used |= 1 << e
            at += k
        assert at <= 17 and used == t["EDGE_CROSSING_MASK"][case], case
        if any(v != -1 for v in row[at:]):
            stray.append(case)
    return stray


def fan_order(t, case):
    """The crossing edges of a feature cell in order of first use by its fans
    (extended_marching_cubes.rs:136-153 adds e0, then e1, of each fan
    triangle), and the number of fan triangles."""
    row = t["EDGE_LOOPS"][case]
    n = row[0]
    at = 1 + n
    order, tris = [], 0
    for k in row[1:1 + n]:
        loop = row[at:at + k]
        for i in range(k):
            for e in (loop[i], loop[(i + 1) % k]):
                if e not in order:
                    order.append(e)
            tris += 1
        at += k
    return order, tris


def edge_geometry(t):
    """Per cube edge: its axis and the offsets of its lower end point in the
    cell; and the edge at (axis, offsets) for each axis and offset pattern."""
    axis, lo = [], []
    for u, v in t["EDGE_CONNECTION"]:
        a, b = t["CORNERS"][u], t["CORNERS"][v]
        d = [i for i in range(3) if a[i] != b[i]]
        assert len(d) == 1
        axis.append(d[0])
        lo.append([min(a[i], b[i]) for i in range(3)])
    at = [[-1] * 8 for _ in range(3)]
    for e in range(12):
        at[axis[e]][lo[e][0] | lo[e][1] << 1 | lo[e][2] << 2] = e
    return axis, lo, at


def write_emc_header(t, path):
    s = [LICENSE, "#pragma once", "#include <stdint.h>", "",
         "// Storage class of the tables; a CUDA translation unit defines it as",
         "// `static __device__ const` before including this header.",
         "#ifndef ISO_TABLE", "#define ISO_TABLE static const", "#endif", "",
         "// EDGE_LOOPS (marching_cubes_tables.rs:333-594): loop count, each loop's",
         "// length, then the loops' edges",
         "ISO_TABLE int8_t iso_emc_loops[256][17] = {"]
    for row in t["EDGE_LOOPS"]:
        s.append("    {" + ", ".join(str(v) for v in row) + "},")
    s.append("};")
    orders, counts = [], []
    for case in range(256):
        order, tris = fan_order(t, case)
        assert sorted(order) == [e for e in range(12) if (t["EDGE_CROSSING_MASK"][case] >> e) & 1], case
        w = 0
        for k, e in enumerate(order):
            w |= e << (4 * k)
        orders.append(w)
        counts.append(tris)
    s += ["// fan triangles of a feature cell (the loops' total length)",
          "ISO_TABLE uint8_t iso_emc_fan_count[256] = {", fmt_rows(counts, 16, str), "};",
          "// crossing edges in order of first use by the fans, 4 bits each",
          "ISO_TABLE uint64_t iso_emc_fan_order[256] = {", fmt_rows(orders, 4, lambda v: "0x%012xull" % v), "};"]
    axis, lo, at = edge_geometry(t)
    s += ["// per cube edge: axis, and the offsets of its lower end (x | y << 1 | z << 2)",
          "ISO_TABLE uint8_t iso_emc_edge_axis[12] = {" + ", ".join(str(a) for a in axis) + "};",
          "ISO_TABLE uint8_t iso_emc_edge_lo[12] = {" + ", ".join(str(l[0] | l[1] << 1 | l[2] << 2) for l in lo) + "};",
          "// the edge along an axis whose lower end has the given offsets (-1: none)",
          "ISO_TABLE int8_t iso_emc_edge_at[3][8] = {" + ", ".join("{" + ", ".join(str(v) for v in r) + "}" for r in at) + "};",
          ""]
    open(path, "w").write("\n".join(s))


def write_oracle_header(t, path):
    s = [LICENSE, "#pragma once", "#include <stdint.h>", "",
         "namespace ref_tables {",
         "static const int CORNERS[8][3] = {" + ", ".join("{%d, %d, %d}" % tuple(c) for c in t["CORNERS"]) + "};",
         "static const int REMAP_CUBE[8] = {" + ", ".join(str(v) for v in t["REMAP_CUBE"]) + "};",
         "static const int EDGE_CONNECTION[12][2] = {" + ", ".join("{%d, %d}" % tuple(e) for e in t["EDGE_CONNECTION"]) + "};",
         "static const uint16_t EDGE_CROSSING_MASK[256] = {",
         fmt_rows(t["EDGE_CROSSING_MASK"], 13, lambda v: "0x%03x" % v),
         "};",
         "static const int8_t TRIANGLE_CONNECTION[256][16] = {"]
    for row in t["TRIANGLE_CONNECTION"]:
        s.append("    {" + ", ".join(str(v) for v in row) + "},")
    s.append("};")
    s.append("// loop count, each loop's length, then the loops' edges")
    s.append("static const int8_t EDGE_LOOPS[256][17] = {")
    for row in t["EDGE_LOOPS"]:
        s.append("    {" + ", ".join(str(v) for v in row) + "},")
    s.append("};")
    s.append("}  // namespace ref_tables")
    open(path, "w").write("\n".join(s) + "\n")


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "mc_tables.json")
    t = json.load(open(src))
    assert check_edge_loops(t) == [167, 181, 229]
    write_device_header(t, os.path.join(HERE, "mc_tables.h"))
    write_oracle_header(t, os.path.join(ROOT, "oracle", "ref_tables.h"))
    write_emc_header(t, os.path.join(HERE, "emc_tables.h"))
    print("wrote mc_tables.h, emc_tables.h and oracle/ref_tables.h")


if __name__ == "__main__":
    main()
