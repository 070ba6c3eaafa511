"""Failure handling under an injected allocation failure (a host-side fake
of a failed cudaMalloc, iso_debug_fail_allocation): every extractor reports
ISO_ERR_OUT_OF_MEMORY, and the same context then extracts the right mesh.
Nothing faults, traps or waits on the device.  Skipped unless
ISO_PENDING_GPU_TESTS=1 until it has run once on a GB300."""
import os

import numpy as np
import pytest

import oracle
from isosurface_gb300 import Context, IsoError, scenes
from isosurface_gb300 import source as S

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("ISO_PENDING_GPU_TESTS") != "1",
                                 reason="fault injection not yet run on a GB300 (set ISO_PENDING_GPU_TESTS=1)")]

OUT_OF_MEMORY = 7


def _extract(c, kind, src):
    if kind == "mc":
        return c.mc_extract(src, 65)
    if kind == "dc":
        return c.dc_extract(src, 33)
    if kind == "lhmc":
        return c.lhmc_extract(src, 5)
    if kind == "point_cloud":
        return c.point_cloud_extract(src, 33)
    return c.emc_extract(src, 33)[0]


def _reference(kind, src):
    p = oracle.Program(S.lower(src))
    return {"mc": lambda: p.marching_cubes(65), "dc": lambda: p.dual_contouring(33),
            "lhmc": lambda: p.lhmc(5), "point_cloud": lambda: p.point_cloud(33),
            "emc": lambda: p.extended_marching_cubes(33)}[kind]()


@pytest.mark.parametrize("kind", ["mc", "dc", "lhmc", "point_cloud", "emc"])
def test_allocation_failure_is_reported_and_the_context_recovers(kind):
    src = S.Translate(S.Sphere(0.3), (0.5, 0.5, 0.5)) if kind == "emc" else scenes.sphere()
    ref = _reference(kind, src)
    failures = 0
    for after in range(6):
        c = Context(0)
        try:
            c.debug_fail_allocation(after)
            try:
                _extract(c, kind, src)
            except IsoError as e:
                assert e.status == OUT_OF_MEMORY
                failures += 1
            c.debug_fail_allocation(-1)
            m = c.download(_extract(c, kind, src))
            if kind == "lhmc":  # the reference's order is HashMap order: compare triangle sets
                a = {tuple(sorted(map(tuple, m.vertices[t]))) for t in m.triangles}
                b = {tuple(sorted(map(tuple, ref.vertices[t]))) for t in ref.triangles}
                assert a == b
            else:
                assert np.array_equal(m.vertices, ref.vertices)
                assert np.array_equal(m.indices, ref.indices)
        finally:
            c.close()
    assert failures > 0
