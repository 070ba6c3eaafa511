"""The library's ExtendedMarchingCubes code (isosurface_gb300/csrc/emc.cuh,
the per-item work of the kernels in emc.cu) built for the host and run item
by item in the kernels' pass order (tests/emc_host), against the oracle: bit
for bit, vertices, indices and the number of rotated edges.

This checks on any machine the device code's arithmetic, vertex ownership,
output order and flips; tests/test_emc_gpu.py checks the kernels themselves
on a GPU."""
import ctypes
import json
import os
import sys

import numpy as np
import pytest

import oracle
from isosurface_gb300 import source as S

from emc_scenes import FIXED, random_scenes

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host_lib():
    sys.path.insert(0, os.path.join(HERE, "emc_host"))
    try:
        import build as host_build
    finally:
        sys.path.pop(0)
    L = ctypes.CDLL(host_build.build())
    L.emc_host_extract.restype = ctypes.c_int
    return L


def host_emc(L, src, n):
    b = S.lower(src)
    cap = 4 * n * n * (n + 1) + 16
    v = np.empty(3 * cap, np.float32)
    i = np.empty(12 * cap, np.uint32)
    c = np.zeros(4, np.uint64)
    r = L.emc_host_extract(b, len(b), n, v.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(cap),
                           i.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(4 * cap),
                           c.ctypes.data_as(ctypes.c_void_p))
    assert r == 0
    assert int(c[3]) == 0  # no QR sweep bound
    return v[:3 * int(c[0])].reshape(-1, 3), i[:3 * int(c[1])], int(c[2])


def test_host_directed_evaluator_reference_kats(host_lib):
    """The device's Directed evaluator (emc.cuh eval_vector), built for the
    host, on every sample_vector assertion of the reference's primitive tests."""
    kats = [k for k in json.load(open(os.path.join(HERE, "golden", "kats.json"))) if k["kind"] == "vector"]
    assert len(kats) == 31
    for k in kats:
        b = S.lower(S.from_spec(k["source"]))
        pt = np.asarray(k["point"], np.float32)
        out = np.empty(3, np.float32)
        assert host_lib.emc_host_sample_vector(b, len(b), pt.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(1),
                                               out.ctypes.data_as(ctypes.c_void_p)) == 0
        assert np.array_equal(out, np.asarray(k["expected"], np.float32)), k


def _check(L, src, n):
    p = oracle.Program(S.lower(src))
    m = p.extended_marching_cubes(n)
    v, i, flips = host_emc(L, src, n)
    assert np.array_equal(v, m.vertices)
    assert np.array_equal(i, m.indices)
    assert flips == m.flips
    return m


@pytest.mark.parametrize("name", sorted(FIXED))
@pytest.mark.parametrize("size", [1, 2, 3, 9, 16, 33])
def test_host_emc_matches_oracle(host_lib, name, size):
    _check(host_lib, FIXED[name], size)


def test_host_emc_random_csg(host_lib):
    features = flips = 0
    for n, src in random_scenes(11, 40):
        m = _check(host_lib, src, n)
        assert m.conflicts == 0
        features += m.features
        flips += m.flips
    assert features > 0 and flips > 0


def test_host_emc_bench_scene(host_lib):
    """The bench's ExtendedMarchingCubes workload: new(128) of box minus
    sphere, union torus."""
    src = S.Translate(S.Union(S.Difference(S.Sphere(0.35), S.RectangularPrism((0.3, 0.3, 0.3))),
                              S.Torus(0.25, 0.06)), (0.5, 0.5, 0.5))
    m = _check(host_lib, src, 128)
    assert m.features > 1000 and m.conflicts == 0
