"""Checkpoint / resume of the surrogate network's training state
(iso_mlp_save / iso_mlp_load / iso_mlp_checkpoint_info).

CPU: the header and size checks of the documented format.  GPU: a run
resumed from a checkpoint follows the original loss trajectory (up to the
rounding of the float atomics in the gradient and loss reductions)."""
import struct

import numpy as np
import pytest

from isosurface_gb300 import IsoError
from isosurface_gb300._capi import lib
from isosurface_gb300 import surrogate as SG


def _nparams():
    from isosurface_gb300 import build as gbuild
    gbuild.build()
    return int(lib().iso_mlp_num_params())


def _write(path, magic=b"ISOMLP01", version=1, header=32, nparams=None, step=7, floats=None):
    n = _nparams() if nparams is None else nparams
    body = np.zeros(3 * _nparams() if floats is None else floats, np.float32)
    with open(path, "wb") as f:
        f.write(magic + struct.pack("<IIQQ", version, header, n, step))
        f.write(body.tobytes())


def test_checkpoint_info_reads_header(tmp_path):
    p = tmp_path / "a.ckpt"
    _write(p, step=1234)
    assert SG.checkpoint_info(p) == (_nparams(), 1234)


@pytest.mark.parametrize("kw", [dict(magic=b"ISOMLP02"), dict(version=2), dict(header=40), dict(nparams=17),
                                dict(floats=10)])
def test_checkpoint_info_rejects_foreign_files(tmp_path, kw):
    p = tmp_path / "bad.ckpt"
    _write(p, **kw)
    with pytest.raises(IsoError):
        SG.checkpoint_info(p)


def test_checkpoint_info_missing_file(tmp_path):
    with pytest.raises(IsoError):
        SG.checkpoint_info(tmp_path / "none.ckpt")


@pytest.mark.gpu
def test_resume_follows_the_same_trajectory(ctx, tmp_path):
    from isosurface_gb300 import scenes
    net = SG.Surrogate(ctx, seed=3)
    net.make_dataset(scenes.smooth_spheres(count=256), 1 << 16, seed=5)
    net.train(20, batch=4096)
    path = tmp_path / "net.ckpt"
    net.save(path)
    assert SG.checkpoint_info(path) == (net.nparams, 20)
    params = net.params
    first = net.train(10, batch=4096)
    net.load(path)
    assert np.array_equal(net.params, params)
    again = net.train(10, batch=4096)
    np.testing.assert_allclose(again, first, rtol=1e-3)
    # a fresh network restored from the file computes what the saved one did
    other = SG.Surrogate(ctx, seed=99)
    other.load(path)
    assert np.array_equal(other.params, params)
    pts = np.random.default_rng(1).uniform(-1, 1, (1000, 3)).astype(np.float32)
    net.load(path)
    np.testing.assert_allclose(other.forward(pts), net.forward(pts), rtol=1e-6, atol=1e-7)
