"""The surrogate's hand-written training kernels against the float64 numpy
oracle (oracle/mlp_ref.py): forward values, loss and the full parameter
gradient; and a short training run that must reduce the loss on the
4096-sphere smooth-union scene."""
import numpy as np
import pytest

from oracle import mlp_ref
from isosurface_gb300 import scenes
from isosurface_gb300.surrogate import Surrogate

pytestmark = pytest.mark.gpu


def test_forward_matches_oracle(ctx):
    net = Surrogate(ctx, seed=3)
    x = np.random.default_rng(1).uniform(-1, 1, (512, 3)).astype(np.float32)
    got = net.forward(x)
    want, _, _ = mlp_ref.forward(net.params, x)
    assert np.max(np.abs(got - want)) <= 1e-4 * max(1.0, np.max(np.abs(want)))
    net.close()


def test_gradient_matches_oracle(ctx):
    net = Surrogate(ctx, seed=4)
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, (256, 3)).astype(np.float32)
    y0, _, _ = mlp_ref.forward(net.params, x)
    t = (y0 + rng.normal(0, 0.05, len(x))).astype(np.float32)  # targets near the outputs: clamp inactive mostly
    loss, g = net.loss_grad(x, t, clamp_d=10.0)
    wl, wg = mlp_ref.loss_grad(net.params, x, t, 10.0)
    assert abs(loss - wl) <= 1e-5 + 1e-4 * abs(wl)
    # fp32 GPU accumulation vs float64: relative error of the whole gradient
    assert np.linalg.norm(g - wg) <= 1e-4 * np.linalg.norm(wg)
    # and per layer block
    offs = [0]
    for l in range(6):
        fin = 96 if l == 0 else 256
        offs.append(offs[-1] + 256 * fin + 256)
    for a, b in zip(offs[:-1], offs[1:]):
        assert np.linalg.norm(g[a:b] - wg[a:b]) <= 1e-3 * np.linalg.norm(wg[a:b]) + 1e-9
    net.close()


def test_training_reduces_loss(ctx):
    net = Surrogate(ctx, seed=5)
    src = scenes.smooth_spheres()
    # the surrogate learns the source in its own coordinates (inside the domain map)
    net.make_dataset(src.source, 1 << 20, -1.0, 1.0, seed=9)
    hist = net.train(200, batch=16384, lr=2e-3)
    assert np.all(np.isfinite(hist))
    assert hist[-20:].mean() < 0.5 * hist[:20].mean()
    net.close()


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 40000])
def test_bf16_tensor_core_forward(ctx, n):
    """tcgen05 inference against a numpy emulation of the same bf16 rounding
    points (features, weights, activations), then against the fp32 path."""
    net = Surrogate(ctx, seed=5)
    rng = np.random.default_rng(n)
    p = net.params
    x = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    got = net.forward(x, bf16=True)
    emu = mlp_ref.forward_bf16(p, x)
    want = net.forward(x)
    scale = max(1e-3, float(np.max(np.abs(want))))
    # same roundings, different fp32 accumulation order: a bf16 rounding of an
    # activation may flip, so allow a few bf16 ulps of the output scale
    assert np.max(np.abs(got - emu)) <= 2e-2 * scale
    assert np.median(np.abs(got - emu)) <= 2e-3 * scale
    # and the bf16 path stays close to fp32
    assert np.max(np.abs(got - want)) <= 5e-2 * scale + 2e-3
    net.close()


def test_bf16_refreshes_after_set_params(ctx):
    net = Surrogate(ctx, seed=6)
    x = np.random.default_rng(9).uniform(-1, 1, (300, 3)).astype(np.float32)
    a = net.forward(x, bf16=True)
    p = net.params
    p[-1] += 0.25  # output bias
    net.params = p
    b = net.forward(x, bf16=True)
    assert np.allclose(b - a, 0.25, atol=1e-5)
    net.close()
