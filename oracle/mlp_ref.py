"""float64 numpy restatement of the surrogate MLP's forward pass, training loss
and gradient (TEST INFRASTRUCTURE ONLY: the checker for the library's
hand-written CUDA forward/backward kernels).

Same network as the library: Fourier features sin/cos(w_j x_a), w_j =
pi * 2^(7j/15), feature a*32 + 2j (+1 for cos); six 256-wide layers with
softplus_beta (beta = 100); linear output.  Parameter layout: W0[256][96], b0[256],
W1..W5[256][256], b1..b5[256], w_out[256], b_out."""
import numpy as np

FF, HID, NL = 96, 256, 6


def unpack(params):
    p = np.asarray(params, np.float64)
    out, at = [], 0
    for l in range(NL):
        fin = FF if l == 0 else HID
        W = p[at:at + HID * fin].reshape(HID, fin)
        at += HID * fin
        b = p[at:at + HID]
        at += HID
        out.append((W, b))
    w_out = p[at:at + HID]
    b_out = p[at + HID]
    assert at + HID + 1 == len(p)
    return out, w_out, b_out


def fourier(x):
    x = np.asarray(x, np.float64).reshape(-1, 3)
    w = np.pi * 2.0 ** (7.0 * np.arange(16) / 15.0)
    f = np.empty((len(x), FF))
    for a in range(3):
        arg = x[:, a:a + 1] * w[None, :]
        f[:, a * 32 + 0:a * 32 + 32:2] = np.sin(arg)
        f[:, a * 32 + 1:a * 32 + 32:2] = np.cos(arg)
    return f


BETA = 100.0


def softplus(z):
    """softplus_beta(z) = log(1 + exp(beta z)) / beta, beta = 100"""
    return np.maximum(z, 0) + np.log1p(np.exp(-BETA * np.abs(z))) / BETA


def forward(params, x):
    layers, w_out, b_out = unpack(params)
    h = fourier(x)
    zs, hs = [], [h]
    for W, b in layers:
        z = h @ W.T + b
        h = softplus(z)
        zs.append(z)
        hs.append(h)
    return h @ w_out + b_out, zs, hs


def loss_grad(params, x, t, d):
    layers, w_out, b_out = unpack(params)
    y, zs, hs = forward(params, x)
    t = np.asarray(t, np.float64)
    n = len(y)
    # truncated L1: y - t inside |t| < d, one-sided where the target saturates
    e = np.where(t >= d, np.minimum(y - d, 0.0), np.where(t <= -d, np.maximum(y + d, 0.0), y - t))
    loss = np.mean(np.abs(e))
    dy = np.sign(e) / n
    g_out_w = hs[-1].T @ dy
    g_out_b = dy.sum()
    da = dy[:, None] * w_out[None, :]
    grads = [None] * NL
    for l in range(NL - 1, -1, -1):
        dz = da / (1.0 + np.exp(-BETA * zs[l]))
        gW = dz.T @ hs[l]
        gb = dz.sum(0)
        grads[l] = (gW, gb)
        da = dz @ layers[l][0]
    flat = []
    for gW, gb in grads:
        flat += [gW.ravel(), gb]
    flat += [g_out_w, np.array([g_out_b])]
    return loss, np.concatenate(flat)


def bf16(a):
    """Round to bfloat16 (round to nearest, ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_bf16(params, x):
    """The tensor-core inference path: features, weights and hidden
    activations rounded to bf16, products accumulated exactly (float64 here,
    fp32 on the device), biases and w_out kept in fp32."""
    layers, w_out, b_out = unpack(params)
    h = bf16(fourier(x))
    for l, (W, b) in enumerate(layers):
        a = softplus(h @ bf16(W).T + np.asarray(b, np.float32))
        h = bf16(a) if l + 1 < NL else a
    return h @ np.asarray(w_out, np.float32) + np.float32(b_out)
