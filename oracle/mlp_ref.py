"""CPU restatement of the learned warm start's network and its training loss
(test infrastructure only): forward pass, loss and gradient in float64 with
the weights rounded to bf16 as the GPU reads them.

Parameter layout (fp32, 6009 floats): W1[64][24] b1[64] W2[64][64] b2[64]
W3[3][64] b3[3] x_mean[24] x_inv_std[24] y_mean[3] y_std[3]. A sample is 28
floats: 24 features, 3 converged impulses, a new-contact flag.

Loss = mean over the batch and the 3 outputs of (y - (t - y_mean) / y_std)^2,
with y = W3 relu(W2 relu(W1 x + b1) + b2) + b3 and x = (f - x_mean) * x_inv_std.

The GPU runs the hidden layer's three 64 x 64 products on the tensor cores
with bf16 operands: the first hidden activations enter the second layer (and
its weight gradient) rounded to bf16, and so does the second layer's
back-propagated gradient. This restatement rounds at the same points.
"""
import numpy as np

N_IN, N_H, N_OUT = 24, 64, 3
W1, B1 = 0, 64 * 24
W2, B2 = B1 + 64, B1 + 64 + 64 * 64
W3, B3 = B2 + 64, B2 + 64 + 3 * 64
TRAINABLE = B3 + 3
XM, XS, YM, YS = TRAINABLE, TRAINABLE + 24, TRAINABLE + 48, TRAINABLE + 51
PARAMS = YS + 3


def bf16(a):
    """Round float32 values to bf16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float32)
    w1 = bf16(p[W1:B1]).reshape(N_H, N_IN).astype(np.float64)
    w2 = bf16(p[W2:B2]).reshape(N_H, N_H).astype(np.float64)
    w3 = bf16(p[W3:B3]).reshape(N_OUT, N_H).astype(np.float64)
    b1, b2, b3 = (p[B1:W2].astype(np.float64), p[B2:W3].astype(np.float64), p[B3:TRAINABLE].astype(np.float64))
    return w1, b1, w2, b2, w3, b3


def loss_and_grad(p, samples):
    p = np.asarray(p, np.float32)
    s = np.asarray(samples, np.float32)
    w1, b1, w2, b2, w3, b3 = unpack(p)
    xm, xs = p[XM:XS].astype(np.float32), p[XS:YM].astype(np.float32)
    ym, ys = p[YM:YS].astype(np.float32), p[YS:PARAMS].astype(np.float32)
    x = ((s[:, :N_IN] - xm) * xs).astype(np.float64)
    t = ((s[:, N_IN:N_IN + N_OUT] - ym) / ys).astype(np.float64)
    a1 = x @ w1.T + b1
    h1 = np.maximum(a1, 0.0)
    h1b = bf16(h1.astype(np.float32)).astype(np.float64)
    a2 = h1b @ w2.T + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ w3.T + b3
    r = y - t
    n = s.shape[0]
    loss = float(np.mean(r * r))
    dy = 2.0 * r / (n * N_OUT)
    g = np.zeros(TRAINABLE)
    g[W3:B3] = (dy.T @ h2).ravel()
    g[B3:TRAINABLE] = dy.sum(0)
    d2 = (dy @ w3) * (a2 > 0)
    d2b = bf16(d2.astype(np.float32)).astype(np.float64)
    g[W2:B2] = (d2b.T @ h1b).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = (d2b @ w2) * (a1 > 0)
    g[W1:B1] = (d1.T @ x).ravel()
    g[B1:W2] = d1.sum(0)
    return loss, g


def random_params(rng, samples=None):
    """He-uniform weights, small random biases, and the normalisation of
    `samples` (or unit normalisation)."""
    p = np.zeros(PARAMS, np.float32)
    p[W1:B1] = rng.uniform(-1, 1, 64 * 24) * np.sqrt(6 / 24)
    p[W2:B2] = rng.uniform(-1, 1, 64 * 64) * np.sqrt(6 / 64)
    p[W3:B3] = rng.uniform(-1, 1, 3 * 64) * np.sqrt(6 / 64)
    p[B1:W2] = rng.uniform(-0.1, 0.1, 64)
    p[B2:W3] = rng.uniform(-0.1, 0.1, 64)
    p[B3:TRAINABLE] = rng.uniform(-0.1, 0.1, 3)
    if samples is None:
        p[XS:YM] = 1.0
        p[YS:PARAMS] = 1.0
    else:
        f = samples[:, :N_IN].astype(np.float64)
        t = samples[:, N_IN:N_IN + N_OUT].astype(np.float64)
        sd = f.std(0)
        p[XM:XS] = f.mean(0)
        p[XS:YM] = np.where(sd > 1e-12, 1.0 / np.maximum(sd, 1e-300), 0.0)
        p[YM:YS] = t.mean(0)
        p[YS:PARAMS] = np.where(t.std(0) > 1e-12, t.std(0), 1.0)
    return p
