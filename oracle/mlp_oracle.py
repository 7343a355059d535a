"""CPU oracle of the surrogate network (test infrastructure only: imported by tests/).

Restates, in numpy, the forward pass, the training loss gradient and the input gradient
of the 7 -> 64 -> 64 -> 64 -> 1 SiLU MLP that hoomd-oxdna_gb300/csrc/oxg_mlp.cu runs on
BF16 tensor cores, rounding to BF16 (round to nearest even) at exactly the points where
the GPU kernels form tensor-core operands, and accumulating in float64 (the GPU
accumulates in FP32, which differs by round-off only). The network is this project's
extension; the reference has no learned part, so there is no reference file to cite.
"""

import numpy as np

N_IN = 7


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, np.float64)
    return dict(W1=p[0:1024].reshape(64, 16)[:, :N_IN], b1=p[1024:1088], W2=p[1088:5184].reshape(64, 64),
                b2=p[5184:5248], W3=p[5248:9344].reshape(64, 64), b3=p[9344:9408],
                w4=p[9408:9472], b4=p[9472])


def _silu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return z * s, s * (1.0 + z * (1.0 - s))


def normalise(feats, mu, inv_sd):
    return ((np.asarray(feats, np.float32)[:, :N_IN] - np.asarray(mu, np.float32))
            * np.asarray(inv_sd, np.float32)).astype(np.float32)


def split(a):
    """(hi, lo) BF16 parts of float32 values: hi = bf16(a), lo = bf16(a - hi)."""
    hi = bf16(a)
    return hi, bf16(np.asarray(a, np.float32).astype(np.float64) - hi)


def wsum(W):
    """The weights as the tensor-core GEMMs use them: W_hi + W_lo."""
    hi, lo = split(W)
    return hi + lo


def forward(params, xn):
    """Network output y of normalised inputs xn (n x 7) and the intermediates. Inputs
    and weights enter the GEMMs as hi + lo BF16 pairs (the kernels' layer 1 sums
    x_hi W_hi + x_lo W_hi + x_hi W_lo; the hidden layers h W_hi + h W_lo), the hidden
    activations as single BF16 values."""
    w = unpack(params)
    xh, xl = split(xn)
    W1h, W1l = split(w["W1"])
    z1 = xh @ W1h.T + xl @ W1h.T + xh @ W1l.T + w["b1"]
    h1, s1 = _silu(z1)
    h1b = bf16(h1)
    z2 = h1b @ wsum(w["W2"]).T + w["b2"]
    h2, s2 = _silu(z2)
    h2b = bf16(h2)
    z3 = h2b @ wsum(w["W3"]).T + w["b3"]
    h3, s3 = _silu(z3)
    y = h3 @ w["w4"] + w["b4"]
    return y, dict(xb=xh, s1=s1, h1b=h1b, s2=s2, h2b=h2b, h3=h3, s3=s3, w=w)


def loss_gradient(params, xn, yt):
    """Gradient of L = sum_s (y_s - yt_s)^2 / n with respect to the masters of one class
    (flat, the kernels' layout) and the sum of squared errors, as k_mlp_train computes."""
    y, c = forward(params, xn)
    w = c["w"]
    n = len(y)
    dy = 2.0 * (y - yt) / n
    g = np.zeros(len(params))
    g[9408:9472] = dy @ c["h3"]
    g[9472] = dy.sum()
    # the bias gradients are sums of the BF16 operands (a row of ones in the weight-
    # gradient GEMM's B operand yields them)
    dz3 = dy[:, None] * w["w4"][None, :] * c["s3"]
    g[9344:9408] = bf16(dz3).sum(0)
    g[5248:9344] = (bf16(dz3).T @ c["h2b"]).ravel()
    dh2 = bf16(dz3) @ wsum(w["W3"])
    dz2 = dh2 * c["s2"]
    g[5184:5248] = bf16(dz2).sum(0)
    g[1088:5184] = (bf16(dz2).T @ c["h1b"]).ravel()
    dh1 = bf16(dz2) @ wsum(w["W2"])
    dz1 = dh1 * c["s1"]
    g[1024:1088] = bf16(dz1).sum(0)
    gw1 = np.zeros((64, 16))
    gw1[:, :N_IN] = bf16(dz1).T @ c["xb"]
    g[0:1024] = gw1.ravel()
    return g, float(((y - yt) ** 2).sum())


def input_gradient(params, xn, round_silu_grad=False):
    """y and dy/dxn of each sample as the inference passes compute them: every GEMM
    operand BF16, the weights as hi + lo pairs; the SiLU derivatives of the first two layers FP32 (the tensor-core
    pass recomputes them from the accumulators kept in tensor memory) or, with
    round_silu_grad, rounded to BF16 (the in-kernel warp pass keeps them packed)."""
    y, c = forward(params, xn)
    w = c["w"]
    r = bf16 if round_silu_grad else (lambda v: v)
    dz3 = c["s3"] * w["w4"][None, :]
    dh2 = bf16(dz3) @ wsum(w["W3"])
    dz2 = dh2 * r(c["s2"])
    dh1 = bf16(dz2) @ wsum(w["W2"])
    dz1 = dh1 * r(c["s1"])
    dx = bf16(dz1) @ wsum(w["W1"])
    return y, dx


def loss_exact(params, xn, yt):
    """The same loss in exact float64 arithmetic (no BF16), for finite-difference checks
    of the oracle's own backward pass."""
    w = unpack(params)
    h1, _ = _silu(xn @ w["W1"].T + w["b1"])
    h2, _ = _silu(h1 @ w["W2"].T + w["b2"])
    h3, _ = _silu(h2 @ w["W3"].T + w["b3"])
    y = h3 @ w["w4"] + w["b4"]
    return float(((y - yt) ** 2).sum() / len(y))


def loss_gradient_exact(params, xn, yt):
    """Analytic gradient of loss_exact (the backward pass without BF16 rounding)."""
    w = unpack(params)
    z1 = xn @ w["W1"].T + w["b1"]
    h1, s1 = _silu(z1)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2, s2 = _silu(z2)
    z3 = h2 @ w["W3"].T + w["b3"]
    h3, s3 = _silu(z3)
    y = h3 @ w["w4"] + w["b4"]
    n = len(y)
    dy = 2.0 * (y - yt) / n
    g = np.zeros(len(params))
    g[9408:9472] = dy @ h3
    g[9472] = dy.sum()
    dz3 = dy[:, None] * w["w4"][None, :] * s3
    g[9344:9408] = dz3.sum(0)
    g[5248:9344] = (dz3.T @ h2).ravel()
    dz2 = (dz3 @ w["W3"]) * s2
    g[5184:5248] = dz2.sum(0)
    g[1088:5184] = (dz2.T @ h1).ravel()
    dz1 = (dz2 @ w["W2"]) * s1
    g[1024:1088] = dz1.sum(0)
    gw1 = np.zeros((64, 16))
    gw1[:, :N_IN] = dz1.T @ xn
    g[0:1024] = gw1.ravel()
    return g
