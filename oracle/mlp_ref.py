"""Float64 oracle of the smoothing-length MLP (TEST INFRASTRUCTURE ONLY).

The network: 4 -> 64 -> 64 -> 1, ReLU hidden layers, predicting the log distance of the
48th nearest neighbour from (log cell density, log previous h, leaf count, velocity
divergence), standardised by a
per-feature affine map. The GPU kernels store weights in bfloat16 and accumulate in
float32; this oracle takes the same (bfloat16-rounded) weights and evaluates the forward
pass, the mean-squared-error loss on the standardised target and its gradients in float64, so that the
GPU gradients can be checked against it.
"""

import numpy as np

H = 64


def bf16_round(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounding = ((a >> 16) & 1) + 0x7FFF
    b = ((a + rounding) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    """params: flat float array [W1 (64x4), b1 (64), W2 (64x64), b2 (64), w3 (64), b3 (1)]."""
    p = np.asarray(params, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * 4].reshape(H, 4); o += H * 4
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


N_PARAMS = H * 4 + H + H * H + H + H + 1


def forward(params, x, act_bf16=False):
    """act_bf16: the layer-2 inputs rounded to bfloat16, as the inference kernels feed the
    tensor cores (training keeps them in float32)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    z1 = x @ W1.T + b1
    a1 = np.maximum(z1, 0)
    if act_bf16:
        a1 = bf16_round(a1.astype(np.float32))
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0)
    y = a2 @ w3 + b3
    return y, (x, z1, a1, z2, a2)


def loss_and_grad(params, x, target):
    """Mean squared error 0.5 * mean((y - t)^2) and its gradient w.r.t. the flat params."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    y, (x, z1, a1, z2, a2) = forward(params, x)
    n = len(y)
    r = (y - target) / n
    loss = 0.5 * np.sum((y - target) ** 2) / n
    g_w3 = a2.T @ r
    g_b3 = r.sum()
    d2 = np.outer(r, w3) * (z2 > 0)
    g_W2 = d2.T @ a1
    g_b2 = d2.sum(0)
    d1 = (d2 @ W2) * (z1 > 0)
    g_W1 = d1.T @ x
    g_b1 = d1.sum(0)
    grad = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, grad
