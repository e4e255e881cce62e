"""TEST INFRASTRUCTURE -- CPU restatement of the learned closure's network
(forward, loss, backward) for the gradient checks of the GPU kernels.

With bf16=True every operand is rounded to bfloat16 where the GPU's tensor
cores read it (inputs, weights, the ReLU activations, dY, dH2, dH1) and sums
are carried in float64 (the GPU accumulates in FP32); with bf16=False the same
formulas run in float64, which tests/test_mlp.py checks against central finite
differences.
"""
import numpy as np

IN, HID, OUT = 16, 64, 8
IN_USED, OUT_USED = 14, 7


def to_bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def _r(a, bf16):
    return to_bf16(a).astype(np.float64) if bf16 else np.asarray(a, np.float64)


def forward(net, x, bf16=True):
    """net: dict with w1 [64,16], b1, w2 [64,64], b2, w3 [8,64], b3."""
    X = _r(x, bf16)
    W1, W2, W3 = _r(net["w1"], bf16), _r(net["w2"], bf16), _r(net["w3"], bf16)
    h1 = np.maximum(X @ W1.T + net["b1"], 0.0)
    H1 = _r(h1, bf16)
    h2 = np.maximum(H1 @ W2.T + net["b2"], 0.0)
    H2 = _r(h2, bf16)
    Y = H2 @ W3.T + net["b3"]
    return Y, (X, W1, W2, W3, H1, H2)


def loss_grad(net, x, y, bf16=True):
    n = x.shape[0]
    Y, (X, W1, W2, W3, H1, H2) = forward(net, x, bf16)
    e = np.zeros_like(Y)
    e[:, :OUT_USED] = Y[:, :OUT_USED] - y[:, :OUT_USED]
    loss = float((e ** 2).sum() / n)
    dY = _r(2.0 * e / n, bf16)
    g = {}
    g["w3"] = dY.T @ H2
    g["b3"] = dY.sum(axis=0)
    dH2 = _r((dY @ W3) * (H2 > 0), bf16)
    g["w2"] = dH2.T @ H1
    g["b2"] = dH2.sum(axis=0)
    dH1 = _r((dH2 @ W2) * (H1 > 0), bf16)
    g["w1"] = dH1.T @ X
    g["b1"] = dH1.sum(axis=0)
    g["w1"][:, IN_USED:] = 0.0
    g["w3"][OUT_USED:, :] = 0.0
    g["b3"][OUT_USED:] = 0.0
    return loss, g


def random_net(rng, scale=0.3):
    net = {"w1": rng.normal(0, scale, (HID, IN)), "b1": rng.normal(0, 0.1, HID),
           "w2": rng.normal(0, scale / 2, (HID, HID)), "b2": rng.normal(0, 0.1, HID),
           "w3": rng.normal(0, scale / 2, (OUT, HID)), "b3": rng.normal(0, 0.1, OUT)}
    net["w1"][:, IN_USED:] = 0.0
    net["w3"][OUT_USED:, :] = 0.0
    net["b3"][OUT_USED:] = 0.0
    return {k: v.astype(np.float32).astype(np.float64) for k, v in net.items()}
