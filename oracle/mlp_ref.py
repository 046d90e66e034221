"""Test infrastructure: CPU FP64 reference of the surrogate MLP (include/rc_mlp.h).

Forward pass, mean-squared loss and parameter gradient in numpy FP64, in the
same order of layers and with the same parameter layout as the GPU kernels.
With bf16=True the values the GPU keeps in BF16 (hidden weights, the
activations fed to the tensor cores, the backward signals fed to them) are
rounded to BF16 the same way (round to nearest even), so the remaining
difference from the GPU is FP32 accumulation and the hardware tanh.
"""
from __future__ import annotations

import numpy as np

NIN, NOUT, HID = 7, 4, 128
K0, K1 = 0.7978845608, 0.044715  # GELU, tanh form


def bf16(a):
    """Round to BF16 (nearest even) and back, elementwise."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(h):
    return 0.5 * h * (1 + np.tanh(K0 * (h + K1 * h ** 3)))


def gelu_d(h):
    t = np.tanh(K0 * (h + K1 * h ** 3))
    return 0.5 * (1 + t) + 0.5 * h * (1 - t * t) * K0 * (1 + 3 * K1 * h * h)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shp in (("W0", (HID, NIN)), ("b0", (HID,)), ("W1", (HID, HID)), ("b1", (HID,)), ("W2", (HID, HID)),
                      ("b2", (HID,)), ("W3", (HID, HID)), ("b3", (HID,)), ("W4", (NOUT, HID)), ("b4", (NOUT,))):
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    return out


def features(x, mean, std):
    """(T, p, Y_1..Y_4, dt) -> (1000/T, log10 p, log10(Y + 1e-10), log10 dt), normalised."""
    x = np.asarray(x, dtype=np.float64)
    f = np.empty_like(x)
    f[:, 0] = 1000.0 / np.maximum(x[:, 0], 1.0)
    f[:, 1] = np.log10(np.maximum(x[:, 1], 1e-30))
    f[:, 2:6] = np.log10(np.maximum(x[:, 2:6], 0.0) + 1e-10)
    f[:, 6] = np.log10(np.maximum(x[:, 6], 1e-30))
    return (f - mean) / std


def forward(p, x, mean, std, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    P = unpack(p)
    xn = features(x, mean, std)
    c = {"xn": xn}
    h = xn @ P["W0"].T + P["b0"]
    c["h0"] = h
    a = r(gelu(h))
    c["a0"] = a
    for l in (1, 2, 3):
        h = a @ r(P[f"W{l}"]).T + P[f"b{l}"]
        c[f"h{l}"] = h
        a = gelu(h) if l == 3 else r(gelu(h))
        c[f"a{l}"] = a
    y = a @ P["W4"].T + P["b4"]
    return y, c


def loss_and_grad(p, x, t, mean, std, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    P = unpack(p)
    y, c = forward(p, x, mean, std, bf)
    n = x.shape[0]
    e = y - t
    loss = float((e * e).sum() / (4 * n))
    dy = 2 * e / (4 * n)
    g = {"W4": dy.T @ c["a3"], "b4": dy.sum(0)}
    dh = r((dy @ P["W4"]) * gelu_d(c["h3"]))
    for l in (3, 2, 1):
        g[f"W{l}"] = dh.T @ c[f"a{l - 1}"]
        g[f"b{l}"] = dh.sum(0)
        dh = r((dh @ r(P[f"W{l}"])) * gelu_d(c[f"h{l - 1}"]))
    g["W0"] = dh.T @ c["xn"]
    g["b0"] = dh.sum(0)
    flat = np.concatenate([g[k].ravel() for k in ("W0", "b0", "W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4")])
    return loss, flat, y
