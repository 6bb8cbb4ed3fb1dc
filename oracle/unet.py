"""CPU restatement of the learned hillslope preconditioner -- TEST
INFRASTRUCTURE ONLY.

The reference has no learned component; this module defines the network the
GPU kernels implement (lsdtt_gb300/csrc/unet.cu), with the same rounding
points, and is the oracle for the GPU forward pass and gradients.

Network (4 levels, additive skips, 3x3 convolutions with zero padding):
    x0  = bf16(r / rms(r))                                  1 channel
    e0  = bf16(relu(conv(x0;  1->16)))                      level 0
    e1  = bf16(relu(conv(pool(e0); 16->32)))                level 1
    e2  = bf16(relu(conv(pool(e1); 32->64)))                level 2
    e3  = bf16(relu(conv(pool(e2); 64->64)))                level 3
    d2  = bf16(relu(conv(up(e3); 64->64)) + e2)
    d1  = bf16(relu(conv(up(d2); 64->32)) + e1)
    d0  = bf16(relu(conv(up(d1); 32->16)) + e0)
    y   = rms(r) * conv(d0; 16->1)                          FP32 output
pool = 2x2 mean (rounded to bf16), up = nearest 2x. Weights are bf16, every
accumulation FP32. Loss = sum (y - e)^2 / sum e^2.
"""
from __future__ import annotations

import numpy as np

CH = [(1, 16), (16, 32), (32, 64), (64, 64), (64, 64), (64, 32), (32, 16), (16, 1)]
NAMES = ["enc0", "enc1", "enc2", "enc3", "dec2", "dec1", "dec0", "out"]


def bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as float32."""
    a = np.asarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rnd = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rnd) & 0xFFFF0000).astype(np.uint32)
    out = u.view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def init_params(seed=0):
    """He-style init, rounded to bf16. Weight layout [Cout][3][3][Cin]."""
    rng = np.random.default_rng(seed)
    P = {}
    for name, (ci, co) in zip(NAMES, CH):
        std = np.sqrt(2.0 / (9 * ci)) if name != "out" else np.sqrt(1.0 / (9 * ci)) * 0.1
        P[name + ".w"] = bf16(rng.normal(0.0, std, size=(co, 3, 3, ci)).astype(np.float32))
        P[name + ".b"] = np.zeros(co, np.float32)
    return P


def conv(x, w, b):
    """x [H][W][Ci] float32, w [Co][3][3][Ci], b [Co] -> [H][W][Co] FP32."""
    H, W, Ci = x.shape
    xp = np.zeros((H + 2, W + 2, Ci), np.float32)
    xp[1:-1, 1:-1] = x
    out = np.zeros((H, W, w.shape[0]), np.float64)
    for dy in range(3):
        for dx in range(3):
            out += xp[dy:dy + H, dx:dx + W].astype(np.float64) @ w[:, dy, dx, :].T.astype(np.float64)
    return (out + b).astype(np.float32)


def conv_bwd(x, w, g):
    """Gradients of conv wrt x, w, b given dL/dout g [H][W][Co]."""
    H, W, Ci = x.shape
    xp = np.zeros((H + 2, W + 2, Ci), np.float64)
    xp[1:-1, 1:-1] = x
    gw = np.zeros(w.shape, np.float64)
    gxp = np.zeros((H + 2, W + 2, Ci), np.float64)
    g64 = g.astype(np.float64)
    for dy in range(3):
        for dx in range(3):
            gw[:, dy, dx, :] = g64.reshape(-1, w.shape[0]).T @ xp[dy:dy + H, dx:dx + W].reshape(-1, Ci)
            gxp[dy:dy + H, dx:dx + W] += g64 @ w[:, dy, dx, :].astype(np.float64)
    return gxp[1:-1, 1:-1], gw, g64.sum(axis=(0, 1))


def pool(x):
    H, W, C = x.shape
    return bf16(x.reshape(H // 2, 2, W // 2, 2, C).mean(axis=(1, 3), dtype=np.float32))


def up(x):
    return np.repeat(np.repeat(x, 2, axis=0), 2, axis=1)


def forward(P, r):
    """r [H][W] float32 -> (y [H][W] float32, cache)."""
    r = np.asarray(r, np.float32)
    rms = np.float32(np.sqrt(np.mean(r.astype(np.float64) ** 2)))
    if rms == 0:
        rms = np.float32(1.0)
    x0 = bf16((r / rms)[..., None])
    c = {"x0": x0, "rms": rms}
    e0 = bf16(np.maximum(conv(x0, P["enc0.w"], P["enc0.b"]), 0)); c["e0"] = e0
    p0 = pool(e0); c["p0"] = p0
    e1 = bf16(np.maximum(conv(p0, P["enc1.w"], P["enc1.b"]), 0)); c["e1"] = e1
    p1 = pool(e1); c["p1"] = p1
    e2 = bf16(np.maximum(conv(p1, P["enc2.w"], P["enc2.b"]), 0)); c["e2"] = e2
    p2 = pool(e2); c["p2"] = p2
    e3 = bf16(np.maximum(conv(p2, P["enc3.w"], P["enc3.b"]), 0)); c["e3"] = e3
    u3 = up(e3); c["u3"] = u3
    a2 = conv(u3, P["dec2.w"], P["dec2.b"]); c["a2"] = a2
    d2 = bf16(np.maximum(a2, 0) + e2); c["d2"] = d2
    u2 = up(d2); c["u2"] = u2
    a1 = conv(u2, P["dec1.w"], P["dec1.b"]); c["a1"] = a1
    d1 = bf16(np.maximum(a1, 0) + e1); c["d1"] = d1
    u1 = up(d1); c["u1"] = u1
    a0 = conv(u1, P["dec0.w"], P["dec0.b"]); c["a0"] = a0
    d0 = bf16(np.maximum(a0, 0) + e0); c["d0"] = d0
    o = conv(d0, P["out.w"], P["out.b"])[..., 0]
    y = (o * rms).astype(np.float32)
    return y, c


def loss_and_grads(P, r, e):
    """Loss sum (y-e)^2 / sum e^2 and dLoss/dparam (FP64 accumulations of the
    FP32/bf16 forward, the same quantities the GPU backward computes)."""
    y, c = forward(P, r)
    e = np.asarray(e, np.float32)
    den = float(np.sum(e.astype(np.float64) ** 2)) or 1.0
    diff = y.astype(np.float64) - e
    L = float(np.sum(diff * diff) / den)
    gy = 2.0 * diff / den
    G = {}
    go = (gy * c["rms"])[..., None]
    gd0, G["out.w"], G["out.b"] = conv_bwd(c["d0"], P["out.w"], go)
    # d0 = relu(a0) + e0
    ga0 = gd0 * (c["a0"] > 0)
    ge0 = gd0.copy()
    gu1, G["dec0.w"], G["dec0.b"] = conv_bwd(c["u1"], P["dec0.w"], ga0)
    gd1 = gu1.reshape(gu1.shape[0] // 2, 2, gu1.shape[1] // 2, 2, -1).sum(axis=(1, 3))
    ga1 = gd1 * (c["a1"] > 0)
    ge1 = gd1.copy()
    gu2, G["dec1.w"], G["dec1.b"] = conv_bwd(c["u2"], P["dec1.w"], ga1)
    gd2 = gu2.reshape(gu2.shape[0] // 2, 2, gu2.shape[1] // 2, 2, -1).sum(axis=(1, 3))
    ga2 = gd2 * (c["a2"] > 0)
    ge2 = gd2.copy()
    gu3, G["dec2.w"], G["dec2.b"] = conv_bwd(c["u3"], P["dec2.w"], ga2)
    ge3 = gu3.reshape(gu3.shape[0] // 2, 2, gu3.shape[1] // 2, 2, -1).sum(axis=(1, 3))
    # encoder: e3 = relu(conv(p2)); e_k (bf16) > 0 marks the active units
    g = ge3 * (c["e3"] > 0)
    gp2, G["enc3.w"], G["enc3.b"] = conv_bwd(c["p2"], P["enc3.w"], g)
    ge2 = ge2 + np.repeat(np.repeat(gp2, 2, 0), 2, 1) / 4.0
    g = ge2 * (c["e2"] > 0)
    gp1, G["enc2.w"], G["enc2.b"] = conv_bwd(c["p1"], P["enc2.w"], g)
    ge1 = ge1 + np.repeat(np.repeat(gp1, 2, 0), 2, 1) / 4.0
    g = ge1 * (c["e1"] > 0)
    gp0, G["enc1.w"], G["enc1.b"] = conv_bwd(c["p0"], P["enc1.w"], g)
    ge0 = ge0 + np.repeat(np.repeat(gp0, 2, 0), 2, 1) / 4.0
    g = ge0 * (c["e0"] > 0)
    _, G["enc0.w"], G["enc0.b"] = conv_bwd(c["x0"], P["enc0.w"], g)
    return L, G, y
