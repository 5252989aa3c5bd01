"""CPU reference of the learned solver's 3D U-Net: forward, backward (input and weight gradients) and loss.

TEST INFRASTRUCTURE ONLY (the oracle of the learned part): the tests compare the CUDA kernels' activations
and gradients with this numpy code on small volumes; torch's CPU conv3d is a second witness in the tests.

Network (4 levels, 16/32/64/64 channels, 3x3x3 convolutions with zero padding, ReLU, additive skips):
  E0: c(Cin->16) c(16->16)  = s0                         (full resolution)
  E1: pool  c(16->32) c(32->32) = s1                     (1/2)
  E2: pool  c(32->64) c(64->64) = s2                     (1/4)
  E3: pool  c(64->64) c(64->64)                          (1/8, bottleneck)
  D2: up + s2  c(64->64) c(64->32)
  D1: up + s1  c(32->32) c(32->16)
  D0: up + s0  c(16->16) c(16->16)  head 1x1 (16->1, no ReLU)
pool = 2x2x2 average, up = nearest-neighbour x2 (cropped to the finer level's size).  Every 3x3x3 conv is
followed by a bias and ReLU.  Volumes are channels-last arrays (X, Y, Z, C) in the solver's cell layout.
"""
from __future__ import annotations

import numpy as np

# (name, cin, cout, level) in execution order; 'head' is 1x1
LAYERS = [
    ("e0a", None, 16, 0), ("e0b", 16, 16, 0),
    ("e1a", 16, 32, 1), ("e1b", 32, 32, 1),
    ("e2a", 32, 64, 2), ("e2b", 64, 64, 2),
    ("e3a", 64, 64, 3), ("e3b", 64, 64, 3),
    ("d2a", 64, 64, 2), ("d2b", 64, 32, 2),
    ("d1a", 32, 32, 1), ("d1b", 32, 16, 1),
    ("d0a", 16, 16, 0), ("d0b", 16, 16, 0),
    ("head", 16, 1, 0),
]


def layer_specs(cin0: int):
    out = []
    for name, ci, co, lv in LAYERS:
        out.append((name, cin0 if ci is None else ci, co, lv, 1 if name == "head" else 3))
    return out


def init_params(cin0: int, seed: int = 0):
    """He-normal weights (taps, cout, cin) and zero biases, FP32."""
    rng = np.random.default_rng(seed)
    P = {}
    for name, ci, co, lv, ks in layer_specs(cin0):
        taps = ks ** 3
        std = np.sqrt(2.0 / (taps * ci)) if name != "head" else np.sqrt(1.0 / ci)
        P[name + ".w"] = (rng.standard_normal((taps, co, ci)) * std).astype(np.float32)
        P[name + ".b"] = np.zeros(co, np.float32)
    return P


def offsets(ks):
    if ks == 1:
        return [(0, 0, 0)]
    return [(dx, dy, dz) for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)]


def _shift(x, off):
    """y[v] = x[v + off] with zero padding; x is (X, Y, Z, C)."""
    out = np.zeros_like(x)
    sx = [slice(None)] * 3
    dx = [slice(None)] * 3
    for a, o in enumerate(off):
        n = x.shape[a]
        if o >= 0:
            sx[a] = slice(o, n)
            dx[a] = slice(0, n - o)
        else:
            sx[a] = slice(0, n + o)
            dx[a] = slice(-o, n)
    out[tuple(dx)] = x[tuple(sx)]
    return out


def conv(x, w, b):
    """y[v, co] = b[co] + sum_t sum_ci w[t, co, ci] x[v + off_t, ci] (tap order dx, dy, dz in -1..1)."""
    ks = 3 if w.shape[0] == 27 else 1
    y = np.zeros(x.shape[:3] + (w.shape[1],), np.float64)
    for t, off in enumerate(offsets(ks)):
        y += np.einsum("xyzc,oc->xyzo", _shift(x, off).astype(np.float64), w[t].astype(np.float64))
    return y + b.astype(np.float64)


def conv_grads(x, w, dy):
    """Returns (dx, dw, db) of conv for upstream gradient dy."""
    ks = 3 if w.shape[0] == 27 else 1
    dx = np.zeros(x.shape, np.float64)
    dw = np.zeros(w.shape, np.float64)
    for t, off in enumerate(offsets(ks)):
        xs = _shift(x, off).astype(np.float64)
        dw[t] = np.einsum("xyzo,xyzc->oc", dy, xs)
        dx += _shift(np.einsum("xyzo,oc->xyzc", dy, w[t].astype(np.float64)), tuple(-o for o in off))
    db = dy.sum(axis=(0, 1, 2))
    return dx, dw, db


def pool(x):
    X, Y, Z, C = x.shape
    Xc, Yc, Zc = (X + 1) // 2, (Y + 1) // 2, (Z + 1) // 2
    p = np.zeros((2 * Xc, 2 * Yc, 2 * Zc, C), x.dtype)
    p[:X, :Y, :Z] = x
    return p.reshape(Xc, 2, Yc, 2, Zc, 2, C).sum(axis=(1, 3, 5)) / 8.0


def pool_back(dyc, shape):
    d = np.repeat(np.repeat(np.repeat(dyc, 2, 0), 2, 1), 2, 2) / 8.0
    return d[:shape[0], :shape[1], :shape[2]]


def up(xc, shape):
    u = np.repeat(np.repeat(np.repeat(xc, 2, 0), 2, 1), 2, 2)
    return u[:shape[0], :shape[1], :shape[2]]


def up_back(dy, shape_c):
    X, Y, Z, C = dy.shape
    p = np.zeros((2 * shape_c[0], 2 * shape_c[1], 2 * shape_c[2], C), dy.dtype)
    p[:X, :Y, :Z] = dy
    return p.reshape(shape_c[0], 2, shape_c[1], 2, shape_c[2], 2, C).sum(axis=(1, 3, 5))


def forward(P, x):
    """Returns (output (X,Y,Z), cache).  Activations in float64 (the reference), x (X,Y,Z,Cin)."""
    cache = {}

    def cr(name, inp):
        pre = conv(inp, P[name + ".w"], P[name + ".b"])
        cache[name] = (inp, pre)
        return np.maximum(pre, 0.0)

    a = cr("e0b", cr("e0a", x))
    s0 = a
    a = cr("e1b", cr("e1a", pool(s0)))
    s1 = a
    a = cr("e2b", cr("e2a", pool(s1)))
    s2 = a
    a = cr("e3b", cr("e3a", pool(s2)))
    a = cr("d2b", cr("d2a", up(a, s2.shape) + s2))
    a = cr("d1b", cr("d1a", up(a, s1.shape) + s1))
    a = cr("d0b", cr("d0a", up(a, s0.shape) + s0))
    out = conv(a, P["head.w"], P["head.b"])
    cache["head"] = (a, out)
    cache["shapes"] = (s0.shape, s1.shape, s2.shape)
    return out[..., 0], cache


def backward(P, cache, dout):
    """Gradients of a scalar loss with d loss / d output = dout (X,Y,Z).  Returns dict of grads + dx."""
    G = {}

    def back(name, dpost, relu=True):
        inp, pre = cache[name]
        dpre = dpost * (pre > 0) if relu else dpost
        dx, dw, db = conv_grads(inp, P[name + ".w"], dpre)
        G[name + ".w"] = dw
        G[name + ".b"] = db
        return dx

    s0s, s1s, s2s = cache["shapes"]
    d = back("head", dout[..., None], relu=False)
    d = back("d0a", back("d0b", d))       # d wrt (up(a) + s0)
    ds0 = d.copy()
    d = up_back(d, cache["d1b"][1].shape[:3])
    d = back("d1a", back("d1b", d))
    ds1 = d.copy()
    d = up_back(d, cache["d2b"][1].shape[:3])
    d = back("d2a", back("d2b", d))
    ds2 = d.copy()
    d = up_back(d, cache["e3b"][1].shape[:3])
    d = back("e3a", back("e3b", d))
    d = pool_back(d, s2s) + ds2
    d = back("e2a", back("e2b", d))
    d = pool_back(d, s1s) + ds1
    d = back("e1a", back("e1b", d))
    d = pool_back(d, s0s) + ds0
    dx = back("e0a", back("e0b", d))
    return G, dx


def flops_per_voxel(cin0: int) -> float:
    """Forward multiply-adds x 2 per finest-level voxel (coarser levels weighted by 8^-level)."""
    f = 0.0
    for name, ci, co, lv, ks in layer_specs(cin0):
        f += 2.0 * ks ** 3 * ci * co / 8.0 ** lv
    return f


# ------------------------------------------------------------------------------------------------ BF16 emulation
def bf16(a):
    """Round to bfloat16 (nearest even) and return float32 values."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def flatten(P):
    """Flat FP32 parameter vector in the CUDA network's order: per layer, weights then bias."""
    return np.concatenate([np.concatenate([P[n + ".w"].ravel(), P[n + ".b"].ravel()]) for n, *_ in LAYERS]).astype(
        np.float32)


def unflatten(flat, cin0=16):
    P, o = {}, 0
    for name, ci, co, lv, ks in layer_specs(cin0):
        m = ks ** 3 * co * ci
        P[name + ".w"] = flat[o:o + m].reshape(ks ** 3, co, ci)
        o += m
        P[name + ".b"] = flat[o:o + co]
        o += co
    return P


def forward_bf16(P, x):
    """The CUDA forward's rounding: BF16 weights/features/stored activations, FP64 accumulation here."""
    cache = {}
    W = {k: (bf16(v) if k.endswith(".w") and not k.startswith("head") else v) for k, v in P.items()}

    def cr(name, inp):
        pre = conv(inp, W[name + ".w"], W[name + ".b"])
        post = bf16(np.maximum(pre, 0.0))
        cache[name] = (inp, post)
        return post

    x = bf16(x)
    s0 = cr("e0b", cr("e0a", x))
    s1 = cr("e1b", cr("e1a", bf16(pool(s0))))
    s2 = cr("e2b", cr("e2a", bf16(pool(s1))))
    a = cr("e3b", cr("e3a", bf16(pool(s2))))
    a = cr("d2b", cr("d2a", bf16(up(a, s2.shape) + s2)))
    a = cr("d1b", cr("d1a", bf16(up(a, s1.shape) + s1)))
    a = cr("d0b", cr("d0a", bf16(up(a, s0.shape) + s0)))
    out = conv(a, P["head.w"], P["head.b"])[..., 0]
    cache["head"] = (a, None)
    cache["shapes"] = (s0.shape, s1.shape, s2.shape)
    cache["W"] = W
    return out, cache


def backward_bf16(P, cache, dout):
    """Gradients with the CUDA backward's rounding: the ReLU-masked upstream gradient is BF16."""
    G = {}
    W = cache["W"]

    def back(name, dpost, need_dx=True):
        inp, post = cache[name]
        dpre = bf16(dpost * (post > 0))
        dx, dw, db = conv_grads(inp, W[name + ".w"], dpre)
        G[name + ".w"] = dw
        G[name + ".b"] = db
        return dx

    s0s, s1s, s2s = cache["shapes"]
    a, _ = cache["head"]
    G["head.w"] = np.einsum("xyz,xyzc->c", dout, a)[None, None, :]
    G["head.b"] = np.array([dout.sum()])
    d = dout[..., None] * P["head.w"][0, 0][None, None, None, :]
    d = back("d0a", back("d0b", d))
    ds0 = d
    d = back("d1a", back("d1b", up_back(d, cache["d1b"][1].shape[:3])))
    ds1 = d
    d = back("d2a", back("d2b", up_back(d, cache["d2b"][1].shape[:3])))
    ds2 = d
    d = back("e3a", back("e3b", up_back(d, cache["e3b"][1].shape[:3])))
    d = back("e2a", back("e2b", pool_back(d, s2s) + ds2))
    d = back("e1a", back("e1b", pool_back(d, s1s) + ds1))
    back("e0a", back("e0b", pool_back(d, s0s) + ds0))
    return G
