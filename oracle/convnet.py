"""CPU reference (test infrastructure only) of the learned multilevel preconditioner.

The network maps a residual r (one n x n field) to a correction z ~ (I - gamma A)^{-1} r. It is
linear in r: the input channels are r, r*s_k and r*s_g, where s_k and s_g are the normalised
log10(ky) and log10(gamma*h / dx^2) of the system, so the parameters modulate the operator
while M(a r) = a M(r) holds exactly (as a Krylov preconditioner needs).

Architecture (4 levels, C = 16 channels, 3x3 convolutions with zero padding, no bias):
    a0 = conv(x, W_in)                      3 -> C   at n
    a1 = conv(pool(a0), W_d1)               C -> C   at n/2
    a2 = conv(pool(a1), W_d2)               C -> C   at n/4
    a3 = conv(conv(pool(a2), W_d3), W_c)    C -> C   at n/8 (two convolutions)
    b2 = conv(up(a3) + a2, W_u2)            C -> C   at n/4
    b1 = conv(up(b2) + a1, W_u1)            C -> C   at n/2
    b0 = conv(up(b1) + a0, W_u0)            C -> C   at n
    z  = (r + conv(b0, W_out)) * jacobi     C -> 1   at n   (Jacobi skip: z = D r + D N(r))
pool = 2x2 mean; up = nearest-neighbour copy (its adjoint is the 2x2 sum). Weights are
stored in BF16 (rounded to nearest even from FP32), activations in BF16 with FP32
accumulation on the GPU; this reference computes in FP64 from the same BF16 weights. The
skip term D r makes the untrained network (small W_out) the Jacobi preconditioner, and the
network learns the correction beyond it.

Loss (energy norm of the shifted operator M = I - gamma A, the norm CG minimises): with
d = z - e, L = 0.5 d^T M d / (e^T M e), M applied on the crop with zero values outside it:
(M d)_ij = (1 + 2 (gcx + gcy)) d_ij - gcx (d_i-1,j + d_i+1,j) - gcy (d_i,j-1 + d_i,j+1),
gcx = gamma kx / dx^2, gcy = gamma ky / dy^2; dL/dz = M d / (e^T M e).

forward() returns the output and a cache; backward() returns dL/dW for every weight given
dL/dz, written out by hand (the GPU kernels are checked against it).
"""
import numpy as np

C = 16
NAMES = ["W_in", "W_d1", "W_d2", "W_d3", "W_c", "W_u2", "W_u1", "W_u0", "W_out"]
SHAPES = {"W_in": (C, 3, 3, 3), "W_out": (1, C, 3, 3)}


def shape(name):
    return SHAPES.get(name, (C, C, 3, 3))


def bf16_round(a):
    """Round FP32 values to BF16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def init_weights(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    W = {}
    for nm in NAMES:
        co, ci, kh, kw = shape(nm)
        std = scale * np.sqrt(1.0 / (ci * kh * kw))
        W[nm] = bf16_round(rng.standard_normal((co, ci, kh, kw)) * std)
    return W


def conv(x, w):
    """3x3 'same' convolution (cross-correlation), zero padding. x: (Ci, n, m), w: (Co, Ci, 3, 3)."""
    ci, n, m = x.shape
    xp = np.zeros((ci, n + 2, m + 2))
    xp[:, 1:-1, 1:-1] = x
    out = np.zeros((w.shape[0], n, m))
    for dy in range(3):
        for dx in range(3):
            patch = xp[:, dy:dy + n, dx:dx + m]
            out += np.einsum("oc,cnm->onm", w[:, :, dy, dx], patch)
    return out


def conv_backward(x, w, g):
    """Gradients of conv: returns (dx, dw) for upstream gradient g (Co, n, m)."""
    ci, n, m = x.shape
    xp = np.zeros((ci, n + 2, m + 2))
    xp[:, 1:-1, 1:-1] = x
    dw = np.zeros_like(w, dtype=np.float64)
    dxp = np.zeros((ci, n + 2, m + 2))
    for dy in range(3):
        for dx in range(3):
            patch = xp[:, dy:dy + n, dx:dx + m]
            dw[:, :, dy, dx] = np.einsum("onm,cnm->oc", g, patch)
            dxp[:, dy:dy + n, dx:dx + m] += np.einsum("oc,onm->cnm", w[:, :, dy, dx], g)
    return dxp[:, 1:-1, 1:-1], dw


def pool(x):
    c, n, m = x.shape
    return x.reshape(c, n // 2, 2, m // 2, 2).mean(axis=(2, 4))


def pool_backward(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_backward(g):
    c, n, m = g.shape
    return g.reshape(c, n // 2, 2, m // 2, 2).sum(axis=(2, 4))


def inputs(r, sk, sg):
    return np.stack([r, r * sk, r * sg])


def forward(W, r, sk, sg, jacobi):
    """r: (n, n) residual; returns z (n, n) and a cache for backward."""
    Wd = {k: v.astype(np.float64) for k, v in W.items()}
    x = inputs(np.asarray(r, dtype=np.float64), sk, sg)
    a0 = conv(x, Wd["W_in"])
    p0 = pool(a0)
    a1 = conv(p0, Wd["W_d1"])
    p1 = pool(a1)
    a2 = conv(p1, Wd["W_d2"])
    p2 = pool(a2)
    c3 = conv(p2, Wd["W_d3"])
    a3 = conv(c3, Wd["W_c"])
    s2 = up(a3) + a2
    b2 = conv(s2, Wd["W_u2"])
    s1 = up(b2) + a1
    b1 = conv(s1, Wd["W_u1"])
    s0 = up(b1) + a0
    b0 = conv(s0, Wd["W_u0"])
    z = (conv(b0, Wd["W_out"])[0] + x[0]) * jacobi
    cache = dict(x=x, a0=a0, p0=p0, a1=a1, p1=p1, a2=a2, p2=p2, c3=c3, a3=a3, s2=s2, b2=b2, s1=s1,
                 b1=b1, s0=s0, b0=b0, Wd=Wd, jacobi=jacobi)
    return z, cache


def backward(cache, gz):
    """dL/dW for all weights given dL/dz (n, n)."""
    Wd = cache["Wd"]
    dW = {}
    g = (np.asarray(gz, dtype=np.float64) * cache["jacobi"])[None]
    gb0, dW["W_out"] = conv_backward(cache["b0"], Wd["W_out"], g)
    gs0, dW["W_u0"] = conv_backward(cache["s0"], Wd["W_u0"], gb0)
    ga0 = gs0.copy()
    gb1 = up_backward(gs0)
    gs1, dW["W_u1"] = conv_backward(cache["s1"], Wd["W_u1"], gb1)
    ga1 = gs1.copy()
    gb2 = up_backward(gs1)
    gs2, dW["W_u2"] = conv_backward(cache["s2"], Wd["W_u2"], gb2)
    ga2 = gs2.copy()
    ga3 = up_backward(gs2)
    gc3, dW["W_c"] = conv_backward(cache["c3"], Wd["W_c"], ga3)
    gp2, dW["W_d3"] = conv_backward(cache["p2"], Wd["W_d3"], gc3)
    ga2 += pool_backward(gp2)
    gp1, dW["W_d2"] = conv_backward(cache["p1"], Wd["W_d2"], ga2)
    ga1 += pool_backward(gp1)
    gp0, dW["W_d1"] = conv_backward(cache["p0"], Wd["W_d1"], ga1)
    ga0 += pool_backward(gp0)
    _, dW["W_in"] = conv_backward(cache["x"], Wd["W_in"], ga0)
    return dW


def apply_M(d, gcx, gcy):
    """(I - gamma A) d on one crop, zero outside it (axis 0 = y rows, axis 1 = x columns)."""
    p = np.zeros((d.shape[0] + 2, d.shape[1] + 2))
    p[1:-1, 1:-1] = d
    return (1.0 + 2.0 * (gcx + gcy)) * d - gcx * (p[1:-1, :-2] + p[1:-1, 2:]) \
        - gcy * (p[:-2, 1:-1] + p[2:, 1:-1])


def loss_and_grad(W, r, e, sk, sg, jacobi, gcx, gcy):
    """L = 0.5 (z - e)^T M (z - e) / (e^T M e) and its weight gradients."""
    z, cache = forward(W, r, sk, sg, jacobi)
    d = z - e
    den = float(np.sum(e * apply_M(e, gcx, gcy)))
    Md = apply_M(d, gcx, gcy)
    L = 0.5 * float(np.sum(d * Md)) / den
    return L, backward(cache, Md / den)
