"""CPU reference (test infrastructure only) of the learned multilevel preconditioner.

The preconditioner maps a residual r (one n x n field) to a correction
    z = D (r + E^T E r)
with the Jacobi diagonal D and a 4-level linear convolutional encoder E. E^T is the exact
adjoint of E (the same weights, transposed and flipped), so E^T E is symmetric positive
semi-definite and z = P r with an SPD operator P: an additive multilevel (BPX-like)
preconditioner whose level operators are learned. The system parameters enter as input
channels: E acts on x = [r, r*s_k, r*s_g] (s_k, s_g: normalised log10(ky/kx) and
log10(gamma/dx^2)), which keeps P linear in r and symmetric for every system.

Encoder (16 channels, 3x3 convolutions with zero padding, no bias; pool = 2x2 mean):
    h0 = conv(x, W_in)                 3 -> C   at n
    h1 = conv(pool(h0), W_1)           C -> C   at n/2
    h2 = conv(pool(h1), W_2)           C -> C   at n/4
    h3 = conv(pool(h2), W_3)           C -> C   at n/8
Adjoint pass with the features as its input (convT = transposed, flipped convolution,
poolT = 0.25 * nearest upsampling, the adjoint of the 2x2 mean):
    g3 = h3
    g2 = h2 + poolT(convT(g3, W_3))
    g1 = h1 + poolT(convT(g2, W_2))
    g0 = h0 + poolT(convT(g1, W_1))
    gx = convT(g0, W_in)               C -> 3   at n
    u  = gx[0] + s_k gx[1] + s_g gx[2]
    z  = jacobi * (r + u)
Weights are stored in BF16 (rounded to nearest even from FP32); the GPU keeps activations in
BF16 with FP32 accumulation, this reference computes in FP64 from the same BF16 weights.

Loss (energy norm of the shifted operator M = I - gamma A, the norm CG minimises): with
d = z - e, L = 0.5 d^T M d / (e^T M e), M applied on the crop with zero values outside it:
(M d)_ij = (1 + 2 (gcx + gcy)) d_ij - gcx (d_i-1,j + d_i+1,j) - gcy (d_i,j-1 + d_i,j+1),
gcx = gamma kx / dx^2, gcy = gamma ky / dy^2; dL/dz = M d / (e^T M e).

forward() returns z and a cache; backward() returns dL/dW for every weight given dL/dz,
written out by hand through both uses of each weight (encoder and adjoint pass); the GPU
kernels are checked against it.
"""
import numpy as np

C = 16
NAMES = ["W_in", "W_1", "W_2", "W_3"]
SHAPES = {"W_in": (C, 3, 3, 3)}


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


def convT(g, w):
    """Adjoint of conv(., w): g (Co, n, m) -> (Ci, n, m)."""
    co, n, m = g.shape
    out = np.zeros((w.shape[1], n + 2, m + 2))
    for dy in range(3):
        for dx in range(3):
            out[:, dy:dy + n, dx:dx + m] += np.einsum("oc,onm->cnm", w[:, :, dy, dx], g)
    return out[:, 1:-1, 1:-1]


def wgrad(g, x):
    """dW of conv(x, W) for output gradient g: dW[o, c, dy, dx] = sum g[o] * shifted x[c]."""
    ci, n, m = x.shape
    xp = np.zeros((ci, n + 2, m + 2))
    xp[:, 1:-1, 1:-1] = x
    dw = np.zeros((g.shape[0], ci, 3, 3))
    for dy in range(3):
        for dx in range(3):
            dw[:, :, dy, dx] = np.einsum("onm,cnm->oc", g, xp[:, dy:dy + n, dx:dx + m])
    return dw


def pool(x):
    c, n, m = x.shape
    return x.reshape(c, n // 2, 2, m // 2, 2).mean(axis=(2, 4))


def poolT(y):
    """Adjoint of the 2x2 mean: 0.25 * nearest upsampling."""
    return np.repeat(np.repeat(y, 2, axis=1), 2, axis=2) * 0.25


def inputs(r, sk, sg):
    return np.stack([r, r * sk, r * sg])


def forward(W, r, sk, sg, jacobi):
    """r: (n, n) residual; returns z (n, n) and a cache for backward."""
    Wd = {k: v.astype(np.float64) for k, v in W.items()}
    r = np.asarray(r, dtype=np.float64)
    x = inputs(r, sk, sg)
    h0 = conv(x, Wd["W_in"])
    p0 = pool(h0)
    h1 = conv(p0, Wd["W_1"])
    p1 = pool(h1)
    h2 = conv(p1, Wd["W_2"])
    p2 = pool(h2)
    h3 = conv(p2, Wd["W_3"])
    g3 = h3
    g2 = h2 + poolT(convT(g3, Wd["W_3"]))
    g1 = h1 + poolT(convT(g2, Wd["W_2"]))
    g0 = h0 + poolT(convT(g1, Wd["W_1"]))
    gx = convT(g0, Wd["W_in"])
    u = gx[0] + sk * gx[1] + sg * gx[2]
    z = (r + u) * jacobi
    cache = dict(x=x, p0=p0, p1=p1, p2=p2, g3=g3, g2=g2, g1=g1, g0=g0, Wd=Wd, jacobi=jacobi, sk=sk,
                 sg=sg)
    return z, cache


def backward(cache, gz):
    """dL/dW for all weights given dL/dz (n, n)."""
    c = cache
    Wd = c["Wd"]
    gu = np.asarray(gz, dtype=np.float64) * c["jacobi"]
    dgx = np.stack([gu, c["sk"] * gu, c["sg"] * gu])
    # adjoint pass: each convT(a, W) contributes dW = wgrad(a, dy) and passes conv(dy, W) down
    dW = {"W_in": wgrad(c["g0"], dgx)}
    dg0 = conv(dgx, Wd["W_in"])
    dh0 = dg0.copy()
    dy1 = pool(dg0)
    dW["W_1"] = wgrad(c["g1"], dy1)
    dg1 = conv(dy1, Wd["W_1"])
    dh1 = dg1.copy()
    dy2 = pool(dg1)
    dW["W_2"] = wgrad(c["g2"], dy2)
    dg2 = conv(dy2, Wd["W_2"])
    dh2 = dg2.copy()
    dy3 = pool(dg2)
    dW["W_3"] = wgrad(c["g3"], dy3)
    dh3 = conv(dy3, Wd["W_3"])
    # encoder
    dW["W_3"] += wgrad(dh3, c["p2"])
    dh2 += poolT(convT(dh3, Wd["W_3"]))
    dW["W_2"] += wgrad(dh2, c["p1"])
    dh1 += poolT(convT(dh2, Wd["W_2"]))
    dW["W_1"] += wgrad(dh1, c["p0"])
    dh0 += poolT(convT(dh1, Wd["W_1"]))
    dW["W_in"] += wgrad(dh0, c["x"])
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
