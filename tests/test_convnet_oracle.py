"""The CPU reference of the learned preconditioner (oracle/convnet.py) checked by itself:
hand-written gradients against central finite differences, linearity in the residual,
symmetry and positive definiteness of the preconditioner, and BF16 rounding against numpy's
float32 bit patterns."""
import numpy as np

from oracle import convnet


def test_bf16_round_nearest_even():
    a = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5e-3, 3.0e30],
                 dtype=np.float32)
    r = convnet.bf16_round(a)
    # exactly representable values stay, ties go to the even mantissa
    assert r[0] == 1.0
    assert r[1] == 1.0
    assert r[2] == np.float32(1.0 + 2 ** -6)
    assert r[3] == np.float32(1.0 + 2 ** -7)
    # low 16 bits cleared, relative error at most 2^-9
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)
    assert np.all(np.abs(r - a) <= np.abs(a) * 2 ** -8)


def test_linear_in_the_residual():
    W = convnet.init_weights(seed=2)
    rng = np.random.default_rng(0)
    r1, r2 = rng.standard_normal((2, 16, 16))
    z1, _ = convnet.forward(W, r1, 0.3, -0.4, 0.7)
    z2, _ = convnet.forward(W, r2, 0.3, -0.4, 0.7)
    z12, _ = convnet.forward(W, 2.0 * r1 - 3.0 * r2, 0.3, -0.4, 0.7)
    assert np.allclose(z12, 2.0 * z1 - 3.0 * z2, rtol=1e-12, atol=1e-12)


def test_preconditioner_is_symmetric_positive_definite():
    """P r = D (r + E^T E r): <P a, b> = <a, P b> and <P a, a> > 0, checked on the dense
    matrix of P for a 16 x 16 grid."""
    W = convnet.init_weights(seed=7)
    n = 16
    P = np.zeros((n * n, n * n))
    for k in range(n * n):
        e = np.zeros(n * n)
        e[k] = 1.0
        P[:, k] = convnet.forward(W, e.reshape(n, n), 0.4, -0.3, 0.2)[0].ravel()
    assert np.allclose(P, P.T, rtol=1e-12, atol=1e-12 * np.abs(P).max())
    assert np.linalg.eigvalsh(0.5 * (P + P.T)).min() >= 0.2 * (1 - 1e-12)


def test_zero_network_is_jacobi():
    W = {k: np.zeros_like(v) for k, v in convnet.init_weights(seed=2).items()}
    r = np.random.default_rng(3).standard_normal((16, 16))
    z, _ = convnet.forward(W, r, 0.1, 0.2, 0.25)
    assert np.array_equal(z, 0.25 * r)


def test_energy_operator_is_the_shifted_stencil():
    rng = np.random.default_rng(4)
    d = rng.standard_normal((8, 6))
    gcx, gcy = 3.0, 0.5
    Md = convnet.apply_M(d, gcx, gcy)
    # dense (I - gamma A) with the Dirichlet 5-point stencil, x fastest
    ny, nx = d.shape
    M = np.zeros((ny * nx, ny * nx))
    for j in range(ny):
        for i in range(nx):
            k = j * nx + i
            M[k, k] = 1 + 2 * (gcx + gcy)
            if i > 0:
                M[k, k - 1] = -gcx
            if i < nx - 1:
                M[k, k + 1] = -gcx
            if j > 0:
                M[k, k - nx] = -gcy
            if j < ny - 1:
                M[k, k + nx] = -gcy
    assert np.allclose(Md.ravel(), M @ d.ravel(), rtol=1e-14, atol=1e-14)
    assert np.all(np.linalg.eigvalsh(M) > 0)


def test_gradients_match_finite_differences():
    W = convnet.init_weights(seed=5)
    rng = np.random.default_rng(1)
    n = 16
    r = rng.standard_normal((n, n))
    e = rng.standard_normal((n, n))
    sk, sg, jac, gcx, gcy = 0.2, -0.6, 0.9, 40.0, 4.0
    _, g = convnet.loss_and_grad(W, r, e, sk, sg, jac, gcx, gcy)
    h = 1e-6
    for nm in convnet.NAMES:
        Wd = {k: v.astype(np.float64) for k, v in W.items()}
        idx = tuple(rng.integers(0, s) for s in convnet.shape(nm))
        Wd[nm][idx] += h
        lp, _ = convnet.loss_and_grad(Wd, r, e, sk, sg, jac, gcx, gcy)
        Wd[nm][idx] -= 2 * h
        lm, _ = convnet.loss_and_grad(Wd, r, e, sk, sg, jac, gcx, gcy)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[nm][idx]) <= 1e-6 * max(1.0, abs(fd)), nm
