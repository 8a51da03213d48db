"""Implicit comparator on the GPU: fused Jacobi-PCG on (I - gamma A) x = b
(SUNLinSol_PCG + preconditioner_jacobi.cpp) bit for bit against the oracle; the generic
callback-driven PCG; SDIRK2 (ARKStep DIRK) against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def smooth_rhs(nx, ny, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 1.0) / (nx + 1)
    y = (np.arange(ny) + 1.0) / (ny + 1)
    b = np.zeros((ny, nx))
    for _ in range(6):
        p, q = rng.integers(1, 8, size=2)
        b += rng.standard_normal() * np.outer(np.sin(q * np.pi * y), np.sin(p * np.pi * x))
    return b.ravel()


@pytest.mark.parametrize("nx,ny,kx,ky,gamma,jacobi", [
    (33, 17, 1.0, 1.0, 1e-3, True),
    (64, 64, 1.0, 1e-3, 1e-2, True),
    (128, 96, 1.0, 0.2, 1e-4, False),
    (257, 129, 1.0, 0.05, 5e-3, True),
])
def test_fused_pcg_bitwise(ctx, stslib, oracle, nx, ny, kx, ky, gamma, jacobi):
    pk = dict(kind=0, nx=nx, ny=ny, kx=kx, ky=ky)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = smooth_rhs(nx, ny, nx)
    B = stslib.NVector.from_numpy(ctx, b)
    X = G.vector()
    it_g, rel_g, rc = stslib.implicit_solve_pcg(G, gamma, B, X, tol=1e-8, jacobi=jacobi)
    x_o, it_o, rel_o = O.pcg(gamma, b, tol=1e-8, jacobi=jacobi)
    assert rc == 0 and it_g == it_o and rel_g == rel_o <= 1e-8
    assert np.array_equal(X.numpy(), x_o)


def test_pcg_iteration_limit_is_recoverable(ctx, stslib, oracle):
    pk = dict(kind=0, nx=64, ny=64)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = smooth_rhs(64, 64, 1)
    X = G.vector()
    it, rel, rc = stslib.implicit_solve_pcg(G, 1e-2, stslib.NVector.from_numpy(ctx, b), X,
                                            tol=1e-14, maxit=5)
    x_o, it_o, rel_o = O.pcg(1e-2, b, tol=1e-14, maxit=5)
    assert rc == 1 and it == it_o == 5 and rel == rel_o
    assert np.array_equal(X.numpy(), x_o)


def test_generic_pcg_with_callbacks(ctx, stslib, oracle):
    pk = dict(kind=0, nx=48, ny=40, kx=1.0, ky=0.1)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    gamma = 2e-3
    b = smooth_rhs(48, 40, 7)
    B = stslib.NVector.from_numpy(ctx, b)
    tmp = G.vector()

    def atimes(v, z):
        G.jac_times(v, tmp)
        z.linear_sum(1.0, v, -gamma, tmp)
        return 0

    G.psetup(gamma)

    def psolve(r, z):
        return G.psolve(r, z, gamma)

    S = stslib.PCGSolver(ctx, B, atimes, psolve, maxl=500)
    X = G.vector()
    rc, it, res = S.solve(X, B, 1e-10)
    x_o, it_o, _ = O.pcg(gamma, b, tol=1e-10)
    assert rc == 0 and res <= 1e-10 and abs(it - it_o) <= 2
    assert np.linalg.norm(X.numpy() - x_o) / np.linalg.norm(x_o) < 1e-8


def test_sdirk2_bitwise(ctx, stslib, oracle):
    pk = dict(kind=0, nx=40, ny=32, kx=1.0, ky=0.3)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    y = G.initial()
    iters = stslib.sdirk2_evolve(G, y, 0.0, 0.01, 5, tol=1e-10)
    y_o, it_o = O.sdirk2(O.initial(), 0.0, 0.01, 5, tol=1e-10)
    assert iters == it_o
    assert np.array_equal(y.numpy(), y_o)
    ex = O.exact(0.05)
    assert np.linalg.norm(y_o - ex) / np.linalg.norm(ex) < 1e-2
