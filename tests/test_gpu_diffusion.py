"""Problem callbacks on the device against the oracle: RHS (diffusion.cpp:9-209 restated),
J v, dom_eig (main.cpp:536-550), power iteration, Jacobi PSetup/PSolve
(preconditioner_jacobi.cpp). Bit-for-bit: both sides evaluate the same IEEE expressions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind=0, nx=17, ny=9, kx=1.0, ky=1.0),
    dict(kind=0, nx=64, ny=64, kx=1.0, ky=0.01),
    dict(kind=0, nx=255, ny=33, kx=0.3, ky=2.0),
    dict(kind=1, nx=33, ny=20, kx=0.05, ky=0.7),
    dict(kind=2, nx=24, ny=16, kx=1.0, ky=1.0, inhomogeneous=False),
    dict(kind=2, nx=31, ny=18, kx=1.0, ky=0.5, inhomogeneous=True),
]


def pair(ctx, stslib, oracle, case):
    return stslib.Problem(ctx, **case), oracle.Problem(**case)


@pytest.mark.parametrize("case", CASES)
def test_rhs_bitwise(ctx, stslib, oracle, case):
    G, O = pair(ctx, stslib, oracle, case)
    rng = np.random.default_rng(1)
    u = rng.standard_normal(O.n)
    U = stslib.NVector.from_numpy(ctx, u)
    F = G.vector()
    for t in (0.0, 0.0371, 0.5):
        assert G.rhs(t, U, F) == 0
        assert np.array_equal(F.numpy(), O.rhs(t, u))
    G.jac_times(U, F)
    assert np.array_equal(F.numpy(), O.apply_A(u))


@pytest.mark.parametrize("case", CASES)
def test_initial_and_exact_bitwise(ctx, stslib, oracle, case):
    G, O = pair(ctx, stslib, oracle, case)
    assert np.array_equal(G.initial().numpy(), O.initial())
    if case["kind"] == 0:
        assert np.array_equal(G.exact(0.3).numpy(), O.exact(0.3))


def test_initial_modes_bitwise(ctx, stslib, oracle):
    case = dict(kind=1, nx=40, ny=30, kx=0.1, ky=0.5)
    G, O = pair(ctx, stslib, oracle, case)
    pm, qm, amp = [1, 5, 16], [2, 9, 3], [0.3, -1.2, 0.05]
    assert np.array_equal(G.initial_modes(pm, qm, amp).numpy(), O.initial_modes(pm, qm, amp))


@pytest.mark.parametrize("case", CASES[:4])
def test_dom_eig_and_power_iteration(ctx, stslib, oracle, case):
    G, O = pair(ctx, stslib, oracle, case)
    assert G.dom_eig() == O.dom_eig()
    v0 = np.random.default_rng(2).standard_normal(O.n)
    V = stslib.NVector.from_numpy(ctx, v0)
    lam_g, it_g = G.power_iteration(V, 100, 0.01)
    lam_o, it_o, v_o = O.power_iteration(v0, 100, 0.01)
    assert (lam_g, it_g) == (lam_o, it_o)
    assert np.array_equal(V.numpy(), v_o)


def test_jacobi_psolve(ctx, stslib, oracle):
    case = dict(kind=0, nx=40, ny=21, kx=1.0, ky=0.2)
    G, O = pair(ctx, stslib, oracle, case)
    r = np.random.default_rng(3).standard_normal(O.n)
    R = stslib.NVector.from_numpy(ctx, r)
    Z = G.vector()
    gamma = 3.7e-4
    assert G.psetup(gamma) == 0
    assert G.psolve(R, Z, gamma) == 0
    cc = O.p.contents.cc
    assert np.array_equal(Z.numpy(), (1.0 / (1.0 - gamma * cc)) * r)


def test_bad_arguments_fail_loudly(ctx, stslib):
    L = stslib.lib()
    assert not L.STS_ProblemCreate(ctx.h, 0, 0, 10, 1.0, 1.0, 0, 0, 1, 0, 1)
    assert b"invalid" in L.STS_GetLastError()
    G = stslib.Problem(ctx, nx=8, ny=8)
    wrong = stslib.NVector(ctx, 10)
    assert G.rhs(0.0, wrong, wrong) == -1
    assert b"length" in L.STS_GetLastError()


def test_periodic_problem_against_the_reference_code(ctx, stslib):
    """The GPU RHS, initial state and Jacobi PSolve of the reference's periodic problem
    against outputs of the reference's own sources (oracle/_ref, fixture
    tests/golden/reference_periodic.npz, made by tests/golden/make_reference_goldens.py).
    Bit for bit where the host libm rounds sin / exp like the machine that made the
    fixture; otherwise within a few ulp of the terms' scale."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "reference_periodic.npz"))
    nx, ny, kx, ky = int(g["nx"]), int(g["ny"]), float(g["kx"]), float(g["ky"])
    u = g["u"]
    U = stslib.NVector.from_numpy(ctx, u)

    def close(a, b, scale):
        return np.array_equal(a, b) or np.max(np.abs(a - b)) <= 8e-16 * scale

    H = stslib.Problem(ctx, kind=2, nx=nx, ny=ny, kx=kx, ky=ky, inhomogeneous=False)
    I = stslib.Problem(ctx, kind=2, nx=nx, ny=ny, kx=kx, ky=ky, inhomogeneous=True)
    assert close(H.initial().numpy(), g["ic"], np.max(np.abs(g["ic"])))
    F = H.vector()
    assert H.rhs(float(g["t"]), U, F) == 0
    assert np.array_equal(F.numpy(), g["f_hom"])  # constant coefficients: no libm involved
    assert I.rhs(float(g["t"]), U, F) == 0
    dx = (2 * np.pi) / (nx - 1)
    assert close(F.numpy(), g["f_inh"], 4 * 1.99 * max(kx, ky) / (dx * dx) * np.max(np.abs(u)))
    Z = H.vector()
    gamma = float(g["gamma"])
    assert H.psetup(gamma) == 0 and H.psolve(U, Z, gamma) == 0
    assert np.array_equal(Z.numpy(), g["z_hom"])
