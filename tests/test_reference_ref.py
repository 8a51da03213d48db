"""The oracle against the reference's own code (oracle/_ref) on the reference's problem.

oracle/_ref/libdiffusion_ref.so is the reference's diffusion_2D sources (diffusion_2D.cpp,
diffusion.cpp, initial.cpp, buffers.cpp, preconditioner_jacobi.cpp) compiled unmodified with
single-rank MPI and serial-vector stand-ins (oracle/ref_shim). These tests pin the oracle's
restatement of the RHS (both operation orders), the initial state, the coefficients and the
Jacobi preconditioner to it bit for bit, and pin the committed fixture
tests/golden/reference_periodic.npz (which the GPU tests use) to a fresh run. They need the
reference tree and are skipped where it is absent."""
import os

import numpy as np
import pytest

from oracle import refbind

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.skipif(not os.path.isdir(refbind.REF_DIR), reason="reference tree absent")

SIZES = [(48, 40), (33, 17), (8, 8), (96, 64)]


@pytest.fixture(scope="module")
def rb():
    refbind.lib()
    return refbind


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("inhomogeneous", [False, True])
def test_rhs_and_initial_bitwise(rb, oracle, nx, ny, inhomogeneous):
    kx, ky = 1.0, 0.37
    R = rb.RefProblem(nx, ny, kx, ky, inhomogeneous)
    O = oracle.Problem(oracle.PERIODIC, nx, ny, kx=kx, ky=ky, inhomogeneous=inhomogeneous)
    P = O.p.contents
    assert R.grid() == (P.dx, P.dy, P.xl, P.yl)
    assert np.array_equal(R.initial(), O.initial())
    rng = np.random.default_rng(nx * 1000 + ny)
    for t in (0.0, 0.7):
        u = rng.standard_normal(nx * ny)
        fr = R.rhs(t, u)
        # reference operation order (laplacian) and the kernel order of the GPU stencil
        assert np.array_equal(fr, O.rhs(t, u, ref=True))
        assert np.array_equal(fr, O.rhs(t, u))


def test_face_coefficients_bitwise(rb, oracle):
    """The oracle's periodic face tables are Diffusion_Coeff_X/Y at the faces / d^2."""
    nx, ny, kx, ky = 40, 24, 0.8, 0.3
    R = rb.RefProblem(nx, ny, kx, ky, True)
    O = oracle.Problem(oracle.PERIODIC, nx, ny, kx=kx, ky=ky, inhomogeneous=True)
    P = O.p.contents
    dxw = np.ctypeslib.as_array(P.Dxw, shape=(nx,))
    dyn = np.ctypeslib.as_array(P.Dyn, shape=(ny,))
    for i in range(nx):
        assert dxw[i] == R.coeff_x(P.xl + (i - 0.5) * P.dx) / (P.dx * P.dx)
    for j in range(ny):
        assert dyn[j] == R.coeff_y(P.yl + (j + 0.5) * P.dy) / (P.dy * P.dy)


@pytest.mark.parametrize("gamma", [1e-4, 3e-2])
def test_jacobi_homogeneous_bitwise(rb, oracle, gamma):
    """PSetup / PSolve (preconditioner_jacobi.cpp): D = 1/(1 - gamma diag), z = D r, the
    oracle's D = 1/(1 - gamma cc) for constant coefficients."""
    nx, ny = 36, 28
    R = rb.RefProblem(nx, ny, 1.0, 0.2, False)
    O = oracle.Problem(oracle.PERIODIC, nx, ny, kx=1.0, ky=0.2)
    r = np.random.default_rng(3).standard_normal(nx * ny)
    d, z = R.jacobi(gamma, r)
    D = 1.0 / (1.0 - gamma * O.p.contents.cc)
    assert np.all(d == D)
    assert np.array_equal(z, D * r)


def test_jacobi_inhomogeneous_deviation_is_the_documented_one(rb, oracle):
    """With spatially varying coefficients the reference's PSetup evaluates them at the
    nodes (js+j) dy, (is+i) dx without the domain offset (preconditioner_jacobi.cpp:23-37),
    while the product and the oracle use the faces of the RHS (the exact diagonal of J).
    The reference's diagonal is exactly the node formula, restated here."""
    nx, ny, kx, ky, gamma = 30, 22, 1.0, 0.6, 2e-3
    R = rb.RefProblem(nx, ny, kx, ky, True)
    O = oracle.Problem(oracle.PERIODIC, nx, ny, kx=kx, ky=ky, inhomogeneous=True)
    P = O.p.contents
    d, _ = R.jacobi(gamma, np.ones(nx * ny))
    dx2, dy2 = P.dx * P.dx, P.dy * P.dy
    want = np.empty(nx * ny)
    for j in range(ny):
        dys, dyn = R.coeff_y(j * P.dy) / dy2, R.coeff_y((j + 1) * P.dy) / dy2
        for i in range(nx):
            dxw, dxe = R.coeff_x(i * P.dx) / dx2, R.coeff_x((i + 1) * P.dx) / dx2
            want[j * nx + i] = 1.0 / (1.0 - gamma * (-((dxw + dxe) + (dys + dyn))))
    assert np.array_equal(d, want)
    fw = np.ctypeslib.as_array(P.Dxw, shape=(nx,))
    fe = np.ctypeslib.as_array(P.Dxe, shape=(nx,))
    fs = np.ctypeslib.as_array(P.Dys, shape=(ny,))
    fn = np.ctypeslib.as_array(P.Dyn, shape=(ny,))
    faces = 1.0 / (1.0 - gamma * -((fw[None, :] + fe[None, :]) + (fs[:, None] + fn[:, None])))
    assert not np.array_equal(d, faces.ravel())


def test_committed_fixture_is_a_fresh_reference_run(rb):
    g = np.load(os.path.join(GOLD, "reference_periodic.npz"))
    nx, ny, kx, ky = int(g["nx"]), int(g["ny"]), float(g["kx"]), float(g["ky"])
    H = rb.RefProblem(nx, ny, kx, ky, False)
    I = rb.RefProblem(nx, ny, kx, ky, True)
    u = g["u"]
    assert np.array_equal(H.initial(), g["ic"])
    assert np.array_equal(H.rhs(float(g["t"]), u), g["f_hom"])
    assert np.array_equal(I.rhs(float(g["t"]), u), g["f_inh"])
    assert np.array_equal(H.jacobi(float(g["gamma"]), u)[1], g["z_hom"])
    assert np.array_equal(I.jacobi(float(g["gamma"]), u)[0], g["d_inh"])
