"""Generic Krylov solvers of the SUNLinearSolver interface on the GPU (diffusion_2D/main.cpp:
209-218: SUNLinSol_PCG and SUNLinSol_SPGMR with the Jacobi PSolve of preconditioner_jacobi.cpp;
SUNLinSol_SPFGMR, SUNDIALS' flexible GMRES)
against the oracle's restatement of the same operation sequence, bit for bit: ATimes
v - gamma A v through J*v and N_VLinearSum, exact dot products (N_VDotProd, N_VDotProdMulti),
N_VLinearCombination; SDIRK2 with a generic solver object attached by the driver; the
command-line driver's --ls gmres."""
import os
import subprocess

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


def shifted_callbacks(stslib, G, gamma):
    tmp = G.vector()

    def atimes(v, z):
        G.jac_times(v, tmp)
        z.linear_sum(1.0, v, -gamma, tmp)
        return 0

    def psolve(r, z):
        return G.psolve(r, z, gamma)

    return atimes, psolve


def test_dot_prod_multi_matches_single_dots(ctx, stslib):
    rng = np.random.default_rng(5)
    n = 100_003
    x = stslib.NVector.from_numpy(ctx, rng.standard_normal(n))
    Y = [stslib.NVector.from_numpy(ctx, rng.standard_normal(n) * 10.0 ** k) for k in range(60)]
    multi = x.dot_multi(Y)
    assert multi == [x.dot(y) for y in Y]


@pytest.mark.parametrize("gstype", [1, 2], ids=["mgs", "cgs2"])
@pytest.mark.parametrize("jacobi", [True, False], ids=["jacobi", "noprec"])
@pytest.mark.parametrize("maxl,restarts", [(40, 0), (8, 50)], ids=["gmres40", "gmres8_restarted"])
def test_spgmr_bitwise(ctx, stslib, oracle, gstype, jacobi, maxl, restarts):
    nx, ny, gamma = 48, 40, 2e-4
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=0.1)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = smooth_rhs(nx, ny, 3)
    B = stslib.NVector.from_numpy(ctx, b)
    atimes, psolve = shifted_callbacks(stslib, G, gamma)
    S = stslib.SPGMRSolver(ctx, B, atimes, psolve if jacobi else None, maxl=maxl,
                           max_restarts=restarts, gstype=gstype)
    X = G.vector()
    rc, it, res = S.solve(X, B, 1e-9)
    x_o, rc_o, it_o, res_o = O.spgmr(gamma, b, tol=1e-9, maxl=maxl, max_restarts=restarts,
                                     gstype=gstype, jacobi=jacobi)
    assert rc == rc_o == 0 and it == it_o and res == res_o <= 1e-9
    assert np.array_equal(X.numpy(), x_o)
    true = np.linalg.norm(b - (x_o - gamma * O.apply_A(x_o))) / np.linalg.norm(b)
    assert true < 1e-8


@pytest.mark.parametrize("gstype", [1, 2], ids=["mgs", "cgs2"])
@pytest.mark.parametrize("jacobi", [True, False], ids=["jacobi", "noprec"])
@pytest.mark.parametrize("maxl,restarts", [(40, 0), (8, 50)], ids=["fgmres40", "fgmres8_restarted"])
def test_spfgmr_bitwise(ctx, stslib, oracle, gstype, jacobi, maxl, restarts):
    """SUNLinSol_SPFGMR through the native driver (shifted ATimes, the Jacobi PSolve) against
    the oracle's flexible GMRES, bit for bit."""
    nx, ny, gamma = 48, 40, 2e-4
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=0.1)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = smooth_rhs(nx, ny, 3)
    B = stslib.NVector.from_numpy(ctx, b)
    S = stslib.SPFGMRSolver(ctx, B, maxl=maxl, max_restarts=restarts, gstype=gstype, precond=jacobi)
    X = G.vector()
    rc, it, res = stslib.implicit_solve_ls(G, gamma, S, B, X, tol=1e-9,
                                           prec=stslib.PREC_JACOBI if jacobi else stslib.PREC_NONE)
    x_o, rc_o, it_o, res_o = O.spgmr(gamma, b, tol=1e-9, maxl=maxl, max_restarts=restarts,
                                     gstype=gstype, jacobi=jacobi, flexible=True)
    assert rc == rc_o == 0 and it == it_o and res == res_o <= 1e-9
    assert np.array_equal(X.numpy(), x_o)
    true = np.linalg.norm(b - (x_o - gamma * O.apply_A(x_o))) / np.linalg.norm(b)
    assert true < 1e-8
    if not jacobi:
        # without a preconditioner the flexible method is GMRES itself
        x_g = O.spgmr(gamma, b, tol=1e-9, maxl=maxl, max_restarts=restarts, gstype=gstype,
                      jacobi=False)[0]
        assert np.array_equal(x_g, x_o)


def test_generic_driver_with_pfmg_and_rejects(ctx, stslib):
    """The generic driver with a caller's native PSolve (the PFMG-role cycle) in CG, GMRES and
    flexible GMRES; a preconditioner on a solver made without one is refused."""
    import ctypes as C
    n, gamma = 96, 1e-3
    G = stslib.Problem(ctx, stslib.UNFORCED, n, n, 1.0, 0.05)
    b = smooth_rhs(n, n, 12)
    B = stslib.NVector.from_numpy(ctx, b)
    mg = stslib.PFMG(G)
    mg.setup(gamma)
    fn = C.cast(stslib.lib().STS_PFMGPrecSolve, C.c_void_p)
    its = {}
    for name, S in (("pcg", stslib.PCGSolver(ctx, B, maxl=500, precond=True)),
                    ("gmres", stslib.SPGMRSolver(ctx, B, maxl=30, max_restarts=10, precond=True)),
                    ("fgmres", stslib.SPFGMRSolver(ctx, B, maxl=30, max_restarts=10, precond=True))):
        X = G.vector()
        rc, it, res = stslib.implicit_solve_ls(G, gamma, S, B, X, tol=1e-9, prec=stslib.PREC_USER,
                                               pdata=mg.h, psolve=fn)
        assert rc == 0 and res <= 1e-9, (name, rc, res)
        its[name] = it
    assert max(its.values()) < 40, its
    S = stslib.SPFGMRSolver(ctx, B, maxl=10, precond=False)
    with pytest.raises(stslib.STSError):
        stslib.implicit_solve_ls(G, gamma, S, B, G.vector(), prec=stslib.PREC_JACOBI)


def test_spgmr_not_converged_is_recoverable(ctx, stslib, oracle):
    nx, ny, gamma = 40, 40, 1e-2
    pk = dict(kind=0, nx=nx, ny=ny)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = smooth_rhs(nx, ny, 9)
    B = stslib.NVector.from_numpy(ctx, b)
    atimes, psolve = shifted_callbacks(stslib, G, gamma)
    S = stslib.SPGMRSolver(ctx, B, atimes, psolve, maxl=5, max_restarts=1)
    X = G.vector()
    rc, it, res = S.solve(X, B, 1e-12)
    x_o, rc_o, it_o, res_o = O.spgmr(gamma, b, tol=1e-12, maxl=5, max_restarts=1)
    assert rc == rc_o == 1 and it == it_o == 10 and res == res_o > 1e-12
    assert np.array_equal(X.numpy(), x_o)


def test_generic_pcg_bitwise(ctx, stslib, oracle):
    nx, ny, gamma = 64, 48, 1e-3
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=0.02)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = smooth_rhs(nx, ny, 4)
    B = stslib.NVector.from_numpy(ctx, b)
    atimes, psolve = shifted_callbacks(stslib, G, gamma)
    S = stslib.PCGSolver(ctx, B, atimes, psolve, maxl=5000)
    X = G.vector()
    rc, it, res = S.solve(X, B, 1e-10)
    x_o, rc_o, it_o, res_o = O.pcg_generic(gamma, b, tol=1e-10, maxl=5000)
    assert rc == rc_o == 0 and it == it_o and res == res_o
    assert np.array_equal(X.numpy(), x_o)


@pytest.mark.parametrize("kind,gstype,precond", [("gmres", 1, True), ("gmres", 2, False),
                                                 ("pcg", 0, True)])
def test_sdirk2_with_generic_solver_bitwise(ctx, stslib, oracle, kind, gstype, precond):
    pk = dict(kind=0, nx=40, ny=32, kx=1.0, ky=0.3)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    y = G.initial()
    if kind == "gmres":
        S = stslib.SPGMRSolver(ctx, y, maxl=15, max_restarts=100, gstype=gstype, precond=precond)
    else:
        S = stslib.PCGSolver(ctx, y, maxl=10000, precond=precond)
    its = stslib.sdirk2_evolve_ls(G, S, y, 0.0, 0.01, 4, tol=1e-10, precond=precond)
    y_o, it_o = O.sdirk2_ls(O.initial(), 0.0, 0.01, 4, tol=1e-10, ls=1 if kind == "gmres" else 0,
                            maxl=15 if kind == "gmres" else 10000, max_restarts=100,
                            gstype=max(gstype, 1), jacobi=precond)
    assert its == it_o > 0
    assert np.array_equal(y.numpy(), y_o)
    # the same time steps as the fused Jacobi-PCG driver, to the solve tolerance
    y_f, _ = O.sdirk2(O.initial(), 0.0, 0.01, 4, tol=1e-10)
    assert np.linalg.norm(y_o - y_f) / np.linalg.norm(y_f) < 1e-8


def test_cli_dirk_gmres_matches_cg(stslib):
    stslib.lib()
    exe = os.path.join(os.path.dirname(stslib.__file__), "_build", "diffusion_2D_gpu")
    outs = {}
    for ls in ("cg", "gmres"):
        r = subprocess.run([exe, "--problem", "manufactured", "--nx", "48", "--ny", "48", "--integrator",
                            "dirk", "--fixedstep", "1e-3", "--tf", "0.01", "--nout", "2", "--ls", ls,
                            "--liniters", "25", "--epslin", "1e-6"], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        line = [l for l in r.stdout.split("\n") if l.startswith("Relative L2 error vs exact")][0]
        its = [l for l in r.stdout.split("\n") if l.startswith("LS iters ")][0]
        outs[ls] = (float(line.split("=")[1]), int(its.split("=")[1]))
    assert abs(outs["gmres"][0] - outs["cg"][0]) <= 1e-6 * outs["cg"][0]
    assert outs["gmres"][1] > 0 and outs["cg"][1] > 0
    r = subprocess.run([exe, "--problem", "manufactured", "--integrator", "dirk", "--fixedstep", "1e-3",
                        "--ls", "bicg"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 1 and "linear solver" in r.stderr
