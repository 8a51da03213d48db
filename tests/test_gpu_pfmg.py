"""The structured multigrid preconditioner in hypre PFMG's role (diffusion_2D/
preconditioner_hypre.cpp: one V-cycle per PSolve, semicoarsening, non-Galerkin coarse
operators, weighted Jacobi, symmetric or nonsymmetric red/black Gauss-Seidel relaxation) on the GPU against
the oracle's restatement, bit for bit: the V-cycle itself and CG with it."""
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


CASES = [(32, 24, 0.3, 1e-2), (64, 64, 1e-3, 1e-2), (130, 66, 0.05, 5e-3), (257, 129, 1.0, 1e-3)]


@pytest.mark.parametrize("relax", [1, 2, 3], ids=["jacobi", "rbgs", "rbgs_nonsym"])
@pytest.mark.parametrize("nx,ny,ky,gamma", CASES)
def test_vcycle_bitwise(ctx, stslib, oracle, relax, nx, ny, ky, gamma):
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=ky)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    r = np.random.default_rng(nx + ny).standard_normal(nx * ny)
    mg = stslib.PFMG(G, relax=relax, nrelax=2)
    R = stslib.NVector.from_numpy(ctx, r)
    Z = G.vector()
    mg.psolve(R, Z, gamma)
    z_o, nl = oracle.Problem(**pk).pfmg_vcycle(gamma, r, relax=relax, nrelax=2)
    assert mg.levels() == nl
    assert np.array_equal(Z.numpy(), z_o)


@pytest.mark.parametrize("relax", [1, 2], ids=["jacobi", "rbgs"])
def test_pcg_pfmg_bitwise_and_fast(ctx, stslib, oracle, relax):
    nx, ny, ky, gamma = 128, 96, 0.02, 0.1  # kappa ~ 7000
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=ky)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = np.random.default_rng(5).standard_normal(nx * ny)  # broadband: all modes present
    mg = stslib.PFMG(G, relax=relax)
    B = stslib.NVector.from_numpy(ctx, b)
    X = G.vector()
    it, rel, rc = stslib.implicit_solve_pfmg(G, gamma, mg, B, X, tol=1e-10)
    x_o, rc_o, it_o, rel_o = O.pcg_pfmg(gamma, b, tol=1e-10, relax=relax)
    assert rc == rc_o == 0 and it == it_o and rel == rel_o <= 1e-10
    assert np.array_equal(X.numpy(), x_o)
    _, it_j, _ = O.pcg(gamma, b, tol=1e-10)
    assert it * 10 < it_j  # multigrid against the Jacobi-preconditioned iteration count


def test_pfmg_rejects_bad_options(ctx, stslib):
    D = stslib.Problem(ctx, kind=0, nx=32, ny=32)
    for bad in (dict(relax=0), dict(relax=4), dict(nrelax=0), dict(nrelax=17)):
        with pytest.raises(stslib.STSError):
            stslib.PFMG(D, **bad)


PERIODIC_CASES = [(32, 32, 0.0, False, 5e-2), (48, 40, 0.3, True, 1e-2), (30, 18, 1.0, True, 2e-2),
                  (64, 16, 0.05, False, 1e-3)]


@pytest.mark.parametrize("relax", [1, 2, 3], ids=["jacobi", "rbgs", "rbgs_nonsym"])
@pytest.mark.parametrize("nx,ny,ky,inh,gamma", PERIODIC_CASES)
def test_periodic_vcycle_bitwise(ctx, stslib, oracle, relax, nx, ny, ky, inh, gamma):
    """The V-cycle on the reference's periodic problem (per-face couplings, homogeneous or
    k (1 + 0.99 sin), ky = 0 as in the harness, odd coarse sizes), GPU and oracle bit for bit."""
    pk = dict(kind=2, nx=nx, ny=ny, kx=1.0, ky=ky, inhomogeneous=inh)
    G = stslib.Problem(ctx, **pk)
    r = np.random.default_rng(nx * ny).standard_normal(nx * ny)
    mg = stslib.PFMG(G, relax=relax, nrelax=2)
    R = stslib.NVector.from_numpy(ctx, r)
    Z = G.vector()
    mg.psolve(R, Z, gamma)
    z_o, nl = oracle.Problem(**pk).pfmg_vcycle(gamma, r, relax=relax, nrelax=2)
    assert mg.levels() == nl
    assert np.array_equal(Z.numpy(), z_o)


def test_periodic_pcg_pfmg_bitwise_and_fast(ctx, stslib, oracle):
    pk = dict(kind=2, nx=64, ny=64, kx=1.0, ky=0.0, inhomogeneous=True)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    b = np.random.default_rng(9).standard_normal(64 * 64)
    mg = stslib.PFMG(G, relax=2)
    B = stslib.NVector.from_numpy(ctx, b)
    X = G.vector()
    it, rel, rc = stslib.implicit_solve_pfmg(G, 0.05, mg, B, X, tol=1e-10)
    x_o, rc_o, it_o, rel_o = O.pcg_pfmg(0.05, b, tol=1e-10, relax=2)
    assert rc == rc_o == 0 and it == it_o and rel == rel_o <= 1e-10
    assert np.array_equal(X.numpy(), x_o)
    _, rc_j, it_j, _ = O.pcg_generic(0.05, b, tol=1e-10, maxl=100000, jacobi=True)
    assert it * 4 < it_j


def test_dirk_with_periodic_pfmg_bitwise(ctx, stslib, oracle):
    """ARKStep DIRK on the harness's problem with the PFMG-role preconditioner, --pfmg_relax 3
    --pfmg_nrelax 3 (runtests-diffusion2d.py:60,62,89), GPU and oracle bit for bit."""
    pk = dict(kind=2, nx=32, ny=32, kx=1.0, ky=0.0, inhomogeneous=True)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    mg = stslib.PFMG(G, relax=3, nrelax=3)
    ak = dict(implicit=True, order=3, rtol=1e-4, atol=1e-11, controller=2, ls="cg", maxl=20, msbp=1)
    I = stslib.ARKStep(ctx, G, 0.0, G.initial(), prec="pfmg", pfmg=mg, **ak)
    J = oracle.ArkIntegrator(O, O.initial(), prec="pfmg", pfmg_relax=3, pfmg_nrelax=3, **ak)
    y = G.vector()
    I.evolve(0.2, y)
    assert J.evolve(0.2) == 0
    sg, so = I.stats(), J.stats()
    assert (sg["nst"], sg["nli"], sg["nps"]) == (so["nst"], so["nli"], so["nps"])
    assert np.array_equal(y.numpy(), J.y)


def test_nonsymmetric_rbgs_in_gmres_bitwise(ctx, stslib, oracle):
    """--pfmg_relax 3 (nonsymmetric red/black Gauss-Seidel, runtests-diffusion2d.py:60,62):
    the V-cycle is not symmetric, so it preconditions GMRES here; GPU and oracle agree bit for
    bit in a DIRK run with it (ARKStep, SPGMR)."""
    pk = dict(kind=0, nx=48, ny=40, kx=1.0, ky=0.2)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    mg = stslib.PFMG(G, relax=3, nrelax=3)
    ak = dict(implicit=True, order=2, rtol=1e-5, atol=1e-10, controller=2, ls="gmres", maxl=20, msbp=1)
    I = stslib.ARKStep(ctx, G, 0.0, G.initial(), prec="pfmg", pfmg=mg, **ak)
    J = oracle.ArkIntegrator(O, O.initial(), prec="pfmg", pfmg_relax=3, pfmg_nrelax=3, **ak)
    y = G.vector()
    I.evolve(0.05, y)
    assert J.evolve(0.05) == 0
    assert I.stats()["nli"] == J.stats()["nli"] > 0
    assert np.array_equal(y.numpy(), J.y)


def test_sdirk2_pfmg_bitwise(ctx, stslib, oracle):
    pk = dict(kind=0, nx=40, ny=32, kx=1.0, ky=0.3)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    mg = stslib.PFMG(G, relax=2, nrelax=2)
    y = G.initial()
    its = stslib.sdirk2_evolve_pfmg(G, mg, y, 0.0, 0.01, 4, tol=1e-10)
    y_o, it_o = O.sdirk2_pfmg(O.initial(), 0.0, 0.01, 4, tol=1e-10)
    assert its == it_o > 0
    assert np.array_equal(y.numpy(), y_o)
    y_f, it_j = O.sdirk2(O.initial(), 0.0, 0.01, 4, tol=1e-10)
    assert np.linalg.norm(y_o - y_f) / np.linalg.norm(y_f) < 1e-8 and its < it_j


def test_cli_dirk_pfmg(stslib):
    import os
    import subprocess
    stslib.lib()
    exe = os.path.join(os.path.dirname(stslib.__file__), "_build", "diffusion_2D_gpu")
    out = {}
    for extra in ([], ["--pfmg_relax", "1", "--pfmg_nrelax", "3"], ["--pfmg"],
                  ["--pfmg_relax", "3", "--ls", "gmres"]):
        r = subprocess.run([exe, "--problem", "manufactured", "--nx", "48", "--ny", "48", "--integrator", "dirk",
                            "--fixedstep", "1e-3", "--tf", "0.01", "--nout", "2", "--epslin", "1e-6",
                            "--liniters", "400"] + extra,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        line = [l for l in r.stdout.split("\n") if l.startswith("Relative L2 error vs exact")][0]
        its = [l for l in r.stdout.split("\n") if l.startswith("LS iters ")][0]
        out[" ".join(extra)] = (float(line.split("=")[1]), int(its.split("=")[1]))
        if extra:
            assert "pfmg relaxtype" in r.stdout and "Total PFMG iterations" in r.stdout
    base = out[""]
    for k, (err, its) in out.items():
        assert abs(err - base[0]) <= 1e-6 * base[0]
        if k:
            assert its < base[1]
