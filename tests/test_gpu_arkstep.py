"""ARKStep (ARKStepCreate / ARKodeSetOrder / linear solver + PSetup/PSolve, diffusion_2D/
main.cpp:239-330) on the GPU against the oracle's restatement (orc_arkstep_evolve), bit for
bit: the final field and every counter (steps, attempts, error-test and Newton failures, RHS
evaluations, Newton and linear iterations, preconditioner setups and solves, J v products)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS_G2O = {"nst": "nst", "nst_attempts": "nst_att", "netf": "netf", "ncfn": "ncfn", "nfe": "nfe",
            "nfi": "nfi", "nni": "nni", "nnf": "nnf", "nli": "nli", "nlcf": "nlcf", "npe": "npe",
            "nps": "nps", "njv": "njv", "nsetups": "nsetups"}


def run_pair(ctx, stslib, oracle, pk, ak, touts):
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    y0 = G.initial()
    mg = None
    if ak.get("prec") == "pfmg":
        mg = stslib.PFMG(G, relax=ak.get("pfmg_relax", 2), nrelax=ak.get("pfmg_nrelax", 2))
    gk = {k: v for k, v in ak.items() if k not in ("pfmg_relax", "pfmg_nrelax")}
    I = stslib.ARKStep(ctx, G, 0.0, y0, pfmg=mg, **gk)
    J = oracle.ArkIntegrator(O, O.initial(), **ak)
    y = G.vector()
    for tout in touts:
        t, rc = I.evolve(tout, y)
        rc_o = J.evolve(tout)
        assert rc >= 0 and rc_o >= 0, (rc, rc_o)
        sg, so = I.stats(), J.stats()
        # no stop time: the last step passes tout and both return the dense output at tout
        assert t == J.tret == tout and sg["t"] == so["t"] >= tout
        for kg, ko in KEYS_G2O.items():
            assert sg[kg] == so[ko], (kg, sg[kg], so[ko])
        assert np.array_equal(y.numpy(), J.y), np.max(np.abs(y.numpy() - J.y))
    return I, J


@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("ls", ["cg", "gmres"])
def test_dirk_dirichlet_jacobi_bitwise(ctx, stslib, oracle, order, ls):
    pk = dict(kind=0, nx=33, ny=29, kx=1.0, ky=0.3)
    ak = dict(implicit=True, order=order, rtol=1e-5, atol=1e-10, controller=2, ls=ls, maxl=20,
              prec="jacobi", msbp=1)
    I, J = run_pair(ctx, stslib, oracle, pk, ak, [0.02, 0.05])
    assert J.stats()["nst"] > 5 and J.stats()["nli"] > 0


@pytest.mark.parametrize("order", [2, 3])
def test_dirk_reference_problem_bitwise(ctx, stslib, oracle, order):
    """The reference's periodic problem with inhomogeneous coefficients and ky = 0, the
    harness's flags (--inhomogeneous --atol 1e-11 --controller 2 --nonlinear --msbp 1,
    runtests-diffusion2d.py:76-83) at a 32^2 grid."""
    pk = dict(kind=2, nx=32, ny=32, kx=1.0, ky=0.0, inhomogeneous=True)
    ak = dict(implicit=True, order=order, rtol=1e-4, atol=1e-11, controller=2, ls="cg", maxl=20,
              prec="jacobi", msbp=1)
    run_pair(ctx, stslib, oracle, pk, ak, [0.1, 0.3])


@pytest.mark.parametrize("variant", ["noprec", "linear", "msbp20", "pid", "pfmg", "pfmg_gmres"])
def test_dirk_options_bitwise(ctx, stslib, oracle, variant):
    pk = dict(kind=1, nx=40, ny=24, kx=0.4, ky=1.0)
    ak = dict(implicit=True, order=3, rtol=1e-6, atol=1e-10, controller=2, ls="cg", maxl=40,
              prec="jacobi", msbp=1)
    if variant == "noprec":
        ak["prec"] = None
    elif variant == "linear":
        ak["linear"] = True
    elif variant == "msbp20":
        ak["msbp"] = 0
    elif variant == "pid":
        ak["controller"] = 0
    elif variant == "pfmg":
        ak.update(prec="pfmg", pfmg_relax=2, pfmg_nrelax=2)
    elif variant == "pfmg_gmres":
        ak.update(prec="pfmg", pfmg_relax=1, pfmg_nrelax=3, ls="gmres")
    run_pair(ctx, stslib, oracle, pk, ak, [0.01, 0.04])


@pytest.mark.parametrize("order", [2, 3, 4])
def test_erk_bitwise(ctx, stslib, oracle, order):
    pk = dict(kind=0, nx=24, ny=20, kx=0.05, ky=0.02)
    ak = dict(implicit=False, order=order, rtol=1e-6, atol=1e-10, controller=1)
    run_pair(ctx, stslib, oracle, pk, ak, [0.01, 0.03])


def test_dirk_fixed_step_and_one_step_mode(ctx, stslib, oracle):
    pk = dict(kind=0, nx=30, ny=30, kx=1.0, ky=1.0)
    ak = dict(implicit=True, order=2, hfixed=2e-3, ls="cg", maxl=200, prec="jacobi", msbp=1)
    run_pair(ctx, stslib, oracle, pk, ak, [0.01, 0.02])
    G = stslib.Problem(ctx, **pk)
    I = stslib.ARKStep(ctx, G, 0.0, G.initial(), implicit=True, order=3, rtol=1e-6, prec="jacobi")
    y = G.vector()
    t1, _ = I.evolve(1.0, y, stslib.ONE_STEP)
    assert I.stats()["nst"] == 1 and 0 < t1 < 1.0


def test_dirk_converges_at_its_order(ctx, stslib):
    """Fixed steps on the manufactured problem (24^2, h rho ~ 20: stiff): halving h cuts the
    temporal error by about 2^q (q = 2, 3) against a small-step run of the same method."""
    pk = dict(kind=0, nx=24, ny=24, kx=1.0, ky=1.0)
    G = stslib.Problem(ctx, **pk)
    for order in (2, 3):
        ref = None
        errs = []
        for h in (1e-4, 4e-3, 2e-3):
            I = stslib.ARKStep(ctx, G, 0.0, G.initial(), implicit=True, order=order, hfixed=h, ls="cg",
                               maxl=500, prec="jacobi", msbp=1, epslin=1e-6)
            I.set_stop_time(0.08)
            y = G.vector()
            I.evolve(0.08, y)
            if ref is None:
                ref = y.numpy()
            else:
                errs.append(np.linalg.norm(y.numpy() - ref))
        rate = np.log2(errs[0] / errs[1])
        assert abs(rate - order) < 0.35, (order, rate)


def test_print_stats_has_the_harness_labels(ctx, stslib):
    """runtests-diffusion2d.py:36-54 reads Steps, Error test fails and the RHS evaluation
    lines of ARKodePrintAllStats' table output."""
    G = stslib.Problem(ctx, kind=2, nx=16, ny=16, kx=1.0, ky=0.0, inhomogeneous=True)
    I = stslib.ARKStep(ctx, G, 0.0, G.initial(), implicit=True, order=2, rtol=1e-4, atol=1e-11)
    y = G.vector()
    I.evolve(0.05, y)
    st = I.stats()
    fe = 0
    for line in I.print_stats().splitlines():
        txt = line.split()
        if "Steps" in txt:
            assert int(txt[2]) == st["nst"]
        elif ("Error" in txt) and ("test" in txt):
            assert int(txt[4]) == st["netf"]
        elif ("Explicit" in txt) and ("RHS" in txt):
            fe += int(txt[5])
        elif ("Implicit" in txt) and ("RHS" in txt):
            fe += int(txt[5])
        elif ("LS" in txt) and ("RHS" in txt):
            fe += int(txt[5])
    assert fe == st["nfe"] + st["nfi"] + st["nfe_ls"]


@pytest.mark.parametrize("implicit,order", [(True, 3), (False, 4)])
def test_stop_time_and_dense_output_rules(ctx, stslib, oracle, implicit, order):
    """ARKStep's return rules against the oracle, bit for bit: dense output of degree 2 (DIRK3,
    with f(t_n, y_n) evaluated for it) and 3 (ERK4), a tout the last step already passed, the
    stop time (returned once, then cleared); then ONE_STEP after an interpolated return."""
    pk = dict(kind=0, nx=24, ny=20, kx=1.0, ky=0.5)
    ak = dict(implicit=implicit, order=order, rtol=1e-6, atol=1e-10, controller=0)
    if implicit:
        ak.update(ls="cg", maxl=50, prec="jacobi", msbp=1)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    I = stslib.ARKStep(ctx, G, 0.0, G.initial(), **ak)
    J = oracle.ArkIntegrator(O, O.initial(), **ak)
    I.set_stop_time(0.004)
    J.set_stop_time(0.004)
    y = G.vector()

    def both(tout, rc_expect):
        t, rc = I.evolve(tout, y)
        assert rc == rc_expect and J.evolve(tout) == rc_expect
        sg, so = I.stats(), J.stats()
        assert t == J.tret and sg["t"] == so["t"]
        for kg, ko in KEYS_G2O.items():
            assert sg[kg] == so[ko], (kg, sg[kg], so[ko])
        assert np.array_equal(y.numpy(), J.y), np.max(np.abs(y.numpy() - J.y))
        return t
    for tout in (0.0004, 0.0011, 0.0019):
        assert both(tout, 0) == tout
    tn = I.stats()["t"]
    assert tn > 0.0019
    both(0.0019 + 0.5 * (tn - 0.0019), 0)  # already passed: dense output, no step
    assert I.stats()["t"] == tn
    assert both(0.01, stslib.TSTOP_RETURN) == 0.004
    both(0.005, 0)
    nst, tn = I.stats()["nst"], I.stats()["t"]
    t1, rc = I.evolve(1.0, y, stslib.ONE_STEP)
    assert rc == 0 and t1 == tn and I.stats()["nst"] == nst
    t2, rc = I.evolve(1.0, y, stslib.ONE_STEP)
    assert rc == 0 and t2 > tn and I.stats()["nst"] == nst + 1
