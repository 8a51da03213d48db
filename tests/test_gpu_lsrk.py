"""LSRKStep STS integration on the GPU against the CPU oracle.

Fused FP64 path: bit-for-bit equal to the oracle (same stage arithmetic, exact WRMS, same
host step control), hence also within the 1e-12 relative-L2 bar of the target. Mixed path:
bit-for-bit equal to the oracle's restatement of the FP32-increment scheme, and within
1e-6 relative L2 of the FP64 solution. Generic path (any ARKRhsFn): the reference's scalar
known-answer problem gkeyll_diffusion/analytic_CR_test.c."""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAT_KEYS = ("nst", "nst_attempts", "netf", "nfe", "ndee", "nst_exp", "stage_max", "stages_total")
STS_ILL_INPUT = -22  # include/stsgpu.h


def run_pair(ctx, stslib, oracle, pk, ok, touts, graphs=True):
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    y0 = G.initial()
    I = stslib.LSRKStep(ctx, G, 0.0, y0, graphs=graphs, **ok)
    J = oracle.Integrator(O, O.initial(), **{k: v for k, v in ok.items() if k != "fused_periodic"})
    yout = G.vector()
    for tout in touts:
        t, rc = I.evolve(tout, yout)
        rc_o = J.evolve(tout)
        assert rc_o == 0 and rc >= 0
        # no stop time: the last step passes tout and both return the dense output at tout
        assert t == J.tret == tout and I.stats()["t"] == J.stats()["t"] >= tout
        yg = yout.numpy()
        sg, so = I.stats(), J.stats()
        for k in STAT_KEYS:
            assert sg[k] == so[k], (k, sg[k], so[k])
        assert sg["hnext"] == so["hnext"]
        assert np.array_equal(yg, J.y), np.max(np.abs(yg - J.y))
    return yg, J.y, I.stats()


@pytest.mark.parametrize("nx,ny", [(8, 8), (17, 9), (33, 32), (64, 64), (130, 66)])
@pytest.mark.parametrize("method", [0, 1])
def test_fused_fp64_bitwise(ctx, stslib, oracle, nx, ny, method):
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=0.3)
    ok = dict(method=method, rtol=1e-6, atol=1e-10)
    run_pair(ctx, stslib, oracle, pk, ok, [0.02, 0.05])


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "nvector"])
@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("inhomogeneous", [False, True])
def test_reference_mode_periodic_bitwise(ctx, stslib, oracle, method, inhomogeneous, fused):
    """The reference's own problem (periodic wrap, Gaussian x sine initial state,
    initial.cpp:42-43; optional inhomogeneous faces, diffusion.cpp:36-46) through the
    generic integrator path (fused stage / step-end kernels, or the plain RHS and N_Vector
    sequence), bit for bit against the oracle."""
    pk = dict(kind=2, nx=48, ny=40, kx=1.0, ky=0.5, inhomogeneous=inhomogeneous)
    ok = dict(method=method, rtol=1e-5, atol=1e-9, fused_periodic=fused)
    run_pair(ctx, stslib, oracle, pk, ok, [0.002, 0.01])


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("inhomogeneous", [False, True])
def test_reference_mode_mixed_bitwise(ctx, stslib, oracle, method, inhomogeneous):
    """The mixed form on the reference's own periodic problem (FP32 increments in the
    difference form with FP32 face tables, diffusion.cpp:36-46 coefficients): GPU and the
    oracle's mixed integrator bit for bit, adaptive steps."""
    pk = dict(kind=2, nx=64, ny=48, kx=1.0, ky=0.5, inhomogeneous=inhomogeneous)
    ok = dict(method=method, rtol=1e-5, atol=1e-9, mixed=True)
    run_pair(ctx, stslib, oracle, pk, ok, [0.05, 0.2])


@pytest.mark.parametrize("method,inhomogeneous", [(0, False), (1, False), (0, True)])
def test_reference_mode_mixed_within_1e6_of_fp64(ctx, stslib, method, inhomogeneous):
    """Same step sequence (fixed h): mixed reference mode against the FP64 reference mode at
    256^2 stays far inside 1e-6 relative L2 (about 1e-9)."""
    pk = dict(kind=2, nx=256, ny=256, kx=1.0, ky=0.5, inhomogeneous=inhomogeneous)
    out = {}
    for mixed in (False, True):
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=method, mixed=mixed, hfixed=1e-3)
        y = G.vector()
        I.evolve(0.5, y)
        out[mixed] = y.numpy()
    rel = np.linalg.norm(out[True] - out[False]) / np.linalg.norm(out[False])
    assert np.isfinite(rel) and rel < 1e-7, rel


@pytest.mark.parametrize("controller", [0, 1, 2, 3, 4, 5])
def test_controllers_bitwise(ctx, stslib, oracle, controller):
    pk = dict(kind=0, nx=48, ny=40, kx=1.0, ky=0.01)
    ok = dict(method=1, rtol=1e-5, atol=1e-9, controller=controller)
    run_pair(ctx, stslib, oracle, pk, ok, [0.03])


@pytest.mark.parametrize("method", [0, 1])
def test_mixed_bitwise(ctx, stslib, oracle, method):
    pk = dict(kind=0, nx=96, ny=64, kx=1.0, ky=0.01)
    ok = dict(method=method, rtol=1e-6, atol=1e-10, mixed=True)
    run_pair(ctx, stslib, oracle, pk, ok, [0.01, 0.03])


@pytest.mark.parametrize("nx,ny", [(96, 64), (260, 70), (130, 66), (1024, 1000)])
def test_tma_stage_kernel_matches_register_kernel(ctx, stslib, oracle, nx, ny):
    """The TMA-pipelined mixed stage kernel and the register-marching one give the same bits
    (and both equal the oracle), including ragged tiles and rows not a multiple of 4."""
    pk = dict(kind=0, nx=nx, ny=ny, kx=1.0, ky=0.05)
    out = []
    for variant in (1, 0, 2, 3, 4, 5, 6, 7):
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, rtol=1e-6, atol=1e-10, mixed=True,
                            stage_kernel=variant)
        y = G.vector()
        I.evolve(0.01, y)
        out.append((y.numpy(), I.stats()))
    for y, _ in out[1:]:
        assert np.array_equal(out[0][0], y)
    O = oracle.Problem(**pk)
    J = oracle.Integrator(O, O.initial(), method=1, rtol=1e-6, atol=1e-10, mixed=True)
    assert J.evolve(0.01) == 0
    assert np.array_equal(out[0][0], J.y)


@pytest.mark.parametrize("nx,ny,kx", [(8, 8, 200.0), (96, 64, 1.0), (260, 70, 1.0), (248, 130, 1.0)])
@pytest.mark.parametrize("kind", [0, 1])
def test_fused_stage_groups_bitwise(ctx, stslib, oracle, nx, ny, kx, kind):
    """Several mixed stages per launch (temporal blocking on 120 x 32 and 120 x 64 shared-memory
    tiles with a 4-cell halo) give the oracle's bits: groups of 2, 3 and 4 stages, both tile
    heights, the forced (kind 0) and unforced (kind 1) problems, ragged tiles, and the shorter
    last group of every step whose stage count leaves a remainder (steps of 9 to 42 stages)."""
    pk = dict(kind=kind, nx=nx, ny=ny, kx=kx, ky=0.05 * kx)
    pm, qm, amp = [1, 3, 7], [2, 5, 1], [1.0, -0.5, 0.25]
    O = oracle.Problem(**pk)
    ok = dict(method=1, rtol=1e-6 if kind == 0 else 1e-3, atol=1e-10 if kind == 0 else 1e-6, mixed=True)
    J = oracle.Integrator(O, O.initial() if kind == 0 else O.initial_modes(pm, qm, amp), **ok)
    assert J.evolve(0.01) == 0
    so = J.stats()
    assert so["stage_max"] >= 5
    for ks in (2, 3, 4):
        for cfg in range(1, 7):
            G = stslib.Problem(ctx, **pk)
            y0 = G.initial() if kind == 0 else G.initial_modes(pm, qm, amp)
            I = stslib.LSRKStep(ctx, G, 0.0, y0, stage_fusion=(ks, cfg), **ok)
            y = G.vector()
            I.evolve(0.01, y)
            info = I.stage_fusion_info()
            assert info["ks"] == ks and info["config"] == cfg, info
            sg = I.stats()
            for k in STAT_KEYS:
                assert sg[k] == so[k], (ks, cfg, k, sg[k], so[k])
            assert np.array_equal(y.numpy(), J.y), (ks, cfg, np.max(np.abs(y.numpy() - J.y)))


def test_fused_stage_groups_1024(ctx, stslib, oracle):
    """Four stages per launch on a 1024 x 1000 grid (nine tile columns, the last one 64 wide),
    every tile configuration, against one launch per stage and against the oracle; the
    autotuned choice, whichever it is, gives the same bits."""
    pk = dict(kind=0, nx=1024, ny=1000, kx=1.0, ky=0.05)
    ok = dict(method=0, rtol=1e-6, atol=1e-10, mixed=True)
    out = []
    for fusion in ((1, 0),) + tuple((4, cfg) for cfg in range(1, 7)) + ((0, 0),):
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), stage_fusion=fusion, **ok)
        y = G.vector()
        I.evolve(0.002, y)
        out.append((y.numpy(), I.stats(), I.stage_fusion_info()))
    assert out[0][2]["ks"] == 1 and out[1][2]["ks"] == 4
    assert [o[2]["tile_rows"] for o in out[1:7]] == [32, 64, 60, 64, 58, 64]
    for y, st, _ in out[1:]:
        assert np.array_equal(out[0][0], y)
        assert all(st[k] == out[0][1][k] for k in STAT_KEYS)
    O = oracle.Problem(**pk)
    J = oracle.Integrator(O, O.initial(), **ok)
    assert J.evolve(0.002) == 0
    assert np.array_equal(out[0][0], J.y)


def test_stage_fusion_rejects_bad_arguments(ctx, stslib):
    G = stslib.Problem(ctx, kind=0, nx=32, ny=32)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), mixed=True)
    L = stslib.lib()
    assert L.STS_LSRKStepSetStageFusion(I.mem, 5, 0) == STS_ILL_INPUT
    assert L.STS_LSRKStepSetStageFusion(I.mem, 4, 7) == STS_ILL_INPUT
    assert L.STS_LSRKStepSetStageFusion(I.mem, -1, 0) == STS_ILL_INPUT
    assert L.STS_LSRKStepSetStageFusion(I.mem, 4, 3) == 0


def test_unforced_and_small_stage_cap_bitwise(ctx, stslib, oracle):
    pk = dict(kind=1, nx=128, ny=80, kx=0.2, ky=0.9)
    ok = dict(method=1, rtol=1e-3, atol=1e-6, smax=4)
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    pm, qm, amp = [1, 3, 7], [2, 5, 1], [1.0, -0.5, 0.25]
    y0 = G.initial_modes(pm, qm, amp)
    I = stslib.LSRKStep(ctx, G, 0.0, y0, **ok)
    J = oracle.Integrator(O, O.initial_modes(pm, qm, amp), **ok)
    yout = G.vector()
    I.evolve(0.01, yout)
    assert J.evolve(0.01) == 0
    sg, so = I.stats(), J.stats()
    assert sg["stage_max"] == so["stage_max"] == 4
    assert sg["nst_exp"] == so["nst_exp"] > 0
    assert np.array_equal(yout.numpy(), J.y)


def test_power_iteration_estimator_bitwise(ctx, stslib, oracle):
    pk = dict(kind=0, nx=40, ny=40, kx=1.0, ky=1.0)
    ok = dict(method=0, rtol=1e-6, atol=1e-10, power=(100, 0.01))
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), **ok)
    J = oracle.Integrator(O, O.initial(), method=0, rtol=1e-6, atol=1e-10, internaleig=True)
    yout = G.vector()
    I.evolve(0.02, yout)
    assert J.evolve(0.02) == 0
    assert I.stats()["spectral_radius"] == J.stats()["spectral_radius"]
    assert np.array_equal(yout.numpy(), J.y)


def test_power_iteration_warmups_bitwise(ctx, stslib, oracle):
    """Warm-up ("preprocessing") power iterations before the first and the later estimates
    (LSRKStepSetNumDomEigEst[Init]PreprocessIters) against the oracle, bit for bit."""
    pk = dict(kind=0, nx=40, ny=32, kx=1.0, ky=0.5)
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, rtol=1e-6, atol=1e-10,
                        power=(100, 0.01), dee_warmups=(7, 2))
    J = oracle.Integrator(O, O.initial(), method=1, rtol=1e-6, atol=1e-10, internaleig=True,
                          dee_warmups=(7, 2))
    yout = G.vector()
    I.evolve(0.05, yout)
    assert J.evolve(0.05) == 0
    si, sj = I.stats(), J.stats()
    assert si["ndee"] >= 2 and si["nfe_dee"] == sj["nfe_dee"]
    assert si["spectral_radius"] == sj["spectral_radius"]
    assert np.array_equal(yout.numpy(), J.y)


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("fused", [True, False], ids=["fused", "nvector"])
def test_stop_time_and_dense_output_rules(ctx, stslib, oracle, mixed, fused):
    """ARKodeEvolve's return rules on the GPU against the oracle, bit for bit: outputs past
    which the last step went (dense output), a tout that the last step already passed (no
    step taken), the stop time (TSTOP_RETURN, then cleared), and ONE_STEP after an
    interpolated return (y_n returned without a step)."""
    if fused:
        pk = dict(kind=0, nx=48, ny=40, kx=1.0, ky=0.05)
    else:
        pk = dict(kind=2, nx=40, ny=32, kx=1.0, ky=0.5, inhomogeneous=True)
    ok = dict(method=1, rtol=1e-6, atol=1e-10, mixed=mixed)
    G, O = stslib.Problem(ctx, **pk), oracle.Problem(**pk)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), **ok)
    J = oracle.Integrator(O, O.initial(), **ok)
    I.set_stop_time(0.004)
    J.set_stop_time(0.004)
    y = G.vector()

    def both(tout, rc_expect):
        t, rc = I.evolve(tout, y)
        assert rc == rc_expect and J.evolve(tout) == rc_expect
        assert t == J.tret and I.stats()["t"] == J.stats()["t"]
        assert I.stats()["nst"] == J.stats()["nst"]
        assert np.array_equal(y.numpy(), J.y), np.max(np.abs(y.numpy() - J.y))
        return t
    for tout in (0.0005, 0.0011, 0.0023):
        assert both(tout, 0) == tout
    assert I.stats()["t"] > 0.0023
    nst = I.stats()["nst"]
    both(0.0023 + 0.25 * (I.stats()["t"] - 0.0023), 0)  # already passed: dense output only
    assert I.stats()["nst"] == nst
    assert both(0.01, stslib.TSTOP_RETURN) == 0.004
    both(0.006, 0)  # the stop time was cleared
    # ONE_STEP after an interpolated NORMAL return: y_n at t_n, no step
    nst, tn = I.stats()["nst"], I.stats()["t"]
    t1, rc = I.evolve(1.0, y, stslib.ONE_STEP)
    assert rc == 0 and t1 == tn and I.stats()["nst"] == nst
    t2, rc = I.evolve(1.0, y, stslib.ONE_STEP)
    assert rc == 0 and t2 > tn and I.stats()["nst"] == nst + 1


def test_graphs_do_not_change_results(ctx, stslib, oracle):
    pk = dict(kind=0, nx=64, ny=32, kx=1.0, ky=1.0)
    ok = dict(method=1, rtol=1e-6, atol=1e-10)
    a, _, _ = run_pair(ctx, stslib, oracle, pk, ok, [0.02], graphs=True)
    b, _, _ = run_pair(ctx, stslib, oracle, pk, ok, [0.02], graphs=False)
    assert np.array_equal(a, b)


def test_golden_fixtures(ctx, stslib):
    for name in ("oracle_rkc_17x9", "oracle_rkl_32", "oracle_rkl_mixed_32"):
        g = np.load(os.path.join(GOLD, name + ".npz"))
        pk = json.loads(str(g["problem"]))
        ok = json.loads(str(g["opts"]))
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), **ok)
        I.set_stop_time(float(g["tf"]))  # as the fixtures' runs (diffusion_2D/main.cpp:384)
        yout = G.vector()
        assert I.evolve(float(g["tf"]), yout)[1] == stslib.TSTOP_RETURN
        assert I.stats()["nst"] == int(g["nst"])
        assert np.max(np.abs(yout.numpy() - g["y"])) <= 1e-12 * np.max(np.abs(g["y"]))


def test_mixed_within_1e6_of_fp64(ctx, stslib):
    """Same step sequence (fixed h): the FP32-increment error stays below 1e-6 rel L2."""
    pk = dict(kind=0, nx=512, ny=512, kx=1.0, ky=0.01)
    out = {}
    for mixed in (False, True):
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, mixed=mixed, hfixed=1e-3)
        y = G.vector()
        I.evolve(0.05, y)
        out[mixed] = y.numpy()
    rel = np.linalg.norm(out[True] - out[False]) / np.linalg.norm(out[False])
    assert rel < 1e-6


def fixed_step_for(G, method, s):
    """A step size just inside the stability bound of `s` stages for this problem."""
    rho = 1.01 * abs(G.dom_eig())
    if method == 0:
        return ((s - 1.0) ** 2 - 1.0) / (1.54 * rho) * 0.999
    return (s * s + s - 2.0) / (2.0 * rho) * 0.999


@pytest.mark.parametrize("method", [0, 1])
def test_mixed_drift_long_stage_chains(ctx, stslib, oracle, method):
    """Reduced-size form of the 8192^2 anisotropic workload (kx = 1, ky = 1e-2, t in [0, 0.05])
    with the per-step stage count of the full run (about 190): at 1024^2 that is 19-23 fixed
    steps. This is the regime where the FP32 stage arithmetic accumulates: summing the
    O(|d|) terms directly ended 2.2e-6 (RKC2) / 1.7e-6 (RKL2) from FP64 here; the difference
    form ends near 1e-8. The accuracy target is 1e-6; the test holds 1e-7. The mixed
    result also equals the oracle's mixed integrator bit for bit."""
    pk = dict(kind=0, nx=1024, ny=1024, kx=1.0, ky=0.01)
    tf = 0.05
    out = {}
    for mixed in (False, True):
        G = stslib.Problem(ctx, **pk)
        h = fixed_step_for(G, method, 196)
        h = tf / math.ceil(tf / h)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=method, mixed=mixed, hfixed=h)
        y = G.vector()
        t, rc = I.evolve(tf, y)
        assert t == tf and I.stats()["stage_max"] > 180
        out[mixed] = y.numpy()
    rel = np.linalg.norm(out[True] - out[False]) / np.linalg.norm(out[False])
    assert rel < 1e-7, rel
    O = oracle.Problem(**pk)
    J = oracle.Integrator(O, O.initial(), method=method, mixed=True, hfixed=h)
    assert J.evolve(tf) == 0
    assert np.array_equal(out[True], J.y)


def test_mixed_drift_adaptive_rkc_2048(ctx, stslib):
    """RKC2 at rtol 1e-4 on the 2048^2 anisotropic problem to t = 0.05, adaptive steps in
    both precisions (their step sequences differ: the mixed error estimate carries FP32
    noise). The mixed field stays within 1e-6 relative L2 of the FP64 one."""
    pk = dict(kind=0, nx=2048, ny=2048, kx=1.0, ky=0.01)
    out = {}
    for mixed in (False, True):
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=0, rtol=1e-4, atol=1e-10, mixed=mixed)
        I.set_stop_time(0.05)
        y = G.vector()
        t, rc = I.evolve(0.05, y)
        assert t == 0.05 and rc == stslib.TSTOP_RETURN
        out[mixed] = y.numpy()
    rel = np.linalg.norm(out[True] - out[False]) / np.linalg.norm(out[False])
    assert rel < 1e-6, rel


def test_4096_rkl2_first_steps_bitwise(ctx, stslib, oracle):
    """Config-2 size (4096^2, RKL2, rtol 1e-6, atol 1e-10): the first steps bit for bit."""
    pk = dict(kind=0, nx=4096, ny=4096, kx=1.0, ky=1.0)
    ok = dict(method=1, rtol=1e-6, atol=1e-10, maxsteps=6)
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), **ok)
    J = oracle.Integrator(O, O.initial(), **ok)
    yout = G.vector()
    I.evolve(0.1, yout)
    J.evolve(0.1)
    sg, so = I.stats(), J.stats()
    assert sg["nst"] == so["nst"] == 6
    assert sg["stage_max"] == so["stage_max"] and sg["stage_max"] > 100
    assert np.array_equal(yout.numpy(), J.y)


def test_8192_mixed_properties(ctx, stslib):
    """Full config-3 size: two fixed steps of 148 RKL2 stages stay finite, near the exact
    solution, and the mixed result agrees with the FP64 one to 1e-6 relative L2."""
    pk = dict(kind=0, nx=8192, ny=8192, kx=1.0, ky=0.01)
    out = {}
    for mixed in (True, False):
        G = stslib.Problem(ctx, **pk)
        I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, mixed=mixed, hfixed=2e-5)
        y = G.vector()
        t, rc = I.evolve(4e-5, y)
        assert I.stats()["stage_max"] > 100
        out[mixed] = (y.numpy(), t)
        ex = G.exact(t).numpy()
        err = np.linalg.norm(out[mixed][0] - ex) / np.linalg.norm(ex)
        assert np.isfinite(out[mixed][0]).all() and err < 1e-4
    assert out[True][1] == out[False][1]
    rel = np.linalg.norm(out[True][0] - out[False][0]) / np.linalg.norm(out[False][0])
    assert rel < 1e-6


def test_generic_path_analytic_cr(ctx, stslib):
    """analytic_CR_test.c: y' = lambda (y - atan t) + 1/(1+t^2), exact atan t."""
    with open(os.path.join(GOLD, "reference_kats.json")) as f:
        k = json.load(f)["analytic_CR"]
    lam = k["lambda"]
    L = stslib.lib()

    def f(t, y, ydot):
        L.N_VScale_Sts(lam, y.h, ydot.h)
        L.N_VAddConst_Sts(ydot.h, 1.0 / (1.0 + t * t) - lam * math.atan(t), ydot.h)
        return 0

    # as the reference test runs it (no stop time: outputs from the dense output, degree 1 for
    # this order-2 method), and with every output time a stop time
    for stops, bound in ((False, 1e-4), (True, 1e-5)):
        y0 = stslib.NVector.from_numpy(ctx, np.array([k["y0"]]))
        I = stslib.LSRKStep(ctx, f, 0.0, y0, method=1, rtol=k["rtol"], atol=k["atol"],
                            smax=k["stage_max_limit"], dom_eig=lambda t: lam)
        stslib.lib().STS_LSRKStepSetDomEigSafetyFactor(I.mem, k["eigsafety"])
        stslib.lib().STS_LSRKStepSetDomEigFrequency(I.mem, k["eigfrequency"])
        y = stslib.NVector(ctx, 1)
        maxerr = 0.0
        for i in range(1, k["nout"] + 1):
            tout = k["tf"] * i / k["nout"]
            if stops:
                I.set_stop_time(tout)
            t, rc = I.evolve(tout, y)
            assert abs(t - tout) < 1e-14
            maxerr = max(maxerr, abs(y.numpy()[0] - math.atan(t)))
        assert maxerr < bound, (stops, maxerr)
        assert I.stats()["ndee"] == 1


def test_generic_path_matches_fused(ctx, stslib):
    pk = dict(kind=0, nx=32, ny=24, kx=1.0, ky=0.5)
    G = stslib.Problem(ctx, **pk)
    L = stslib.lib()

    def f(t, y, ydot):
        return L.STS_Diffusion(t, y.h, ydot.h, G.h)

    out = []
    for rhs in (G, f):
        I = stslib.LSRKStep(ctx, rhs, 0.0, G.initial(), method=0, rtol=1e-6, atol=1e-10,
                            dom_eig=lambda t: G.dom_eig())
        y = G.vector()
        I.evolve(0.05, y)
        out.append(y.numpy())
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[0]) < 1e-10


def test_recoverable_rhs_failure_retries(ctx, stslib):
    """Host-side fault injection: an RHS that returns +1 once (recoverable,
    diffusion_2D.cpp:900-933 convention) makes the step retry with a smaller h; -1 aborts."""
    pk = dict(kind=0, nx=16, ny=16)
    G = stslib.Problem(ctx, **pk)
    L = stslib.lib()
    calls = {"n": 0}

    def flaky(t, y, ydot):
        calls["n"] += 1
        if calls["n"] == 6:
            return 1
        return L.STS_Diffusion(t, y.h, ydot.h, G.h)

    I = stslib.LSRKStep(ctx, flaky, 0.0, G.initial(), method=0, dom_eig=lambda t: G.dom_eig())
    y = G.vector()
    t, rc = I.evolve(0.01, y)
    assert t == 0.01 and rc >= 0

    def broken(t, y, ydot):
        return -1

    J = stslib.LSRKStep(ctx, broken, 0.0, G.initial(), method=0, dom_eig=lambda t: G.dom_eig())
    with pytest.raises(stslib.STSError):
        J.evolve(0.01, y)


def test_evolve_rejects_bad_arguments(ctx, stslib):
    """The C ABI turns misuse into error codes and keeps the integrator usable: a NULL or
    wrong-length output vector, an invalid task, a tout behind the last step (no dense output
    there), a stage count beyond the fixed-step limit."""
    import ctypes as C
    L = stslib.lib()
    G = stslib.Problem(ctx, kind=0, nx=32, ny=24, kx=1.0, ky=0.5)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, rtol=1e-6, atol=1e-10)
    y = G.vector()
    t = C.c_double()
    assert L.STS_ARKodeEvolve(I.mem, 0.01, None, C.byref(t), stslib.NORMAL) == STS_ILL_INPUT
    short = stslib.NVector(ctx, 32 * 24 - 1)
    assert L.STS_ARKodeEvolve(I.mem, 0.01, short.h, C.byref(t), stslib.NORMAL) == STS_ILL_INPUT
    assert L.STS_ARKodeEvolve(I.mem, 0.01, y.h, C.byref(t), 7) == STS_ILL_INPUT  # no such task
    t1, rc = I.evolve(0.01, y)
    assert rc == 0 and t1 == 0.01
    tn, hl = I.stats()["t"], I.stats()["hlast"]
    assert L.STS_ARKodeEvolve(I.mem, tn - 3.0 * hl, y.h, C.byref(t), stslib.NORMAL) == STS_ILL_INPUT
    t2, rc = I.evolve(0.02, y)  # still usable
    assert rc == 0 and t2 == 0.02 and np.isfinite(y.numpy()).all()
    J = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, hfixed=1.0, smax=10)
    assert L.STS_ARKodeEvolve(J.mem, 0.5, y.h, C.byref(t), stslib.NORMAL) == STS_ILL_INPUT

