"""Failure detection without a GPU fault.

Device side: the bounded-wait path of the pipeline kernels (a barrier that nothing completes,
polled a bounded number of times, the context's error word set and read back by the host),
then the same context runs an integration bit for bit against the oracle.
Host side: non-finite values injected into the host buffer of the initial state, into one
instance of the batched launch, and into an RHS evaluation in the middle of a run. The
reference's integrator fails the step (a NaN error estimate is an error-test failure that
no step-size reduction can cure, returned as ARK_ERR_FAILURE = -3); the GPU paths must return
the same status after the same attempts, RHS evaluations and stage counts as the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
FAIL_KEYS = ("nst", "nst_attempts", "netf", "nfe", "stages_total", "stage_max")


def test_bounded_wait_times_out_and_context_survives(ctx, stslib, oracle):
    assert ctx.wait_self_test(True, 1000) == 0
    assert ctx.wait_self_test(False, 1000) == -3
    assert b"timed out after 1000 polls" in stslib.lib().STS_GetLastError()
    # the word was cleared: the next wait that completes reports success
    assert ctx.wait_self_test(True, 10) == 0
    assert ctx.wait_self_test(False, 1) == -3
    assert ctx.wait_self_test(False, 0) == -22
    assert ctx.wait_self_test(False, (1 << 20) + 1) == -22
    # the context still runs the TMA-pipelined mixed path, bit for bit
    pk = dict(kind=0, nx=96, ny=64, kx=1.0, ky=0.01)
    G = stslib.Problem(ctx, **pk)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), method=1, rtol=1e-6, atol=1e-10, mixed=True)
    y = G.vector()
    I.evolve(0.01, y)
    O = oracle.Problem(**pk)
    J = oracle.Integrator(O, O.initial(), method=1, rtol=1e-6, atol=1e-10, mixed=True)
    assert J.evolve(0.01) == 0
    assert np.array_equal(y.numpy(), J.y)


CASES = [
    ("fp64_rkc", dict(kind=0, nx=33, ny=32), dict(method=0)),
    ("fp64_rkl", dict(kind=0, nx=33, ny=32), dict(method=1)),
    ("mixed_rkl", dict(kind=0, nx=96, ny=64), dict(method=1, mixed=True)),
    ("periodic_fused", dict(kind=2, nx=48, ny=40), dict(method=1, fused_periodic=True)),
    ("periodic_nvector", dict(kind=2, nx=48, ny=40), dict(method=0, fused_periodic=False)),
]


@pytest.mark.parametrize("value", [np.nan, np.inf], ids=["nan", "inf"])
@pytest.mark.parametrize("name,pk,ok", CASES, ids=[c[0] for c in CASES])
def test_nonfinite_initial_state_fails_like_oracle(ctx, stslib, oracle, name, pk, ok, value):
    ok = dict(ok, rtol=1e-6, atol=1e-10)
    O = oracle.Problem(**pk)
    y0 = O.initial()
    y0[37] = value
    J = oracle.Integrator(O, y0, **{k: v for k, v in ok.items() if k != "fused_periodic"})
    assert J.evolve(0.01) == -3
    G = stslib.Problem(ctx, **pk)
    I = stslib.LSRKStep(ctx, G, 0.0, stslib.NVector.from_numpy(ctx, y0), **ok)
    y = G.vector()
    with pytest.raises(stslib.STSError):
        I.evolve(0.01, y)
    sg, so = I.stats(), J.stats()
    assert sg["t"] == so["t"] == 0.0
    for k in FAIL_KEYS:
        assert sg[k] == so[k], (k, sg[k], so[k])
    # a clean integrator on the same context is unaffected
    K = stslib.LSRKStep(ctx, G, 0.0, G.initial(), **ok)
    K.evolve(0.01, y)
    Jc = oracle.Integrator(O, O.initial(), **{k: v for k, v in ok.items() if k != "fused_periodic"})
    assert Jc.evolve(0.01) == 0
    assert np.array_equal(y.numpy(), Jc.y)


def test_nan_rhs_mid_run_fails_the_step(ctx, stslib):
    """An RHS that returns NaN values at one evaluation (return code 0): the step in progress
    fails its error test, the integrator returns the failure and keeps the last accepted
    state; t never passes the last accepted step."""
    pk = dict(kind=0, nx=16, ny=16)
    G = stslib.Problem(ctx, **pk)
    L = stslib.lib()
    calls = {"n": 0}

    def poisoned(t, y, ydot):
        calls["n"] += 1
        rc = L.STS_Diffusion(t, y.h, ydot.h, G.h)
        if calls["n"] == 40:
            ydot.const(float("nan"))
        return rc

    I = stslib.LSRKStep(ctx, poisoned, 0.0, G.initial(), method=0, dom_eig=lambda t: G.dom_eig())
    y = G.vector()
    with pytest.raises(stslib.STSError):
        I.evolve(0.05, y)
    s = I.stats()
    assert s["netf"] >= 1 and s["nst"] >= 1 and 0.0 < s["t"] < 0.05
    assert calls["n"] >= 40
    # the same RHS without the poisoned call reaches the end
    calls["n"] = -10 ** 9
    J = stslib.LSRKStep(ctx, poisoned, 0.0, G.initial(), method=0, dom_eig=lambda t: G.dom_eig())
    t, rc = J.evolve(0.05, y)
    assert t == 0.05 and rc >= 0 and np.all(np.isfinite(y.numpy()))


def test_batch_isolates_a_nonfinite_instance(ctx, stslib, oracle):
    """One instance of the batched launch starts from a state holding a NaN: that instance
    fails after the oracle's attempts, every other instance ends bit for bit as the oracle's."""
    inst = stslib.make_batch_instances(count=12, seed=7, sizes=(16, 24, 32, 48, 40), nmodes=4,
                                       pmax=6)
    B = stslib.Batch(ctx, inst)
    y = B.state()
    bad = 5
    y[B.offsets[bad] + 11] = np.nan
    B.set_state(y)
    with pytest.raises(stslib.STSError):
        B.evolve(0.01, method=stslib.RKL, rtol=1e-6, atol=1e-10)
    yb = B.state()
    for i, (n, kx, ky, p, q, a) in enumerate(inst):
        P = oracle.Problem(oracle.UNFORCED, n, n, kx=kx, ky=ky)
        y0 = P.initial_modes(p, q, a)
        if i == bad:
            y0[11] = np.nan
        J = oracle.Integrator(P, y0, method=oracle.RKL, rtol=1e-6, atol=1e-10, tstop=0.01)
        rc = J.evolve(0.01)
        st, so = B.stats(i), J.stats()
        for k in ("nst", "nst_attempts", "netf", "stages_total", "stage_max"):
            assert st[k] == so[k], (i, k, st[k], so[k])
        if i == bad:
            assert rc == -3 and st["t"] == 0.0
        else:
            assert rc == 1 and st["t"] == 0.01
            assert np.array_equal(B.instance_state(yb, i), J.y), i
