"""Batched persistent STS launch against the CPU oracle, instance by instance.

Each instance is integrated by the oracle's single-problem integrator with the same method,
tolerances and step rules. The batch kernel takes its stage coefficients from the host's
table and evaluates the controllers with the deterministic pow shared with the oracle, so
every instance must reproduce the oracle's step sequence and final state bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(stslib, count=20, seed=7):
    return stslib.make_batch_instances(count=count, seed=seed, sizes=(16, 24, 32, 48, 40),
                                       nmodes=4, pmax=6)


@pytest.mark.parametrize("method,controller", [(1, 0), (0, 0), (1, 1), (0, 2), (1, 3), (0, 4), (1, 5)])
def test_batch_matches_oracle_per_instance(ctx, stslib, oracle, method, controller):
    inst = small_batch(stslib)
    B = stslib.Batch(ctx, inst)
    B.evolve(0.01, method=method, rtol=1e-6, atol=1e-10, controller=controller)
    y = B.state()
    for i, (n, kx, ky, p, q, a) in enumerate(inst):
        P = oracle.Problem(oracle.UNFORCED, n, n, kx=kx, ky=ky)
        J = oracle.Integrator(P, P.initial_modes(p, q, a), method=method, rtol=1e-6, atol=1e-10,
                              controller=controller, tstop=0.01)
        assert J.evolve(0.01) == 1
        yi = B.instance_state(y, i)
        st, so = B.stats(i), J.stats()
        assert st["t"] == 0.01
        for k in ("nst", "nst_attempts", "netf", "stages_total", "stage_max"):
            assert st[k] == so[k], (i, k, st[k], so[k])
        assert np.array_equal(yi, J.y), (i, np.abs(yi - J.y).max())


@pytest.mark.parametrize("method,controller", [(1, 0), (0, 0), (1, 3), (0, 5)])
def test_batch_mixed_matches_oracle_per_instance(ctx, stslib, oracle, method, controller):
    """FP32 stage increments in the batched launch: every instance equals the oracle's mixed
    single-problem integrator bit for bit. Against the FP64 batch the two adaptive runs take
    their own step sequences, so they agree to the tolerance level (1e-5 relative L2 at
    rtol 1e-6), not to rounding."""
    inst = small_batch(stslib)
    B = stslib.Batch(ctx, inst)
    B.set_mixed(True)
    B.evolve(0.01, method=method, rtol=1e-6, atol=1e-10, controller=controller)
    y = B.state()
    C64 = stslib.Batch(ctx, inst)
    C64.evolve(0.01, method=method, rtol=1e-6, atol=1e-10, controller=controller)
    y64 = C64.state()
    for i, (n, kx, ky, p, q, a) in enumerate(inst):
        P = oracle.Problem(oracle.UNFORCED, n, n, kx=kx, ky=ky)
        J = oracle.Integrator(P, P.initial_modes(p, q, a), method=method, rtol=1e-6, atol=1e-10,
                              controller=controller, mixed=True, tstop=0.01)
        assert J.evolve(0.01) == 1
        yi = B.instance_state(y, i)
        st, so = B.stats(i), J.stats()
        assert st["t"] == 0.01
        for k in ("nst", "nst_attempts", "netf", "stages_total", "stage_max"):
            assert st[k] == so[k], (i, k, st[k], so[k])
        assert np.array_equal(yi, J.y), (i, np.abs(yi - J.y).max())
        ref = C64.instance_state(y64, i)
        assert np.linalg.norm(yi - ref) <= 1e-5 * np.linalg.norm(ref), i


def test_batch_mixed_launch_shapes_agree_bitwise(ctx, stslib):
    inst = small_batch(stslib, count=12, seed=3)
    outs = []
    for threads, cps, cluster in ((256, 1, 1), (512, 2, 1), (256, 2, 2), (256, 4, 8)):
        B = stslib.Batch(ctx, inst)
        B.set_mixed(True)
        assert B.set_launch(threads, cps, cluster, big_n=32) == 0
        B.evolve(0.005, method=stslib.RKC, rtol=1e-6, atol=1e-10)
        outs.append(B.state())
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)


def test_batch_launch_shapes_agree_bitwise(ctx, stslib):
    """Launch shape and thread-block clusters (instances with n >= 32 split over 2, 4 or 8
    CTAs, exact reductions combined through distributed shared memory) change nothing."""
    inst = small_batch(stslib, count=12, seed=3)
    outs = []
    for threads, cps, cluster in ((256, 1, 1), (256, 2, 1), (512, 1, 1), (256, 2, 2), (512, 2, 4),
                                  (256, 4, 8), (256, 4, 16)):
        B = stslib.Batch(ctx, inst)
        assert B.set_launch(threads, cps, cluster, big_n=32) == 0
        try:
            B.evolve(0.005, method=stslib.RKC, rtol=1e-6, atol=1e-10)
        except stslib.STSError as e:
            # a 16-CTA cluster is a non-portable size: the library refuses it where the device
            # cannot schedule one
            assert cluster == 16 and "cannot be scheduled" in str(e)
            continue
        outs.append(B.state())
        assert B.launch() == (threads, cps, cluster, 32)
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)


def test_batch_clusters_match_oracle(ctx, stslib, oracle):
    inst = small_batch(stslib, count=10, seed=11)
    B = stslib.Batch(ctx, inst)
    assert B.set_launch(256, 2, 4, big_n=16) == 0  # every instance on a 4-CTA cluster
    B.evolve(0.01, method=stslib.RKL, rtol=1e-6, atol=1e-10)
    y = B.state()
    for i, (n, kx, ky, p, q, a) in enumerate(inst):
        P = oracle.Problem(oracle.UNFORCED, n, n, kx=kx, ky=ky)
        J = oracle.Integrator(P, P.initial_modes(p, q, a), method=oracle.RKL, rtol=1e-6, atol=1e-10,
                              tstop=0.01)
        assert J.evolve(0.01) == 1
        assert np.array_equal(B.instance_state(y, i), J.y), i
        assert B.stats(i)["nst"] == J.stats()["nst"]


def test_batch_autotune_keeps_results(ctx, stslib):
    inst = small_batch(stslib, count=10, seed=5)
    B = stslib.Batch(ctx, inst)
    th, cp, ms = B.autotune(0.001)
    assert th in (256, 512) and cp in (1, 2, 4) and ms > 0 and B.launch()[2] in (1, 4, 8, 16)
    B.evolve(0.005)
    C = stslib.Batch(ctx, inst)
    C.set_launch(th, cp)
    C.evolve(0.005)
    assert np.array_equal(B.state(), C.state())
