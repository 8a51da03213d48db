"""SSP methods of LSRKStepCreateSSP (diffusion_2D/main.cpp:250-294): SSP(s,2), SSP(n^2,3),
SSP(10,4) through the integrator's N_Vector path, against the oracle's restatement bit for bit
on the manufactured heat problem, and their orders of convergence on the known-answer problem
of gkeyll_diffusion/analytic_CR_test.c with fixed steps."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

METHODS = [(2, 2), (2, 10), (3, 4), (3, 9), (4, 10)]


@pytest.mark.parametrize("ssp", METHODS, ids=["ssp2_2", "ssp2_10", "ssp3_4", "ssp3_9", "ssp10_4"])
def test_ssp_matches_oracle_bitwise(ctx, stslib, oracle, ssp):
    pk = dict(kind=0, nx=24, ny=16, kx=1.0, ky=0.5)
    G = stslib.Problem(ctx, **pk)
    O = oracle.Problem(**pk)
    I = stslib.LSRKStep(ctx, G, 0.0, G.initial(), rtol=1e-5, atol=1e-9, ssp=ssp)
    J = oracle.Integrator(O, O.initial(), rtol=1e-5, atol=1e-9, ssp=ssp)
    y = G.vector()
    for tout in (0.002, 0.005):
        I.evolve(tout, y)
        assert J.evolve(tout) == 0
        assert np.array_equal(y.numpy(), J.y)
    si, sj = I.stats(), J.stats()
    for k in ("nst", "nst_attempts", "netf", "nfe", "stages_total"):
        assert si[k] == sj[k], k
    assert si["stage_max"] == ssp[1] and si["nst"] >= 3


@pytest.mark.parametrize("ssp,order", [((2, 5), 2), ((3, 9), 3), ((4, 10), 4)])
def test_ssp_fixed_step_order(ctx, stslib, ssp, order):
    lam = -1.0
    L = stslib.lib()

    def f(t, y, ydot):
        L.N_VScale_Sts(lam, y.h, ydot.h)
        L.N_VAddConst_Sts(ydot.h, 1.0 / (1.0 + t * t) - lam * math.atan(t), ydot.h)
        return 0

    errs = []
    for h in (0.1, 0.05):
        y0 = stslib.NVector.from_numpy(ctx, np.array([0.0]))
        I = stslib.LSRKStep(ctx, f, 0.0, y0, hfixed=h, ssp=ssp)
        I.set_stop_time(2.0)
        y = stslib.NVector(ctx, 1)
        I.evolve(2.0, y)
        errs.append(abs(y.numpy()[0] - math.atan(2.0)))
    rate = math.log2(errs[0] / errs[1])
    assert abs(rate - order) < 0.3, (errs, rate)


def test_ssp_rejects_invalid_stage_counts(ctx, stslib):
    G = stslib.Problem(ctx, 0, 16, 16)
    with pytest.raises(stslib.STSError):
        stslib.LSRKStep(ctx, G, 0.0, G.initial(), ssp=(3, 10))  # not a square
    with pytest.raises(stslib.STSError):
        stslib.LSRKStep(ctx, G, 0.0, G.initial(), ssp=(4, 9))
