"""Checkpoint / restart of the LSRK integrator: a run that is written to disk at t1 and
restarted from the file in a fresh integrator must reach t2 with the same bits and the same
step statistics as the uninterrupted run."""
import numpy as np
import pytest

import ceda_demonstrations_gb300 as sts

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind=sts.MANUFACTURED, n=96, mixed=False, method=sts.RKL, power=None),
    dict(kind=sts.MANUFACTURED, n=96, mixed=True, method=sts.RKC, power=None),
    dict(kind=sts.MANUFACTURED, n=64, mixed=False, method=sts.RKC, power=(100, 0.01)),
    dict(kind=sts.PERIODIC, n=48, mixed=False, method=sts.RKL, power=None),  # generic path
    # the implicit Gustafsson controller reads the previous step size from the checkpoint
    dict(kind=sts.MANUFACTURED, n=64, mixed=False, method=sts.RKL, power=None, controller=sts.IMP_GUS),
]


def _integrator(ctx, P, case):
    return sts.LSRKStep(ctx, P, 0.0, P.initial(), method=case["method"], rtol=1e-6, atol=1e-10,
                        mixed=case["mixed"], power=case["power"], maxsteps=100000,
                        controller=case.get("controller", sts.PID))


@pytest.mark.parametrize("case", CASES, ids=["rkl_fp64", "rkc_mixed", "rkc_power", "periodic", "rkl_impgus"])
def test_restart_continues_bitwise(ctx, tmp_path, case):
    P = sts.Problem(ctx, case["kind"], case["n"], case["n"], 1.0, 0.5)
    t1, t2 = 0.003, 0.007
    ref = _integrator(ctx, P, case)
    y = P.vector()
    ref.evolve(t1, y)
    ck = tmp_path / "state.ckpt"
    ref.write_checkpoint(str(ck))
    ref.evolve(t2, y)
    ya, sa = y.numpy(), ref.stats()

    again = _integrator(ctx, P, case)
    again.read_checkpoint(str(ck))
    y2 = P.vector()
    again.evolve(t2, y2)
    yb, sb = y2.numpy(), again.stats()
    assert sa["nst"] >= 2 and sa["t"] == sb["t"] >= t2
    assert np.array_equal(ya, yb)
    for k in ("nst", "nst_attempts", "netf", "nfe", "nfe_dee", "ndee", "stages_total"):
        assert sa[k] == sb[k], k


def test_checkpoint_of_another_problem_is_rejected(ctx, tmp_path):
    case = CASES[0]
    P = sts.Problem(ctx, sts.MANUFACTURED, 64, 64, 1.0, 1.0)
    I = _integrator(ctx, P, case)
    y = P.vector()
    I.evolve(0.001, y)
    ck = tmp_path / "a.ckpt"
    I.write_checkpoint(str(ck))
    Q = sts.Problem(ctx, sts.MANUFACTURED, 80, 80, 1.0, 1.0)
    J = _integrator(ctx, Q, case)
    with pytest.raises(sts.STSError):
        J.read_checkpoint(str(ck))
    with pytest.raises(sts.STSError):
        J.read_checkpoint(str(tmp_path / "missing.ckpt"))
