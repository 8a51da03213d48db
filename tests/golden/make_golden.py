"""Generate the golden fixtures under tests/golden/ (run from the repo root).

reference_kats.json  Known-answer values from the reference's own tests, transcribed as
                     data with their file:line (gkeyll_diffusion/test_nvector_gkylzero.c,
                     gkeyll_diffusion/analytic_CR_test.c + src/input_handler.c defaults).
oracle_*.npz         Outputs of the CPU oracle on small cases, used to pin the oracle across
                     machines (compared with a tolerance: libm may differ by an ulp between
                     x86 and Arm) and as GPU parity fixtures.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import pyoracle as po  # noqa: E402

KATS = {
    "source": "gkeyll_diffusion/test_nvector_gkylzero.c",
    "tolerance": 1e-10,                       # :9 eq_check_tol
    "shape": [100, 100],                      # :7-8 num_basis x size
    "init_ramp": "x_i = i",                   # :31-34
    "scale": {"c": 2.0},                      # :97  N_VScale(2.0, x) = 2 x
    "const": {"c": 173.0},                    # :122
    "linear_sum": {"a": 2.0, "b": 3.0, "x": 1.75, "y": 2.89,
                   "expect": 2.0 * 1.75 + 3.0 * 2.89},          # :145-171
    "wrms": {"x": -0.5, "w": 0.5, "expect": 0.25},              # :185-191
    "div": {"x": 1.75, "y": 2.89, "expect": 1.75 / 2.89},        # :208-220
    "abs": {"x": -1.0, "expect": 1.0},                          # :238-249
    "inv": {"x": 1.75, "expect": 1.0 / 1.75},                   # :267-278
    "maxnorm": {"x": 0.0, "expect": 0.0},                       # :292-296
    "addconst": {"x": 1.75, "b": 2.89, "expect": 1.75 + 2.89},  # :313-324
    "analytic_CR": {
        "source": "gkeyll_diffusion/analytic_CR_test.c",
        "lambda": -10.0,              # :505
        "rhs": "y' = lambda (y - atan t) + 1/(1+t^2)",  # :168-185
        "exact": "atan(t)",           # :188-199
        "y0": 0.0,                    # :539 true_sol(0)
        "tf": 1.0,                    # input_handler.c:34 (ctx.t_end = udata->tf, :470)
        "nout": 10,                   # input_handler.c:56
        "rtol": 1e-5, "atol": 1e-12,  # input_handler.c:37-38
        "method": "RKL2",             # input_handler.c:45
        "stage_max_limit": 200,       # input_handler.c:47
        "eigsafety": 1.1,             # input_handler.c:49
        "eigfrequency": 0,            # input_handler.c:46 (computed once)
    },
}


def main():
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(KATS, f, indent=1, sort_keys=True)
    cases = [
        ("oracle_rkc_17x9", dict(kind=po.MANUFACTURED, nx=17, ny=9), dict(method=po.RKC), 0.1),
        ("oracle_rkl_32", dict(kind=po.MANUFACTURED, nx=32, ny=32, ky=0.01), dict(method=po.RKL), 0.05),
        ("oracle_rkl_mixed_32", dict(kind=po.MANUFACTURED, nx=32, ny=32, ky=0.01),
         dict(method=po.RKL, mixed=True), 0.05),
    ]
    for name, pk, ok, tf in cases:
        P = po.Problem(**pk)
        I = po.Integrator(P, P.initial(), **ok)
        I.set_stop_time(tf)  # diffusion_2D/main.cpp:384
        rc = I.evolve(tf)
        assert rc == 1  # ARK_TSTOP_RETURN
        st = I.stats()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), y=I.y, tf=tf,
                            **{k: np.array(v) for k, v in st.items()},
                            problem=json.dumps(pk), opts=json.dumps(ok))
        print(name, st)


if __name__ == "__main__":
    main()
