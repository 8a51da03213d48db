"""Generate the end-to-end fixtures of the two FP64 benchmark configurations (CPU only).

config1_oracle.npz  128 x 128 interior nodes, kx = ky = 1, RKC adaptive (rtol 1e-6,
                    atol 1e-10), manufactured problem, t in [0, 1]: the serial CPU case.
config2_oracle.npz  4096 x 4096 interior nodes, kx = ky = 1, RKL2 adaptive (rtol 1e-6,
                    atol 1e-10), manufactured problem, t in [0, 0.1]: the FP64 GPU case
                    (about 2.3e12 DOF-stages; two hours on 8 x86 cores, so it is run once and
                    its result kept here).

Each file holds the oracle's step statistics, the SHA-256 of the final field's bytes, its
relative L2 error against the manufactured solution (the error metric of
diffusion_2D/main.cpp:461-465 with the exact solution as reference), its L2 norm, and a
64 x 64 subsample of the field (every (n/64)-th node in each direction). The GPU tests
compare the FP64 GPU path with these: the same step sequence, and the same bits (hash) or,
where the host's libm rounds a table entry differently (x86 here, Arm beside the GPU),
1e-12 relative agreement of the subsample and the norms.

Usage (from the repository root):  python tests/golden/make_config_goldens.py [1] [2]
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import pyoracle as po  # noqa: E402

CONFIGS = {
    1: dict(n=128, kx=1.0, ky=1.0, method=po.RKC, rtol=1e-6, atol=1e-10, tf=1.0),
    2: dict(n=4096, kx=1.0, ky=1.0, method=po.RKL, rtol=1e-6, atol=1e-10, tf=0.1),
}
SAMPLE = 64


def field_summary(y, n, ex):
    Y = y.reshape(n, n)
    step = n // SAMPLE
    return dict(
        sha256=hashlib.sha256(np.ascontiguousarray(y, dtype="<f8").tobytes()).hexdigest(),
        rel_l2_vs_exact=float(np.linalg.norm(y - ex) / np.linalg.norm(ex)),
        l2=float(np.linalg.norm(y)),
        sample=np.ascontiguousarray(Y[step // 2::step, step // 2::step][:SAMPLE, :SAMPLE]),
    )


def run(k):
    c = CONFIGS[k]
    n = c["n"]
    P = po.Problem(po.MANUFACTURED, n, n, kx=c["kx"], ky=c["ky"])
    J = po.Integrator(P, P.initial(), method=c["method"], rtol=c["rtol"], atol=c["atol"],
                      maxsteps=10 ** 7)
    J.set_stop_time(c["tf"])  # diffusion_2D/main.cpp:384
    t0 = time.time()
    rc = J.evolve(c["tf"])
    secs = time.time() - t0
    assert rc == 1, rc  # ARK_TSTOP_RETURN
    st = J.stats()
    summ = field_summary(J.y, n, P.exact(c["tf"]))
    out = os.path.join(HERE, "config%d_oracle.npz" % k)
    np.savez_compressed(out, n=n, kx=c["kx"], ky=c["ky"], method=c["method"], rtol=c["rtol"],
                        atol=c["atol"], tf=c["tf"], t=st["t"],
                        **{key: st[key] for key in ("nst", "nst_attempts", "netf", "nfe",
                                                     "stage_max", "stages_total")},
                        sha256=summ["sha256"], rel_l2_vs_exact=summ["rel_l2_vs_exact"],
                        l2=summ["l2"], sample=summ["sample"], oracle_seconds=secs,
                        oracle_threads=po.lib().orc_nthreads())
    print("config %d: %s nst=%d nfe=%d err=%.6e %.0f s" % (k, out, st["nst"], st["nfe"],
                                                            summ["rel_l2_vs_exact"], secs), flush=True)


if __name__ == "__main__":
    for k in [int(a) for a in sys.argv[1:]] or [1, 2]:
        run(k)
