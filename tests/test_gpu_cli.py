"""The command-line driver: reference flags (diffusion_2D/main.cpp:556-687,
diffusion_2D.cpp:42-163) and the stdout labels diffusion_2D/runtests-diffusion2d.py:36-54
parses, run on the GPU."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "ceda_demonstrations_gb300", "_build", "diffusion_2D_gpu")


def parse_like_runtests(stdout):
    """The parsing rules of runtests-diffusion2d.py:36-54, restated."""
    stats = {"Steps": None, "Fails": None, "Accuracy": None, "FEvals": 0, "Runtime": None}
    for line in stdout.split("\n"):
        txt = line.split()
        if "Steps" in txt:
            stats["Steps"] = int(txt[2])
        elif ("Error" in txt) and ("test" in txt):
            stats["Fails"] = int(txt[4])
        elif ("Maximum" in txt) and ("relative" in txt):
            stats["Accuracy"] = float(txt[4])
        elif ("Explicit" in txt) and ("RHS" in txt):
            stats["FEvals"] += int(txt[5])
        elif ("Implicit" in txt) and ("RHS" in txt):
            stats["FEvals"] += int(txt[5])
        elif ("LS" in txt) and ("RHS" in txt):
            stats["FEvals"] += int(txt[5])
        elif ("RHS" in txt) and ("fn" in txt):
            stats["FEvals"] += int(txt[4])
        elif "simulation" in txt:
            stats["Runtime"] = float(txt[4])
    return stats


def run(args, cwd=None):
    r = subprocess.run([EXE] + args, capture_output=True, text=True, cwd=cwd, timeout=600)
    return r.returncode, r.stdout, r.stderr


@pytest.mark.parametrize("controller", [2, 5])
def test_cli_manufactured_rkc_with_error_mode(stslib, oracle, controller):
    stslib.lib()
    rc, out, err = run(["--problem", "manufactured", "--nx", "64", "--ny", "48", "--integrator", "rkc",
                        "--rtol", "1e-6", "--atol", "1e-10", "--tf", "0.05", "--nout", "5", "--error",
                        "--controller", str(controller), "--maxsteps", "10000"])
    assert rc == 0, err
    st = parse_like_runtests(out)
    assert st["Steps"] > 0 and st["Fails"] >= 0 and st["FEvals"] > 0 and st["Runtime"] > 0
    assert 0 < st["Accuracy"] < 1e-3
    # the same run on the oracle (same outputs times, same controller)
    P = oracle.Problem(oracle.MANUFACTURED, 64, 48)
    J = oracle.Integrator(P, P.initial(), method=oracle.RKC, rtol=1e-6, atol=1e-10,
                          controller=controller)
    # output times accumulate like the reference program's (main.cpp: tout += dTout, capped at
    # tf); with --error every output time is a stop time (main.cpp:437-441)
    dt, tout = 0.05 / 5, 0.05 / 5
    for k in range(5):
        J.set_stop_time(tout)
        assert J.evolve(tout) == 1
        tout = min(tout + dt, 0.05)
    assert st["Steps"] == J.stats()["nst"]
    ex = P.exact(0.05)
    rel = np.linalg.norm(J.y - ex) / np.linalg.norm(ex)
    line = [l for l in out.split("\n") if l.startswith("Relative L2 error vs exact")][0]
    assert abs(float(line.split("=")[1]) - rel) <= 1e-12 * rel


def test_cli_outputs_without_error_mode_follow_the_dense_output(stslib, oracle):
    """The reference program's default run (no --error): the stop time is the final time
    (main.cpp:384) and the intermediate outputs come from the dense output, so the steps pass
    them; the step count and the final field equal the oracle's run under the same rules."""
    stslib.lib()
    rc, out, err = run(["--problem", "manufactured", "--nx", "64", "--ny", "48", "--integrator", "rkc",
                        "--rtol", "1e-6", "--atol", "1e-10", "--tf", "0.05", "--nout", "5", "--maxsteps", "10000"])
    assert rc == 0, err
    st = parse_like_runtests(out)
    P = oracle.Problem(oracle.MANUFACTURED, 64, 48)
    J = oracle.Integrator(P, P.initial(), method=oracle.RKC, rtol=1e-6, atol=1e-10, tstop=0.05)
    dt, tout = 0.05 / 5, 0.05 / 5
    for k in range(5):
        assert J.evolve(tout) == (1 if k == 4 else 0)
        tout = min(tout + dt, 0.05)
    assert st["Steps"] == J.stats()["nst"]
    ex = P.exact(0.05)
    rel = np.linalg.norm(J.y - ex) / np.linalg.norm(ex)
    line = [l for l in out.split("\n") if l.startswith("Relative L2 error vs exact")][0]
    assert abs(float(line.split("=")[1]) - rel) <= 1e-12 * rel


def test_cli_reference_mode_and_solution_file(stslib, tmp_path):
    stslib.lib()
    rc, out, err = run(["--nx", "40", "--ny", "32", "--integrator", "rkl", "--inhomogeneous",
                        "--internaleig", "--tf", "0.2", "--nout", "4", "--output", "2"], cwd=str(tmp_path))
    assert rc == 0, err
    st = parse_like_runtests(out)
    assert st["Steps"] > 0 and st["FEvals"] > 0
    f = tmp_path / "diffusion_2d_solution.00000.txt"
    lines = f.read_text().strip().split("\n")
    header = [l for l in lines if l.startswith("#")]
    rows = [l for l in lines if not l.startswith("#")]
    assert header[0] == "# title Diffusion 2D" and "# nx  40" in header
    assert len(rows) == 5 and all(len(r.split()) == 1 + 40 * 32 for r in rows)
    assert np.isfinite(np.array(rows[-1].split(), dtype=float)).all()


def test_cli_dirk_and_errors(stslib):
    stslib.lib()
    rc, out, err = run(["--problem", "manufactured", "--nx", "32", "--ny", "32", "--integrator", "dirk",
                        "--fixedstep", "1e-3", "--tf", "0.01", "--nout", "2"])
    assert rc == 0, err
    assert parse_like_runtests(out)["Steps"] == 10
    rc, out, err = run(["--bogus"])
    assert rc == 1 and "Unknown inputs" in err
    rc, out, err = run(["--integrator", "foo"])
    assert rc == 1 and "illegal integrator" in err
    rc, out, err = run(["--integrator", "erk", "--order", "5"])
    assert rc == 1 and "order" in err
    rc, out, err = run(["--integrator", "dirk", "--order", "4"])
    assert rc == 1 and "order" in err
    rc, out, err = run(["--controller", "6"])
    assert rc == 1 and "controller" in err


def test_cli_checkpoint_restart_matches_uninterrupted_run(stslib, tmp_path):
    stslib.lib()
    # --error makes every output time a stop time (main.cpp:437-441), so the uninterrupted run
    # ends a step on the checkpoint's time as the first half did
    common = ["--problem", "manufactured", "--nx", "64", "--ny", "64", "--integrator", "rkl",
              "--rtol", "1e-6", "--maxsteps", "10000", "--error"]
    ck = str(tmp_path / "half.ckpt")
    rc, out1, err = run(common + ["--tf", "0.005", "--nout", "1", "--checkpoint", ck])
    assert rc == 0, err
    rc, out2, err = run(common + ["--tf", "0.01", "--nout", "2", "--restart", ck])
    assert rc == 0, err
    rc, full, err = run(common + ["--tf", "0.01", "--nout", "2"])
    assert rc == 0, err

    def last_rms(out):
        rows = [l.split() for l in out.split("\n") if len(l.split()) == 2]
        return rows[-1]

    def l2(out):
        return [l for l in out.split("\n") if l.startswith("Relative L2 error vs exact")][0]

    assert last_rms(out2) == last_rms(full)
    assert l2(out2) == l2(full)
    assert parse_like_runtests(out2)["Steps"] == parse_like_runtests(full)["Steps"]


# the solver rows of runtests-diffusion2d.py:59-67,95-103 (the hypre rows run the PFMG-role
# multigrid in hypre's place, with the harness's --pfmg_relax 3 and the --pfmg_nrelax of its
# one-process grid, :23-24,89; the harness builds them as diffusion_2D_mpi_hypre)
HARNESS_ROWS = {
    "dirk2-Jacobi": ["--integrator", "dirk", "--order", "2"],
    "dirk2-hypre": ["--integrator", "dirk", "--order", "2", "--pfmg_relax", "3", "--pfmg_nrelax", "3"],
    "dirk3-Jacobi": ["--integrator", "dirk", "--order", "3"],
    "dirk3-hypre": ["--integrator", "dirk", "--order", "3", "--pfmg_relax", "3", "--pfmg_nrelax", "3"],
    "erk2": ["--integrator", "erk", "--order", "-2"],
    "erk3": ["--integrator", "erk", "--order", "-3"],
    "erk4": ["--integrator", "erk", "--order", "-4"],
    "rkc": ["--integrator", "rkc"],
    "rkl": ["--integrator", "rkl"],
}
# the common flags of runtests-diffusion2d.py:76-83
COMMON = ["--inhomogeneous", "--atol", "1.e-11", "--controller", "2", "--error", "--nonlinear", "--msbp", "1",
          "--maxsteps", "100000", "--internaleig"]


@pytest.mark.parametrize("kx", [0.1, 1.0, 10.0])
def test_cli_runs_the_reference_harness_rows(stslib, kx):
    """Every solver row of the reference's experiment harness with its common flags, on one
    process at the harness's smallest grid (32^2), kx in {0.1, 1, 10}, ky = 0, rtol 1e-4,
    parsed the harness's way (a shorter final time keeps the --error self-oracle short)."""
    stslib.lib()
    for name, row in HARNESS_ROWS.items():
        args = row + ["--nx", "32", "--ny", "32", "--rtol", "%e" % 1e-4, "--kx", "%e" % kx, "--ky", "%e" % 0.0,
                      "--tf", "0.2"] + COMMON
        rc, out, err = run(args)
        assert rc == 0, (name, err)
        st = parse_like_runtests(out)
        assert st["Steps"] > 0 and st["Fails"] is not None and st["FEvals"] > st["Steps"], (name, st)
        assert st["Accuracy"] is not None and st["Accuracy"] < 5e-3, (name, st)
        assert st["Runtime"] is not None and st["Runtime"] >= 0.0
        if "hypre" in name:
            assert "Total PFMG iterations" in out
