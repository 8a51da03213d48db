"""Debug-bounds build (-DSTS_DEBUG_BOUNDS) in place of a sanitizer on the GPU.

The library is rebuilt with index-range checks in the stage, step-end, TMA-stage, fused-stage
and batched kernels (a violation writes the context's error word and skips the access; nothing traps),
and the bitwise parity tests of those kernels run against it in a child process: a check that
fired would fail its step, and the results must still equal the oracle's bit for bit."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SUBSET = ("fused_fp64_bitwise or mixed_bitwise or tma_stage_kernel_matches or controllers_bitwise"
          " or fused_stage_groups"
          " or batch_matches_oracle_per_instance or batch_launch_shapes or batch_clusters")


def test_parity_suite_under_the_debug_bounds_build(stslib):
    from ceda_demonstrations_gb300 import build as b
    path = b.build(variant="bounds")
    assert os.path.exists(path) and os.sep + "bounds" + os.sep in path
    env = dict(os.environ, STS_LIBRARY_VARIANT="bounds")
    r = subprocess.run([sys.executable, "-c",
                        "import ceda_demonstrations_gb300 as s; print(s.lib()._name)"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and os.sep + "bounds" + os.sep in r.stdout, r.stdout + r.stderr
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        "tests/test_gpu_lsrk.py", "tests/test_gpu_batch.py", "-k", SUBSET],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert " passed" in r.stdout and "failed" not in r.stdout
