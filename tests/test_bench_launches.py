"""The bench's kernel count per step attempt on the mixed path against the integrator's stage
schedule (record_step in ceda_demonstrations_gb300/csrc/lsrk.cu): stage 1, then stages 2..s
in groups of ks (a shorter last group; a last group of one stage is a single-stage launch),
then the step end."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def schedule(s, ks):
    launches, j = 2, 2  # stage 1 and the step end
    while j <= s:
        g = min(ks, s - j + 1)
        launches += 1
        j += g if g >= 2 else 1
    return launches


@pytest.mark.parametrize("ks", [1, 2, 3, 4])
def test_step_launches_follow_the_stage_schedule(ks):
    for s in range(2, 201):
        want = s + 1 if ks == 1 else schedule(s, ks)
        assert bench.step_launches(s, ks) == want, (s, ks)
    assert bench.step_launches(196, 4) == 51  # the 8192^2 workload's steps
