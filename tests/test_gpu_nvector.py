"""Device N_Vector: the known-answer tests of gkeyll_diffusion/test_nvector_gkylzero.c
(tolerance 1e-10, 100 x 100 values, :4-363) and exact reductions against the oracle."""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kats():
    with open(os.path.join(GOLD, "reference_kats.json")) as f:
        return json.load(f)


def test_nvector_known_answers(ctx, stslib):
    k = kats()
    tol = k["tolerance"]
    n = k["shape"][0] * k["shape"][1]
    NV = stslib.NVector
    ramp = np.arange(n, dtype=np.float64)                        # :31-34
    x = NV.from_numpy(ctx, ramp)
    assert np.array_equal(x.numpy(), ramp)                       # N_VMake/GetVector :36-62
    cl = x.clone()                                               # :68-89
    assert len(cl) == n and cl.ptr != x.ptr
    ret = x.clone()
    ret.scale(k["scale"]["c"], x)                                # :95-116
    assert np.max(np.abs(ret.numpy() - 2.0 * ramp)) <= tol
    ret.const(k["const"]["c"])                                   # :122-139
    assert np.max(np.abs(ret.numpy() - 173.0)) <= tol
    ls = k["linear_sum"]
    v1, v2, out = NV(ctx, n), NV(ctx, n), NV(ctx, n)
    v1.const(ls["x"])
    v2.const(ls["y"])
    out.linear_sum(ls["a"], v1, ls["b"], v2)                     # :145-179
    assert np.max(np.abs(out.numpy() - ls["expect"])) <= tol
    v1.const(k["wrms"]["x"])
    v2.const(k["wrms"]["w"])
    assert abs(v1.wrms_norm(v2) - k["wrms"]["expect"]) <= tol    # :185-198
    v1.const(k["div"]["x"])
    v2.const(k["div"]["y"])
    out.div(v1, v2)                                              # :204-228
    assert np.max(np.abs(out.numpy() - k["div"]["expect"])) <= tol
    v1.const(k["abs"]["x"])
    out.abs(v1)                                                  # :234-257
    assert np.max(np.abs(out.numpy() - k["abs"]["expect"])) <= tol
    v1.const(k["inv"]["x"])
    out.inv(v1)                                                  # :263-286
    assert np.max(np.abs(out.numpy() - k["inv"]["expect"])) <= tol
    v1.const(0.0)
    m = v1.max_norm()                                            # :292-303
    assert 0.0 <= m < tol
    v1.const(k["addconst"]["x"])
    out.add_const(v1, k["addconst"]["b"])                        # :309-332
    assert np.max(np.abs(out.numpy() - k["addconst"]["expect"])) <= tol
    out.prod(v1, v2)
    assert np.max(np.abs(out.numpy() - k["inv"]["x"] * k["div"]["y"])) <= tol


@pytest.mark.parametrize("n", [1, 7, 1000, 262147, 4_000_037])
def test_exact_reductions_match_oracle(ctx, stslib, oracle, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n) * np.exp2(rng.integers(-40, 40, size=n))
    b = rng.standard_normal(n)
    w = np.abs(rng.standard_normal(n)) + 0.1
    A, B, W = (stslib.NVector.from_numpy(ctx, v) for v in (a, b, w))
    assert A.dot(B) == oracle.xdot(a, b)
    assert A.wrms_norm(W) == oracle.wrms(a, w)
    assert A.max_norm() == np.max(np.abs(a))


def test_reductions_nan_and_zero(ctx, stslib):
    z = stslib.NVector(ctx, 100)
    assert z.dot(z) == 0.0 and z.max_norm() == 0.0
    a = np.ones(100)
    a[37] = np.nan
    A = stslib.NVector.from_numpy(ctx, a)
    assert math.isnan(A.dot(A)) and math.isnan(A.max_norm())
    one = stslib.NVector.from_numpy(ctx, np.ones(100))
    assert one.dot(one) == 100.0


def test_linear_combination(ctx, stslib):
    rng = np.random.default_rng(9)
    n = 50_001
    xs = [rng.standard_normal(n) for _ in range(11)]
    cs = list(rng.standard_normal(11))
    X = [stslib.NVector.from_numpy(ctx, v) for v in xs]
    z = stslib.NVector(ctx, n)
    z.linear_combination(cs, X)
    want = sum(c * v for c, v in zip(cs, xs))
    assert np.max(np.abs(z.numpy() - want)) <= 1e-13 * np.max(np.abs(want))


def test_make_wraps_without_copy(ctx, stslib):
    L = stslib.lib()
    x = stslib.NVector.from_numpy(ctx, np.arange(10.0))
    w = stslib.NVector(ctx, handle=L.N_VMake_Sts(10, x.ptr, ctx.h), own=True)
    assert w.ptr == x.ptr
    w.scale(3.0, w)
    assert np.array_equal(x.numpy(), 3.0 * np.arange(10.0))
    w.destroy()  # does not free x's memory
    assert np.array_equal(x.numpy(), 3.0 * np.arange(10.0))
