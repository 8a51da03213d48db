"""CPU tests: the oracle against the reference's known answers and analytic facts, and the
product's host-side rules (stage coefficients, stage counts, controllers, tables, exact sum)
against the oracle bit for bit. No GPU is used here."""
import json
import math
import os
from fractions import Fraction

import numpy as np


def mpmath_pow(x, y):
    """x**y to double precision through exact rational arithmetic on a 60-digit decimal
    expansion (python's decimal module), independent of the C library."""
    import decimal
    with decimal.localcontext() as c:
        c.prec = 60
        return float((decimal.Decimal(x).ln() * decimal.Decimal(y)).exp())
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kats():
    with open(os.path.join(GOLD, "reference_kats.json")) as f:
        return json.load(f)


# ---------------------------------------------------------------- exact reductions
def exact_round(xs):
    return float(sum((Fraction(float(x)) for x in xs), Fraction(0)))


def test_xsum_is_exact_and_order_independent(oracle):
    rng = np.random.default_rng(1)
    for trial in range(20):
        n = int(rng.integers(1, 3000))
        e = rng.integers(-60, 40, size=n)
        x = rng.standard_normal(n) * np.exp2(e)
        want = exact_round(x)
        assert oracle.xsum(x) == want
        assert oracle.xsum(x[::-1]) == want
        assert oracle.xsum(rng.permutation(x)) == want


def test_xsum_edges(oracle):
    assert oracle.xsum(np.zeros(0)) == 0.0
    assert oracle.xsum(np.array([1e18, 1.0, -1e18])) == 1.0
    assert oracle.xsum(np.array([2.0 ** -170])) == 0.0  # below the 2^-160 grid
    assert math.isnan(oracle.xsum(np.array([1.0, np.nan])))
    assert math.isinf(oracle.xsum(np.array([1.0, np.inf])))
    assert oracle.xsum(np.array([2.0 ** 70])) == 2.0 ** 70
    assert math.isinf(oracle.xsum(np.array([2.0 ** 130])))


def test_product_host_exact_sum_matches_oracle(oracle, stslib):
    L = stslib.lib()
    rng = np.random.default_rng(2)
    for trial in range(20):
        n = int(rng.integers(1, 2000))
        x = rng.standard_normal(n) * np.exp2(rng.integers(-150, 125, size=n))
        x[np.abs(x) > 2.0 ** 127] = 1.0
        got = L.STS_ExactSumHost(x.ctypes.data_as(stslib._dp), n)
        assert got == oracle.xsum(x)
    for special in ([np.nan, 1.0], [np.inf], [2.0 ** 128], [2.0 ** 100, -1.0], []):
        a = np.array(special, dtype=np.float64)
        g = L.STS_ExactSumHost(a.ctypes.data_as(stslib._dp), a.size)
        o = oracle.xsum(a)
        assert (math.isnan(g) and math.isnan(o)) or g == o


def test_nvector_reduction_kats(oracle):
    """WRMS and max-norm known answers of test_nvector_gkylzero.c:185-198, 292-303."""
    k = kats()
    n = k["shape"][0] * k["shape"][1]
    x = np.full(n, k["wrms"]["x"])
    w = np.full(n, k["wrms"]["w"])
    assert abs(oracle.wrms(x, w) - k["wrms"]["expect"]) <= k["tolerance"]
    assert oracle.maxnorm(np.zeros(n)) == k["maxnorm"]["expect"]
    r = np.arange(n, dtype=np.float64)
    assert oracle.xdot(r, r) == exact_round(r * r)


# ---------------------------------------------------------------- method coefficients
def stability_function(c, z):
    mu, nu, mus, ajm1, _ = c
    s = len(mu) - 1
    y0, f0 = 1.0, z
    ym2, ym1 = y0, y0 + mus[1] * f0
    for j in range(2, s + 1):
        yj = mu[j] * ym1 + nu[j] * ym2 + (1 - mu[j] - nu[j]) * y0 + mus[j] * (z * ym1) - mus[j] * ajm1[j] * f0
        ym2, ym1 = ym1, yj
    return ym1


@pytest.mark.parametrize("method", [0, 1])
def test_stage_coefficients_second_order_and_stable(oracle, method):
    for s in (2, 3, 5, 10, 40, 120, 200):
        c = oracle.stage_coeffs(method, s)
        for z in (-1e-2, -2e-2):
            R = stability_function(c, z)
            assert abs(R - (1 + z + z * z / 2)) < 0.3 * abs(z) ** 3 + 1e-15
        if method == 0:  # RKC stability boundary (1 + w0)/w1
            w0 = 1 + 2 / (13 * s * s)
            w1 = c[2][1] * (2 * w0) ** 2
            beta = (1 + w0) / w1
        else:
            beta = (s * s + s - 2) / 2.0
        for z in np.linspace(-beta * 0.999, 0.0, 401):
            assert abs(stability_function(c, z)) <= 1.0 + 1e-9


@pytest.mark.parametrize("method", [0, 1])
def test_product_coefficients_equal_oracle(oracle, stslib, method):
    L = stslib.lib()
    for s in range(2, 201):
        o = oracle.stage_coeffs(method, s)
        g = [np.zeros(s + 1) for _ in range(5)]
        assert L.STS_LSRKStageCoeffs(method, s, *[a.ctypes.data_as(stslib._dp) for a in g]) == 0
        for a, b in zip(o, g):
            assert np.array_equal(a[1:], b[1:])


def test_product_step_rules_equal_oracle(oracle, stslib):
    import ctypes as C
    L = stslib.lib()
    rng = np.random.default_rng(3)
    for _ in range(500):
        method = int(rng.integers(0, 2))
        h = float(10 ** rng.uniform(-8, -1))
        rho = float(10 ** rng.uniform(2, 9))
        smax = int(rng.integers(2, 400))
        hm = C.c_double()
        s = L.STS_LSRKStagesNeeded(method, h, rho, smax, C.byref(hm))
        so, hmo = oracle.stages_needed(method, h, rho, smax)
        assert s == so and hm.value == hmo
        ctrl = int(rng.integers(0, 6))
        dsm, ep1, ep2 = (float(10 ** rng.uniform(-4, 1)) for _ in range(3))
        hp = h * float(10 ** rng.uniform(-1, 1))
        nh = int(rng.integers(0, 4))
        assert L.STS_AdaptControllerEstimate(ctrl, h, dsm, ep1, ep2, hp, nh) == \
            oracle.controller(ctrl, h, dsm, ep1, ep2, hp, nh)
    # a non-finite step (from a NaN state) takes the 2-stage minimum on both sides, the
    # semantics of max(ss, 2) with an unordered comparison, not an undefined integer conversion
    for method in (0, 1):
        for h in (float("nan"), float("-inf")):
            s = L.STS_LSRKStagesNeeded(method, h, 1e4, 200, C.byref(hm))
            assert s == 2 and oracle.stages_needed(method, h, 1e4, 200)[0] == 2


def test_gustafsson_controllers(oracle):
    """ExpGus / ImpGus / ImExGus (diffusion_2D/main.cpp:366-376): the published formulas,
    evaluated here with numpy's pow, agree with the oracle to a few ulp; the first step is the
    I controller; ImExGus is the smaller of the two."""
    rng = np.random.default_rng(11)
    p = 3.0
    for _ in range(300):
        h = float(10 ** rng.uniform(-8, -1))
        hp = h * float(10 ** rng.uniform(-1, 1))
        dsm, ep1 = (float(10 ** rng.uniform(-4, 1)) for _ in range(2))
        e1, e2 = max(1.5 * dsm, 1e-10), max(1.5 * ep1, 1e-10)
        exp_ = h * e1 ** (-0.367 / p) * (e1 / e2) ** (-0.268 / p)
        imp_ = h * (h / hp) * e1 ** (-0.98 / p) * (e1 / e2) ** (-0.95 / p)
        for ctrl, want in ((3, exp_), (4, imp_), (5, min(exp_, imp_))):
            got = oracle.controller(ctrl, h, dsm, ep1, 0.5, hp, 1)
            assert abs(got - want) <= 1e-13 * want
            first = oracle.controller(ctrl, h, dsm, ep1, 0.5, hp, 0)
            assert abs(first - h * e1 ** (-1 / p)) <= 1e-13 * first


def test_product_tables_equal_oracle(oracle, stslib):
    L = stslib.lib()
    for nx, ny in ((17, 9), (128, 128), (1000, 3)):
        P = oracle.Problem(oracle.MANUFACTURED, nx, ny)
        Sx, Sxx, Sy, Syy = P.tables()
        for n, S0, D0 in ((nx, Sx, Sxx), (ny, Sy, Syy)):
            S = np.zeros(n)
            D = np.zeros(n)
            L.STS_ManufacturedTables(n, 1.0 / (n + 1), S.ctypes.data_as(stslib._dp),
                                     D.ctypes.data_as(stslib._dp))
            assert np.array_equal(S, S0) and np.array_equal(D, D0)


# ---------------------------------------------------------------- oracle physics
def test_kernel_form_rhs_matches_reference_form(oracle):
    for kx, ky in ((1.0, 1.0), (1.0, 0.01)):
        P = oracle.Problem(oracle.MANUFACTURED, 33, 17, kx=kx, ky=ky)
        rng = np.random.default_rng(4)
        u = rng.standard_normal(P.n)
        for t in (0.0, 0.13):
            a = P.rhs(t, u)
            b = P.rhs(t, u, ref=True)
            assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))


def test_manufactured_rhs_is_consistent(oracle):
    """F(t, u_exact) -> u_exact_t as the grid is refined (second order)."""
    errs = []
    for n in (32, 64, 128):
        P = oracle.Problem(oracle.MANUFACTURED, n)
        t = 0.1
        f = P.rhs(t, P.exact(t))
        Sx, _, Sy, _ = P.tables()
        ut = np.outer(Sy, Sx).ravel() * oracle.lib().orc_cdot(t)
        errs.append(np.max(np.abs(f - ut)))
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5


def test_spatial_convergence_second_order(oracle):
    """Discretisation error of the full STS run decreases as O(dx^2)."""
    errs = []
    for n in (16, 32, 64):
        P = oracle.Problem(oracle.MANUFACTURED, n)
        I = oracle.Integrator(P, P.initial(), method=oracle.RKC, rtol=1e-9, atol=1e-12)
        I.set_stop_time(0.25)
        assert I.evolve(0.25) == 1
        ex = P.exact(0.25)
        errs.append(np.linalg.norm(I.y - ex) / np.linalg.norm(ex))
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5


def test_power_iteration_closed_form_spectral_radius(oracle):
    nx, ny, kx, ky = 16, 12, 1.0, 0.3
    P = oracle.Problem(oracle.MANUFACTURED, nx, ny, kx=kx, ky=ky)
    dx, dy = 1.0 / (nx + 1), 1.0 / (ny + 1)
    rho = 4 * kx / dx ** 2 * math.sin(nx * math.pi / (2 * (nx + 1))) ** 2 + \
        4 * ky / dy ** 2 * math.sin(ny * math.pi / (2 * (ny + 1))) ** 2
    v0 = np.random.default_rng(6).standard_normal(P.n)
    lam, it, _ = P.power_iteration(v0, maxiters=5000, reltol=1e-12)
    assert abs(-lam - rho) / rho < 1e-4
    assert -P.dom_eig() >= rho  # main.cpp:544 is an upper bound


def test_pcg_solves_shifted_operator(oracle):
    P = oracle.Problem(oracle.MANUFACTURED, 64, 48, kx=1.0, ky=0.05)
    gamma = 1e-3
    rng = np.random.default_rng(5)
    xs = rng.standard_normal(P.n)
    b = xs - gamma * P.apply_A(xs)
    for jac in (True, False):
        x, it, rel = P.pcg(gamma, b, tol=1e-10, jacobi=jac)
        assert rel <= 1e-10
        assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-7
        assert 1 <= it < 2000


def test_sdirk2_second_order_in_time(oracle):
    P = oracle.Problem(oracle.MANUFACTURED, 24)
    y0 = P.initial()
    ref, _ = P.sdirk2(y0, 0.0, 0.2 / 256, 256, tol=1e-13)
    e = []
    for m in (8, 16):
        y, _ = P.sdirk2(y0, 0.0, 0.2 / m, m, tol=1e-13)
        e.append(np.linalg.norm(y - ref))
    assert 3.0 < e[0] / e[1] < 5.0


def test_mixed_matches_fp64_for_equal_steps(oracle):
    P = oracle.Problem(oracle.MANUFACTURED, 96, kx=1.0, ky=0.01)
    out = {}
    for mixed in (False, True):
        I = oracle.Integrator(P, P.initial(), method=oracle.RKL, mixed=mixed, hfixed=2e-3)
        I.set_stop_time(0.05)
        assert I.evolve(0.05) == 1
        out[mixed] = I.y
    rel = np.linalg.norm(out[True] - out[False]) / np.linalg.norm(out[False])
    assert rel < 1e-6


def test_mixed_difference_form_long_stage_chains(oracle):
    """The oracle's FP32-increment arithmetic on long stage chains (256^2, kx = 1,
    ky = 1e-2, fixed RKL2 steps of about 60 stages to t = 0.2): the difference form ends
    about 8e-8 from FP64, where summing the O(|d|) terms directly ended 1.2e-6."""
    P = oracle.Problem(oracle.MANUFACTURED, 256, kx=1.0, ky=0.01)
    rho = 1.01 * abs(P.dom_eig())
    s, tf = 60, 0.2
    h = (s * s + s - 2.0) / (2.0 * rho) * 0.999
    h = tf / math.ceil(tf / h)
    out = {}
    for mixed in (False, True):
        I = oracle.Integrator(P, P.initial(), method=oracle.RKL, mixed=mixed, hfixed=h)
        I.set_stop_time(tf)
        assert I.evolve(tf) == 1
        assert I.stats()["stage_max"] > 50
        out[mixed] = I.y
    rel = np.linalg.norm(out[True] - out[False]) / np.linalg.norm(out[False])
    assert rel < 3e-7, rel


def test_oracle_reproduces_golden_runs(oracle):
    """Pins the oracle's integrator across machines (libm may differ by an ulp)."""
    for name in ("oracle_rkc_17x9", "oracle_rkl_32", "oracle_rkl_mixed_32"):
        g = np.load(os.path.join(GOLD, name + ".npz"))
        pk = json.loads(str(g["problem"]))
        ok = json.loads(str(g["opts"]))
        P = oracle.Problem(**pk)
        I = oracle.Integrator(P, P.initial(), **ok)
        I.set_stop_time(float(g["tf"]))  # as diffusion_2D/main.cpp:384 does
        assert I.evolve(float(g["tf"])) == 1
        assert I.stats()["nst"] == int(g["nst"])
        assert np.max(np.abs(I.y - g["y"])) <= 1e-12 * np.max(np.abs(g["y"]))


# ---------------------------------------------------------------- the C ABI
def header_functions():
    import re
    root = os.path.dirname(GOLD)
    src = open(os.path.join(os.path.dirname(root), "include", "stsgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"struct _generic_N_Vector_Ops \{.*?\};", "", src, flags=re.S)
    typedefs = set(re.findall(r"\(\s*\*\s*(\w+)\s*\)", src))
    names = re.findall(r"\b((?:STS|N_V)\w+)\s*\(", src)
    return sorted(set(n for n in names if n not in typedefs))


def test_library_exports_every_declared_symbol(stslib):
    L = stslib.lib()
    names = header_functions()
    assert len(names) > 60
    for n in names:
        assert hasattr(L, n), n
    declared = {s[0] for s in stslib.SIGNATURES}
    assert set(names) == declared


def test_deterministic_pow_accuracy(oracle):
    """The controllers' pow (series log/exp built from exactly rounded operations) stays within
    a few ulp of the exact value over the controllers' range."""
    L = oracle.lib()
    rng = np.random.default_rng(0)
    xs = np.concatenate([10.0 ** rng.uniform(-10, 10, 2000), [1.0, 0.5, 2.0, 1e-10, 1.5e-10, 7.3]])
    for y in (-0.58 / 3, 0.21 / 3, -0.1 / 3, -0.8 / 3, 0.31 / 3, -1.0 / 3, 1.0 / 3, 2.5):
        got = np.array([L.orc_pow(float(x), y) for x in xs])
        want = np.array([float(mpmath_pow(x, y)) for x in xs])
        # the rounding of y log x is amplified by |y log x| in exp: a few ulp times (1 + |y log x|)
        bound = 4.5e-16 * (1.0 + np.abs(y * np.log(xs)))
        assert np.all(np.abs(got - want) / want < bound)


@pytest.mark.parametrize("type_,s,order", [(2, 2, 2), (2, 10, 2), (2, 37, 2), (3, 4, 3), (3, 9, 3),
                                           (3, 16, 3), (3, 25, 3), (4, 10, 4)])
def test_ssp_weights_order_and_parity(oracle, stslib, type_, s, order):
    """SSP(s,2) / SSP(n^2,3) / SSP(10,4) (Ketcheson 2008) as the integrator builds them: the
    product's host weights equal the oracle's bit for bit; the method meets its order
    conditions on b, the embedded weights bhat = b - w exactly one order less."""
    b, c, w = stslib.ssp_weights(type_, s)
    ob, oc, ow = oracle.ssp_weights(type_, s)
    assert np.array_equal(b, ob) and np.array_equal(c, oc) and np.array_equal(w, ow)
    bh = b - w
    # quadrature conditions sum b c^(k-1) = 1/k (sufficient to tell the orders apart here)
    for k in range(1, order + 1):
        assert abs(np.dot(b, c ** (k - 1)) - 1.0 / k) < 1e-12, ("main", k)
    for k in range(1, order):
        assert abs(np.dot(bh, c ** (k - 1)) - 1.0 / k) < 1e-12, ("embedded", k)
    assert abs(np.dot(bh, c ** (order - 1)) - 1.0 / order) > 1e-6  # embedding exactly one order less
    assert np.abs(w).max() > 1e-6


def test_oracle_krylov_solvers_against_dense_solve(oracle):
    """The oracle's SUNLinSol_SPGMR / generic PCG restatements solve (I - gamma A) x = b to the
    requested tolerance (checked against a dense solve); GMRES residual estimates equal the
    true residuals; restarting and both Gram-Schmidt variants converge."""
    nx, ny, gamma = 20, 16, 2e-3
    P = oracle.Problem(oracle.MANUFACTURED, nx, ny, kx=1.0, ky=0.2)
    n = nx * ny
    M = np.zeros((n, n))
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        M[:, k] = e - gamma * P.apply_A(e)
    b = np.random.default_rng(2).standard_normal(n)
    xt = np.linalg.solve(M, b)
    for gs in (1, 2):
        for maxl, rs in ((60, 0), (7, 40)):
            x, rc, it, rel = P.spgmr(gamma, b, tol=1e-10, maxl=maxl, max_restarts=rs, gstype=gs)
            true = np.linalg.norm(b - M @ x) / np.linalg.norm(b)
            assert rc == 0 and rel <= 1e-10 and abs(true - rel) < 1e-12
            assert np.linalg.norm(x - xt) / np.linalg.norm(xt) < 1e-8
    x, rc, it, rel = P.spgmr(gamma, b, tol=1e-14, maxl=3, max_restarts=0)
    assert rc == 1 and it == 3
    x, rc, it, rel = P.pcg_generic(gamma, b, tol=1e-10)
    assert rc == 0 and np.linalg.norm(x - xt) / np.linalg.norm(xt) < 1e-8


def test_oracle_pfmg_vcycle_is_spd_and_converges(oracle):
    """The PFMG-role V-cycle is a symmetric positive definite operator (so it preconditions
    CG), and CG with it needs a handful of iterations where Jacobi-PCG needs hundreds."""
    nx, ny, gamma = 24, 20, 1e-2
    for relax in (1, 2):
        for ky in (1.0, 1e-3):
            P = oracle.Problem(oracle.MANUFACTURED, nx, ny, kx=1.0, ky=ky)
            n = nx * ny
            B = np.zeros((n, n))
            for k in range(n):
                e = np.zeros(n)
                e[k] = 1.0
                B[:, k] = P.pfmg_vcycle(gamma, e, relax=relax)[0]
            assert np.abs(B - B.T).max() <= 1e-12 * np.abs(B).max()
            assert np.linalg.eigvalsh(0.5 * (B + B.T)).min() > 0
            b = np.random.default_rng(3).standard_normal(n)
            x, rc, it, rel = P.pcg_pfmg(gamma, b, tol=1e-10, relax=relax)
            _, it_j, _ = P.pcg(gamma, b, tol=1e-10)
            assert rc == 0 and rel <= 1e-10 and it <= 12 and it_j > 3 * it


def test_oracle_nonfinite_state_fails_cleanly(oracle):
    """A NaN or Inf in the initial state: the initial step estimate is not finite, so the call
    ends with ARK_ERR_FAILURE (-3) before any step attempt, with the counters consistent."""
    for kind in (0, 2):
        for mixed in ((False, True) if kind == 0 else (False,)):
            for val in (np.nan, np.inf, -np.inf):
                P = oracle.Problem(kind=kind, nx=16, ny=12)
                y = P.initial()
                y[37] = val
                J = oracle.Integrator(P, y, method=1, mixed=mixed)
                assert J.evolve(0.01) == -3
                s = J.stats()
                assert s["t"] == 0.0 and s["nst"] == 0
                assert s["nst_attempts"] == 0 and s["netf"] == 0
                assert s["stages_total"] == 0 and s["nfe"] == 2


def test_oracle_under_address_and_ub_sanitizers():
    """The oracle built with AddressSanitizer and UndefinedBehaviorSanitizer (float-to-int
    overflow included, every report fatal) walks every entry point on tiny and ragged grids."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None or shutil.which("make") is None:
        pytest.skip("no gcc / make")
    d = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
    r = subprocess.run(["make", "-s", "-C", d, "sanitize", "CC=gcc"], capture_output=True,
                       text=True, timeout=600)
    if r.returncode != 0 and "cannot find" in r.stderr and "asan" in r.stderr:
        pytest.skip("no sanitizer runtime for this compiler")
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "sanitize_check: ok" in r.stdout


@pytest.mark.parametrize("implicit,order", [(True, 2), (True, 3), (False, 2), (False, 3), (False, 4)])
def test_arkstep_tables_order_conditions_and_parity(oracle, stslib, implicit, order):
    """The ARKStep Butcher tables (ARKODE_SDIRK_2_1_2, ARKODE_ARK324L2SA_DIRK_4_2_3, Heun-Euler,
    Bogacki-Shampine, Zonneveld): product and oracle hold the same bits, rows sum to c, the
    method meets the order conditions of order q and the embedding those of order p."""
    A, b, d, c, q, p = stslib.arkstep_table(implicit, order)
    Ao, bo, do, co, qo, po_ = oracle.ark_table(implicit, order)
    for x, y in ((A, Ao), (b, bo), (d, do), (c, co)):
        assert np.array_equal(x, y)
    assert (q, p) == (qo, po_) == (order, order - 1)
    assert np.allclose(A.sum(axis=1), c, atol=1e-15)
    if implicit:
        assert np.all(np.diag(A)[1:] > 0)
    else:
        assert np.all(np.triu(A) == 0)

    def conds(w, k):
        out = [w.sum() - 1.0]
        if k >= 2:
            out.append(w @ c - 0.5)
        if k >= 3:
            out += [w @ c ** 2 - 1.0 / 3.0, w @ (A @ c) - 1.0 / 6.0]
        if k >= 4:
            out += [w @ c ** 3 - 0.25, w @ (c * (A @ c)) - 0.125, w @ (A @ c ** 2) - 1.0 / 12.0,
                    w @ (A @ (A @ c)) - 1.0 / 24.0]
        return np.abs(out)
    assert np.all(conds(b, q) < 1e-14)
    assert np.all(conds(d, p) < 1e-14)
    assert conds(d, p + 1).max() > 1e-6  # the embedding is of order p exactly


def test_oracle_arkstep_converges_at_its_order(oracle):
    P = oracle.Problem(oracle.MANUFACTURED, 24, 24, kx=1.0, ky=1.0)
    for order in (2, 3):
        ref, errs = None, []
        for h in (1e-4, 4e-3, 2e-3):
            I = oracle.ArkIntegrator(P, P.initial(), implicit=True, order=order, hfixed=h, ls="cg", maxl=500,
                                     prec="jacobi", msbp=1, epslin=1e-6)
            I.set_stop_time(0.08)
            assert I.evolve(0.08) == 1
            if ref is None:
                ref = I.y.copy()
            else:
                errs.append(np.linalg.norm(I.y - ref))
        assert abs(np.log2(errs[0] / errs[1]) - order) < 0.35


# ---------------------------------------------------------------- stop time and dense output
def test_hermite_dense_output_reproduces_polynomials(oracle):
    """orc_hermite of degree d is exact for polynomials of degree <= d (y_old, y_new and, for
    d >= 2, the derivatives at the ends), the property of ARKODE's Hermite interpolant."""
    import ctypes as C
    rng = np.random.default_rng(3)
    t0, h = 0.3, 0.125
    t1 = t0 + h
    for deg in (1, 2, 3):
        c = rng.standard_normal((deg + 1, 5))  # five components, degree-deg polynomials

        def p(t, k=0):
            out = np.zeros(5)
            for j in range(k, deg + 1):
                out += c[j] * math.perm(j, k) * t ** (j - k)
            return out
        yold, ynew, fold, fnew = p(t0), p(t1), p(t0, 1), p(t1, 1)
        for tq in (t0, t0 + 0.3 * h, t0 + 0.77 * h, t1):
            out = np.empty(5)
            oracle.lib().orc_hermite(5, deg, (tq - t1) / h, h, oracle.dptr(yold), oracle.dptr(ynew),
                                     oracle.dptr(fold), oracle.dptr(fnew), oracle.dptr(out))
            assert np.allclose(out, p(tq), rtol=1e-13, atol=1e-13), (deg, tq)


def _lsrk(oracle, P, **kw):
    return oracle.Integrator(P, P.initial(), rtol=1e-6, atol=1e-10, **kw)


@pytest.mark.parametrize("kind", ["rkc", "rkl_mixed", "ssp3_9", "ssp10_4", "erk4", "erk3", "dirk3"])
def test_outputs_without_stop_time_leave_the_steps_alone(oracle, kind):
    """ARKodeEvolve in NORMAL mode with only the final stop time (diffusion_2D/main.cpp:384,
    :431-470 without --error): the intermediate outputs come from the dense output and do not
    change the step sequence, so the final state and the step count equal a run that outputs
    only at the first tout (the initial step depends on it, as ARKODE's does) and at tf. Each
    output is the solution at its tout to the tolerance's order."""
    P = oracle.Problem(oracle.MANUFACTURED, 24, 20, kx=1.0, ky=0.5)
    tf = 0.02

    def make():
        if kind == "rkc":
            return _lsrk(oracle, P, method=oracle.RKC, tstop=tf)
        if kind == "rkl_mixed":
            return _lsrk(oracle, P, method=oracle.RKL, mixed=True, tstop=tf)
        if kind.startswith("ssp"):
            return _lsrk(oracle, P, ssp=(3, 9) if kind == "ssp3_9" else (4, 10), tstop=tf)
        if kind.startswith("erk"):
            return oracle.ArkIntegrator(P, P.initial(), implicit=False, order=int(kind[-1]), rtol=1e-6,
                                        atol=1e-10, tstop=tf)
        return oracle.ArkIntegrator(P, P.initial(), implicit=True, order=3, rtol=1e-6, atol=1e-10, ls="cg",
                                    maxl=50, prec="jacobi", msbp=1, tstop=tf)
    A = make()
    assert A.evolve(tf / 8) == 0
    assert A.evolve(tf) == 1 and A.tret == tf
    B = make()
    worst = 0.0
    for k in range(1, 8):
        tout = tf * k / 8
        assert B.evolve(tout) == 0 and B.tret == tout
        assert B.stats()["t"] >= tout
        C = make()  # a run that lands on tout (stop time there)
        C.set_stop_time(tout)
        assert C.evolve(tout) == 1
        worst = max(worst, np.linalg.norm(B.y - C.y) / np.linalg.norm(C.y))
    assert 0.0 < worst < 1e-4, worst
    assert B.evolve(tf) == 1
    assert B.stats()["nst"] == A.stats()["nst"]
    assert np.array_equal(A.y, B.y)


def test_stop_time_is_cleared_and_tout_behind_interpolates(oracle):
    P = oracle.Problem(oracle.MANUFACTURED, 24, 20, kx=1.0, ky=0.5)
    I = _lsrk(oracle, P, method=oracle.RKL, tstop=0.01)
    assert I.evolve(0.02) == 1 and I.tret == 0.01 and I.stats()["t"] == 0.01
    # the stop time was cleared: the next call steps past tout and interpolates
    assert I.evolve(0.015) == 0 and I.stats()["t"] > 0.015
    nst, y1 = I.stats()["nst"], I.y.copy()
    # a tout the last step already passed: dense output again, no step taken
    t_prev = 0.015 - 0.25 * (I.stats()["t"] - 0.015)
    assert I.evolve(max(t_prev, I.stats()["t"] - I.stats()["hlast"])) == 0
    assert I.stats()["nst"] == nst and not np.array_equal(I.y, y1)
    # tout before the last step: rejected
    assert I.evolve(0.001) == -22
