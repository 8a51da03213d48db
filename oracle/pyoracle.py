"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg; the CUDA
product never imports it. ``build()`` compiles ``oracle/sts_oracle.c`` with the committed
Makefile into ``oracle/_build/libsts_oracle.so``.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsts_oracle.so")

MANUFACTURED, UNFORCED, PERIODIC = 0, 1, 2
RKC, RKL = 0, 1

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


class Prob(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("kind", C.c_int), ("inhomogeneous", C.c_int),
                ("kx", C.c_double), ("ky", C.c_double), ("xl", C.c_double), ("xu", C.c_double),
                ("yl", C.c_double), ("yu", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("cc", C.c_double),
                ("Sx", _dp), ("Sxx", _dp), ("Sy", _dp), ("Syy", _dp),
                ("Dxw", _dp), ("Dxe", _dp), ("Dys", _dp), ("Dyn", _dp)]


class ArkOpts(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("implicit", "order", "controller", "ls", "maxl", "max_restarts", "gstype",
                                       "prec", "pfmg_relax", "pfmg_nrelax", "msbp", "linear", "onestep")] + \
               [("maxsteps", C.c_long)] + [(k, C.c_double) for k in ("rtol", "atol", "hfixed", "eplifac")]


class Dense(C.Structure):
    """orc_dense: the integrator's y_n, the last step's y_old / f_old, stop time, last return."""
    _fields_ = [("ycur", C.POINTER(C.c_double)), ("yold", C.POINTER(C.c_double)),
                ("fold", C.POINTER(C.c_double)), ("tstop", C.c_double), ("tretlast", C.c_double),
                ("tstopset", C.c_int), ("interp_ready", C.c_int)]


ARK_STAT_KEYS = ("t", "hnext", "hlast", "h0", "ep1", "ep2", "gamma_setup", "nst", "nst_att", "netf", "ncfn",
                 "nfe", "nfi", "nni", "nnf", "nli", "nlcf", "npe", "nps", "njv", "nsetups", "nhist", "nst_setup",
                 "initialized", "after_fail", "force_setup")


class ArkState(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("t", "hnext", "hlast", "h0", "ep1", "ep2", "gamma_setup")] + \
               [(k, C.c_long) for k in ("nst", "nst_att", "netf", "ncfn", "nfe", "nfi", "nni", "nnf", "nli", "nlcf",
                                        "npe", "nps", "njv", "nsetups", "nhist", "nst_setup")] + \
               [(k, C.c_int) for k in ("initialized", "after_fail", "force_setup", "fn_current")] + \
               [("Fn", C.POINTER(C.c_double)), ("d", Dense)]


class Opts(C.Structure):
    _fields_ = [("method", C.c_int), ("mixed", C.c_int), ("controller", C.c_int),
                ("smax", C.c_int), ("internaleig", C.c_int), ("dee_maxiters", C.c_int),
                ("dom_eig_freq", C.c_int), ("pad_", C.c_int), ("maxsteps", C.c_long),
                ("rtol", C.c_double), ("atol", C.c_double), ("hfixed", C.c_double),
                ("eig_safety", C.c_double), ("dee_reltol", C.c_double),
                ("dee_init_warmups", C.c_int), ("dee_succ_warmups", C.c_int)]


class State(C.Structure):
    _fields_ = [("t", C.c_double), ("hnext", C.c_double), ("hlast", C.c_double),
                ("spectral_radius", C.c_double), ("ep1", C.c_double), ("ep2", C.c_double),
                ("nst", C.c_long), ("nst_attempts", C.c_long), ("netf", C.c_long),
                ("nfe", C.c_long), ("nfe_dee", C.c_long), ("ndee", C.c_long),
                ("nst_exp", C.c_long), ("stage_max", C.c_long), ("stages_total", C.c_long),
                ("nhist", C.c_long), ("steps_since_dee", C.c_long),
                ("initialized", C.c_int), ("after_fail", C.c_int),
                ("F", _dp), ("Ff", _fp), ("evec", _dp), ("d", Dense)]


def build(force=False):
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "sts_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_xsum.restype = C.c_double
        L.orc_xsum.argtypes = [_dp, C.c_long]
        L.orc_xdot.restype = C.c_double
        L.orc_xdot.argtypes = [_dp, _dp, C.c_long]
        L.orc_wrms.restype = C.c_double
        L.orc_wrms.argtypes = [_dp, _dp, C.c_long]
        L.orc_maxnorm.restype = C.c_double
        L.orc_maxnorm.argtypes = [_dp, C.c_long]
        L.orc_prob_create.restype = C.POINTER(Prob)
        L.orc_prob_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                      C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_prob_free.argtypes = [C.POINTER(Prob)]
        L.orc_initial.argtypes = [C.POINTER(Prob), _dp]
        L.orc_initial_modes.argtypes = [C.POINTER(Prob), C.c_int, C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), _dp, _dp]
        L.orc_exact.argtypes = [C.POINTER(Prob), C.c_double, _dp]
        L.orc_c.restype = C.c_double
        L.orc_c.argtypes = [C.c_double]
        L.orc_cdot.restype = C.c_double
        L.orc_cdot.argtypes = [C.c_double]
        for name in ("orc_rhs", "orc_rhs_ref"):
            getattr(L, name).argtypes = [C.POINTER(Prob), C.c_double, _dp, _dp]
        L.orc_apply_A.argtypes = [C.POINTER(Prob), _dp, _dp]
        L.orc_dom_eig.restype = C.c_double
        L.orc_dom_eig.argtypes = [C.POINTER(Prob)]
        L.orc_power_iteration.restype = C.c_int
        L.orc_power_iteration.argtypes = [C.POINTER(Prob), _dp, C.c_int, C.c_double, _dp]
        L.orc_stage_coeffs.restype = C.c_int
        L.orc_stage_coeffs.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_stages_needed.restype = C.c_int
        L.orc_stages_needed.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp]
        L.orc_ssp_weights.restype = C.c_int
        L.orc_ssp_weights.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_ssp_evolve.restype = C.c_int
        L.orc_pow.restype = C.c_double
        L.orc_pow.argtypes = [C.c_double, C.c_double]
        L.orc_controller.restype = C.c_double
        L.orc_controller.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_long]
        L.orc_state_init.argtypes = [C.POINTER(State), C.c_double]
        L.orc_state_free.argtypes = [C.POINTER(State)]
        L.orc_lsrk_evolve.restype = C.c_int
        L.orc_lsrk_evolve.argtypes = [C.POINTER(Prob), C.POINTER(Opts), C.POINTER(State),
                                      C.c_double, _dp]
        L.orc_pcg.restype = C.c_int
        L.orc_pcg.argtypes = [C.POINTER(Prob), C.c_double, C.c_int, _dp, _dp, C.c_double,
                              C.c_int, _dp]
        L.orc_sdirk2.restype = C.c_int
        L.orc_sdirk2.argtypes = [C.POINTER(Prob), C.c_double, C.c_double, C.c_int, C.c_double,
                                 C.c_int, _dp, C.POINTER(C.c_long)]
        L.orc_pcg_generic.restype = C.c_int
        L.orc_pcg_generic.argtypes = [C.POINTER(Prob), C.c_double, C.c_int, _dp, _dp, C.c_double,
                                      C.c_int, C.POINTER(C.c_int), _dp]
        L.orc_spgmr.restype = C.c_int
        L.orc_spgmr.argtypes = [C.POINTER(Prob), C.c_double, C.c_int, _dp, _dp, C.c_double, C.c_int,
                                C.c_int, C.c_int, C.POINTER(C.c_int), _dp]
        L.orc_spfgmr.restype = C.c_int
        L.orc_spfgmr.argtypes = L.orc_spgmr.argtypes
        L.orc_sdirk2_ls.restype = C.c_int
        L.orc_sdirk2_ls.argtypes = [C.POINTER(Prob), C.c_double, C.c_double, C.c_int, C.c_double,
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp,
                                    C.POINTER(C.c_long)]
        L.orc_pfmg_vcycle.restype = C.c_int
        L.orc_pfmg_vcycle.argtypes = [C.POINTER(Prob), C.c_double, C.c_int, C.c_int, _dp, _dp,
                                      C.POINTER(C.c_int)]
        L.orc_pcg_pfmg.restype = C.c_int
        L.orc_pcg_pfmg.argtypes = [C.POINTER(Prob), C.c_double, C.c_int, C.c_int, _dp, _dp, C.c_double,
                                   C.c_int, C.POINTER(C.c_int), _dp]
        L.orc_sdirk2_pfmg.restype = C.c_int
        L.orc_sdirk2_pfmg.argtypes = [C.POINTER(Prob), C.c_double, C.c_double, C.c_int, C.c_double, C.c_int,
                                      C.c_int, C.c_int, _dp, C.POINTER(C.c_long)]
        L.orc_arkstep_evolve.restype = C.c_int
        L.orc_arkstep_evolve.argtypes = [C.POINTER(Prob), C.POINTER(ArkOpts), C.POINTER(ArkState), C.c_double, _dp]
        L.orc_ark_state_free.argtypes = [C.POINTER(ArkState)]
        L.orc_hermite.argtypes = [C.c_long, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp]
        L.orc_ark_table.restype = C.c_int
        L.orc_ark_table.argtypes = [C.c_int, C.c_int] + [C.POINTER(C.c_int)] * 3 + [_dp] * 4
        L.orc_nthreads.restype = C.c_int
        L.orc_set_nthreads.argtypes = [C.c_int]
        _lib = L
    return _lib


def dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def xsum(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().orc_xsum(dptr(x), x.size)


def xdot(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return lib().orc_xdot(dptr(x), dptr(y), x.size)


def wrms(x, w):
    x = np.ascontiguousarray(x, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib().orc_wrms(dptr(x), dptr(w), x.size)


def maxnorm(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().orc_maxnorm(dptr(x), x.size)


def stage_coeffs(method, s):
    arrs = [np.zeros(s + 1) for _ in range(5)]
    rc = lib().orc_stage_coeffs(method, s, *[dptr(a) for a in arrs])
    assert rc == 0
    return arrs


def stages_needed(method, h, rho, smax):
    hmax = C.c_double()
    s = lib().orc_stages_needed(method, h, rho, smax, C.byref(hmax))
    return s, hmax.value


def controller(kind, h, dsm, ep1, ep2, hp, nhist):
    return lib().orc_controller(kind, h, dsm, ep1, ep2, hp, nhist)


class Problem:
    """Host problem: grid, coefficients and manufactured tables."""

    def __init__(self, kind=MANUFACTURED, nx=128, ny=None, kx=1.0, ky=1.0, inhomogeneous=False,
                 xl=-np.pi, xu=np.pi, yl=-6.0, yu=6.0):
        ny = nx if ny is None else ny
        self.p = lib().orc_prob_create(kind, nx, ny, kx, ky, int(inhomogeneous), xl, xu, yl, yu)
        if not self.p:
            raise ValueError("bad problem")
        self.nx, self.ny, self.kind = nx, ny, kind

    def __del__(self):
        try:
            lib().orc_prob_free(self.p)
        except Exception:
            pass

    @property
    def n(self):
        return self.nx * self.ny

    def field(self):
        return np.zeros(self.n)

    def initial(self):
        u = self.field()
        lib().orc_initial(self.p, dptr(u))
        return u

    def initial_modes(self, pm, qm, amp):
        u = self.field()
        pm = np.ascontiguousarray(pm, dtype=np.int32)
        qm = np.ascontiguousarray(qm, dtype=np.int32)
        amp = np.ascontiguousarray(amp, dtype=np.float64)
        lib().orc_initial_modes(self.p, len(amp), pm.ctypes.data_as(C.POINTER(C.c_int)),
                                qm.ctypes.data_as(C.POINTER(C.c_int)), dptr(amp), dptr(u))
        return u

    def exact(self, t):
        u = self.field()
        lib().orc_exact(self.p, t, dptr(u))
        return u

    def rhs(self, t, u, ref=False):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = self.field()
        (lib().orc_rhs_ref if ref else lib().orc_rhs)(self.p, t, dptr(u), dptr(f))
        return f

    def apply_A(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = self.field()
        lib().orc_apply_A(self.p, dptr(v), dptr(w))
        return w

    def dom_eig(self):
        return lib().orc_dom_eig(self.p)

    def power_iteration(self, v0, maxiters=100, reltol=0.01):
        v = np.array(v0, dtype=np.float64)
        lam = C.c_double()
        it = lib().orc_power_iteration(self.p, dptr(v), maxiters, reltol, C.byref(lam))
        return lam.value, it, v

    def tables(self):
        P = self.p.contents
        g = lambda ptr, n: np.ctypeslib.as_array(ptr, shape=(n,)).copy()
        return g(P.Sx, self.nx), g(P.Sxx, self.nx), g(P.Sy, self.ny), g(P.Syy, self.ny)

    def pcg(self, gamma, b, tol=1e-8, maxit=10000, jacobi=True):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = self.field()
        rel = C.c_double()
        it = lib().orc_pcg(self.p, gamma, int(jacobi), dptr(b), dptr(x), tol, maxit, C.byref(rel))
        return x, it, rel.value

    def pcg_generic(self, gamma, b, tol=1e-8, maxl=10000, jacobi=True):
        """SUNLinSol_PCG through callbacks: (x, status, iterations, relative residual)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = self.field()
        it, rel = C.c_int(), C.c_double()
        rc = lib().orc_pcg_generic(self.p, gamma, int(jacobi), dptr(b), dptr(x), tol, maxl,
                                   C.byref(it), C.byref(rel))
        return x, rc, it.value, rel.value

    def spgmr(self, gamma, b, tol=1e-8, maxl=20, max_restarts=0, gstype=1, jacobi=True,
              flexible=False):
        """SUNLinSol_SPGMR (flexible: SUNLinSol_SPFGMR): (x, status, iterations, relative
        residual estimate)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = self.field()
        it, rel = C.c_int(), C.c_double()
        fn = lib().orc_spfgmr if flexible else lib().orc_spgmr
        rc = fn(self.p, gamma, int(jacobi), dptr(b), dptr(x), tol, maxl, max_restarts, gstype,
                C.byref(it), C.byref(rel))
        return x, rc, it.value, rel.value

    def pfmg_vcycle(self, gamma, r, relax=2, nrelax=2):
        """One PFMG-role V-cycle z = B r: (z, number of levels)."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = self.field()
        nl = C.c_int()
        lib().orc_pfmg_vcycle(self.p, gamma, relax, nrelax, dptr(r), dptr(z), C.byref(nl))
        return z, nl.value

    def pcg_pfmg(self, gamma, b, tol=1e-8, maxl=10000, relax=2, nrelax=2):
        """CG with the PFMG-role preconditioner: (x, status, iterations, relative residual)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = self.field()
        it, rel = C.c_int(), C.c_double()
        rc = lib().orc_pcg_pfmg(self.p, gamma, relax, nrelax, dptr(b), dptr(x), tol, maxl, C.byref(it),
                                C.byref(rel))
        return x, rc, it.value, rel.value

    def sdirk2_pfmg(self, y0, t0, h, nsteps, tol=1e-10, maxl=100000, relax=2, nrelax=2):
        y = np.array(y0, dtype=np.float64)
        it = C.c_long()
        lib().orc_sdirk2_pfmg(self.p, t0, h, nsteps, tol, maxl, relax, nrelax, dptr(y), C.byref(it))
        return y, it.value

    def sdirk2_ls(self, y0, t0, h, nsteps, tol=1e-10, ls=1, maxl=20, max_restarts=0, gstype=1,
                  jacobi=True):
        y = np.array(y0, dtype=np.float64)
        it = C.c_long()
        lib().orc_sdirk2_ls(self.p, t0, h, nsteps, tol, ls, maxl, max_restarts, gstype, int(jacobi),
                            dptr(y), C.byref(it))
        return y, it.value

    def sdirk2(self, y0, t0, h, nsteps, tol=1e-10, maxit=10000):
        y = np.array(y0, dtype=np.float64)
        it = C.c_long()
        lib().orc_sdirk2(self.p, t0, h, nsteps, tol, maxit, dptr(y), C.byref(it))
        return y, it.value


def make_opts(method=RKC, mixed=False, controller=0, smax=200, rtol=1e-6, atol=1e-10,
              hfixed=0.0, internaleig=False, maxsteps=100000, eig_safety=1.01, dee_maxiters=100,
              dee_reltol=0.01, dom_eig_freq=25, dee_warmups=(0, 0)):
    return Opts(method=method, mixed=int(mixed), controller=controller, smax=smax,
                internaleig=int(internaleig), dee_maxiters=dee_maxiters, dom_eig_freq=dom_eig_freq,
                maxsteps=maxsteps, rtol=rtol, atol=atol, hfixed=hfixed, eig_safety=eig_safety,
                dee_reltol=dee_reltol, dee_init_warmups=dee_warmups[0],
                dee_succ_warmups=dee_warmups[1])


class Integrator:
    """The oracle's LSRK integrator (state persists across evolve calls)."""

    def __init__(self, prob, y0, t0=0.0, ssp=None, tstop=None, **opts):
        self.prob = prob
        self.ssp = ssp  # (type, stages) for the SSP methods
        self.opts = make_opts(**opts)
        self.st = State()
        lib().orc_state_init(C.byref(self.st), t0)
        self.y = np.array(y0, dtype=np.float64)
        if tstop is not None:
            self.set_stop_time(tstop)

    def evolve(self, tout):
        """ARKodeEvolve (NORMAL): self.y receives the solution at tret (tout, by dense output
        when the last step passed it; the stop time when reached, return code 1)."""
        if self.ssp is not None:
            return lib().orc_ssp_evolve(self.prob.p, C.byref(self.opts), self.ssp[0], self.ssp[1],
                                        C.byref(self.st), C.c_double(tout), dptr(self.y))
        rc = lib().orc_lsrk_evolve(self.prob.p, C.byref(self.opts), C.byref(self.st), tout,
                                   dptr(self.y))
        return rc

    def set_stop_time(self, tstop):
        self.st.d.tstop = tstop
        self.st.d.tstopset = 1

    @property
    def tret(self):
        return self.st.d.tretlast

    def stats(self):
        s = self.st
        return {k: getattr(s, k) for k in ("t", "hlast", "hnext", "spectral_radius", "nst",
                                           "nst_attempts", "netf", "nfe", "nfe_dee", "ndee",
                                           "nst_exp", "stage_max", "stages_total")}

    def __del__(self):
        try:
            lib().orc_state_free(C.byref(self.st))
        except Exception:
            pass


def ssp_weights(type_, s):
    b, c, w = np.empty(s), np.empty(s), np.empty(s)
    if lib().orc_ssp_weights(type_, s, dptr(b), dptr(c), dptr(w)) != 0:
        raise ValueError("invalid SSP method / stage count")
    return b, c, w


class ArkIntegrator:
    """The oracle's ARKStep (orc_arkstep_evolve): implicit DIRK with Newton + PCG / SPGMR
    (prec None / "jacobi" / "pfmg") or explicit ERK; state persists across evolve calls."""

    def __init__(self, prob, y0, t0=0.0, implicit=True, order=2, rtol=1e-5, atol=1e-10, controller=0,
                 hfixed=0.0, maxsteps=100000, ls="cg", maxl=20, prec="jacobi", pfmg_relax=2, pfmg_nrelax=2,
                 msbp=0, epslin=0.0, linear=False, max_restarts=0, gstype=1, onestep=False, tstop=None):
        self.prob = prob
        pc = {None: 0, "jacobi": 1, "pfmg": 2}[prec]
        self.opts = ArkOpts(implicit=int(implicit), order=order, controller=controller,
                            ls=0 if ls == "cg" else 1, maxl=maxl, max_restarts=max_restarts, gstype=gstype,
                            prec=pc, pfmg_relax=pfmg_relax, pfmg_nrelax=pfmg_nrelax, msbp=msbp,
                            linear=int(linear), onestep=int(onestep), maxsteps=maxsteps, rtol=rtol, atol=atol,
                            hfixed=hfixed, eplifac=epslin if epslin > 0 else 0.05)
        self.st = ArkState()
        self.st.t = t0
        self.st.force_setup = 1
        self.y = np.array(y0, dtype=np.float64)
        if tstop is not None:
            self.set_stop_time(tstop)

    def evolve(self, tout):
        return lib().orc_arkstep_evolve(self.prob.p, C.byref(self.opts), C.byref(self.st), tout, dptr(self.y))

    def set_stop_time(self, tstop):
        self.st.d.tstop = tstop
        self.st.d.tstopset = 1

    @property
    def tret(self):
        return self.st.d.tretlast

    def stats(self):
        return {k: getattr(self.st, k) for k in ARK_STAT_KEYS}

    def __del__(self):
        try:
            lib().orc_ark_state_free(C.byref(self.st))
        except Exception:
            pass


def ark_table(implicit, order):
    s, q, p = C.c_int(), C.c_int(), C.c_int()
    A, b, d, c = np.zeros(25), np.zeros(5), np.zeros(5), np.zeros(5)
    if lib().orc_ark_table(int(implicit), order, C.byref(s), C.byref(q), C.byref(p), dptr(A), dptr(b), dptr(d),
                           dptr(c)) != 0:
        raise ValueError("no table")
    n = s.value
    return A[:n * n].reshape(n, n), b[:n], d[:n], c[:n], q.value, p.value
