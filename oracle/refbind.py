"""ctypes binding of oracle/_ref/libdiffusion_ref.so: the reference's own diffusion_2D
sources (RHS, initial state, Jacobi PSetup/PSolve, coefficients) compiled unmodified with
single-rank stand-ins for MPI and SUNDIALS' serial vector (TEST INFRASTRUCTURE ONLY).

Built by ``make -C oracle ref`` where the reference tree is present; ``available()`` says
whether it can be used on this machine."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libdiffusion_ref.so")
REF_DIR = os.environ.get("STS_REFERENCE_DIR", "/root/reference/diffusion_2D")
_dp = C.POINTER(C.c_double)
_lib = None


def build():
    """Compile the reference sources if the reference tree is present; returns the path or None."""
    if os.path.isdir(REF_DIR):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_DIR], check=True)
    return LIB_PATH if os.path.exists(LIB_PATH) else None


def available():
    return build() is not None


def lib():
    global _lib
    if _lib is None:
        if build() is None:
            raise RuntimeError("oracle/_ref is not built and the reference tree is absent")
        L = C.CDLL(LIB_PATH)
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_grid.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.ref_rhs.argtypes = [C.c_void_p, C.c_double, _dp, _dp]
        L.ref_initial.argtypes = [C.c_void_p, _dp]
        L.ref_jacobi.argtypes = [C.c_void_p, C.c_double, _dp, _dp, _dp]
        L.ref_coeff_x.restype = C.c_double
        L.ref_coeff_x.argtypes = [C.c_void_p, C.c_double]
        L.ref_coeff_y.restype = C.c_double
        L.ref_coeff_y.argtypes = [C.c_void_p, C.c_double]
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class RefProblem:
    """The reference's UserData for the periodic problem (default domain [-pi,pi] x [-6,6])."""

    def __init__(self, nx, ny, kx=1.0, ky=1.0, inhomogeneous=False):
        self.nx, self.ny = nx, ny
        self.h = lib().ref_create(nx, ny, kx, ky, int(inhomogeneous))
        if not self.h:
            raise ValueError("reference setup failed")

    def __del__(self):
        try:
            lib().ref_free(self.h)
        except Exception:
            pass

    def grid(self):
        v = [C.c_double() for _ in range(4)]
        lib().ref_grid(self.h, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)  # dx, dy, xl, yl

    def rhs(self, t, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = np.empty_like(u)
        if lib().ref_rhs(self.h, t, _p(u), _p(f)) != 0:
            raise RuntimeError("reference RHS failed")
        return f

    def initial(self):
        u = np.empty(self.nx * self.ny)
        if lib().ref_initial(self.h, _p(u)) != 0:
            raise RuntimeError("reference Initial failed")
        return u

    def jacobi(self, gamma, r):
        """(diag of PSetup, z = PSolve(r))"""
        r = np.ascontiguousarray(r, dtype=np.float64)
        d, z = np.empty_like(r), np.empty_like(r)
        if lib().ref_jacobi(self.h, gamma, _p(d), _p(r), _p(z)) != 0:
            raise RuntimeError("reference PSetup/PSolve failed")
        return d, z

    def coeff_x(self, x):
        return lib().ref_coeff_x(self.h, x)

    def coeff_y(self, y):
        return lib().ref_coeff_y(self.h, y)
