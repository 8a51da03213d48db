"""GB300-native diffusion_2D super-time-stepping path: Python host interface.

This package is a thin ctypes layer over ``libstsgpu.so`` (C ABI declared in
``include/stsgpu.h``). It mirrors the reference's interfaces for the path:

* :class:`NVector`  - N_Vector ops (gkeyll_diffusion/src/nvector_gkylzero.c:45-514)
* :class:`Problem`  - UserData + the diffusion/dom_eig/PSetup/PSolve callbacks
  (diffusion_2D/diffusion_2D.hpp:66-214, diffusion_2D.cpp:23, main.cpp:536,
  preconditioner_jacobi.cpp)
* :class:`LSRKStep` - LSRKStepCreateSTS + ARKode* (diffusion_2D/main.cpp:257-486)
* :func:`implicit_solve_pcg`, :func:`sdirk2_evolve`, :class:`PCGSolver` - SUNLinSol_PCG with
  the Jacobi preconditioner (main.cpp:207-231)

There is no CPU fallback: if the CUDA library cannot be built or loaded, importing the
compute entry points raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["lib", "Context", "NVector", "Problem", "LSRKStep", "PCGSolver", "implicit_solve_pcg",
           "sdirk2_evolve", "RKC", "RKL", "PID", "PI", "I", "MANUFACTURED", "UNFORCED", "PERIODIC",
           "Net", "fcg_solve", "implicit_solve_learned", "harvest_pcg_pairs", "net_features", "smooth_field", "STSError"]

RKC, RKL = 0, 1
SSP_S_2, SSP_S_3, SSP_10_4 = 2, 3, 4
PID, PI, I, EXP_GUS, IMP_GUS, IMEX_GUS = 0, 1, 2, 3, 4, 5
MODIFIED_GS, CLASSICAL_GS = 1, 2
MANUFACTURED, UNFORCED, PERIODIC = 0, 1, 2
NORMAL, ONE_STEP = 1, 2
TOO_MUCH_WORK = -1
TSTOP_RETURN = 1

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
_ll = C.c_longlong


class STSError(RuntimeError):
    pass


class NVOps(C.Structure):
    pass


class NVStruct(C.Structure):
    _fields_ = [("content", _vp), ("ops", C.POINTER(NVOps)), ("sunctx", _vp)]


_NV = C.POINTER(NVStruct)
RHSFN = C.CFUNCTYPE(C.c_int, C.c_double, _NV, _NV, _vp)
DOMEIGFN = C.CFUNCTYPE(C.c_int, C.c_double, _NV, _NV, _dp, _dp, _vp, _NV, _NV, _NV)
ATIMESFN = C.CFUNCTYPE(C.c_int, _vp, _NV, _NV)
PSOLVEFN = C.CFUNCTYPE(C.c_int, _vp, _NV, _NV, C.c_double, C.c_int)


class Stats(C.Structure):
    _fields_ = [("nst", _ll), ("nst_attempts", _ll), ("netf", _ll), ("nfe", _ll),
                ("nfe_dee", _ll), ("ndee", _ll), ("nst_exp", _ll), ("stage_max", _ll),
                ("stages_total", _ll), ("t", C.c_double), ("hlast", C.c_double),
                ("hnext", C.c_double), ("spectral_radius", C.c_double)]


class ARKStepStats(C.Structure):
    _fields_ = [(k, _ll) for k in ("nst", "nst_attempts", "netf", "ncfn", "nfe", "nfi", "nfe_ls", "nni", "nnf",
                                   "nli", "nlcf", "npe", "nps", "njv", "nsetups")] + \
               [(k, C.c_double) for k in ("t", "h0", "hlast", "hnext")]


# (name, restype, argtypes) for every entry point of include/stsgpu.h
SIGNATURES = [
    ("STS_ProbeFP64Rate", C.c_int, [_vp, _dp]),
    ("STS_ARKStepCreate", _vp, [_vp, _vp, C.c_double, _NV, _vp]),
    ("STS_ARKodeSetOrder", C.c_int, [_vp, C.c_int]),
    ("STS_ARKodeSetLinearSolver", C.c_int, [_vp, _vp, _vp]),
    ("STS_ARKodeSetPreconditioner", C.c_int, [_vp, _vp, _vp]),
    ("STS_ARKStepSetPrecData", C.c_int, [_vp, _vp]),
    ("STS_ARKodeSetLSetupFrequency", C.c_int, [_vp, C.c_int]),
    ("STS_ARKodeSetEpsLin", C.c_int, [_vp, C.c_double]),
    ("STS_ARKodeSetLinear", C.c_int, [_vp, C.c_int]),
    ("STS_ARKodeSetNonlinear", C.c_int, [_vp]),
    ("STS_ARKStepGetStats", C.c_int, [_vp, C.POINTER(ARKStepStats)]),
    ("STS_ARKStepTable", C.c_int, [C.c_int, C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _dp]),
    ("STS_ContextCreate", C.c_int, [C.c_int, C.POINTER(_vp)]),
    ("STS_ContextFree", C.c_int, [C.POINTER(_vp)]),
    ("STS_ContextSynchronize", C.c_int, [_vp]),
    ("STS_ContextGetStream", _vp, [_vp]),
    ("STS_GetLastError", C.c_char_p, []),
    ("STS_DeviceCount", C.c_int, []),
    ("STS_WaitSelfTest", C.c_int, [_vp, C.c_int, C.c_longlong]),
    ("N_VNew_Sts", _NV, [_ll, _vp]),
    ("N_VNewEmpty_Sts", _NV, [_vp]),
    ("N_VMake_Sts", _NV, [_ll, _vp, _vp]),
    ("N_VCloneEmpty_Sts", _NV, [_NV]),
    ("N_VClone_Sts", _NV, [_NV]),
    ("N_VDestroy_Sts", None, [_NV]),
    ("N_VGetDeviceArrayPointer_Sts", _vp, [_NV]),
    ("N_VGetLength_Sts", _ll, [_NV]),
    ("N_VSpace_Sts", None, [_NV, C.POINTER(_ll), C.POINTER(_ll)]),
    ("N_VSetShape_Sts", C.c_int, [_NV, _ll, _ll]),
    ("N_VCopyFromHost_Sts", C.c_int, [_NV, _dp]),
    ("N_VCopyToHost_Sts", C.c_int, [_NV, _dp]),
    ("N_VLinearSum_Sts", None, [C.c_double, _NV, C.c_double, _NV, _NV]),
    ("N_VConst_Sts", None, [C.c_double, _NV]),
    ("N_VProd_Sts", None, [_NV, _NV, _NV]),
    ("N_VDiv_Sts", None, [_NV, _NV, _NV]),
    ("N_VScale_Sts", None, [C.c_double, _NV, _NV]),
    ("N_VAbs_Sts", None, [_NV, _NV]),
    ("N_VInv_Sts", None, [_NV, _NV]),
    ("N_VAddConst_Sts", None, [_NV, C.c_double, _NV]),
    ("N_VDotProd_Sts", C.c_double, [_NV, _NV]),
    ("N_VMaxNorm_Sts", C.c_double, [_NV]),
    ("N_VWrmsNorm_Sts", C.c_double, [_NV, _NV]),
    ("N_VLinearCombination_Sts", C.c_int, [C.c_int, _dp, C.POINTER(_NV), _NV]),
    ("N_VDotProdMulti_Sts", C.c_int, [C.c_int, _NV, C.POINTER(_NV), _dp]),
    ("STS_WrmsNormNoAlloc", C.c_int, [_vp, _vp, _ll, _vp, _vp]),
    ("STS_ProblemCreate", _vp, [_vp, C.c_int, _ll, _ll, C.c_double, C.c_double, C.c_int,
                                C.c_double, C.c_double, C.c_double, C.c_double]),
    ("STS_ProblemFree", C.c_int, [C.POINTER(_vp)]),
    ("STS_ProblemGetInfo", C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    ("STS_Initial", C.c_int, [C.c_double, _NV, _vp]),
    ("STS_InitialModes", C.c_int, [_NV, _vp, C.c_int, _ip, _ip, _dp]),
    ("STS_Exact", C.c_int, [C.c_double, _NV, _vp]),
    ("STS_Diffusion", C.c_int, [C.c_double, _NV, _NV, _vp]),
    ("STS_JacTimes", C.c_int, [_NV, _NV, C.c_double, _NV, _NV, _vp, _NV]),
    ("STS_DomEig", C.c_int, [C.c_double, _NV, _NV, _dp, _dp, _vp, _NV, _NV, _NV]),
    ("STS_PowerIteration", C.c_int, [_vp, _NV, C.c_int, C.c_double, _dp, _ip]),
    ("STS_PSetup", C.c_int, [C.c_double, _NV, _NV, C.c_int, _ip, C.c_double, _vp]),
    ("STS_PSolve", C.c_int, [C.c_double, _NV, _NV, _NV, _NV, C.c_double, C.c_double, C.c_int,
                             _vp]),
    ("STS_LSRKStepCreateSTS", _vp, [_vp, C.c_double, _NV, _vp]),
    ("STS_LSRKStepSetSTSMethod", C.c_int, [_vp, C.c_int]),
    ("STS_ARKodeSStolerances", C.c_int, [_vp, C.c_double, C.c_double]),
    ("STS_ARKodeSetUserData", C.c_int, [_vp, _vp]),
    ("STS_LSRKStepSetDomEigFn", C.c_int, [_vp, _vp]),
    ("STS_LSRKStepSetDomEigEstimatorPower", C.c_int, [_vp, C.c_int, C.c_double]),
    ("STS_LSRKStepSetDomEigFrequency", C.c_int, [_vp, _ll]),
    ("STS_LSRKStepSetMaxNumStages", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepSetDomEigSafetyFactor", C.c_int, [_vp, C.c_double]),
    ("STS_ARKodeSetAdaptController", C.c_int, [_vp, C.c_int]),
    ("STS_ARKodeSetFixedStep", C.c_int, [_vp, C.c_double]),
    ("STS_ARKodeSetMaxNumSteps", C.c_int, [_vp, _ll]),
    ("STS_ARKodeSetStopTime", C.c_int, [_vp, C.c_double]),
    ("STS_LSRKStepSetMixedPrecision", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepSetStageKernel", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepGetStageKernelInfo", C.c_int, [_vp, _ip, _dp, C.c_char_p, C.c_int]),
    ("STS_LSRKStepSetStageFusion", C.c_int, [_vp, C.c_int, C.c_int]),
    ("STS_LSRKStepGetStageFusion", C.c_int, [_vp, _ip, _ip, _ip, _dp]),
    ("STS_LSRKStepSetUseGraphs", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepSetFusedPeriodic", C.c_int, [_vp, C.c_int]),
    ("STS_ARKodeEvolve", C.c_int, [_vp, C.c_double, _NV, _dp, C.c_int]),
    ("STS_ARKodeReset", C.c_int, [_vp, C.c_double, _NV]),
    ("STS_LSRKStepTimeStageKernel", C.c_int, [_vp, C.c_int, _dp]),
    ("STS_ARKodeGetStats", C.c_int, [_vp, C.POINTER(Stats)]),
    ("STS_ARKodePrintAllStats", C.c_int, [_vp, C.c_char_p, C.c_int]),
    ("STS_ARKodeFree", None, [C.POINTER(_vp)]),
    ("STS_LSRKStageCoeffs", C.c_int, [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    ("STS_LSRKStagesNeeded", C.c_int, [C.c_int, C.c_double, C.c_double, C.c_int, _dp]),
    ("STS_AdaptControllerEstimate", C.c_double, [C.c_int, C.c_double, C.c_double, C.c_double,
                                                 C.c_double, C.c_double, _ll]),
    ("STS_ManufacturedTables", C.c_int, [_ll, C.c_double, _dp, _dp]),
    ("STS_ExactSumHost", C.c_double, [_dp, _ll]),
    ("STS_SUNLinSol_PCG", _vp, [_NV, C.c_int, C.c_int, _vp]),
    ("STS_SUNLinSolSetATimes", C.c_int, [_vp, _vp, _vp]),
    ("STS_SUNLinSolSetPreconditioner", C.c_int, [_vp, _vp, _vp]),
    ("STS_SUNLinSolSolve", C.c_int, [_vp, _NV, _NV, C.c_double]),
    ("STS_SUNLinSolNumIters", C.c_int, [_vp]),
    ("STS_SUNLinSolResNorm", C.c_double, [_vp]),
    ("STS_SUNLinSolFree", C.c_int, [_vp]),
    ("STS_SUNLinSol_SPGMR", _vp, [_NV, C.c_int, C.c_int, _vp]),
    ("STS_SUNLinSol_SPGMRSetMaxRestarts", C.c_int, [_vp, C.c_int]),
    ("STS_SUNLinSol_SPGMRSetGSType", C.c_int, [_vp, C.c_int]),
    ("STS_SUNLinSol_SPFGMR", _vp, [_NV, C.c_int, C.c_int, _vp]),
    ("STS_SUNLinSol_SPFGMRSetMaxRestarts", C.c_int, [_vp, C.c_int]),
    ("STS_SUNLinSol_SPFGMRSetGSType", C.c_int, [_vp, C.c_int]),
    ("STS_ImplicitSolveLS", C.c_int, [_vp, C.c_double, _vp, C.c_int, _vp, _vp, _NV, _NV,
                                      C.c_double, C.POINTER(C.c_int), _dp]),
    ("STS_NetPrecCreate", C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    ("STS_NetPrecFree", C.c_int, [C.POINTER(_vp)]),
    ("STS_NetPSetup", C.c_int, [C.c_double, _NV, _NV, C.c_int, C.POINTER(C.c_int), C.c_double, _vp]),
    ("STS_NetPSolve", C.c_int, [C.c_double, _NV, _NV, _NV, _NV, C.c_double, C.c_double, C.c_int, _vp]),
    ("STS_NetPrecSolve", C.c_int, [_vp, _NV, _NV, C.c_double, C.c_int]),
    ("STS_PFMGCreate", _vp, [_vp, C.c_int, C.c_int]),
    ("STS_PFMGFree", None, [C.POINTER(_vp)]),
    ("STS_PFMGPSetup", C.c_int, [C.c_double, _NV, _NV, C.c_int, C.POINTER(C.c_int), C.c_double, _vp]),
    ("STS_PFMGPSolve", C.c_int, [C.c_double, _NV, _NV, _NV, _NV, C.c_double, C.c_double, C.c_int, _vp]),
    ("STS_PFMGPrecSolve", C.c_int, [_vp, _NV, _NV, C.c_double, C.c_int]),
    ("STS_PFMGNumLevels", C.c_int, [_vp]),
    ("STS_PFMGNumVCycles", _ll, [_vp]),
    ("STS_ImplicitSolvePFMG", C.c_int, [_vp, C.c_double, _vp, _NV, _NV, C.c_double, C.c_int,
                                        C.POINTER(C.c_int), _dp]),
    ("STS_SDIRK2EvolvePFMG", C.c_int, [_vp, _vp, _NV, C.c_double, C.c_double, C.c_int, C.c_double,
                                       C.c_int, C.POINTER(_ll)]),
    ("STS_SDIRK2EvolveLS", C.c_int, [_vp, _vp, C.c_int, _NV, C.c_double, C.c_double, C.c_int,
                                     C.c_double, C.POINTER(_ll)]),
    ("STS_ImplicitSolvePCG", C.c_int, [_vp, C.c_double, _NV, _NV, C.c_double, C.c_int, C.c_int,
                                       _ip, _dp]),
    ("STS_SDIRK2Evolve", C.c_int, [_vp, _NV, C.c_double, C.c_double, C.c_int, C.c_double,
                                   C.c_int, C.POINTER(_ll)]),
    ("STS_SDIRK2EvolveLearned", C.c_int, [_vp, _vp, _NV, C.c_double, C.c_double, C.c_int,
                                          C.c_double, C.c_int, C.POINTER(_ll)]),
    ("STS_BatchCreate", _vp, [_vp, C.c_int, _ip, _dp, _dp]),
    ("STS_BatchFree", C.c_int, [C.POINTER(_vp)]),
    ("STS_BatchTotalDOF", _ll, [_vp]),
    ("STS_BatchSetState", C.c_int, [_vp, _dp]),
    ("STS_BatchGetState", C.c_int, [_vp, _dp]),
    ("STS_BatchSetInitialModes", C.c_int, [_vp, C.c_int, _ip, _ip, _dp]),
    ("STS_BatchEvolve", C.c_int, [_vp, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                  C.c_int, _ll]),
    ("STS_BatchLastMilliseconds", C.c_double, [_vp]),
    ("STS_BatchGetInstanceStats", C.c_int, [_vp, C.c_int, C.POINTER(Stats)]),
    ("STS_BatchSetLaunch", C.c_int, [_vp, C.c_int, C.c_int]),
    ("STS_BatchSetMixed", C.c_int, [_vp, C.c_int]),
    ("STS_BatchAutotune", C.c_int, [_vp, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                    _ip, _ip, _dp]),
    ("STS_BatchSetCluster", C.c_int, [_vp, C.c_int, C.c_int]),
    ("STS_BatchGetLaunch", C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    ("STS_LSRKStepCreateSSP", _vp, [_vp, C.c_double, _NV, _vp]),
    ("STS_LSRKStepSetSSPMethod", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepSetNumSSPStages", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKSSPWeights", C.c_int, [C.c_int, C.c_int, _dp, _dp, _dp]),
    ("STS_LSRKStepSetNumDomEigEstInitPreprocessIters", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepSetNumDomEigEstPreprocessIters", C.c_int, [_vp, C.c_int]),
    ("STS_LSRKStepWriteCheckpoint", C.c_int, [_vp, C.c_char_p]),
    ("STS_LSRKStepReadCheckpoint", C.c_int, [_vp, C.c_char_p]),
    ("STS_NetCreate", _vp, [_vp, C.c_int, C.c_ulonglong]),
    ("STS_NetFree", C.c_int, [C.POINTER(_vp)]),
    ("STS_NetSetWeights", C.c_int, [_vp, _fp]),
    ("STS_NetGetWeights", C.c_int, [_vp, _fp]),
    ("STS_NetSetTensorPath", C.c_int, [_vp, C.c_int]),
    ("STS_NetSetCollapsedLevel0", C.c_int, [_vp, C.c_int]),
    ("STS_NetApply", C.c_int, [_vp, C.c_int, _vp, _vp, C.c_double, C.c_double, C.c_double,
                               C.c_double]),
    ("STS_NetLossGrad", C.c_int, [_vp, C.c_int, _vp, _vp, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, _dp, _fp]),
    ("STS_NetTrain", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, C.c_float,
                               C.c_ulonglong, _dp]),
    ("STS_HarvestPCGPairs", C.c_int, [_vp, C.c_double, _NV, C.c_int, C.c_int, C.c_int, C.c_int,
                                      _vp, _vp, _vp, C.c_ulonglong, _ip, _ip]),
    ("STS_FCGSolve", C.c_int, [_vp, C.c_double, _vp, _NV, _NV, C.c_double, C.c_int, _ip, _dp]),
    ("STS_ImplicitSolveLearned", C.c_int, [_vp, C.c_double, _vp, _NV, _NV, C.c_double, C.c_int,
                                           C.c_double, _ip, _dp, _ip]),
]

_lib = None
_exiting = False


def _at_exit():
    # At interpreter exit the order in which objects are finalised is arbitrary; a vector
    # finalised after its context would touch freed memory. The process is ending, so the
    # driver reclaims everything: stop freeing from finalisers.
    global _exiting
    _exiting = True


import atexit  # noqa: E402
atexit.register(_at_exit)


def lib(build=True):
    """Load libstsgpu.so (building it first if needed). The environment variable
    STS_LIBRARY_VARIANT=bounds selects the debug-bounds build instead."""
    global _lib
    if _lib is None:
        variant = os.environ.get("STS_LIBRARY_VARIANT", "")
        path = _build.build(variant=variant) if build else _build.lib_path(variant)
        if not os.path.exists(path):
            raise STSError("libstsgpu.so is not built: run __graft_entry__.build()")
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _err(msg):
    e = lib().STS_GetLastError()
    raise STSError("%s: %s" % (msg, e.decode() if e else ""))


def _dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class Context:
    """STS_Context (SUNContext analogue): CUDA stream + reduction workspace of one device."""

    def __init__(self, device=0):
        self.h = _vp()
        self.live = 0  # objects holding C resources of this context
        if lib().STS_ContextCreate(device, C.byref(self.h)) != 0:
            _err("STS_ContextCreate")

    def synchronize(self):
        lib().STS_ContextSynchronize(self.h)

    @property
    def stream(self):
        return lib().STS_ContextGetStream(self.h)

    def wait_self_test(self, arrive, limit=1000):
        """Run the bounded-wait failure path on one pipeline barrier: returns the status
        (0 when the barrier completed, STS_ERR_FAILURE when the wait ran out after `limit`
        polls and the context's error word was read and cleared)."""
        return lib().STS_WaitSelfTest(self.h, int(bool(arrive)), limit)

    def free(self):
        # Garbage collection of reference cycles (for example frames kept by a traceback)
        # may finalise the context before objects that still use it; then it is left for
        # process exit instead of being freed under them.
        if self.h and not _exiting and self.live <= 0:
            lib().STS_ContextFree(C.byref(self.h))
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class NVector:
    """Device N_Vector (owned unless wrapping an existing device pointer)."""

    def __init__(self, ctx, n=None, handle=None, own=True):
        self.ctx = ctx
        if handle is not None:
            self.h = handle
        else:
            self.h = lib().N_VNew_Sts(n, ctx.h)
            if not self.h:
                _err("N_VNew_Sts")
        self.own = own
        if own:
            ctx.live += 1

    @classmethod
    def from_numpy(cls, ctx, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        v = cls(ctx, a.size)
        v.copy_from(a)
        return v

    @classmethod
    def wrap(cls, ctx, handle):
        return cls(ctx, handle=handle, own=False)

    def __len__(self):
        return lib().N_VGetLength_Sts(self.h)

    @property
    def ptr(self):
        return lib().N_VGetDeviceArrayPointer_Sts(self.h)

    def copy_from(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        assert a.size == len(self)
        if lib().N_VCopyFromHost_Sts(self.h, _dptr(a)) != 0:
            _err("N_VCopyFromHost_Sts")

    def numpy(self):
        out = np.empty(len(self))
        if lib().N_VCopyToHost_Sts(self.h, _dptr(out)) != 0:
            _err("N_VCopyToHost_Sts")
        return out

    def clone(self):
        return NVector(self.ctx, handle=lib().N_VClone_Sts(self.h))

    def destroy(self):
        if self.own and self.h and not _exiting:
            lib().N_VDestroy_Sts(self.h)
            self.h = None
            self.ctx.live -= 1

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # ops (N_VLinearSum etc.)
    def linear_sum(self, a, x, b, y):
        lib().N_VLinearSum_Sts(a, x.h, b, y.h, self.h)

    def const(self, c):
        lib().N_VConst_Sts(c, self.h)

    def prod(self, x, y):
        lib().N_VProd_Sts(x.h, y.h, self.h)

    def div(self, x, y):
        lib().N_VDiv_Sts(x.h, y.h, self.h)

    def scale(self, c, x):
        lib().N_VScale_Sts(c, x.h, self.h)

    def abs(self, x):
        lib().N_VAbs_Sts(x.h, self.h)

    def inv(self, x):
        lib().N_VInv_Sts(x.h, self.h)

    def add_const(self, x, b):
        lib().N_VAddConst_Sts(x.h, b, self.h)

    def dot(self, y):
        return lib().N_VDotProd_Sts(self.h, y.h)

    def dot_multi(self, vecs):
        """N_VDotProdMulti: exact dot products with each vector of ``vecs``."""
        n = len(vecs)
        out = (C.c_double * n)()
        X = (_NV * n)(*[v.h for v in vecs])
        if lib().N_VDotProdMulti_Sts(n, self.h, X, out) != 0:
            _err("N_VDotProdMulti_Sts")
        return list(out)

    def max_norm(self):
        return lib().N_VMaxNorm_Sts(self.h)

    def wrms_norm(self, w):
        return lib().N_VWrmsNorm_Sts(self.h, w.h)

    def linear_combination(self, coeffs, vecs):
        n = len(vecs)
        c = (C.c_double * n)(*coeffs)
        X = (_NV * n)(*[v.h for v in vecs])
        if lib().N_VLinearCombination_Sts(n, c, X, self.h) != 0:
            _err("N_VLinearCombination_Sts")


class Problem:
    """The diffusion_2D problem (UserData + RHS/DomEig/PSetup/PSolve callbacks)."""

    def __init__(self, ctx, kind=MANUFACTURED, nx=128, ny=None, kx=1.0, ky=1.0,
                 inhomogeneous=False, xl=-np.pi, xu=np.pi, yl=-6.0, yu=6.0):
        ny = nx if ny is None else ny
        self.ctx, self.nx, self.ny, self.kind = ctx, nx, ny, kind
        self.h = lib().STS_ProblemCreate(ctx.h, kind, nx, ny, kx, ky, int(inhomogeneous), xl, xu,
                                         yl, yu)
        if not self.h:
            _err("STS_ProblemCreate")
        ctx.live += 1

    @property
    def n(self):
        return self.nx * self.ny

    def vector(self):
        v = NVector(self.ctx, self.n)
        lib().N_VSetShape_Sts(v.h, self.nx, self.ny)
        return v

    def initial(self, t=0.0):
        v = self.vector()
        if lib().STS_Initial(t, v.h, self.h) != 0:
            _err("STS_Initial")
        return v

    def initial_modes(self, pm, qm, amp):
        v = self.vector()
        pm = np.ascontiguousarray(pm, dtype=np.int32)
        qm = np.ascontiguousarray(qm, dtype=np.int32)
        amp = np.ascontiguousarray(amp, dtype=np.float64)
        if lib().STS_InitialModes(v.h, self.h, len(amp), pm.ctypes.data_as(_ip),
                                  qm.ctypes.data_as(_ip), _dptr(amp)) != 0:
            _err("STS_InitialModes")
        return v

    def exact(self, t):
        v = self.vector()
        if lib().STS_Exact(t, v.h, self.h) != 0:
            _err("STS_Exact")
        return v

    def rhs(self, t, u, f):
        return lib().STS_Diffusion(t, u.h, f.h, self.h)

    def jac_times(self, v, Jv):
        return lib().STS_JacTimes(v.h, Jv.h, 0.0, None, None, self.h, None)

    def dom_eig(self):
        lr, li = C.c_double(), C.c_double()
        lib().STS_DomEig(0.0, None, None, C.byref(lr), C.byref(li), self.h, None, None, None)
        return lr.value

    def power_iteration(self, v, maxiters=100, reltol=0.01):
        lam, it = C.c_double(), C.c_int()
        if lib().STS_PowerIteration(self.h, v.h, maxiters, reltol, C.byref(lam), C.byref(it)):
            _err("STS_PowerIteration")
        return lam.value, it.value

    def psetup(self, gamma):
        jc = C.c_int()
        return lib().STS_PSetup(0.0, None, None, 0, C.byref(jc), gamma, self.h)

    def psolve(self, r, z, gamma):
        return lib().STS_PSolve(0.0, None, None, r.h, z.h, gamma, 0.0, 2, self.h)

    def free(self):
        if self.h and not _exiting:
            lib().STS_ProblemFree(C.byref(C.c_void_p(self.h)))
            self.h = None
            self.ctx.live -= 1

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class LSRKStep:
    """LSRKStepCreateSTS + ARKode* configuration and evolve (diffusion_2D/main.cpp:257-486).

    ``rhs`` is either a :class:`Problem` (its built-in STS_Diffusion RHS; fused kernels) or a
    Python callable ``f(t, y: NVector, ydot: NVector) -> int`` (generic path).
    ``stage_fusion = (stages per launch, tile configuration)`` sets the mixed form's temporal
    blocking (``STS_LSRKStepSetStageFusion``; (0, 0) autotuned, (1, 0) off)."""

    def __init__(self, ctx, rhs, t0, y0, method=RKC, rtol=1e-6, atol=1e-10, controller=PID,
                 smax=200, mixed=False, graphs=True, dom_eig=None, power=None, maxsteps=100000,
                 hfixed=0.0, stage_kernel=0, dee_warmups=(0, 0), ssp=None, fused_periodic=True,
                 stage_fusion=(0, 0)):
        self.ctx = ctx
        L = lib()
        self._keep = []
        if isinstance(rhs, Problem):
            fn = C.cast(L.STS_Diffusion, _vp)
            ud = rhs.h
            self.problem = rhs
        else:
            def tramp(t, y, ydot, _ud):
                return int(rhs(t, NVector.wrap(ctx, y), NVector.wrap(ctx, ydot)) or 0)
            cb = RHSFN(tramp)
            self._keep.append(cb)
            fn = C.cast(cb, _vp)
            ud = None
            self.problem = None
        if ssp is None:
            self.mem = L.STS_LSRKStepCreateSTS(fn, t0, y0.h, ctx.h)
        else:  # ssp = (type, stages)
            self.mem = L.STS_LSRKStepCreateSSP(fn, t0, y0.h, ctx.h)
        if not self.mem:
            _err("STS_LSRKStepCreate")
        ctx.live += 1
        self.n = len(y0)
        L.STS_ARKodeSetUserData(self.mem, ud)
        if ssp is None:
            L.STS_LSRKStepSetSTSMethod(self.mem, method)
        else:
            if L.STS_LSRKStepSetSSPMethod(self.mem, ssp[0]) != 0 or \
                    L.STS_LSRKStepSetNumSSPStages(self.mem, ssp[1]) != 0:
                _err("STS_LSRKStepSetSSPMethod")
        L.STS_ARKodeSStolerances(self.mem, rtol, atol)
        L.STS_ARKodeSetAdaptController(self.mem, controller)
        L.STS_LSRKStepSetMaxNumStages(self.mem, smax)
        L.STS_LSRKStepSetMixedPrecision(self.mem, int(mixed))
        L.STS_LSRKStepSetUseGraphs(self.mem, int(graphs))
        L.STS_LSRKStepSetFusedPeriodic(self.mem, int(fused_periodic))
        L.STS_LSRKStepSetStageKernel(self.mem, int(stage_kernel))
        if L.STS_LSRKStepSetStageFusion(self.mem, int(stage_fusion[0]), int(stage_fusion[1])) != 0:
            _err("STS_LSRKStepSetStageFusion")
        L.STS_ARKodeSetMaxNumSteps(self.mem, maxsteps)
        L.STS_LSRKStepSetNumDomEigEstInitPreprocessIters(self.mem, int(dee_warmups[0]))
        L.STS_LSRKStepSetNumDomEigEstPreprocessIters(self.mem, int(dee_warmups[1]))
        if hfixed > 0:
            L.STS_ARKodeSetFixedStep(self.mem, hfixed)
        if power is not None:
            L.STS_LSRKStepSetDomEigEstimatorPower(self.mem, power[0], power[1])
        elif dom_eig is not None:
            def dtramp(t, y, fn_, lr, li, _ud, t1, t2, t3):
                lam = dom_eig(t)
                lr[0] = lam
                li[0] = 0.0
                return 0
            cb = DOMEIGFN(dtramp)
            self._keep.append(cb)
            L.STS_LSRKStepSetDomEigFn(self.mem, C.cast(cb, _vp))
        elif isinstance(rhs, Problem):
            L.STS_LSRKStepSetDomEigFn(self.mem, C.cast(L.STS_DomEig, _vp))

    def evolve(self, tout, yout, itask=NORMAL):
        """ARKodeEvolve: returns (tret, flag). NORMAL mode steps past tout (never past a stop
        time) and returns the dense output at tret = tout; a reached stop time returns y_n with
        flag TSTOP_RETURN (1) and is cleared; ONE_STEP returns y_n after one step. Flag
        TOO_MUCH_WORK (-1): the step limit of this call was reached before tout (y_n at tret);
        other negative flags raise."""
        t = C.c_double()
        rc = lib().STS_ARKodeEvolve(self.mem, tout, yout.h, C.byref(t), itask)
        if rc < TOO_MUCH_WORK:
            _err("STS_ARKodeEvolve returned %d" % rc)
        return t.value, rc

    def reset(self, t, y):
        rc = lib().STS_ARKodeReset(self.mem, t, y.h)
        if rc != 0:
            _err("STS_ARKodeReset returned %d" % rc)

    def write_checkpoint(self, path):
        if lib().STS_LSRKStepWriteCheckpoint(self.mem, os.fsencode(path)) != 0:
            _err("STS_LSRKStepWriteCheckpoint")

    def read_checkpoint(self, path):
        if lib().STS_LSRKStepReadCheckpoint(self.mem, os.fsencode(path)) != 0:
            _err("STS_LSRKStepReadCheckpoint")

    def stage_kernel_info(self):
        v, ms = C.c_int(), C.c_double()
        buf = C.create_string_buffer(64)
        lib().STS_LSRKStepGetStageKernelInfo(self.mem, C.byref(v), C.byref(ms), buf, 64)
        return {"variant": v.value, "ms": ms.value, "name": buf.value.decode()}

    def stage_fusion_info(self):
        """Stages per launch in use (1: one launch per stage), the tile configuration (0: none)
        and its rows, and the autotuner's milliseconds per four-stage launch."""
        ks, cfg, rows, ms = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        lib().STS_LSRKStepGetStageFusion(self.mem, C.byref(ks), C.byref(cfg), C.byref(rows), C.byref(ms))
        return {"ks": ks.value, "config": cfg.value, "tile_rows": rows.value, "ms": ms.value}

    def time_stage_kernel(self, nlaunch=20):
        ms = C.c_double()
        if lib().STS_LSRKStepTimeStageKernel(self.mem, nlaunch, C.byref(ms)) != 0:
            _err("STS_LSRKStepTimeStageKernel")
        return ms.value

    def set_stop_time(self, tstop):
        lib().STS_ARKodeSetStopTime(self.mem, tstop)

    def stats(self):
        s = Stats()
        lib().STS_ARKodeGetStats(self.mem, C.byref(s))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def print_stats(self):
        buf = C.create_string_buffer(4096)
        lib().STS_ARKodePrintAllStats(self.mem, buf, 4096)
        return buf.value.decode()

    def free(self):
        if self.mem and not _exiting:
            m = _vp(self.mem)
            lib().STS_ARKodeFree(C.byref(m))
            self.mem = None
            self.ctx.live -= 1

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ARKStep:
    """ARKStepCreate + ARKode* configuration (diffusion_2D/main.cpp:239-330): implicit DIRK
    (``implicit=True``, order 2 or 3) with a Newton iteration whose linear systems go to a
    generic solver (``ls`` "cg" or "gmres", ``maxl`` iterations) preconditioned by nothing
    (``prec=None``), the Jacobi PSetup/PSolve ("jacobi") or a :class:`PFMG` ("pfmg", with
    ``pfmg``); or explicit ERK (order 2, 3 or 4). ``problem`` is a :class:`Problem` (its
    STS_Diffusion RHS)."""

    def __init__(self, ctx, problem, t0, y0, implicit=True, order=2, rtol=1e-5, atol=1e-10,
                 controller=PID, hfixed=0.0, maxsteps=100000, ls="cg", maxl=20, prec="jacobi",
                 pfmg=None, msbp=0, epslin=0.0, linear=False, max_restarts=0, gstype=1):
        L = lib()
        self.ctx = ctx
        self.problem = problem
        self.pfmg = pfmg
        fn = C.cast(L.STS_Diffusion, _vp)
        self.mem = L.STS_ARKStepCreate(None if implicit else fn, fn if implicit else None, t0, y0.h, ctx.h)
        if not self.mem:
            _err("STS_ARKStepCreate")
        ctx.live += 1
        self.n = len(y0)
        self.LS = None
        L.STS_ARKodeSetUserData(self.mem, problem.h)
        if L.STS_ARKodeSetOrder(self.mem, order) != 0:
            _err("STS_ARKodeSetOrder")
        L.STS_ARKodeSStolerances(self.mem, rtol, atol)
        L.STS_ARKodeSetAdaptController(self.mem, controller)
        L.STS_ARKodeSetMaxNumSteps(self.mem, maxsteps)
        if hfixed > 0:
            L.STS_ARKodeSetFixedStep(self.mem, hfixed)
        if implicit:
            pretype = 0 if prec is None else 2  # SUN_PREC_NONE / SUN_PREC_RIGHT
            if ls == "cg":
                self.LS = L.STS_SUNLinSol_PCG(y0.h, pretype, maxl, ctx.h)
            else:
                self.LS = L.STS_SUNLinSol_SPGMR(y0.h, pretype, maxl, ctx.h)
                L.STS_SUNLinSol_SPGMRSetMaxRestarts(self.LS, max_restarts)
                L.STS_SUNLinSol_SPGMRSetGSType(self.LS, gstype)
            L.STS_ARKodeSetLinearSolver(self.mem, self.LS, None)
            if prec == "jacobi":
                L.STS_ARKodeSetPreconditioner(self.mem, C.cast(L.STS_PSetup, _vp), C.cast(L.STS_PSolve, _vp))
            elif prec == "pfmg":
                # PSetup / PSolve of the PFMG object: its handle is the data they receive
                L.STS_ARKStepSetPrecData(self.mem, pfmg.h)
                L.STS_ARKodeSetPreconditioner(self.mem, C.cast(L.STS_PFMGPSetup, _vp),
                                              C.cast(L.STS_PFMGPSolve, _vp))
            L.STS_ARKodeSetLSetupFrequency(self.mem, msbp)
            L.STS_ARKodeSetEpsLin(self.mem, epslin)
            if linear:
                L.STS_ARKodeSetLinear(self.mem, 0)

    def evolve(self, tout, yout, itask=NORMAL):
        """ARKodeEvolve with the return rules of LSRKStep.evolve."""
        t = C.c_double()
        rc = lib().STS_ARKodeEvolve(self.mem, tout, yout.h, C.byref(t), itask)
        if rc < TOO_MUCH_WORK:
            _err("STS_ARKodeEvolve returned %d" % rc)
        return t.value, rc

    def set_stop_time(self, tstop):
        lib().STS_ARKodeSetStopTime(self.mem, tstop)

    def stats(self):
        s = ARKStepStats()
        lib().STS_ARKStepGetStats(self.mem, C.byref(s))
        return {k: getattr(s, k) for k, _ in ARKStepStats._fields_}

    def print_stats(self):
        buf = C.create_string_buffer(4096)
        lib().STS_ARKodePrintAllStats(self.mem, buf, 4096)
        return buf.value.decode()

    def free(self):
        if self.mem and not _exiting:
            m = _vp(self.mem)
            lib().STS_ARKodeFree(C.byref(m))
            self.mem = None
            if self.LS:
                lib().STS_SUNLinSolFree(self.LS)
                self.LS = None
            self.ctx.live -= 1

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def arkstep_table(implicit, order):
    """(A, b, d, c, q, p) of the ARKStep method table"""
    import numpy as np
    s, q, p = C.c_int(), C.c_int(), C.c_int()
    A, b, d, c = np.zeros(25), np.zeros(5), np.zeros(5), np.zeros(5)
    if lib().STS_ARKStepTable(int(implicit), order, C.byref(s), C.byref(q), C.byref(p), _dptr(A), _dptr(b),
                              _dptr(d), _dptr(c)) != 0:
        raise ValueError("no table")
    n = s.value
    return A[:n * n].reshape(n, n), b[:n], d[:n], c[:n], q.value, p.value


class PCGSolver:
    """SUNLinSol_PCG through ATimes / PSolve callbacks (generic path). With ``atimes=None``
    the object is a bare solver for :func:`sdirk2_evolve_ls`, which attaches its own
    callbacks; ``precond`` then selects SUN_PREC_RIGHT."""

    _create = "STS_SUNLinSol_PCG"

    def __init__(self, ctx, y, atimes=None, psolve=None, maxl=100, precond=None):
        L = lib()
        self.ctx = ctx
        pre = bool(psolve) if precond is None else bool(precond)
        self.LS = getattr(L, self._create)(y.h, 2 if pre else 0, maxl, ctx.h)
        if not self.LS:
            _err(self._create)
        ctx.live += 1
        self._keep = []
        if atimes is None:
            return

        def at(_d, v, z):
            return int(atimes(NVector.wrap(ctx, v), NVector.wrap(ctx, z)) or 0)
        cb = ATIMESFN(at)
        self._keep.append(cb)
        L.STS_SUNLinSolSetATimes(self.LS, None, C.cast(cb, _vp))
        if psolve:
            def ps(_d, r, z, tol, lr):
                return int(psolve(NVector.wrap(ctx, r), NVector.wrap(ctx, z)) or 0)
            cb2 = PSOLVEFN(ps)
            self._keep.append(cb2)
            L.STS_SUNLinSolSetPreconditioner(self.LS, None, C.cast(cb2, _vp))

    def solve(self, x, b, delta):
        rc = lib().STS_SUNLinSolSolve(self.LS, x.h, b.h, delta)
        return rc, lib().STS_SUNLinSolNumIters(self.LS), lib().STS_SUNLinSolResNorm(self.LS)

    def __del__(self):
        try:
            if not _exiting and self.LS:
                lib().STS_SUNLinSolFree(self.LS)
                self.LS = None
                self.ctx.live -= 1
        except Exception:
            pass


def implicit_solve_pcg(problem, gamma, b, x, tol=1e-8, maxit=100000, jacobi=True):
    it, rel = C.c_int(), C.c_double()
    rc = lib().STS_ImplicitSolvePCG(problem.h, gamma, b.h, x.h, tol, maxit, int(jacobi),
                                    C.byref(it), C.byref(rel))
    if rc < 0:
        _err("STS_ImplicitSolvePCG")
    return it.value, rel.value, rc


class PFMG:
    """Structured multigrid preconditioner in hypre PFMG's role (preconditioner_hypre.cpp):
    relax 1 = weighted Jacobi, 2 = symmetric red/black Gauss-Seidel; nrelax pre/post sweeps."""

    def __init__(self, problem, relax=2, nrelax=2):
        self.problem = problem
        self.h = lib().STS_PFMGCreate(problem.h, relax, nrelax)
        if not self.h:
            _err("STS_PFMGCreate")

    def setup(self, gamma):
        cur = C.c_int()
        if lib().STS_PFMGPSetup(0.0, None, None, 0, C.byref(cur), gamma, self.h) != 0:
            _err("STS_PFMGPSetup")

    def psolve(self, r, z, gamma):
        if lib().STS_PFMGPSolve(0.0, None, None, r.h, z.h, gamma, 0.0, 2, self.h) != 0:
            _err("STS_PFMGPSolve")

    def levels(self):
        return lib().STS_PFMGNumLevels(self.h)

    def vcycles(self):
        return lib().STS_PFMGNumVCycles(self.h)

    def __del__(self):
        try:
            if not _exiting and self.h:
                h = _vp(self.h)
                lib().STS_PFMGFree(C.byref(h))
                self.h = None
        except Exception:
            pass


def implicit_solve_pfmg(problem, gamma, mg, b, x, tol=1e-8, maxit=100000):
    """(I - gamma A) x = b by CG with the PFMG preconditioner: (iterations, rel. residual, rc)."""
    it, rel = C.c_int(), C.c_double()
    rc = lib().STS_ImplicitSolvePFMG(problem.h, gamma, mg.h, b.h, x.h, tol, maxit, C.byref(it),
                                     C.byref(rel))
    if rc < 0:
        _err("STS_ImplicitSolvePFMG")
    return it.value, rel.value, rc


class SPGMRSolver(PCGSolver):
    """SUNLinSol_SPGMR (restarted GMRES, right preconditioning) through ATimes / PSolve
    callbacks; ``gstype`` 1 = modified, 2 = classical Gram-Schmidt."""

    _create = "STS_SUNLinSol_SPGMR"

    def __init__(self, ctx, y, atimes=None, psolve=None, maxl=20, max_restarts=0, gstype=MODIFIED_GS,
                 precond=None):
        super().__init__(ctx, y, atimes, psolve, maxl, precond)
        L = lib()
        if L.STS_SUNLinSol_SPGMRSetMaxRestarts(self.LS, max_restarts) != 0 or \
                L.STS_SUNLinSol_SPGMRSetGSType(self.LS, gstype) != 0:
            _err("SPGMR options")


class SPFGMRSolver(PCGSolver):
    """SUNLinSol_SPFGMR (flexible restarted GMRES, right preconditioning): the solver for a
    preconditioner that may differ between applications, such as :class:`NetPrec`."""

    _create = "STS_SUNLinSol_SPFGMR"

    def __init__(self, ctx, y, atimes=None, psolve=None, maxl=20, max_restarts=0, gstype=MODIFIED_GS,
                 precond=None):
        super().__init__(ctx, y, atimes, psolve, maxl, precond)
        L = lib()
        if L.STS_SUNLinSol_SPFGMRSetMaxRestarts(self.LS, max_restarts) != 0 or \
                L.STS_SUNLinSol_SPFGMRSetGSType(self.LS, gstype) != 0:
            _err("SPFGMR options")


PREC_NONE, PREC_JACOBI, PREC_USER = 0, 1, 2


def implicit_solve_ls(problem, gamma, solver, b, x, tol=1e-8, prec=PREC_JACOBI, pdata=None,
                      psolve=None):
    """(I - gamma A) x = b with a generic solver object (:class:`PCGSolver`,
    :class:`SPGMRSolver`, :class:`SPFGMRSolver`); ``prec`` PREC_NONE, PREC_JACOBI or PREC_USER
    with ``pdata`` (a handle) and ``psolve`` (a C function pointer, e.g. ``NetPrec.psolve_fn``).
    Returns (status, iterations, residual estimate)."""
    it, rel = C.c_int(), C.c_double()
    rc = lib().STS_ImplicitSolveLS(problem.h, gamma, solver.LS, prec, pdata, psolve, b.h, x.h, tol,
                                   C.byref(it), C.byref(rel))
    if rc < 0:
        _err("STS_ImplicitSolveLS")
    return rc, it.value, rel.value


class NetPrec:
    """The learned network behind the PSetup / PSolve interface (STS_NetPrec) for the generic
    solvers; call :meth:`setup` with gamma before solving."""

    def __init__(self, net, problem):
        self.net, self.problem = net, problem
        self.h = _vp()
        if lib().STS_NetPrecCreate(net.h, problem.h, C.byref(self.h)) != 0:
            _err("STS_NetPrecCreate")
        self.psolve_fn = C.cast(lib().STS_NetPrecSolve, _vp)

    def setup(self, gamma):
        cur = C.c_int()
        if lib().STS_NetPSetup(0.0, None, None, 0, C.byref(cur), gamma, self.h) != 0:
            _err("STS_NetPSetup")

    def psolve(self, r, z, gamma):
        if lib().STS_NetPSolve(0.0, None, None, r.h, z.h, gamma, 0.0, 2, self.h) != 0:
            _err("STS_NetPSolve")

    def __del__(self):
        try:
            if not _exiting and self.h:
                lib().STS_NetPrecFree(C.byref(self.h))
                self.h = None
        except Exception:
            pass


def sdirk2_evolve_ls(problem, solver, y, t0, h, nsteps, tol=1e-10, precond=True):
    """Fixed-step SDIRK2 with the stage systems solved by a generic SUNLinearSolver
    (:class:`PCGSolver` or :class:`SPGMRSolver`); returns the total Krylov iterations."""
    it = _ll()
    rc = lib().STS_SDIRK2EvolveLS(problem.h, solver.LS, int(precond), y.h, t0, h, nsteps, tol,
                                  C.byref(it))
    if rc < 0:
        _err("STS_SDIRK2EvolveLS")
    return it.value


def sdirk2_evolve_pfmg(problem, mg, y, t0, h, nsteps, tol=1e-10, maxit=100000):
    """SDIRK2 steps with CG + the PFMG-role multigrid in every stage solve."""
    it = _ll()
    rc = lib().STS_SDIRK2EvolvePFMG(problem.h, mg.h, y.h, t0, h, nsteps, tol, maxit, C.byref(it))
    if rc < 0:
        _err("STS_SDIRK2EvolvePFMG")
    return it.value


def sdirk2_evolve(problem, y, t0, h, nsteps, tol=1e-10, maxit=100000):
    it = _ll()
    rc = lib().STS_SDIRK2Evolve(problem.h, y.h, t0, h, nsteps, tol, maxit, C.byref(it))
    if rc < 0:
        _err("STS_SDIRK2Evolve")
    return it.value


def sdirk2_evolve_learned(problem, net, y, t0, h, nsteps, tol=1e-10, maxit=100000):
    """SDIRK2 steps with the stage solves by the learned-or-Jacobi shifted solve."""
    it = _ll()
    rc = lib().STS_SDIRK2EvolveLearned(problem.h, net.h, y.h, t0, h, nsteps, tol, maxit, C.byref(it))
    if rc < 0:
        _err("STS_SDIRK2EvolveLearned")
    return it.value


def make_batch_instances(count=512, seed=20261203, sizes=(64, 96, 128, 192, 256, 384, 512),
                         nmodes=8, pmax=16):
    """The batched workload: n uniform from `sizes`, kx, ky log-uniform in [1e-2, 1], initial
    state a sum of `nmodes` sine modes sin(p pi x) sin(q pi y), p, q in [1, pmax], N(0,1)
    amplitudes; numpy's PCG64 generator with the given seed."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        kx = float(10 ** rng.uniform(-2, 0))
        ky = float(10 ** rng.uniform(-2, 0))
        p = rng.integers(1, pmax + 1, nmodes)
        q = rng.integers(1, pmax + 1, nmodes)
        a = rng.standard_normal(nmodes)
        out.append((n, kx, ky, p, q, a))
    return out


class Batch:
    """STS_Batch: independent problems advanced in one persistent launch."""

    def __init__(self, ctx, instances):
        L = lib()
        self.ctx = ctx
        self.instances = instances
        k = len(instances)
        ns = np.array([i[0] for i in instances], dtype=np.int32)
        kx = np.array([i[1] for i in instances], dtype=np.float64)
        ky = np.array([i[2] for i in instances], dtype=np.float64)
        self.h = L.STS_BatchCreate(ctx.h, k, ns.ctypes.data_as(_ip), _dptr(kx), _dptr(ky))
        if not self.h:
            _err("STS_BatchCreate")
        ctx.live += 1
        nm = len(instances[0][3])
        p = np.concatenate([i[3] for i in instances]).astype(np.int32)
        q = np.concatenate([i[4] for i in instances]).astype(np.int32)
        a = np.concatenate([i[5] for i in instances]).astype(np.float64)
        if L.STS_BatchSetInitialModes(self.h, nm, p.ctypes.data_as(_ip), q.ctypes.data_as(_ip),
                                      _dptr(a)) != 0:
            _err("STS_BatchSetInitialModes")
        self.total = L.STS_BatchTotalDOF(self.h)
        self.offsets = np.concatenate([[0], np.cumsum([i[0] ** 2 for i in instances])])

    def set_mixed(self, mixed):
        """FP32 stage increments (True) or FP64 stages (False, the default)."""
        if lib().STS_BatchSetMixed(self.h, int(bool(mixed))) != 0:
            _err("STS_BatchSetMixed")

    def evolve(self, tf, method=RKL, rtol=1e-6, atol=1e-10, smax=200, controller=PID, maxsteps=0):
        rc = lib().STS_BatchEvolve(self.h, tf, method, rtol, atol, smax, controller, maxsteps)
        if rc < 0:
            _err("STS_BatchEvolve returned %d" % rc)
        return lib().STS_BatchLastMilliseconds(self.h)

    def autotune(self, tf_probe, method=RKL, rtol=1e-6, atol=1e-10, smax=200, cache_file=None):
        """Pick the launch shape (threads per instance CTA, CTAs per SM) by timing a short
        probe evolve of each candidate; with `cache_file`, a JSON map from the workload
        signature to the chosen shape is read first and updated after tuning."""
        import json
        key = "n%d_dof%d_m%d_rtol%g_atol%g_smax%d" % (len(self.instances), self.total, method, rtol,
                                                     atol, smax)
        cache = {}
        if cache_file and os.path.exists(cache_file):
            with open(cache_file) as f:
                cache = json.load(f)
            if key in cache:
                th, cp = cache[key]["threads"], cache[key]["ctas_per_sm"]
                self.set_launch(th, cp, cache[key].get("cluster", 1))
                return th, cp, cache[key]["probe_ms"]
        th, cp, ms = C.c_int(), C.c_int(), C.c_double()
        if lib().STS_BatchAutotune(self.h, tf_probe, method, rtol, atol, smax, C.byref(th),
                                   C.byref(cp), C.byref(ms)) != 0:
            _err("STS_BatchAutotune")
        if cache_file:
            cache[key] = {"threads": th.value, "ctas_per_sm": cp.value, "cluster": self.launch()[2],
                          "probe_ms": ms.value}
            with open(cache_file, "w") as f:
                json.dump(cache, f, indent=1, sort_keys=True)
        return th.value, cp.value, ms.value

    def set_launch(self, threads, ctas_per_sm, cluster=None, big_n=256):
        rc = lib().STS_BatchSetLaunch(self.h, threads, ctas_per_sm)
        if rc == 0 and cluster is not None:
            rc = lib().STS_BatchSetCluster(self.h, cluster, big_n)
        return rc

    def launch(self):
        """(threads per CTA, CTAs per SM, cluster size, smallest n on clusters)"""
        v = [C.c_int() for _ in range(4)]
        lib().STS_BatchGetLaunch(self.h, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)

    def state(self):
        out = np.empty(self.total)
        if lib().STS_BatchGetState(self.h, _dptr(out)) != 0:
            _err("STS_BatchGetState")
        return out

    def set_state(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64)
        lib().STS_BatchSetState(self.h, _dptr(y))

    def instance_state(self, y, i):
        n = self.instances[i][0]
        return y[self.offsets[i]:self.offsets[i + 1]]

    def stats(self, i):
        s = Stats()
        lib().STS_BatchGetInstanceStats(self.h, i, C.byref(s))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def free(self):
        if self.h and not _exiting:
            lib().STS_BatchFree(C.byref(_vp(self.h)))
            self.h = None
            self.ctx.live -= 1

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass



# ---------------------------------------------------------------------------------------
# learned multilevel preconditioner
# ---------------------------------------------------------------------------------------
NET_LAYERS = ["W_in", "W_1", "W_2", "W_3"]
NET_WSZ = 16 * 16 * 9


def smooth_field(n, rng, nbumps=24):
    """A seeded random smooth field on the interior grid x_i = (i + 1) / (n + 1): a sum of
    Gaussian bumps with centres uniform in (0.1, 0.9)^2, widths uniform in [0.03, 0.15]
    and N(0, 1) amplitudes (separable, built as outer products)."""
    x = (np.arange(n) + 1.0) / (n + 1)
    f = np.zeros((n, n))
    for _ in range(nbumps):
        cx, cy = rng.uniform(0.1, 0.9, 2)
        w = rng.uniform(0.03, 0.15)
        a = rng.standard_normal()
        f += a * np.outer(np.exp(-(x - cy) ** 2 / (2 * w * w)), np.exp(-(x - cx) ** 2 / (2 * w * w)))
    return f


def net_features(kx, ky, gamma, dx):
    """(sk, sg, jacobi, gcx, gcy) of the shifted system (I - gamma A) on a square grid: the
    normalised anisotropy log10(ky/kx), the normalised log10(gamma/dx^2), the Jacobi factor
    1/(1 - gamma cc) and the scaled stencil weights gamma kx/dx^2, gamma ky/dx^2."""
    cc = -2.0 * (kx + ky) / (dx * dx)
    sk = (np.log10(ky / kx) + 1.5) / 1.5
    sg = np.log10(gamma / (dx * dx)) - 3.6
    return sk, sg, 1.0 / (1.0 - gamma * cc), gamma * kx / (dx * dx), gamma * ky / (dx * dx)


class Net:
    """STS_Net: the learned SPD multilevel preconditioner z = D (r + E^T E r) (BF16
    tensor-core kernels).

    Device arrays are passed as raw device pointers (ints), e.g. ``NVector.ptr`` or a
    ``torch`` CUDA tensor's ``data_ptr()``; the caller orders work on other streams."""

    def __init__(self, ctx, nmax, seed=0):
        self.ctx = ctx
        self.h = lib().STS_NetCreate(ctx.h, nmax, seed)
        if not self.h:
            _err("STS_NetCreate")
        ctx.live += 1
        self.nmax = nmax

    def weights(self):
        """FP32 master weights as a dict name -> (16, 16, 3, 3) array."""
        w = np.empty(len(NET_LAYERS) * NET_WSZ, dtype=np.float32)
        if lib().STS_NetGetWeights(self.h, w.ctypes.data_as(_fp)) != 0:
            _err("STS_NetGetWeights")
        return {nm: w[i * NET_WSZ:(i + 1) * NET_WSZ].reshape(16, 16, 3, 3).copy()
                for i, nm in enumerate(NET_LAYERS)}

    def set_weights(self, W):
        """W: dict name -> array of shape (co, ci, 3, 3) with co, ci <= 16 (zero padded)."""
        w = np.zeros((len(NET_LAYERS), 16, 16, 3, 3), dtype=np.float32)
        for i, nm in enumerate(NET_LAYERS):
            a = np.asarray(W[nm], dtype=np.float32)
            w[i, :a.shape[0], :a.shape[1]] = a
        w = np.ascontiguousarray(w.ravel())
        if lib().STS_NetSetWeights(self.h, w.ctypes.data_as(_fp)) != 0:
            _err("STS_NetSetWeights")

    def set_collapsed_level0(self, on):
        """Inference level 0 collapsed into two kernels (default) or layer by layer."""
        if lib().STS_NetSetCollapsedLevel0(self.h, int(on)) != 0:
            _err("STS_NetSetCollapsedLevel0")

    def set_tensor_path(self, path):
        """Inference convolutions: 0 = mma.sync (default), 1 = tcgen05 + TMEM + TMA."""
        if lib().STS_NetSetTensorPath(self.h, int(path)) != 0:
            _err("STS_NetSetTensorPath")

    def apply(self, n, r_ptr, z_ptr, sk, sg, jacobi, scale=1.0):
        if lib().STS_NetApply(self.h, n, r_ptr, z_ptr, sk, sg, jacobi, scale) != 0:
            _err("STS_NetApply")

    def loss_grad(self, n, r_ptr, e_ptr, sk, sg, jacobi, gcx, gcy):
        loss = C.c_double()
        g = np.empty(len(NET_LAYERS) * NET_WSZ, dtype=np.float32)
        if lib().STS_NetLossGrad(self.h, n, r_ptr, e_ptr, sk, sg, jacobi, gcx, gcy, C.byref(loss),
                                 g.ctypes.data_as(_fp)) != 0:
            _err("STS_NetLossGrad")
        return loss.value, {nm: g[i * NET_WSZ:(i + 1) * NET_WSZ].reshape(16, 16, 3, 3).copy()
                            for i, nm in enumerate(NET_LAYERS)}

    def train(self, n, nsamples, r_ptr, e_ptr, meta_ptr, epochs, batch, lr, seed=0):
        loss = C.c_double()
        if lib().STS_NetTrain(self.h, n, nsamples, r_ptr, e_ptr, meta_ptr, epochs, batch, lr, seed,
                              C.byref(loss)) != 0:
            _err("STS_NetTrain")
        return loss.value

    def free(self):
        if self.h and not _exiting:
            lib().STS_NetFree(C.byref(_vp(self.h)))
            self.h = None
            self.ctx.live -= 1

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def harvest_pcg_pairs(problem, gamma, b, ncrops, crop, every, max_pairs, r_ptr, e_ptr, meta_ptr,
                      seed=0):
    """Run Jacobi-PCG to 1e-10 on (I - gamma A) x = b, recording crop x crop windows of r_k
    and e_k = x* - x_k every `every` batches of 8 iterations (device FP32 buffers of
    max_pairs * crop^2) with their training metadata (7 floats per pair, may be 0).
    Returns (pairs recorded, PCG iterations)."""
    npairs, iters = C.c_int(), C.c_int()
    rc = lib().STS_HarvestPCGPairs(problem.h, gamma, b.h, ncrops, crop, every, max_pairs, r_ptr,
                                   e_ptr, meta_ptr, seed, C.byref(npairs), C.byref(iters))
    if rc < 0:
        _err("STS_HarvestPCGPairs")
    return npairs.value, iters.value


def fcg_solve(problem, gamma, net, b, x, tol=1e-8, maxit=10000):
    """Flexible CG on (I - gamma A) x = b with the network as preconditioner; returns
    (iterations, true relative residual, status): status 0 converged, 2 converged through
    the Jacobi-PCG fallback (after FCG stagnated or broke down), 1 not converged."""
    it, rel = C.c_int(), C.c_double()
    rc = lib().STS_FCGSolve(problem.h, gamma, net.h, b.h, x.h, tol, maxit, C.byref(it),
                            C.byref(rel))
    if rc < 0:
        _err("STS_FCGSolve")
    return it.value, rel.value, rc


def implicit_solve_learned(problem, gamma, net, b, x, tol=1e-8, maxit=20000, kappa_min=0.0):
    """Shifted solve choosing FCG + network (kappa = 1 + 4 gamma (cx + cy) >= kappa_min) or
    Jacobi-PCG; returns (iterations, relative residual, status, used_net)."""
    it, rel, used = C.c_int(), C.c_double(), C.c_int()
    rc = lib().STS_ImplicitSolveLearned(problem.h, gamma, net.h if net else None, b.h, x.h, tol,
                                        maxit, kappa_min, C.byref(it), C.byref(rel), C.byref(used))
    if rc < 0:
        _err("STS_ImplicitSolveLearned")
    return it.value, rel.value, rc, bool(used.value)


def ssp_weights(type_, s):
    """(b, c, w = b - bhat) of an SSP method, as the integrator uses them."""
    b, c, w = np.empty(s), np.empty(s), np.empty(s)
    if lib().STS_LSRKSSPWeights(type_, s, _dptr(b), _dptr(c), _dptr(w)) != 0:
        _err("STS_LSRKSSPWeights")
    return b, c, w
