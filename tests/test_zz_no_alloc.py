"""The allocation-free WRMS norm (STS_WrmsNormNoAlloc), called through the C ABI.

This entry point serves callers that cannot allocate GPU or pinned memory when they need a
norm; it keeps its scratch in a fixed device array instead. The test compares it with the
context-based N_VWrmsNorm_Sts on two calls in a row (the second on different data, so a
scratch block left over from the first call would show up), using the exact equality the
other reduction tests use. It lives in its own file, collected last."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_no_alloc_wrms_matches_context_path(ctx, stslib):
    L = stslib.lib()
    out = stslib.NVector(ctx, 1)  # device location for the result
    for call, (n, seed) in enumerate(((1_000_003, 11), (65_537, 12))):
        rng = np.random.default_rng(seed)
        x = rng.standard_normal(n) * np.exp2(rng.integers(-30, 30, size=n))
        w = np.abs(rng.standard_normal(n)) + 0.5
        X = stslib.NVector.from_numpy(ctx, x)
        W = stslib.NVector.from_numpy(ctx, w)
        want = X.wrms_norm(W)
        rc = L.STS_WrmsNormNoAlloc(X.ptr, W.ptr, n, out.ptr, ctx.stream)
        assert rc == 0, L.STS_GetLastError()
        ctx.synchronize()
        got = out.numpy()[0]
        assert got == want, (call, got, want)


def test_no_alloc_rejects_bad_sizes(ctx, stslib):
    L = stslib.lib()
    X = stslib.NVector.from_numpy(ctx, np.ones(4))
    assert L.STS_WrmsNormNoAlloc(X.ptr, X.ptr, 0, X.ptr, ctx.stream) == -1
    assert b"outside" in L.STS_GetLastError()
    assert L.STS_WrmsNormNoAlloc(X.ptr, X.ptr, 2 ** 31, X.ptr, ctx.stream) == -1
    assert b"outside" in L.STS_GetLastError()


CHILD = r'''
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import ceda_demonstrations_gb300 as sts
L = sts.lib()

def once(seed):
    ctx = sts.Context(0)
    rng = np.random.default_rng(seed)
    n = 300_007
    X = sts.NVector.from_numpy(ctx, rng.standard_normal(n))
    W = sts.NVector.from_numpy(ctx, np.abs(rng.standard_normal(n)) + 0.5)
    out = sts.NVector(ctx, 1)
    want = X.wrms_norm(W)
    assert L.STS_WrmsNormNoAlloc(X.ptr, W.ptr, n, out.ptr, ctx.stream) == 0, L.STS_GetLastError()
    ctx.synchronize()
    got = out.numpy()[0]
    for v in (X, W, out):
        v.destroy()
    ctx.free()
    return got == want

assert once(1)
cudart = None
for line in open("/proc/self/maps"):
    if "libcudart.so" in line:
        cudart = ctypes.CDLL(line.split()[-1])
        break
assert cudart is not None
assert cudart.cudaDeviceReset() == 0  # ends this process's context; the next call makes a new one
assert once(2)
print("ok")
'''


def test_no_alloc_after_device_reset(ctx, stslib):
    """A new CUDA context on the same device (here the primary context that follows
    cudaDeviceReset, in a child process so the session's context is untouched) gets its own
    lookup of the scratch address: the entry point still matches the context path."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", CHILD, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
