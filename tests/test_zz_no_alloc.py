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
