"""pf_sizer_predict_noalloc: the sizer's prediction without any device allocation.

Callers that cannot call cudaMalloc (a render loop that must not stall the device, GPU memory
owned by another allocator) use this entry point;
it stages its data in a fixed device array of the library instead of context buffers.  The
test calls it through the C-ABI twice in a row and checks it against pf_sizer_predict, the
allocating entry point, with the tolerance of the other sizer-prediction test; it also checks
that a request above the array's limit is refused with a clear error.  It creates its own
context so it passes alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 16384


def _noalloc(lib, ctx, x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.full((x.shape[0], 2), np.nan, np.float32)
    st = lib.pf_sizer_predict_noalloc(ctx, C.c_void_p(x.ctypes.data), C.c_uint32(x.shape[0]),
                                      C.c_void_p(out.ctypes.data))
    return st, out


def test_noalloc_prediction_matches_allocating_entry_point(pf):
    import os
    r = pf.Renderer()
    try:
        if os.path.exists(pf.DEFAULT_WEIGHTS):
            r.sizer_load(pf.DEFAULT_WEIGHTS)
        else:
            r.sizer_init(seed=11)
        rng = np.random.default_rng(5)
        for call, n in enumerate((5000, 1234)):  # two calls in a row, the second smaller
            x = np.abs(rng.normal(3.0, 1.5, (n, 12))).astype(np.float32)
            want = r.sizer_predict(x)
            st, got = _noalloc(r.lib, r.ctx, x)
            assert st == 0, r.lib.pf_last_error(r.ctx)
            assert np.all(np.isfinite(got)), call
            assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max() + 1e-5, call
        st, _ = _noalloc(r.lib, r.ctx, np.zeros((LIMIT + 1, 12), np.float32))
        assert st == 1
        assert b"limit" in r.lib.pf_last_error(r.ctx)
    finally:
        r.close()
