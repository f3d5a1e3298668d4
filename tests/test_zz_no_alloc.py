"""hgb_dot_f64_noalloc: the dot product for callers that may not allocate device memory (a memory
pool or budget owned by another component, or an integration that cannot create the context
object, which allocates).  It needs no context and keeps its scratch in a static device array.
Checked through the C ABI against the context entry point hgb_dot_f64 and against an FP64 numpy
dot, on calls in a row that share the static scratch, at n = 0 and at the size limit.  Collected
last on purpose (a failure here stops a -x run only after every other test has run)."""
import ctypes as C

import numpy as np
import pytest
import torch

from hala_gb300 import build, hgb

pytestmark = pytest.mark.gpu

LIMIT = 2048 * 16384   # entries the static scratch holds (one partial sum per 2048)


def _noalloc(L, x, y, out, stream):
    hgb.check(L.hgb_dot_f64_noalloc(int(x.numel()), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                    C.c_void_p(out.data_ptr()), stream), "dot_f64_noalloc")


def test_noalloc_dot_matches_context_dot_and_numpy():
    build.build()
    L = hgb.lib()
    dev = torch.device("cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ctx = C.c_void_p()
    hgb.check(L.hgb_ctx_create(0, C.byref(ctx)))
    rng = np.random.default_rng(21)
    try:
        # calls in a row sharing the static scratch: large, small, empty, at the limit, large again
        for n in (1_000_003, 4097, 0, LIMIT, 1_000_003):
            xh, yh = rng.standard_normal(n), rng.standard_normal(n)
            x, y = torch.from_numpy(xh).to(dev), torch.from_numpy(yh).to(dev)
            out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
            _noalloc(L, x, y, out, stream)
            torch.cuda.synchronize()
            got = out.item()
            if n == 0:
                assert got == 0.0
                continue
            ref = C.c_double()
            hgb.check(L.hgb_dot_f64(ctx, n, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.byref(ref), 0))
            # reductions are compared within 1e-13 relative, as for the other dot products
            assert abs(got - ref.value) <= 1e-13 * abs(ref.value) + 1e-13
            # FP64 numpy dot: a different summation order, so the bound scales with sum |x_i y_i|
            assert abs(got - float(np.dot(xh, yh))) <= 1e-13 * float(np.sum(np.abs(xh * yh)))
            del x, y
        # sizes beyond the static scratch are rejected before any launch
        z = torch.zeros(1, dtype=torch.float64, device=dev)
        out = torch.full((1,), 7.0, dtype=torch.float64, device=dev)
        st = L.hgb_dot_f64_noalloc(LIMIT + 1, C.c_void_p(z.data_ptr()), C.c_void_p(z.data_ptr()),
                                   C.c_void_p(out.data_ptr()), stream)
        assert st == hgb.HGB_ERR_ARG and b"static scratch" in L.hgb_last_error()
        torch.cuda.synchronize()
        assert out.item() == 7.0
    finally:
        L.hgb_ctx_destroy(ctx)
