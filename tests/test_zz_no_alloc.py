"""hgb_dot_f64_noalloc: the dot product for callers that may not allocate device memory (it needs
no context and keeps its scratch in a static device array) against the context entry point
hgb_dot_f64, through the C ABI, on two calls in a row.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest
import torch

from hala_gb300 import build, hgb

pytestmark = pytest.mark.gpu


def test_noalloc_dot_matches_context_dot():
    build.build()
    L = hgb.lib()
    dev = torch.device("cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ctx = C.c_void_p()
    hgb.check(L.hgb_ctx_create(0, C.byref(ctx)))
    rng = np.random.default_rng(21)
    try:
        for n in (1_000_003, 4097):      # two calls in a row, sharing the static scratch
            x = torch.from_numpy(rng.standard_normal(n)).to(dev)
            y = torch.from_numpy(rng.standard_normal(n)).to(dev)
            out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
            hgb.check(L.hgb_dot_f64_noalloc(n, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                            C.c_void_p(out.data_ptr()), stream), "dot_f64_noalloc")
            torch.cuda.synchronize()
            ref = C.c_double()
            hgb.check(L.hgb_dot_f64(ctx, n, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.byref(ref), 0))
            # reductions are compared within 1e-13 relative, as for the other dot products
            assert abs(out.item() - ref.value) <= 1e-13 * abs(ref.value) + 1e-13
        # sizes beyond the static scratch are rejected before any launch
        too_big = 2048 * 16384 + 1
        st = L.hgb_dot_f64_noalloc(too_big, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                   C.c_void_p(out.data_ptr()), stream)
        assert st == hgb.HGB_ERR_ARG and b"static scratch" in L.hgb_last_error()
    finally:
        L.hgb_ctx_destroy(ctx)
