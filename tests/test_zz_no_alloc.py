"""The allocation-free weighted inner product (nrsg_weighted_inner_prod_f64_noalloc).

It serves callers that cannot call cudaMalloc (device memory owned by another
allocator, or no implicit device synchronisation allowed), so it keeps its
scratch in a fixed array of the library.  Checked through the C ABI against
the allocating entry point nrsg_weighted_inner_prod_f64 on two calls in a row
(the shared scratch keeps the previous call's contents), within the 1e-12
relative tolerance used for the reductions elsewhere.  This file is collected
last so that a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 8192 * 8192


def test_noalloc_matches_allocating_entry_point(product_lib, torch_cuda):
    torch = torch_cuda
    L = product_lib
    vp = ctypes.c_void_p
    L.nrsg_weighted_inner_prod_f64_noalloc.argtypes = [ctypes.c_longlong, vp, vp, vp, vp, vp]
    L.nrsg_weighted_inner_prod_f64.argtypes = [ctypes.c_longlong, vp, vp, vp, vp, vp]
    rng = np.random.default_rng(2026)
    for call, n in enumerate((3_000_017, 3_000_017)):
        w, a, b = (torch.from_numpy(rng.uniform(0.1, 1.0, n)).cuda() for _ in range(3))
        out_na = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        out_ref = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        assert L.nrsg_weighted_inner_prod_f64_noalloc(n, w.data_ptr(), a.data_ptr(), b.data_ptr(),
                                                      out_na.data_ptr(), None) == 0
        assert L.nrsg_weighted_inner_prod_f64(n, w.data_ptr(), a.data_ptr(), b.data_ptr(), out_ref.data_ptr(),
                                              None) == 0
        torch.cuda.synchronize()
        ref = out_ref.item()
        assert abs(out_na.item() - ref) <= 1e-12 * abs(ref), (call, out_na.item(), ref)


def test_noalloc_full_width(product_lib, torch_cuda):
    """n at the scratch limit (8192 x 8192 entries): every one of the 8192 partial-sum slots is written and the
    final reduction runs over all of them; one below the limit leaves the last slot partly filled."""
    torch = torch_cuda
    L = product_lib
    vp = ctypes.c_void_p
    L.nrsg_weighted_inner_prod_f64_noalloc.argtypes = [ctypes.c_longlong, vp, vp, vp, vp, vp]
    L.nrsg_weighted_inner_prod_f64.argtypes = [ctypes.c_longlong, vp, vp, vp, vp, vp]
    g = torch.Generator(device="cuda")
    g.manual_seed(8192)
    w, a, b = (torch.rand(MAX_N, dtype=torch.float64, device="cuda", generator=g) for _ in range(3))
    for n in (MAX_N, MAX_N - 1):
        out_na = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        out_ref = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        assert L.nrsg_weighted_inner_prod_f64_noalloc(n, w.data_ptr(), a.data_ptr(), b.data_ptr(),
                                                      out_na.data_ptr(), None) == 0
        assert L.nrsg_weighted_inner_prod_f64(n, w.data_ptr(), a.data_ptr(), b.data_ptr(), out_ref.data_ptr(),
                                              None) == 0
        torch.cuda.synchronize()
        ref = out_ref.item()
        assert abs(out_na.item() - ref) <= 1e-12 * abs(ref), (n, out_na.item(), ref)
    del w, a, b
    torch.cuda.empty_cache()


def test_noalloc_small_and_unweighted(product_lib, torch_cuda):
    torch = torch_cuda
    L = product_lib
    vp = ctypes.c_void_p
    L.nrsg_weighted_inner_prod_f64_noalloc.argtypes = [ctypes.c_longlong, vp, vp, vp, vp, vp]
    a = torch.arange(1, 101, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert L.nrsg_weighted_inner_prod_f64_noalloc(100, None, a.data_ptr(), None, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert out.item() == float(sum(k * k for k in range(1, 101)))


def test_noalloc_rejects_sizes_beyond_its_scratch(product_lib):
    L = product_lib
    vp = ctypes.c_void_p
    L.nrsg_weighted_inner_prod_f64_noalloc.argtypes = [ctypes.c_longlong, vp, vp, vp, vp, vp]
    L.nrsg_last_error.restype = ctypes.c_char_p
    # rejected before any launch, so the (dummy) pointers are never touched
    assert L.nrsg_weighted_inner_prod_f64_noalloc(MAX_N + 1, None, 16, None, 16, None) == 8
    assert b"exceeds the fixed scratch limit" in L.nrsg_last_error()
