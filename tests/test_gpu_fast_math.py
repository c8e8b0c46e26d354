"""The FP64 reciprocal the fused FP64 kernels use in place of IEEE division
(rcp.approx seed + two Newton-Raphson steps) against CUDA's correctly rounded
1/x over many binades, and the packed FP32 (FFMA2) rate probe."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulps(a, b):
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    return np.abs(ia - ib)


def test_fast_reciprocal_within_one_ulp():
    import torch
    import ocfd
    L = ocfd.load()
    rng = np.random.default_rng(5)
    # magnitudes the kernels feed it: eps + smoothness indicators, densities,
    # products of squared indicators (1e-6 .. 1e150), both mantissa ends
    x = np.concatenate([10.0 ** rng.uniform(-12, 150, 400000), rng.uniform(1.0, 2.0, 100000),
                        np.nextafter(np.array([1.0, 2.0, 4.0, 1e-6]), np.inf),
                        np.nextafter(np.array([2.0, 4.0, 8.0, 1e-6]), 0.0)])
    xt = torch.from_numpy(x).cuda()
    fast = torch.empty_like(xt)
    ieee = torch.empty_like(xt)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ocfd.check(L.ocfd_check_rcp_f64(ctypes.c_void_p(xt.data_ptr()), ctypes.c_void_p(fast.data_ptr()),
                                    ctypes.c_void_p(ieee.data_ptr()), x.size, stream), "ocfd_check_rcp_f64")
    torch.cuda.synchronize()
    f, r = fast.cpu().numpy(), ieee.cpu().numpy()
    assert np.array_equal(r, 1.0 / x)          # CUDA's 1/x is the correctly rounded host value
    assert ulps(f, r).max() <= 1
    assert np.mean(f == r) > 0.9


def test_ffma2_peak_measured():
    import ocfd
    L = ocfd.load()
    v2, v64, v32 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    ocfd.check(L.ocfd_measure_ffma2_peak(ctypes.byref(v2)), "ocfd_measure_ffma2_peak")
    ocfd.check(L.ocfd_measure_fma_peaks(ctypes.byref(v64), ctypes.byref(v32)), "ocfd_measure_fma_peaks")
    print("FP64 %.0f  FP32 %.0f  FP32x2 %.0f GFLOP/s" % (v64.value, v32.value, v2.value))
    assert v2.value > 0 and v32.value > 0 and v64.value > 0
