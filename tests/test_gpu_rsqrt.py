"""Accuracy of the FP64 reciprocal square root of far-field separations
(rsqrt_far: an FP32 hardware seed refined by one third-order Householder
step, 5 FP64 operations; the FP64 pair kernels use it for every far pair)
over r^2 in [4, 1e12] -- touching particles out to separations of 1e6 radii
-- against a host reference in extended or quadruple precision
(numpy.longdouble) and against CUDA's FP64 rsqrt on the same inputs.

Bar: at most 2 ulp (units in the last place of the double result) from the
reference; measured about 1. The reference pair function takes
1/(sqrt(r^2) + 1e-20) (cuda_functions.cu:212-213), itself up to ~1.5 ulp
from the exact value.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_rsqrt_far_within_two_ulp():
    import torch

    from timfilsimmod_gb300 import _native as N

    lib = N.load()
    rng = np.random.default_rng(2024)
    n = 1 << 20
    x = np.exp(rng.uniform(np.log(4.0), np.log(1e12), size=n))
    x[:4] = [4.0, 4.0 * (1 + 2 ** -52), 1e12, 7.0]  # ends of the range and an odd value
    dev = torch.device("cuda", 0)
    xd = torch.tensor(x, dtype=torch.float64, device=dev)
    yd = torch.empty_like(xd)
    st = torch.cuda.current_stream(dev)
    rc = lib.tfs_rsqrt_far(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()), n,
                           ctypes.c_void_p(st.cuda_stream))
    assert rc == N.TFS_OK, lib.tfs_last_error()
    cuda_rsqrt = torch.rsqrt(xd).cpu().numpy()
    y = yd.cpu().numpy()
    ref = 1 / np.sqrt(x.astype(np.longdouble))
    ulp = np.spacing(ref.astype(np.float64))
    err = np.abs(y.astype(np.longdouble) - ref) / ulp
    err_cuda = np.abs(cuda_rsqrt.astype(np.longdouble) - ref) / ulp
    print(f"\nrsqrt_far: max {float(err.max()):.3f} ulp, mean {float(err.mean()):.3f}; "
          f"CUDA rsqrt: max {float(err_cuda.max()):.3f} ulp; "
          f"identical to CUDA's on {np.mean(y == cuda_rsqrt):.1%}")
    assert np.isfinite(y).all()
    assert float(err.max()) <= 2.0
