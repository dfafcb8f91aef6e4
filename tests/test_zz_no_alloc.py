"""tfs_mss_noalloc: the segment-segment product for callers that cannot
allocate device memory (their working memory is a fixed file-scope device
array inside the library), called through the C ABI and compared with the
solver entry point tfs_evaluate_segment_segment_mobility on two calls in a
row, at the FP64 parity tolerance of the other GPU tests (1e-12 relative).

This file is collected last on purpose (test_zz_*): it runs after every
other test, and it also passes on its own in a fresh process.
"""
import ctypes
import os

import numpy as np
import pytest

TOL64 = 1e-12
GOLD = os.path.join(os.path.dirname(__file__), "golden")

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("config", ["small", "medium"])
def test_noalloc_matches_solver_entry_point_twice(config):
    """The small swimmer (640 segments) and the medium one (12 800 segments,
    TFS_NOALLOC_MAX_SEGS: the record and partial-sum regions of the array
    filled to their ends)."""
    import torch

    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.geometry import make_config
    from timfilsimmod_gb300.mobility import RpyMobilitySolver

    lib = N.load()
    sw = make_config(config, seed=12)
    rng = np.random.default_rng(4)
    forces = [sw.f_segs, rng.normal(size=sw.f_segs.shape)]
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    x = torch.tensor(sw.x_segs.ravel(), dtype=torch.float64, device=dev)
    v = torch.empty(6 * sw.num_segs, dtype=torch.float64, device=dev)
    solver = RpyMobilitySolver(1, sw.nfil, sw.nseg, sw.num_blobs, precision="fp64")
    for call, fs in enumerate(forces):
        # the existing entry point
        solver.set_state(sw.x_segs, fs, sw.x_blobs, sw.f_blobs)
        solver.evaluate_segment_segment_mobility()
        solver.copy_segment_velocities_to_host()
        solver.wait_for_device()
        want = solver.v_segs_host.copy()
        # the no-allocation entry point on caller-owned device arrays
        f = torch.tensor(np.asarray(fs).ravel(), dtype=torch.float64, device=dev)
        v.fill_(float("nan"))
        rc = lib.tfs_mss_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                                 ctypes.c_void_p(v.data_ptr()), sw.num_segs, 1.0, 1.0,
                                 ctypes.c_void_p(stream.cuda_stream))
        assert rc == N.TFS_OK, lib.tfs_last_error()
        torch.cuda.synchronize(dev)
        got = v.cpu().numpy()
        assert np.isfinite(got).all()
        err = rel_max(got, want)
        print(f"call {call}: rel err {err:.2e}")
        assert err < TOL64
    solver.finalise()


def test_noalloc_no_segments_is_ok():
    from timfilsimmod_gb300 import _native as N

    lib = N.load()
    assert lib.tfs_mss_noalloc(None, None, None, 0, 1.0, 1.0, None) == N.TFS_OK


def test_noalloc_rejects_oversize():
    from timfilsimmod_gb300 import _native as N

    lib = N.load()
    n = N.load().tfs_mss_noalloc  # noqa: F841 - the symbol is exported
    rc = lib.tfs_mss_noalloc(None, None, None, 12801, 1.0, 1.0, None)
    assert rc == N.TFS_EINVAL
    assert b"no-allocation limit" in lib.tfs_last_error()
