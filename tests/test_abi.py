"""The C-ABI library loads on a CPU-only host and exports every entry point
that include/tfs_gb300.h declares (no compute call is made without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tfs_gb300.h")


def declared_functions(path=HEADER):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\**\s*\*?\s*(tfs_\w+)\s*\(", text,
                                 flags=re.M)))


def test_header_declares_the_hooks():
    names = declared_functions()
    hooks = ["copy_segment_positions_to_device", "copy_segment_forces_to_device",
             "copy_blob_positions_to_device", "copy_blob_forces_to_device",
             "copy_interparticle_blob_forces_to_host", "copy_blob_velocities_to_host",
             "copy_segment_velocities_to_host", "apply_interparticle_forces", "wait_for_device",
             "evaluate_segment_segment_mobility", "evaluate_segment_blob_mobility",
             "evaluate_blob_blob_mobility", "evaluate_blob_segment_mobility",
             "evaluate_full_mobility"]
    for h in hooks:
        assert "tfs_" + h in names, h
    assert "tfs_solver_create" in names and "tfs_solver_destroy" in names


def test_library_exports_every_declared_symbol():
    from timfilsimmod_gb300 import _native

    if not os.path.exists(_native.lib_path()):
        pytest.skip("libtfs_gb300.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(_native.lib_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers every declared entry point
    assert set(declared_functions()) <= set(_native.exported_symbols())


def test_last_error_and_argument_checks_without_gpu():
    """Argument validation happens before any CUDA call."""
    from timfilsimmod_gb300 import _native as N

    if not os.path.exists(N.lib_path()):
        pytest.skip("libtfs_gb300.so not built")
    lib = N.load()
    cfg = N.Config()
    assert lib.tfs_config_default(ctypes.byref(cfg), 1, 32, 20, 642) == N.TFS_OK
    # END_FORCE_MAGNITUDE with the default DL = 2.6, truncated to int
    assert cfg.end_force_magnitude == int(220.0 * 1800.0 / (2.6 * 2.6 * 400))
    bad = N.Config()
    lib.tfs_config_default(ctypes.byref(bad), 1, 2, 3, 4)
    bad.mu = -1.0
    h = ctypes.c_void_p()
    assert lib.tfs_solver_create(ctypes.byref(bad), ctypes.byref(h)) == N.TFS_EINVAL
    assert b"positive" in lib.tfs_last_error()
    bad.mu = 1.0
    bad.nswim = -1
    assert lib.tfs_solver_create(ctypes.byref(bad), ctypes.byref(h)) == N.TFS_EINVAL
    assert lib.tfs_evaluate_segment_segment_mobility(None) == N.TFS_EINVAL
    assert lib.tfs_wait_for_device(None) == N.TFS_EINVAL
    assert lib.tfs_set_refinement_vectors(None, 0) == N.TFS_EINVAL


def test_stepper_argument_checks_without_gpu():
    """The implicit-step entry points validate handles before any CUDA call."""
    from timfilsimmod_gb300 import _native as N

    if not os.path.exists(N.lib_path()):
        pytest.skip("libtfs_gb300.so not built")
    lib = N.load()
    cfg = N.StepConfig()
    assert lib.tfs_step_config_default(ctypes.byref(cfg), 32, 20) == N.TFS_OK
    assert cfg.tol == 1e-4 and cfg.max_broyden_iter == 400 and cfg.body_q[0] == 1.0
    assert abs(cfg.end_force_magnitude - 220.0 * 1800.0 / (2.6 * 2.6 * 400)) < 1e-12
    h = ctypes.c_void_p()
    assert lib.tfs_stepper_create(None, ctypes.byref(cfg), None, None, ctypes.byref(h)) == N.TFS_EINVAL
    assert b"null" in lib.tfs_last_error()
    assert lib.tfs_stepper_step(None, 0, None, None) == N.TFS_EINVAL
    assert lib.tfs_stepper_destroy(None) == N.TFS_OK
