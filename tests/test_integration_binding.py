"""The binding a maintainer of the reference adds (timfilsimmod_gb300/integration:
a replacement rpy_mobility_solver.cu for the 17 hooks, the device-resident
compute_velocities and make_body_reference_matrices of mobility_solver, and
flow_field_evaluator::velocities; for the prescribed-cilia configuration, the
weakly coupled solver class and the prescribed-cilia compute_velocities)
compiles against the reference's unchanged
headers (rpy_mobility_solver.hpp, mobility_solver.hpp, swimmer.hpp,
flow_field_evaluator.hpp) with Real = double and with the shipped
Real = float, and links against libtfs_gb300.so: every library symbol the
binding calls is exported, the float build through the float entry points.

Needs the reference tree (this machine; skipped elsewhere) and nvcc; no GPU.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INTEG = os.path.join(ROOT, "timfilsimmod_gb300", "integration")
LIB = os.path.join(ROOT, "timfilsimmod_gb300", "libtfs_gb300.so")


def reference_tree():
    import sys

    sys.path.insert(0, ROOT)
    import __graft_entry__

    return __graft_entry__.REFERENCE_TREE


def symbols(path, defined):
    flag = "--defined-only" if defined else "--undefined-only"
    out = subprocess.run(["nm", "-D", flag, path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.split() and ln.split()[-1].startswith("tfs_")}


@pytest.fixture(scope="module")
def bindings():
    ref = reference_tree()
    if not os.path.isdir(os.path.join(ref, "src", "cilia", "mobility")):
        pytest.skip("the reference tree is not on this machine")
    if shutil.which("nvcc") is None or not os.path.exists(LIB):
        pytest.skip("needs nvcc and the built libtfs_gb300.so")
    res = subprocess.run(["make", "-C", INTEG, "check", f"REF={ref}"], capture_output=True,
                         text=True)
    assert res.returncode == 0, res.stdout[-3000:] + res.stderr[-3000:]
    return {c: os.path.join(INTEG, "_build", f"binding_{c}.so")
            for c in ("fp64", "fp32", "pres_fp64", "pres_fp32")}


def test_binding_compiles_and_links_in_both_precisions(bindings):
    exported = symbols(LIB, defined=True)
    for cfg, path in bindings.items():
        needed = symbols(path, defined=False)
        assert needed, cfg
        assert needed <= exported, (cfg, sorted(needed - exported))


def test_float_build_uses_the_float_entry_points(bindings):
    f64 = symbols(bindings["fp64"], defined=False)
    f32 = symbols(bindings["fp32"], defined=False)
    hooks = ["tfs_copy_segment_positions_to_device", "tfs_copy_segment_forces_to_device",
             "tfs_copy_blob_positions_to_device", "tfs_copy_blob_forces_to_device",
             "tfs_copy_interparticle_blob_forces_to_host", "tfs_copy_blob_velocities_to_host",
             "tfs_copy_segment_velocities_to_host", "tfs_copy_blob_forces_to_host"]
    for h in hooks:
        assert h in f64 and h + "_f32" not in f64, h
        assert h + "_f32" in f32 and h not in f32, h


def test_prescribed_binding_calls_the_prescribed_solve(bindings):
    """The prescribed-cilia build (the shipped CILIA_TYPE 3 branches with the
    weakly coupled mobility) binds compute_velocities to tfs_prescribed_* and
    the weakly coupled class's segment product to its library call."""
    for cfg in ("pres_fp64", "pres_fp32"):
        need = symbols(bindings[cfg], defined=False)
        for name in ("tfs_prescribed_setup", "tfs_prescribed_compute_velocities",
                     "tfs_prescribed_solution", "tfs_evaluate_weakly_coupled_segment_mobility"):
            assert name in need, (cfg, name)
    assert "tfs_copy_segment_positions_to_device_f32" in symbols(bindings["pres_fp32"], False)
