"""ctypes binding of libtfs_gb300.so (the C ABI in include/tfs_gb300.h).

There is no CPU fallback: if the library is missing or does not load, every
entry point raises. Build it with `python -m timfilsimmod_gb300.build` or
`__graft_entry__.build()`.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

TFS_OK = 0
TFS_EINVAL = -1
TFS_ENOMEM = -2
TFS_ECUDA = -3
TFS_ENOTCONV = -4
TFS_ENAN = -5
TFS_ETIMEOUT = -6
TFS_ESTATE = -7

TFS_FP64 = 0
TFS_FP32C = 1

_STATUS = {TFS_EINVAL: "EINVAL", TFS_ENOMEM: "ENOMEM", TFS_ECUDA: "ECUDA",
           TFS_ENOTCONV: "ENOTCONV", TFS_ENAN: "ENAN", TFS_ETIMEOUT: "ETIMEOUT",
           TFS_ESTATE: "ESTATE"}


class TfsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{_STATUS.get(code, code)}: {message}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("nswim", ctypes.c_int), ("nfil", ctypes.c_int), ("nseg", ctypes.c_int),
                ("nblob", ctypes.c_int), ("mu", ctypes.c_double), ("a_seg", ctypes.c_double),
                ("a_blob", ctypes.c_double), ("end_force_magnitude", ctypes.c_int),
                ("repulsive_force_factor", ctypes.c_double), ("free_body", ctypes.c_int),
                ("precision", ctypes.c_int)]


class DeviceBuffers(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("x_segs", "f_segs", "v_segs", "x_blobs",
                                                "f_blobs", "v_blobs", "f_blobs_repulsion")]


class StepConfig(ctypes.Structure):
    _fields_ = [("nfil", ctypes.c_int), ("nseg", ctypes.c_int), ("seg_sep", ctypes.c_double),
                ("dt", ctypes.c_double), ("tol", ctypes.c_double),
                ("max_broyden_iter", ctypes.c_int), ("kb", ctypes.c_double),
                ("kt", ctypes.c_double), ("end_force_magnitude", ctypes.c_double),
                ("jacobian_confidence", ctypes.c_double), ("body_radius", ctypes.c_double),
                ("perturb_first_step", ctypes.c_int), ("body_x", ctypes.c_double * 3),
                ("body_q", ctypes.c_double * 4)]


class PrescribedConfig(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_int), ("gen_force_magnitude_factor", ctypes.c_double),
                ("torsional_spring_magnitude_factor", ctypes.c_double),
                ("fil_length", ctypes.c_double)]


class PrescribedKinematics(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("vel_dir_phase", "vel_dir_angle", "phase",
                                                "omega0", "shape_rotation_angle", "phase_dot",
                                                "v_body")]


TFS_PRESCRIBED_BODY = 1
TFS_DYNAMIC_PHASE = 2
TFS_DYNAMIC_ANGLE = 4
TFS_WEAKLY_COUPLED = 8


class Request(ctypes.Structure):
    _fields_ = [("nfil", ctypes.c_int), ("nseg", ctypes.c_int), ("nblob", ctypes.c_int),
                ("blob_refs", ctypes.c_void_p), ("fil_refs", ctypes.c_void_p),
                ("fil_dirs", ctypes.c_void_p), ("body_radius", ctypes.c_double),
                ("seg_rotation", ctypes.c_void_p),
                ("num_steps", ctypes.c_int), ("x_out", ctypes.c_void_p),
                ("body_out", ctypes.c_void_p), ("q_out", ctypes.c_void_p)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("num_workers", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t),
                ("precision", ctypes.c_int), ("linear_tol", ctypes.c_double),
                ("step", StepConfig), ("max_bypass_ms", ctypes.c_double)]


class ServerCounters(ctypes.Structure):
    _fields_ = [(n, ctypes.c_longlong) for n in ("resident_instances", "created", "reused",
                                                  "evicted", "queued", "inflight")] + \
               [("bytes_in_use", ctypes.c_size_t), ("bypassed", ctypes.c_longlong)]


_P = ctypes.c_void_p
_H = ctypes.c_void_p  # opaque handle
_IP = ctypes.POINTER(ctypes.c_int)
_LLP = ctypes.POINTER(ctypes.c_longlong)

# name -> argument types (all return int unless listed in _RESTYPES)
_SIGNATURES = {
    "tfs_config_default": [ctypes.POINTER(Config), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                           ctypes.c_int],
    "tfs_solver_create": [ctypes.POINTER(Config), ctypes.POINTER(_H)],
    "tfs_solver_destroy": [_H],
    "tfs_solver_set_stream": [_H, _P],
    "tfs_solver_set_precision": [_H, ctypes.c_int],
    "tfs_solver_device_buffers": [_H, ctypes.POINTER(DeviceBuffers)],
    "tfs_solver_positions_updated": [_H],
    "tfs_copy_segment_positions_to_device": [_H, _P],
    "tfs_copy_segment_forces_to_device": [_H, _P],
    "tfs_copy_blob_positions_to_device": [_H, _P],
    "tfs_copy_blob_forces_to_device": [_H, _P],
    "tfs_copy_interparticle_blob_forces_to_host": [_H, _P],
    "tfs_copy_blob_velocities_to_host": [_H, _P],
    "tfs_copy_segment_velocities_to_host": [_H, _P],
    "tfs_apply_interparticle_forces": [_H],
    "tfs_wait_for_device": [_H],
    "tfs_evaluate_segment_segment_mobility": [_H],
    "tfs_evaluate_segment_blob_mobility": [_H],
    "tfs_evaluate_blob_blob_mobility": [_H],
    "tfs_evaluate_blob_blob_mobility_ff": [_H],
    "tfs_evaluate_weakly_coupled_segment_mobility": [_H],
    "tfs_evaluate_blob_segment_mobility": [_H],
    "tfs_evaluate_full_mobility": [_H, _P, _P],
    "tfs_apply_grand_mobility": [_H],
    "tfs_set_blob_references": [_H, _P],
    "tfs_set_body_pose": [_H, _P, _P],
    "tfs_set_linear_solver": [_H, ctypes.c_double, ctypes.c_int],
    "tfs_set_refinement": [_H, ctypes.c_double, ctypes.c_int],
    "tfs_set_refinement_vectors": [_H, ctypes.c_int],
    "tfs_set_persistent_gmres": [_H, ctypes.c_int],
    "tfs_inject_barrier_stall": [_H, ctypes.c_int],
    "tfs_make_body_reference_matrices": [_H],
    "tfs_get_body_reference_matrices": [_H, _P, _P],
    "tfs_set_body_reference_matrices": [_H, _P, _P],
    "tfs_compute_velocities": [_H, _P, ctypes.POINTER(ctypes.c_int)],
    "tfs_solve_linear_system": [_H, _P, ctypes.POINTER(ctypes.c_int)],
    "tfs_get_body_velocities": [_H, _P],
    "tfs_set_body_velocities": [_H, _P],
    "tfs_copy_blob_forces_to_host": [_H, _P],
    "tfs_refinement_retries": [_H, ctypes.POINTER(ctypes.c_longlong)],
    "tfs_prescribed_config_default": [ctypes.POINTER(PrescribedConfig), ctypes.c_int,
                                      ctypes.c_int, ctypes.c_double],
    "tfs_prescribed_setup": [_H, ctypes.POINTER(PrescribedConfig), _P, ctypes.c_int, _P,
                             ctypes.c_int],
    "tfs_prescribed_set_kinematics": [_H, ctypes.POINTER(PrescribedKinematics)],
    "tfs_prescribed_solve": [_H, _IP],
    "tfs_prescribed_compute_velocities": [_H, ctypes.POINTER(PrescribedKinematics), _IP],
    "tfs_prescribed_apply": [_H, ctypes.c_int, _P, _P],
    "tfs_prescribed_size": [_H, _IP],
    "tfs_prescribed_precon_matrix": [_H, _P],
    "tfs_prescribed_solution": [_H, _P, _P, _P, _P, _P],
    "tfs_prescribed_set_solution": [_H, _P, _P, _P, _P, _P],
    "tfs_solve_info": [_H, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                       ctypes.POINTER(ctypes.c_double)],
    "tfs_solver_enable_kernel_timing": [_H, ctypes.c_int],
    "tfs_solver_kernel_timing": [_H, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_int)],
    "tfs_solver_autotune": [_H, ctypes.c_int, ctypes.c_int],
    "tfs_solver_tuning_report": [_H, ctypes.c_char_p, ctypes.c_size_t,
                                 ctypes.POINTER(ctypes.c_size_t)],
    "tfs_solver_set_tuning": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "tfs_num_tile_variants": [ctypes.c_int],
    "tfs_solver_set_queue_variant": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "tfs_num_queue_variants": [ctypes.c_int],
    "tfs_flow_create": [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                        ctypes.POINTER(_H)],
    "tfs_flow_destroy": [_H],
    "tfs_flow_set_stream": [_H, _P],
    "tfs_flow_copy_inputs_to_device": [_H, _P, _P, _P, _P, _P, _P],
    "tfs_flow_velocities": [_H, ctypes.c_double, ctypes.c_int],
    "tfs_flow_copy_velocities_to_host": [_H, _P],
    "tfs_flow_device_buffers": [_H, ctypes.POINTER(_P), ctypes.POINTER(_P)],
    "tfs_flow_wait": [_H],
    "tfs_flow_num_variants": [ctypes.c_int],
    "tfs_flow_set_variant": [_H, ctypes.c_int],
    "tfs_flow_autotune": [_H, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                          ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)],
    "tfs_mss_noalloc": [_P, _P, _P, ctypes.c_int, ctypes.c_double, ctypes.c_double, _P],
    "tfs_rsqrt_far": [_P, _P, ctypes.c_int, _P],
    "tfs_pg_trace": [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "tfs_copy_segment_positions_to_device_f32": [_H, _P],
    "tfs_copy_segment_forces_to_device_f32": [_H, _P],
    "tfs_copy_blob_positions_to_device_f32": [_H, _P],
    "tfs_copy_blob_forces_to_device_f32": [_H, _P],
    "tfs_copy_interparticle_blob_forces_to_host_f32": [_H, _P],
    "tfs_copy_blob_velocities_to_host_f32": [_H, _P],
    "tfs_copy_segment_velocities_to_host_f32": [_H, _P],
    "tfs_copy_blob_forces_to_host_f32": [_H, _P],
    "tfs_step_config_default": [ctypes.POINTER(StepConfig), ctypes.c_int, ctypes.c_int],
    "tfs_stepper_create": [_H, ctypes.POINTER(StepConfig), _P, _P, ctypes.POINTER(_H)],
    "tfs_stepper_destroy": [_H],
    "tfs_stepper_step": [_H, ctypes.c_int, _IP, _IP],
    "tfs_stepper_initial_guess": [_H, ctypes.c_int],
    "tfs_stepper_forces": [_H, ctypes.c_int, _P],
    "tfs_stepper_compute_velocities": [_H, ctypes.c_int, _IP],
    "tfs_stepper_compute_errors": [_H, ctypes.c_int, ctypes.c_int, _P, _IP],
    "tfs_stepper_prepare_jacobian_inv": [_H, ctypes.c_int, _P],
    "tfs_stepper_inverse_jacobian": [_H, ctypes.c_int, _P],
    "tfs_stepper_jacobian_inv_mult": [_H, ctypes.c_int, _P, _P],
    "tfs_stepper_broyden_reset": [_H],
    "tfs_stepper_find_update": [_H, ctypes.c_int, _P],
    "tfs_stepper_apply_update": [_H, ctypes.c_int],
    "tfs_stepper_end_of_iter": [_H, ctypes.c_int, ctypes.c_int],
    "tfs_stepper_state": [_H, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "tfs_stepper_reset": [_H, _P],
    "tfs_stepper_backup_size": [_H, ctypes.POINTER(ctypes.c_size_t)],
    "tfs_stepper_get_backup": [_H, _P],
    "tfs_stepper_set_backup": [_H, _P],
    "tfs_stepper_write_backup": [_H, ctypes.c_int, ctypes.c_char_p],
    "tfs_stepper_read_backup": [_H, ctypes.c_char_p, _IP],
    "tfs_stepper_write_files": [_H, ctypes.c_int, ctypes.c_char_p, ctypes.c_int],
    "tfs_batch_create": [ctypes.c_int, ctypes.POINTER(_H)],
    "tfs_batch_destroy": [_H],
    "tfs_batch_add": [_H, _H, _IP],
    "tfs_batch_size": [_H, _IP],
    "tfs_batch_share_inner_solves": [_H, ctypes.c_int],
    "tfs_batch_shared_solves": [_H, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "tfs_batch_share_products": [_H, ctypes.c_int],
    "tfs_batch_shared_products": [_H, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "tfs_batch_step": [_H, ctypes.c_int, _P, _P, _P],
    "tfs_server_config_default": [ctypes.POINTER(ServerConfig)],
    "tfs_server_create": [ctypes.POINTER(ServerConfig), ctypes.POINTER(_H)],
    "tfs_server_submit": [_H, ctypes.POINTER(Request), _LLP],
    "tfs_server_request_bytes": [_H, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_size_t)],
    "tfs_server_poll": [_H, ctypes.c_longlong, ctypes.c_int, _IP,
                        ctypes.POINTER(ctypes.c_double), _IP, _IP],
    "tfs_server_drain": [_H],
    "tfs_server_stats": [_H, ctypes.POINTER(ServerCounters)],
    "tfs_server_shared_solves": [_H, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "tfs_server_shared_products": [_H, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "tfs_server_destroy": [_H],
    "tfs_last_error": [],
    "tfs_kernel_launch_count": [],
    "tfs_measure_fma_peak": [ctypes.c_int, ctypes.POINTER(ctypes.c_double)],
}
_RESTYPES = {"tfs_last_error": ctypes.c_char_p, "tfs_kernel_launch_count": ctypes.c_longlong}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libtfs_gb300.so (building it first if asked). Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"{path} is missing: build it with __graft_entry__.build() "
                              "(the RPY path has no CPU fallback)")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, ctypes.c_int)
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != TFS_OK:
        msg = load().tfs_last_error().decode(errors="replace")
        raise TfsError(rc, msg)


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)
