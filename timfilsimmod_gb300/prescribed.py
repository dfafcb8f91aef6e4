"""Prescribed-cilia mobility solve (the reference's mobility_solver under
PRESCRIBED_CILIA): the host-side mirror of compute_velocities for filaments
that follow a prescribed sequence of shapes, over the C ABI of
include/tfs_gb300.h (tfs_prescribed_*).

The reference's filament code writes the segment positions into the
solver's x_segs_host and keeps d x / d phase (vel_dir_phase), d x / d angle
(vel_dir_angle), phase, omega0, shape_rotation_angle and the phase and angle
rates on each filament (filament.hpp:97-118); compute_velocities then solves
for segment forces, blob forces, body velocities (free body) and the rates
(dynamic phase / shape rotation) (mobility_solver.cpp:2574-2596). Here the
same state is passed as arrays; the solution stays on the device as the next
solve's warm start and is read with `solution()`.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .mobility import RpyMobilitySolver

PRESCRIBED_BODY = N.TFS_PRESCRIBED_BODY
DYNAMIC_PHASE = N.TFS_DYNAMIC_PHASE
DYNAMIC_ANGLE = N.TFS_DYNAMIC_ANGLE
WEAKLY_COUPLED = N.TFS_WEAKLY_COUPLED


def _arr(a) -> np.ndarray | None:
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


class PrescribedCiliaSolver:
    """One swimmer of nfil prescribed filaments x nseg segments and nblob
    blobs.

    flags: PRESCRIBED_BODY (PRESCRIBED_BODY_VELOCITIES), DYNAMIC_PHASE
    (DYNAMIC_PHASE_EVOLUTION), DYNAMIC_ANGLE (DYNAMIC_SHAPE_ROTATION),
    WEAKLY_COUPLED (the weakly coupled filaments' mobility). seg_sep: DL, for
    FIL_LENGTH = DL (NSEG - 1). phase_force_refs / angle_force_refs: the
    generalised-force tables over one period (the reference's
    data/forcing/*_reference_*_generalised_forces files). precision "fp64"
    (the reference's FP64 build) or "fp32c": inner GMRES solves with FP32 pair
    sums (compensated accumulation), refined on FP64 residuals to the same
    tolerance.
    """

    def __init__(self, flags: int, nfil: int, nseg: int, blob_refs, seg_sep: float,
                 phase_force_refs=None, angle_force_refs=None, body_x=(0.0, 0.0, 0.0),
                 body_q=(1.0, 0.0, 0.0, 0.0), mu: float = 1.0, a_seg: float = 1.0,
                 a_blob: float = 1.0, tol: float = 1e-4,
                 gen_force_magnitude_factor: float = 1.0,
                 torsional_spring_magnitude_factor: float = 2.0, precision: str = "fp64"):
        refs = _arr(blob_refs)
        self.flags, self.nfil, self.nseg = int(flags), int(nfil), int(nseg)
        self.nblob = refs.size // 3
        self.solver = RpyMobilitySolver(1, nfil, nseg, self.nblob, precision, mu=mu, a_seg=a_seg,
                                        a_blob=a_blob)
        self.lib = self.solver.lib
        s = self.solver
        s.set_blob_references(refs)
        s.set_body_pose(body_x, body_q)
        cfg = N.PrescribedConfig()
        N.check(self.lib.tfs_prescribed_config_default(ctypes.byref(cfg), self.flags, self.nseg,
                                                       float(seg_sep)))
        cfg.gen_force_magnitude_factor = float(gen_force_magnitude_factor)
        cfg.torsional_spring_magnitude_factor = float(torsional_spring_magnitude_factor)
        self._tab_p, self._tab_a = _arr(phase_force_refs), _arr(angle_force_refs)
        s._call("tfs_prescribed_setup", ctypes.byref(cfg), _p(self._tab_p),
                0 if self._tab_p is None else self._tab_p.size, _p(self._tab_a),
                0 if self._tab_a is None else self._tab_a.size)
        n = ctypes.c_int()
        s._call("tfs_prescribed_size", ctypes.byref(n))
        self.n = n.value
        self.set_linear_solver(tol)

    def set_linear_solver(self, tol: float) -> None:
        """LINEAR_SYSTEM_TOL (the iteration cap is MAX_LINEAR_SYSTEM_ITER,
        min(350, unknowns))."""
        self.solver.set_linear_solver(float(tol))

    def set_body_pose(self, x, q=None) -> None:
        self.solver.set_body_pose(x, q)

    def _kinematics(self, vel_dir_phase, vel_dir_angle=None, phase=None, omega0=None,
                    shape_rotation_angle=None, phase_dot=None, v_body=None):
        self._kin = [_arr(a) for a in (vel_dir_phase, vel_dir_angle, phase, omega0,
                                       shape_rotation_angle, phase_dot, v_body)]
        k = N.PrescribedKinematics(*[_p(a) for a in self._kin])
        return k

    def set_kinematics(self, x_segs, vel_dir_phase, vel_dir_angle=None, phase=None, omega0=None,
                       shape_rotation_angle=None, phase_dot=None, v_body=None) -> None:
        """Segment positions and the filaments' kinematics of this step;
        computes swimmer.KTMinvK_inv (make_precon_mat) on them."""
        s = self.solver
        s.x_segs_host[:] = np.asarray(x_segs, dtype=np.float64).ravel()
        s.copy_segment_positions_to_device()
        k = self._kinematics(vel_dir_phase, vel_dir_angle, phase, omega0, shape_rotation_angle,
                             phase_dot, v_body)
        s._call("tfs_prescribed_set_kinematics", ctypes.byref(k))

    def solve(self) -> int:
        """assemble_rhs and solve_linear_system; returns the GMRES iterations."""
        it = ctypes.c_int()
        self.solver._call("tfs_prescribed_solve", ctypes.byref(it))
        return it.value

    def compute_velocities(self, x_segs, vel_dir_phase, vel_dir_angle=None, phase=None,
                           omega0=None, shape_rotation_angle=None, phase_dot=None,
                           v_body=None) -> int:
        """compute_velocities (mobility_solver.cpp:2574-2596) on this step's
        kinematics; returns the GMRES iterations."""
        self.set_kinematics(x_segs, vel_dir_phase, vel_dir_angle, phase, omega0,
                            shape_rotation_angle, phase_dot, v_body)
        return self.solve()

    def solution(self) -> dict:
        """Segment forces (Ns, 3), blob forces (Nb, 3), body velocities (6),
        phase and angle rates (nfil each) of the last solve."""
        ns = self.nfil * self.nseg
        fs, fb = np.zeros(3 * ns), np.zeros(3 * self.nblob)
        vb, pd, ad = np.zeros(6), np.zeros(self.nfil), np.zeros(self.nfil)
        self.solver._call("tfs_prescribed_solution", _p(fs), _p(fb), _p(vb), _p(pd), _p(ad))
        return dict(f_segs=fs.reshape(-1, 3), f_blobs=fb.reshape(-1, 3), v_body=vb,
                    phase_dot=pd, angle_dot=ad)

    def set_solution(self, f_segs=None, f_blobs=None, v_body=None, phase_dot=None,
                     angle_dot=None) -> None:
        """The next solve's warm start (the reference keeps the last solution
        in its force arrays, v_bodies and the filaments' rates)."""
        arrs = [_arr(a) for a in (f_segs, f_blobs, v_body, phase_dot, angle_dot)]
        self.solver._call("tfs_prescribed_set_solution", *[_p(a) for a in arrs])

    def apply(self, which: str, v=None) -> np.ndarray:
        """One piece on the kinematics set last: "operator" (A v),
        "preconditioner" (P^-1 v) or "rhs"."""
        code = {"operator": 0, "preconditioner": 1, "rhs": 2}[which]
        vin = _arr(v) if v is not None else None
        out = np.zeros(self.n)
        self.solver._call("tfs_prescribed_apply", code, _p(vin), _p(out))
        return out

    def precon_matrix(self) -> np.ndarray:
        """swimmer.KTMinvK_inv (6 x 6, column-major as the reference stores it)."""
        m = np.zeros(36)
        self.solver._call("tfs_prescribed_precon_matrix", _p(m))
        return m

    def solve_info(self) -> dict:
        return self.solver.solve_info()

    def finalise(self) -> None:
        self.solver.finalise()
