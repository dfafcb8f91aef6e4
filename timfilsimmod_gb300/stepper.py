"""Python mirror of the reference's implicit time step for one free swimmer
with elastic filaments (src/cilia/cilia_sim_main.cu:355-527 over swimmer.cpp,
filament.cpp, rigid_body.cpp, broyden_solver.cpp and
mobility_solver::compute_errors), over the C ABI (tfs_stepper_*).

The stage methods carry the reference's names and run in its order:

    initial_guess(nt) -> forces_and_torques(nt) -> compute_velocities(nt)
    -> compute_errors(nt) -> prepare_jacobian_inv(nt) -> [find_update(nt)
    -> update(nt) -> compute_velocities(nt) -> compute_errors(nt, 1)
    -> end_of_iter(nt, big)]*

and step(nt) runs them all on the device. Everything computes on the GPU
through libtfs_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .mobility import RpyMobilitySolver


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class ImplicitStepper:
    """The implicit step of one swimmer driven through `solver`.

    fil_refs (nfil, 3): filament bases in the body frame
    (swimmer::filament_references); fil_dirs (nfil, 3): initial filament
    directions. The solver must have its blob references set; the body
    reference matrices are made here unless make_body_matrices is False.
    Keyword arguments override tfs_step_config_default (seg_sep, dt, tol,
    max_broyden_iter, kb, kt, end_force_magnitude, jacobian_confidence,
    body_radius, perturb_first_step, body_x, body_q).
    """

    def __init__(self, solver: RpyMobilitySolver, nfil: int, nseg: int, fil_refs, fil_dirs,
                 make_body_matrices: bool = True, **overrides):
        self.lib = N.load()
        self.solver = solver
        cfg = N.StepConfig()
        N.check(self.lib.tfs_step_config_default(ctypes.byref(cfg), nfil, nseg))
        for k, v in overrides.items():
            if k in ("body_x", "body_q"):
                arr = getattr(cfg, k)
                for i, x in enumerate(v):
                    arr[i] = float(x)
            elif not hasattr(cfg, k):
                raise TypeError(f"unknown step setting {k!r}")
            else:
                setattr(cfg, k, type(getattr(cfg, k))(v))
        self.cfg = cfg
        self.nfil, self.nseg = nfil, nseg
        self.ns = nfil * nseg
        self.nbroy = 6 * (self.ns + 1)
        if make_body_matrices:
            solver.set_body_pose(np.array(cfg.body_x[:]), np.array(cfg.body_q[:]))
            solver.make_body_reference_matrices()
        refs, dirs = _f64(fil_refs), _f64(fil_dirs)
        if refs.size != 3 * nfil or dirs.size != 3 * nfil:
            raise ValueError("fil_refs and fil_dirs need 3 values per filament")
        h = ctypes.c_void_p()
        N.check(self.lib.tfs_stepper_create(solver._h, ctypes.byref(cfg), _p(refs), _p(dirs),
                                            ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self.lib.tfs_stepper_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name: str, *args) -> int:
        if self._h is None:
            raise N.TfsError(N.TFS_ESTATE, "stepper has been closed")
        return getattr(self.lib, name)(self._h, *args)

    # -- the whole step --------------------------------------------------------
    def step(self, nt: int, allow_unconverged: bool = False) -> tuple[int, int]:
        """One time step; returns (Broyden iterations, GMRES iterations)."""
        b, g = ctypes.c_int(0), ctypes.c_int(0)
        rc = self._call("tfs_stepper_step", int(nt), ctypes.byref(b), ctypes.byref(g))
        if not (allow_unconverged and rc == N.TFS_ENOTCONV):
            N.check(rc)
        return b.value, g.value

    # -- stages ------------------------------------------------------------------
    def initial_guess(self, nt: int) -> None:
        N.check(self._call("tfs_stepper_initial_guess", int(nt)))

    def forces_and_torques(self, nt: int) -> np.ndarray:
        """Internal forces into the solver's f_segs; returns swimmer::f (6)."""
        sf = np.zeros(6)
        N.check(self._call("tfs_stepper_forces", int(nt), _p(sf)))
        return sf

    def compute_velocities(self, nt: int) -> int:
        it = ctypes.c_int(0)
        N.check(self._call("tfs_stepper_compute_velocities", int(nt), ctypes.byref(it)))
        return it.value

    def compute_errors(self, nt: int, which: int = 0) -> tuple[bool, np.ndarray]:
        e = np.zeros(self.nbroy)
        big = ctypes.c_int(0)
        N.check(self._call("tfs_stepper_compute_errors", int(nt), int(which), _p(e),
                           ctypes.byref(big)))
        return bool(big.value), e

    def prepare_jacobian_inv(self, nt: int) -> np.ndarray:
        """Returns the inverted 6x6 Schur complement, column-major (36)."""
        si = np.zeros(36)
        N.check(self._call("tfs_stepper_prepare_jacobian_inv", int(nt), _p(si)))
        return si

    def inverse_jacobian(self, i: int) -> np.ndarray:
        n = 6 * self.nseg
        out = np.zeros(n * n)
        N.check(self._call("tfs_stepper_inverse_jacobian", int(i), _p(out)))
        return out.reshape(n, n, order="F")

    def jacobian_inv_mult(self, nt: int, v) -> np.ndarray:
        v = _f64(v)
        out = np.zeros(self.nbroy)
        N.check(self._call("tfs_stepper_jacobian_inv_mult", int(nt), _p(v), _p(out)))
        return out

    def broyden_reset(self) -> None:
        N.check(self._call("tfs_stepper_broyden_reset"))

    def find_update(self, nt: int) -> np.ndarray:
        u = np.zeros(self.nbroy)
        N.check(self._call("tfs_stepper_find_update", int(nt), _p(u)))
        return u

    def update(self, nt: int) -> None:
        """swimmer::update with the last update, then forces_and_torques."""
        N.check(self._call("tfs_stepper_apply_update", int(nt)))

    apply_update = update

    def end_of_iter(self, nt: int, big: bool) -> None:
        N.check(self._call("tfs_stepper_end_of_iter", int(nt), int(bool(big))))

    def reset(self, seg_rotation=None) -> None:
        """Back to the straight start (and the solver's warm start at creation),
        each segment turned by exp(seg_rotation[j]) if given (Ns x 3)."""
        if seg_rotation is None:
            N.check(self._call("tfs_stepper_reset", None))
        else:
            r = _f64(seg_rotation)
            if r.size != 3 * self.ns:
                raise ValueError("seg_rotation needs 3 values per segment")
            N.check(self._call("tfs_stepper_reset", _p(r)))

    # -- the reference's data files ------------------------------------------------
    def backup(self) -> np.ndarray:
        """The swimmer's backup record (swimmer::write_backup order)."""
        n = ctypes.c_size_t(0)
        N.check(self._call("tfs_stepper_backup_size", ctypes.byref(n)))
        v = np.zeros(n.value)
        N.check(self._call("tfs_stepper_get_backup", _p(v)))
        return v

    def restore(self, values) -> None:
        v = _f64(values)
        N.check(self._call("tfs_stepper_set_backup", _p(v)))

    def write_backup(self, save_step: int, path: str) -> None:
        N.check(self._call("tfs_stepper_write_backup", int(save_step), path.encode()))

    def read_backup(self, path: str) -> int:
        """Restore from a backup file; returns the step to run next."""
        step = ctypes.c_int(0)
        N.check(self._call("tfs_stepper_read_backup", path.encode(), ctypes.byref(step)))
        return step.value

    def write_files(self, nt: int, prefix: str, backup: bool = True) -> None:
        """The reference's plot-step records after step nt (and the backup)."""
        N.check(self._call("tfs_stepper_write_files", int(nt), prefix.encode(), int(bool(backup))))

    def state(self) -> dict:
        ns, nf, sg = self.ns, self.nfil, self.nseg
        out = dict(x=np.zeros(3 * ns), q=np.zeros(4 * ns), u=np.zeros(3 * ns),
                   lam=np.zeros(3 * (sg - 1) * nf), tether=np.zeros(3 * nf),
                   clamp=np.zeros(3 * nf), body_x=np.zeros(3), body_q=np.zeros(4),
                   body_u=np.zeros(3))
        N.check(self._call("tfs_stepper_state", *[_p(out[k]) for k in (
            "x", "q", "u", "lam", "tether", "clamp", "body_x", "body_q", "body_u")]))
        return out
