"""Python mirror of the reference's `rpy_mobility_solver`
(src/cilia/mobility/rpy_mobility_solver.{hpp,cu}) over the C ABI.

Method names, argument meaning and call order are the reference's: the host
arrays `x_segs_host`, `f_segs_host`, `f_blobs_host`, `v_segs_host`,
`v_blobs_host`, `f_blobs_repulsion_host` are owned by the solver (pinned when
PyTorch is available, mobility_solver.hpp:57-63), callers write positions and
forces into them in place, and the hooks move them to and from the device.
Everything computes on the GPU through libtfs_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


class _DeviceArray:
    """A view of one solver device buffer with __cuda_array_interface__, so
    torch.as_tensor(view, device="cuda") aliases it without copying."""

    def __init__(self, ptr: int, n: int, owner):
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}


def _host_array(n: int, pinned: bool, keep: list) -> np.ndarray:
    """A float64 host array, page-locked when PyTorch can pin it (copies to
    and from the device then run at DMA speed without staging); the owning
    tensor is kept in `keep` for the array's lifetime."""
    if pinned:
        try:
            import torch
            if torch.cuda.is_available():
                t = torch.zeros(n, dtype=torch.float64, pin_memory=True)
                keep.append(t)
                return t.numpy()
        except Exception:  # pragma: no cover - pinned memory is an optimisation only
            pass
    return np.zeros(n, dtype=np.float64)


def host_array_pinned(a: np.ndarray) -> bool:
    """Whether a host array is page-locked (False without a GPU)."""
    try:
        import torch
        return torch.cuda.is_available() and bool(torch.from_numpy(a).is_pinned())
    except Exception:
        return False


def _ptr(a: np.ndarray) -> int:
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


PRECISIONS = {"fp64": N.TFS_FP64, "fp32c": N.TFS_FP32C}


class RpyMobilitySolver:
    """RPY mobility solver on one GB300.

    nswim, nfil, nseg, nblob: NSWIM, NFIL, NSEG, NBLOB of the reference.
    precision: "fp64" (plain FP64, the parity form) or "fp32c" (FP32 pairwise
    sums with compensated accumulation).
    """

    def __init__(self, nswim: int, nfil: int, nseg: int, nblob: int, precision: str = "fp64",
                 mu: float = 1.0, a_seg: float = 1.0, a_blob: float = 1.0,
                 end_force_magnitude: int | None = None, repulsive_force_factor: float = 2.0,
                 free_body: bool = True, pinned: bool = True):
        self.lib = N.load()
        cfg = N.Config()
        N.check(self.lib.tfs_config_default(ctypes.byref(cfg), nswim, nfil, nseg, nblob))
        cfg.mu, cfg.a_seg, cfg.a_blob = mu, a_seg, a_blob
        if end_force_magnitude is not None:
            cfg.end_force_magnitude = int(end_force_magnitude)
        cfg.repulsive_force_factor = repulsive_force_factor
        cfg.free_body = int(bool(free_body))
        cfg.precision = PRECISIONS[precision]
        self.cfg = cfg
        self.precision = precision
        self.num_segs = nswim * nfil * nseg
        self.num_blobs = nswim * nblob
        self._pinned = pinned
        self._h = None
        self.initialise()

    # -- allocate_host_memory / allocate_device_memory (rpy_mobility_solver.cu:54-117)
    def initialise(self) -> None:
        if self._h is not None:
            return
        h = ctypes.c_void_p()
        N.check(self.lib.tfs_solver_create(ctypes.byref(self.cfg), ctypes.byref(h)))
        self._h = h
        ns, nb, pin = self.num_segs, self.num_blobs, self._pinned
        self._host_tensors: list = []
        keep = self._host_tensors
        self.x_segs_host = _host_array(3 * ns, pin, keep)
        self.f_segs_host = _host_array(6 * ns, pin, keep)
        self.v_segs_host = _host_array(6 * ns, pin, keep)
        self.x_blobs_host = _host_array(3 * nb, pin, keep)
        self.f_blobs_host = _host_array(3 * nb, pin, keep)
        self.v_blobs_host = _host_array(3 * nb, pin, keep)
        self.f_blobs_repulsion_host = _host_array(3 * nb, pin, keep)

    # -- free_host_memory / free_device_memory
    def finalise(self) -> None:
        if self._h is not None:
            self.lib.tfs_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.finalise()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.finalise()

    def _call(self, name: str, *args) -> None:
        if self._h is None:
            raise N.TfsError(N.TFS_ESTATE, "solver has been finalised")
        N.check(getattr(self.lib, name)(self._h, *args))

    # -- configuration
    def set_stream(self, stream: int | None) -> None:
        """Run on a cudaStream_t handle (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._call("tfs_solver_set_stream", ctypes.c_void_p(stream or 0))

    def set_precision(self, precision: str) -> None:
        self._call("tfs_solver_set_precision", PRECISIONS[precision])
        self.precision = precision

    def device_arrays(self) -> dict:
        """Device buffers as __cuda_array_interface__ views (float64, AoS)."""
        b = N.DeviceBuffers()
        self._call("tfs_solver_device_buffers", ctypes.byref(b))
        ns, nb = self.num_segs, self.num_blobs
        sizes = dict(x_segs=3 * ns, f_segs=6 * ns, v_segs=6 * ns, x_blobs=3 * nb,
                     f_blobs=3 * nb, v_blobs=3 * nb, f_blobs_repulsion=3 * nb)
        return {k: _DeviceArray(getattr(b, k), n, self) for k, n in sizes.items()}

    def enable_kernel_timing(self, enable: bool = True) -> None:
        self._call("tfs_solver_enable_kernel_timing", int(bool(enable)))

    def kernel_timing(self) -> list[float]:
        """Durations (ms) of the RPY product launches (work-queue and tile
        kernels) since the last call, in launch order."""
        buf = (ctypes.c_double * 4096)()
        n = ctypes.c_int()
        self._call("tfs_solver_kernel_timing", buf, 4096, ctypes.byref(n))
        return list(buf[:min(n.value, 4096)])

    def autotune(self, precisions=("fp64", "fp32c"), reps: int = 2) -> dict:
        """Pick the fastest work-queue variant per product kind (and tile
        variant for the kernel-sequence GMRES's blob-blob product) for this
        solver's sizes (on its current data); returns the tuning table."""
        import json

        mask = sum(1 << PRECISIONS[p] for p in precisions)
        self._call("tfs_solver_autotune", mask, int(reps))
        return json.loads(self.tuning_report())

    def set_tuning(self, combo: int, variant: int, waves: int = 1,
                   precision: str | None = None) -> None:
        """Pin the tile-kernel launch of one (target, source-set) combination."""
        prec = PRECISIONS[precision or self.precision]
        self._call("tfs_solver_set_tuning", prec, int(combo), int(variant), int(waves))

    def set_queue_variant(self, kind: int, variant: int, precision: str | None = None) -> None:
        """Pin the work-queue variant of one product kind (0..5: M_ss, M_bs,
        M_ss with M_bs, M_sb, M_bb, grand mobility)."""
        prec = PRECISIONS[precision or self.precision]
        self._call("tfs_solver_set_queue_variant", prec, int(kind), int(variant))

    def tuning_report(self) -> str:
        need = ctypes.c_size_t()
        self._call("tfs_solver_tuning_report", None, 0, ctypes.byref(need))
        buf = ctypes.create_string_buffer(need.value)
        self._call("tfs_solver_tuning_report", buf, need.value, None)
        return buf.value.decode()

    def positions_updated(self) -> None:
        self._call("tfs_solver_positions_updated")

    # -- the hooks (mobility_solver.hpp:26-46)
    def copy_segment_positions_to_device(self):
        self._call("tfs_copy_segment_positions_to_device", _ptr(self.x_segs_host))

    def copy_segment_forces_to_device(self):
        self._call("tfs_copy_segment_forces_to_device", _ptr(self.f_segs_host))

    def copy_blob_positions_to_device(self):
        self._call("tfs_copy_blob_positions_to_device", _ptr(self.x_blobs_host))

    def copy_blob_forces_to_device(self):
        self._call("tfs_copy_blob_forces_to_device", _ptr(self.f_blobs_host))

    def copy_interparticle_blob_forces_to_host(self):
        self._call("tfs_copy_interparticle_blob_forces_to_host", _ptr(self.f_blobs_repulsion_host))

    def copy_blob_velocities_to_host(self):
        self._call("tfs_copy_blob_velocities_to_host", _ptr(self.v_blobs_host))

    def copy_segment_velocities_to_host(self):
        self._call("tfs_copy_segment_velocities_to_host", _ptr(self.v_segs_host))

    def apply_interparticle_forces(self):
        self._call("tfs_apply_interparticle_forces")

    def wait_for_device(self):
        self._call("tfs_wait_for_device")

    def evaluate_segment_segment_mobility(self):
        self._call("tfs_evaluate_segment_segment_mobility")

    def evaluate_segment_blob_mobility(self):
        self._call("tfs_evaluate_segment_blob_mobility")

    def evaluate_blob_blob_mobility(self):
        self._call("tfs_evaluate_blob_blob_mobility")

    def evaluate_blob_blob_mobility_ff(self):
        """v_blobs = Mbb f_blobs in float-float arithmetic (~1e-13): the
        product FP32C refinement computes its residuals with."""
        self._call("tfs_evaluate_blob_blob_mobility_ff")

    def evaluate_weakly_coupled_segment_mobility(self):
        """The weakly coupled filaments' segment product (the reference's
        weakly_coupled_filaments_rpy_mobility_solver: RPY within a filament,
        Stokeslets of the other filaments' total forces at their means)."""
        self._call("tfs_evaluate_weakly_coupled_segment_mobility")

    def evaluate_blob_segment_mobility(self):
        self._call("tfs_evaluate_blob_segment_mobility")

    def evaluate_full_mobility(self):
        """rpy_mobility_solver.cu:330-337, including its D2H copies."""
        self._call("tfs_evaluate_full_mobility", _ptr(self.v_segs_host), _ptr(self.v_blobs_host))

    def apply_grand_mobility(self):
        """v_segs = Mss f_segs + Msb f_blobs; v_blobs = Mbs f_segs + Mbb f_blobs."""
        self._call("tfs_apply_grand_mobility")

    # -- the free-body solve (mobility_solver.cpp: compute_velocities,
    #    solve_linear_system, make_body_reference_matrices)
    def set_blob_references(self, blob_refs) -> None:
        """rigid_body::blob_references: blob offsets in the body frame."""
        self._refs = np.ascontiguousarray(np.asarray(blob_refs, dtype=np.float64).ravel())
        self._call("tfs_set_blob_references", _ptr(self._refs))

    def set_body_pose(self, x, q=None) -> None:
        """rigid_body::x and q (q0, q1, q2, q3); places the blobs on the device."""
        xx = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
        if q is None:
            self._call("tfs_set_body_pose", _ptr(xx), None)
        else:
            qq = np.ascontiguousarray(np.asarray(q, dtype=np.float64).ravel())
            self._call("tfs_set_body_pose", _ptr(xx), _ptr(qq))

    def set_linear_solver(self, tol: float, max_iter: int | None = None) -> None:
        """LINEAR_SYSTEM_TOL and MAX_LINEAR_SYSTEM_ITER."""
        if max_iter is None:
            max_iter = min(350, 3 * self.num_blobs + 6)
        self._call("tfs_set_linear_solver", float(tol), int(max_iter))

    def set_refinement(self, inner_tol: float = 1e-4, max_cycles: int = 12) -> None:
        self._call("tfs_set_refinement", float(inner_tol), int(max_cycles))

    def set_refinement_vectors(self, mode: str = "fp32") -> None:
        """FP32C: Arnoldi vectors of the cooperative inner solves. "fp32"
        (default; a refinement that stalls is rerun with FP64 vectors) or
        "fp64" (every solve)."""
        modes = {"fp32": 0, "fp64": 1}
        if mode not in modes:
            raise ValueError(f"mode is one of {sorted(modes)}")
        self._call("tfs_set_refinement_vectors", modes[mode])

    def set_persistent_gmres(self, enable: bool = True) -> None:
        """FP32C inner GMRES as one cooperative kernel (default) or as a
        sequence of kernels per Arnoldi step."""
        self._call("tfs_set_persistent_gmres", int(bool(enable)))

    def inject_barrier_stall(self, on: bool = True) -> None:
        """Test hook: the cooperative inner GMRES's grid barriers wait for one
        CTA more than the launch has, so each wait runs out its 2 s bound and
        the solve raises TfsError(TFS_ETIMEOUT); off restores normal solves."""
        self._call("tfs_inject_barrier_stall", int(bool(on)))

    def make_body_reference_matrices(self) -> tuple[np.ndarray, np.ndarray]:
        """Returns (body_mobility_reference, KTKinv_reference), 6x6 column-major flat."""
        self._call("tfs_make_body_reference_matrices")
        return self.body_reference_matrices()

    def body_reference_matrices(self) -> tuple[np.ndarray, np.ndarray]:
        bm, kt = np.zeros(36), np.zeros(36)
        self._call("tfs_get_body_reference_matrices", _ptr(bm), _ptr(kt))
        return bm, kt

    def set_body_reference_matrices(self, body_mobility=None, ktkinv=None) -> None:
        a = None if body_mobility is None else np.ascontiguousarray(body_mobility, dtype=np.float64)
        b = None if ktkinv is None else np.ascontiguousarray(ktkinv, dtype=np.float64)
        self._call("tfs_set_body_reference_matrices", None if a is None else _ptr(a),
                   None if b is None else _ptr(b))

    def compute_velocities(self, swimmer_f) -> tuple[int, np.ndarray]:
        """compute_velocities on the device-resident positions/forces; returns
        (GMRES iterations, swimmer force with the blob repulsion added)."""
        f = np.ascontiguousarray(np.array(swimmer_f, dtype=np.float64).ravel())
        it = ctypes.c_int()
        self._call("tfs_compute_velocities", _ptr(f), ctypes.byref(it))
        return it.value, f

    def solve_linear_system(self, rhs) -> int:
        r = np.ascontiguousarray(np.asarray(rhs, dtype=np.float64).ravel())
        it = ctypes.c_int()
        self._call("tfs_solve_linear_system", _ptr(r), ctypes.byref(it))
        return it.value

    def body_velocities(self) -> np.ndarray:
        v = np.zeros(6)
        self._call("tfs_get_body_velocities", _ptr(v))
        return v

    def set_body_velocities(self, v) -> None:
        vv = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
        self._call("tfs_set_body_velocities", _ptr(vv))

    def blob_forces(self) -> np.ndarray:
        """The solved blob forces (synchronises)."""
        self._call("tfs_copy_blob_forces_to_host", _ptr(self.f_blobs_host))
        self.wait_for_device()
        return self.f_blobs_host.copy()

    def solve_info(self) -> dict:
        it, cyc, rel = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._call("tfs_solve_info", ctypes.byref(it), ctypes.byref(cyc), ctypes.byref(rel))
        return {"iters": it.value, "cycles": cyc.value, "rel_residual": rel.value}

    def refinement_retries(self) -> int:
        """FP32C refinements rerun with FP64 Arnoldi vectors after a stall."""
        n = ctypes.c_longlong()
        self._call("tfs_refinement_retries", ctypes.byref(n))
        return n.value

    # -- convenience: set all inputs from arrays (AoS float64)
    def set_state(self, x_segs, f_segs, x_blobs, f_blobs) -> None:
        self.x_segs_host[:] = np.asarray(x_segs, dtype=np.float64).ravel()
        self.f_segs_host[:] = np.asarray(f_segs, dtype=np.float64).ravel()
        self.x_blobs_host[:] = np.asarray(x_blobs, dtype=np.float64).ravel()
        self.f_blobs_host[:] = np.asarray(f_blobs, dtype=np.float64).ravel()
        self.copy_segment_positions_to_device()
        self.copy_segment_forces_to_device()
        self.copy_blob_positions_to_device()
        self.copy_blob_forces_to_device()


def measure_fma_peak(precision: str = "fp64") -> float:
    """FMA throughput of the current device, FLOP/s (2 per FMA)."""
    lib = N.load()
    out = ctypes.c_double()
    N.check(lib.tfs_measure_fma_peak(PRECISIONS[precision], ctypes.byref(out)))
    return out.value


def num_tile_variants(precision: str) -> int:
    return int(N.load().tfs_num_tile_variants(PRECISIONS[precision]))


def num_queue_variants(precision: str) -> int:
    return int(N.load().tfs_num_queue_variants(PRECISIONS[precision]))


QUEUE_KINDS = ("seg<-seg", "blob<-seg", "seg,blob<-seg", "seg<-blob", "blob<-blob", "grand")


def kernel_launch_count() -> int:
    return int(N.load().tfs_kernel_launch_count())


PG_TRACE_PHASES = ("M_bb + barrier", "w = A z", "pass-1 dots + barrier", "h1 sum",
                   "w' + pass-2 dots + barrier", "h2 sum", "Q_k, z_k, records",
                   "last barrier")


def pg_trace() -> np.ndarray:
    """The phase trace of the last cooperative inner GMRES solve, from a
    library built with -DTFS_PG_TRACE: per-phase durations (ns) of every
    Arnoldi step of that solve, shape (2 CTAs, steps, 8 phases), phases as
    PG_TRACE_PHASES (each phase ends where the next begins; the last ends at
    the next step's start). Raises TfsError in other builds."""
    lib = N.load()
    steps = ctypes.c_int()
    lib.tfs_pg_trace(None, 0, ctypes.byref(steps))  # the capacity it needs
    if steps.value <= 0:
        N.check(lib.tfs_pg_trace(None, 0, ctypes.byref(steps)))
    buf = np.zeros((2, steps.value, 8), dtype=np.uint64)
    N.check(lib.tfs_pg_trace(buf.ctypes.data_as(ctypes.c_void_p), buf.size,
                             ctypes.byref(steps)))
    t = buf.astype(np.int64)
    # steps of the last solve (or restart cycle): from step 1 while the
    # starts keep increasing (later entries are left over from longer,
    # earlier solves, so they start earlier)
    n = 1
    while n + 1 < t.shape[1] and t[0, n + 1, 0] > t[0, n, 0] and t[1, n + 1, 0] > t[1, n, 0]:
        n += 1
    # step n (the last) stopped after its M_bb phase; steps 1 .. n-1 are whole
    if n < 2:
        return np.zeros((2, 0, 8), dtype=np.int64)
    ends = np.concatenate([t[:, 1:n, 1:], t[:, 2:n + 1, :1]], axis=2)
    return ends - t[:, 1:n, :]
