"""ctypes bindings for the CPU oracle (test infrastructure only).

`Oracle` wraps liboracle.so, the C restatement of the reference's RPY path
(tfs_oracle.c). `ReferenceKernels` wraps oracle/_ref/libref_kernels_*.so, the
reference's own cuda_functions.cu compiled unchanged for the CPU, which exists
only where the reference tree was present at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_P = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P)


def build_oracle(quiet: bool = True) -> str:
    """Compile liboracle.so with make (gcc; seconds)."""
    out = subprocess.run(["make", "-C", HERE, "liboracle.so"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "liboracle.so")


class _Params(ctypes.Structure):
    _fields_ = [("mu", ctypes.c_double), ("a_seg", ctypes.c_double), ("a_blob", ctypes.c_double)]


class Oracle:
    """FP64 CPU restatement of the reference's mobility blocks, barrier forces
    and flow field. Inputs/outputs are the reference's AoS float64 arrays."""

    def __init__(self, mu: float = 1.0, a_seg: float = 1.0, a_blob: float = 1.0, threads: int = 1):
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build_oracle()
        self.lib = ctypes.CDLL(path)
        self.p = _Params(mu, a_seg, a_blob)
        self.set_threads(threads)

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(int(n))
        self.threads = self.lib.orc_get_threads()

    def mss(self, x_segs, f_segs):
        x, f = _c(x_segs), _c(f_segs)
        ns = x.size // 3
        v = np.zeros(6 * ns)
        self.lib.orc_mss(ctypes.byref(self.p), _ptr(v), _ptr(f), _ptr(x), ns)
        return v

    def msf(self, x_segs, f_segs, nfil, nseg):
        """Weakly coupled filaments' segment product (orc_msf)."""
        x, f = _c(x_segs), _c(f_segs)
        v = np.zeros(f.size)
        self.lib.orc_msf(ctypes.byref(self.p), _ptr(v), _ptr(f), _ptr(x), int(nfil), int(nseg))
        return v

    def msb(self, x_segs, x_blobs, f_blobs, v_segs=None):
        xs, xb, fb = _c(x_segs), _c(x_blobs), _c(f_blobs)
        ns, nb = xs.size // 3, xb.size // 3
        v = np.zeros(6 * ns) if v_segs is None else np.array(v_segs, dtype=np.float64).ravel()
        self.lib.orc_msb(ctypes.byref(self.p), _ptr(v), _ptr(fb), _ptr(xs), _ptr(xb), ns, nb)
        return v

    def mbb(self, x_blobs, f_blobs):
        x, f = _c(x_blobs), _c(f_blobs)
        nb = x.size // 3
        v = np.zeros(3 * nb)
        self.lib.orc_mbb(ctypes.byref(self.p), _ptr(v), _ptr(f), _ptr(x), nb)
        return v

    def mbs(self, x_blobs, x_segs, f_segs):
        xb, xs, fs = _c(x_blobs), _c(x_segs), _c(f_segs)
        nb, ns = xb.size // 3, xs.size // 3
        v = np.zeros(3 * nb)
        self.lib.orc_mbs(ctypes.byref(self.p), _ptr(v), _ptr(fs), _ptr(xb), _ptr(xs), nb, ns)
        return v

    def full(self, x_segs, f_segs, x_blobs, f_blobs):
        """All four blocks, in the order of rpy_mobility_solver.cu:330-337."""
        v_segs = self.mss(x_segs, f_segs)
        v_segs = self.msb(x_segs, x_blobs, f_blobs, v_segs)
        v_blobs = self.mbb(x_blobs, f_blobs)
        v_bs = self.mbs(x_blobs, x_segs, f_segs)
        return v_segs, v_blobs, v_bs

    def block(self, vd, fd, x_tgt, a_tgt, x_src, f_src, a_src, v=None):
        """General block (orc_rpy_block); v given = accumulate into it."""
        xt, xs, fs = _c(x_tgt), _c(x_src), _c(f_src)
        nt, ns = xt.size // 3, xs.size // 3
        acc = v is not None
        out = np.array(v, dtype=np.float64).ravel() if acc else np.zeros(vd * nt)
        self.lib.orc_rpy_block(ctypes.byref(self.p), int(vd), int(fd), _ptr(out), _ptr(xt), nt,
                               ctypes.c_double(a_tgt), _ptr(xs), _ptr(fs), ns,
                               ctypes.c_double(a_src), int(acc))
        return out

    def barrier_forces(self, x_segs, x_blobs, f_segs, nseg, end_force_magnitude: int,
                       repulsive_force_factor=2.0, free_body=True):
        xs, xb = _c(x_segs), _c(x_blobs)
        fs = np.array(f_segs, dtype=np.float64).ravel().copy()
        ns, nb = xs.size // 3, xb.size // 3
        frep = np.zeros(3 * nb)
        self.lib.orc_barrier_forces(ctypes.byref(self.p), _ptr(fs), _ptr(frep), _ptr(xs),
                                    _ptr(xb), ns, nb, int(nseg), int(end_force_magnitude),
                                    ctypes.c_double(repulsive_force_factor), int(bool(free_body)))
        return fs, frep

    def flow_velocities(self, x_flow, x_segs, f_segs, segs_per_body, x_blobs, f_blobs,
                        blobs_per_body, x_bodies, prefac, remove_net_force=False):
        xf, xs, fs = _c(x_flow), _c(x_segs), _c(f_segs)
        xb = _c(x_blobs) if blobs_per_body else np.zeros(3)
        fb = _c(f_blobs) if blobs_per_body else np.zeros(3)
        xbod = _c(x_bodies)
        nf = xf.size // 3
        nbod = xbod.size // 3
        v = np.zeros(3 * nf)
        self.lib.orc_flow_velocities(_ptr(v), _ptr(xf), nf, _ptr(fs), _ptr(xs), int(segs_per_body),
                                     _ptr(fb), _ptr(xb), int(blobs_per_body), _ptr(xbod), nbod,
                                     ctypes.c_double(prefac), int(bool(remove_net_force)))
        return v


def _c(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())


class ReferenceKernels:
    """The reference's own kernels (cuda_functions.cu), compiled unchanged for
    the CPU by `make -C oracle ref`. `variant` is "a1" (RSEG = RBLOB = 1) or
    "a16" (RSEG = 1, RBLOB = 1.6)."""

    def __init__(self, variant: str = "a1"):
        path = os.path.join(REF_DIR, f"libref_kernels_{variant}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        for name in ("ref_rseg", "ref_rblob", "ref_mu"):
            getattr(self.lib, name).restype = ctypes.c_double
        self.a_seg = self.lib.ref_rseg()
        self.a_blob = self.lib.ref_rblob()
        self.mu = self.lib.ref_mu()

    @staticmethod
    def available(variant: str = "a1") -> bool:
        return os.path.exists(os.path.join(REF_DIR, f"libref_kernels_{variant}.so"))

    def sync(self, nswim, nseg, nfil, nblob, end_force_magnitude=0, seg_sep=2.2):
        self.lib.ref_sync_var(int(nswim), int(nseg), int(nfil), int(nblob),
                              int(end_force_magnitude), ctypes.c_double(seg_sep))

    def mss(self, x_segs, f_segs):
        x, f = _c(x_segs), _c(f_segs)
        v = np.zeros(f.size)
        self.lib.ref_mss(_ptr(v), _ptr(f), _ptr(x), x.size // 3)
        return v

    def msb(self, x_segs, x_blobs, f_blobs, v_segs=None):
        xs, xb, fb = _c(x_segs), _c(x_blobs), _c(f_blobs)
        v = np.zeros(2 * xs.size) if v_segs is None else np.array(v_segs, dtype=np.float64).ravel()
        self.lib.ref_msb(_ptr(v), _ptr(fb), _ptr(xs), _ptr(xb), xs.size // 3)
        return v

    def mbb(self, x_blobs, f_blobs):
        x, f = _c(x_blobs), _c(f_blobs)
        v = np.zeros(x.size)
        self.lib.ref_mbb(_ptr(v), _ptr(f), _ptr(x), x.size // 3)
        return v

    def mbs(self, x_blobs, x_segs, f_segs):
        xb, xs, fs = _c(x_blobs), _c(x_segs), _c(f_segs)
        v = np.zeros(xb.size)
        self.lib.ref_mbs(_ptr(v), _ptr(fs), _ptr(xb), _ptr(xs), xb.size // 3)
        return v

    def msf(self, x_segs, f_segs, nfil, nseg):
        """The reference's weakly coupled filaments' product (filament means,
        total forces, Msf_mult); sync() first with these nfil and nseg."""
        x, f = _c(x_segs), _c(f_segs)
        v = np.zeros(f.size)
        self.lib.ref_msf(_ptr(v), _ptr(f), _ptr(x), x.size // 3, int(nfil))
        return v

    def barrier_forces(self, x_segs, x_blobs, f_segs):
        xs, xb = _c(x_segs), _c(x_blobs)
        fs = np.array(f_segs, dtype=np.float64).ravel().copy()
        frep = np.zeros(xb.size)
        self.lib.ref_barrier_forces(_ptr(fs), _ptr(frep), _ptr(xs), _ptr(xb), xs.size // 3,
                                    xb.size // 3)
        return fs, frep


class ReferenceFlow:
    """The reference's flow_velocities kernel (flow_field_evaluator.cu:13-228),
    compiled unchanged for the CPU by `make -C oracle ref`."""

    def __init__(self):
        path = os.path.join(REF_DIR, "libref_flow.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(REF_DIR, "libref_flow.so"))

    def flow_velocities(self, x_flow, x_segs, f_segs, segs_per_body, x_blobs, f_blobs,
                        blobs_per_body, x_bodies, prefac, remove_net_force=False):
        xf, xs, fs = _c(x_flow), _c(x_segs), _c(f_segs)
        xb = _c(x_blobs) if blobs_per_body else np.zeros(3)
        fb = _c(f_blobs) if blobs_per_body else np.zeros(3)
        xbod = _c(x_bodies)
        v = np.zeros(xf.size)
        self.lib.ref_flow_velocities(_ptr(v), _ptr(xf), _ptr(fs), _ptr(fb), _ptr(xs), _ptr(xbod),
                                     _ptr(xb), xf.size // 3, int(segs_per_body), xbod.size // 3,
                                     int(blobs_per_body), ctypes.c_double(prefac),
                                     int(bool(remove_net_force)))
        return v


class OracleSolver:
    """CPU restatement of the reference's free-body mobility solve
    (tfs_oracle_solve.c): one swimmer, barrier forces, Mss/Mbs, the
    right-preconditioned GMRES saddle-point solve for blob forces and body
    velocity, then Msb."""

    def __init__(self, nfil, nseg, blob_refs, end_force_magnitude: int, tol=1e-10,
                 max_iter=350, mu=1.0, a_seg=1.0, a_blob=1.0, repulsive_force_factor=2.0,
                 threads=1):
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build_oracle()
        self.lib = ctypes.CDLL(path)
        self.lib.orc_solver_create.restype = ctypes.c_void_p
        self.lib.orc_solver_create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, _P, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_int]
        for name in ("orc_solver_destroy", "orc_solver_set_body", "orc_solver_gmres",
                     "orc_solver_make_body_reference_matrices", "orc_solver_compute_velocities",
                     "orc_solver_state", "orc_solver_set_state"):
            getattr(self.lib, name).argtypes = None
        self.lib.orc_set_threads(int(threads))
        self.p = _Params(mu, a_seg, a_blob)
        self.refs = _c(blob_refs)
        self.nblob = self.refs.size // 3
        self.ns = nfil * nseg
        self.h = self.lib.orc_solver_create(ctypes.byref(self.p), nfil, nseg, self.nblob,
                                            _ptr(self.refs), int(end_force_magnitude),
                                            repulsive_force_factor, tol, max_iter)

    def __del__(self):
        try:
            self.lib.orc_solver_destroy(ctypes.c_void_p(self.h))
        except Exception:
            pass

    def set_body(self, x, q):
        x, q = _c(x), _c(q)
        self.lib.orc_solver_set_body(ctypes.c_void_p(self.h), _ptr(x), _ptr(q))

    def make_body_reference_matrices(self, x_segs, f_segs):
        xs, fs = _c(x_segs), _c(f_segs)
        self.lib.orc_solver_make_body_reference_matrices(ctypes.c_void_p(self.h), _ptr(xs), _ptr(fs))
        return self.state()

    def compute_velocities(self, x_segs, f_segs, swimmer_f):
        xs, fs = _c(x_segs), _c(f_segs)
        sf = np.array(swimmer_f, dtype=np.float64).ravel().copy()
        vs = np.zeros(6 * self.ns)
        vb = np.zeros(3 * self.nblob)
        it = self.lib.orc_solver_compute_velocities(ctypes.c_void_p(self.h), _ptr(xs), _ptr(fs),
                                                    _ptr(sf), _ptr(vs), _ptr(vb))
        st = self.state()
        return dict(iters=it, v_segs=vs, v_blobs_rhs=vb, swimmer_f=sf, **st)

    def state(self):
        fb, vb, bm, kt = np.zeros(3 * self.nblob), np.zeros(6), np.zeros(36), np.zeros(36)
        self.lib.orc_solver_state(ctypes.c_void_p(self.h), _ptr(fb), _ptr(vb), _ptr(bm), _ptr(kt))
        return dict(f_blobs=fb, v_bodies=vb, body_mobility=bm, ktkinv=kt)

    def set_state(self, f_blobs=None, v_bodies=None, body_mobility=None, ktkinv=None):
        args = [None if a is None else _c(a) for a in (f_blobs, v_bodies, body_mobility, ktkinv)]
        self.lib.orc_solver_set_state(ctypes.c_void_p(self.h),
                                      *[None if a is None else _ptr(a) for a in args])


class ReferenceSolver:
    """The reference's own mobility_solver.cpp (compute_velocities, GMRES,
    make_body_reference_matrices) compiled for the CPU by `make -C oracle ref`
    with LINEAR_SYSTEM_TOL = 1e-10; single instance per process."""

    def __init__(self, nfil, nseg, blob_refs, end_force_magnitude_real, seg_sep=2.2,
                 body_x=(0, 0, 0), body_q=(1, 0, 0, 0)):
        path = os.path.join(REF_DIR, "libref_solver_s1.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.lib.ref_linear_system_tol.restype = ctypes.c_double
        self.refs = _c(blob_refs)
        self.nblob = self.refs.size // 3
        self.ns = nfil * nseg
        bx, bq = _c(body_x), _c(body_q)
        self.lib.ref_solver_setup(nfil, nseg, self.nblob, ctypes.c_double(end_force_magnitude_real),
                                  ctypes.c_double(seg_sep), _ptr(self.refs), _ptr(bx), _ptr(bq))

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(REF_DIR, "libref_solver_s1.so"))

    def make_body_reference_matrices(self, x_segs, f_segs):
        xs, fs = _c(x_segs), _c(f_segs)
        bm, kt = np.zeros(36), np.zeros(36)
        self.lib.ref_make_body_reference_matrices(_ptr(xs), _ptr(fs), _ptr(bm), _ptr(kt))
        return dict(body_mobility=bm, ktkinv=kt)

    def set_body(self, x, q):
        x, q = _c(x), _c(q)
        self.lib.ref_set_body(_ptr(x), _ptr(q))

    def compute_velocities(self, x_segs, f_segs, swimmer_f, nt=0):
        xs, fs, sf = _c(x_segs), _c(f_segs), _c(swimmer_f)
        vs, vb = np.zeros(6 * self.ns), np.zeros(3 * self.nblob)
        fb, vbod, sfo = np.zeros(3 * self.nblob), np.zeros(6), np.zeros(6)
        it = self.lib.ref_compute_velocities(_ptr(xs), _ptr(fs), _ptr(sf), int(nt), _ptr(vs),
                                             _ptr(vb), _ptr(fb), _ptr(vbod), _ptr(sfo))
        return dict(iters=it, v_segs=vs, v_blobs_rhs=vb, f_blobs=fb, v_bodies=vbod,
                    swimmer_f=sfo)


class ReferenceStep:
    """The reference's implicit time step (cilia_sim_main.cu:355-527 with
    swimmer.cpp, filament.cpp, rigid_body.cpp, segment.cpp,
    broyden_solver.cpp and mobility_solver.cpp compiled unchanged by
    `make -C oracle ref`; LINEAR_SYSTEM_TOL = 1e-10, DT = 1e-3, the
    reference's Broyden TOL 1e-4), for one free swimmer with elastic
    filaments; single instance per process. The pair sums come from the
    pinned C restatement (multi-threaded). The stage methods mirror the main
    loop so tests can compare every stage."""

    def __init__(self, nfil, nseg, blob_refs, fil_refs, fil_dirs, end_force_magnitude_real,
                 seg_sep=2.2, body_length=40.0, body_x=(0, 0, 0), body_q=(1, 0, 0, 0),
                 threads=None, config="s1"):
        """config "s1": DT = 1e-3; "s2": the reference's default DT = 36.3833/300."""
        threads = threads or (os.cpu_count() or 1)
        path = os.path.join(REF_DIR, f"libref_solver_{config}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.lib.ref_linear_system_tol.restype = ctypes.c_double
        self.nfil, self.nseg = nfil, nseg
        self.refs = _c(blob_refs)
        self.nblob = self.refs.size // 3
        self.ns = nfil * nseg
        self.nbroy = 6 * (self.ns + 1)
        fr, fd, bx, bq = _c(fil_refs), _c(fil_dirs), _c(body_x), _c(body_q)
        self.lib.ref_use_port_kernels(int(threads))
        self.lib.ref_step_setup(nfil, nseg, self.nblob, ctypes.c_double(end_force_magnitude_real),
                                ctypes.c_double(seg_sep), ctypes.c_double(body_length),
                                _ptr(self.refs), _ptr(fr), _ptr(fd), _ptr(bx), _ptr(bq))

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(REF_DIR, "libref_solver_s1.so"))

    def make_body_reference_matrices(self):
        bm, kt = np.zeros(36), np.zeros(36)
        self.lib.ref_step_make_body_reference_matrices(_ptr(bm), _ptr(kt))
        return bm, kt

    def initial_guess(self, nt):
        self.lib.ref_step_initial_guess(int(nt))

    def forces(self, nt):
        fs, sf = np.zeros(6 * self.ns), np.zeros(6)
        self.lib.ref_step_forces(int(nt), _ptr(fs), _ptr(sf))
        return fs, sf

    def compute_velocities(self, nt):
        vs, vb, fb = np.zeros(6 * self.ns), np.zeros(6), np.zeros(3 * self.nblob)
        it = self.lib.ref_step_compute_velocities(int(nt), _ptr(vs), _ptr(vb), _ptr(fb))
        return it, vs, vb, fb

    def compute_errors(self, nt, which=0):
        e = np.zeros(self.nbroy)
        big = self.lib.ref_step_compute_errors(int(nt), int(which), _ptr(e))
        return bool(big), e

    def prepare_jacobian_inv(self, nt):
        si = np.zeros(36)
        self.lib.ref_step_prepare_jacobian_inv(int(nt), _ptr(si))
        return si

    def inverse_jacobian(self, i):
        n = 6 * self.nseg
        out = np.zeros(n * n)
        self.lib.ref_step_inverse_jacobian(int(i), _ptr(out))
        return out.reshape(n, n, order="F")

    def jacobian_inv_mult(self, nt, v):
        v = _c(v)
        out = np.zeros(self.nbroy)
        self.lib.ref_step_jacobian_inv_mult(int(nt), _ptr(v), _ptr(out))
        return out

    def broyden_reset(self):
        self.lib.ref_step_broyden_reset()

    def find_update(self, nt):
        u = np.zeros(self.nbroy)
        self.lib.ref_step_find_update(int(nt), _ptr(u))
        return u

    def apply_update(self, nt):
        self.lib.ref_step_apply_update(int(nt))

    def end_of_iter(self, nt, big):
        self.lib.ref_step_end_of_iter(int(nt), int(bool(big)))

    def run(self, nt):
        g = ctypes.c_int(0)
        it = self.lib.ref_step_run(int(nt), ctypes.byref(g))
        return it, g.value

    def write_files(self, prefix, nt):
        """The reference's own plot-step writers after step nt (data files and backup)."""
        self.lib.ref_step_write_files(prefix.encode(), int(nt))

    def state(self):
        ns, nf, sg = self.ns, self.nfil, self.nseg
        out = dict(x=np.zeros(3 * ns), q=np.zeros(4 * ns), u=np.zeros(3 * ns),
                   lam=np.zeros(3 * (sg - 1) * nf), tether=np.zeros(3 * nf),
                   clamp=np.zeros(3 * nf), body_x=np.zeros(3), body_q=np.zeros(4),
                   body_u=np.zeros(3))
        self.lib.ref_step_state(*[_ptr(out[k]) for k in ("x", "q", "u", "lam", "tether", "clamp",
                                                         "body_x", "body_q", "body_u")])
        return out


class ReferencePrescribed:
    """The reference's prescribed-cilia mobility solve (mobility_solver.cpp
    compute_velocities, assemble_rhs, solve_linear_system,
    apply_preconditioner_new and system_matrix_mult_new under PRESCRIBED_CILIA,
    with swimmer::make_precon_mat) compiled for the CPU by `make -C oracle ref`
    in one of the configurations p1, p2, p3 (oracle/Makefile); FP64, GMRES
    tolerance 1e-10; single instance per process."""

    FLAG_NAMES = {1: "prescribed_body", 2: "dynamic_phase", 4: "dynamic_angle", 8: "weakly_coupled"}

    def __init__(self, config, nfil, nseg, blob_refs, seg_sep, body_x, body_q, phase_refs=(),
                 angle_refs=()):
        path = os.path.join(REF_DIR, f"libref_pres_{config}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.nfil, self.nseg = nfil, nseg
        self.ns = nfil * nseg
        self.refs = _c(blob_refs)
        self.nblob = self.refs.size // 3
        pr, ar = _c(phase_refs if len(phase_refs) else [0.0]), _c(angle_refs if len(angle_refs) else [0.0])
        bx, bq = _c(body_x), _c(body_q)
        scratch = os.path.join(REF_DIR, "scratch")  # the tables' temporary directory
        os.makedirs(scratch, exist_ok=True)
        rc = self.lib.ref_pres_setup(nfil, nseg, self.nblob, ctypes.c_double(seg_sep),
                                     _ptr(self.refs), _ptr(bx), _ptr(bq), _ptr(pr), len(phase_refs),
                                     _ptr(ar), len(angle_refs), scratch.encode())
        if rc != 0:
            raise RuntimeError("ref_pres_setup failed")
        self.flags = self.lib.ref_pres_flags()
        self.n = self.lib.ref_pres_system_size()

    @staticmethod
    def available(config="p1") -> bool:
        return os.path.exists(os.path.join(REF_DIR, f"libref_pres_{config}.so"))

    def set_kinematics(self, x_segs, vel_dir_phase, vel_dir_angle, phase, omega0, angle, phase_dot):
        arrs = [_c(a) for a in (x_segs, vel_dir_phase, vel_dir_angle, phase, omega0, angle,
                                phase_dot)]
        self.lib.ref_pres_set_kinematics(*[_ptr(a) for a in arrs])

    def set_rates(self, phase_dot, angle_dot):
        p, a = _c(phase_dot), _c(angle_dot)
        self.lib.ref_pres_set_rates(_ptr(p), _ptr(a))

    def ktminvk(self):
        out = np.zeros(36)
        self.lib.ref_pres_ktminvk(_ptr(out))
        return out

    def rhs(self, nt=0):
        out = np.zeros(self.n)
        self.lib.ref_pres_rhs(int(nt), _ptr(out))
        return out

    def apply(self, which, v):
        v = _c(v)
        out = np.zeros(self.n)
        self.lib.ref_pres_apply(int(which), _ptr(v), _ptr(out))
        return out

    def compute_velocities(self, nt=0):
        fs, fb = np.zeros(3 * self.ns), np.zeros(3 * self.nblob)
        vb, pd, ad = np.zeros(6), np.zeros(self.nfil), np.zeros(self.nfil)
        it = self.lib.ref_pres_compute_velocities(int(nt), _ptr(fs), _ptr(fb), _ptr(vb), _ptr(pd),
                                                  _ptr(ad))
        return dict(iters=it, f_segs=fs, f_blobs=fb, v_body=vb, phase_dot=pd, angle_dot=ad)
