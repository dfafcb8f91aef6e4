"""GPU parity of the device-resident free-body solve (compute_velocities,
GMRES, make_body_reference_matrices) against the reference's own
mobility_solver.cpp (golden vectors, LINEAR_SYSTEM_TOL = 1e-10) and the CPU
oracle.

Tolerances (GMRES stops at a relative residual of 1e-10, so two correct
implementations agree to about that level, not to rounding):
  FP64:  max-abs error <= 1e-8 x max-abs reference value; GMRES iteration
         counts within 1 of the reference's
  FP32C: the pairwise sums (Mss, Mbs, Msb and the blob-blob products inside
         GMRES) run in FP32 with compensated accumulation, so results carry
         their ~1e-6 relative error: <= 2e-5; the linear system itself is
         refined to the FP64 residual tolerance (checked). "fp32c" runs each
         inner GMRES as one cooperative kernel (the default), "fp32c_kernels"
         as a sequence of kernels per Arnoldi step; both meet the same bars.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-8
TOLS = {"fp64": 1e-8, "fp32c": 2e-5, "fp32c_kernels": 2e-5}
FORMS = ["fp64", "fp32c", "fp32c_kernels"]

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def load(name):
    return np.load(os.path.join(GOLD, f"{name}.npz"))


def new_solver(nfil, nseg, nblob, form, **kw):
    """A solver in one of FORMS."""
    from timfilsimmod_gb300.mobility import RpyMobilitySolver

    s = RpyMobilitySolver(1, nfil, nseg, nblob, precision=form.split("_")[0], **kw)
    if form == "fp32c":
        s.set_persistent_gmres(True)  # raises if the cooperative kernel cannot run
    elif form == "fp32c_kernels":
        s.set_persistent_gmres(False)
    return s


def make_solver(d, precision):
    s = new_solver(int(d["nfil"]), int(d["nseg"]), d["blob_refs"].shape[0], precision,
                   end_force_magnitude=int(d["end_force_magnitude"]))
    s.set_blob_references(d["blob_refs"])
    s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
    s.set_linear_solver(float(d["tol"]))
    return s


def set_segments(s, xs, fs):
    s.x_segs_host[:] = np.asarray(xs).ravel()
    s.f_segs_host[:] = np.asarray(fs).ravel()
    s.copy_segment_positions_to_device()
    s.copy_segment_forces_to_device()


@pytest.mark.parametrize("precision", FORMS)
def test_solve_sequence_matches_reference(precision):
    d = load("solve_small")
    s = make_solver(d, precision)
    set_segments(s, d["x_segs"], d["f_segs"])
    bm, kt = s.make_body_reference_matrices()
    assert rel_max(kt, d["bodyref_ktkinv"]) < 1e-12
    assert rel_max(bm, d["bodyref_body_mobility"]) < TOLS[precision]
    # first step: body at the origin
    set_segments(s, d["x_segs"], d["f_segs"])
    it1, sf1 = s.compute_velocities(d["cv1_swimmer_f_in"])
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    out1 = dict(v_segs=s.v_segs_host.copy(), f_blobs=s.blob_forces(), v_bodies=s.body_velocities())
    # second step: moved and rotated body, new forces, warm start from the first
    s.set_body_pose(d["cv2_body_x"], d["cv2_body_q"])
    set_segments(s, d["cv2_x_segs"], d["cv2_f_segs"])
    it2, sf2 = s.compute_velocities(d["cv2_swimmer_f_in"])
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    out2 = dict(v_segs=s.v_segs_host.copy(), f_blobs=s.blob_forces(), v_bodies=s.body_velocities())
    info = s.solve_info()
    s.finalise()
    print(precision, "iters", it1, it2, "ref", int(d["cv1_iters"]), int(d["cv2_iters"]), info)
    assert rel_max(sf1, d["cv1_swimmer_f"]) < 1e-12
    assert rel_max(sf2, d["cv2_swimmer_f"]) < 1e-12
    for k in ("v_segs", "f_blobs", "v_bodies"):
        e1, e2 = rel_max(out1[k], d[f"cv1_{k}"]), rel_max(out2[k], d[f"cv2_{k}"])
        print(precision, k, e1, e2)
        assert e1 < TOLS[precision] and e2 < TOLS[precision], (k, e1, e2)
    if precision == "fp64":
        assert abs(it1 - int(d["cv1_iters"])) <= 1 and abs(it2 - int(d["cv2_iters"])) <= 1
    assert info["rel_residual"] <= float(d["tol"])


def test_zero_rhs_and_warm_start_exit():
    d = load("solve_small")
    s = make_solver(d, "fp64")
    n = 3 * d["blob_refs"].shape[0] + 6
    assert s.solve_linear_system(np.zeros(n)) == 0
    assert np.all(s.body_velocities() == 0) and np.all(s.blob_forces() == 0)
    rhs = np.random.default_rng(3).normal(size=n)
    # at a tolerance well above rounding, the GMRES residual estimate and the
    # true residual of the solution agree: a second solve of the same system
    # starts from the first one's solution and exits before iterating
    # (mobility_solver.cpp:2304-2307)
    s.set_linear_solver(1e-6)
    it = s.solve_linear_system(rhs)
    assert it > 0
    assert s.solve_linear_system(rhs) == 0
    s.finalise()


@pytest.mark.parametrize("precision", FORMS)
def test_medium_swimmer_solve_vs_oracle(precision):
    """compute_velocities of the medium swimmer (12 800 segments, 2562 blobs)
    against the oracle's restatement, at LINEAR_SYSTEM_TOL = 1e-10, after
    make_body_reference_matrices as the reference runs it; the oracle gets the
    same body matrices and warm start."""
    from oracle import OracleSolver

    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=3)
    efm = int(220.0 * 1800.0 / (2.6 * 2.6 * sw.nseg ** 2))
    F = sw.f_segs[:, :3].sum(0)
    T = (np.cross(sw.x_segs, sw.f_segs[:, :3]) + sw.f_segs[:, 3:]).sum(0)
    sf = np.concatenate([F, T])
    s = new_solver(sw.nfil, sw.nseg, sw.num_blobs, precision, end_force_magnitude=efm)
    s.set_blob_references(sw.blob_references)
    s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
    s.set_linear_solver(1e-10)
    set_segments(s, sw.x_segs, sw.f_segs)
    bm, kt = s.make_body_reference_matrices()
    warm_f, warm_v = s.blob_forces(), s.body_velocities()
    it, sf_out = s.compute_velocities(sf)
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    vs, fb, vb = s.v_segs_host.copy(), s.blob_forces(), s.body_velocities()
    s.finalise()
    # Stokes drag of the blob sphere (R = 60): the reference's start-up check
    # (mobility_solver.cpp:3017-3033); a discretised sphere is within a few %
    R = 60.0
    drag = np.array([1 / (6 * np.pi * R)] * 3 + [1 / (8 * np.pi * R ** 3)] * 3)
    assert np.allclose(bm.reshape(6, 6).T.diagonal(), drag, rtol=0.05)
    o = OracleSolver(sw.nfil, sw.nseg, sw.blob_references, efm, tol=1e-10,
                     threads=os.cpu_count() or 1)
    o.set_state(f_blobs=warm_f, v_bodies=warm_v, body_mobility=bm, ktkinv=kt)
    r = o.compute_velocities(sw.x_segs, sw.f_segs, sf)
    print(precision, "iters", it, r["iters"])
    assert rel_max(sf_out, r["swimmer_f"]) < 1e-12
    # two correct GMRES runs that stop at a relative residual of 1e-10 one
    # iteration apart differ by that residual times the conditioning of the
    # saddle-point system (~1e4 here): bound at 1e-6 for FP64
    tol = {"fp64": 1e-6, "fp32c": 2e-5, "fp32c_kernels": 2e-5}[precision]
    for k, v in (("v_segs", vs), ("f_blobs", fb), ("v_bodies", vb)):
        e = rel_max(v, r[k])
        print(precision, k, e)
        assert e < tol, (k, e)
    if precision == "fp64":
        assert abs(it - r["iters"]) <= 1


def test_persistent_and_kernel_sequence_agree():
    """The cooperative-kernel inner GMRES and the kernel-sequence one solve
    the same refinement: same results to the FP32 product error, iteration
    totals within a few (their FP32 sums round differently)."""
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=11)
    F = sw.f_segs[:, :3].sum(0)
    T = (np.cross(sw.x_segs, sw.f_segs[:, :3]) + sw.f_segs[:, 3:]).sum(0)
    out = {}
    for form in ("fp32c", "fp32c_kernels"):
        s = new_solver(sw.nfil, sw.nseg, sw.num_blobs, form)
        s.set_blob_references(sw.blob_references)
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        s.set_linear_solver(1e-8)
        set_segments(s, sw.x_segs, sw.f_segs)
        bm, _ = s.make_body_reference_matrices()
        it, _ = s.compute_velocities(np.concatenate([F, T]))
        s.copy_segment_velocities_to_host()
        s.wait_for_device()
        out[form] = (it, s.v_segs_host.copy(), s.blob_forces(), s.body_velocities(), bm,
                     s.solve_info())
        s.finalise()
    a, b = out["fp32c"], out["fp32c_kernels"]
    print("iters", a[0], b[0], a[5], b[5])
    assert a[5]["rel_residual"] <= 1e-8 and b[5]["rel_residual"] <= 1e-8
    assert abs(a[0] - b[0]) <= max(3, b[0] // 10)
    for x, y in zip(a[1:5], b[1:5]):
        assert rel_max(x, y) < 2e-5


def test_refinement_vector_modes_agree():
    """FP32C Arnoldi vectors in FP32 (the default) and FP64: each mode
    refines the medium swimmer's solve to the FP64 residual target, and their
    solutions agree to the FP32 product error. An unknown mode is refused
    with TFS_EINVAL."""
    from timfilsimmod_gb300._native import TFS_EINVAL, TfsError
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=11)
    F = sw.f_segs[:, :3].sum(0)
    T = (np.cross(sw.x_segs, sw.f_segs[:, :3]) + sw.f_segs[:, 3:]).sum(0)
    out = {}
    for mode in ("fp32", "fp64"):
        s = new_solver(sw.nfil, sw.nseg, sw.num_blobs, "fp32c")
        s.set_refinement_vectors(mode)
        s.set_blob_references(sw.blob_references)
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        s.set_linear_solver(1e-8)
        set_segments(s, sw.x_segs, sw.f_segs)
        s.make_body_reference_matrices()
        it, _ = s.compute_velocities(np.concatenate([F, T]))
        s.copy_segment_velocities_to_host()
        s.wait_for_device()
        out[mode] = (it, s.v_segs_host.copy(), s.blob_forces(), s.body_velocities(),
                     s.solve_info())
        if mode == "fp32":
            with pytest.raises(TfsError) as e:
                s._call("tfs_set_refinement_vectors", 2)
            assert e.value.code == TFS_EINVAL
        s.finalise()
    print({m: (v[0], v[4]) for m, v in out.items()})
    for mode, v in out.items():
        assert v[4]["rel_residual"] <= 1e-8 and v[4]["cycles"] > 0, mode
        for x, y in zip(v[1:4], out["fp32"][1:4]):
            assert rel_max(x, y) < 2e-5, mode


def test_persistent_large_slices_agree():
    """10 242 blobs (the large swimmer's body, R = 150) with 64 filaments: 68
    blobs per cooperative CTA on 152 SMs, beyond the 64 of the smaller
    swimmers' slices. The cooperative inner GMRES and the kernel sequence
    reach the same refined solve, as at the medium swimmer."""
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("large", seed=3, nfil=64, shape="straight")
    F = sw.f_segs[:, :3].sum(0)
    T = (np.cross(sw.x_segs, sw.f_segs[:, :3]) + sw.f_segs[:, 3:]).sum(0)
    out = {}
    for form in ("fp32c", "fp32c_kernels"):
        s = new_solver(sw.nfil, sw.nseg, sw.num_blobs, form)
        s.set_blob_references(sw.blob_references)
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        s.set_linear_solver(1e-8)
        set_segments(s, sw.x_segs, sw.f_segs)
        bm, _ = s.make_body_reference_matrices()
        it, _ = s.compute_velocities(np.concatenate([F, T]))
        s.copy_segment_velocities_to_host()
        s.wait_for_device()
        out[form] = (it, s.v_segs_host.copy(), s.blob_forces(), s.body_velocities(), bm,
                     s.solve_info(), s.refinement_retries())
        s.finalise()
    a, b = out["fp32c"], out["fp32c_kernels"]
    print("iters", a[0], b[0], a[5], b[5], "retries", a[6])
    assert a[5]["rel_residual"] <= 1e-8 and b[5]["rel_residual"] <= 1e-8
    assert a[5]["cycles"] > 0 and a[6] == 0  # refined with FP32 vectors, no fallback
    assert abs(a[0] - b[0]) <= max(3, b[0] // 10)
    for x, y in zip(a[1:5], b[1:5]):
        assert rel_max(x, y) < 2e-5


def test_barrier_stall_times_out_and_solver_recovers():
    """Fault injection on the host: the cooperative inner GMRES's grid
    barriers wait for one CTA more than the launch has. Every wait runs out
    its bound (2 s of globaltimer), the kernel ends with an error status, the
    solve raises TFS_ETIMEOUT, and the same solver -- the injection removed --
    then solves bit for bit as a solver that never failed (the context stays
    usable; a failed refinement leaves the warm start untouched)."""
    import time

    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=11)
    F = sw.f_segs[:, :3].sum(0)
    T = (np.cross(sw.x_segs, sw.f_segs[:, :3]) + sw.f_segs[:, 3:]).sum(0)
    sf = np.concatenate([F, T])

    def setup():
        s = new_solver(sw.nfil, sw.nseg, sw.num_blobs, "fp32c")
        s.set_blob_references(sw.blob_references)
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        s.set_linear_solver(1e-8)
        set_segments(s, sw.x_segs, sw.f_segs)
        s.make_body_reference_matrices()
        return s

    def result(s):
        # compute_velocities adds the barrier forces into the device's segment
        # forces (as the reference's apply_interparticle_forces does): upload
        # them afresh before each call
        set_segments(s, sw.x_segs, sw.f_segs)
        it, sf_out = s.compute_velocities(sf)
        s.copy_segment_velocities_to_host()
        s.wait_for_device()
        return it, sf_out, s.v_segs_host.copy(), s.blob_forces(), s.body_velocities()

    clean = setup()
    want = result(clean)
    clean.finalise()

    s = setup()
    s.inject_barrier_stall(True)
    t0 = time.perf_counter()
    with pytest.raises(N.TfsError) as e:
        result(s)
    took = time.perf_counter() - t0
    assert e.value.code == N.TFS_ETIMEOUT, e.value
    assert 1.5 < took < 60.0, took
    s.inject_barrier_stall(False)
    got = result(s)
    assert got[0] == want[0]
    for x, y in zip(got[1:], want[1:]):
        assert np.array_equal(x, y)
    s.finalise()
