"""GPU parity of the prescribed-cilia solve (tfs_prescribed_*) against the
reference's own solver in three prescribed-cilia configurations
(tests/golden/prescribed_p*.npz: mobility_solver.cpp under PRESCRIBED_CILIA,
LINEAR_SYSTEM_TOL = 1e-10) and against the CPU restatement
(oracle/prescribed.py) on a larger swimmer.

Tolerances:
  pieces (right-hand side, operator, preconditioner, KTMinvK_inv), FP64:
  relative max-abs error <= 1e-12 (the pair sums differ from the reference's
  sequential order only by rounding);
  solves: <= 1e-8 relative max-abs error (two GMRES runs stopped at a 1e-10
  relative residual agree to about cond(A) x 1e-10); FP64 GMRES iteration
  counts within one of the reference's. FP32C (inner solves with FP32 pair
  sums, refined on FP64 residuals): FP64 residual <= 1e-10 as the
  reference's, solutions within 5e-6 (two solutions with residuals below
  1e-10 ||b|| differ by at most cond(A) x 2e-10 ~ 5e-6 for these systems,
  whose condition number is ~2.6e4 (tests/test_prescribed_oracle.py);
  measured 2e-8 to 4e-7).
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CONFIGS = ("p1", "p2", "p3", "p4", "p5", "p6")

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def load(cfg):
    return dict(np.load(os.path.join(GOLD, f"prescribed_{cfg}.npz")))


def make(d, tol=1e-10, precision="fp64"):
    from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver
    return PrescribedCiliaSolver(int(d["flags"]), int(d["nfil"]), int(d["nseg"]), d["blob_refs"],
                                 float(d["seg_sep"]), d["phase_refs"], d["angle_refs"],
                                 body_x=d["body_x"], body_q=d["body_q"], tol=tol,
                                 precision=precision,
                                 gen_force_magnitude_factor=float(d["gen_force_magnitude_factor"]),
                                 torsional_spring_magnitude_factor=float(
                                     d["torsional_spring_magnitude_factor"]))


def kin(d, nt):
    return dict(x_segs=d["x_segs"][nt], vel_dir_phase=d["vel_dir_phase"][nt],
                vel_dir_angle=d["vel_dir_angle"][nt], phase=d["phase"][nt], omega0=d["omega0"],
                shape_rotation_angle=d["angle"][nt], phase_dot=d["omega0"])


@pytest.mark.parametrize("cfg", CONFIGS)
def test_pieces_match_reference(cfg):
    d = load(cfg)
    ps = make(d)
    assert ps.n == int(d["n"])
    ps.set_kinematics(**kin(d, 0))
    assert rel(ps.apply("rhs"), d["rhs0"]) <= 1e-12
    assert rel(ps.apply("operator", d["v_in"]), d["a_v"]) <= 1e-12
    assert rel(ps.apply("preconditioner", d["v_in"]), d["pinv_v"]) <= 1e-12
    if not int(d["flags"]) & 1:  # free body: swimmer.KTMinvK_inv
        assert rel(ps.precon_matrix(), d["ktminvk"]) <= 1e-12
    ps.finalise()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_warm_started_solves_match_reference(cfg, precision):
    """Three consecutive solves, each warm started from the last (the first
    from phase rates omega0 and zero angle rates, as the golden's). FP32C:
    the refinement drives the FP64 residual to the same tolerance, so the
    same bar holds; its iteration count is the inner steps' sum."""
    d = load(cfg)
    ps = make(d, precision=precision)
    ps.set_solution(phase_dot=d["phase_dot0"], angle_dot=d["angle_dot0"])
    flags = int(d["flags"])
    for nt in range(d["phase"].shape[0]):
        iters = ps.compute_velocities(**kin(d, nt))
        if precision == "fp64":
            assert abs(iters - int(d["iters"][nt])) <= 1, (nt, iters, int(d["iters"][nt]))
        else:
            assert ps.solve_info()["rel_residual"] <= 1e-10
        sol = ps.solution()
        bar = 1e-8 if precision == "fp64" else 5e-6
        assert rel(sol["f_segs"], d["f_segs"][nt]) <= bar
        assert rel(sol["f_blobs"], d["f_blobs"][nt]) <= bar
        if not flags & 1:
            assert rel(sol["v_body"], d["v_body"][nt]) <= bar
        if flags & 2:
            assert rel(sol["phase_dot"], d["phase_dot"][nt]) <= bar
        if flags & 4:
            assert rel(sol["angle_dot"], d["angle_dot"][nt]) <= bar
    ps.finalise()


def test_zero_rhs_gives_zero_solution():
    """A zero right-hand side (no prescribed rates, no generalised forces)
    zeroes the whole solution and takes no GMRES step
    (mobility_solver.cpp:2121-2200)."""
    d = load("p3")
    ps = make(d)
    ps.set_solution(f_segs=np.ones(3 * int(d["nfil"]) * int(d["nseg"])))
    k = kin(d, 0)
    k["phase_dot"] = np.zeros_like(d["omega0"])
    assert ps.compute_velocities(**k) == 0
    sol = ps.solution()
    assert np.all(sol["f_segs"] == 0.0) and np.all(sol["f_blobs"] == 0.0)
    assert np.all(sol["v_body"] == 0.0)
    ps.finalise()


@pytest.mark.parametrize("flags", [0, 6, 15])
def test_larger_swimmer_vs_oracle(flags):
    """160 filaments x 20 segments on a 642-blob sphere (3 842 particles):
    the operator and preconditioner against the CPU restatement, and the
    solve's residual ||b - A x|| <= 1e-10 ||b|| through the GPU operator."""
    from prescribed import PrescribedSystem
    from timfilsimmod_gb300.geometry import prescribed_swimmer
    from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver
    g = prescribed_swimmer(160, 20, radius=20.0, subdivisions=3, seg_sep=2.2)
    rng = np.random.default_rng(3)
    q = np.array([0.9, -0.1, 0.3, 0.2])
    q /= np.linalg.norm(q)
    bx = np.array([1.0, 2.0, -0.5])
    phase = rng.uniform(0, 2 * np.pi, g.nfil)
    angle = rng.uniform(-0.2, 0.2, g.nfil)
    omega0 = 2 * np.pi * (1 + 0.1 * rng.uniform(-1, 1, g.nfil))
    x, vp, va = g.kinematics(phase, angle, bx, q)
    t = 2 * np.pi * np.arange(64) / 64
    tp, ta = 1 + 0.4 * np.sin(t), 0.2 * np.cos(t)
    ps = PrescribedCiliaSolver(flags, g.nfil, g.nseg, g.blob_references, g.seg_sep, tp, ta,
                               body_x=bx, body_q=q, tol=1e-10)
    k = dict(x_segs=x, vel_dir_phase=vp, vel_dir_angle=va, phase=phase, omega0=omega0,
             shape_rotation_angle=angle, phase_dot=omega0)
    ps.set_kinematics(**k)
    S = PrescribedSystem(flags, g.nfil, g.nseg, x, g.blob_references, bx, q, vp, va)
    S.orc.set_threads(os.cpu_count() or 1)
    v = rng.normal(size=ps.n)
    assert rel(ps.apply("operator", v), S.apply_a(v)) <= 1e-12
    assert rel(ps.apply("preconditioner", v), S.apply_pinv(v)) <= 1e-12
    b = ps.apply("rhs")
    assert rel(b, S.rhs(phase, omega0, angle, omega0, tp, ta,
                        fil_length=g.seg_sep * (g.nseg - 1))) <= 1e-13
    iters = ps.solve()
    assert 0 < iters < 350
    sol = ps.solution()
    xs = np.concatenate([sol["f_segs"].ravel(), sol["f_blobs"].ravel()]
                        + ([sol["v_body"]] if not flags & 1 else [])
                        + ([sol["phase_dot"]] if flags & 2 else [])
                        + ([sol["angle_dot"]] if flags & 4 else []))
    assert np.linalg.norm(b - ps.apply("operator", xs)) <= 1.5e-10 * np.linalg.norm(b)
    ps.finalise()


def test_flag_validation():
    """Free body with only one of the dynamic flags is rejected (the
    reference's free-body preconditioner indexes both)."""
    from timfilsimmod_gb300 import _native as N
    d = load("p1")
    with pytest.raises(N.TfsError):
        from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver
        PrescribedCiliaSolver(2, int(d["nfil"]), int(d["nseg"]), d["blob_refs"],
                              float(d["seg_sep"]), d["phase_refs"], d["angle_refs"])


@pytest.mark.parametrize("cfg", ["p1", "p2"])
def test_block_hooks_take_the_prescribed_form(cfg):
    """After the prescribed setup the four block hooks are the reference's
    PRESCRIBED_CILIA kernels (cuda_functions.cu:362-757): 3x3 pairs on the
    forces only (the torque slots of f_segs, here random, are not read), zero
    rotational segment velocities, Mbs adding to Mbb's result. Checked
    through evaluate_full_mobility against the CPU restatement's blocks."""
    from prescribed import PrescribedSystem
    d = load(cfg)
    ps = make(d)
    ps.set_kinematics(**kin(d, 0))
    s = ps.solver
    nfil, nseg = int(d["nfil"]), int(d["nseg"])
    ns, nb = nfil * nseg, d["blob_refs"].size // 3
    rng = np.random.default_rng(9)
    s.f_segs_host[:] = rng.normal(size=6 * ns)
    s.f_blobs_host[:] = rng.normal(size=3 * nb)
    s.copy_segment_forces_to_device()
    s.copy_blob_forces_to_device()
    s.evaluate_full_mobility()
    S = PrescribedSystem(int(d["flags"]), nfil, nseg, d["x_segs"][0], d["blob_refs"], d["body_x"],
                         d["body_q"], d["vel_dir_phase"][0], d["vel_dir_angle"][0])
    o = S.orc
    fs3 = s.f_segs_host.reshape(-1, 6)[:, :3].copy()
    fb = s.f_blobs_host.copy()
    vs = o.block(3, 3, S.x_segs, 1.0, S.x_segs, fs3, 1.0)
    vs = o.block(3, 3, S.x_segs, 1.0, S.x_blobs, fb, 1.0, v=vs)
    vb = o.block(3, 3, S.x_blobs, 1.0, S.x_blobs, fb, 1.0)
    vb = o.block(3, 3, S.x_blobs, 1.0, S.x_segs, fs3, 1.0, v=vb)
    v6 = s.v_segs_host.reshape(-1, 6)
    assert rel(v6[:, :3], vs) <= 1e-12
    assert np.all(v6[:, 3:] == 0.0)
    assert rel(s.v_blobs_host, vb) <= 1e-12
    ps.finalise()


@pytest.mark.parametrize("flags", [0, 7])
def test_filaments_without_blobs(flags):
    """A body without blobs (NBLOB = 0): the operator, preconditioner and
    right-hand side against the CPU restatement, and a solve to its
    residual; the blob parts of the solution are empty."""
    from prescribed import PrescribedSystem
    from timfilsimmod_gb300.geometry import prescribed_swimmer
    from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver
    g = prescribed_swimmer(6, 8, radius=8.0, subdivisions=1, seg_sep=2.6)
    refs = np.zeros((0, 3))
    rng = np.random.default_rng(4)
    phase = rng.uniform(0, 2 * np.pi, g.nfil)
    angle = rng.uniform(-0.2, 0.2, g.nfil)
    omega0 = 2 * np.pi * np.ones(g.nfil)
    x, vp, va = g.kinematics(phase, angle)
    t = 2 * np.pi * np.arange(32) / 32
    tp, ta = 1 + 0.3 * np.sin(t), 0.1 * np.cos(t)
    ps = PrescribedCiliaSolver(flags, g.nfil, g.nseg, refs, g.seg_sep, tp, ta, tol=1e-10)
    k = dict(x_segs=x, vel_dir_phase=vp, vel_dir_angle=va, phase=phase, omega0=omega0,
             shape_rotation_angle=angle, phase_dot=omega0)
    ps.set_kinematics(**k)
    S = PrescribedSystem(flags, g.nfil, g.nseg, x, refs, (0, 0, 0), (1, 0, 0, 0), vp, va)
    assert ps.n == S.n
    v = rng.normal(size=ps.n)
    assert rel(ps.apply("operator", v), S.apply_a(v)) <= 1e-12
    assert rel(ps.apply("preconditioner", v), S.apply_pinv(v)) <= 1e-12
    b = ps.apply("rhs")
    assert rel(b, S.rhs(phase, omega0, angle, omega0, tp, ta,
                        fil_length=g.seg_sep * (g.nseg - 1))) <= 1e-13
    ps.solve()
    sol = ps.solution()
    assert sol["f_blobs"].size == 0
    x_sol, _ = S.solve(b, np.zeros(S.n), tol=1e-10)
    assert rel(sol["f_segs"], x_sol[:3 * g.nfil * g.nseg]) <= 1e-6
    ps.finalise()


def test_error_paths():
    """Calls out of order and missing kinematics fail with the library's
    status and leave the solver usable: a solve before any kinematics
    (ESTATE), dynamic shape rotation without d x / d angle (EINVAL), dynamic
    phase without its table (EINVAL)."""
    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver
    d = load("p1")
    ps = make(d)
    with pytest.raises(N.TfsError) as e:
        ps.solve()
    assert e.value.code == N.TFS_ESTATE
    k = kin(d, 0)
    k["vel_dir_angle"] = None
    with pytest.raises(N.TfsError) as e:
        ps.set_kinematics(**k)
    assert e.value.code == N.TFS_EINVAL
    ps.set_kinematics(**kin(d, 0))  # still usable
    assert ps.solve() > 0
    ps.finalise()
    with pytest.raises(N.TfsError) as e:
        PrescribedCiliaSolver(7, int(d["nfil"]), int(d["nseg"]), d["blob_refs"],
                              float(d["seg_sep"]), None, d["angle_refs"])
    assert e.value.code == N.TFS_EINVAL
