"""GPU parity of the implicit time step (tfs_stepper_*, timfilsimmod_gb300.stepper)
against the reference's own time step (cilia_sim_main.cu:355-527 with
swimmer.cpp, filament.cpp, rigid_body.cpp, broyden_solver.cpp and
mobility_solver.cpp compiled unchanged; tests/golden/step_small.npz): the
small swimmer (642 blobs, 32 x 20 segments), DT = 1e-3, Broyden TOL = 1e-4,
LINEAR_SYSTEM_TOL = 1e-10.

Tolerances. Stages that do not pass through GMRES (initial guess, internal
forces, inverse approximate Jacobians) agree to rounding: <= 1e-12 of the
largest reference value. Stages after a mobility solve carry its 1e-10
relative residual: velocities and everything computed from them <= 1e-8
(residual vectors, whose entries are differences of nearly equal terms,
<= 1e-6 of their largest entry). Over ten whole steps the Broyden
iteration counts must match and segment positions and body pose agree to
<= 1e-10 of the largest reference position (body pose: <= 1e-10 of the
body radius; quaternions <= 1e-10). FP32C steps (FP32 pairwise sums,
compensated, inside an FP64-refined solve) keep segment positions within
1e-8 of the largest reference position.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def load():
    return np.load(os.path.join(GOLD, "step_small.npz"))


def make(d, precision="fp64"):
    from timfilsimmod_gb300.mobility import RpyMobilitySolver
    from timfilsimmod_gb300.stepper import ImplicitStepper

    nfil, nseg = int(d["nfil"]), int(d["nseg"])
    efm = float(d["end_force_magnitude_real"])
    s = RpyMobilitySolver(1, nfil, nseg, d["blob_refs"].shape[0], precision=precision,
                          end_force_magnitude=int(efm))
    s.set_blob_references(d["blob_refs"])
    s.set_linear_solver(float(d["linear_tol"]))
    st = ImplicitStepper(s, nfil, nseg, d["fil_refs"], d["fil_dirs"], seg_sep=2.2,
                         dt=float(d["dt"]), tol=float(d["tol"]), end_force_magnitude=efm,
                         body_radius=float(d["body_radius"]))
    return s, st


def device_copy(view):
    import torch

    return torch.as_tensor(view, device="cuda").cpu().numpy().copy()


def test_step_zero_stage_by_stage():
    d = load()
    s, st = make(d)
    bm, kt = s.body_reference_matrices()
    assert rel_max(kt, d["ktkinv"]) < 1e-12
    assert rel_max(bm, d["body_mobility"]) < 1e-8
    nt = 0
    st.initial_guess(nt)
    assert rel_max(st.state()["x"], d["s0_guess"]) < 1e-14
    sf = st.forces_and_torques(nt)
    fs = device_copy(s.device_arrays()["f_segs"])
    assert rel_max(fs, d["s0_f_segs"]) < 1e-12
    assert rel_max(sf, d["s0_swimmer_f"]) < 1e-12
    it = st.compute_velocities(nt)
    assert abs(it - int(d["s0_gmres"])) <= 2, (it, int(d["s0_gmres"]))
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    assert rel_max(s.v_segs_host, d["s0_v_segs"]) < 1e-8
    assert rel_max(s.body_velocities(), d["s0_v_bodies"]) < 1e-8
    assert rel_max(s.blob_forces(), d["s0_f_blobs"]) < 1e-8
    big, err = st.compute_errors(nt, 0)
    assert big == bool(d["s0_big"])
    assert rel_max(err, d["s0_error"]) < 1e-6, rel_max(err, d["s0_error"])
    si = st.prepare_jacobian_inv(nt)
    assert rel_max(si, d["s0_schur_inv"]) < 1e-8, rel_max(si, d["s0_schur_inv"])
    jf = st.inverse_jacobian(0)
    assert rel_max(jf, d["s0_jinv_first"]) < 1e-12, rel_max(jf, d["s0_jinv_first"])
    jl = st.inverse_jacobian(int(d["nfil"]) - 1)[:12]
    assert rel_max(jl, d["s0_jinv_last_rows"]) < 1e-12
    out = st.jacobian_inv_mult(nt, d["s0_probe"])
    assert rel_max(out, d["s0_probe_out"]) < 1e-8, rel_max(out, d["s0_probe_out"])
    st.broyden_reset()
    upd = st.find_update(nt)
    assert rel_max(upd, d["s0_update0"]) < 1e-6, rel_max(upd, d["s0_update0"])
    st.update(nt)
    assert rel_max(st.state()["x"], d["s0_state0_x"]) < 1e-10
    st.compute_velocities(nt)
    big, nerr = st.compute_errors(nt, 1)
    assert rel_max(nerr, d["s0_new_error0"]) < 1e-6, rel_max(nerr, d["s0_new_error0"])
    st.end_of_iter(nt, big)
    st.close()
    s.finalise()


def run_steps(d, precision):
    s, st = make(d, precision)
    broy, states = [], []
    for nt in range(10):
        b, _ = st.step(nt)
        broy.append(b)
        states.append(st.state())
    st.close()
    s.finalise()
    return broy, states


def test_ten_steps_match_reference_fp64():
    d = load()
    broy, states = run_steps(d, "fp64")
    assert broy == list(d["broyden_iters"]), (broy, list(d["broyden_iters"]))
    scale = np.max(np.abs(d["traj_x_last"]))
    assert np.max(np.abs(states[0]["x"] - d["traj_x_first"])) / scale < 1e-10
    assert np.max(np.abs(states[-1]["x"] - d["traj_x_last"])) / scale < 1e-10
    R = float(d["body_radius"])
    for nt, stt in enumerate(states):
        assert np.max(np.abs(stt["body_x"] - d["traj_body_x"][nt])) / R < 1e-10, nt
        assert np.max(np.abs(stt["body_q"] - d["traj_body_q"][nt])) < 1e-10, nt
        assert np.max(np.abs(stt["tether"] - d["traj_tether"][nt])) <= \
            1e-8 * np.max(np.abs(d["traj_tether"][nt])) + 1e-12, nt
    last = states[-1]
    assert np.max(np.abs(last["q"] - d["final_q"])) < 1e-10
    assert np.max(np.abs(last["u"] - d["final_u"])) < 1e-10
    assert rel_max(last["lam"], d["final_lam"]) < 1e-8


def test_ten_steps_fp32c_within_1e8():
    d = load()
    broy, states = run_steps(d, "fp32c")
    scale = np.max(np.abs(d["traj_x_last"]))
    assert np.max(np.abs(states[-1]["x"] - d["traj_x_last"])) / scale < 1e-8
    R = float(d["body_radius"])
    assert np.max(np.abs(states[-1]["body_x"] - d["traj_body_x"][-1])) / R < 1e-8
    assert abs(sum(broy) - int(np.sum(d["broyden_iters"]))) <= 2, broy


def run_steps_default_dt(precision):
    d = np.load(os.path.join(GOLD, "step_default_dt.npz"))
    broy, states = run_steps(d, precision)
    return d, broy, states


def test_ten_steps_at_the_default_time_step():
    """The reference's default DT = 36.3833/300, where every step iterates
    Broyden's method (25, 10, 10, 8, 6, 4, 4, 4, 6, 5 iterations): FP64 keeps
    the same counts and positions and body pose within 1e-10; FP32C the same
    counts and positions within 1e-6 of the largest position."""
    for precision, bar in (("fp64", 1e-10), ("fp32c", 1e-6)):
        d, broy, states = run_steps_default_dt(precision)
        assert broy == list(d["broyden_iters"]), (precision, broy)
        scale = np.max(np.abs(d["traj_x_last"]))
        assert np.max(np.abs(states[0]["x"] - d["traj_x_first"])) / scale < bar, precision
        assert np.max(np.abs(states[-1]["x"] - d["traj_x_last"])) / scale < bar, precision
        R = float(d["body_radius"])
        for nt, stt in enumerate(states):
            assert np.max(np.abs(stt["body_x"] - d["traj_body_x"][nt])) / R < bar, (precision, nt)
            assert np.max(np.abs(stt["body_q"] - d["traj_body_q"][nt])) < bar, (precision, nt)
