"""GPU parity of the implicit time step on the medium swimmer (R = 60, 2562
blobs, 640 straight filaments x 20 segments = 12 800 segments) against the
reference's own time step (cilia_sim_main.cu:355-527 with swimmer.cpp,
filament.cpp, rigid_body.cpp, broyden_solver.cpp and mobility_solver.cpp
compiled unchanged; pair sums from the C restatement pinned to the
reference's kernels; tests/golden/step_medium*.npz):

* DT = 1e-3, steps 0-9 (Broyden TOL 1e-4, LINEAR_SYSTEM_TOL 1e-10);
* the reference's default DT = 36.3833/300, steps 0-3, where every step
  iterates Broyden's method.

After every step the golden holds the filament tip positions, body pose and
tether forces; all segment positions after a few steps.

Tolerances. FP64: the same Broyden iteration count every step, tip and
segment positions within 1e-10 of the largest reference position, body
position within 1e-10 of the body radius, body quaternion within 1e-10.
FP32C (FP32 pairwise sums inside an FP64-refined solve to the same linear
tolerance): the same Broyden iteration counts (their sum within 2 at
DT = 1e-3) and positions within 1e-6 of the largest position, the error of
every step printed and asserted. What sets the FP32C error is the FP32
velocity product, not the solve: velocities carry a relative error of
~7e-7 (FP32 positions relative to the swimmer's centre, rounded to 2^-24 of
its size), so one step moves the state by DT |v| ~ 3 (|v| ~ 3000 in the
straight start) with an error of ~2e-6, 1.8e-8 of the largest position.
Steps 1-9 at DT = 1e-3 need no Broyden iteration: the state is the BDF
extrapolation of the earlier ones, which carries the step-0 offset forward
(1.8e-8 per step, 1.8e-7 after ten). At the default DT Broyden's method
iterates every step and stops within TOL = 1e-4 of the nonlinear residual.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")

pytestmark = pytest.mark.gpu


def make(d, precision):
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


def run_and_compare(name, precision, bar):
    d = np.load(os.path.join(GOLD, f"{name}.npz"))
    nfil, nseg = int(d["nfil"]), int(d["nseg"])
    nsteps = len(d["broyden_iters"])
    full = set(int(k) for k in d["full_steps"])
    s, st = make(d, precision)
    scale = max(np.max(np.abs(d[f"x_step{k}"])) for k in full)
    R = float(d["body_radius"])
    broy, errs = [], []
    try:
        for nt in range(nsteps):
            b, _ = st.step(nt)
            broy.append(b)
            stt = st.state()
            x = stt["x"]
            tips = x.reshape(nfil, nseg, 3)[:, -1, :].ravel()
            e_tip = np.max(np.abs(tips - d["traj_tips"][nt])) / scale
            e_full = (np.max(np.abs(x - d[f"x_step{nt}"])) / scale) if nt in full else float("nan")
            e_bx = np.max(np.abs(stt["body_x"] - d["traj_body_x"][nt])) / R
            e_bq = np.max(np.abs(stt["body_q"] - d["traj_body_q"][nt]))
            errs.append((nt, b, int(d["broyden_iters"][nt]), e_tip, e_full, e_bx, e_bq))
        last = st.state()
    finally:
        st.close()
        s.finalise()
    print(f"\n{name} {precision}: step, Broyden (ours, reference), tip error, "
          "segment error, body position error / R, body quaternion error")
    for row in errs:
        print("  %d  %2d %2d  %.2e  %.2e  %.2e  %.2e" % row)
    for nt, b, bref, e_tip, e_full, e_bx, e_bq in errs:
        assert e_tip < bar, (precision, nt, e_tip)
        if not np.isnan(e_full):
            assert e_full < bar, (precision, nt, e_full)
        assert e_bx < bar, (precision, nt, e_bx)
        assert e_bq < bar, (precision, nt, e_bq)
    if precision == "fp64":  # segment orientations and Lie algebra elements, last step
        assert np.max(np.abs(last["q"] - d["final_q"])) < bar
        assert np.max(np.abs(last["u"] - d["final_u"])) < bar
    return broy, list(d["broyden_iters"]), errs, d


def test_medium_ten_steps_fp64_match_reference():
    broy, ref, _, d = run_and_compare("step_medium", "fp64", 1e-10)
    assert broy == ref, (broy, ref)


def test_medium_ten_steps_fp32c_within_1e6():
    broy, ref, errs, _ = run_and_compare("step_medium", "fp32c", 1e-6)
    assert abs(sum(broy) - sum(ref)) <= 2, (broy, ref)
    # the first step's offset is the FP32 product error of one step
    assert errs[0][3] < 1e-7, errs[0]


def test_medium_default_time_step_fp64_match_reference():
    broy, ref, _, _ = run_and_compare("step_medium_default_dt", "fp64", 1e-10)
    assert broy == ref, (broy, ref)


def test_medium_default_time_step_fp32c_within_1e6():
    broy, ref, _, _ = run_and_compare("step_medium_default_dt", "fp32c", 1e-6)
    assert broy == ref, (broy, ref)


def test_fp32c_extrapolated_warm_start():
    """FP32C: from the third step on, the first solve of a step starts from
    the linear extrapolation of the last two steps' solutions. Every solve
    still meets the linear tolerance; the inner GMRES needs far fewer Arnoldi
    steps than at step 1 (which starts from the last solution); and a reset
    forgets the history, so the same steps run again give the same states,
    bit for bit."""
    d = np.load(os.path.join(GOLD, "step_medium.npz"))
    s, st = make(d, "fp32c")
    tol = float(d["linear_tol"])
    try:
        runs = []
        for _ in range(2):
            gm, states = [], []
            for nt in range(8):
                _, g = st.step(nt)
                info = s.solve_info()
                assert info["rel_residual"] <= tol, (nt, info)
                gm.append(g)
                states.append(st.state())
            runs.append((gm, states))
            st.reset()
        gm, states = runs[0]
        print("GMRES iterations per step", gm)
        assert sum(gm[3:]) <= 0.5 * len(gm[3:]) * gm[1], gm
        assert runs[1][0] == gm
        for a, b in zip(states, runs[1][1]):
            for k in a:
                assert np.array_equal(a[k], b[k]), k
    finally:
        st.close()
        s.finalise()
