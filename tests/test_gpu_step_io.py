"""The reference's data files for the implicit step: the backup and the
plot-step records written by tfs_stepper_write_backup / _write_files against
the same files written by the reference's own writers
(tests/golden/step_io/ref*, from swimmer::write_data, write_backup and
mobility_solver::write_data compiled unchanged), and resuming from the
reference's backup.

Bars: a backup read and written back, and the state records of the restored
state, are byte-identical to the reference's (the same numbers in the same
%.10e text). Records written after our own steps 0-2 agree with the
reference's to 1e-8 of each file's largest value (the solves stop at a 1e-10
residual). Resuming from the reference's backup reproduces its next two
steps (same Broyden counts, positions within 1e-8 of the largest: the backup
keeps 11 significant digits).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
IO = os.path.join(GOLD, "step_io")
FILES = ["_seg_states.dat", "_body_states.dat", "_tether_force.dat", "_body_vels.dat",
         "_blob_forces.dat", "_seg_vels.dat", "_seg_forces.dat", ".backup"]


def load():
    return np.load(os.path.join(GOLD, "step_io.npz"))


def make(d):
    from timfilsimmod_gb300.mobility import RpyMobilitySolver
    from timfilsimmod_gb300.stepper import ImplicitStepper

    nfil, nseg = int(d["nfil"]), int(d["nseg"])
    efm = float(d["end_force_magnitude_real"])
    s = RpyMobilitySolver(1, nfil, nseg, d["blob_refs"].shape[0], precision="fp64",
                          end_force_magnitude=int(efm))
    s.set_blob_references(d["blob_refs"])
    s.set_linear_solver(float(d["linear_tol"]))
    st = ImplicitStepper(s, nfil, nseg, d["fil_refs"], d["fil_dirs"], seg_sep=2.2,
                         dt=float(d["dt"]), tol=float(d["tol"]), end_force_magnitude=efm,
                         body_radius=float(d["body_radius"]))
    return s, st


def test_backup_and_state_records_byte_identical(tmp_path):
    d = load()
    s, st = make(d)
    step = st.read_backup(os.path.join(IO, "ref.backup"))
    assert step == 3
    out = str(tmp_path / "ours")
    st.write_backup(step, out + ".backup")
    assert open(out + ".backup").read() == open(os.path.join(IO, "ref.backup")).read()
    st.write_files(step - 1, out, backup=False)
    for f in ("_seg_states.dat", "_body_states.dat", "_tether_force.dat"):
        assert open(out + f).read() == open(os.path.join(IO, "ref" + f)).read(), f
    st.close()
    s.finalise()


def test_records_after_steps_match_reference(tmp_path):
    d = load()
    s, st = make(d)
    for nt in range(3):
        st.step(nt)
    out = str(tmp_path / "ours")
    st.write_files(2, out, backup=True)
    for f in FILES:
        ours, ref = open(out + f).read(), open(os.path.join(IO, "ref" + f)).read()
        assert ours.count("\n") == ref.count("\n") == 1, f
        to, tr = ours.split(), ref.split()
        assert len(to) == len(tr), f
        if f != "_body_vels.dat":
            assert to[0] == tr[0], f  # the step number
            to, tr = to[1:], tr[1:]
        a, b = np.array(to, dtype=float), np.array(tr, dtype=float)
        assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b)), (f, np.max(np.abs(a - b)))
    st.close()
    s.finalise()


def test_resume_from_reference_backup():
    d = load()
    s, st = make(d)
    step = st.read_backup(os.path.join(IO, "ref.backup"))
    broy = []
    for nt in (step, step + 1):
        b, _ = st.step(nt)
        broy.append(b)
        got, k = st.state(), nt
        ref_x = d[f"after{k}_x"]
        assert np.max(np.abs(got["x"] - ref_x)) <= 1e-8 * np.max(np.abs(ref_x)), nt
        assert np.max(np.abs(got["body_x"] - d[f"after{k}_body_x"])) <= 1e-8 * float(d["body_radius"])
    assert broy == list(d["broyden_iters"][3:])
    st.close()
    s.finalise()
