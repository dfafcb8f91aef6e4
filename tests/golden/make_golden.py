"""Generate the golden vectors in tests/golden/ from the reference itself.

The outputs come from the reference's own kernels (src/cilia/cuda_functions.cu
and the flow_velocities kernel of src/flow_field/flow_field_evaluator.cu),
compiled unchanged for the CPU by `make -C oracle ref REF=<reference checkout>`
(see oracle/Makefile).
That needs the reference tree, so this script runs only where it is present;
the .npz files it writes are committed and travel with the tests.

    make -C oracle ref REF=<reference checkout> && python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import (ReferenceFlow, ReferenceKernels, ReferencePrescribed, ReferenceSolver,  # noqa: E402
                    ReferenceStep)

from timfilsimmod_gb300.geometry import fibonacci_sphere, make_config, prescribed_swimmer  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
END_FORCE = 100      # integer device copy of END_FORCE_MAGNITUDE (globals.hpp:14)
REPULSIVE = 2.0      # REPULSIVE_FORCE_FACTOR for elastic cilia (config.hpp:404)


def run_blocks(ref: ReferenceKernels, xs, fs, xb, fb, nseg, nfil):
    ref.sync(1, nseg, nfil, xb.shape[0], END_FORCE, 2.2)
    out = dict(
        v_mss=ref.mss(xs, fs),
        v_msb=ref.msb(xs, xb, fb),             # accumulates onto zeros
        v_mbb=ref.mbb(xb, fb),
        v_mbs=ref.mbs(xb, xs, fs),
    )
    fsb, frep = ref.barrier_forces(xs, xb, fs)
    out.update(f_segs_barrier=fsb, f_blobs_repulsion=frep)
    return out


def case_small():
    """The small swimmer (R = 20, 642 blobs, 32 x 20 segments), seed 1, with
    three segments pushed into the barrier range of others."""
    sw = make_config("small", seed=1)
    xs = sw.x_segs.copy()
    xs[45] = xs[230] + np.array([0.9, 1.2, 0.3])     # inter-filament contact
    xs[101] = xs[103] + np.array([0.0, 0.5, 1.5])    # same filament, two apart
    xb = sw.x_blobs.copy()
    xb[17] = xs[0] + np.array([1.1, -0.9, 0.4])      # segment-blob contact
    ref = ReferenceKernels("a1")
    out = run_blocks(ref, xs, sw.f_segs, xb, sw.f_blobs, sw.nseg, sw.nfil)
    return dict(x_segs=xs, f_segs=sw.f_segs, x_blobs=xb, f_blobs=sw.f_blobs, nseg=sw.nseg,
                nfil=sw.nfil, a_seg=ref.a_seg, a_blob=ref.a_blob, mu=ref.mu,
                end_force_magnitude=END_FORCE, repulsive_force_factor=REPULSIVE, **out)


def case_overlap():
    """Ragged sizes (77 segments of 7 per filament, 45 blobs), unequal radii
    (RSEG 1, RBLOB 1.6), particles packed so that every branch of the RPY pair
    function is taken: far, overlapping, nested, and self (r = 0)."""
    rng = np.random.default_rng(7)
    xs = rng.uniform(-4.0, 4.0, size=(77, 3))
    xb = rng.uniform(-4.0, 4.0, size=(45, 3))
    xb[:10] = xs[:10] + rng.normal(0.0, 0.25, size=(10, 3))  # nested (r < 0.6)
    xb[10:20] = xs[10:20] + rng.normal(0.0, 1.2, size=(10, 3))  # overlapping
    xs[30] = xs[31] + np.array([0.3, 0.2, -0.1])
    fs = rng.normal(size=(77, 6))
    fb = rng.normal(size=(45, 3))
    ref = ReferenceKernels("a16")
    out = run_blocks(ref, xs, fs, xb, fb, 7, 11)
    return dict(x_segs=xs, f_segs=fs, x_blobs=xb, f_blobs=fb, nseg=7, nfil=11,
                a_seg=ref.a_seg, a_blob=ref.a_blob, mu=ref.mu, end_force_magnitude=END_FORCE,
                repulsive_force_factor=REPULSIVE, **out)


def case_tiny():
    """One segment, one blob; and 65 segments (one past a 64-thread tile)
    with 3 blobs."""
    rng = np.random.default_rng(11)
    ref = ReferenceKernels("a1")
    res = {}
    for tag, ns, nb, nseg in (("one", 1, 1, 1), ("tile", 65, 3, 5)):
        xs = rng.uniform(-10, 10, size=(ns, 3))
        xb = rng.uniform(-10, 10, size=(nb, 3))
        fs = rng.normal(size=(ns, 6))
        fb = rng.normal(size=(nb, 3))
        out = run_blocks(ref, xs, fs, xb, fb, nseg, ns // nseg)
        res.update({f"{tag}_{k}": v for k, v in
                    dict(x_segs=xs, f_segs=fs, x_blobs=xb, f_blobs=fb, nseg=nseg, **out).items()})
    res.update(a_seg=ref.a_seg, a_blob=ref.a_blob, mu=ref.mu, end_force_magnitude=END_FORCE,
               repulsive_force_factor=REPULSIVE)
    return res


def case_weak():
    """Weakly coupled filaments' product (the reference's filament means,
    total forces and Msf_mult, a1 config): 6 filaments x 20 segments leaving
    a sphere of radius 10 along random directions, two of them crossing
    close by; and a ragged 5 x 7 case."""
    rng = np.random.default_rng(21)
    ref = ReferenceKernels("a1")
    res = {}
    for tag, nfil, nseg in (("six", 6, 20), ("ragged", 5, 7)):
        d = rng.normal(size=(nfil, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        xs = np.concatenate([10.0 * u + 2.2 * np.arange(nseg)[:, None] * u for u in d])
        xs += rng.normal(scale=0.05, size=xs.shape)
        if tag == "six":
            xs[25] = xs[3] + np.array([0.4, 0.3, -0.2])  # overlapping segments of two filaments
        fs = rng.normal(size=(nfil * nseg, 6))
        ref.sync(1, nseg, nfil, 0)
        v = ref.msf(xs, fs, nfil, nseg)
        res.update({f"{tag}_x_segs": xs, f"{tag}_f_segs": fs, f"{tag}_v_segs": v,
                    f"{tag}_nfil": nfil, f"{tag}_nseg": nseg})
    res.update(a_seg=ref.a_seg, mu=ref.mu)
    return res


def case_flow():
    """Flow field of the small swimmer at 333 points, with blobs (free space)
    with and without the net-force Stokeslet removed, and with no blobs (the
    Blakelet wall form)."""
    sw = make_config("small", seed=2)
    rng = np.random.default_rng(13)
    xf = rng.uniform(-70.0, 70.0, size=(333, 3))
    xf[:, 2] = np.abs(xf[:, 2]) + 1.0   # above the z = 0 wall for the Blakelet case
    xbod = np.zeros((1, 3))
    prefac = 1.0 / (8.0 * np.pi * 1.0)
    flow = ReferenceFlow()
    res = dict(x_flow=xf, x_segs=sw.x_segs, f_segs=sw.f_segs, x_blobs=sw.x_blobs,
               f_blobs=sw.f_blobs, x_bodies=xbod, prefac=prefac)
    # the wall case lifts the swimmer above z = 0
    lift = np.array([0.0, 0.0, 90.0])
    res["x_segs_wall"] = sw.x_segs + lift
    res["v_blobs"] = flow.flow_velocities(xf, sw.x_segs, sw.f_segs, sw.num_segs, sw.x_blobs,
                                          sw.f_blobs, sw.num_blobs, xbod, prefac, False)
    res["v_blobs_rnf"] = flow.flow_velocities(xf, sw.x_segs, sw.f_segs, sw.num_segs, sw.x_blobs,
                                              sw.f_blobs, sw.num_blobs, xbod, prefac, True)
    res["v_wall"] = flow.flow_velocities(xf, res["x_segs_wall"], sw.f_segs, sw.num_segs,
                                         sw.x_blobs, sw.f_blobs, 0, xbod + lift, prefac, False)
    return res


def quat_rot(q):
    s, a, b, c = q
    return np.array([[1 - 2 * b * b - 2 * c * c, 2 * a * b - 2 * s * c, 2 * a * c + 2 * s * b],
                     [2 * a * b + 2 * s * c, 1 - 2 * a * a - 2 * c * c, 2 * b * c - 2 * s * a],
                     [2 * a * c - 2 * s * b, 2 * b * c + 2 * s * a, 1 - 2 * a * a - 2 * b * b]])


def swimmer_force(x_segs, f_segs, body_x):
    F = f_segs[:, :3].sum(0)
    T = (np.cross(x_segs - body_x, f_segs[:, :3]) + f_segs[:, 3:]).sum(0)
    return np.concatenate([F, T])


def case_solve():
    """The reference's own free-body mobility solve (mobility_solver.cpp,
    LINEAR_SYSTEM_TOL = 1e-10) on the small swimmer: make_body_reference_
    matrices, then compute_velocities twice -- at the start pose, then with
    the body translated and rotated (segments moved with it) and new forces,
    warm-started from the first solution as in a time step sequence."""
    sw = make_config("small", seed=1)
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * sw.nseg ** 2)  # END_FORCE_MAGNITUDE, default DL
    ref = ReferenceSolver(sw.nfil, sw.nseg, sw.blob_references, efm, seg_sep=2.2)
    res = dict(x_segs=sw.x_segs, f_segs=sw.f_segs, blob_refs=sw.blob_references,
               nfil=sw.nfil, nseg=sw.nseg, end_force_magnitude_real=efm,
               end_force_magnitude=int(efm), tol=ref.lib.ref_linear_system_tol())
    bref = ref.make_body_reference_matrices(sw.x_segs, sw.f_segs)
    res.update({f"bodyref_{k}": v for k, v in bref.items()})
    sf = swimmer_force(sw.x_segs, sw.f_segs, np.zeros(3))
    r1 = ref.compute_velocities(sw.x_segs, sw.f_segs, sf, nt=0)
    res.update({f"cv1_{k}": v for k, v in r1.items() if k != "v_blobs_rhs"})
    res["cv1_swimmer_f_in"] = sf
    q = np.array([0.9, 0.1, -0.3, 0.2])
    q /= np.linalg.norm(q)
    bx = np.array([1.5, -2.0, 0.7])
    R = quat_rot(q)
    xs2 = bx + sw.x_segs @ R.T
    f2 = np.random.default_rng(17).normal(size=sw.f_segs.shape)
    ref.set_body(bx, q)
    sf2 = swimmer_force(xs2, f2, bx)
    r2 = ref.compute_velocities(xs2, f2, sf2, nt=1)
    res.update({f"cv2_{k}": v for k, v in r2.items() if k != "v_blobs_rhs"})
    res.update(cv2_x_segs=xs2, cv2_f_segs=f2, cv2_body_x=bx, cv2_body_q=q, cv2_swimmer_f_in=sf2)
    return res


def step_setup(nfil=None):
    """The small swimmer's body (R = 20, 642 blobs) with 32 straight
    filaments of 20 segments along the surface normals, bases one blob radius
    plus half a segment gap above the surface; END_FORCE_MAGNITUDE with the
    default DL = 2.6."""
    sw = make_config("small", seed=1)
    nfil = nfil or sw.nfil
    normals = fibonacci_sphere(nfil)
    fil_refs = (sw.radius + 1.0 + 0.5 * 2.2) * normals
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * sw.nseg ** 2)
    return sw, nfil, normals, fil_refs, efm


def case_step():
    """The reference's implicit time step (DT = 1e-3, Broyden TOL 1e-4,
    LINEAR_SYSTEM_TOL 1e-10) on the small swimmer with elastic filaments:
    step 0 stage by stage (internal forces, velocities, residuals, Schur
    complement, inverse approximate Jacobians, a jacobian_inv_mult probe, the
    first Broyden iteration), then the whole of steps 0-9 with the state
    after each."""
    sw, nfil, normals, fil_refs, efm = step_setup()
    nseg = sw.nseg
    ref = ReferenceStep(nfil, nseg, sw.blob_references, fil_refs, normals, efm, seg_sep=2.2,
                        body_length=2.0 * sw.radius)
    res = dict(blob_refs=sw.blob_references, fil_refs=fil_refs, fil_dirs=normals, nfil=nfil,
               nseg=nseg, end_force_magnitude_real=efm, body_radius=sw.radius, dt=1e-3,
               tol=1e-4, linear_tol=ref.lib.ref_linear_system_tol())
    bm, ktk = ref.make_body_reference_matrices()
    res.update(body_mobility=bm, ktkinv=ktk)
    nt = 0
    ref.initial_guess(nt)
    res["s0_guess"] = ref.state()["x"]
    fs, sf = ref.forces(nt)
    res.update(s0_f_segs=fs, s0_swimmer_f=sf)
    it, vs, vb, fb = ref.compute_velocities(nt)
    res.update(s0_v_segs=vs, s0_v_bodies=vb, s0_f_blobs=fb, s0_gmres=it)
    big, err = ref.compute_errors(nt, 0)
    res.update(s0_error=err, s0_big=int(big))
    res["s0_schur_inv"] = ref.prepare_jacobian_inv(nt)
    res["s0_jinv_first"] = ref.inverse_jacobian(0)
    res["s0_jinv_last_rows"] = ref.inverse_jacobian(nfil - 1)[:12]
    probe = np.random.default_rng(5).normal(size=ref.nbroy)
    res.update(s0_probe=probe, s0_probe_out=ref.jacobian_inv_mult(nt, probe))
    ref.broyden_reset()
    iters, gm = 0, it
    while big:
        upd = ref.find_update(nt)
        if iters < 1:
            res[f"s0_update{iters}"] = upd
        ref.apply_update(nt)
        it, vs, vb, fb = ref.compute_velocities(nt)
        gm += it
        big, nerr = ref.compute_errors(nt, 1)
        if iters < 1:
            res[f"s0_new_error{iters}"] = nerr
            res[f"s0_state{iters}_x"] = ref.state()["x"]
        ref.end_of_iter(nt, big)
        iters += 1
    st = ref.state()
    traj = {k: [v] for k, v in st.items()}
    broy, gmres = [iters], [gm]
    for nt in range(1, 10):
        b, g = ref.run(nt)
        broy.append(b)
        gmres.append(g)
        for k, v in ref.state().items():
            traj[k].append(v)
    for k, v in traj.items():
        if k in ("q", "u", "lam"):
            res[f"final_{k}"] = v[-1]
        elif k == "x":
            res["traj_x_first"], res["traj_x_last"] = v[0], v[-1]
        else:
            res[f"traj_{k}"] = np.array(v)
    res.update(broyden_iters=np.array(broy), gmres_iters=np.array(gmres))
    return res


def case_step_io():
    """The reference's data files and backup (its own writers) after steps
    0-2 of a small swimmer (162 blobs, R = 10, 3 filaments x 14 segments),
    written to tests/golden/step_io/ref*, and the states after steps 3 and 4
    continuing from there."""
    from timfilsimmod_gb300.geometry import icosphere

    radius, nfil, nseg = 10.0, 3, 14
    blob_refs = radius * icosphere(2)
    normals = fibonacci_sphere(nfil)
    fil_refs = (radius + 1.0 + 1.1) * normals
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * nseg ** 2)
    ref = ReferenceStep(nfil, nseg, blob_refs, fil_refs, normals, efm, seg_sep=2.2,
                        body_length=2.0 * radius)
    ref.make_body_reference_matrices()
    d = os.path.join(OUT, "step_io")
    os.makedirs(d, exist_ok=True)
    for f in os.listdir(d):
        if f.startswith("ref"):
            os.remove(os.path.join(d, f))
    broy = [ref.run(nt)[0] for nt in range(3)]
    ref.write_files(os.path.join(d, "ref"), 2)
    later = []
    for nt in (3, 4):
        broy.append(ref.run(nt)[0])
        later.append(ref.state())
    res = dict(blob_refs=blob_refs, fil_refs=fil_refs, fil_dirs=normals, nfil=nfil, nseg=nseg,
               end_force_magnitude_real=efm, body_radius=radius, dt=1e-3, tol=1e-4,
               linear_tol=ref.lib.ref_linear_system_tol(), broyden_iters=np.array(broy))
    for i, st in enumerate(later):
        res.update({f"after{3 + i}_{k}": v for k, v in st.items()})
    return res


def case_step_default_dt():
    """Steps 0-9 of the small swimmer at the reference's default time step
    (DT = 36.3833/300; Broyden TOL 1e-4, LINEAR_SYSTEM_TOL 1e-10), where
    every step iterates Broyden's method: per-step Broyden counts, body pose
    and tether forces after each step, segment positions after steps 0 and 9,
    the final orientations, Lie algebra elements and multipliers."""
    sw, nfil, normals, fil_refs, efm = step_setup()
    ref = ReferenceStep(nfil, sw.nseg, sw.blob_references, fil_refs, normals, efm, seg_sep=2.2,
                        body_length=2.0 * sw.radius, config="s2")
    ref.make_body_reference_matrices()
    res = dict(blob_refs=sw.blob_references, fil_refs=fil_refs, fil_dirs=normals, nfil=nfil,
               nseg=sw.nseg, end_force_magnitude_real=efm, body_radius=sw.radius,
               dt=36.3833 / 300.0, tol=1e-4, linear_tol=ref.lib.ref_linear_system_tol())
    broy, gm, traj = [], [], {}
    for nt in range(10):
        b, g = ref.run(nt)
        broy.append(b)
        gm.append(g)
        for k, v in ref.state().items():
            traj.setdefault(k, []).append(v)
    for k, v in traj.items():
        if k in ("q", "u", "lam"):
            res[f"final_{k}"] = v[-1]
        elif k == "x":
            res["traj_x_first"], res["traj_x_last"] = v[0], v[-1]
        else:
            res[f"traj_{k}"] = np.array(v)
    res.update(broyden_iters=np.array(broy), gmres_iters=np.array(gm))
    return res


def medium_setup():
    """The medium swimmer's body (R = 60, 2562 blobs) with 640 straight
    filaments of 20 segments along the surface normals."""
    sw = make_config("medium", seed=1)
    normals = fibonacci_sphere(sw.nfil)
    fil_refs = (sw.radius + 1.0 + 0.5 * 2.2) * normals
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * sw.nseg ** 2)
    return sw, normals, fil_refs, efm


def _medium_trajectory(config, dt, nsteps, full_steps):
    sw, normals, fil_refs, efm = medium_setup()
    nfil, nseg = sw.nfil, sw.nseg
    ref = ReferenceStep(nfil, nseg, sw.blob_references, fil_refs, normals, efm, seg_sep=2.2,
                        body_length=2.0 * sw.radius, config=config)
    bm, ktk = ref.make_body_reference_matrices()
    res = dict(blob_refs=sw.blob_references, fil_refs=fil_refs, fil_dirs=normals, nfil=nfil,
               nseg=nseg, end_force_magnitude_real=efm, body_radius=sw.radius, dt=dt,
               tol=1e-4, linear_tol=ref.lib.ref_linear_system_tol(), body_mobility=bm,
               ktkinv=ktk, full_steps=np.array(full_steps))
    broy, gm, tips, keep = [], [], [], {}
    for nt in range(nsteps):
        b, g = ref.run(nt)
        broy.append(b)
        gm.append(g)
        st = ref.state()
        x = st["x"].reshape(nfil, nseg, 3)
        tips.append(x[:, -1, :].ravel())
        for k in ("body_x", "body_q", "body_u", "tether", "clamp"):
            keep.setdefault(k, []).append(st[k])
        if nt in full_steps:
            res[f"x_step{nt}"] = st["x"]
        print(f"  step {nt}: Broyden {b}, GMRES {g}", flush=True)
    last = ref.state()
    res.update(final_q=last["q"], final_u=last["u"], final_lam=last["lam"],
               traj_tips=np.array(tips), broyden_iters=np.array(broy), gmres_iters=np.array(gm))
    res.update({f"traj_{k}": np.array(v) for k, v in keep.items()})
    return res


def case_step_medium():
    """The reference's implicit time step on the medium swimmer (R = 60,
    2562 blobs, 640 straight filaments x 20 segments), DT = 1e-3, Broyden
    TOL 1e-4, LINEAR_SYSTEM_TOL 1e-10: steps 0-9 with, after every step, the
    filament tip positions, body pose and tether and clamp forces, and all
    segment positions after steps 0, 4 and 9."""
    return _medium_trajectory("s1", 1e-3, 10, (0, 4, 9))


def case_step_medium_default_dt():
    """The same swimmer at the reference's default DT = 36.3833/300, where
    Broyden iterates every step: steps 0-3, all segment positions after each."""
    return _medium_trajectory("s2", 36.3833 / 300.0, 4, (0, 1, 2, 3))


def prescribed_inputs(nsteps=3, seed=7):
    """Kinematics of 8 prescribed filaments x 10 segments on a 162-blob sphere
    (R = 10) in a rotated, shifted body pose, over nsteps steps, plus
    generalised-force tables of 40 points."""
    g = prescribed_swimmer(8, 10, radius=10.0, subdivisions=2, seg_sep=2.6)
    rng = np.random.default_rng(seed)
    q = np.array([0.95, 0.1, -0.2, 0.15])
    q /= np.linalg.norm(q)
    bx = np.array([0.5, -1.0, 2.0])
    t = 2.0 * np.pi * np.arange(40) / 40
    phase_refs = 1.0 + 0.5 * np.sin(t) + 0.2 * np.cos(2.0 * t)
    angle_refs = 0.1 + 0.3 * np.sin(t) - 0.05 * np.cos(3.0 * t)
    phase0 = rng.uniform(0.0, 2.0 * np.pi, g.nfil)
    omega0 = 2.0 * np.pi * (1.0 + 0.2 * rng.uniform(-1.0, 1.0, g.nfil))
    angle0 = rng.uniform(-0.3, 0.3, g.nfil)
    phase = np.stack([phase0 + 0.05 * omega0 * nt for nt in range(nsteps)])
    angle = np.stack([angle0 * np.cos(nt) for nt in range(nsteps)])
    kin = [g.kinematics(phase[nt], angle[nt], bx, q) for nt in range(nsteps)]
    return dict(nfil=g.nfil, nseg=g.nseg, seg_sep=g.seg_sep, blob_refs=g.blob_references,
                body_x=bx, body_q=q, phase_refs=phase_refs, angle_refs=angle_refs, omega0=omega0,
                phase=phase, angle=angle, x_segs=np.stack([k[0] for k in kin]),
                vel_dir_phase=np.stack([k[1] for k in kin]),
                vel_dir_angle=np.stack([k[2] for k in kin]),
                phase_dot0=omega0.copy(), angle_dot0=np.zeros(g.nfil),
                gen_force_magnitude_factor=1.0, torsional_spring_magnitude_factor=2.0)


def case_prescribed(config):
    """The reference's prescribed-cilia solve (configuration p1 ... p6 of
    oracle/Makefile): three consecutive solves (warm started from the last),
    then, on the first step's kinematics, the right-hand side, swimmer
    KTMinvK_inv, and the operator and preconditioner applied to a seeded
    vector."""
    d = prescribed_inputs()
    ref = ReferencePrescribed(config, d["nfil"], d["nseg"], d["blob_refs"], d["seg_sep"],
                              d["body_x"], d["body_q"], d["phase_refs"], d["angle_refs"])
    ref.set_rates(d["phase_dot0"], d["angle_dot0"])
    outs = []
    for nt in range(d["phase"].shape[0]):
        ref.set_kinematics(d["x_segs"][nt], d["vel_dir_phase"][nt], d["vel_dir_angle"][nt],
                           d["phase"][nt], d["omega0"], d["angle"][nt], d["omega0"])
        outs.append(ref.compute_velocities(nt))
    ref.set_kinematics(d["x_segs"][0], d["vel_dir_phase"][0], d["vel_dir_angle"][0],
                       d["phase"][0], d["omega0"], d["angle"][0], d["omega0"])
    v_in = np.random.default_rng(11).normal(size=ref.n)
    d.update(flags=ref.flags, n=ref.n, ktminvk=ref.ktminvk(), rhs0=ref.rhs(0), v_in=v_in,
             a_v=ref.apply(0, v_in), pinv_v=ref.apply(1, v_in),
             iters=np.array([o["iters"] for o in outs]))
    for key in ("f_segs", "f_blobs", "v_body", "phase_dot", "angle_dot"):
        d[key] = np.stack([o[key] for o in outs])
    return d


CASES = {"small_matvec": case_small, "overlap_a16": case_overlap, "tiny": case_tiny,
         "flow_small": case_flow, "solve_small": case_solve, "step_small": case_step,
         "step_io": case_step_io, "step_default_dt": case_step_default_dt,
         "weak_coupled": case_weak, "step_medium": case_step_medium,
         "step_medium_default_dt": case_step_medium_default_dt,
         "prescribed_p1": lambda: case_prescribed("p1"),
         "prescribed_p2": lambda: case_prescribed("p2"),
         "prescribed_p3": lambda: case_prescribed("p3"),
         "prescribed_p4": lambda: case_prescribed("p4"),
         "prescribed_p5": lambda: case_prescribed("p5"),
         "prescribed_p6": lambda: case_prescribed("p6")}


def main():
    # one case per process: the reference's solver library keeps global state
    names = sys.argv[1:] or list(CASES)
    if len(names) > 1:
        import subprocess
        for name in names:
            subprocess.run([sys.executable, os.path.abspath(__file__), name], check=True)
        return
    for name, fn in ((n, CASES[n]) for n in names):
        data = fn()
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in data.items()})
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
