"""Run a few grand-mobility products of one synthetic swimmer, for profiling.

    python -m timfilsimmod_gb300.profile_case --config medium --precision fp32c --reps 2

Each repetition is one tfs_apply_grand_mobility call (the pack kernels and
one work-queue launch), or with --op the named block, solve, flow
evaluation or implicit time step. Meant to be run under
`ncu -k regex:rpy_queue_kernel -c N` (or `ncu --metrics gpu__time_duration.sum`
for a launch list).
"""
from __future__ import annotations

import argparse
import time

from .geometry import make_config
from .mobility import RpyMobilitySolver


def run_flow(sw, args):
    import numpy as np

    from .flow_field import FlowFieldEvaluator
    from .geometry import flow_grid

    reach = float(np.max(np.linalg.norm(sw.x_segs, axis=1)))
    xf = flow_grid(args.flow_grid, 1.25 * reach)
    ev = FlowFieldEvaluator(1, sw.nfil, sw.nseg, sw.num_blobs, xf.shape[0],
                            precision=args.precision)
    ev.read_positions_and_forces(xf, sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs, sw.body_x)
    if args.variant is not None:
        ev.set_variant(args.variant)
    t0 = time.perf_counter()
    for _ in range(args.reps):
        ev.velocities(copy_to_host=False)
    ev.wait()
    dt = time.perf_counter() - t0
    print(f"flow {args.precision} {xf.shape[0]} points x {sw.num_segs + sw.num_blobs} sources: "
          f"{dt / args.reps * 1e3:.3f} ms per evaluation")
    ev.close()


def run_steps(sw, args):
    """Implicit time steps 0 .. reps-1 of the swimmer with straight elastic
    filaments (DT --dt, default 1e-3; Broyden TOL 1e-4, linear residual
    1e-8); step 0 iterates Broyden's method from the straight start."""
    from .geometry import fibonacci_sphere
    from .stepper import ImplicitStepper

    normals = fibonacci_sphere(sw.nfil)
    fil_refs = (sw.radius + 1.0 + 0.5 * sw.seg_sep) * normals
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * sw.nseg * sw.nseg)
    s = RpyMobilitySolver(1, sw.nfil, sw.nseg, sw.num_blobs, precision=args.precision,
                          end_force_magnitude=int(efm))
    s.set_blob_references(sw.blob_references)
    s.set_linear_solver(1e-8)
    if args.precision == "fp32c":
        s.set_refinement_vectors(args.vectors)
    st = ImplicitStepper(s, sw.nfil, sw.nseg, fil_refs, normals, seg_sep=sw.seg_sep, dt=args.dt,
                         tol=1e-4, end_force_magnitude=efm, body_radius=sw.radius)
    t0 = time.perf_counter()
    from .mobility import kernel_launch_count

    ms, gm = [], []
    for nt in range(args.reps):
        # the launch index where step nt begins (ncu -s skips the ones before)
        print(f"kernel launches before step {nt}: {kernel_launch_count()}")
        r0 = s.refinement_retries() if args.precision == "fp32c" else 0
        t1 = time.perf_counter()
        b, g = st.step(nt, allow_unconverged=True)
        s.wait_for_device()
        ms.append((time.perf_counter() - t1) * 1e3)
        gm.append(g)
        r = (s.refinement_retries() - r0) if args.precision == "fp32c" else 0
        print(f"step {nt}: {b} Broyden iterations, {g} GMRES iterations, "
              f"{r} FP64-vector retries, {ms[-1]:.2f} ms")
    s.wait_for_device()
    dt = time.perf_counter() - t0
    print(f"{args.reps} steps ({args.precision}, {args.config}): {dt * 1e3:.2f} ms")
    if args.reps > 4:
        import numpy as np

        print(f"steps 4..{args.reps - 1} ({args.vectors} vectors): median {np.median(ms[4:]):.2f} ms, "
              f"mean {np.mean(ms[4:]):.2f} ms, {np.mean(gm[4:]):.1f} GMRES iterations per step")
    if args.pg_trace:
        print_pg_trace()
    st.close()
    s.finalise()


def run_prescribed(args):
    """Prescribed-cilia solves (tfs_prescribed_*) of 640 beating filaments x
    20 segments on the 2562-blob sphere (dynamic phase and shape rotation,
    zero prescribed body velocities, RPY mobility, linear residual 1e-8):
    one warm-up solve, then --reps warm-started solves."""
    import hashlib

    import numpy as np

    from .geometry import prescribed_swimmer
    from .prescribed import PrescribedCiliaSolver

    g = prescribed_swimmer(640, 20, radius=60.0, subdivisions=4, seg_sep=2.6)
    rng = np.random.default_rng(5)
    phase0 = rng.uniform(0.0, 2.0 * np.pi, g.nfil)
    omega0 = 2.0 * np.pi * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, g.nfil))
    angle0 = rng.uniform(-0.1, 0.1, g.nfil)
    t = 2.0 * np.pi * np.arange(100) / 100
    ps = PrescribedCiliaSolver(7, g.nfil, g.nseg, g.blob_references, g.seg_sep,
                               1.0 + 0.5 * np.sin(t), 0.2 * np.cos(t), tol=1e-8,
                               precision=args.precision)
    ps.set_solution(phase_dot=omega0)
    dts = []
    for nt in range(args.reps + 1):
        ph = phase0 + omega0 * 1e-2 * nt
        x, vp, va = g.kinematics(ph, angle0)
        t0 = time.perf_counter()
        it = ps.compute_velocities(x, vp, va, ph, omega0, angle0, omega0)
        dts.append(time.perf_counter() - t0)
        info = ps.solve_info()
        print(f"solve {nt}: {it} GMRES steps, {info['cycles']} cycles, residual "
              f"{info['rel_residual']:.2e}, {dts[-1] * 1e3:.1f} ms")
    # the bits of the last solution, for comparing two builds
    sol = ps.solution()
    digest = hashlib.sha256(b"".join(np.ascontiguousarray(sol[k]).tobytes()
                                     for k in sorted(sol))).hexdigest()[:16]
    print(f"solution digest: {digest}")
    ps.finalise()


def print_pg_trace():
    """Median duration (us) of each phase of an Arnoldi step of the last
    cooperative GMRES solve, as CTA 0 (which also runs the Givens step) and
    CTA 1 saw it."""
    import numpy as np

    from .mobility import PG_TRACE_PHASES, pg_trace

    d = pg_trace()
    if d.shape[1] == 0:
        print("pg trace: the last solve took fewer than two Arnoldi steps")
        return
    print(f"pg trace: {d.shape[1]} Arnoldi steps, median us per step (CTA 0 / CTA 1)")
    for ph, name in enumerate(PG_TRACE_PHASES):
        print(f"  {name:28s} {np.median(d[0, :, ph]) / 1e3:8.2f} {np.median(d[1, :, ph]) / 1e3:8.2f}")
    tot = d.sum(axis=2)
    print(f"  {'step':28s} {np.median(tot[0]) / 1e3:8.2f} {np.median(tot[1]) / 1e3:8.2f}")


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--config", default="medium")
    p.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--dt", type=float, default=1e-3, help="time step (op step)")
    p.add_argument("--op", default="grand", choices=["grand", "mss", "mbb", "barrier", "solve", "flow", "step",
                            "prescribed"])
    p.add_argument("--flow-grid", type=int, default=64, help="flow points per axis (op flow)")
    p.add_argument("--variant", type=int, default=None,
                   help="pin every combination to this tile-kernel variant")
    p.add_argument("--waves", type=int, default=1)
    p.add_argument("--queue-variant", type=int, default=None,
                   help="pin every work-queue product kind to this variant")
    p.add_argument("--vectors", default="fp32", choices=["fp32", "fp64"],
                   help="Arnoldi vectors of the FP32C inner solves (op step)")
    p.add_argument("--autotune", action="store_true", help="print the autotuner's table")
    p.add_argument("--pg-trace", action="store_true",
                   help="print the phase table of the last cooperative GMRES solve (ops solve, "
                        "step; needs a library built with -DTFS_PG_TRACE)")
    args = p.parse_args()
    sw = make_config(args.config, seed=1)
    if args.op == "prescribed":
        run_prescribed(args)
        return
    if args.op == "flow":
        return run_flow(sw, args)
    if args.op == "step":
        return run_steps(sw, args)
    s = RpyMobilitySolver(1, sw.nfil, sw.nseg, sw.num_blobs, precision=args.precision)
    s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
    if args.autotune:
        import json
        print(json.dumps(s.autotune((args.precision,), reps=3)))
    if args.variant is not None:
        for combo in range(6):
            s.set_tuning(combo, args.variant, args.waves)
    if args.queue_variant is not None:
        for kind in range(6):
            s.set_queue_variant(kind, args.queue_variant)
    if args.op == "solve":
        import numpy as np

        s.set_blob_references(sw.blob_references)
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        s.set_linear_solver(1e-8)
        s.make_body_reference_matrices()
        rng = np.random.default_rng(5)
    from .mobility import kernel_launch_count

    s.wait_for_device()
    # the launch index where the timed repetitions begin (ncu -s skips the ones before)
    print(f"kernel launches before timed reps: {kernel_launch_count()}")
    t0 = time.perf_counter()
    for _ in range(args.reps):
        if args.op == "grand":
            s.apply_grand_mobility()
        elif args.op == "mss":
            s.evaluate_segment_segment_mobility()
        elif args.op == "mbb":
            s.evaluate_blob_blob_mobility()
        elif args.op == "solve":
            f = sw.f_segs + 1e-3 * rng.normal(size=sw.f_segs.shape)
            s.f_segs_host[:] = f.ravel()
            s.copy_segment_forces_to_device()
            sf = np.concatenate([f[:, :3].sum(0),
                                 (np.cross(sw.x_segs, f[:, :3]) + f[:, 3:]).sum(0)])
            s.compute_velocities(sf)
        else:
            s.apply_interparticle_forces()
    s.wait_for_device()
    dt = time.perf_counter() - t0
    print(f"{args.reps} x {args.op} ({args.precision}, {args.config}): {dt * 1e3:.2f} ms")
    if args.pg_trace:
        print_pg_trace()
    s.finalise()


if __name__ == "__main__":
    main()
