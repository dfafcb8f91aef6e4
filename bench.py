"""Benchmark of the RPY grand-mobility product (one GB300).

A step is one application of the whole grand mobility -- all four blocks,
v_segs = Mss f_segs + Msb f_blobs and v_blobs = Mbs f_segs + Mbb f_blobs --
to the medium swimmer (R = 60a sphere of 2562 blobs carrying 640 filaments x
20 segments = 12 800 segments; seeded synthetic geometry, N(0,1) forces), in
the mixed-precision form (FP32 pairs with compensated accumulation, FP64
inputs/outputs). Printed: one JSON line (rank 0).

  value    matvecs/s with inputs resident in HBM, CUDA events around each step,
           L2 flushed between steps (outside the events)
  e2e      matvecs/s through the C-ABI hooks with pinned host buffers: the H2D
           copies of positions and forces and the D2H copies of velocities are
           inside the timed region
  roofline the dominant kernel (the work-queue kernel: both target kinds,
           all four blocks and the source-split sums in one persistent launch)
           against the measured FP32 FMA peak
  fp64     the same product in plain FP64 (the parity drop-in) for comparison

  solve    compute_velocities (the free-body GMRES solve of one Broyden
           iteration) at a 1e-8 linear residual, FP64 vs FP32C refinement
  implicit_steps  100 whole implicit time steps (forces, solve, residuals,
           Broyden) at a 1e-8 linear residual, FP64 vs FP32C, steps/s with
           p50/p99 per-step latency, the FP32C position error per step against
           FP64 and the error of both against the reference's own trajectory
  implicit_steps_default_dt  the same at the reference's default
           DT = 36.3833/300, where every step iterates Broyden's method
  batched  64 uneven swimmers stepped together (FP32C, host worker pool)
           vs the FP64 drop-in one swimmer at a time, swimmer-steps/s
  served   Poisson streams of step requests of log-uniform size into the
           request server: steps/s and p50/p99 latency per arrival rate, vs
           FP64 requests served one at a time
  flow     the flow-field evaluator on a 128^3 grid around the large swimmer
           (80 000 segments, 10 242 blobs), FP32C, with an FP64 subset
  large    the large swimmer: grand mobility FP32C and FP64 with rooflines,
           one mobility solve at a 1e-8 residual, FP32C implicit steps

`--impl reference` times the reference's RPY sums on the host cores instead
(the CPU restatement in oracle/, all threads), on a bounded sample of the
same workload.

With torchrun (N > 1) every rank runs an independent replica on its own GPU
(the product of one swimmer is not split across GPUs); value is the total
over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_66, FLOPS_63, FLOPS_36, FLOPS_33 = 93, 56, 56, 40  # canonical flops per pair


def grand_flops(ns, nb):
    return ns * ns * FLOPS_66 + ns * nb * FLOPS_63 + nb * ns * FLOPS_36 + nb * nb * FLOPS_33


def queue_bytes(ns, nb):
    """Algorithmic bytes of one FP32C grand-mobility launch: the records read
    (48 B per segment, 32 B per blob; the targets' positions come from the
    same records) and the FP64 velocities written."""
    return 48 * ns + 32 * nb + 8 * (6 * ns + 3 * nb)


def grand_pairs(ns, nb):
    return (ns + nb) ** 2


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        busy = [s for s in sm if s >= 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(busy)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": float(max(power)) if power else None}


# DRAM bytes per launch of the segment-target tile kernel (FP32C grand
# mobility), from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum,
# rpy_tile_kernel<float,6,6,3,128,1,256,8>, medium swimmer): 1 043 200 + 0.
# DRAM bytes per launch of the grand-mobility work-queue launch (dram__bytes_read.sum +
# dram__bytes_write.sum, one ncu capture of this workload); None until captured
QUEUE_TRAFFIC = {"medium": 795392}


def max_over_ranks(values, world: int, device: str):
    """Each value's maximum over the ranks (the slowest replica's time); with
    one rank, the values themselves."""
    import torch

    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units processed by all replicas per second of the slowest one."""
    return world * units_per_rank / seconds


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def bench_ours(args):
    import torch
    import torch.distributed as dist

    from timfilsimmod_gb300 import _native
    from timfilsimmod_gb300.geometry import make_config
    from timfilsimmod_gb300.mobility import (RpyMobilitySolver, kernel_launch_count,
                                             measure_fma_peak)

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    _native.load()  # fails loudly without the library

    sw = make_config(args.config, seed=1234 + rank)
    ns, nb = sw.num_segs, sw.num_blobs
    # a dedicated stream: the solver and every timing event run on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    tuning = {}

    def make(precision):
        s = RpyMobilitySolver(1, sw.nfil, sw.nseg, nb, precision=precision)
        s.set_stream(stream.cuda_stream)
        s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
        if not args.no_tune:
            # pick the tile-kernel launch variant per block for these sizes
            table = s.autotune((precision,), reps=2 if precision == "fp32c" else 1)[precision]
            tuning[precision] = {k: [v["block"], v["tpt"], v["ts"], v["x2"], v["waves"]]
                                 for k, v in table.items()}
        return s

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def timed_steps(solver, steps, warmup, timing=False):
        for _ in range(warmup):
            solver.apply_grand_mobility()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        if timing:
            solver.enable_kernel_timing(True)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        launches0 = kernel_launch_count()
        for k in range(steps):
            flush.zero_()  # L2 flush, outside the timed events
            starts[k].record(stream)
            solver.apply_grand_mobility()
            ends[k].record(stream)
        torch.cuda.synchronize()
        launches = kernel_launch_count() - launches0
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
        ktimes = solver.kernel_timing() if timing else []
        if timing:
            solver.enable_kernel_timing(False)
        return ms, launches, ktimes

    peak32 = measure_fma_peak("fp32c")
    peak64 = measure_fma_peak("fp64")

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)

    # --- mixed precision, device resident (value) ---------------------------
    s32 = make("fp32c")
    ms32, launches, ktimes = timed_steps(s32, args.steps, args.warmup, timing=True)
    seg_launches = ktimes  # one work-queue launch per step

    # --- end to end through the C-ABI hooks, pinned host buffers ----------------
    s32.f_segs_host[:] = sw.f_segs.ravel()
    s32.f_blobs_host[:] = sw.f_blobs.ravel()
    e2e_steps = max(1, args.steps)
    for _ in range(args.warmup):
        s32.copy_segment_positions_to_device()
        s32.copy_segment_forces_to_device()
        s32.copy_blob_positions_to_device()
        s32.copy_blob_forces_to_device()
        s32.apply_grand_mobility()
        s32.copy_segment_velocities_to_host()
        s32.copy_blob_velocities_to_host()
        s32.wait_for_device()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t_e2e = 0.0
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s32.copy_segment_positions_to_device()
        s32.copy_segment_forces_to_device()
        s32.copy_blob_positions_to_device()
        s32.copy_blob_forces_to_device()
        s32.apply_grand_mobility()
        s32.copy_segment_velocities_to_host()
        s32.copy_blob_velocities_to_host()
        b.record(stream)
        s32.wait_for_device()
        t_e2e += a.elapsed_time(b)
    v32 = np.concatenate([s32.v_segs_host, s32.v_blobs_host]).copy()

    # --- plain FP64 drop-in, same product ------------------------------------
    s64 = make("fp64")
    steps64 = max(3, min(args.steps, 10))
    ms64, _, ktimes64 = timed_steps(s64, steps64, 1, timing=True)
    s64.copy_segment_velocities_to_host()
    s64.copy_blob_velocities_to_host()
    s64.wait_for_device()
    v64 = np.concatenate([s64.v_segs_host, s64.v_blobs_host]).copy()
    # --- the mobility solve of one Broyden iteration (compute_velocities) -----
    solve = None if args.no_solve else solve_bench(sw, stream, args, RpyMobilitySolver)
    # --- implicit time steps (initial guess, forces, solve, Broyden) -----------
    gold = os.path.join(ROOT, "tests", "golden", "step_medium.npz")
    steps = None if args.no_steps else step_bench(sw, stream, args, total=100, warm=3,
                                                  golden=gold)
    # the reference's default DT = 36.3833/300: every step iterates Broyden's method
    gold_dt = os.path.join(ROOT, "tests", "golden", "step_medium_default_dt.npz")
    steps_dt = None if args.no_steps else step_bench(sw, stream, args, dt=36.3833 / 300.0,
                                                     total=23, warm=2, golden=gold_dt)
    # --- many swimmers: a batch stepped together, and a request stream ---------
    batched = None if args.no_batch else batch_bench(args)
    served = None if args.no_serve else serve_bench(args)
    # --- the large swimmer: grand mobility, one solve, implicit steps ----------
    large = None if args.no_large else large_bench(stream, flush, args, peak32, peak64)
    # --- the flow-field evaluator on a 128^3 grid around the large swimmer -----
    flow = None if args.no_flow else flow_bench(stream, flush, args, peak32, peak64, rank)
    # --- the prescribed-cilia solve on the medium swimmer's sizes ---------------
    prescribed = None if args.no_prescribed else prescribed_bench(args)
    clocks = sampler.stop()

    # max over ranks
    ms32, t_e2e, ms64 = max_over_ranks([ms32, t_e2e, ms64], world, "cuda")

    per_step_ms = ms32 / args.steps
    value = whole_job_rate(args.steps, world, ms32 * 1e-3)
    e2e_value = whole_job_rate(e2e_steps, world, t_e2e * 1e-3)
    value64 = whole_job_rate(steps64, world, ms64 * 1e-3)
    seg_flops = grand_flops(ns, nb)  # the launch computes the whole grand mobility
    seg_ms = float(np.mean(seg_launches)) if seg_launches else float("nan")
    achieved = seg_flops / (seg_ms * 1e-3) / 1e12
    seg64 = ktimes64
    seg64_ms = float(np.mean(seg64)) if seg64 else float("nan")
    achieved64 = seg_flops / (seg64_ms * 1e-3) / 1e12
    err = float(np.linalg.norm(v32 - v64) / np.linalg.norm(v64))

    result = None
    if rank == 0:
        cpu = cpu_baseline(sw, args.cpu_sample) if not args.no_cpu else None
        h2d = 8 * (3 * ns + 6 * ns + 3 * nb + 3 * nb)
        d2h = 8 * (6 * ns + 3 * nb)
        result = {
            "metric": "RPY grand-mobility matvecs/s (4 blocks, medium swimmer)",
            "value": value,
            "unit": "matvecs/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": per_step_ms,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "fp32 pairs, compensated accumulation; fp64 in/out",
            "data": "synthetic (seeded icosphere + Fibonacci filaments, N(0,1) forces)",
            "config": bench_config(args.config, ns, nb, world),
            "pair_interactions_per_s": value * grand_pairs(ns, nb),
            "e2e": {"value": e2e_value, "unit": "matvecs/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "fp32-fma", "kernel": "rpy_queue_kernel<float,6,3>",
                         "achieved": achieved, "peak": peak32 / 1e12, "unit": "TFLOP/s",
                         "frac": achieved / (peak32 / 1e12),
                         "peak_source": "measured live (FMA-chain microbenchmark, this run)",
                         "flops_per_launch": seg_flops, "avg_launch_ms": seg_ms,
                         "traffic": QUEUE_TRAFFIC.get(args.config),
                         "algorithmic_bytes": queue_bytes(ns, nb),
                         "traffic_note": "bytes per launch, dram__bytes_read.sum + "
                                         "dram__bytes_write.sum of one ncu capture of the "
                                         "grand-mobility launch on this workload "
                                         "(profiles/rpy_queue_f32_grand_medium.md); "
                                         "algorithmic bytes: FP32 records read, FP64 "
                                         "velocities written (the written velocities and "
                                         "the chunk partial sums stay in L2)"},
            "fp64": {"value": value64, "unit": "matvecs/s", "steps": steps64,
                     "roofline": {"bound": "fp64-fma", "achieved": achieved64,
                                  "peak": peak64 / 1e12, "unit": "TFLOP/s",
                                  "frac": achieved64 / (peak64 / 1e12),
                                  "avg_launch_ms": seg64_ms}},
            "speedup_vs_fp64": value / value64,
            "rel_l2_error_vs_fp64": err,
            "clocks": clocks,
            "gpu_launches": launches,
            "tuning": {"columns": ["threads/CTA", "targets/thread", "sources/tile",
                                   "packed fp32x2", "waves"], **tuning},
        }
        if cpu is not None:
            result["cpu_baseline"] = cpu
        if solve is not None:
            result["solve"] = solve
        if steps is not None:
            result["implicit_steps"] = steps
        if steps_dt is not None:
            result["implicit_steps_default_dt"] = steps_dt
        if batched is not None:
            result["batched"] = batched
        if served is not None:
            result["served"] = served
        if flow is not None:
            result["flow"] = flow
        if large is not None:
            result["large"] = large
        if prescribed is not None:
            result["prescribed"] = prescribed
    for sv in (s32, s64):
        sv.finalise()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return result


def prescribed_bench(args, timed=4):
    """The prescribed-cilia solve (compute_velocities under PRESCRIBED_CILIA,
    tfs_prescribed_*) at the medium swimmer's sizes: 640 beating filaments x
    20 segments on the 2562-blob sphere (R = 60), 47 366 unknowns; the
    shipped branches (zero prescribed body velocities, dynamic phase and
    shape rotation) and the free body with the same dynamic unknowns, RPY
    mobility, LINEAR_SYSTEM_TOL 1e-8. One warm-up solve, then `timed`
    consecutive warm-started solves with the phases advanced by omega0 dt
    (dt = 1e-2); wall clock per compute_velocities (it ends with a stream
    synchronisation), FP64 and FP32C."""
    from timfilsimmod_gb300.geometry import prescribed_swimmer
    from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver
    g = prescribed_swimmer(640, 20, radius=60.0, subdivisions=4, seg_sep=2.6)
    rng = np.random.default_rng(5)
    phase0 = rng.uniform(0.0, 2.0 * np.pi, g.nfil)
    omega0 = 2.0 * np.pi * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, g.nfil))
    angle0 = rng.uniform(-0.1, 0.1, g.nfil)
    t = 2.0 * np.pi * np.arange(100) / 100
    tab_p, tab_a = 1.0 + 0.5 * np.sin(t), 0.2 * np.cos(t)
    out = {"workload": (f"{g.nfil} prescribed filaments x {g.nseg} segments, "
                        f"{g.blob_references.shape[0]} blobs; RPY mobility, dynamic phase and "
                        "shape rotation, linear residual 1e-8; solves warm started from the "
                        "previous step's solution")}
    for name, flags in (("prescribed_body", 7), ("free_body", 6)):
        leg, sols = {}, {}
        for prec in ("fp64", "fp32c"):
            ps = PrescribedCiliaSolver(flags, g.nfil, g.nseg, g.blob_references, g.seg_sep, tab_p,
                                       tab_a, tol=1e-8, precision=prec)
            ps.set_solution(phase_dot=omega0)
            ms, its, cyc, rels = [], [], [], []
            for nt in range(timed + 1):
                ph = phase0 + omega0 * 1e-2 * nt
                x, vp, va = g.kinematics(ph, angle0, (0.0, 0.0, 0.0), (1.0, 0.0, 0.0, 0.0))
                t0 = time.perf_counter()
                it = ps.compute_velocities(x, vp, va, ph, omega0, angle0, omega0)
                t1 = time.perf_counter()
                if nt == 0:
                    continue
                info = ps.solve_info()
                ms.append((t1 - t0) * 1e3)
                its.append(it)
                cyc.append(info["cycles"])
                rels.append(info["rel_residual"])
            sols[prec] = ps.solution()
            leg[prec] = {"ms_per_solve": float(np.mean(ms)), "solves_per_s": 1e3 / float(np.mean(ms)),
                         "gmres_iters_mean": float(np.mean(its)), "cycles_last": int(cyc[-1]),
                         "rel_residual_max": float(np.max(rels)), "unknowns": ps.n,
                         "timed_solves": timed}
            ps.finalise()
        ref = sols["fp64"]
        dev = max(float(np.abs(sols["fp32c"][k] - ref[k]).max() / max(np.abs(ref[k]).max(), 1e-300))
                  for k in ("f_segs", "f_blobs", "phase_dot", "angle_dot"))
        leg["speedup_fp32c_vs_fp64"] = leg["fp64"]["ms_per_solve"] / leg["fp32c"]["ms_per_solve"]
        leg["fp32c_rel_dev_vs_fp64"] = dev
        out[name] = leg
    if not args.no_cpu:
        out["cpu_baseline"] = prescribed_cpu_baseline(
            g, phase0, omega0, angle0, out["prescribed_body"]["fp64"]["gmres_iters_mean"])
    return out


def prescribed_cpu_baseline(g, phase, omega0, angle, gmres_steps):
    """The prescribed-cilia solve's cost on the host cores: one application
    of the operator by the CPU restatement of the reference's solve
    (oracle/prescribed.py, pair sums in the C oracle on all threads), after one
    warm-up, times (the FP64 solve's GMRES steps + 1): one operator
    application per Arnoldi step and one for the start's residual."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from prescribed import PrescribedSystem

    x, vp, va = g.kinematics(phase, angle)
    S = PrescribedSystem(7, g.nfil, g.nseg, x, g.blob_references, (0.0, 0.0, 0.0),
                         (1.0, 0.0, 0.0, 0.0), vp, va)
    threads = os.cpu_count() or 1
    S.orc.set_threads(threads)
    v = np.random.default_rng(0).normal(size=S.n)
    S.apply_a(v)  # warm-up
    t0 = time.perf_counter()
    S.apply_a(v)
    op = time.perf_counter() - t0
    ms = op * (gmres_steps + 1) * 1e3
    return {"value": 1e3 / ms, "unit": "solves/s", "ms_per_solve": ms, "cores": threads,
            "kind": "port",
            "sample": (f"one operator application of the CPU restatement ({op:.2f} s, "
                       f"{S.n} unknowns) x (the FP64 solve's {gmres_steps:.1f} GMRES steps + 1 "
                       "residual), extrapolated")}


def solve_bench(sw, stream, args, RpyMobilitySolver, steps=None):
    """compute_velocities (barrier forces, Mss, Mbs, the free-body GMRES
    solve for blob forces and body velocity, Msb) per Broyden iteration, FP64
    vs FP32C (iterative refinement), at a 1e-8 relative linear residual. Each
    step uploads positions and slightly perturbed forces (a Broyden sequence:
    the warm start is close but not exact) and reads back the segment
    velocities, all inside the timed region."""
    import torch

    ns, nb = sw.num_segs, sw.num_blobs
    F = sw.f_segs[:, :3].sum(0)
    T = (np.cross(sw.x_segs, sw.f_segs[:, :3]) + sw.f_segs[:, 3:]).sum(0)
    rng = np.random.default_rng(99)
    steps = steps or {"fp64": max(3, min(args.steps, 5)), "fp32c": max(3, min(args.steps, 20))}
    perturb = [1e-3 * rng.normal(size=sw.f_segs.shape) for _ in range(max(steps.values()) + 2)]
    out, results = {}, {}
    for precision in ("fp64", "fp32c"):
        s = RpyMobilitySolver(1, sw.nfil, sw.nseg, nb, precision=precision)
        s.set_stream(stream.cuda_stream)
        s.set_blob_references(sw.blob_references)
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        s.set_linear_solver(1e-8)
        s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
        s.make_body_reference_matrices()

        def step(k):
            f = sw.f_segs + perturb[k]
            s.f_segs_host[:] = f.ravel()
            s.copy_segment_positions_to_device()
            s.copy_segment_forces_to_device()
            sf = np.concatenate([f[:, :3].sum(0),
                                 (np.cross(sw.x_segs, f[:, :3]) + f[:, 3:]).sum(0)])
            it, _ = s.compute_velocities(sf)
            s.copy_segment_velocities_to_host()
            s.wait_for_device()
            return it

        step(0)  # warm-up
        iters, ms = [], 0.0
        for k in range(1, steps[precision] + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            iters.append(step(k))
            b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        info = s.solve_info()
        results[precision] = s.v_segs_host.copy()
        out[precision] = {"value": steps[precision] / (ms * 1e-3), "unit": "solves/s",
                          "ms_per_solve": ms / steps[precision],
                          "gmres_iters_mean": float(np.mean(iters)),
                          "refinement_cycles_last": info["cycles"],
                          "rel_residual_last": info["rel_residual"], "steps": steps[precision]}
        s.finalise()
    # both forms ended on the same step only if their step counts match; compare the
    # FP32C result with an FP64 solve of its last step
    s = RpyMobilitySolver(1, sw.nfil, sw.nseg, nb, precision="fp64")
    s.set_stream(stream.cuda_stream)
    s.set_blob_references(sw.blob_references)
    s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
    s.set_linear_solver(1e-8)
    s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
    s.make_body_reference_matrices()
    f = sw.f_segs + perturb[steps["fp32c"]]
    s.f_segs_host[:] = f.ravel()
    s.copy_segment_forces_to_device()
    sf = np.concatenate([f[:, :3].sum(0), (np.cross(sw.x_segs, f[:, :3]) + f[:, 3:]).sum(0)])
    s.compute_velocities(sf)
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    ref = s.v_segs_host.copy()
    s.finalise()
    err = float(np.linalg.norm(results["fp32c"] - ref) / np.linalg.norm(ref))
    return {"workload": "compute_velocities (one Broyden iteration's mobility solve), "
                        "linear residual 1e-8", **out,
            "speedup_fp32c_vs_fp64": out["fp32c"]["value"] / out["fp64"]["value"],
            "fp32c_rel_l2_error_v_segs_vs_fp64": err}


def step_bench(sw, stream, args, dt=1e-3, total=100, warm=3, precisions=("fp64", "fp32c"),
               golden=None):
    """Implicit time steps of the swimmer with elastic filaments (the
    reference's cilia_sim_main.cu:355-527 loop: initial guess, internal
    forces, compute_velocities, BDF residuals, Broyden's method with the
    approximate inverse Jacobian), everything on the device, FP64 vs FP32C at
    a 1e-8 relative linear residual, Broyden TOL 1e-4. The filaments start
    straight along the surface normals; steps 0 .. total-1 run, step 0 (where
    Broyden iterates from the straight start) is reported apart, the next
    `warm` steps run untimed and the rest are timed. Each step is bracketed by
    CUDA events on the solver's stream (host gaps inside the step included),
    giving per-step latency percentiles. The FP32C segment positions are
    compared with the FP64 trajectory after every step (the error per step,
    relative to the largest position); with `golden` (the reference's own
    trajectory of this swimmer, tests/golden/step_medium*.npz) both are
    compared with the reference's positions after the steps it holds."""
    import torch

    from timfilsimmod_gb300.geometry import fibonacci_sphere
    from timfilsimmod_gb300.mobility import RpyMobilitySolver, kernel_launch_count
    from timfilsimmod_gb300.stepper import ImplicitStepper

    nfil, nseg, nb = sw.nfil, sw.nseg, sw.num_blobs
    normals = fibonacci_sphere(nfil)
    fil_refs = (sw.radius + 1.0 + 0.5 * sw.seg_sep) * normals
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * nseg * nseg)
    timed = total - 1 - warm
    out, traj, vs_ref = {}, {}, {}
    gold = None
    if golden is not None and os.path.exists(golden):
        gold = np.load(golden)
        if int(gold["nfil"]) != nfil or int(gold["nseg"]) != nseg or abs(float(gold["dt"]) - dt) > 0:
            gold = None
    for precision in precisions:
        s = RpyMobilitySolver(1, nfil, nseg, nb, precision=precision,
                              end_force_magnitude=int(efm))
        s.set_stream(stream.cuda_stream)
        s.set_blob_references(sw.blob_references)
        s.set_linear_solver(1e-8)
        st = ImplicitStepper(s, nfil, nseg, fil_refs, normals, seg_sep=sw.seg_sep, dt=dt,
                             tol=1e-4, end_force_magnitude=efm, body_radius=sw.radius)
        lat, broy, gm, xs = [], [], [], []
        launches = 0
        for nt in range(total):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = kernel_launch_count()
            a.record(stream)
            bi, gi = st.step(nt, allow_unconverged=True)
            b.record(stream)
            torch.cuda.synchronize()
            if nt > warm:
                launches += kernel_launch_count() - l0
            lat.append(a.elapsed_time(b))
            broy.append(bi)
            gm.append(gi)
            x = st.state()["x"]
            xs.append(x)
            if gold is not None and nt < len(gold["broyden_iters"]):
                tips = x.reshape(nfil, nseg, 3)[:, -1, :].ravel()
                sc = np.max(np.abs(gold["traj_tips"][-1]))
                vs_ref.setdefault(precision, []).append(
                    float(np.max(np.abs(tips - gold["traj_tips"][nt])) / sc))
        traj[precision] = xs
        tl = np.array(lat[1 + warm:])
        out[precision] = {
            "value": timed / (tl.sum() * 1e-3), "unit": "implicit steps/s",
            "ms_per_step": float(tl.mean()), "p50_ms": float(np.percentile(tl, 50)),
            "p99_ms": float(np.percentile(tl, 99)), "timed_steps": timed,
            "broyden_iters_timed": int(sum(broy[1 + warm:])),
            "gmres_iters_per_step": float(np.mean(gm[1 + warm:])),
            "step0": {"ms": lat[0], "broyden_iters": broy[0], "gmres_iters": gm[0]},
            "gpu_launches_per_step": launches / timed,
        }
        st.close()
        s.finalise()
    res = {"workload": f"{nfil} filaments x {nseg} segments, {nb} blobs; dt {dt:.6g}, "
                       f"steps 0-{total - 1} ({timed} timed), Broyden TOL 1e-4, linear residual 1e-8",
           **out}
    if "fp64" in out and "fp32c" in out:
        x64, x32 = np.array(traj["fp64"]), np.array(traj["fp32c"])
        scale = np.max(np.abs(x64), axis=1)
        dev = np.max(np.abs(x32 - x64), axis=1) / scale
        res.update({"speedup_fp32c_vs_fp64": out["fp32c"]["value"] / out["fp64"]["value"],
                    "fp32c_max_rel_position_dev_vs_fp64": float(dev.max()),
                    "fp32c_rel_position_dev_vs_fp64_last": float(dev[-1]),
                    "fp32c_rel_position_dev_vs_fp64_per_step": [float(f"{v:.3e}") for v in dev]})
    if vs_ref:
        res["rel_tip_error_vs_reference_per_step"] = {
            k: [float(f"{v:.3e}") for v in vals] for k, vals in vs_ref.items()}
        res["reference_trajectory"] = ("the reference's own step code on this swimmer "
                                       f"({os.path.basename(golden)}; its linear residual "
                                       "1e-10, here 1e-8)")
    return res


def _step_instance(nf, precision, cache, rot_seed=None):
    """One swimmer for the batch and serving legs: solver + stepper (DT 1e-3,
    TOL 1e-4, linear residual 1e-8); body reference matrices made once per
    (precision, blob count) and shared."""
    from timfilsimmod_gb300.geometry import elastic_swimmer
    from timfilsimmod_gb300.mobility import RpyMobilitySolver
    from timfilsimmod_gb300.stepper import ImplicitStepper

    blob_refs, fil_refs, dirs, radius = elastic_swimmer(int(nf))
    nb = blob_refs.shape[0]
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * 400)
    s = RpyMobilitySolver(1, int(nf), 20, nb, precision=precision, end_force_magnitude=int(efm))
    s.set_blob_references(blob_refs)
    s.set_linear_solver(1e-8, min(350, 3 * nb + 6))
    key = (precision, nb)
    if key not in cache:
        s.set_body_pose([0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])
        cache[key] = s.make_body_reference_matrices()
    else:
        s.set_body_reference_matrices(*cache[key])
    st = ImplicitStepper(s, int(nf), 20, fil_refs, dirs, make_body_matrices=False, seg_sep=2.2,
                         dt=1e-3, tol=1e-4, end_force_magnitude=efm, body_radius=radius)
    if rot_seed is not None:
        st.reset(1e-6 * np.random.default_rng(rot_seed).normal(size=(int(nf) * 20, 3)))
    return s, st


def batch_bench(args):
    """Uneven swimmers stepped together (filaments U[16, 512] x 20 segments,
    642 blobs below 128 filaments, else 2562; per-swimmer seeded N(0, 1e-6)
    segment rotations of the straight start): the FP32C batch (host worker
    pool, one stream per swimmer, all in flight at once) against the plain
    FP64 drop-in stepping the same swimmers one at a time. Steps 0-2 warm up
    (step 0 iterates Broyden from the start); the timed steps follow, timed
    on the host clock around whole batch steps (every swimmer's step ends
    with its stream synchronised)."""
    from timfilsimmod_gb300.serving import SwimmerBatch

    rng = np.random.default_rng(4242)
    nfils = rng.integers(16, 513, size=args.batch_size)
    warm, timed = 3, max(2, min(args.steps, 4))
    out, final = {}, {}
    for precision in ("fp32c", "fp64"):
        cache = {}
        inst = [_step_instance(nf, precision, cache, rot_seed=1000 + i) for i, nf in enumerate(nfils)]
        if precision == "fp32c":
            batch = SwimmerBatch(num_workers=args.batch_workers)
            for _, st in inst:
                batch.add(st)
            for nt in range(warm):
                batch.step(nt, allow_unconverged=True)
            t0 = time.perf_counter()
            iters = []
            for nt in range(warm, warm + timed):
                iters.append(batch.step(nt, allow_unconverged=True)["gmres_iters"].mean())
            sec = time.perf_counter() - t0
            shared = batch.shared_solves()
            shared_products = batch.shared_products()
            batch.close()
        else:
            for nt in range(warm):
                for _, st in inst:
                    st.step(nt, allow_unconverged=True)
            t0 = time.perf_counter()
            iters = []
            for nt in range(warm, warm + timed):
                iters.append(np.mean([st.step(nt, allow_unconverged=True)[1] for _, st in inst]))
            sec = time.perf_counter() - t0
        final[precision] = [st.state()["x"] for _, st in inst]
        n = len(inst)
        out[precision] = {"value": n * timed / sec, "unit": "swimmer-steps/s",
                          "ms_per_batch_step": 1e3 * sec / timed,
                          "gmres_iters_per_swimmer_step": float(np.mean(iters)),
                          "mode": (f"batch, {args.batch_workers} host workers, one stream per "
                                   "swimmer, inner solves and pair products in shared launches"
                                   if precision == "fp32c" else "one swimmer at a time")}
        if precision == "fp32c":
            out[precision]["shared_inner_solves"] = shared
            out[precision]["shared_products"] = shared_products
        for s, st in inst:
            st.close()
            s.finalise()
    dev = max(float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
              for a, b in zip(final["fp32c"], final["fp64"]))
    return {"workload": f"{len(nfils)} swimmers, filaments {int(nfils.min())}-{int(nfils.max())} "
                        f"x 20 segments ({int(nfils.sum()) * 20} segments in all), 642/2562 blobs; "
                        "dt 1e-3, Broyden TOL 1e-4, linear residual 1e-8",
            **out, "speedup_fp32c_batch_vs_fp64_one_at_a_time":
                out["fp32c"]["value"] / out["fp64"]["value"],
            "fp32c_max_rel_position_dev_vs_fp64": dev}


def serve_bench(args):
    """Request stream: implicit-step requests (step 0 of a base swimmer with
    N(0, 1e-6) segment rotations, as an orbit search perturbs a state), sizes
    log-uniform in 64-20 000 segments over a fixed set of base swimmers
    (filaments = segments / 20; 642 blobs below 128 filaments, else 2562),
    Poisson arrivals at each rate. FP32C server (worker pool, instances kept
    resident, admission by a device-memory budget) after one warm-up request
    per base; latency = arrival to completion. Baseline: the plain FP64
    drop-in serving the same requests one at a time."""
    from timfilsimmod_gb300.geometry import elastic_swimmer
    from timfilsimmod_gb300.serving import StepServer

    rng = np.random.default_rng(777)
    # the ends of the size range (80 segments: the smallest whole number of
    # 20-segment filaments >= 64; 20 000) and log-uniform sizes between them
    ns = np.exp(rng.uniform(np.log(64), np.log(20000), size=max(0, args.serve_bases - 2)))
    bases = sorted({4, 1000} | {max(4, min(1000, int(round(x / 20)))) for x in ns})
    geo = {nf: elastic_swimmer(nf) for nf in bases}
    efm = 220.0 * 1800.0 / (2.6 * 2.6 * 400)
    nreq = args.serve_requests

    def stream(seed):
        r = np.random.default_rng(seed)
        picks = r.integers(0, len(bases), size=nreq)
        return [(bases[k], 1e-6 * r.normal(size=(bases[k] * 20, 3))) for k in picks]

    def submit(sv, nf, rot):
        b, f, d, radius = geo[nf]
        return sv.submit(b, f, d, 20, num_steps=1, seg_rotation=rot, body_radius=radius)

    def server(precision, workers):
        sv = StepServer(num_workers=workers, hbm_budget_gb=160.0, precision=precision,
                        linear_tol=1e-8, dt=1e-3, tol=1e-4, seg_sep=2.2, end_force_magnitude=efm)
        for t in [submit(sv, nf, None) for nf in bases]:
            sv.poll(t, wait=True)
        return sv

    rates = {}
    sv = server("fp32c", args.serve_workers)
    for lam in args.serve_rates:
        reqs = stream(int(lam))
        gaps = np.random.default_rng(int(lam) + 1).exponential(1.0 / lam, size=nreq)
        t0 = time.perf_counter()
        arrive, tickets = t0, []
        for (nf, rot), gap in zip(reqs, gaps):
            arrive += gap
            while time.perf_counter() < arrive:
                time.sleep(min(1e-3, max(0.0, arrive - time.perf_counter())))
            tickets.append(submit(sv, nf, rot))
        lat = np.array([sv.poll(t, wait=True)["latency_ms"] for t in tickets])
        sec = time.perf_counter() - t0
        segs = np.array([nf * 20 for nf, _ in reqs])
        buckets = {}
        for name, lo, hi in (("<1000 segments", 0, 1000), ("1000-5000", 1000, 5000),
                             (">=5000", 5000, 1 << 30)):
            sel = lat[(segs >= lo) & (segs < hi)]
            if sel.size:
                buckets[name] = {"requests": int(sel.size), "p50_ms": float(np.percentile(sel, 50)),
                                 "p99_ms": float(np.percentile(sel, 99))}
        rates[str(lam)] = {"offered_req_per_s": lam, "steps_per_s": nreq / sec,
                           "p50_ms": float(np.percentile(lat, 50)),
                           "p99_ms": float(np.percentile(lat, 99)), "requests": nreq,
                           "by_size": buckets}
    # orbit-search requests: four Newton-Krylov searches at once (the client
    # of timfilsimmod_gb300.orbit: one Newton iteration each, GMRES(4), a
    # period of 2 steps, every period map one request) on a 128-filament base
    from timfilsimmod_gb300.orbit import OrbitSearch, search_many

    nf_o = 128
    bo, fo, do, ro = elastic_swimmer(nf_o)
    searches = [OrbitSearch(sv, bo, fo, do, 20, num_steps=2, body_radius=ro, eps_j=1e-2)
                for _ in range(4)]
    starts = [0.01 * np.random.default_rng(90 + k).normal(size=3 * nf_o * 20) for k in range(4)]
    t0 = time.perf_counter()
    recs = search_many(searches, starts, m=4, iters=1)
    sec = time.perf_counter() - t0
    lat = np.concatenate([np.array(o.latencies_ms) for o in searches])
    nreq_o = int(sum(o.requests for o in searches))
    orbit = {"workload": f"4 concurrent Newton-Krylov searches on a {nf_o * 20}-segment swimmer "
                         "(GMRES(4), one Newton iteration, period = 2 steps, eps_j 1e-2)",
             "requests": nreq_o, "requests_per_s": nreq_o / sec, "seconds": sec,
             "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
             "residual_norms": [[float(f"{v:.4e}") for v in r["residual"]] for r in recs]}
    stats = sv.stats()
    shared = sv.shared_solves()
    shared_products = sv.shared_products()
    sv.close()
    sv = server("fp64", 1)
    reqs = stream(int(args.serve_rates[0]))
    t0 = time.perf_counter()
    lat = np.array([sv.poll(submit(sv, nf, rot), wait=True)["latency_ms"] for nf, rot in reqs])
    sec = time.perf_counter() - t0
    sv.close()
    base = {"steps_per_s": nreq / sec, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "requests": nreq,
            "mode": "one request at a time (service time, no queueing)"}
    best = max(v["steps_per_s"] for v in rates.values())
    return {"workload": f"{len(bases)} base swimmers of {min(bases) * 20}-{max(bases) * 20} "
                        "segments (log-uniform), step-0 requests with N(0,1e-6) segment "
                        "rotations, Poisson arrivals; dt 1e-3, Broyden TOL 1e-4, linear "
                        "residual 1e-8",
            "fp32c_server": {"workers": args.serve_workers, "by_rate": rates,
                             "resident_instances": stats["resident_instances"],
                             "created": stats["created"], "reused": stats["reused"],
                             "shared_inner_solves": shared, "shared_products": shared_products},
            "orbit_search": orbit,
            "fp64_one_at_a_time": base,
            "speedup_best_rate_vs_fp64": best / base["steps_per_s"]}


def large_bench(stream, flush, args, peak32, peak64):
    """The large swimmer (R = 150a sphere of 10 242 blobs, 4 000 filaments x 20
    segments = 80 000 segments in planar beat shapes at uniform-random phases,
    N(0,1) forces): the grand mobility in FP32C (the work-queue launch against
    the FP32 FMA peak; autotuned) and in FP64 (the launch against the FP64 FMA
    peak; default variant), CUDA events per matvec, L2 flushed between them;
    one compute_velocities solve per Broyden iteration at a 1e-8 linear
    residual in both precisions; FP32C implicit steps from a straight start
    (DT 1e-3): step 0, where Broyden iterates, and the steps after it."""
    import torch

    from timfilsimmod_gb300.geometry import make_config
    from timfilsimmod_gb300.mobility import RpyMobilitySolver

    sw = make_config("large", seed=4321)
    ns, nb = sw.num_segs, sw.num_blobs
    flops = grand_flops(ns, nb)
    out, vel = {"workload": f"large swimmer: {ns} segments (beat shapes), {nb} blobs",
                "pairs_per_matvec": grand_pairs(ns, nb), "flops_per_matvec": flops}, {}
    for precision, reps, peak in (("fp32c", 5, peak32), ("fp64", 2, peak64)):
        s = RpyMobilitySolver(1, sw.nfil, sw.nseg, nb, precision=precision)
        s.set_stream(stream.cuda_stream)
        s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
        if precision == "fp32c" and not args.no_tune:
            s.autotune(("fp32c",), reps=1)
        s.apply_grand_mobility()  # warm-up
        torch.cuda.synchronize()
        s.enable_kernel_timing(True)
        ms = 0.0
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.apply_grand_mobility()
            b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        kt = s.kernel_timing()
        s.enable_kernel_timing(False)
        s.copy_segment_velocities_to_host()
        s.copy_blob_velocities_to_host()
        s.wait_for_device()
        vel[precision] = np.concatenate([s.v_segs_host, s.v_blobs_host]).copy()
        launch_ms = float(np.mean(kt))
        achieved = flops / (launch_ms * 1e-3) / 1e12
        out[precision] = {"value": reps / (ms * 1e-3), "unit": "matvecs/s",
                          "ms_per_matvec": ms / reps, "reps": reps,
                          "pair_interactions_per_s": grand_pairs(ns, nb) * reps / (ms * 1e-3),
                          "roofline": {"bound": f"{'fp32' if precision == 'fp32c' else 'fp64'}-fma",
                                       "achieved": achieved, "peak": peak / 1e12,
                                       "unit": "TFLOP/s", "frac": achieved / (peak / 1e12),
                                       "avg_launch_ms": launch_ms}}
        s.finalise()
    out["fp32c_rel_l2_error_vs_fp64"] = float(np.linalg.norm(vel["fp32c"] - vel["fp64"])
                                              / np.linalg.norm(vel["fp64"]))
    out["speedup_fp32c_vs_fp64"] = out["fp32c"]["value"] / out["fp64"]["value"]
    out["solve"] = solve_bench(sw, stream, args, RpyMobilitySolver,
                               steps={"fp64": 1, "fp32c": 3})
    out["implicit_steps"] = step_bench(sw, stream, args, total=5, warm=1, precisions=("fp32c",))
    return out


FLOW_SEG, FLOW_BLOB, FLOW_POINT = 44, 28, 3  # canonical flops per source, per point


def flow_bench(stream, flush, args, peak32, peak64, rank):
    """flow_velocities on a 128^3 grid (2 097 152 points) around the large
    swimmer (80 000 segments, 10 242 blobs): FP32C on the whole grid (CUDA
    events per evaluation on the flow's stream, L2 flushed between them), FP64
    on every 256th grid point (its error against FP32C stated there), the
    end-to-end call with host arrays, and the CPU oracle on a sample."""
    import torch

    from timfilsimmod_gb300.flow_field import FlowFieldEvaluator
    from timfilsimmod_gb300.geometry import flow_grid, make_config

    sw = make_config("large", seed=7 + rank)
    ns, nb = sw.num_segs, sw.num_blobs
    reach = float(np.max(np.linalg.norm(sw.x_segs, axis=1)))
    n = args.flow_grid
    xf = flow_grid(n, 1.25 * reach)
    nf = xf.shape[0]
    flops_per_point = ns * FLOW_SEG + nb * FLOW_BLOB + FLOW_POINT
    flops = flops_per_point * nf

    ev = FlowFieldEvaluator(1, sw.nfil, sw.nseg, nb, nf, precision="fp32c")
    ev.set_stream(stream.cuda_stream)
    ev.read_positions_and_forces(xf, sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs, sw.body_x)
    variant, _ = ev.autotune(reps=1)
    steps = max(3, min(args.steps, 5))
    ev.velocities(copy_to_host=False)  # warm-up
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ev.velocities(copy_to_host=False)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    ms32 = float(np.mean(ms))
    # end to end: points and sources from host arrays, velocities back to the host
    e2e_ms = []
    for _ in range(2):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev.read_positions_and_forces()
        v32 = ev.velocities().copy()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    ev.close()
    # FP64 (the reference's arithmetic) on a subset of the grid
    sub = slice(None, None, 256)
    xs_ = np.ascontiguousarray(xf[sub])
    ev64 = FlowFieldEvaluator(1, sw.nfil, sw.nseg, nb, xs_.shape[0], precision="fp64")
    ev64.set_stream(stream.cuda_stream)
    ev64.read_positions_and_forces(xs_, sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs,
                                   sw.body_x)
    ev64.velocities(copy_to_host=False)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ev64.velocities(copy_to_host=False)
    b.record(stream)
    v64 = ev64.velocities().copy()
    ms64 = a.elapsed_time(b)
    ev64.close()
    err = float(np.linalg.norm(v32[sub] - v64) / np.linalg.norm(v64))
    achieved32 = flops / (ms32 * 1e-3) / 1e12
    achieved64 = flops_per_point * xs_.shape[0] / (ms64 * 1e-3) / 1e12
    out = {"workload": f"flow_velocities, {n}^3 grid around the large swimmer "
                       f"(cube of half-width {1.25 * reach:.0f})",
           "points": nf, "segments": ns, "blobs": nb, "pairs": nf * (ns + nb),
           "value": nf / (ms32 * 1e-3), "unit": "points/s", "ms_per_grid": ms32,
           "steps": steps, "launch_variant": variant,
           "e2e": {"value": nf / (np.mean(e2e_ms) * 1e-3), "unit": "points/s",
                   "ms_per_grid": float(np.mean(e2e_ms)), "h2d_bytes_per_step":
                   8 * (3 * nf + 9 * ns + 6 * nb + 3), "d2h_bytes_per_step": 8 * 3 * nf},
           "roofline": {"bound": "fp32-fma", "kernel": "flow_kernel<float>",
                        "achieved": achieved32, "peak": peak32 / 1e12, "unit": "TFLOP/s",
                        "frac": achieved32 / (peak32 / 1e12),
                        "flops_per_launch": flops,
                        "note": "event time of velocities(): the two pack kernels "
                                "(90 242 records) inside it take microseconds"},
           "fp64_subset": {"points": xs_.shape[0], "ms": ms64,
                           "value": xs_.shape[0] / (ms64 * 1e-3), "unit": "points/s",
                           "roofline": {"bound": "fp64-fma", "achieved": achieved64,
                                        "peak": peak64 / 1e12, "unit": "TFLOP/s",
                                        "frac": achieved64 / (peak64 / 1e12)}},
           "fp32c_rel_l2_error_vs_fp64": err,
           "l2": "flushed between evaluations (256 MB write, outside the events)"}
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from oracle import Oracle

        threads = os.cpu_count() or 1
        o = Oracle(threads=threads)
        xc = np.ascontiguousarray(xf[::1024])
        t0 = time.perf_counter()
        o.flow_velocities(xc, sw.x_segs, sw.f_segs, ns, sw.x_blobs, sw.f_blobs, nb,
                          sw.body_x.reshape(1, 3), 1.0 / (8.0 * np.pi), False)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": xc.shape[0] / dt, "unit": "points/s", "cores": threads,
                               "kind": "port",
                               "sample": f"every 1024th grid point ({xc.shape[0]} points, "
                                         f"{dt:.2f} s)"}
    return out


def cpu_sample_step(o, sw, stride):
    """One sampled grand matvec on the host cores: every `stride`-th segment
    and blob target against all sources, four blocks (the oracle port of
    cuda_functions.cu:362-757). Returns the pair count."""
    xs_t, xb_t = sw.x_segs[::stride], sw.x_blobs[::stride]
    o.block(6, 6, xs_t, 1.0, sw.x_segs, sw.f_segs, 1.0)
    o.block(6, 3, xs_t, 1.0, sw.x_blobs, sw.f_blobs, 1.0)
    o.block(3, 6, xb_t, 1.0, sw.x_segs, sw.f_segs, 1.0)
    o.block(3, 3, xb_t, 1.0, sw.x_blobs, sw.f_blobs, 1.0)
    return (xs_t.shape[0] + xb_t.shape[0]) * (sw.num_segs + sw.num_blobs)


def cpu_baseline(sw, stride: int, min_seconds: float = 0.5):
    """The reference's RPY sums on the host cores (oracle port, all threads):
    one warm-up sample, then repeated samples for at least `min_seconds`,
    extrapolated to a full grand matvec by the pair count."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle

    threads = os.cpu_count() or 1
    o = Oracle(threads=threads)
    cpu_sample_step(o, sw, stride)  # warm-up (thread pool, caches)
    pairs, reps = 0, 0
    t0 = time.perf_counter()
    while True:
        pairs += cpu_sample_step(o, sw, stride)
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    rate = pairs / dt / grand_pairs(sw.num_segs, sw.num_blobs)
    return {"value": rate, "unit": "matvecs/s", "cores": threads, "kind": "port",
            "sample": f"every {stride}th target of the full grand matvec, {reps} samples "
                      f"after one warm-up ({pairs} pairs, {dt:.2f} s), extrapolated by pair count"}


def bench_config(config, ns, nb, world):
    """The `config` object of both arms' lines (the same keys and values)."""
    return {"workload": f"grand mobility, {config} swimmer", "segments": ns, "blobs": nb,
            "pairs_per_matvec": grand_pairs(ns, nb),
            "l2": "GPU arm: flushed between steps (256 MB write, outside the timed events); "
                  "CPU arm: no flush",
            "parallelism": f"replicas x{world}"}


def reference_gpu_leg(sw, reps64=3, reps32=10):
    """The reference's own kernels on this GPU (oracle/ref_gpu.py: its
    cuda_functions.cu compiled unchanged for sm_103a, launched as its
    rpy_mobility_solver launches them): one grand matvec = Mss, Msb, Mbb,
    Mbs (rpy_mobility_solver.cu:258-328), CUDA events around each kernel,
    FP64 and its shipped FP32 build. None when the kernels were not built
    here (they need the reference tree at build time)."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu

    if not torch.cuda.is_available() or not (ref_gpu.available("fp64") and ref_gpu.available("fp32")):
        return None
    ns, nb = sw.num_segs, sw.num_blobs
    out = {"kernels": "cuda_functions.cu Mss/Msb/Mbb/Mbs_mult, 64 threads per CTA, one target "
                      "per thread (the reference's launches)", "pairs_per_matvec": grand_pairs(ns, nb)}
    for precision, reps in (("fp64", reps64), ("fp32", reps32)):
        k = ref_gpu.RefGpuKernels(precision)
        dt = k.dtype
        t = {n: torch.tensor(np.asarray(a).ravel(), dtype=dt, device="cuda")
             for n, a in (("xs", sw.x_segs), ("fs", sw.f_segs), ("xb", sw.x_blobs),
                          ("fb", sw.f_blobs))}
        vs = torch.zeros(6 * ns, dtype=dt, device="cuda")
        vb = torch.zeros(3 * nb, dtype=dt, device="cuda")
        k.sync(1, sw.nseg, sw.nfil, nb)
        calls = [("Mss", lambda: k.mss(vs, t["fs"], t["xs"])),
                 ("Msb", lambda: k.msb(vs, t["fb"], t["xs"], t["xb"])),
                 ("Mbb", lambda: k.mbb(vb, t["fb"], t["xb"])),
                 ("Mbs", lambda: k.mbs(vb, t["fs"], t["xb"], t["xs"]))]
        for _, c in calls:  # warm-up
            c()
        torch.cuda.synchronize()
        per = {n: 0.0 for n, _ in calls}
        for _ in range(reps):
            for n, c in calls:
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                c()
                b.record()
                torch.cuda.synchronize()
                per[n] += a.elapsed_time(b)
        ms = sum(per.values()) / reps
        out[precision] = {"value": 1e3 / ms, "unit": "matvecs/s", "ms_per_matvec": ms,
                          "ms_per_kernel": {n: v / reps for n, v in per.items()}, "reps": reps,
                          "achieved_tflops": grand_flops(ns, nb) / (ms * 1e-3) / 1e12}
        k.close()
    return out


def reference_gpu_prescribed_leg(reps64=2, reps32=5):
    """The reference's own kernels of its prescribed-cilia build on this GPU
    (oracle/ref_gpu.py, configuration p1: forces only, rpy_interaction<3,3>,
    Mbs_mult adding): the four products of one application of the
    prescribed-cilia operator (system_matrix_mult_new's evaluate_full_mobility,
    mobility_solver.cpp:1829-1840) at the sizes of our arm's prescribed leg
    (640 beating filaments x 20 segments, 2 562 blobs), launched as its
    rpy_mobility_solver launches them, CUDA events around each kernel. Only
    the pair products: the reference's GMRES and its host-device copies per
    step come on top. None when the cubins were not built here."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu
    from timfilsimmod_gb300.geometry import prescribed_swimmer

    if not torch.cuda.is_available() or not (ref_gpu.available("fp64", "prescribed")
                                             and ref_gpu.available("fp32", "prescribed")):
        return None
    g = prescribed_swimmer(640, 20, radius=60.0, subdivisions=4, seg_sep=2.6)
    rng = np.random.default_rng(5)
    x, _, _ = g.kinematics(rng.uniform(0.0, 2.0 * np.pi, g.nfil), np.zeros(g.nfil))
    ns, nb = g.nfil * g.nseg, g.blob_references.shape[0]
    fs = np.zeros((ns, 6))
    fs[:, :3] = rng.normal(size=(ns, 3))  # the prescribed build reads forces only
    fb = rng.normal(size=(nb, 3))
    out = {"kernels": "cuda_functions.cu Mss/Msb/Mbb/Mbs_mult of the prescribed-cilia build "
                      "(configuration p1), 64 threads per CTA (the reference's launches)",
           "pairs_per_application": (ns + nb) ** 2}
    for precision, reps in (("fp64", reps64), ("fp32", reps32)):
        k = ref_gpu.RefGpuKernels(precision, "prescribed")
        dt = k.dtype
        t = {n: torch.tensor(np.asarray(a).ravel(), dtype=dt, device="cuda")
             for n, a in (("xs", x), ("fs", fs), ("xb", g.blob_references), ("fb", fb))}
        vs = torch.zeros(6 * ns, dtype=dt, device="cuda")
        vb = torch.zeros(3 * nb, dtype=dt, device="cuda")
        k.sync(1, g.nseg, g.nfil, nb)
        calls = [("Mss", lambda: k.mss(vs, t["fs"], t["xs"])),
                 ("Msb", lambda: k.msb(vs, t["fb"], t["xs"], t["xb"])),
                 ("Mbb", lambda: k.mbb(vb, t["fb"], t["xb"])),
                 ("Mbs", lambda: k.mbs(vb, t["fs"], t["xb"], t["xs"]))]
        for _, c in calls:  # warm-up
            c()
        torch.cuda.synchronize()
        ms = 0.0
        for _ in range(reps):
            for _, c in calls:
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                c()
                b.record()
                torch.cuda.synchronize()
                ms += a.elapsed_time(b)
        ms /= reps
        out[precision] = {"ms_per_application": ms, "reps": reps,
                          "achieved_tflops": 40.0 * (ns + nb) ** 2 / (ms * 1e-3) / 1e12}
        k.close()
    return out


def bench_reference(args):
    """Reference arm: the reference's RPY sums on the host cores."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return None
    from timfilsimmod_gb300.geometry import make_config

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle

    sw = make_config(args.config, seed=1234)
    threads = os.cpu_count() or 1
    o = Oracle(threads=threads)
    stride = args.cpu_sample
    ns, nb = sw.num_segs, sw.num_blobs
    pairs = 0
    for _ in range(args.warmup):
        cpu_sample_step(o, sw, stride)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pairs = cpu_sample_step(o, sw, stride)
    dt = time.perf_counter() - t0
    value = args.steps * pairs / dt / grand_pairs(ns, nb)
    sample = (f"every {stride}th target of the full grand matvec per step ({pairs} pairs), "
              f"extrapolated by pair count")
    line = {
        "impl": "reference",
        "metric": "RPY grand-mobility matvecs/s (4 blocks, medium swimmer)",
        "value": value,
        "unit": "matvecs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp64",
        "data": "synthetic (seeded icosphere + Fibonacci filaments, N(0,1) forces)",
        "config": bench_config(args.config, ns, nb, world),
        "cpu_baseline": {"value": value, "unit": "matvecs/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "matvecs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference's RPY sums (cuda_functions.cu:205-757) restated in C "
                "(oracle/tfs_oracle.c, pinned bit-close to the reference's own kernels), "
                "OpenMP over targets on the host cores",
    }
    gpu = reference_gpu_leg(sw)
    if gpu is not None:
        line["reference_gpu"] = gpu
    pres = None if args.no_prescribed else reference_gpu_prescribed_leg()
    if pres is not None:
        line["reference_gpu_prescribed"] = pres
    return line


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default="medium")
    p.add_argument("--cpu-sample", type=int, default=16,
                   help="CPU legs use every n-th target of the workload")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-tune", action="store_true", help="skip the launch autotuner")
    p.add_argument("--no-solve", action="store_true", help="skip the solve timing")
    p.add_argument("--no-flow", action="store_true", help="skip the flow-field timing")
    p.add_argument("--no-steps", action="store_true", help="skip the implicit-step timing")
    p.add_argument("--no-batch", action="store_true", help="skip the batched-swimmers timing")
    p.add_argument("--no-serve", action="store_true", help="skip the request-stream timing")
    p.add_argument("--no-large", action="store_true", help="skip the large-swimmer timing")
    p.add_argument("--no-prescribed", action="store_true",
                   help="skip the prescribed-cilia solve timing")
    p.add_argument("--batch-size", type=int, default=64, help="swimmers in the batch leg")
    p.add_argument("--batch-workers", type=int, default=32, help="host workers of the batch")
    p.add_argument("--serve-bases", type=int, default=12, help="base swimmers of the stream")
    p.add_argument("--serve-requests", type=int, default=96, help="requests per arrival rate")
    p.add_argument("--serve-workers", type=int, default=16, help="server workers")
    p.add_argument("--serve-rates", type=float, nargs="+", default=[50.0, 200.0, 1000.0, 2000.0],
                   help="Poisson arrival rates (requests/s)")
    p.add_argument("--flow-grid", type=int, default=128, help="flow points per grid axis")
    args = p.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    res = bench_reference(args) if args.impl == "reference" else bench_ours(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
