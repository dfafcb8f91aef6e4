"""GPU parity of libtfs_gb300.so, called through its C ABI (ctypes), against
the reference's own outputs (golden vectors) and the CPU oracle.

Tolerances:
  FP64 (TFS_FP64):   max-abs error <= 1e-12 x max-abs reference value
  FP32C (TFS_FP32C): ||v - v_ref||_2 <= 2e-5 ||v_ref||_2
"""
import os

import numpy as np
import pytest

from oracle import Oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12
TOL32 = 2e-5

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def rel_l2(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def load(name):
    return np.load(os.path.join(GOLD, f"{name}.npz"))


def make_solver(ns, nb, nseg, precision="fp64", **kw):
    from timfilsimmod_gb300.mobility import RpyMobilitySolver

    assert ns % nseg == 0
    return RpyMobilitySolver(1, ns // nseg, nseg, nb, precision=precision, **kw)


def run_blocks(solver, xs, fs, xb, fb):
    """Each hook on its own, in the reference's order, returning host copies."""
    out = {}
    solver.set_state(xs, fs, xb, fb)
    solver.evaluate_segment_segment_mobility()
    solver.copy_segment_velocities_to_host()
    solver.wait_for_device()
    out["v_mss"] = solver.v_segs_host.copy()
    solver.evaluate_blob_blob_mobility()
    solver.copy_blob_velocities_to_host()
    solver.wait_for_device()
    out["v_mbb"] = solver.v_blobs_host.copy()
    solver.evaluate_blob_segment_mobility()
    solver.copy_blob_velocities_to_host()
    solver.wait_for_device()
    out["v_mbs"] = solver.v_blobs_host.copy()
    # Msb accumulates (cuda_functions.cu:625-630): start from Mss, subtract
    solver.evaluate_segment_segment_mobility()
    solver.evaluate_segment_blob_mobility()
    solver.copy_segment_velocities_to_host()
    solver.wait_for_device()
    out["v_mss_plus_msb"] = solver.v_segs_host.copy()
    return out


@pytest.mark.parametrize("case", ["small_matvec", "overlap_a16"])
def test_blocks_fp64_match_reference(case):
    d = load(case)
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]), a_seg=float(d["a_seg"]),
                    a_blob=float(d["a_blob"]), mu=float(d["mu"]))
    out = run_blocks(s, xs, fs, xb, fb)
    s.finalise()
    assert rel_max(out["v_mss"], d["v_mss"]) < TOL64
    assert rel_max(out["v_mbb"], d["v_mbb"]) < TOL64
    assert rel_max(out["v_mbs"], d["v_mbs"]) < TOL64
    assert rel_max(out["v_mss_plus_msb"], d["v_mss"] + d["v_msb"]) < TOL64


@pytest.mark.parametrize("tag", ["one", "tile"])
def test_tiny_and_ragged_fp64(tag):
    d = load("tiny")
    g = {k[len(tag) + 1:]: d[k] for k in d.files if k.startswith(tag + "_")}
    xs, fs, xb, fb = g["x_segs"], g["f_segs"], g["x_blobs"], g["f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(g["nseg"]))
    out = run_blocks(s, xs, fs, xb, fb)
    s.apply_interparticle_forces()
    s.wait_for_device()
    s.finalise()
    assert rel_max(out["v_mss"], g["v_mss"]) < TOL64
    assert rel_max(out["v_mbb"], g["v_mbb"]) < TOL64
    assert rel_max(out["v_mbs"], g["v_mbs"]) < TOL64
    assert rel_max(out["v_mss_plus_msb"], g["v_mss"] + g["v_msb"]) < TOL64


@pytest.mark.parametrize("case", ["small_matvec", "overlap_a16"])
def test_barrier_forces_match_reference(case):
    """Barrier forces against the reference's own kernels. small_matvec runs
    the hashed-grid path (at most 2 particles per cell); overlap_a16 puts 17
    particles in one cell, overflows its bucket and runs the sequential
    fallback."""
    import torch

    d = load(case)
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]), a_seg=float(d["a_seg"]),
                    a_blob=float(d["a_blob"]), end_force_magnitude=int(d["end_force_magnitude"]),
                    repulsive_force_factor=float(d["repulsive_force_factor"]))
    s.set_state(xs, fs, xb, fb)
    s.apply_interparticle_forces()
    s.copy_interparticle_blob_forces_to_host()
    s.wait_for_device()
    f_dev = torch.as_tensor(s.device_arrays()["f_segs"], device="cuda").cpu().numpy()
    frep = s.f_blobs_repulsion_host.copy()
    s.finalise()
    assert rel_max(f_dev, d["f_segs_barrier"]) < TOL64
    assert rel_max(frep, d["f_blobs_repulsion"]) < TOL64


def test_full_mobility_hook_semantics():
    """evaluate_full_mobility leaves v_blobs = Mbs f_segs (rpy_mobility_solver.cu:330-337)."""
    d = load("small_matvec")
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]))
    s.set_state(xs, fs, xb, fb)
    s.evaluate_full_mobility()
    s.wait_for_device()
    vs, vb = s.v_segs_host.copy(), s.v_blobs_host.copy()
    s.finalise()
    assert rel_max(vs, d["v_mss"] + d["v_msb"]) < TOL64
    assert rel_max(vb, d["v_mbs"]) < TOL64


@pytest.mark.parametrize("case", ["small_matvec", "overlap_a16"])
def test_blocks_fp32c_error_bound(case):
    d = load(case)
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]), precision="fp32c",
                    a_seg=float(d["a_seg"]), a_blob=float(d["a_blob"]))
    out = run_blocks(s, xs, fs, xb, fb)
    s.finalise()
    errs = {k: rel_l2(out[k], d[k]) for k in ("v_mss", "v_mbb", "v_mbs")}
    errs["v_mss_plus_msb"] = rel_l2(out["v_mss_plus_msb"], d["v_mss"] + d["v_msb"])
    print("fp32c relative L2 errors", errs)
    assert max(errs.values()) < TOL32, errs


def test_weakly_coupled_product_matches_reference():
    """tfs_evaluate_weakly_coupled_segment_mobility against the reference's
    own kernels (tests/golden/weak_coupled.npz: 6 x 20 segments with an
    overlapping pair, and 5 x 7) and the oracle on the medium swimmer's
    12 800 segments: max-abs error <= 1e-12 x max-abs value, in both solver
    precisions (the product is FP64 in both)."""
    d = load("weak_coupled")
    for tag in ("six", "ragged"):
        nfil, nseg = int(d[f"{tag}_nfil"]), int(d[f"{tag}_nseg"])
        xs, fs = d[f"{tag}_x_segs"], d[f"{tag}_f_segs"]
        for precision in ("fp64", "fp32c"):
            s = make_solver(nfil * nseg, 1, nseg, precision=precision, a_seg=float(d["a_seg"]),
                            mu=float(d["mu"]))
            s.set_state(xs, fs, np.zeros((1, 3)), np.zeros((1, 3)))
            s.evaluate_weakly_coupled_segment_mobility()
            s.copy_segment_velocities_to_host()
            s.wait_for_device()
            err = rel_max(s.v_segs_host, d[f"{tag}_v_segs"])
            s.finalise()
            assert err < TOL64, (tag, precision, err)
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=9)
    s = make_solver(sw.num_segs, sw.num_blobs, sw.nseg)
    s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
    s.evaluate_weakly_coupled_segment_mobility()
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    got = s.v_segs_host.copy()
    s.finalise()
    ref = Oracle(threads=os.cpu_count() or 1).msf(sw.x_segs, sw.f_segs, sw.nfil, sw.nseg)
    assert rel_max(got, ref) < TOL64, rel_max(got, ref)


TOLFF = 1e-12


@pytest.mark.parametrize("case", ["small_matvec", "overlap_a16"])
def test_blob_blob_float_float_matches_reference(case):
    """The float-float M_bb product (the FP32C refinement residual's) against
    the reference's own M_bb: max-abs error <= 1e-12 x max-abs value, as
    FP64. overlap_a16 has overlapping blobs (the near-field branch)."""
    d = load(case)
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    for precision in ("fp64", "fp32c"):
        s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]), precision=precision,
                        a_seg=float(d["a_seg"]), a_blob=float(d["a_blob"]), mu=float(d["mu"]))
        s.set_state(xs, fs, xb, fb)
        s.evaluate_blob_blob_mobility_ff()
        s.copy_blob_velocities_to_host()
        s.wait_for_device()
        err = rel_max(s.v_blobs_host, d["v_mbb"])
        s.finalise()
        print(case, precision, "float-float M_bb error", err)
        assert err < TOLFF, (case, precision, err)


@pytest.mark.parametrize("tag", ["one", "tile"])
def test_blob_blob_float_float_tiny(tag):
    """The float-float M_bb on the reference's tiny cases (1 blob: only the
    self term; 3 blobs beside 65 segments) against the reference's M_bb."""
    d = load("tiny")
    xs, fs = d[f"{tag}_x_segs"], d[f"{tag}_f_segs"]
    xb, fb = d[f"{tag}_x_blobs"], d[f"{tag}_f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(d[f"{tag}_nseg"]), precision="fp32c",
                    a_seg=float(d["a_seg"]), a_blob=float(d["a_blob"]), mu=float(d["mu"]))
    s.set_state(xs, fs, xb, fb)
    s.evaluate_blob_blob_mobility_ff()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    err = rel_max(s.v_blobs_host, d[f"{tag}_v_mbb"])
    s.finalise()
    assert err < TOLFF, (tag, err)


def test_blob_blob_float_float_large_vs_fp64():
    """The same on the large swimmer's 10 242 blobs with N(0, 1) forces
    against the FP64 hook. The float-float rounding error is a fixed fraction
    (~2^-46) of the sum of |pair terms|, which grows with the blob count
    while random forces keep |v| small: the bar here is 1e-11 of the largest
    velocity (measured 1.8e-12), still far below what the 1e-8 refinement
    residual needs."""
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("large", seed=8)
    s = make_solver(sw.num_segs, sw.num_blobs, sw.nseg)
    s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
    s.evaluate_blob_blob_mobility()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    ref = s.v_blobs_host.copy()
    s.evaluate_blob_blob_mobility_ff()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    err = rel_max(s.v_blobs_host, ref)
    s.finalise()
    print("large float-float M_bb error vs FP64", err)
    assert err < 1e-11


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_grand_mobility_medium_vs_oracle(precision):
    """The whole grand mobility of the medium swimmer (12 800 segments, 2562
    blobs) against the oracle."""
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=5)
    s = make_solver(sw.num_segs, sw.num_blobs, sw.nseg, precision=precision)
    s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
    s.apply_grand_mobility()
    s.copy_segment_velocities_to_host()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    vs, vb = s.v_segs_host.copy(), s.v_blobs_host.copy()
    s.finalise()
    o = Oracle(threads=os.cpu_count() or 1)
    ref_s = o.msb(sw.x_segs, sw.x_blobs, sw.f_blobs, o.mss(sw.x_segs, sw.f_segs))
    ref_b = o.mbs(sw.x_blobs, sw.x_segs, sw.f_segs) + o.mbb(sw.x_blobs, sw.f_blobs)
    if precision == "fp64":
        assert rel_max(vs, ref_s) < TOL64 and rel_max(vb, ref_b) < TOL64
    else:
        es, eb = rel_l2(vs, ref_s), rel_l2(vb, ref_b)
        print("fp32c medium errors", es, eb)
        assert es < TOL32 and eb < TOL32


def _grand(s, fs, fb):
    s.f_segs_host[:] = fs
    s.f_blobs_host[:] = fb
    s.copy_segment_forces_to_device()
    s.copy_blob_forces_to_device()
    s.apply_grand_mobility()
    s.copy_segment_velocities_to_host()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    return np.concatenate([s.v_segs_host, s.v_blobs_host])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp32c", 2e-5)])
def test_large_swimmer_symmetry_and_linearity(precision, tol):
    """Size-independent properties at the full large size (80 000 segments,
    10 242 blobs): the grand mobility is symmetric (u.Mw = w.Mu) and linear."""
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("large", seed=6)
    rng = np.random.default_rng(8)
    s = make_solver(sw.num_segs, sw.num_blobs, sw.nseg, precision=precision)
    s.x_segs_host[:] = sw.x_segs.ravel()
    s.x_blobs_host[:] = sw.x_blobs.ravel()
    s.copy_segment_positions_to_device()
    s.copy_blob_positions_to_device()
    ns, nb = 6 * sw.num_segs, 3 * sw.num_blobs
    u = rng.normal(size=ns + nb)
    w = rng.normal(size=ns + nb)
    Mu = _grand(s, u[:ns], u[ns:])
    Mw = _grand(s, w[:ns], w[ns:])
    M2u = _grand(s, 2.5 * u[:ns], 2.5 * u[ns:])
    s.finalise()
    a, b = np.dot(w, Mu), np.dot(u, Mw)
    assert abs(a - b) <= tol * np.linalg.norm(w) * np.linalg.norm(Mu)
    assert rel_l2(M2u, 2.5 * Mu) < tol


def test_native_library_is_loaded_and_counts_launches():
    from timfilsimmod_gb300 import _native
    from timfilsimmod_gb300.mobility import kernel_launch_count

    before = kernel_launch_count()
    d = load("tiny")
    s = make_solver(65, 3, 5)
    s.set_state(d["tile_x_segs"], d["tile_f_segs"], d["tile_x_blobs"], d["tile_f_blobs"])
    s.evaluate_segment_segment_mobility()
    s.wait_for_device()
    s.finalise()
    assert kernel_launch_count() > before
    maps = open("/proc/self/maps").read()
    assert os.path.basename(_native.lib_path()) in maps


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_every_launch_variant_matches_reference(precision):
    """Every compiled work-queue variant (the products) and tile-kernel
    variant at two split targets (set for every combination; the
    kernel-sequence GMRES's blob-blob product uses it), on the ragged
    unequal-radius case (all branches) and on the small swimmer."""
    from timfilsimmod_gb300.mobility import QUEUE_KINDS, num_queue_variants, num_tile_variants

    nq = num_queue_variants(precision)
    for case in ("overlap_a16", "small_matvec"):
        d = load(case)
        xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
        s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]), precision=precision,
                        a_seg=float(d["a_seg"]), a_blob=float(d["a_blob"]))
        for var in range(max(num_tile_variants(precision), nq)):
            for cps in (1, 3):
                for combo in range(6):
                    s.set_tuning(combo, var % num_tile_variants(precision), cps)
                for kind in range(len(QUEUE_KINDS)):
                    s.set_queue_variant(kind, var % nq)
                out = run_blocks(s, xs, fs, xb, fb)
                s.apply_grand_mobility()
                s.copy_segment_velocities_to_host()
                s.copy_blob_velocities_to_host()
                s.wait_for_device()
                gs, gb = s.v_segs_host.copy(), s.v_blobs_host.copy()
                ref = {"v_mss": d["v_mss"], "v_mbb": d["v_mbb"], "v_mbs": d["v_mbs"],
                       "v_mss_plus_msb": d["v_mss"] + d["v_msb"]}
                for k, r in ref.items():
                    e = rel_max(out[k], r) if precision == "fp64" else rel_l2(out[k], r)
                    assert e < (TOL64 if precision == "fp64" else TOL32), (case, var, cps, k, e)
                eg = (rel_max if precision == "fp64" else rel_l2)(
                    np.concatenate([gs, gb]),
                    np.concatenate([d["v_mss"] + d["v_msb"], d["v_mbs"] + d["v_mbb"]]))
                assert eg < (TOL64 if precision == "fp64" else TOL32), (case, var, cps, "grand", eg)
        s.finalise()


def test_autotune_table_and_parity():
    d = load("small_matvec")
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    s = make_solver(xs.shape[0], xb.shape[0], int(d["nseg"]))
    s.set_state(xs, fs, xb, fb)
    table = s.autotune(reps=1)
    assert set(table) == {"fp64", "fp32c"}
    for p in ("fp64", "fp32c"):
        for k in ("queue seg<-seg", "queue grand", "queue seg,blob<-seg", "blob<-blob"):
            assert table[p][k]["ms"] > 0, (p, k)
    out = run_blocks(s, xs, fs, xb, fb)
    s.finalise()
    assert rel_max(out["v_mss"], d["v_mss"]) < TOL64


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("nfil,nblob", [(0, 40), (6, 0), (0, 0)])
def test_one_sided_and_empty_systems(precision, nfil, nblob):
    """Systems without segments, without blobs, or with neither (the
    reference's NFIL = 0 and NBLOB = 0 builds): every hook returns TFS_OK, a
    product with no sources assigns zero (or leaves an accumulation alone),
    and what is there matches the oracle."""
    nseg = 4
    ns = nfil * nseg
    rng = np.random.default_rng(17)
    # distinct sites of a 2.3-spaced lattice: no pair inside contact
    sites = 2.3 * np.stack(np.meshgrid(*[np.arange(5)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pick = rng.permutation(len(sites))
    xs, xb = sites[pick[:ns]], sites[pick[ns:ns + nblob]]
    fs, fb = rng.normal(size=(ns, 6)), rng.normal(size=(nblob, 3))
    s = make_solver(ns, nblob, nseg, precision=precision)
    out = run_blocks(s, xs, fs, xb, fb)
    s.apply_grand_mobility()
    s.copy_segment_velocities_to_host()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    vs, vb = s.v_segs_host.copy(), s.v_blobs_host.copy()
    s.apply_interparticle_forces()
    s.wait_for_device()
    s.finalise()
    assert vs.size == 6 * ns and vb.size == 3 * nblob
    o = Oracle()
    cmp = rel_max if precision == "fp64" else rel_l2
    tol = TOL64 if precision == "fp64" else TOL32
    if ns:
        ref_ss = o.mss(xs, fs)
        assert cmp(out["v_mss"], ref_ss) < tol
        # no blobs: Msb adds nothing to Mss
        assert cmp(out["v_mss_plus_msb"], ref_ss if not nblob else
                   o.msb(xs, xb, fb, ref_ss.copy())) < tol
        assert cmp(vs, ref_ss) < tol
    if nblob:
        ref_bb = o.mbb(xb, fb)
        assert cmp(out["v_mbb"], ref_bb) < tol
        # no segments: Mbs assigns zero
        assert np.all(out["v_mbs"] == 0.0)
        assert cmp(vb, ref_bb) < tol


def test_float_host_arrays_match_float64_path():
    """The float host-array copies (the reference's Real = float build):
    positions and forces given as float32, velocities and the blob repulsion
    read back as float32, equal bit for bit to the float32 rounding of the
    float64 path on the same (float32-representable) inputs."""
    import ctypes

    d = load("small_matvec")
    xs, fs = d["x_segs"].astype(np.float32), d["f_segs"].astype(np.float32)
    xb, fb = d["x_blobs"].astype(np.float32), d["f_blobs"].astype(np.float32)
    ns, nb = xs.shape[0], xb.shape[0]

    def p(a):
        return ctypes.c_void_p(a.ctypes.data)

    s64 = make_solver(ns, nb, int(d["nseg"]))
    s64.set_state(xs, fs, xb, fb)
    s64.apply_interparticle_forces()
    s64.evaluate_segment_segment_mobility()
    s64.evaluate_segment_blob_mobility()
    s64.evaluate_blob_segment_mobility()
    s64.copy_segment_velocities_to_host()
    s64.copy_blob_velocities_to_host()
    s64.copy_interparticle_blob_forces_to_host()
    s64.wait_for_device()
    want = [s64.v_segs_host.copy(), s64.v_blobs_host.copy(), s64.f_blobs_repulsion_host.copy()]
    s64.finalise()

    s = make_solver(ns, nb, int(d["nseg"]))
    xs_, fs_, xb_, fb_ = (np.ascontiguousarray(a.ravel()) for a in (xs, fs, xb, fb))
    s._call("tfs_copy_segment_positions_to_device_f32", p(xs_))
    s._call("tfs_copy_segment_forces_to_device_f32", p(fs_))
    s._call("tfs_copy_blob_positions_to_device_f32", p(xb_))
    s._call("tfs_copy_blob_forces_to_device_f32", p(fb_))
    s.apply_interparticle_forces()
    s.evaluate_segment_segment_mobility()
    s.evaluate_segment_blob_mobility()
    s.evaluate_blob_segment_mobility()
    got = [np.empty(6 * ns, np.float32), np.empty(3 * nb, np.float32), np.empty(3 * nb, np.float32)]
    s._call("tfs_copy_segment_velocities_to_host_f32", p(got[0]))
    s._call("tfs_copy_blob_velocities_to_host_f32", p(got[1]))
    s._call("tfs_copy_interparticle_blob_forces_to_host_f32", p(got[2]))
    s.wait_for_device()
    s.finalise()
    for g, w in zip(got, want):
        assert np.array_equal(g, w.astype(np.float32))


def test_host_arrays_are_page_locked():
    """The solver's and the flow evaluator's host arrays are page-locked, so
    the copy hooks run at DMA speed without staging through pageable memory."""
    from timfilsimmod_gb300.flow_field import FlowFieldEvaluator
    from timfilsimmod_gb300.mobility import RpyMobilitySolver, host_array_pinned

    s = RpyMobilitySolver(1, 4, 5, 12, precision="fp64")
    try:
        for name in ("x_segs_host", "f_segs_host", "v_segs_host", "x_blobs_host",
                     "f_blobs_host", "v_blobs_host", "f_blobs_repulsion_host"):
            assert host_array_pinned(getattr(s, name)), name
    finally:
        s.finalise()
    ev = FlowFieldEvaluator(1, 4, 5, 12, 64, precision="fp64")
    try:
        for name in ("x_flow_host", "v_flow_host", "x_segs_host", "f_segs_host"):
            assert host_array_pinned(getattr(ev, name)), name
    finally:
        ev.close()
