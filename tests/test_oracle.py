"""The CPU oracle (oracle/tfs_oracle.c) against the reference's own outputs.

Golden vectors in tests/golden/ were produced by the reference's kernels
(cuda_functions.cu, flow_field_evaluator.cu) compiled unchanged for the CPU
(tests/golden/make_golden.py). Where that reference build is present
(oracle/_ref/), the oracle is also checked against it on fresh seeded cases.
Analytic known answers of the RPY tensor pin the physics independently.
"""
import os

import numpy as np
import pytest

from oracle import Oracle, ReferenceFlow, ReferenceKernels

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-13  # max-abs error relative to the max-abs reference value


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def load(name):
    return np.load(os.path.join(GOLD, f"{name}.npz"))


def oracle_for(d, threads=4):
    return Oracle(float(d["mu"]), float(d["a_seg"]), float(d["a_blob"]), threads=threads)


@pytest.mark.parametrize("case", ["small_matvec", "overlap_a16"])
def test_blocks_match_reference_golden(case):
    d = load(case)
    o = oracle_for(d)
    xs, fs, xb, fb = d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    assert rel(o.mss(xs, fs), d["v_mss"]) < TOL
    assert rel(o.msb(xs, xb, fb), d["v_msb"]) < TOL
    assert rel(o.mbb(xb, fb), d["v_mbb"]) < TOL
    assert rel(o.mbs(xb, xs, fs), d["v_mbs"]) < TOL


@pytest.mark.parametrize("case", ["small_matvec", "overlap_a16"])
def test_barrier_matches_reference_golden(case):
    d = load(case)
    o = oracle_for(d)
    fsb, frep = o.barrier_forces(d["x_segs"], d["x_blobs"], d["f_segs"], int(d["nseg"]),
                                 int(d["end_force_magnitude"]),
                                 float(d["repulsive_force_factor"]), free_body=True)
    assert np.isfinite(fsb).all()
    assert rel(fsb, d["f_segs_barrier"]) < TOL
    assert rel(frep, d["f_blobs_repulsion"]) < TOL
    # the case has contacts, so the barrier did something
    assert np.max(np.abs(fsb - d["f_segs"].ravel())) > 1.0


@pytest.mark.parametrize("tag", ["one", "tile"])
def test_tiny_and_ragged(tag):
    d = load("tiny")
    o = Oracle(float(d["mu"]), float(d["a_seg"]), float(d["a_blob"]))
    g = {k[len(tag) + 1:]: d[k] for k in d.files if k.startswith(tag + "_")}
    xs, fs, xb, fb = g["x_segs"], g["f_segs"], g["x_blobs"], g["f_blobs"]
    assert rel(o.mss(xs, fs), g["v_mss"]) < TOL
    assert rel(o.msb(xs, xb, fb), g["v_msb"]) < TOL
    assert rel(o.mbb(xb, fb), g["v_mbb"]) < TOL
    assert rel(o.mbs(xb, xs, fs), g["v_mbs"]) < TOL
    fsb, frep = o.barrier_forces(xs, xb, fs, int(g["nseg"]), int(d["end_force_magnitude"]))
    assert rel(fsb, g["f_segs_barrier"]) < TOL


def test_flow_matches_reference_golden():
    d = load("flow_small")
    o = Oracle(threads=4)
    xf, xs, fs, xb, fb = d["x_flow"], d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"]
    ns, nb = xs.shape[0], xb.shape[0]
    pre = float(d["prefac"])
    assert rel(o.flow_velocities(xf, xs, fs, ns, xb, fb, nb, d["x_bodies"], pre), d["v_blobs"]) < TOL
    assert rel(o.flow_velocities(xf, xs, fs, ns, xb, fb, nb, d["x_bodies"], pre, True),
               d["v_blobs_rnf"]) < TOL
    lift = np.array([[0.0, 0.0, 90.0]])
    assert rel(o.flow_velocities(xf, d["x_segs_wall"], fs, ns, xb, fb, 0, d["x_bodies"] + lift,
                                 pre), d["v_wall"]) < TOL


def test_thread_count_does_not_change_results():
    d = load("small_matvec")
    a = Oracle(threads=1).mss(d["x_segs"], d["f_segs"])
    b = Oracle(threads=4).mss(d["x_segs"], d["f_segs"])
    assert np.array_equal(a, b)


# --------------------------------------------------------------------------
# analytic known answers (cuda_functions.cu:251-254, :339-344; Zuk et al.)
# --------------------------------------------------------------------------
def pair_matrix(o, vd, fd, xi, xj, ai, aj, mu=1.0):
    import ctypes
    M = np.zeros((vd, fd))
    P = ctypes.POINTER(ctypes.c_double)
    for k in range(fd):
        F = np.zeros(fd)
        F[k] = 1.0
        V = np.zeros(vd)
        o.lib.orc_rpy_pair(vd, fd, V.ctypes.data_as(P), F.ctypes.data_as(P),
                           *[ctypes.c_double(v) for v in (*xi, ai, *xj, aj, mu)])
        M[:, k] = V
    return M


def test_self_mobility_known_answer():
    o = Oracle()
    for a in (1.0, 0.7):
        M = pair_matrix(o, 6, 6, (1.0, 2.0, 3.0), (1.0, 2.0, 3.0), a, a)
        np.testing.assert_allclose(M[:3, :3], np.eye(3) / (6 * np.pi * a), rtol=1e-15)
        np.testing.assert_allclose(M[3:, 3:], np.eye(3) / (8 * np.pi * a ** 3), rtol=1e-15)
        assert np.all(M[:3, 3:] == 0) and np.all(M[3:, :3] == 0)


@pytest.mark.parametrize("r", [0.3, 1.2, 1.999, 2.5, 7.0])
def test_pair_symmetry(r):
    """M_ij = M_ji^T for the grand mobility (equal radii)."""
    o = Oracle()
    rng = np.random.default_rng(int(r * 1000))
    e = rng.normal(size=3)
    e /= np.linalg.norm(e)
    xi, xj = np.zeros(3), r * e
    Mij = pair_matrix(o, 6, 6, xi, xj, 1.0, 1.0)
    Mji = pair_matrix(o, 6, 6, xj, xi, 1.0, 1.0)
    np.testing.assert_allclose(Mij, Mji.T, atol=1e-15)


def test_far_field_oseen_limit():
    """At large r the translation block tends to the Oseen tensor."""
    o = Oracle()
    r = 1e4
    e = np.array([0.6, 0.0, 0.8])
    M = pair_matrix(o, 3, 3, np.zeros(3), r * e, 1.0, 1.0)
    oseen = (np.eye(3) + np.outer(e, e)) / (8 * np.pi * r)
    np.testing.assert_allclose(M, oseen, rtol=1e-7)


def test_continuity_at_contact():
    """The far and overlap forms agree at r = ai + aj (and for ai != aj)."""
    o = Oracle()
    for ai, aj in ((1.0, 1.0), (1.0, 1.6)):
        e = np.array([0.0, 0.6, 0.8])
        r = ai + aj
        lo = pair_matrix(o, 6, 6, np.zeros(3), (r * (1 - 1e-9)) * e, ai, aj)
        hi = pair_matrix(o, 6, 6, np.zeros(3), (r * (1 + 1e-9)) * e, ai, aj)
        np.testing.assert_allclose(lo, hi, atol=1e-8)


def test_grand_mobility_positive_definite():
    """The RPY grand mobility of a random cloud is symmetric positive definite."""
    o = Oracle()
    rng = np.random.default_rng(4)
    x = rng.uniform(-3, 3, size=(12, 3))
    n = x.shape[0]
    G = np.zeros((6 * n, 6 * n))
    for i in range(n):
        for j in range(n):
            G[6 * i:6 * i + 6, 6 * j:6 * j + 6] = pair_matrix(o, 6, 6, x[i], x[j], 1.0, 1.0)
    np.testing.assert_allclose(G, G.T, atol=1e-14)
    assert np.linalg.eigvalsh(G).min() > 0


# --------------------------------------------------------------------------
# against the reference build itself, where it exists (this container)
# --------------------------------------------------------------------------
@pytest.mark.skipif(not ReferenceKernels.available("a1"), reason="reference build absent")
@pytest.mark.parametrize("seed", [21, 22])
def test_oracle_matches_reference_build(seed):
    from timfilsimmod_gb300.geometry import make_swimmer

    sw = make_swimmer(radius=8.0, subdivisions=2, nfil=6, nseg=9, seed=seed, shape="beat")
    ref = ReferenceKernels("a1")
    ref.sync(1, sw.nseg, sw.nfil, sw.num_blobs, 50, 2.2)
    o = Oracle(threads=4)
    xs, fs, xb, fb = sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs
    assert rel(o.mss(xs, fs), ref.mss(xs, fs)) < TOL
    assert rel(o.msb(xs, xb, fb), ref.msb(xs, xb, fb)) < TOL
    assert rel(o.mbb(xb, fb), ref.mbb(xb, fb)) < TOL
    assert rel(o.mbs(xb, xs, fs), ref.mbs(xb, xs, fs)) < TOL
    fsb_r, frep_r = ref.barrier_forces(xs, xb, fs)
    fsb_o, frep_o = o.barrier_forces(xs, xb, fs, sw.nseg, 50)
    assert rel(fsb_o, fsb_r) < TOL and rel(frep_o, frep_r) < TOL


@pytest.mark.skipif(not ReferenceFlow.available(), reason="reference build absent")
def test_oracle_flow_matches_reference_build():
    from timfilsimmod_gb300.geometry import make_swimmer

    sw = make_swimmer(radius=8.0, subdivisions=2, nfil=6, nseg=9, seed=5)
    rng = np.random.default_rng(9)
    xf = rng.uniform(-30, 30, size=(100, 3))
    xbod = np.zeros((1, 3))
    o, r = Oracle(threads=4), ReferenceFlow()
    for nb, rnf in ((sw.num_blobs, False), (sw.num_blobs, True)):
        a = o.flow_velocities(xf, sw.x_segs, sw.f_segs, sw.num_segs, sw.x_blobs, sw.f_blobs, nb,
                              xbod, 0.04, rnf)
        b = r.flow_velocities(xf, sw.x_segs, sw.f_segs, sw.num_segs, sw.x_blobs, sw.f_blobs, nb,
                              xbod, 0.04, rnf)
        assert rel(a, b) < TOL


def test_reference_data_files_have_the_record_layout():
    """The reference's plot-step files and backup (tests/golden/step_io/ref*,
    written by its own swimmer::write_data / write_backup and
    mobility_solver::write_data) have the record sizes the C ABI writer
    follows: backup 1 + NFIL (9 + 28 NSEG) + 19 numbers, one quaternion per
    segment, body x and q, a tether force per filament, 6 velocities or
    forces per segment, 3 forces per blob, 6 body velocities."""
    d = np.load(os.path.join(GOLD, "step_io.npz"))
    nfil, nseg, nb = int(d["nfil"]), int(d["nseg"]), d["blob_refs"].shape[0]
    ns = nfil * nseg
    io = os.path.join(GOLD, "step_io", "ref")
    sizes = {".backup": 1 + nfil * (9 + 28 * nseg) + 19, "_seg_states.dat": 1 + 4 * ns,
             "_body_states.dat": 1 + 7, "_tether_force.dat": 1 + 3 * nfil,
             "_seg_vels.dat": 1 + 6 * ns, "_seg_forces.dat": 1 + 6 * ns,
             "_blob_forces.dat": 1 + 3 * nb, "_body_vels.dat": 6}
    for suffix, n in sizes.items():
        text = open(io + suffix).read()
        assert text.endswith(" \n") and text.count("\n") == 1, suffix
        toks = text.split()
        assert len(toks) == n, (suffix, len(toks), n)
        if suffix != "_body_vels.dat":
            assert toks[0] in ("2", "3"), suffix  # step nt = 2, save step 3
            assert all(len(t.split("e")[0].split(".")[-1]) == 10 for t in toks[1:]), suffix


def test_weakly_coupled_oracle_matches_reference_golden():
    """orc_msf (the weakly coupled filaments' product) against the
    reference's own filament-mean, total-force and Msf_mult kernels
    (tests/golden/weak_coupled.npz): the reference sums means and totals
    with atomic adds, so agreement is to rounding, <= 1e-14 of the largest
    velocity."""
    d = np.load(os.path.join(GOLD, "weak_coupled.npz"))
    o = Oracle(mu=float(d["mu"]), a_seg=float(d["a_seg"]))
    for tag in ("six", "ragged"):
        v = o.msf(d[f"{tag}_x_segs"], d[f"{tag}_f_segs"], int(d[f"{tag}_nfil"]),
                  int(d[f"{tag}_nseg"]))
        ref = d[f"{tag}_v_segs"]
        assert np.max(np.abs(v - ref)) <= 1e-14 * np.max(np.abs(ref)), tag
        assert np.all(ref.reshape(-1, 6)[:, 3:] == 0.0)
