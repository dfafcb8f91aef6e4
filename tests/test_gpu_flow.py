"""GPU parity of the flow-field evaluator (tfs_flow_*, through the C ABI)
against the reference's own outputs (golden vectors from its flow_velocities
kernel) and the CPU oracle.

Tolerances:
  FP64 (TFS_FP64):   max-abs error <= 1e-12 x max-abs reference value
  FP32C (TFS_FP32C): ||v - v_ref||_2 <= 2e-5 ||v_ref||_2
                     (5e-5 with the net-force Stokeslet removed: the result is
                     a difference of nearly equal sums)
"""
import os

import numpy as np
import pytest

from oracle import Oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12
TOL32 = 2e-5
TOL32_RNF = 5e-5

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def rel_l2(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def evaluate(xf, xs, fs, xb, fb, xbod, segs_per_body, blobs_per_body, rnf, precision,
             mu=1.0):
    from timfilsimmod_gb300.flow_field import FlowFieldEvaluator

    nbod = np.asarray(xbod).size // 3
    nflow = np.asarray(xf).size // 3
    with FlowFieldEvaluator(nbod, 1, segs_per_body, blobs_per_body, nflow, mu=mu,
                            remove_net_force=rnf, precision=precision) as ev:
        ev.read_positions_and_forces(xf, xs, fs, xb if blobs_per_body else None,
                                     fb if blobs_per_body else None, xbod)
        return ev.velocities().ravel().copy()


GOLDEN_CASES = [("v_blobs", False, False), ("v_blobs_rnf", True, False),
                ("v_wall", False, True)]


@pytest.mark.parametrize("key,rnf,wall", GOLDEN_CASES)
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_flow_matches_reference(key, rnf, wall, precision):
    d = np.load(os.path.join(GOLD, "flow_small.npz"))
    ns, nb = d["x_segs"].shape[0], d["x_blobs"].shape[0]
    xs = d["x_segs_wall"] if wall else d["x_segs"]
    xbod = d["x_bodies"] + (np.array([0.0, 0.0, 90.0]) if wall else 0.0)
    v = evaluate(d["x_flow"], xs, d["f_segs"], d["x_blobs"], d["f_blobs"], xbod, ns,
                 0 if wall else nb, rnf, precision)
    assert np.all(np.isfinite(v))
    if precision == "fp64":
        assert rel_max(v, d[key]) < TOL64
    else:
        assert rel_l2(v, d[key]) < (TOL32_RNF if rnf else TOL32)


def random_bodies(rng, nbod, segs_per_body, blobs_per_body, wall):
    centres = rng.uniform(-60.0, 60.0, size=(nbod, 3))
    if wall:
        centres[:, 2] = rng.uniform(30.0, 50.0, size=nbod)
    xs = (centres[:, None, :] + rng.uniform(-12.0, 12.0, size=(nbod, segs_per_body, 3))
          ).reshape(-1, 3)
    xb = (centres[:, None, :] + rng.uniform(-10.0, 10.0, size=(nbod, blobs_per_body, 3))
          ).reshape(-1, 3)
    fs = rng.normal(size=(nbod * segs_per_body, 6))
    fb = rng.normal(size=(nbod * blobs_per_body, 3))
    return centres, xs, fs, xb, fb


@pytest.mark.parametrize("wall", [False, True])
@pytest.mark.parametrize("rnf", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_flow_many_bodies_matches_oracle(wall, rnf, precision):
    """Three bodies (the net-force term uses each source's own body centre),
    ragged sizes: 1001 points, 77 segments and 45 blobs per body."""
    rng = np.random.default_rng(31 + 2 * wall + rnf)
    nbod, spb, bpb = 3, 77, 0 if wall else 45
    centres, xs, fs, xb, fb = random_bodies(rng, nbod, spb, max(bpb, 1), wall)
    if bpb == 0:
        xb, fb = xb[:0], fb[:0]
    xf = rng.uniform(-90.0, 90.0, size=(1001, 3))
    if wall:
        xf[:, 2] = np.abs(xf[:, 2]) + 0.5
    mu = 0.7
    prefac = 1.0 / (8.0 * np.pi * mu)
    ref = Oracle().flow_velocities(xf, xs, fs, spb, xb, fb, bpb, centres, prefac, rnf)
    v = evaluate(xf, xs, fs, xb, fb, centres, spb, bpb, rnf, precision, mu=mu)
    if precision == "fp64":
        assert rel_max(v, ref) < TOL64
    else:
        assert rel_l2(v, ref) < (TOL32_RNF if rnf else TOL32)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_flow_large_point_set(precision):
    """200 000 points (more CTAs than fill the GPU: no source splitting)
    against the oracle, FP64 bit-for-bit within the tolerance."""
    rng = np.random.default_rng(5)
    centres, xs, fs, xb, fb = random_bodies(rng, 1, 120, 64, False)
    xf = rng.uniform(-100.0, 100.0, size=(200_000, 3))
    prefac = 1.0 / (8.0 * np.pi)
    ref = Oracle().flow_velocities(xf, xs, fs, 120, xb, fb, 64, centres, prefac, False)
    v = evaluate(xf, xs, fs, xb, fb, centres, 120, 64, False, precision)
    if precision == "fp64":
        assert rel_max(v, ref) < TOL64
    else:
        assert rel_l2(v, ref) < TOL32


def test_flow_no_points_and_errors():
    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.flow_field import FlowFieldEvaluator

    rng = np.random.default_rng(3)
    centres, xs, fs, xb, fb = random_bodies(rng, 1, 10, 5, False)
    with FlowFieldEvaluator(1, 1, 10, 5, 0) as ev:
        ev.read_positions_and_forces(np.zeros(0), xs, fs, xb, fb, centres)
        assert ev.velocities().shape == (0, 3)
    with FlowFieldEvaluator(1, 1, 10, 5, 4, mu=-1.0) as ev:
        ev.read_positions_and_forces(np.ones(12), xs, fs, xb, fb, centres)
        with pytest.raises(N.TfsError) as e:
            ev.velocities()
        assert e.value.code == N.TFS_EINVAL
    with pytest.raises(N.TfsError):
        FlowFieldEvaluator(0, 1, 10, 5, 4)


def test_flow_repeatable():
    """Two evaluations of the same inputs give identical bits (the source
    splits are summed in a fixed order)."""
    d = np.load(os.path.join(GOLD, "flow_small.npz"))
    ns, nb = d["x_segs"].shape[0], d["x_blobs"].shape[0]
    a = evaluate(d["x_flow"], d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"],
                 d["x_bodies"], ns, nb, True, "fp32c")
    b = evaluate(d["x_flow"], d["x_segs"], d["f_segs"], d["x_blobs"], d["f_blobs"],
                 d["x_bodies"], ns, nb, True, "fp32c")
    assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_flow_every_variant_and_autotune(precision):
    """Every launch variant of the flow kernel, and the autotuner's pick, on
    the wall case with the net-force Stokeslet removed (three bodies)."""
    from timfilsimmod_gb300.flow_field import FlowFieldEvaluator

    rng = np.random.default_rng(77)
    centres, xs, fs, _, _ = random_bodies(rng, 3, 60, 1, True)
    xf = rng.uniform(-80.0, 80.0, size=(700, 3))
    xf[:, 2] = np.abs(xf[:, 2]) + 0.5
    ref = Oracle().flow_velocities(xf, xs, fs, 60, np.zeros((0, 3)), np.zeros((0, 3)), 0,
                                   centres, 1.0 / (8.0 * np.pi), True)
    with FlowFieldEvaluator(3, 1, 60, 0, 700, remove_net_force=True, precision=precision) as ev:
        ev.read_positions_and_forces(xf, xs, fs, None, None, centres)
        for var in range(ev.num_variants()):
            ev.set_variant(var)
            v = ev.velocities().ravel().copy()
            if precision == "fp64":
                assert rel_max(v, ref) < TOL64, var
            else:
                assert rel_l2(v, ref) < TOL32_RNF, var
        best, ms = ev.autotune(reps=1)
        assert 0 <= best < ev.num_variants() and ms > 0
        v = ev.velocities().ravel().copy()
        assert rel_max(v, ref) < (TOL64 if precision == "fp64" else 1e-4)
