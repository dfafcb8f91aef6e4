"""The CPU restatement of the reference's prescribed-cilia solve
(oracle/prescribed.py) against the reference's own solver compiled for the
CPU (tests/golden/prescribed_p*.npz: mobility_solver.cpp under
PRESCRIBED_CILIA in three configurations, written by
tests/golden/make_golden.py): right-hand side, swimmer KTMinvK_inv, operator,
preconditioner, and three warm-started solves with their GMRES counts."""
from __future__ import annotations

import os

import numpy as np
import pytest

from prescribed import PrescribedSystem, spline

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CONFIGS = ("p1", "p2", "p3", "p4", "p5", "p6")


def load(cfg):
    return dict(np.load(os.path.join(GOLD, f"prescribed_{cfg}.npz")))


def rel(a, b):
    return float(np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300))


def system(d, nt):
    return PrescribedSystem(int(d["flags"]), int(d["nfil"]), int(d["nseg"]), d["x_segs"][nt],
                            d["blob_refs"], d["body_x"], d["body_q"], d["vel_dir_phase"][nt],
                            d["vel_dir_angle"][nt])


def rhs(S, d, nt):
    return S.rhs(d["phase"][nt], d["omega0"], d["angle"][nt], d["omega0"], d["phase_refs"],
                 d["angle_refs"], fil_length=float(d["seg_sep"]) * (int(d["nseg"]) - 1),
                 gen_force_magnitude_factor=float(d["gen_force_magnitude_factor"]),
                 torsional_spring_magnitude_factor=float(d["torsional_spring_magnitude_factor"]))


@pytest.mark.parametrize("cfg", CONFIGS)
def test_pieces_match_reference(cfg):
    d = load(cfg)
    S = system(d, 0)
    assert S.n == int(d["n"])
    assert rel(rhs(S, d, 0), d["rhs0"]) < 1e-14
    assert rel(S.apply_a(d["v_in"]), d["a_v"]) < 1e-13
    assert rel(S.apply_pinv(d["v_in"]), d["pinv_v"]) < 1e-13
    if S.free:
        assert rel(S.m6inv.ravel(order="F"), d["ktminvk"]) < 1e-13


@pytest.mark.parametrize("cfg", CONFIGS)
def test_warm_started_solves_match_reference(cfg):
    d = load(cfg)
    S = system(d, 0)
    x = np.zeros(S.n)
    if S.phase:
        x[S.o_phase:S.o_phase + S.nfil] = d["phase_dot0"]
    if S.angle:
        x[S.o_angle:S.o_angle + S.nfil] = d["angle_dot0"]
    for nt in range(d["phase"].shape[0]):
        S = system(d, nt)
        x, iters = S.solve(rhs(S, d, nt), x)
        assert iters == int(d["iters"][nt])
        fs, fb, U, pd, ad = S.split(x)
        assert rel(fs, d["f_segs"][nt]) < 1e-12
        assert rel(fb, d["f_blobs"][nt]) < 1e-12
        if S.free:
            assert rel(U, d["v_body"][nt]) < 1e-12
        if S.phase:
            assert rel(pd, d["phase_dot"][nt]) < 1e-12
        if S.angle:
            assert rel(ad, d["angle_dot"][nt]) < 1e-12


def test_solution_solves_the_system():
    """The GMRES solution against a dense direct solve of A x = b (the
    operator assembled column by column): a property independent of the
    reference's iteration."""
    d = load("p1")
    S = system(d, 0)
    b = rhs(S, d, 0)
    A = np.stack([S.apply_a(e) for e in np.eye(S.n)], axis=1)
    x_direct = np.linalg.solve(A, b)
    x, _ = S.solve(b, np.zeros(S.n))
    # the stopping test bounds the residual; the error is at most cond(A)
    # (~3e4 here) times that
    assert np.linalg.norm(A @ x - b) <= 2e-10 * np.linalg.norm(b)
    assert rel(x, x_direct) < 1e-5


def test_spline_interpolates_the_table():
    """At the table's nodes the cyclic Hermite spline returns the entries."""
    t = np.linspace(0.0, 1.0, 17)[:-1]
    table = np.cos(2 * np.pi * t) + 0.3
    for k in range(16):
        assert spline(2 * np.pi * k / 16, table) == pytest.approx(table[k], abs=1e-14)
