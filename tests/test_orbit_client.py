"""The orbit-search client (timfilsimmod_gb300.orbit) on the host, with a
stand-in server whose period map is a known affine map in rotation space:
Phi(x) = M x + c. The client must recover x from the orientations it gets
back (its log inverts the stepper's exp), its finite-difference Jacobian is
then exact up to rounding, and one Newton step with GMRES(n) lands on the
fixed point x* = (I - M)^-1 c. A second test runs two searches in threads
on one stand-in server and checks each matches the same search run alone.
"""
import threading

import numpy as np

from timfilsimmod_gb300.orbit import OrbitSearch, _qconj, _qlog, _qmul, search_many


def lie_exp(u):
    """The stepper's exp (step_math.cuh): (cos |u|/2, sin |u|/2 u/|u|)."""
    th = np.linalg.norm(u, axis=1)
    out = np.zeros((u.shape[0], 4))
    out[:, 0] = np.cos(0.5 * th)
    sc = np.where(th > 0, np.sin(0.5 * th) / np.where(th > 0, th, 1.0), 0.5)
    out[:, 1:] = u * sc[:, None]
    return out


class AffineServer:
    """Answers a request of N steps with orientations exp(M x + c) q0 and a
    body turned by qb (which the client must take out)."""

    def __init__(self, nseg_total, seed=0):
        rng = np.random.default_rng(seed)
        n = 3 * nseg_total
        self.M = 0.3 * rng.normal(size=(n, n)) / np.sqrt(n)
        self.c = 0.05 * rng.normal(size=n)
        self.q0 = lie_exp(rng.normal(size=(nseg_total, 3)))
        self.qb = lie_exp(np.array([[0.1, -0.2, 0.05]]))[0]
        self._out, self._next = {}, 0
        self._lock = threading.Lock()

    def submit(self, blob_refs, fil_refs, fil_dirs, nseg, num_steps=1, seg_rotation=None,
               body_radius=0.0):
        x = np.zeros(self.M.shape[0]) if seg_rotation is None else np.asarray(seg_rotation)
        if num_steps == 0:
            q = _qmul(lie_exp(x.reshape(-1, 3)), self.q0)
            body = np.array([0, 0, 0, 1.0, 0, 0, 0])
        else:
            y = self.M @ x + self.c
            qb = np.tile(self.qb, (self.q0.shape[0], 1))
            q = _qmul(qb, _qmul(lie_exp(y.reshape(-1, 3)), self.q0))
            body = np.concatenate([np.zeros(3), self.qb])
        with self._lock:
            t = self._next
            self._next += 1
            self._out[t] = {"q": q.ravel(), "body": body}
        return t

    def poll(self, ticket, wait=False):
        with self._lock:
            return self._out.pop(ticket)


GEO = (np.zeros((4, 3)), np.zeros((2, 3)), np.tile([0.0, 0.0, 1.0], (2, 1)))


def test_log_inverts_exp():
    u = np.random.default_rng(1).normal(size=(50, 3))
    u *= 2.5 / np.max(np.linalg.norm(u, axis=1))  # below pi
    assert np.allclose(_qlog(lie_exp(u)), u, atol=1e-13)
    q = lie_exp(u)
    assert np.allclose(_qmul(q, _qconj(q)), [[1, 0, 0, 0]] * 50, atol=1e-15)


def test_one_newton_step_finds_the_fixed_point_of_an_affine_map():
    sv = AffineServer(nseg_total=10)
    o = OrbitSearch(sv, *GEO, nseg=5, num_steps=3, eps_j=1e-3)
    assert np.allclose(o.q0, sv.q0)
    x0 = np.zeros(o.n)
    rec = o.newton(x0, m=o.n, iters=1)
    xstar = np.linalg.solve(np.eye(o.n) - sv.M, sv.c)
    assert rec["residual"][1] < 1e-8 * rec["residual"][0]
    assert np.allclose(rec["x"][1], xstar, atol=1e-8)
    # the Krylov basis is orthonormal (its first n vectors: a full-dimension
    # space leaves only rounding for the (n+1)-th)
    V = rec["krylov"][0][:o.n]
    assert np.allclose(V @ V.T, np.eye(V.shape[0]), atol=1e-10)


def test_searches_in_threads_match_each_alone():
    starts = [0.02 * np.random.default_rng(s).normal(size=30) for s in (3, 4, 5)]
    alone = []
    for x0 in starts:
        o = OrbitSearch(AffineServer(nseg_total=10), *GEO, nseg=5, num_steps=2)
        alone.append(o.newton(x0, m=6, iters=2))
    sv = AffineServer(nseg_total=10)
    mix = search_many([OrbitSearch(sv, *GEO, nseg=5, num_steps=2) for _ in starts], starts,
                      m=6, iters=2)
    for a, b in zip(alone, mix):
        for va, vb in zip(a["krylov"], b["krylov"]):
            assert np.array_equal(va, vb)
        for xa, xb in zip(a["x"], b["x"]):
            assert np.array_equal(xa, xb)
