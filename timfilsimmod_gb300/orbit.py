"""Newton-Krylov search for periodic states of an elastic-filament swimmer,
as a client of the request server.

The reference searches for periodic orbits with a Jacobian-free
Newton-Krylov method (pyfile/find_periodic/newton_solver.py): the residual
is F(x) = Phi_T(x) - x, the state after one period minus the start
(`getrhs`, :100-137); the Jacobian acts on a Krylov vector through a finite
difference F(x + eps dx) - F(x) with eps = epsJ |x| / |dx| (`multJ`,
:158-183); every evaluation of Phi_T is one run of the simulation binary
(`run_filament_code`, :48-73). There the state is the prescribed cilia's
phases; this client works on the elastic-filament path, where the state is
the filaments' shape:

* x is the rotation vector of every segment relative to the straight start
  (3 per segment), in the body frame -- the perturbation a server request
  takes (`seg_rotation`, applied as exp(x_j) q0_j);
* Phi_N(x) is N implicit steps of the swimmer from that start (one server
  request; T = N DT, fixed, as the reference's fixT mode), mapped back to
  rotation vectors from the final segment orientations:
  log(q_body^-1 q_j q0_j^-1);
* J dx = (F(x + eps dx) - F(x)) / eps, eps = eps_j max(|x|, 1) / |dx| (the
  reference's scaling, with |x| floored at 1 so that a search can start
  from the straight state);
* each Newton iteration solves J s = F(x) by GMRES(m) (Arnoldi with two
  passes of modified Gram-Schmidt, fixed m, least squares on the Hessenberg
  matrix) and steps x <- x - s, halving s while |F| grows (at most 3 times;
  the reference's hookstep trust region is not restated).

Every evaluation of Phi is a server request, so several searches (a sweep
of starts or parameters) running in threads share one server, and their
requests overlap on the GPU. Each request's result does not depend on the
others in flight (the server's guarantee), so every search's iterates and
Krylov vectors are the same, bit for bit, alone and in a mix.
"""
from __future__ import annotations

import threading

import numpy as np


def _qmul(p, q):
    """Quaternion products of rows (scalar first)."""
    ps, pv = p[:, :1], p[:, 1:]
    qs, qv = q[:, :1], q[:, 1:]
    s = ps * qs - np.sum(pv * qv, axis=1, keepdims=True)
    v = ps * qv + qs * pv + np.cross(pv, qv)
    return np.concatenate([s, v], axis=1)


def _qconj(q):
    return q * np.array([1.0, -1.0, -1.0, -1.0])


def _qlog(q):
    """Rotation vectors u with exp(u) = q (the inverse of the stepper's
    lie_exp: q = (cos |u|/2, sin |u|/2 u/|u|)), principal branch."""
    q = np.where(q[:, :1] < 0.0, -q, q)
    s = np.clip(q[:, 0], -1.0, 1.0)
    vn = np.linalg.norm(q[:, 1:], axis=1)
    th = 2.0 * np.arctan2(vn, s)
    scale = np.where(vn > 1e-300, th / np.maximum(vn, 1e-300), 2.0)
    return q[:, 1:] * scale[:, None]


class OrbitSearch:
    """Newton-Krylov search on one swimmer geometry through a StepServer.

    server: a timfilsimmod_gb300.serving.StepServer; (blob_refs, fil_refs,
    fil_dirs, body_radius): the geometry of every request; nseg: segments per
    filament; num_steps: the steps of one period; eps_j: the finite
    difference's relative size."""

    def __init__(self, server, blob_refs, fil_refs, fil_dirs, nseg: int, num_steps: int,
                 body_radius: float = 0.0, eps_j: float = 1e-2):
        self.sv = server
        self.geo = (np.asarray(blob_refs, dtype=np.float64), np.asarray(fil_refs, dtype=np.float64),
                    np.asarray(fil_dirs, dtype=np.float64))
        self.nseg, self.num_steps = int(nseg), int(num_steps)
        self.radius, self.eps_j = float(body_radius), float(eps_j)
        self.requests = 0
        self.latencies_ms: list[float] = []  # arrival to completion of each request
        self._lock = threading.Lock()
        # the straight start's orientations: a request of no steps
        r = self._run([None], steps=0)[0]
        self.q0 = r["q"].reshape(-1, 4).copy()
        self.n = 3 * self.q0.shape[0]

    def _run(self, rotations, steps):
        tickets = [self.sv.submit(*self.geo, self.nseg, num_steps=steps, seg_rotation=r,
                                  body_radius=self.radius) for r in rotations]
        out = [self.sv.poll(t, wait=True) for t in tickets]
        with self._lock:
            self.requests += len(tickets)
            self.latencies_ms += [r.get("latency_ms", 0.0) for r in out]
        return out

    def phi(self, thetas):
        """Phi_N of each state (submitted together, so they run at once)."""
        out = []
        for r in self._run([np.asarray(t, dtype=np.float64) for t in thetas], self.num_steps):
            q = r["q"].reshape(-1, 4)
            qb = np.tile(r["body"][3:7], (q.shape[0], 1))
            rel = _qmul(_qmul(_qconj(qb), q), _qconj(self.q0))
            out.append(_qlog(rel).ravel())
        return out

    def residual(self, theta):
        """F(x) = Phi_N(x) - x (the reference's getrhs)."""
        return self.phi([theta])[0] - np.asarray(theta, dtype=np.float64)

    def jacobian_times(self, x, fx, dx):
        """J dx by the finite difference of the reference's multJ."""
        nd = np.linalg.norm(dx)
        if nd == 0.0:
            return np.zeros_like(dx)
        eps = self.eps_j * max(np.linalg.norm(x), 1.0) / nd
        return (self.residual(x + eps * dx) - fx) / eps

    def newton(self, x0, m: int = 8, iters: int = 1, tol: float = 0.0):
        """Newton iterations from x0 with GMRES(m) for each step. Returns a
        record: the iterates, |F| of each, the Krylov vectors and Hessenberg
        matrices of every GMRES solve, and the request count."""
        x = np.array(x0, dtype=np.float64)
        fx = self.residual(x)
        rec = {"x": [x.copy()], "residual": [float(np.linalg.norm(fx))], "krylov": [],
               "hessenberg": []}
        for _ in range(iters):
            if rec["residual"][-1] <= tol:
                break
            beta = np.linalg.norm(fx)
            V = np.zeros((m + 1, self.n))
            H = np.zeros((m + 1, m))
            V[0] = fx / beta
            k = m
            for j in range(m):
                w = self.jacobian_times(x, fx, V[j])
                for _pass in range(2):  # modified Gram-Schmidt, twice (orthogonal to rounding)
                    for i in range(j + 1):
                        h = np.dot(V[i], w)
                        H[i, j] += h
                        w = w - h * V[i]
                H[j + 1, j] = np.linalg.norm(w)
                if H[j + 1, j] <= 1e-14 * beta:
                    k = j + 1
                    break
                V[j + 1] = w / H[j + 1, j]
            e1 = np.zeros(k + 1)
            e1[0] = beta
            y = np.linalg.lstsq(H[:k + 1, :k], e1, rcond=None)[0]
            s = V[:k].T @ y
            rec["krylov"].append(V[:k + 1].copy())
            rec["hessenberg"].append(H[:k + 1, :k].copy())
            for _half in range(4):  # backtrack while |F| grows
                xn = x - s
                fn = self.residual(xn)
                if np.linalg.norm(fn) < beta:
                    break
                s = 0.5 * s
            x, fx = xn, fn
            rec["x"].append(x.copy())
            rec["residual"].append(float(np.linalg.norm(fx)))
        rec["requests"] = self.requests
        return rec


def search_many(searches, starts, **newton_kw):
    """Run several searches at once (one thread each, sharing their servers):
    a sweep of starts or parameters. Returns their records in order."""
    out = [None] * len(searches)

    def run(i):
        out[i] = searches[i].newton(starts[i], **newton_kw)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(searches))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    return out
