"""CPU restatement of the reference's prescribed-cilia mobility solve (test
infrastructure only: tests/ use it as the checker of the CUDA path; the
product package never imports it).

The reference, under PRESCRIBED_CILIA (src/cilia/mobility/mobility_solver.cpp):

* unknowns x = [segment forces (3 Ns); blob forces (3 Nb); body U, Omega (6,
  free body only); phase rates (nfil, dynamic phase); shape-rotation rates
  (nfil, dynamic shape rotation)];
* right-hand side assemble_rhs (:282-437), generalised forces by the cyclic
  cubic Hermite interpolation (:240-279);
* operator system_matrix_mult_new (:1806-2026): the translational 3x3 RPY
  mobility of all particles (Mss_mult, Msb_mult, Mbb_mult, Mbs_mult under
  PRESCRIBED_CILIA, cuda_functions.cu:362-757; Msf_mult :1129-1229 for the
  weakly coupled filaments' segment block) minus the rigid-body and
  phase/angle couplings and their transposes;
* right preconditioner apply_preconditioner_new (:1040-1436), with
  swimmer::make_precon_mat (swimmer.cpp:1154-1322);
* right-preconditioned GMRES with modified Gram-Schmidt, warm started from
  the previous solution (:2092-2570).

One swimmer. Pinned against the reference's own solver compiled for the CPU
(tests/golden/prescribed_p*.npz, written by tests/golden/make_golden.py from
oracle/_ref/libref_pres_*.so).
"""
from __future__ import annotations

import numpy as np

from oracle import Oracle

PRESCRIBED_BODY = 1
DYNAMIC_PHASE = 2
DYNAMIC_ANGLE = 4
WEAKLY_COUPLED = 8


def rcross(v) -> np.ndarray:
    """matrix.cpp:665-679: M w = w x v."""
    return np.array([[0.0, v[2], -v[1]], [-v[2], 0.0, v[0]], [v[1], -v[0], 0.0]])


def spline(phase: float, table: np.ndarray) -> float:
    """cyclic_cubic_spline_interpolation (mobility_solver.cpp:240-279)."""
    n = len(table)
    p = 0.5 * phase / np.pi
    p -= np.floor(p)
    p *= n
    lo = int(p)
    if lo == n:
        return float(table[0])
    hi = 0 if lo == n - 1 else lo + 1
    ql, qu = table[lo], table[hi]
    dql = (table[1] - table[0]) if lo == 0 else 0.5 * (table[hi] - table[lo - 1])
    dqu = (table[0] - table[n - 1]) if hi == 0 else 0.5 * (table[0 if hi == n - 1 else hi + 1] - table[lo])
    t = p - lo
    t2, t3 = t * t, t * t * t
    return float(ql * (2 * t3 - 3 * t2 + 1) + dql * (t3 - 2 * t2 + t) + qu * (3 * t2 - 2 * t3)
                 + dqu * (t3 - t2))


class PrescribedSystem:
    """One swimmer's prescribed-cilia system at fixed kinematics."""

    def __init__(self, flags, nfil, nseg, x_segs, blob_refs, body_x, body_q, vel_dir_phase,
                 vel_dir_angle=None, mu=1.0, a_seg=1.0, a_blob=1.0):
        from timfilsimmod_gb300.geometry import quat_rot
        self.flags, self.nfil, self.nseg = int(flags), int(nfil), int(nseg)
        self.ns = nfil * nseg
        self.x_segs = np.asarray(x_segs, dtype=np.float64).reshape(-1, 3)
        self.R = quat_rot(body_q)
        self.body_x = np.asarray(body_x, dtype=np.float64)
        self.d_blobs = np.asarray(blob_refs, dtype=np.float64).reshape(-1, 3) @ self.R.T
        self.x_blobs = self.body_x + self.d_blobs
        self.nb = self.d_blobs.shape[0]
        self.d_segs = self.x_segs - self.body_x
        self.kphi = np.asarray(vel_dir_phase, dtype=np.float64).reshape(nfil, nseg, 3)
        self.kth = (np.asarray(vel_dir_angle, dtype=np.float64).reshape(nfil, nseg, 3)
                    if vel_dir_angle is not None else np.zeros((nfil, nseg, 3)))
        self.mu, self.a_seg, self.a_blob = mu, a_seg, a_blob
        self.c = 6.0 * np.pi * mu * a_seg
        self.cb = 6.0 * np.pi * mu * a_blob
        self.free = not flags & PRESCRIBED_BODY
        self.phase = bool(flags & DYNAMIC_PHASE)
        self.angle = bool(flags & DYNAMIC_ANGLE)
        if self.free and self.phase != self.angle:
            raise ValueError("free body: dynamic phase and shape rotation go together")
        self.o_body = 3 * (self.ns + self.nb)
        self.o_phase = self.o_body + (6 if self.free else 0)
        self.o_angle = self.o_phase + (nfil if self.phase else 0)
        self.n = self.o_angle + (nfil if self.angle else 0)
        self.orc = Oracle(mu, a_seg, a_blob)
        # per filament: c11, c22, c12, v_phi, v_theta, u_phi, u_theta (swimmer.cpp:1255-1287)
        ds = self.d_segs.reshape(nfil, nseg, 3)
        self.c11 = np.einsum("fki,fki->f", self.kphi, self.kphi)
        self.c22 = np.einsum("fki,fki->f", self.kth, self.kth)
        self.c12 = np.einsum("fki,fki->f", self.kphi, self.kth)
        self.vphi, self.vth = self.kphi.sum(1), self.kth.sum(1)
        self.uphi = np.cross(ds, self.kphi).sum(1)
        self.uth = np.cross(ds, self.kth).sum(1)
        self.m6inv = self._make_precon_mat() if self.free else np.zeros((6, 6))

    def _make_precon_mat(self) -> np.ndarray:
        """swimmer::make_precon_mat (swimmer.cpp:1154-1322), free body."""
        c, cb = self.c, self.cb
        M = np.zeros((6, 6))
        M[:3, :3] = np.eye(3) * (self.ns * c + self.nb * cb)
        for d, f in [(d, c) for d in self.d_segs] + [(d, cb) for d in self.d_blobs]:
            rc = rcross(d)
            M[:3, 3:] += f * rc
            M[3:, 3:] -= f * rc @ rc
        M[3:, :3] = -M[:3, 3:]
        if self.phase:
            C = np.zeros((6, 6))
            for m in range(self.nfil):
                vp, up, vt, ut = self.vphi[m], self.uphi[m], self.vth[m], self.uth[m]
                if self.angle:
                    det = self.c11[m] * self.c22[m] - self.c12[m] ** 2
                    i11, i22, i12 = self.c22[m] / det, self.c11[m] / det, -self.c12[m] / det
                    C[:3, :3] += (np.outer(vp, vp) * i11 + np.outer(vp, vt) * i12
                                  + np.outer(vt, vp) * i12 + np.outer(vt, vt) * i22)
                    C[3:, :3] += (np.outer(up, vp) * i11 + np.outer(up, vt) * i12
                                  + np.outer(ut, vp) * i12 + np.outer(ut, vt) * i22)
                    C[3:, 3:] += (np.outer(up, up) * i11 + np.outer(up, ut) * i12
                                  + np.outer(ut, up) * i12 + np.outer(ut, ut) * i22)
                else:
                    C[:3, :3] += np.outer(vp, vp) / self.c11[m]
                    C[3:, :3] += np.outer(up, vp) / self.c11[m]
                    C[3:, 3:] += np.outer(up, up) / self.c11[m]
            C[:3, 3:] = C[3:, :3].T
            M -= c * C
        return np.linalg.inv(M)

    # -- pieces ---------------------------------------------------------------
    def mobility(self, fs, fb):
        """v = M f over all particles, translational only (the PRESCRIBED_CILIA
        kernels: rpy_interaction<3,3> everywhere; Mbs_mult adds)."""
        o = self.orc
        if self.flags & WEAKLY_COUPLED:
            f6 = np.zeros((self.ns, 6))
            f6[:, :3] = fs.reshape(-1, 3)
            vs = o.msf(self.x_segs, f6, self.nfil, self.nseg).reshape(-1, 6)[:, :3].ravel()
        else:
            vs = o.block(3, 3, self.x_segs, self.a_seg, self.x_segs, fs, self.a_seg)
        vs = o.block(3, 3, self.x_segs, self.a_seg, self.x_blobs, fb, self.a_blob, v=vs)
        vb = o.block(3, 3, self.x_blobs, self.a_blob, self.x_blobs, fb, self.a_blob)
        vb = o.block(3, 3, self.x_blobs, self.a_blob, self.x_segs, fs, self.a_seg, v=vb)
        return vs, vb

    def split(self, x):
        ns3, nb3 = 3 * self.ns, 3 * self.nb
        fs, fb = x[:ns3], x[ns3:ns3 + nb3]
        U = x[self.o_body:self.o_body + 6] if self.free else np.zeros(6)
        pd = x[self.o_phase:self.o_phase + self.nfil] if self.phase else np.zeros(self.nfil)
        ad = x[self.o_angle:self.o_angle + self.nfil] if self.angle else np.zeros(self.nfil)
        return fs, fb, U, pd, ad

    def apply_a(self, x):
        """system_matrix_mult_new (mobility_solver.cpp:1806-2026)."""
        fs, fb, U, pd, ad = self.split(x)
        vs, vb = self.mobility(fs, fb)
        out = np.zeros(self.n)
        os_ = out[:3 * self.ns].reshape(self.nfil, self.nseg, 3)
        ob = out[3 * self.ns:3 * (self.ns + self.nb)].reshape(-1, 3)
        f3 = fs.reshape(self.nfil, self.nseg, 3)
        if self.free:
            for d, o, f in ((self.d_segs, os_.reshape(-1, 3), fs.reshape(-1, 3)),
                            (self.d_blobs, ob, fb.reshape(-1, 3))):
                o -= U[:3] + np.cross(U[3:], d)
                out[self.o_body:self.o_body + 3] -= f.sum(0)
                out[self.o_body + 3:self.o_body + 6] -= np.cross(d, f).sum(0)
        if self.phase:
            os_ -= pd[:, None, None] * self.kphi
            out[self.o_phase:self.o_phase + self.nfil] -= np.einsum("fki,fki->f", f3, self.kphi)
        if self.angle:
            os_ -= ad[:, None, None] * self.kth
            out[self.o_angle:self.o_angle + self.nfil] -= np.einsum("fki,fki->f", f3, self.kth)
        out[:3 * self.ns] += vs
        out[3 * self.ns:3 * (self.ns + self.nb)] += vb
        return out

    def apply_pinv(self, r):
        """apply_preconditioner_new (mobility_solver.cpp:1040-1436)."""
        c, cb = self.c, self.cb
        out = np.array(r, dtype=np.float64)
        ns3, nb3 = 3 * self.ns, 3 * self.nb
        out[:ns3] *= c
        out[ns3:ns3 + nb3] *= cb
        s = out[:ns3].reshape(self.nfil, self.nseg, 3)
        sb = out[ns3:ns3 + nb3].reshape(-1, 3)
        ip, ia = slice(self.o_phase, self.o_phase + self.nfil), slice(self.o_angle, self.o_angle + self.nfil)
        dphi = np.einsum("fki,fki->f", self.kphi, s)
        dth = np.einsum("fki,fki->f", self.kth, s)
        if not self.free:
            if self.phase and self.angle:
                p = -out[ip] - dphi
                a = -out[ia] - dth
                det = self.c11 * self.c22 - self.c12 ** 2
                out[ip] = (p * (self.c22 / det) + a * (-self.c12 / det)) / c
                out[ia] = (p * (-self.c12 / det) + a * (self.c11 / det)) / c
                s += c * out[ip][:, None, None] * self.kphi
                s += c * out[ia][:, None, None] * self.kth
            elif self.phase:
                out[ip] = (-out[ip] - dphi) / (self.c11 * c)
                s += c * out[ip][:, None, None] * self.kphi
            elif self.angle:
                out[ia] = (-out[ia] - dth) / (self.c22 * c)
                s += c * out[ia][:, None, None] * self.kth
            return out
        ib = slice(self.o_body, self.o_body + 6)
        t = -out[ib]
        t[:3] -= s.reshape(-1, 3).sum(0) + sb.sum(0)
        t[3:] -= np.cross(self.d_segs, s.reshape(-1, 3)).sum(0) + np.cross(self.d_blobs, sb).sum(0)
        if self.phase:
            p = -out[ip] - dphi
            a = -out[ia] - dth
            det = self.c11 * self.c22 - self.c12 ** 2
            i11, i22, i12 = self.c22 / det, self.c11 / det, -self.c12 / det
            p, a = i11 * p + i12 * a, i12 * p + i22 * a
            t[:3] -= (p[:, None] * self.vphi).sum(0) + (a[:, None] * self.vth).sum(0)
            t[3:] -= (p[:, None] * self.uphi).sum(0) + (a[:, None] * self.uth).sum(0)
            B = self.m6inv @ t
            p, a = p / c, a / c
            b0 = np.einsum("fi,i->f", self.vphi, B[:3]), np.einsum("fi,i->f", self.vth, B[:3])
            b1 = np.einsum("fi,i->f", self.uphi, B[3:]), np.einsum("fi,i->f", self.uth, B[3:])
            p = p - (i11 * b0[0] + i12 * b0[1] + i11 * b1[0] + i12 * b1[1])
            a = a - (i12 * b0[0] + i22 * b0[1] + i12 * b1[0] + i22 * b1[1])
            out[ip], out[ia] = p, a
        else:
            B = self.m6inv @ t
        out[ib] = B
        s += c * (B[:3] + np.cross(B[3:], self.d_segs.reshape(self.nfil, self.nseg, 3)))
        if self.phase:
            s += c * out[ip][:, None, None] * self.kphi
            s += c * out[ia][:, None, None] * self.kth
        sb += cb * (B[:3] + np.cross(B[3:], self.d_blobs))
        return out

    def rhs(self, phase, omega0, angle=None, phase_dot=None, phase_refs=None, angle_refs=None,
            v_body=None, gen_force_magnitude_factor=1.0, torsional_spring_magnitude_factor=2.0,
            fil_length=None):
        """assemble_rhs (mobility_solver.cpp:282-437); v_body = the prescribed
        body velocities (zero in the reference, rigid_body.cpp:584-598)."""
        b = np.zeros(self.n)
        s = b[:3 * self.ns].reshape(self.nfil, self.nseg, 3)
        if fil_length is None:
            raise ValueError("fil_length = DL (NSEG - 1)")
        for m in range(self.nfil):
            if self.angle:
                qa = spline(phase[m], angle_refs) * 0.5 * omega0[m] / np.pi
                qa -= torsional_spring_magnitude_factor * omega0[m] * fil_length ** 3 * angle[m]
                b[self.o_angle + m] = -qa
            if self.phase:
                qp = spline(phase[m], phase_refs) * 0.5 * omega0[m] / np.pi
                b[self.o_phase + m] = -qp * gen_force_magnitude_factor
            else:
                s[m] = phase_dot[m] * self.kphi[m]
        if not self.free:
            V = np.zeros(6) if v_body is None else np.asarray(v_body, dtype=np.float64)
            b[3 * self.ns:3 * (self.ns + self.nb)] += (V[:3] + np.cross(V[3:], self.d_blobs)).ravel()
            b[:3 * self.ns] += (V[:3] + np.cross(V[3:], self.d_segs)).ravel()
        return b

    def solve(self, b, x0, tol=1e-10, max_iter=350):
        """solve_linear_system (mobility_solver.cpp:2092-2570): right
        preconditioning, modified Gram-Schmidt, the warm start x0 kept if its
        residual is below tol ||b||, dropped if above ||b||. Returns (x, iters)."""
        nb_ = np.linalg.norm(b)
        if nb_ == 0.0:
            return np.zeros(self.n), 0
        x = np.array(x0, dtype=np.float64)
        r = b - self.apply_a(x)
        beta0 = np.linalg.norm(r)
        if abs(beta0) <= tol * nb_:
            return x, 0
        if abs(beta0) > nb_:
            x[:] = 0.0
            beta0, r = nb_, b.copy()
        m = min(self.n, max_iter)
        Q = np.zeros((m + 1, self.n))
        H = np.zeros((m + 1, m + 1))
        cs, sn, beta = np.zeros(m), np.zeros(m), np.zeros(m + 1)
        beta[0] = beta0
        Q[0] = r / beta0
        for it in range(1, m + 1):
            w = self.apply_a(self.apply_pinv(Q[it - 1]))
            for i in range(it):
                H[i, it - 1] = w @ Q[i]
                w = w - H[i, it - 1] * Q[i]
            H[it, it - 1] = np.linalg.norm(w)
            Q[it] = w / H[it, it - 1]
            for i in range(1, it):
                t = cs[i - 1] * H[i - 1, it - 1] + sn[i - 1] * H[i, it - 1]
                H[i, it - 1] = cs[i - 1] * H[i, it - 1] - sn[i - 1] * H[i - 1, it - 1]
                H[i - 1, it - 1] = t
            h1, h0 = H[it, it - 1], H[it - 1, it - 1]
            if h1 == 0.0:
                cs[it - 1], sn[it - 1] = 1.0, 0.0
            elif abs(h1) > abs(h0):
                t = h0 / h1
                sn[it - 1] = (2.0 * (h1 > 0) - 1.0) / np.sqrt(1.0 + t * t)
                cs[it - 1] = t * sn[it - 1]
            else:
                t = h1 / h0
                cs[it - 1] = (2.0 * (h0 > 0) - 1.0) / np.sqrt(1.0 + t * t)
                sn[it - 1] = t * cs[it - 1]
            H[it - 1, it - 1] = cs[it - 1] * h0 + sn[it - 1] * h1
            H[it, it - 1] = 0.0
            beta[it] = -sn[it - 1] * beta[it - 1]
            beta[it - 1] = cs[it - 1] * beta[it - 1]
            if abs(beta[it]) / nb_ <= tol or it == m:
                y = np.zeros(it)
                for i in range(it - 1, -1, -1):
                    y[i] = (beta[i] - H[i, i + 1:it] @ y[i + 1:]) / H[i, i]
                x += self.apply_pinv(Q[:it].T @ y)
                return x, it
        raise AssertionError("unreachable")
