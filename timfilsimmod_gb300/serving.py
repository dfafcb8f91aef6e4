"""Many independent swimmers on one GPU (tfs_batch_*, tfs_server_* of the C ABI).

SwimmerBatch advances a set of swimmers (ImplicitStepper instances, each
with its own solver and stream) one implicit step at a time: host worker
threads run the instances' step pipelines so that their kernels overlap on
the GPU, and the inner solves of FP32C swimmers share cooperative launches. StepServer takes requests -- num_steps implicit steps of a swimmer
from a perturbed straight start -- keeps instances resident between
requests, admits requests by a device-memory budget and reports each
request's latency. There is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .mobility import PRECISIONS
from .stepper import ImplicitStepper


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))


class SwimmerBatch:
    def __init__(self, num_workers: int = 8):
        self.lib = N.load()
        h = ctypes.c_void_p()
        N.check(self.lib.tfs_batch_create(int(num_workers), ctypes.byref(h)))
        self._h = h
        self.steppers: list[ImplicitStepper] = []

    def add(self, stepper: ImplicitStepper) -> int:
        idx = ctypes.c_int(0)
        N.check(self.lib.tfs_batch_add(self._h, stepper._h, ctypes.byref(idx)))
        self.steppers.append(stepper)
        return idx.value

    def step(self, nt: int, allow_unconverged: bool = False) -> dict:
        """Step nt of every swimmer; per-swimmer Broyden/GMRES counts and statuses."""
        n = len(self.steppers)
        b, g, st = (np.zeros(n, dtype=np.int32) for _ in range(3))
        rc = self.lib.tfs_batch_step(self._h, int(nt), b.ctypes.data, g.ctypes.data,
                                     st.ctypes.data)
        if rc != N.TFS_OK and not (allow_unconverged and np.all(
                (st == N.TFS_OK) | (st == N.TFS_ENOTCONV))):
            N.check(rc)
        return {"broyden_iters": b, "gmres_iters": g, "status": st}

    def share_inner_solves(self, max_ctas: int | bool = -1) -> None:
        """FP32C swimmers whose inner solve takes at most max_ctas CTAs (one
        per 64 blobs) share cooperative launches; True or -1 (the default):
        all, False / 0: none."""
        if max_ctas is True:
            max_ctas = 1 << 30
        N.check(self.lib.tfs_batch_share_inner_solves(self._h, int(max_ctas)))

    def shared_solves(self) -> dict:
        """Inner solves run in shared cooperative launches, and the launches."""
        la, so = ctypes.c_longlong(0), ctypes.c_longlong(0)
        N.check(self.lib.tfs_batch_shared_solves(self._h, ctypes.byref(la), ctypes.byref(so)))
        return {"launches": la.value, "solves": so.value}

    def share_products(self, enable: bool = True) -> None:
        """Whether the swimmers' pair products share work-queue launches
        (default on)."""
        N.check(self.lib.tfs_batch_share_products(self._h, int(bool(enable))))

    def shared_products(self) -> dict:
        """Products run in shared work-queue launches, and the launches."""
        la, pr = ctypes.c_longlong(0), ctypes.c_longlong(0)
        N.check(self.lib.tfs_batch_shared_products(self._h, ctypes.byref(la), ctypes.byref(pr)))
        return {"launches": la.value, "products": pr.value}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self.lib.tfs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StepServer:
    """Request server. precision "fp64" or "fp32c"; step settings as keyword
    arguments of tfs_step_config (dt, tol, seg_sep, end_force_magnitude,
    body_radius, max_broyden_iter, ...)."""

    def __init__(self, num_workers: int = 16, hbm_budget_gb: float = 160.0,
                 precision: str = "fp32c", linear_tol: float = 1e-8,
                 max_bypass_ms: float | None = None, **step):
        self.lib = N.load()
        cfg = N.ServerConfig()
        N.check(self.lib.tfs_server_config_default(ctypes.byref(cfg)))
        cfg.num_workers = int(num_workers)
        cfg.hbm_budget_bytes = int(hbm_budget_gb * (1 << 30))
        cfg.precision = PRECISIONS[precision]
        cfg.linear_tol = float(linear_tol)
        if max_bypass_ms is not None:
            cfg.max_bypass_ms = float(max_bypass_ms)
        for k, v in step.items():
            if k in ("body_x", "body_q"):
                arr = getattr(cfg.step, k)
                for i, x in enumerate(v):
                    arr[i] = float(x)
            elif not hasattr(cfg.step, k):
                raise TypeError(f"unknown step setting {k!r}")
            else:
                setattr(cfg.step, k, type(getattr(cfg.step, k))(v))
        h = ctypes.c_void_p()
        N.check(self.lib.tfs_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._live: dict[int, tuple] = {}  # ticket -> arrays the request points into

    def submit(self, blob_refs, fil_refs, fil_dirs, nseg: int, num_steps: int = 1,
               seg_rotation=None, body_radius: float = 0.0) -> int:
        br, fr, fd = _f64(blob_refs), _f64(fil_refs), _f64(fil_dirs)
        nfil, nblob = fr.size // 3, br.size // 3
        rot = None if seg_rotation is None else _f64(seg_rotation)
        if rot is not None and rot.size != 3 * nfil * nseg:
            raise ValueError("seg_rotation needs 3 values per segment")
        x = np.zeros(3 * nfil * nseg)
        q = np.zeros(4 * nfil * nseg)
        body = np.zeros(7)
        r = N.Request(nfil=nfil, nseg=int(nseg), nblob=nblob, blob_refs=br.ctypes.data,
                      fil_refs=fr.ctypes.data, fil_dirs=fd.ctypes.data,
                      body_radius=float(body_radius),
                      seg_rotation=None if rot is None else rot.ctypes.data,
                      num_steps=int(num_steps), x_out=x.ctypes.data, body_out=body.ctypes.data,
                      q_out=q.ctypes.data)
        t = ctypes.c_longlong(0)
        N.check(self.lib.tfs_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        self._live[t.value] = (br, fr, fd, rot, x, body, q)
        return t.value

    def request_bytes(self, blob_refs, fil_refs, fil_dirs, nseg: int) -> int:
        """Device bytes the server accounts for a request of this geometry."""
        br, fr, fd = _f64(blob_refs), _f64(fil_refs), _f64(fil_dirs)
        r = N.Request(nfil=fr.size // 3, nseg=int(nseg), nblob=br.size // 3,
                      blob_refs=br.ctypes.data, fil_refs=fr.ctypes.data, fil_dirs=fd.ctypes.data)
        b = ctypes.c_size_t(0)
        N.check(self.lib.tfs_server_request_bytes(self._h, ctypes.byref(r), ctypes.byref(b)))
        return b.value

    def poll(self, ticket: int, wait: bool = False) -> dict | None:
        """None while pending; else the result (x, body, q, latency_ms, counts).
        A failed request raises."""
        st, lat = ctypes.c_int(0), ctypes.c_double(0.0)
        b, g = ctypes.c_int(0), ctypes.c_int(0)
        N.check(self.lib.tfs_server_poll(self._h, ctypes.c_longlong(ticket), int(bool(wait)),
                                         ctypes.byref(st), ctypes.byref(lat), ctypes.byref(b),
                                         ctypes.byref(g)))
        if st.value == 1:
            return None
        arrays = self._live.pop(ticket)
        if st.value != N.TFS_OK:
            raise N.TfsError(st.value, self.lib.tfs_last_error().decode(errors="replace"))
        return {"x": arrays[4], "body": arrays[5], "q": arrays[6], "latency_ms": lat.value,
                "broyden_iters": b.value, "gmres_iters": g.value}

    def drain(self) -> None:
        N.check(self.lib.tfs_server_drain(self._h))

    def stats(self) -> dict:
        c = N.ServerCounters()
        N.check(self.lib.tfs_server_stats(self._h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in c._fields_}

    def shared_solves(self) -> dict:
        la, so = ctypes.c_longlong(0), ctypes.c_longlong(0)
        N.check(self.lib.tfs_server_shared_solves(self._h, ctypes.byref(la), ctypes.byref(so)))
        return {"launches": la.value, "solves": so.value}

    def shared_products(self) -> dict:
        """Products run in shared work-queue launches, and the launches."""
        la, pr = ctypes.c_longlong(0), ctypes.c_longlong(0)
        N.check(self.lib.tfs_server_shared_products(self._h, ctypes.byref(la), ctypes.byref(pr)))
        return {"launches": la.value, "products": pr.value}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self.lib.tfs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
