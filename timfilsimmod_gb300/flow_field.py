"""Python mirror of the reference's `flow_field_evaluator`
(src/flow_field/flow_field_evaluator.{hpp,cu}) over the C ABI.

The reference reads saved swimmer states from files, rebuilds segment and
blob positions, and evaluates the fluid velocity at NFLOW points with the
flow_velocities kernel (flow_field_evaluator.cu:13-228). This class keeps the
evaluation part: the caller supplies positions and forces as arrays (the
`x_flow_host`, `x_segs_host`, ... arrays of the reference, AoS float64) and
`velocities()` fills `v_flow_host`. Everything computes on the GPU through
libtfs_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .mobility import PRECISIONS, _DeviceArray, _host_array, _ptr


class FlowFieldEvaluator:
    """Flow-field evaluator on one GB300.

    nbod, nfil, nseg, nblob, nflow: NBOD, NFIL, NSEG, NBLOB, NFLOW of the
    reference; nblob == 0 selects the wall-bounded (Blakelet) form, as there.
    mu: MU. remove_net_force: REMOVE_NET_FORCE_STOKESLET.
    precision: "fp64" (the reference's arithmetic) or "fp32c".
    """

    def __init__(self, nbod: int, nfil: int, nseg: int, nblob: int, nflow: int,
                 mu: float = 1.0, remove_net_force: bool = False, precision: str = "fp64",
                 pinned: bool = True):
        self.lib = N.load()
        self.NBOD, self.NFIL, self.NSEG, self.NBLOB, self.NFLOW = nbod, nfil, nseg, nblob, nflow
        self.MU = mu
        self.REMOVE_NET_FORCE_STOKESLET = bool(remove_net_force)
        self.precision = precision
        h = ctypes.c_void_p()
        N.check(self.lib.tfs_flow_create(nflow, nbod, nfil * nseg, nblob, PRECISIONS[precision],
                                         ctypes.byref(h)))
        self._h = h
        ns, nb = nbod * nfil * nseg, nbod * nblob
        self._host_tensors: list = []
        keep = self._host_tensors
        self.x_flow_host = _host_array(3 * nflow, pinned, keep)
        self.v_flow_host = _host_array(3 * nflow, pinned, keep)
        self.x_segs_host = _host_array(3 * ns, pinned, keep)
        self.f_segs_host = _host_array(6 * ns, pinned, keep)
        self.x_blobs_host = _host_array(3 * nb, pinned, keep)
        self.f_blobs_host = _host_array(3 * nb, pinned, keep)
        self.x_bods_host = _host_array(3 * nbod, pinned, keep)

    def close(self) -> None:
        if self._h is not None:
            self.lib.tfs_flow_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name: str, *args) -> None:
        if self._h is None:
            raise N.TfsError(N.TFS_ESTATE, "flow evaluator has been closed")
        N.check(getattr(self.lib, name)(self._h, *args))

    def set_stream(self, stream: int | None) -> None:
        self._call("tfs_flow_set_stream", ctypes.c_void_p(stream or 0))

    def read_positions_and_forces(self, x_flow=None, x_segs=None, f_segs=None, x_blobs=None,
                                  f_blobs=None, x_bods=None) -> None:
        """Store the given arrays (those not None) into the host arrays, then
        copy all host arrays to the device (flow_field_evaluator.cu:401-544
        without the file parsing)."""
        for name, val in (("x_flow", x_flow), ("x_segs", x_segs), ("f_segs", f_segs),
                          ("x_blobs", x_blobs), ("f_blobs", f_blobs), ("x_bods", x_bods)):
            if val is not None:
                getattr(self, name + "_host")[:] = np.asarray(val, dtype=np.float64).ravel()
        nb = self.NBOD * self.NBLOB
        self._call("tfs_flow_copy_inputs_to_device", _ptr(self.x_flow_host),
                   _ptr(self.x_segs_host), _ptr(self.f_segs_host),
                   _ptr(self.x_blobs_host) if nb else None,
                   _ptr(self.f_blobs_host) if nb else None, _ptr(self.x_bods_host))

    def velocities(self, copy_to_host: bool = True) -> np.ndarray | None:
        """v_flow = 1/(8 pi MU) (...) at every flow point
        (flow_field_evaluator.cu:546-579); returns v_flow_host reshaped (NFLOW, 3)."""
        self._call("tfs_flow_velocities", float(self.MU), int(self.REMOVE_NET_FORCE_STOKESLET))
        if not copy_to_host:
            return None
        self._call("tfs_flow_copy_velocities_to_host", _ptr(self.v_flow_host))
        return self.v_flow_host.reshape(self.NFLOW, 3)

    def autotune(self, reps: int = 1) -> tuple[int, float]:
        """Time every launch variant on the current device inputs and keep the
        fastest; returns (variant, ms per evaluation)."""
        best, ms = ctypes.c_int(), ctypes.c_double()
        self._call("tfs_flow_autotune", float(self.MU), int(self.REMOVE_NET_FORCE_STOKESLET),
                   int(reps), ctypes.byref(best), ctypes.byref(ms))
        return best.value, ms.value

    def set_variant(self, variant: int) -> None:
        self._call("tfs_flow_set_variant", int(variant))

    def num_variants(self) -> int:
        return int(self.lib.tfs_flow_num_variants(PRECISIONS[self.precision]))

    def wait(self) -> None:
        self._call("tfs_flow_wait")

    def device_arrays(self) -> dict:
        """x_flow and v_flow device buffers as __cuda_array_interface__ views."""
        xf, vf = ctypes.c_void_p(), ctypes.c_void_p()
        self._call("tfs_flow_device_buffers", ctypes.byref(xf), ctypes.byref(vf))
        n = 3 * self.NFLOW
        return {"x_flow": _DeviceArray(xf.value or 0, n, self),
                "v_flow": _DeviceArray(vf.value or 0, n, self)}
