"""The reference's own GPU kernels on this GPU (test infrastructure).

`make -C oracle ref REF=<reference checkout>` compiles the reference's
src/cilia/cuda_functions.cu, unchanged, for sm_103a as device code only
(_ref/ref_kernels_fp64.cubin with Real = double, _ref/ref_kernels_fp32.cubin
with the shipped Real = float; RPY mobility, elastic filaments, free body;
and _ref/ref_kernels_pres_fp{64,32}.cubin in the prescribed-cilia
configuration p1, whose kernels take forces only and pair particles with
rpy_interaction<3,3>).
This module loads such a cubin through the CUDA driver API (ctypes on
libcuda; no host code of the reference runs) in the current context, sets
the kernels' sizes with the reference's own sync_var kernel
(cuda_functions.hpp:36) and launches Mss_mult, Msb_mult, Mbb_mult and
Mbs_mult exactly as the reference's rpy_mobility_solver does
(rpy_mobility_solver.cu:258-328): one launch per block, THREADS_PER_BLOCK = 64
threads per CTA, ceil(N / 64) CTAs, targets from 0 to N-1 on one GPU.

Device arrays are torch tensors of the kernel's Real type; launches go to
the current torch stream. Used by the reference-kernel parity test and by
the benchmark's reference arm, never by the product.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
THREADS_PER_BLOCK = 64  # config.hpp:294

# entry points of the cubins (names as ptxas reports them for these signatures,
# cuda_functions.hpp:9-13,36)
_NAMES = {
    "fp64": {"sync_var": "_Z8sync_variiiiid", "Mss": "_Z8Mss_multPdPKdS1_ii",
             "Msb": "_Z8Msb_multPdPKdS1_S1_ii", "Mbb": "_Z8Mbb_multPdPKdS1_ii",
             "Mbs": "_Z8Mbs_multPdPKdS1_S1_ii"},
    "fp32": {"sync_var": "_Z8sync_variiiiif", "Mss": "_Z8Mss_multPfPKfS1_ii",
             "Msb": "_Z8Msb_multPfPKfS1_S1_ii", "Mbb": "_Z8Mbb_multPfPKfS1_ii",
             "Mbs": "_Z8Mbs_multPfPKfS1_S1_ii"},
}


def cubin_path(precision: str, model: str = "elastic") -> str:
    tag = "pres_" if model == "prescribed" else ""
    return os.path.join(REF_DIR, f"ref_kernels_{tag}{precision}.cubin")


def available(precision: str = "fp64", model: str = "elastic") -> bool:
    return os.path.exists(cubin_path(precision, model))


class RefGpuKernels:
    """The reference's four RPY kernels of one precision ("fp64" or "fp32")
    in the elastic-filament or the prescribed-cilia build."""

    def __init__(self, precision: str = "fp64", model: str = "elastic"):
        import torch

        self.precision = precision
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        torch.zeros(1, device="cuda")  # the primary context exists and is current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._chk(self.cu.cuInit(0), "cuInit")
        self.mod = ctypes.c_void_p()
        self._chk(self.cu.cuModuleLoad(ctypes.byref(self.mod),
                                       cubin_path(precision, model).encode()), "cuModuleLoad")
        self.fn = {}
        for key, name in _NAMES[precision].items():
            f = ctypes.c_void_p()
            self._chk(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()),
                      f"cuModuleGetFunction({name})")
            self.fn[key] = f

    @staticmethod
    def _chk(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUDA driver error {rc}")

    def _launch(self, key, grid, block, args):
        import torch

        holders = []
        for a in args:
            if isinstance(a, torch.Tensor):
                holders.append(ctypes.c_void_p(a.data_ptr()))
            elif isinstance(a, float):
                holders.append(ctypes.c_double(a) if self.precision == "fp64" else ctypes.c_float(a))
            else:
                holders.append(ctypes.c_int(int(a)))
        params = (ctypes.c_void_p * len(holders))(
            *[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._chk(self.cu.cuLaunchKernel(self.fn[key], grid, 1, 1, block, 1, 1, 0, stream, params,
                                         None), f"cuLaunchKernel({key})")

    def sync(self, nswim, nseg, nfil, nblob, end_force_magnitude=0, seg_sep=2.2):
        """sync_var<<<1, 1>>> (cuda_functions.hpp:36): the sizes the kernels
        read. The kernels loop over these counts of sources: every array a
        later launch gets must hold them (checked there)."""
        self.ns, self.nb = int(nswim) * int(nfil) * int(nseg), int(nswim) * int(nblob)
        self._launch("sync_var", 1, 1, [nswim, nseg, nfil, nblob, end_force_magnitude,
                                         float(seg_sep)])

    def _check(self, **arrays):
        want = {"v_segs": 6 * self.ns, "f_segs": 6 * self.ns, "x_segs": 3 * self.ns,
                "v_blobs": 3 * self.nb, "f_blobs": 3 * self.nb, "x_blobs": 3 * self.nb}
        for k, a in arrays.items():
            if a.dtype != self.dtype or not a.is_cuda or not a.is_contiguous() or a.numel() != want[k]:
                raise ValueError(f"{k}: need a contiguous CUDA {self.dtype} array of {want[k]}")

    def _grid(self, n):
        return (n + THREADS_PER_BLOCK - 1) // THREADS_PER_BLOCK

    def mss(self, v_segs, f_segs, x_segs):
        """v_segs = M_ss f_segs (rpy_mobility_solver.cu:258-274)."""
        self._check(v_segs=v_segs, f_segs=f_segs, x_segs=x_segs)
        self._launch("Mss", self._grid(self.ns), THREADS_PER_BLOCK,
                     [v_segs, f_segs, x_segs, 0, self.ns])

    def msb(self, v_segs, f_blobs, x_segs, x_blobs):
        """v_segs += M_sb f_blobs (:276-292)."""
        self._check(v_segs=v_segs, f_blobs=f_blobs, x_segs=x_segs, x_blobs=x_blobs)
        self._launch("Msb", self._grid(self.ns), THREADS_PER_BLOCK,
                     [v_segs, f_blobs, x_segs, x_blobs, 0, self.ns])

    def mbb(self, v_blobs, f_blobs, x_blobs):
        """v_blobs = M_bb f_blobs (:294-310)."""
        self._check(v_blobs=v_blobs, f_blobs=f_blobs, x_blobs=x_blobs)
        self._launch("Mbb", self._grid(self.nb), THREADS_PER_BLOCK,
                     [v_blobs, f_blobs, x_blobs, 0, self.nb])

    def mbs(self, v_blobs, f_segs, x_blobs, x_segs):
        """v_blobs = M_bs f_segs (:312-328)."""
        self._check(v_blobs=v_blobs, f_segs=f_segs, x_blobs=x_blobs, x_segs=x_segs)
        self._launch("Mbs", self._grid(self.nb), THREADS_PER_BLOCK,
                     [v_blobs, f_segs, x_blobs, x_segs, 0, self.nb])

    def close(self):
        if getattr(self, "mod", None) is not None and self.mod.value:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None
