"""GB300 (sm_103a) implementation of TimFilSim's RPY mobility path.

The compute lives in libtfs_gb300.so (hand-written CUDA behind the C ABI of
include/tfs_gb300.h); this package holds the host-side mirror of the
reference's mobility-solver interface and seeded synthetic geometries.
"""
from . import geometry  # noqa: F401

__all__ = ["geometry", "RpyMobilitySolver", "measure_fma_peak", "kernel_launch_count"]


def __getattr__(name):
    # the solver needs the native library; import it lazily so geometry
    # works on machines without CUDA
    if name in ("RpyMobilitySolver", "measure_fma_peak", "kernel_launch_count"):
        from . import mobility
        return getattr(mobility, name)
    raise AttributeError(name)
