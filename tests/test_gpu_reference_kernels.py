"""The reference's own GPU kernels (its cuda_functions.cu compiled unchanged
for sm_103a as a cubin by `make -C oracle ref`, launched as its
rpy_mobility_solver launches them; oracle/ref_gpu.py) against this
library's products on the same GB300, medium swimmer (12 800 segments,
2 562 blobs): FP64 within 1e-12 of the largest velocity, block by block.
The reference's FP32 build (Real = float) is compared too, to FP32 accuracy
(its velocities carry plain FP32 sums: bar 1e-4, error printed).

The cubins exist only where the reference tree was available when oracle/
was built; elsewhere this test skips.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def ours(sw):
    from timfilsimmod_gb300.mobility import RpyMobilitySolver

    s = RpyMobilitySolver(1, sw.nfil, sw.nseg, sw.num_blobs, precision="fp64")
    s.set_state(sw.x_segs, sw.f_segs, sw.x_blobs, sw.f_blobs)
    out = {}
    s.evaluate_segment_segment_mobility()
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    out["mss"] = s.v_segs_host.copy()
    s.evaluate_segment_blob_mobility()
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    out["mss_msb"] = s.v_segs_host.copy()
    s.evaluate_blob_blob_mobility()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    out["mbb"] = s.v_blobs_host.copy()
    s.evaluate_blob_segment_mobility()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    out["mbs"] = s.v_blobs_host.copy()
    s.finalise()
    return out


def reference(sw, precision):
    import torch

    from ref_gpu import RefGpuKernels

    k = RefGpuKernels(precision)
    dt = k.dtype
    t = {n: torch.tensor(np.asarray(a).ravel(), dtype=dt, device="cuda")
         for n, a in (("x_segs", sw.x_segs), ("f_segs", sw.f_segs), ("x_blobs", sw.x_blobs),
                      ("f_blobs", sw.f_blobs))}
    vs = torch.zeros(6 * sw.num_segs, dtype=dt, device="cuda")
    vb = torch.zeros(3 * sw.num_blobs, dtype=dt, device="cuda")
    k.sync(1, sw.nseg, sw.nfil, sw.num_blobs)
    out = {}
    k.mss(vs, t["f_segs"], t["x_segs"])
    out["mss"] = vs.cpu().numpy().astype(np.float64)
    k.msb(vs, t["f_blobs"], t["x_segs"], t["x_blobs"])
    out["mss_msb"] = vs.cpu().numpy().astype(np.float64)
    k.mbb(vb, t["f_blobs"], t["x_blobs"])
    out["mbb"] = vb.cpu().numpy().astype(np.float64)
    k.mbs(vb, t["f_segs"], t["x_blobs"], t["x_segs"])
    out["mbs"] = vb.cpu().numpy().astype(np.float64)
    torch.cuda.synchronize()
    k.close()
    return out


def test_reference_gpu_kernels_match_ours():
    import ref_gpu

    if not (ref_gpu.available("fp64") and ref_gpu.available("fp32")):
        pytest.skip("the reference's kernels were not compiled here (no reference tree)")
    from timfilsimmod_gb300.geometry import make_config

    sw = make_config("medium", seed=5)
    mine = ours(sw)
    r64 = reference(sw, "fp64")
    r32 = reference(sw, "fp32")
    for k in mine:
        e64, e32 = rel_max(r64[k], mine[k]), rel_max(r32[k], mine[k])
        print(f"\n{k}: reference FP64 kernels vs ours {e64:.2e}; reference FP32 kernels {e32:.2e}")
        assert e64 < 1e-12, (k, e64)
        assert e32 < 1e-4, (k, e32)


def test_reference_prescribed_kernels_match_our_hooks():
    """The reference's kernels of its prescribed-cilia build (configuration
    p1 of oracle/Makefile: forces only, rpy_interaction<3,3>, Mbs_mult
    adding) against our block hooks in their prescribed-cilia form (after
    tfs_prescribed_setup), block by block in the reference's launch order,
    FP64 within 1e-12 of the largest velocity; 160 beating filaments x 20
    segments on a 642-blob sphere, with random torques in f_segs that both
    must ignore."""
    import torch

    import ref_gpu

    if not ref_gpu.available("fp64", "prescribed"):
        pytest.skip("the reference's prescribed-cilia kernels were not compiled here")
    from timfilsimmod_gb300.geometry import prescribed_swimmer
    from timfilsimmod_gb300.prescribed import PrescribedCiliaSolver

    g = prescribed_swimmer(160, 20, radius=20.0, subdivisions=3, seg_sep=2.2)
    rng = np.random.default_rng(8)
    phase, angle = rng.uniform(0, 2 * np.pi, g.nfil), np.zeros(g.nfil)
    x, vp, va = g.kinematics(phase, angle)
    ns, nb = g.nfil * g.nseg, g.blob_references.shape[0]
    fs, fb = rng.normal(size=6 * ns), rng.normal(size=3 * nb)
    t = 2 * np.pi * np.arange(16) / 16
    ps = PrescribedCiliaSolver(6, g.nfil, g.nseg, g.blob_references, g.seg_sep, 1 + np.sin(t),
                               np.cos(t))
    ps.set_kinematics(x, vp, va, phase, np.ones(g.nfil), angle)
    s = ps.solver
    s.f_segs_host[:] = fs
    s.f_blobs_host[:] = fb
    s.copy_segment_forces_to_device()
    s.copy_blob_forces_to_device()
    mine = {}
    s.evaluate_segment_segment_mobility()
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    mine["mss"] = s.v_segs_host.copy()
    s.evaluate_segment_blob_mobility()
    s.copy_segment_velocities_to_host()
    s.wait_for_device()
    mine["mss_msb"] = s.v_segs_host.copy()
    s.evaluate_blob_blob_mobility()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    mine["mbb"] = s.v_blobs_host.copy()
    s.evaluate_blob_segment_mobility()
    s.copy_blob_velocities_to_host()
    s.wait_for_device()
    mine["mbb_mbs"] = s.v_blobs_host.copy()
    ps.finalise()

    k = ref_gpu.RefGpuKernels("fp64", "prescribed")
    d = {n: torch.tensor(np.asarray(a).ravel(), dtype=torch.float64, device="cuda")
         for n, a in (("xs", x), ("fs", fs), ("xb", g.blob_references), ("fb", fb))}
    vs = torch.zeros(6 * ns, dtype=torch.float64, device="cuda")
    vb = torch.zeros(3 * nb, dtype=torch.float64, device="cuda")
    k.sync(1, g.nseg, g.nfil, nb)
    ref = {}
    k.mss(vs, d["fs"], d["xs"])
    ref["mss"] = vs.cpu().numpy()
    k.msb(vs, d["fb"], d["xs"], d["xb"])
    ref["mss_msb"] = vs.cpu().numpy()
    k.mbb(vb, d["fb"], d["xb"])
    ref["mbb"] = vb.cpu().numpy()
    k.mbs(vb, d["fs"], d["xb"], d["xs"])
    ref["mbb_mbs"] = vb.cpu().numpy()
    torch.cuda.synchronize()
    k.close()
    for key in mine:
        e = rel_max(mine[key], ref[key])
        print(f"\n{key}: reference prescribed-cilia kernels vs our hooks {e:.2e}")
        assert e < 1e-12, (key, e)
