"""The orbit-search client (timfilsimmod_gb300.orbit) on the request server:
Newton-Krylov iterations whose every period map is a server request (two
implicit steps of a small swimmer, FP64). Two searches from different
starts run each alone (a server of one worker, one search at a time) and
then together (one server of four workers, the searches in threads, their
requests interleaved on the GPU): their iterates, Krylov vectors and
Hessenberg matrices are the same, bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT, TOL = 1e-3, 1e-4


def server(workers):
    from timfilsimmod_gb300.serving import StepServer

    efm = 220.0 * 1800.0 / (2.6 * 2.6 * 400)
    return StepServer(num_workers=workers, precision="fp64", linear_tol=1e-10, dt=DT, tol=TOL,
                      seg_sep=2.2, end_force_magnitude=efm)


def geometry():
    from timfilsimmod_gb300.geometry import fibonacci_sphere, icosphere

    radius, nfil = 10.0, 7
    normals = fibonacci_sphere(nfil)
    return radius * icosphere(2), (radius + 1.0 + 1.1) * normals, normals, radius


def test_orbit_searches_alone_and_concurrent_agree():
    from timfilsimmod_gb300.orbit import OrbitSearch, search_many

    br, fr, fd, radius = geometry()
    starts = [0.01 * np.random.default_rng(s).normal(size=3 * 7 * 20) for s in (11, 12)]
    kw = dict(m=3, iters=1)
    alone = []
    for x0 in starts:
        sv = server(1)
        o = OrbitSearch(sv, br, fr, fd, 20, num_steps=2, body_radius=radius)
        alone.append(o.newton(x0, **kw))
        sv.close()
    sv = server(4)
    searches = [OrbitSearch(sv, br, fr, fd, 20, num_steps=2, body_radius=radius) for _ in starts]
    mix = search_many(searches, starts, **kw)
    sv.close()
    for a, b in zip(alone, mix):
        assert b is not None
        assert np.isfinite(a["residual"]).all() and a["residual"][0] > 0
        for va, vb in zip(a["krylov"], b["krylov"]):
            assert np.array_equal(va, vb)
        for ha, hb in zip(a["hessenberg"], b["hessenberg"]):
            assert np.array_equal(ha, hb)
        for xa, xb in zip(a["x"], b["x"]):
            assert np.array_equal(xa, xb)
    print("\nresiduals:", [r["residual"] for r in alone], "requests:", [r["requests"] for r in alone])
