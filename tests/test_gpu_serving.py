"""Many swimmers on one GPU: a batch of uneven swimmers stepped together, and
the request server (timfilsimmod_gb300.serving).

Each instance owns its solver, stepper and stream and keeps no state on the
device that others touch; FP32C inner solves share cooperative launches, but
each runs on a fixed number of CTAs chosen from its own size, and every
reduction is in a fixed order. So a swimmer's result is the same -- bit for
bit -- alone (a batch of one; a server with one worker) and in the mix: that
is the bar here (tolerance 0), in FP64 and FP32C. The parity of a single
swimmer's step with the reference is covered by test_gpu_step.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# uneven swimmers: (sphere subdivisions -> blobs, filaments), 20 segments each
SHAPES = [(2, 12), (3, 24), (2, 7)]
DT, TOL = 1e-3, 1e-4


def geometry(subdiv, nfil, radius=None):
    from timfilsimmod_gb300.geometry import fibonacci_sphere, icosphere

    radius = radius or (10.0 if subdiv == 2 else 20.0)
    blob_refs = radius * icosphere(subdiv)
    normals = fibonacci_sphere(nfil)
    fil_refs = (radius + 1.0 + 1.1) * normals
    return blob_refs, fil_refs, normals, radius


def efm(nseg=20):
    return 220.0 * 1800.0 / (2.6 * 2.6 * nseg * nseg)


def make_instance(subdiv, nfil, precision):
    from timfilsimmod_gb300.mobility import RpyMobilitySolver
    from timfilsimmod_gb300.stepper import ImplicitStepper

    blob_refs, fil_refs, normals, radius = geometry(subdiv, nfil)
    s = RpyMobilitySolver(1, nfil, 20, blob_refs.shape[0], precision=precision,
                          end_force_magnitude=int(efm()))
    s.set_blob_references(blob_refs)
    s.set_linear_solver(1e-8, min(350, 3 * blob_refs.shape[0] + 6))
    st = ImplicitStepper(s, nfil, 20, fil_refs, normals, seg_sep=2.2, dt=DT, tol=TOL,
                         end_force_magnitude=efm(), body_radius=radius)
    return s, st


@pytest.mark.parametrize("precision,share,products", [
    ("fp64", False, True), ("fp64", False, False), ("fp32c", False, True), ("fp32c", True, True),
    ("fp32c", -1, True), ("fp32c", -1, False)])
def test_batch_same_as_alone(precision, share, products):
    """Each swimmer in a batch of one with its products on its own launches
    (the reference result), in a batch of one and in a batch of three with
    inner solves and pair products shared or not: the same state, bit for
    bit. FP64 swimmers also match a stepper outside any batch."""
    from timfilsimmod_gb300.serving import SwimmerBatch

    steps = 3

    def one_by_one(share_products):
        res = []
        for subdiv, nfil in SHAPES:
            s, st = make_instance(subdiv, nfil, precision)
            one = SwimmerBatch(num_workers=1)
            one.share_inner_solves(share)
            one.share_products(share_products)
            one.add(st)
            for nt in range(steps):
                one.step(nt, allow_unconverged=True)
            if share is True:
                sh = one.shared_solves()
                assert sh["solves"] > 0 and sh["launches"] == sh["solves"], sh
            sp = one.shared_products()
            assert (sp["products"] > 0) == share_products, sp
            res.append(st.state())
            one.close()
            st.close()
            s.finalise()
        return res

    alone = one_by_one(False)
    for got, ref in zip(one_by_one(products), alone):
        for k in ("x", "q", "lam", "body_x", "body_q"):
            assert np.array_equal(got[k], ref[k]), ("batch of one", k)
    if precision == "fp64":  # the FP32C inner solve takes another form outside a batch
        for (subdiv, nfil), ref in zip(SHAPES, alone):
            s, st = make_instance(subdiv, nfil, precision)
            for nt in range(steps):
                st.step(nt, allow_unconverged=True)
            got = st.state()
            for k in ("x", "q", "lam", "body_x", "body_q"):
                assert np.array_equal(got[k], ref[k]), ("outside a batch", k)
            st.close()
            s.finalise()
    inst = [make_instance(subdiv, nfil, precision) for subdiv, nfil in SHAPES]
    batch = SwimmerBatch(num_workers=3)
    batch.share_inner_solves(share)
    batch.share_products(products)
    for _, st in inst:
        batch.add(st)
    for nt in range(steps):
        out = batch.step(nt, allow_unconverged=True)
        assert np.all(out["gmres_iters"] > 0)
    sh = batch.shared_solves()
    if share is not False:  # -1 (the default) shares every FP32C solve
        assert sh["solves"] > 0 and 0 < sh["launches"] <= sh["solves"], sh
    else:
        assert sh == {"launches": 0, "solves": 0}
    sp = batch.shared_products()
    if products:
        assert sp["products"] > 0 and 0 < sp["launches"] <= sp["products"], sp
    else:
        assert sp == {"launches": 0, "products": 0}
    for (s, st), ref in zip(inst, alone):
        got = st.state()
        for k in ("x", "q", "lam", "body_x", "body_q"):
            assert np.array_equal(got[k], ref[k]), k
    batch.close()
    for s, st in inst:
        st.close()
        s.finalise()


def requests(seed=3, repeat=2):
    rng = np.random.default_rng(seed)
    out = []
    for r in range(repeat):
        for subdiv, nfil in SHAPES:
            rot = 1e-6 * rng.normal(size=(nfil * 20, 3))
            out.append((subdiv, nfil, rot))
    return out


def serve(reqs, workers, budget_gb=160.0, one_at_a_time=False, precision="fp32c"):
    from timfilsimmod_gb300.serving import StepServer

    sv = StepServer(num_workers=workers, hbm_budget_gb=budget_gb, precision=precision,
                    linear_tol=1e-8, dt=DT, tol=TOL, seg_sep=2.2, end_force_magnitude=efm())
    results, tickets = [], []
    for subdiv, nfil, rot in reqs:
        blob_refs, fil_refs, normals, radius = geometry(subdiv, nfil)
        t = sv.submit(blob_refs, fil_refs, normals, 20, num_steps=2, seg_rotation=rot,
                      body_radius=radius)
        if one_at_a_time:
            results.append(sv.poll(t, wait=True))
        else:
            tickets.append(t)
    results += [sv.poll(t, wait=True) for t in tickets]
    stats = sv.stats()
    stats.update(sv.shared_solves())
    sv.close()
    return results, stats


def test_server_results_same_alone_and_in_mix():
    reqs = requests()
    alone, stats = serve(reqs, workers=1, one_at_a_time=True)
    # one request at a time: each geometry's instance is built once, then reused
    assert stats["created"] == len(SHAPES) and stats["reused"] == len(reqs) - len(SHAPES)
    assert stats["solves"] > 0 and stats["launches"] == stats["solves"]
    mix, mstats = serve(reqs, workers=4)
    assert 0 < mstats["launches"] <= mstats["solves"]
    for a, m in zip(alone, mix):
        assert np.array_equal(a["x"], m["x"])
        assert np.array_equal(a["body"], m["body"])
        assert m["latency_ms"] > 0 and m["broyden_iters"] > 0
    # two perturbations of one geometry give two different results
    assert not np.array_equal(mix[0]["x"], mix[len(SHAPES)]["x"])


def test_server_budget_evicts_and_rejects():
    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.serving import StepServer

    reqs = requests(repeat=1)
    full, _ = serve(reqs, workers=2)
    # room for one instance at a time (the largest is ~31 MB by the server's
    # estimate): admissions evict
    tight, stats = serve(reqs, workers=2, budget_gb=0.035)
    assert stats["evicted"] >= 1
    for a, b in zip(full, tight):
        assert np.array_equal(a["x"], b["x"])
    sv = StepServer(num_workers=1, hbm_budget_gb=0.001)
    blob_refs, fil_refs, normals, _ = geometry(3, 24)
    with pytest.raises(N.TfsError) as e:
        sv.submit(blob_refs, fil_refs, normals, 20)
    assert e.value.code == N.TFS_ENOMEM
    sv.close()


def test_server_admits_past_a_request_waiting_for_memory():
    """Two workers, a budget that holds one large instance and one small one:
    while the first large request runs, a second large one (another
    geometry) waits for memory, and a small request that arrives after it is
    admitted past it; with max_bypass_ms = 0 nothing passes the waiting
    request. Each result is the same, bit for bit, either way."""
    from timfilsimmod_gb300.serving import StepServer

    big_a, big_b, small = geometry(3, 24), geometry(3, 24, radius=20.5), geometry(2, 7)
    probe = StepServer(num_workers=1)
    nb_big = probe.request_bytes(*big_a[:3], 20)
    nb_small = probe.request_bytes(*small[:3], 20)
    probe.close()
    budget_gb = (nb_big + nb_small + (1 << 20)) / float(1 << 30)
    assert nb_big + nb_big > nb_big + nb_small + (1 << 20)  # two large ones never fit

    def run(max_bypass_ms):
        sv = StepServer(num_workers=2, hbm_budget_gb=budget_gb, precision="fp32c",
                        linear_tol=1e-8, dt=DT, tol=TOL, seg_sep=2.2, end_force_magnitude=efm(),
                        max_bypass_ms=max_bypass_ms)
        t = [sv.submit(*g[:3], 20, num_steps=n, body_radius=g[3])
             for g, n in ((big_a, 4), (big_b, 1), (small, 1))]
        res = [sv.poll(k, wait=True) for k in t]
        st = sv.stats()
        sv.close()
        return res, st

    res, st = run(60_000.0)
    assert st["bypassed"] == 1, st
    # the small request did not wait for the second large one
    assert res[2]["latency_ms"] < res[1]["latency_ms"]
    fifo, st0 = run(0.0)
    assert st0["bypassed"] == 0, st0
    for a, b in zip(res, fifo):
        assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["body"], b["body"])


def test_nan_swimmer_does_not_poison_batch():
    """A swimmer whose state is made non-finite on the host (NaN segment
    rotations) fails alone with TFS_ENAN; the others -- whose inner solves
    share cooperative launches with it -- complete, bit for bit as alone."""
    import numpy as np

    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.serving import SwimmerBatch

    alone = []
    for subdiv, nfil in SHAPES:
        s, st = make_instance(subdiv, nfil, "fp32c")
        one = SwimmerBatch(num_workers=1)
        one.add(st)
        one.step(0, allow_unconverged=True)
        alone.append(st.state())
        one.close()
        st.close()
        s.finalise()
    inst = [make_instance(subdiv, nfil, "fp32c") for subdiv, nfil in SHAPES]
    bad = 1
    inst[bad][1].reset(np.full((SHAPES[bad][1] * 20, 3), np.nan))
    batch = SwimmerBatch(num_workers=3)
    for _, st in inst:
        batch.add(st)
    n = len(inst)
    b, g, status = (np.zeros(n, dtype=np.int32) for _ in range(3))
    rc = batch.lib.tfs_batch_step(batch._h, 0, b.ctypes.data, g.ctypes.data, status.ctypes.data)
    assert rc != N.TFS_OK
    assert status[bad] == N.TFS_ENAN, status
    for i, ((s, st), ref) in enumerate(zip(inst, alone)):
        if i == bad:
            continue
        assert status[i] in (N.TFS_OK, N.TFS_ENOTCONV), (i, status)
        got = st.state()
        for k in ("x", "q", "lam", "body_x", "body_q"):
            assert np.array_equal(got[k], ref[k]), (i, k)
    assert batch.shared_solves()["solves"] > 0
    batch.close()
    for s, st in inst:
        st.close()
        s.finalise()


def test_shared_launches_repeatable_under_load():
    """Twelve uneven FP32C swimmers (shared inner-solve launches, 12 host
    workers) stepped twice from the same start: every state bit-identical
    between the runs -- no result depends on how the solves happened to be
    grouped into launches."""
    import numpy as np

    from timfilsimmod_gb300.serving import SwimmerBatch

    shapes = [(2, 7), (3, 24), (2, 12), (3, 40), (2, 9), (3, 17)] * 2

    def run():
        inst = [make_instance(subdiv, nfil, "fp32c") for subdiv, nfil in shapes]
        for i, (_, st) in enumerate(inst):
            nfil = shapes[i][1]
            st.reset(1e-6 * np.random.default_rng(100 + i).normal(size=(nfil * 20, 3)))
        batch = SwimmerBatch(num_workers=12)
        for _, st in inst:
            batch.add(st)
        for nt in range(3):
            batch.step(nt, allow_unconverged=True)
        out = [st.state() for _, st in inst]
        shared = batch.shared_solves()
        batch.close()
        for s, st in inst:
            st.close()
            s.finalise()
        return out, shared

    a, sa = run()
    b, sb = run()
    assert sa["solves"] > 0 and sb["solves"] > 0
    for i, (x, y) in enumerate(zip(a, b)):
        for k in ("x", "q", "lam", "body_x", "body_q"):
            assert np.array_equal(x[k], y[k]), (i, k)


def test_stalled_swimmer_does_not_stall_batch():
    """A swimmer whose inner solves' grid barriers are made (on the host) to
    wait for one CTA more than their launch has fails alone with TFS_ETIMEOUT
    once the 2 s bound runs out; the others -- whose inner solves share
    cooperative launches with it, each solve on its own CTAs and barrier
    words -- complete, bit for bit as alone."""
    from timfilsimmod_gb300 import _native as N
    from timfilsimmod_gb300.serving import SwimmerBatch

    alone = []
    for subdiv, nfil in SHAPES:
        s, st = make_instance(subdiv, nfil, "fp32c")
        one = SwimmerBatch(num_workers=1)
        one.add(st)
        one.step(0, allow_unconverged=True)
        alone.append(st.state())
        one.close()
        st.close()
        s.finalise()
    inst = [make_instance(subdiv, nfil, "fp32c") for subdiv, nfil in SHAPES]
    bad = 1
    inst[bad][0].inject_barrier_stall(True)
    batch = SwimmerBatch(num_workers=3)
    for _, st in inst:
        batch.add(st)
    n = len(inst)
    b, g, status = (np.zeros(n, dtype=np.int32) for _ in range(3))
    rc = batch.lib.tfs_batch_step(batch._h, 0, b.ctypes.data, g.ctypes.data, status.ctypes.data)
    assert rc != N.TFS_OK
    assert status[bad] == N.TFS_ETIMEOUT, status
    for i, ((s, st), ref) in enumerate(zip(inst, alone)):
        if i == bad:
            continue
        assert status[i] in (N.TFS_OK, N.TFS_ENOTCONV), (i, status)
        got = st.state()
        for k in ("x", "q", "lam", "body_x", "body_q"):
            assert np.array_equal(got[k], ref[k]), (i, k)
    assert batch.shared_solves()["solves"] > 0
    batch.close()
    for s, st in inst:
        st.close()
        s.finalise()
