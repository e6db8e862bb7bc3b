"""Many simulations in one job (gpet_run_batched) vs each simulation alone.

Decays of several simulations share waves of the source and phantom kernels,
their photons share one detector queue and their pulses one digitizer pass
sorted by (simulation, time). Each simulation's random streams are keyed by
its own seed and sim_id and by the decay's index within that simulation, so
every record a context reads after the batch must equal, bit for bit, what
the same context gives when run alone."""
import numpy as np
import pytest

from conftest import make_ctx

pytestmark = pytest.mark.gpu

COUNT_KEYS = ("n_decays", "n_pairs", "n_entered", "n_pulses", "n_hits", "n_threshold", "n_deadtime", "n_singles",
              "n_coinc", "n_true", "n_scatter", "n_random", "n_multiple", "n_overflow", "n_stepcap",
              "phantom_steps", "detector_steps")


def _canon_hits(ids, f):
    rec = np.concatenate([ids.view(np.uint32), f.view(np.uint32)], axis=1)
    return rec[np.lexsort(rec.T[::-1])] if len(rec) else rec


def _results(ctx):
    ev, sc, sl = ctx.pulses()
    s, ssc = ctx.singles()
    pr, cl = ctx.coincidences()
    hid, hf = ctx.hits()
    return {"pulses": ev, "pulse_scat": sc, "pulse_slot": sl, "singles": s, "single_scat": ssc, "pairs": pr,
            "class": cl, "hits": _canon_hits(hid, hf)}


def _specs(scene_small, scene_positron):
    # (scene, options): different sizes, seeds, sim ids, policies, a
    # simulation with no decays, and segments that straddle waves
    return [
        (scene_small, dict(seed=11, n_decays=20000)),
        (scene_positron, dict(seed=12, n_decays=7000)),
        (scene_small, dict(seed=11, sim_id=3, n_decays=1500, coinc_policy=1)),
        (scene_small, dict(seed=13, n_decays=0)),
        (scene_positron, dict(seed=14, n_decays=12345, coinc_window_ns=10)),
        (scene_small, dict(seed=15, n_decays=3, record_hits=0)),
    ]


def _same(a, b, what):
    for k in a:
        x, y = a[k], b[k]
        assert x.shape == y.shape, "%s %s: shapes %s vs %s" % (what, k, x.shape, y.shape)
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), "%s %s differs" % (what, k)


def test_batch_equals_individual_runs(scene_small, scene_positron, data_dir, gpet_lib):
    from gpet_gb300 import api
    specs = _specs(scene_small, scene_positron)
    alone, alone_st = [], []
    for scene, opts in specs:
        ctx = make_ctx(scene, data_dir, sub_decays=4096, **opts)
        alone_st.append(ctx.run())
        alone.append(_results(ctx))
        ctx.close()
    # leader's sub_decays sets the wave size: small waves mix simulations
    ctxs = [make_ctx(scene, data_dir, sub_decays=4096, chunk_decays=16384, **opts) for scene, opts in specs]
    stats = api.run_batched(ctxs)
    assert len(stats) == len(specs)
    for i, ctx in enumerate(ctxs):
        what = "simulation %d" % i
        for k in COUNT_KEYS:
            assert stats[i][k] == alone_st[i][k], "%s %s: batch %r alone %r" % (what, k, stats[i][k], alone_st[i][k])
        _same(_results(ctx), alone[i], what)
    assert sum(s["n_coinc"] for s in stats) > 0
    assert stats[3]["n_decays"] == 0 and stats[3]["n_singles"] == 0


def test_batch_results_survive_later_runs(scene_small, data_dir, gpet_lib):
    from gpet_gb300 import api
    a = make_ctx(scene_small, data_dir, seed=21, n_decays=4000)
    b = make_ctx(scene_small, data_dir, seed=22, n_decays=5000)
    api.run_batched([a, b])
    ra, rb = _results(a), _results(b)
    # b runs alone afterwards: a keeps reading the batch's results
    b.set_option("seed", 23)
    b.run()
    _same(_results(a), ra, "leader after a member's own run")
    # and a's own new run leaves b's newest results alone
    rb2 = _results(b)
    a.run()
    _same(_results(b), rb2, "member after the leader's own run")
    assert not np.array_equal(rb2["singles"].view(np.uint8), rb["singles"].view(np.uint8))


def test_batch_of_one_is_run(scene_positron, data_dir, gpet_lib):
    from gpet_gb300 import api
    a = make_ctx(scene_positron, data_dir, seed=5, n_decays=6000)
    st_a = a.run()
    ra = _results(a)
    b = make_ctx(scene_positron, data_dir, seed=5, n_decays=6000)
    st_b = api.run_batched([b])[0]
    for k in COUNT_KEYS:
        assert st_a[k] == st_b[k], k
    _same(_results(b), ra, "batch of one")


def test_batch_argument_errors(scene_small, data_dir, gpet_lib):
    from gpet_gb300 import api
    a = make_ctx(scene_small, data_dir, n_decays=100)
    with pytest.raises(api.GpetError):
        api.run_batched([a, a])
    b = make_ctx(scene_small, data_dir, n_decays=100, record_exits=1)
    with pytest.raises(api.GpetError):
        api.run_batched([a, b])
    # a context with nothing loaded
    c = api.Context(0)
    with pytest.raises(api.GpetError):
        api.run_batched([a, c])


def test_batch_with_surrogate_equals_individual_runs(scene_positron, data_dir, gpet_lib):
    """The learned detector response inside a batched job: the surrogate's
    draws are keyed by each simulation's own streams, so every simulation's
    pulses, singles and coincidences equal those of its run alone with the
    same surrogate."""
    from gpet_gb300 import api
    gen = make_ctx(scene_positron, data_dir, seed=101, n_decays=300000, record_entries=1)
    gen.run()
    rec = gen.entries()
    sur = api.Surrogate(gen, seed=5)
    sur.train(rec, epochs=2, batch=4096, lr=2e-3)
    sur.set_domain(1.0e5, 5.2e5, 0.3)
    specs = [dict(seed=301, n_decays=60000), dict(seed=302, sim_id=4, n_decays=25000), dict(seed=303, n_decays=90000)]
    alone, alone_st = [], []
    for opts in specs:
        ctx = make_ctx(scene_positron, data_dir, sub_decays=8192, **opts)
        ctx.set_surrogate(sur)
        alone_st.append(ctx.run())
        alone.append(_results(ctx))
        ctx.close()
    ctxs = [make_ctx(scene_positron, data_dir, sub_decays=8192, chunk_decays=32768, **opts) for opts in specs]
    for c in ctxs:
        c.set_surrogate(sur)
    stats = api.run_batched(ctxs)
    for i, ctx in enumerate(ctxs):
        what = "simulation %d" % i
        assert stats[i]["n_surrogate"] == alone_st[i]["n_surrogate"] > 0, what
        for k in ("n_entered", "n_pulses", "n_singles", "n_coinc", "n_true", "n_scatter", "n_random"):
            assert stats[i][k] == alone_st[i][k], "%s %s: batch %r alone %r" % (what, k, stats[i][k], alone_st[i][k])
        _same(_results(ctx), alone[i], what)
