"""The surrogate's tensor-core path (tcgen05.mma, BF16 operands, FP32 in TMEM)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    """float32 -> bf16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def _bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("K,N", [(16, 16), (16, 256), (64, 256), (256, 256), (256, 208), (32, 48)])
def test_umma_tile_exact(K, N, gpet_lib):
    """Small integers: every product and partial sum is exact in FP32, so the
    tile must equal the host product bit for bit whatever the order of the
    accumulation."""
    rng = np.random.default_rng(K * 1000 + N)
    a = rng.integers(-3, 4, (128, K)).astype(np.float32)
    b = rng.integers(-3, 4, (N, K)).astype(np.float32)
    ab, bb = _bf16_bits(a), _bf16_bits(b)
    want = a @ b.T
    got = np.zeros((128, N), np.float32)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    rc = gpet_lib.gpet_umma_selftest(0, p(ab), p(bb), K, N, p(got))
    assert rc == 0
    assert np.array_equal(got, want), np.argwhere(got != want)[:5]


def test_umma_tile_rounding(gpet_lib):
    """General bf16 inputs: FP32 accumulation of exact bf16 products."""
    rng = np.random.default_rng(7)
    a = _bf16_bits(rng.standard_normal((128, 256)).astype(np.float32))
    b = _bf16_bits(rng.standard_normal((256, 256)).astype(np.float32) * 0.1)
    want = _bf16_value(a).astype(np.float64) @ _bf16_value(b).astype(np.float64).T
    got = np.zeros((128, 256), np.float32)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    assert gpet_lib.gpet_umma_selftest(0, p(a), p(b), 256, 256, p(got)) == 0
    # FP32 accumulation error bound: a few ulp of the sum of |products|
    scale = np.abs(_bf16_value(a)).astype(np.float64) @ np.abs(_bf16_value(b)).astype(np.float64).T
    assert np.all(np.abs(got - want) <= 1e-5 * scale + 1e-7)


# ---------------------------------------------------------------- the MLP
import surrogate_ref as S  # noqa: E402
from conftest import make_ctx  # noqa: E402


def _geom(ctx):
    P = ctx.panels()
    moduleNy, moduleN, crystalNy, crystalN = ctx.counts()
    return P.shape[0], P[0, 1] / 2, P[0, 2] / 2, P[0, 0], crystalN, (P[0, 10] + P[0, 13], P[0, 11] + P[0, 14])


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_and_gradients_match_oracle(scene_positron, data_dir, gpet_lib):
    """Fused tcgen05 forward and the tcgen05 backward products against the
    oracle with the same bf16 rounding points; 1000 records (a partial last
    tile of 128)."""
    from gpet_gb300 import api
    ctx = make_ctx(scene_positron, data_dir)
    sur = api.Surrogate(ctx, seed=3)
    npan, hy, hz, dl, ncry, pitch = _geom(ctx)
    assert sur.param_count == S.offsets(npan)[2]
    p = S.init_params(npan, 11)
    sur.set_params(p)
    assert np.array_equal(sur.params(), p)
    rec = S.random_records(1000, npan, hy, hz, dl, ncry, 5)
    loss_ref, g_ref, out_ref = S.forward_backward(p, rec, npan, hy, hz, dl, ncry, rounding=True, pitch=pitch)
    out = sur.forward(rec)
    assert _rel(out[:, :S.OUT_USED], out_ref[:, :S.OUT_USED]) < 5e-3
    loss, g = sur.grad(rec)
    assert abs(loss - loss_ref) <= 2e-4 * abs(loss_ref)
    lay, emb_off, total = S.offsets(npan)
    for l, (w, b) in enumerate(lay):
        assert _rel(g[w:b], g_ref[w:b]) < 2e-2, ("W", l, _rel(g[w:b], g_ref[w:b]))
        e = b + S.fan_out(l)
        assert _rel(g[b:e], g_ref[b:e]) < 1e-2, ("b", l, _rel(g[b:e], g_ref[b:e]))
    assert _rel(g[emb_off:], g_ref[emb_off:]) < 2e-2
    # the gradient is a descent direction of the GPU's own loss
    sur.set_params(p - 1e-3 * g / np.linalg.norm(g))
    loss2, _ = sur.grad(rec)
    assert loss2 < loss


def test_factorised_head_forward_and_gradients_match_oracle(scene_large, data_dir, gpet_lib):
    """The whole-body ring (48 panels of 16 x 16 crystals): the factorised
    crystal head (row and column logits per energy class) through the fused
    forward and the backward products, against the oracle."""
    from gpet_gb300 import api
    ctx = make_ctx(scene_large, data_dir)
    sur = api.Surrogate(ctx, seed=4)
    npan, hy, hz, dl, ncry, pitch = _geom(ctx)
    _, _, cny, _ = ctx.counts()
    assert npan == 48 and ncry == 256 and cny == 16
    p = S.init_params(npan, 12)
    sur.set_params(p)
    rec = S.random_records(1000, npan, hy, hz, dl, ncry, 6)
    loss_ref, g_ref, out_ref = S.forward_backward(p, rec, npan, hy, hz, dl, ncry, rounding=True, pitch=pitch,
                                                  crystal_ny=cny)
    out = sur.forward(rec)
    assert _rel(out[:, :S.OUT_USED], out_ref[:, :S.OUT_USED]) < 5e-3
    loss, g = sur.grad(rec)
    assert abs(loss - loss_ref) <= 2e-4 * abs(loss_ref)
    lay, emb_off, total = S.offsets(npan)
    w4, b4 = lay[-1]
    assert _rel(g[w4:b4], g_ref[w4:b4]) < 2e-2
    assert _rel(g[b4:b4 + S.OUT], g_ref[b4:b4 + S.OUT]) < 1e-2
    assert _rel(g[emb_off:], g_ref[emb_off:]) < 2e-2


def test_entries_train_and_run_with_surrogate(scene_positron, data_dir, gpet_lib):
    from gpet_gb300 import api
    gen = make_ctx(scene_positron, data_dir, seed=101, n_decays=300000, record_entries=1)
    st = gen.run()
    rec = gen.entries()
    assert len(rec) == st["n_entered"]
    has = rec["crystal"] >= 0
    assert has.mean() > 0.3
    assert (rec["depth"][has] >= 0).all() and (rec["Edep"][has] <= rec["E"][has] * 1.0001).all()
    sur = api.Surrogate(gen, seed=5)
    losses = sur.train(rec, epochs=4, batch=4096, lr=2e-3)
    assert np.isfinite(losses).all() and losses[-1] < losses[0]
    sur.set_domain(1.0e5, 5.2e5, 0.3)
    mc = make_ctx(scene_positron, data_dir, seed=202, n_decays=200000)
    st_mc = mc.run()
    sc = make_ctx(scene_positron, data_dir, seed=202, n_decays=200000)
    sc.set_surrogate(sur)
    st_s = sc.run()
    assert st_s["n_entered"] == st_mc["n_entered"]
    assert st_s["n_surrogate"] > 0.5 * st_s["n_entered"]
    assert st_s["n_singles"] > 0 and st_s["n_coinc"] > 0
    ev, scat, slot = sc.pulses()
    P = sc.panels()
    moduleNy, moduleN, crystalNy, crystalN = sc.counts()
    assert (ev["cryn"] >= 0).all() and (ev["cryn"] < crystalN).all()
    assert (ev["E"] > 0).all() and (ev["E"] <= 5.3e5).all()
    assert (np.abs(ev["y"]) <= P[0, 1] / 2).all() and (np.abs(ev["z"]) <= P[0, 2] / 2).all()
    # the same run without the surrogate attached is the plain Monte Carlo again
    sc.set_surrogate(None)
    st_b = sc.run()
    assert st_b["n_surrogate"] == 0 and st_b["n_singles"] == st_mc["n_singles"]


def test_crystal_calibration_matches_observed_counts(scene_positron, data_dir, gpet_lib):
    """gpet_surrogate_calibrate moves only the head's crystal and energy-bin
    biases, and afterwards the model's expected counts over the records of its
    domain — per energy bin, and per (energy class, crystal): class
    probability from the energy-bin softmax times the class's crystal
    softmax, computed here in float64 from the raw head outputs — equal the
    observed counts of those records (within 2 % after 16 passes, and the
    largest log ratio of a pass still shrinking from pass 8 to pass 16, so a
    calibration that stops converging fails)."""
    from gpet_gb300 import api
    gen = make_ctx(scene_positron, data_dir, seed=303, n_decays=600000, record_entries=1)
    gen.run()
    rec = gen.entries()
    sur = api.Surrogate(gen, seed=6)
    sur.train(rec, epochs=2, batch=4096, lr=2e-3)
    sur.set_domain(1.0e5, 5.2e5, 0.3)
    npan, hy, hz, _, ncry, _ = _geom(gen)
    p0 = sur.params()
    adj8 = sur.calibrate(rec, iters=8)
    adj = sur.calibrate(rec, iters=8)       # passes 9-16 continue from the biases of pass 8
    assert adj < adj8, (adj8, adj)
    p1 = sur.params()
    b_head = len(p0) - npan * 6 - 208   # the head's bias sits before the embedding
    changed = np.nonzero(p0 != p1)[0]
    assert len(changed) > 0
    assert changed.min() >= b_head and changed.max() < b_head + 204, (changed.min(), changed.max())
    assert not np.isin(changed - b_head, np.arange(128, 140)).any()   # depth mixture untouched
    dom = rec[(rec["E"] >= 1.0e5) & (rec["E"] <= 5.2e5) & (np.abs(rec["y"]) <= hy - 0.3) &
              (np.abs(rec["z"]) <= hz - 0.3)]
    out = sur.forward(dom).astype(np.float64)
    eb = out[:, 140:204]
    pe = np.exp(eb - eb.max(axis=1, keepdims=True))
    pe /= pe.sum(axis=1, keepdims=True)
    pc = [pe[:, 1:40].sum(axis=1), pe[:, 40:64].sum(axis=1)]
    has = (dom["crystal"] >= 0) & (dom["Edep"] > 0)
    b = np.clip((dom["Edep"][has] / dom["E"][has] * np.float32(64)).astype(np.int64), 1, 63)
    ob = np.bincount(b, minlength=64).astype(np.float64)
    ob[0] = (~has).sum()
    ok = ob >= 20
    assert ok.sum() > 32
    assert np.abs(pe.sum(axis=0)[ok] / ob[ok] - 1.0).max() < 0.02, adj
    for s in range(2):
        lg = out[:, 64 * s:64 * s + ncry]
        pk = np.exp(lg - lg.max(axis=1, keepdims=True))
        pk /= pk.sum(axis=1, keepdims=True)
        expected = (pc[s][:, None] * pk).sum(axis=0)
        sel = (b >= 40) if s else (b < 40)
        observed = np.bincount(dom["crystal"][has][sel], minlength=ncry)[:ncry].astype(np.float64)
        big = observed >= 20    # fitted to these very records: equal up to convergence, not statistics
        assert big.sum() > ncry // 2, (s, observed)
        rel = np.abs(expected[big] / observed[big] - 1.0)
        assert rel.max() < 0.02, (s, rel.max(), adj)
