"""The surrogate's CPU oracle: its hand-written backward pass against finite
differences of its own forward pass (float64, no rounding)."""
import numpy as np
import pytest

import surrogate_ref as S

NP, HY, HZ, DEPTH, NCRY = 3, 1.2, 1.2, 2.0, 64


def _setup(n=24, seed=5):
    p = S.init_params(NP, seed).astype(np.float64)
    rec = S.random_records(n, NP, HY, HZ, DEPTH, NCRY, seed + 1)
    return p, rec


def _loss(p, rec):
    return S.forward_backward(p, rec, NP, HY, HZ, DEPTH, NCRY, rounding=False)[0]


def test_layout():
    lay, emb_off, total = S.offsets(NP)
    assert lay[0] == (0, 16 * 256)
    assert emb_off == 255184
    assert total == 255184 + NP * S.EMB
    macs = 16 * 256 + 3 * 256 * 256 + 256 * 204
    assert macs == 252928


def test_backward_matches_finite_differences():
    p, rec = _setup()
    loss, g, _ = S.forward_backward(p, rec, NP, HY, HZ, DEPTH, NCRY, rounding=False)
    assert np.isfinite(loss) and loss > 0
    lay, emb_off, total = S.offsets(NP)
    rng = np.random.default_rng(3)
    picks = []
    for l, (w, b) in enumerate(lay):
        K = S.fan_in(l)
        rows = S.OUT_USED if l == S.LAYERS - 1 else S.fan_out(l)
        cols = S.FEAT if l == 0 else K
        for _ in range(4):
            picks.append(w + int(rng.integers(rows)) * K + int(rng.integers(cols)))
        picks.append(b + int(rng.integers(rows)))
    picks += [emb_off + int(i) for i in rng.integers(0, NP * S.EMB, 4)]
    # head columns of each kind: crystal, mixture weight / mean / log sigma, energy
    w4, b4 = lay[-1]
    picks += [b4 + 3, b4 + S.CRY + 9, b4 + S.COL_W + 1, b4 + S.COL_MU + 2, b4 + S.COL_LS + 3, b4 + S.COL_E + 5]
    eps = 1e-6
    for i in picks:
        q = p.copy()
        q[i] += eps
        lp = _loss(q, rec)
        q[i] -= 2 * eps
        lm = _loss(q, rec)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_padding_has_no_gradient():
    p, rec = _setup()
    _, g, _ = S.forward_backward(p, rec, NP, HY, HZ, DEPTH, NCRY, rounding=False)
    lay, _, _ = S.offsets(NP)
    w0, b0 = lay[0]
    assert not g[w0:b0].reshape(256, 16)[:, S.FEAT:].any()
    w4, b4 = lay[-1]
    assert not g[w4:b4].reshape(S.OUT, 256)[S.OUT_USED:].any()
    assert not g[b4 + S.OUT_USED:b4 + S.OUT].any()


def test_in_crystal_offset_features():
    """Inputs 14, 15: the entry point's offset from its crystal's centre, in
    pitches (crystal 0 starts at the panel edge)."""
    rec = np.zeros(4, S.ENTRY_DTYPE)
    rec["y"] = [-1.2, -1.05, 0.0, 1.1]
    rec["z"] = [0.15, -0.6, 0.299, -1.2]
    rec["ux"] = -1.0                                  # normal incidence: the mid-depth point is the entry point
    f = S.features(rec, np.zeros((1, S.EMB)), 1.2, 1.2, (0.3, 0.3), 2.0)
    assert np.array_equal(f[:, 6:8], f[:, 14:16])
    assert np.allclose(f[:, 14], [-0.5, 0.0, -0.5, 0.1666667], atol=1e-5)
    assert np.allclose(f[:, 15], [0.0, -0.5, 0.4966667, -0.5], atol=1e-5)
    assert (np.abs(f[:, 14:]) <= 0.5).all()


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-8], np.float32)
    r = S.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-6
    assert (r.view(np.uint32) & 0xFFFF == 0).all()


def test_factorised_head_backward_matches_finite_differences():
    """A ring of 16 x 16 crystals (more than the 64 one softmax holds): each
    energy class's set holds 16 row logits (columns 0-15 of the set) and 16
    column logits (32-47); its gradient against finite differences, and no
    gradient on the set's unused columns."""
    npan, ncry, ny = 4, 256, 16
    p = S.init_params(npan, 9).astype(np.float64)
    rec = S.random_records(32, npan, 3.2, 3.2, DEPTH, ncry, 10)
    pitch = (0.4, 0.4)
    loss, g, _ = S.forward_backward(p, rec, npan, 3.2, 3.2, DEPTH, ncry, rounding=False, pitch=pitch,
                                    crystal_ny=ny)
    assert np.isfinite(loss) and loss > 0
    lay, _, _ = S.offsets(npan)
    w4, b4 = lay[-1]
    eps = 1e-6
    for col in (2, 15, 32 + 3, 32 + 15, S.CRY + 7, S.CRY + 32 + 11):
        q = p.copy()
        q[b4 + col] += eps
        lp = S.forward_backward(q, rec, npan, 3.2, 3.2, DEPTH, ncry, rounding=False, pitch=pitch, crystal_ny=ny)[0]
        q[b4 + col] -= 2 * eps
        lm = S.forward_backward(q, rec, npan, 3.2, 3.2, DEPTH, ncry, rounding=False, pitch=pitch, crystal_ny=ny)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[b4 + col]) <= 1e-6 + 1e-4 * abs(fd), (col, fd, g[b4 + col])
    unused = [c for s in (0, S.CRY) for c in list(range(s + 16, s + 32)) + list(range(s + 48, s + 64))]
    assert not g[[b4 + c for c in unused]].any()
