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
    assert emb_off == 238736
    assert total == 238736 + NP * 8
    macs = 14 * 256 + 3 * 256 * 256 + 256 * 140
    assert macs == 236032


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
    picks += [emb_off + int(i) for i in rng.integers(0, NP * 8, 4)]
    # head columns of each kind: crystal, mixture weight / mean / log sigma, energy
    w4, b4 = lay[-1]
    picks += [b4 + 3, b4 + S.COL_W + 1, b4 + S.COL_MU + 2, b4 + S.COL_LS + 3, b4 + S.COL_E + 5]
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
    assert not g[w0:b0].reshape(256, 16)[:, 14:].any()
    w4, b4 = lay[-1]
    assert not g[w4:b4].reshape(144, 256)[140:].any()
    assert not g[b4 + 140:b4 + 144].any()


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-8], np.float32)
    r = S.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-6
    assert (r.view(np.uint32) & 0xFFFF == 0).all()
