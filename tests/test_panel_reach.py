"""The panel-reach pre-test of the phantom stage (may_reach_panels in
gpet_gb300/csrc/device.cuh, bound built by ring_bound in gpet_api.cu) may only
skip photons that the panel search (enter_panel, photonde's panel loop,
gPET_kernals.cu:963-1009) would not enter: restated here in float32 and run
on random photons of the positron and whole-body rings, inside the ring
(where only the ray ahead counts) and outside it (where the whole line
does)."""
import math
import os

import numpy as np
import pytest

from gpet_gb300 import formats as F, scenes

f32 = np.float32


def _ring_bound(P):
    """ring_bound: (test, zmin, zmax, rin2) with test 2 when every face is
    entered only from the axis side."""
    zmin, zmax, rin, toward = 1e30, -1e30, 1e30, True
    for p in P.astype(np.float64):
        nx, ny, nz = p[21], p[22], p[23]
        nxy = math.sqrt(nx * nx + ny * ny)
        if abs(nz) > 1e-6 or not nxy > 0.5:
            return 0, 0.0, 0.0, 0.0
        rin = min(rin, abs(nx * p[15] + ny * p[16]) / nxy)
        no = nx * p[15] + ny * p[16] + nz * p[17]
        if not (p[18] != 0 and no != 0 and (p[18] > 0) == (no > 0)):
            toward = False
        for sy in (-1, 1):
            for sz in (-1, 1):
                z = p[17] + sy * 0.5 * p[1] * p[26] + sz * 0.5 * p[2] * p[29]
                zmin, zmax = min(zmin, z), max(zmax, z)
    pad = 1e-3
    r = rin * (1.0 - 1e-4) - pad
    return (2 if toward else 1, f32(zmin - pad - 1e-4 * abs(zmin)), f32(zmax + pad + 1e-4 * abs(zmax)),
            f32(r * r))


def _may_reach(bound, x, u):
    test, zmin, zmax, rin2 = bound
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        iu = f32(1) / u[:, 2]
        t1 = (zmin - x[:, 2]) * iu
        t2 = (zmax - x[:, 2]) * iu
        tb = np.maximum(t1, t2)
        ta = np.minimum(t1, t2)
        inside = x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1] < rin2
        fwd = (test == 2) & inside
        ta = np.where(fwd, np.maximum(ta, f32(0)), ta)
        x1, y1 = x[:, 0] + ta * u[:, 0], x[:, 1] + ta * u[:, 1]
        x2, y2 = x[:, 0] + tb * u[:, 0], x[:, 1] + tb * u[:, 1]
        ok = np.maximum(x1 * x1 + y1 * y1, x2 * x2 + y2 * y2) >= rin2
        ok &= ~(fwd & (tb < 0))
    flat = u[:, 2] == 0
    ok[flat] = (x[flat, 2] >= zmin) & (x[flat, 2] <= zmax)
    return ok


def _enter(P, x, u):
    hit = np.zeros(len(x), bool)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for p in P:
            tvx = u[:, 0] * p[21] + u[:, 1] * p[22] + u[:, 2] * p[23]
            px, py, pz = x[:, 0] - p[15], x[:, 1] - p[16], x[:, 2] - p[17]
            tx = px * p[21] + py * p[22] + pz * p[23]
            ty = px * p[24] + py * p[25] + pz * p[26]
            tz = px * p[27] + py * p[28] + pz * p[29]
            tvy = u[:, 0] * p[24] + u[:, 1] * p[25] + u[:, 2] * p[26]
            tvz = u[:, 0] * p[27] + u[:, 1] * p[28] + u[:, 2] * p[29]
            q = tx / tvx
            ty2, tz2 = ty - q * tvy, tz - q * tvz
            hit |= (tvx * p[18] >= 0) & (np.abs(ty2) < p[1] / f32(2)) & (np.abs(tz2) < p[2] / f32(2))
    return hit


def _photons(rng, n, rmax, zmax):
    r = rmax * np.sqrt(rng.random(n))
    ph = 2 * np.pi * rng.random(n)
    x = np.stack([r * np.cos(ph), r * np.sin(ph), zmax * (2 * rng.random(n) - 1)], 1).astype(f32)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    u[: n // 50, 2] = 0.0    # some moving parallel to the faces' band
    u[: n // 50] /= np.linalg.norm(u[: n // 50], axis=1, keepdims=True)
    return x, u.astype(f32)


@pytest.mark.parametrize("ring", ["positron", "large"])
def test_pre_test_never_skips_an_entering_photon(ring, tmp_path):
    d = str(tmp_path)
    sc = scenes.positron(d, n_decays=1000) if ring == "positron" else scenes.large(d, n_decays=1000,
                                                                                    dims=(8, 8, 8))
    cfg = F.read_config(sc.config_path)
    P = F.read_geo(os.path.join(d, os.path.basename(cfg.geofile)) if not os.path.isabs(cfg.geofile)
                   else cfg.geofile).panels.astype(f32)
    bound = _ring_bound(P)
    assert bound[0] == 2
    rin = math.sqrt(float(bound[3]))
    rng = np.random.default_rng(11)
    for rmax, zmax in ((0.9 * rin, 2.0 * float(bound[2])), (1.5 * rin, 3.0 * float(bound[2]))):
        x, u = _photons(rng, 400_000, rmax, zmax)
        hit = _enter(P, x, u)
        ok = _may_reach(bound, x, u)
        assert hit.sum() > 1000
        assert not (hit & ~ok).any(), int((hit & ~ok).sum())
        # the bound is not vacuous: it skips most photons that miss
        assert ok.mean() < 0.8
