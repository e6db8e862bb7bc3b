"""The native loaders (C++) and the Python readers are independent
implementations of gPET's parsers; both must see the same numbers."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, make_ctx

pytestmark = pytest.mark.gpu


def test_tables_identical(scene_small, data_dir, gpet_lib):
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_small, data_dir)
    T = F.read_tables(data_dir)
    for which, arr in enumerate((T.lamph, T.compt, T.phote, T.rayle, T.cmpsf, T.rayff)):
        assert np.array_equal(ctx.table(which), arr.ravel()), which


def test_geometry_and_counts(scene_positron, data_dir, gpet_lib):
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_positron, data_dir)
    g = F.read_geo(os.path.join(scene_positron.directory, "ring.geo"))
    assert np.allclose(ctx.panels(), g.panels, atol=2e-6)
    assert ctx.counts() == g.counts


def test_config8_geometry(data_dir, gpet_lib, tmp_path):
    from gpet_gb300 import api
    ctx = api.Context(0)
    ctx.load_tables(data_dir)
    ctx.load_geometry(os.path.join(GOLDEN, "reference_inputs", "config8.geo"))
    assert ctx.counts() == (9, 117, 8, 64)


def test_source_layout_matches(data_dir, gpet_lib, tmp_path):
    import bridge
    from gpet_gb300 import api, formats as F
    ctx = api.Context(0)
    ctx.load_tables(data_dir)
    src = os.path.join(GOLDEN, "reference_inputs", "source.txt")
    ctx.set_source_file(src, 0.0, 120.0)
    first, count = ctx.source_layout()
    s = F.read_sources(src)
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    f2, c2 = bridge.source_layout(s.natom, s.type, iso.halftime, 0.0, 120.0)
    assert np.array_equal(first, f2) and np.array_equal(count, c2)
    ctx.set_option("n_decays", 1000003)
    first, count = ctx.source_layout()
    f2, c2 = bridge.source_layout(s.natom, s.type, iso.halftime, 0.0, 120.0, 1000003)
    assert count.sum() == 1000003 and np.array_equal(count, c2)


def test_bad_inputs_fail_cleanly(data_dir, gpet_lib, tmp_path):
    from gpet_gb300 import api
    ctx = api.Context(0)
    with pytest.raises(api.GpetError) as e:
        ctx.load_tables(str(tmp_path))
    assert e.value.code == -2
    with pytest.raises(api.GpetError):
        ctx.run()
    with pytest.raises(api.GpetError):
        ctx.set_option("no_such_option", "1")
    ctx.load_tables(data_dir)
    with pytest.raises(api.GpetError):
        ctx.set_phantom(np.full(8, 99, np.int32), np.ones(8, np.float32), (2, 2, 2), (0, 0, 0), (1, 1, 1))
    (tmp_path / "bad.geo").write_text("panel repetition times\n")
    with pytest.raises(api.GpetError):
        ctx.load_geometry(str(tmp_path / "bad.geo"))


def _sinogram_ref(singles, pairs, klass, panels, n_s, n_phi, n_z, s_max, z_max, classes):
    """Single-slice rebinning of the coincidences in float64 (the kernel's arithmetic)."""
    ids = panels[:, 30].astype(int)
    idx = {int(i): k for k, i in enumerate(ids)}
    out = np.zeros((n_z, n_phi, n_s), np.int64)
    for (a, b), k in zip(pairs, klass):
        if k not in classes:
            continue
        g = []
        for e in (a, b):
            s = singles[e]
            P = panels[idx[int(s["pann"])]].astype(np.float64)
            loc = np.array([s["x"], s["y"], s["z"]], np.float64)
            g.append(P[15:18] + loc[0] * P[21:24] + loc[1] * P[24:27] + loc[2] * P[27:30])
        dx, dy = g[1][0] - g[0][0], g[1][1] - g[0][1]
        ln = np.sqrt(dx * dx + dy * dy)
        phi = np.arctan2(dy, dx)
        sd = (g[0][0] * -dy + g[0][1] * dx) / ln
        if phi < 0:
            phi += np.pi
            sd = -sd
        if phi >= np.pi:
            phi -= np.pi
            sd = -sd
        z = 0.5 * (g[0][2] + g[1][2])
        fs = (sd + s_max) / (2 * s_max) * n_s
        fp = phi / np.pi * n_phi
        fz = (z + z_max) / (2 * z_max) * n_z
        if not (0 <= fs < n_s and 0 <= fz < n_z):
            continue
        out[int(fz), min(int(fp), n_phi - 1), int(fs)] += 1
    return out


def test_sinogram_matches_list_mode(scene_positron, data_dir, gpet_lib):
    ctx = make_ctx(scene_positron, data_dir, seed=77, n_decays=3000000, coinc_policy=1)
    ctx.run()
    singles, _ = ctx.singles()
    pairs, klass = ctx.coincidences()
    assert len(pairs) > 500
    panels = ctx.panels()
    for classes in ((0, 1, 2), (0,)):
        got = ctx.sinogram(64, 48, 4, 6.0, 3.2, classes)
        want = _sinogram_ref(singles, pairs, klass, panels, 64, 48, 4, 6.0, 3.2, classes)
        assert got.sum() > 0.8 * np.isin(klass, classes).sum()
        assert np.abs(got.astype(np.int64) - want).sum() <= 2   # atan2 of two libraries at a bin edge
    # the source is a cylinder of radius 3 cm: true lines of response have |s| <~ 3 cm
    t = ctx.sinogram(64, 48, 1, 6.0, 3.2, (0,)).sum(axis=(0, 1))
    assert t[16:48].sum() > 0.9 * t.sum()


def test_cli_writes_the_library_records(scene_positron, data_dir, gpet_lib, tmp_path):
    """`gpet input_PET.in key=value ...` (the drop-in for `./gPET
    input_PET.in`) writes the same records as the library API on the same
    scene and options: adder, singles and coincidence files byte for byte,
    hits as the same multiset (their order across photons is not defined)."""
    import subprocess
    from gpet_gb300 import build as B
    cli = os.path.join(B.OUT, "gpet")
    assert os.path.exists(cli)
    opts = dict(scene_positron.options, seed=4242, n_decays=30000)
    args = ["%s=%s" % (k, v) for k, v in opts.items()] + ["data_dir=" + data_dir, "base_dir=" + scene_positron.directory,
                                                          "out_dir=" + str(tmp_path / "cli")]
    r = subprocess.run([cli, scene_positron.config_path] + args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "coincidences" in r.stdout
    ctx = make_ctx(scene_positron, data_dir, seed=4242, n_decays=30000)
    ctx.run()
    ctx.write_outputs(str(tmp_path / "lib"))
    for name in ("adder.dat", "singles.dat", "coincidences.dat", "coincidences_class.dat"):
        a = (tmp_path / "cli" / name).read_bytes()
        b = (tmp_path / "lib" / name).read_bytes()
        assert a == b, name
    assert os.path.getsize(tmp_path / "cli" / "singles.dat") % 48 == 0
    assert os.path.getsize(tmp_path / "cli" / "singles.dat") > 0

    def hits(d):
        ids = np.fromfile(d / "HitsID.dat", np.int32).reshape(-1, 5)
        f = np.fromfile(d / "Hits.dat", np.float32).reshape(-1, 5)
        rec = np.concatenate([ids.view(np.uint32), f.view(np.uint32)], axis=1)
        return rec[np.lexsort(rec.T[::-1])]
    assert np.array_equal(hits(tmp_path / "cli"), hits(tmp_path / "lib"))


def test_phantom_majorant_bounds_every_material(scene_positron, data_dir, gpet_lib):
    """The Woodcock majorant (quirk Q1 fixed): node i holds 1 / the largest
    mu rho_max over [E_(i-1), E_(i+1)] of the interpolated tables, so on every
    energy the kernels can meet, the interpolated majorant times every
    material's interpolated mu at its largest density stays <= 1 (a real
    interaction probability never exceeds 1, prob never goes below 0)."""
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_positron, data_dir)
    tab, e0, ide = ctx.majorant(0)
    T = F.read_tables(data_dir)
    cfg = F.read_config(scene_positron.config_path)
    mat, den = F.read_phantom(cfg.matfile, cfg.denfile, tuple(cfg.pdim))
    f32 = np.float32
    E = np.linspace(T.eminph, T.emax * 0.9999, 200001).astype(f32)

    def lerp(t, x):
        x = np.clip(x, f32(0), f32(len(t) - 1))
        i = np.minimum(x.astype(np.int64), len(t) - 2)
        fr = (x - i.astype(f32)).astype(f32)
        return (t[i] + fr * (t[i + 1] - t[i])).astype(f32)

    lam = lerp(tab.astype(f32), (f32(ide) * (E - f32(e0))).astype(f32))
    idle = f32((len(T.energy) - 1) / (float(T.energy[-1]) - float(T.energy[0])))
    xe = (idle * (E - f32(T.energy[0]))).astype(f32)
    worst = 0.0
    for m in np.unique(mat):
        rho = f32(den[mat == m].max())
        mu = lerp(np.asarray(T.lamph[m], f32), xe)
        worst = max(worst, float((lam.astype(np.float64) * float(rho) * mu.astype(np.float64)).max()))
    assert worst <= 1.0 + 1e-5
    assert worst > 0.9                                # and it is tight where the densest material dominates


def test_singles_into_pinned_memory_match_the_copy(scene_positron, data_dir, gpet_lib):
    """gpet_get_singles writes straight into pinned buffers (the gather kernel's
    own stores); the records and flags equal those of the staged copy into
    pageable memory, also for an unaligned pinned buffer (the copy path) and
    without flags."""
    import torch
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_positron, data_dir, seed=91, n_decays=2000000)
    ctx.run()
    ev0, sc0 = ctx.singles()
    n = len(ev0)
    assert n > 1000

    def pinned(nbytes):
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()

    for shift in (0, 8):
        raw_ev = pinned(n * 48 + 64)
        raw_sc = pinned(n + 64)
        base = (-raw_ev.ctypes.data) % 16 + shift
        ev_buf = raw_ev[base:base + n * 48].view(F.EVENT_DTYPE)
        sc_buf = raw_sc[:n]
        ev_buf[:] = np.zeros(1, F.EVENT_DTYPE)
        sc_buf[:] = 7
        ev, sc = ctx.singles(out=(ev_buf, sc_buf))
        assert ev.tobytes() == ev0.tobytes(), shift
        assert np.array_equal(sc, sc0), shift
    # pinned records without flags
    raw_ev = pinned(n * 48 + 64)
    base = (-raw_ev.ctypes.data) % 16
    ev_buf = raw_ev[base:base + n * 48].view(F.EVENT_DTYPE)
    m = ctypes.c_int64()
    assert ctx.L.gpet_get_singles(ctx.h, ev_buf.ctypes.data, None, n, ctypes.byref(m)) == 0
    assert m.value == n and ev_buf.tobytes() == ev0.tobytes()


def test_async_copies_equal_the_synchronous_calls(scene_positron, scene_small, data_dir, gpet_lib):
    """gpet_get_singles_async / gpet_get_coincidences_async: the records of a
    run reach pinned buffers while the next run (larger, so the staging
    buffers grow under a pending copy) proceeds, and equal what the
    synchronous calls give for that run; in a batched job each simulation's
    pairs index its own singles."""
    import torch
    from gpet_gb300 import api, formats as F

    def pinned(n, dtype, shape=None):
        nb = int(np.prod(shape or (n,))) * np.dtype(dtype).itemsize
        return torch.empty(nb, dtype=torch.uint8, pin_memory=True).numpy().view(dtype).reshape(shape or (n,))

    ref = make_ctx(scene_positron, data_dir, seed=31, n_decays=1500000)
    ref.run()
    want_a = (ref.singles(), ref.coincidences())
    ref.close()
    ctx = make_ctx(scene_positron, data_dir, seed=31, n_decays=1500000)
    ctx.run()
    cap = 4 * len(want_a[0][0]) + 1024
    outs = [((pinned(cap, F.EVENT_DTYPE), pinned(cap, np.uint8)),
             (pinned(cap, np.int64, (cap, 2)), pinned(cap, np.uint8))) for _ in range(2)]
    s_a = ctx.singles_async(outs[0][0])
    c_a = ctx.coincidences_async(outs[0][1])
    ctx.set_options({"seed": 32, "n_decays": 3000000})
    ctx.run()                                   # overlaps the copies above
    s_b = ctx.singles_async(outs[1][0])
    c_b = ctx.coincidences_async(outs[1][1])
    ctx.wait_copies()
    assert len(s_b[0]) > len(s_a[0]) > 1000 and len(c_a[0]) > 100
    for got, want in zip(s_a + c_a, want_a[0] + want_a[1]):
        assert got.tobytes() == want.tobytes()
    for got, want in zip(s_b + c_b, ctx.singles() + ctx.coincidences()):
        assert got.tobytes() == want.tobytes()
    ctx.close()
    # batched: the second simulation's pairs are rebased onto its own singles
    ctxs = [make_ctx(scene_small, data_dir, seed=41 + i, n_decays=20000) for i in range(2)]
    api.run_batched(ctxs)
    for c in ctxs:
        o = ((pinned(cap, F.EVENT_DTYPE), pinned(cap, np.uint8)), (pinned(cap, np.int64, (cap, 2)), pinned(cap, np.uint8)))
        s = c.singles_async(o[0])
        p = c.coincidences_async(o[1])
        c.wait_copies()
        for got, want in zip(s + p, c.singles() + c.coincidences()):
            assert got.tobytes() == want.tobytes()
        assert len(p[0]) == 0 or p[0].max() < len(s[0])
        c.close()
