"""GPU path vs the single-precision CPU oracle, history by history.

The CUDA kernels and the oracle's FP32 build perform the same IEEE operations
in the same order on the same Philox streams, so every photon's phantom exit
state, every hit, every pulse, every single and every coincidence must agree
bit for bit. Sizes are ones the oracle finishes in about a second."""
import os

import numpy as np
import pytest

from conftest import event_key_sort, make_ctx, oracle_for

pytestmark = pytest.mark.gpu


def _first_diff(a, b, fields):
    for f in fields:
        bad = np.nonzero(a[f] != b[f])[0]
        if len(bad):
            i = bad[0]
            return "%s differs at %d (of %d): gpu %r oracle %r" % (f, i, len(bad), a[f][i], b[f][i])
    return None


def _run_both(scene, data_dir, **extra):
    ctx = make_ctx(scene, data_dir, record_exits=1, **extra)
    st = ctx.run()
    o = oracle_for(scene, data_dir, panels=ctx.panels(), **extra)
    r = o.run(precision="fp32", exits=True, hits=True)
    return ctx, st, r


@pytest.mark.parametrize("which", ["small", "positron", "large"])
def test_histories_bit_exact(which, scene_small, scene_positron, scene_large, data_dir, gpet_lib, oracle_mod):
    scene = {"small": scene_small, "positron": scene_positron, "large": scene_large}[which]
    ctx, st, r = _run_both(scene, data_dir)
    gx = ctx.exits()
    ox = r["exits"]
    assert len(gx) == len(ox) == 2 * st["n_decays"]
    msg = _first_diff(gx, ox, ["status", "panel", "nscat", "E", "x", "y", "z", "ux", "uy", "uz", "t"])
    assert msg is None, msg
    assert st["n_pairs"] == r["n_pairs"]
    assert st["n_entered"] == r["n_entered"]
    # pulses after adder + readout
    gp, gsc, gsl = ctx.pulses()
    assert st["n_pulses"] == r["n_pulses"] == len(gp)
    op, osl = r["pulses"], r["pulse_slot"]
    assert np.array_equal(gp.view(np.uint8), op.view(np.uint8)), _first_diff(
        gp, op, ["parn", "pann", "modn", "cryn", "siten", "eventid", "t", "E", "x", "y", "z"])
    assert np.array_equal(gsl, osl) and np.array_equal(gsc, r["pulse_scat"])
    # hits: same multiset (order across photons is not defined on the GPU)
    gid, gf = ctx.hits()
    assert len(gid) == r["n_hits"]
    def canon(ids, f):
        rec = np.concatenate([ids.view(np.uint32), f.view(np.uint32)], axis=1)
        return rec[np.lexsort(rec.T[::-1])]
    assert np.array_equal(canon(gid, gf), canon(r["hit_id"], r["hit_f"]))


@pytest.mark.parametrize("which", ["small", "positron", "large"])
def test_singles_and_coincidences_bit_exact(which, scene_small, scene_positron, scene_large, data_dir, gpet_lib, oracle_mod):
    scene = {"small": scene_small, "positron": scene_positron, "large": scene_large}[which]
    ctx, st, r = _run_both(scene, data_dir)
    gs, gsc = ctx.singles()
    assert st["n_threshold"] == r["n_threshold"]
    assert st["n_deadtime"] == r["n_deadtime"]
    assert st["n_singles"] == r["n_singles"] == len(gs)
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8)), _first_diff(
        gs, r["singles"], ["parn", "pann", "modn", "cryn", "siten", "eventid", "t", "E", "x", "y", "z"])
    assert np.array_equal(gsc, r["single_scat"])
    pr, cl = ctx.coincidences()
    assert st["n_coinc"] == r["n_coinc"] == len(pr)
    assert np.array_equal(pr, r["coinc"])
    assert np.array_equal(cl, r["coinc_class"])
    assert (st["n_true"], st["n_scatter"], st["n_random"], st["n_multiple"]) == (
        r["n_true"], r["n_scatter"], r["n_random"], r["n_multiple"])
    assert st["n_coinc"] > 0


def _sphere_distance(x, u, sph):
    """getDistance (gPET_kernals.cu:148-171) in float32, the reference's root choice."""
    f = np.float32
    cx, cy, cz = f(x[0] - sph[0]), f(x[1] - sph[1]), f(x[2] - sph[2])
    a = f(f(u[0] * u[0]) + f(u[1] * u[1])) + f(u[2] * u[2])
    b = f(2.0) * (f(f(u[0] * cx) + f(u[1] * cy)) + f(u[2] * cz))
    c = (f(f(cx * cx) + f(cy * cy)) + f(cz * cz)) - f(sph[3]) * f(sph[3])
    disc = f(b * b) - f(f(4.0) * a) * c
    if disc < 0:
        return f(0.0)
    r = np.sqrt(disc, dtype=np.float32)
    if c < 0:
        return f((-b + r) / (f(2.0) * a))
    if b < 0:
        return f((-b - r) / (f(2.0) * a))
    return f((-b + r) / (f(2.0) * a))


@pytest.mark.parametrize("which", ["small", "positron"])
def test_phase_space_records_bit_exact(which, scene_small, scene_positron, data_dir, gpet_lib, oracle_mod, tmp_path):
    """Source and phantom phase space (OUTPUTPSF 1/2) against the FP32 oracle."""
    from gpet_gb300 import formats as F
    scene = scene_small if which == "small" else scene_positron
    ctx = make_ctx(scene, data_dir, record_exits=1, record_source=1)
    st = ctx.run()
    o = oracle_for(scene, data_dir, panels=ctx.panels())
    r = o.run(precision="fp32", exits=True, source=True)
    src = ctx.source_records()
    osrc = r["source"][r["source"]["t"] > 0]
    assert len(src) == len(osrc) > 0
    assert np.array_equal(src.view(np.uint8), osrc.view(np.uint8))
    assert len(src) == 2 * st["n_pairs"] or which == "small"
    ph = ctx.phantom_records()
    ex = r["exits"]
    keep = (ex["status"] == 1) & (ex["t"] > 0)
    assert len(ph) == keep.sum()
    for k in ("x", "y", "z", "ux", "uy", "uz", "E", "t"):
        assert np.array_equal(ph[k], ex[k][keep]), k
    assert np.array_equal(ph["eventid"], np.nonzero(keep)[0] // 2)
    # the files, in the reference's layouts
    ctx.write_outputs(str(tmp_path))
    back = F.read_phase_space(str(tmp_path), "source")
    assert len(back) == len(src) and np.array_equal(back["E"], src["E"]) and np.array_equal(back["t"], src["t"])
    assert (tmp_path / "outphantom.dat").stat().st_size == 28 * len(ph)
    assert (tmp_path / "idphantom.dat").stat().st_size == 4 * len(ph)
    assert (tmp_path / "timephantom.dat").stat().st_size == 8 * len(ph)


def test_phantom_records_on_record_sphere(scene_small, data_dir, gpet_lib):
    """psf_sphere=1: exit photons moved along their direction onto the record
    sphere of input_PET.in (getDistance)."""
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_small, data_dir, record_exits=1)
    ctx.run()
    plain = ctx.phantom_records()
    ctx.set_option("psf_sphere", 1)
    proj = ctx.phantom_records()
    sph = np.array(F.read_config(scene_small.config_path).recordsphere, np.float32)
    assert len(proj) == len(plain) > 100
    on = 0
    for a, b in zip(plain[:500], proj[:500]):
        x = np.array([a["x"], a["y"], a["z"]], np.float32)
        u = np.array([a["ux"], a["uy"], a["uz"]], np.float32)
        d = _sphere_distance(x, u, sph)
        want = x + d * u
        assert np.allclose([b["x"], b["y"], b["z"]], want, rtol=1e-6, atol=1e-6)
        assert abs(b["t"] - (a["t"] + float(d) / 29979.2458)) < 1e-9
        if d > 0:
            on += 1
            assert abs(np.linalg.norm(want - sph[:3]) - sph[3]) < 1e-4
    assert on > 100


def test_quadric_exclusion_bit_exact(scene_small, data_dir, gpet_lib, oracle_mod, tmp_path):
    """crystalSearch's quadratic surfaces (gPET_kernals.cu:1241-1249): a
    cylinder of radius 0.35 cm around each panel's local x axis counts as gap
    material; histories, pulses and singles must still match the oracle."""
    from gpet_gb300 import formats as F
    from gpet_gb300.scenes import Scene
    cfg = F.read_config(scene_small.config_path)
    cfg.surfaces = [[0, 1, 1, 0, 0, 0, 0, 0, 0, -0.35 ** 2]]
    path = str(tmp_path / "input_PET.in")
    F.write_config(path, cfg)
    scene = Scene(scene_small.directory, path, dict(scene_small.options), "quadric")
    ctx, st, r = _run_both(scene, data_dir)
    gx, ox = ctx.exits(), r["exits"]
    assert _first_diff(gx, ox, ["status", "panel", "nscat", "E", "x", "y", "z", "t"]) is None
    gp, gsc, gsl = ctx.pulses()
    assert np.array_equal(gp.view(np.uint8), r["pulses"].view(np.uint8))
    gs, _ = ctx.singles()
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    # the excluded cylinder holds no deposit
    gid, gf = ctx.hits()
    assert len(gid) > 0
    assert (gf[:, 3] ** 2 + gf[:, 4] ** 2 >= 0.35 ** 2 - 1e-6).all()
    # and it changed something against the unexcluded detector
    ref = make_ctx(scene_small, data_dir)
    assert ref.run()["n_hits"] != st["n_hits"]


def test_run_with_background_singles_bit_exact(scene_small, data_dir, gpet_lib, oracle_mod):
    opts = dict(noise_lambda_us=2000.0, noise_emean_ev=480000.0, noise_sigma_ev=40000.0, noise_interval_us=1000.0)
    ctx, st, r = _run_both(scene_small, data_dir, **opts)
    assert st["n_noise"] == r["n_noise"] > 0
    gs, gsc = ctx.singles()
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    pr, cl = ctx.coincidences()
    assert np.array_equal(pr, r["coinc"]) and np.array_equal(cl, r["coinc_class"])
    # adder.dat content: the transport's pulses only
    gp, _, _ = ctx.pulses()
    assert (gp["parn"] >= 0).all() and len(gp) == r["n_pulses"]


def test_multi_material_detector_bit_exact(scene_small, data_dir, gpet_lib, oracle_mod, tmp_path):
    """A third detector material: the back half of every crystal (depth
    beyond 0.5 cm, marked by the plane x + 0.5 < 0 in panel coordinates) is
    LSO (material 9, 7.4 g/cm3) instead of LYSO; both materials collect
    deposits. Histories, hits, pulses and singles bit for bit against the
    oracle."""
    from gpet_gb300 import formats as F
    from gpet_gb300.scenes import Scene, ring_panel0, MAT_LYSO, MAT_AIR
    geo = str(tmp_path / "ring3.geo")
    F.write_geo(geo, 8, (0, 0, 1), 45.0, (MAT_LYSO, MAT_AIR, 9), (7.1, 0.001025, 7.4),
                ring_panel0(4.0, 8, 8, 0.15, 0.001, 1.0))
    g = F.read_geo(geo)
    assert g.det_mat == (MAT_LYSO, MAT_AIR, 9)
    cfg = F.read_config(scene_small.config_path)
    cfg.geofile = geo
    cfg.surfaces = [[0, 0, 0, 0, 0, 0, 1, 0, 0, 0.5]]
    path = str(tmp_path / "input_PET.in")
    F.write_config(path, cfg)
    scene = Scene(scene_small.directory, path, dict(scene_small.options), "three materials")
    ctx, st, r = _run_both(scene, data_dir)
    gx, ox = ctx.exits(), r["exits"]
    assert _first_diff(gx, ox, ["status", "panel", "nscat", "E", "x", "y", "z", "t"]) is None
    gp, _, _ = ctx.pulses()
    assert np.array_equal(gp.view(np.uint8), r["pulses"].view(np.uint8))
    gs, _ = ctx.singles()
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    gid, gf = ctx.hits()
    back = gf[:, 2] < -0.5
    assert back.any() and (~back).any()        # deposits in both materials
    # the same surface without a third material is an exclusion zone instead
    cfg2 = F.read_config(scene_small.config_path)
    cfg2.surfaces = cfg.surfaces
    p2 = str(tmp_path / "input2.in")
    F.write_config(p2, cfg2)
    ctx2 = make_ctx(Scene(scene_small.directory, p2, dict(scene_small.options), "excluded"), data_dir)
    ctx2.run()
    _, gf2 = ctx2.hits()
    assert (gf2[:, 2] >= -0.5 - 1e-6).all()


@pytest.mark.parametrize("which", ["positron", "large"])
def test_voxel_pairs_bit_exact(which, scene_positron, scene_large, data_dir, gpet_lib, oracle_mod):
    """The phantom stored as 8-byte (density, material) pairs instead of the
    default palette form (16-bit indices into the distinct pairs): histories,
    singles and coincidences bit for bit against the oracle."""
    scene = scene_positron if which == "positron" else scene_large
    ctx = make_ctx(scene, data_dir, record_exits=1, voxel_palette=0)
    st = ctx.run()
    r = oracle_for(scene, data_dir, panels=ctx.panels()).run(precision="fp32", exits=True, hits=True)
    msg = _first_diff(ctx.exits(), r["exits"], ["status", "panel", "nscat", "E", "x", "y", "z", "ux", "uy", "uz", "t"])
    assert msg is None, msg
    gs, _ = ctx.singles()
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    pr, cl = ctx.coincidences()
    assert np.array_equal(pr, r["coinc"]) and np.array_equal(cl, r["coinc_class"])


def test_voxel_palette_falls_back_to_pairs(scene_positron, data_dir, gpet_lib):
    """More distinct (density, material) pairs than the palette holds: the
    phantom is stored as pairs and the run equals the one without a palette."""
    from gpet_gb300 import formats as F
    cfg = F.read_config(scene_positron.config_path)
    d = scene_positron.directory
    mat, den = F.read_phantom(os.path.join(d, "phantom_mat.dat"), os.path.join(d, "phantom_den.dat"),
                              tuple(cfg.pdim))
    rng = np.random.default_rng(11)
    den = (den * rng.uniform(0.98, 1.02, den.shape)).astype(np.float32)   # ~110k distinct values
    assert len(np.unique(den)) > 70000
    out = []
    for pal in (1, 0):   # 1 falls back to pairs here
        ctx = make_ctx(scene_positron, data_dir, voxel_palette=pal)
        ctx.set_phantom(mat, den, cfg.pdim, cfg.poffset, cfg.psize)
        st = ctx.run()
        out.append((st["n_singles"], st["n_coinc"], ctx.singles()[0].tobytes(), ctx.coincidences()[0].tobytes()))
    assert out[0] == out[1] and out[0][1] > 0


@pytest.mark.parametrize("n", [0, 1, 7])
def test_tiny_runs_bit_exact(n, scene_positron, data_dir, gpet_lib, oracle_mod):
    """No decays, one decay, a handful: histories and singles against the
    oracle, and empty results read back as empty arrays."""
    ctx, st, r = _run_both(scene_positron, data_dir, n_decays=n)
    assert st["n_decays"] == n
    gx = ctx.exits()
    assert len(gx) == len(r["exits"]) == 2 * n
    if n:
        msg = _first_diff(gx, r["exits"], ["status", "panel", "nscat", "E", "x", "y", "z", "ux", "uy", "uz", "t"])
        assert msg is None, msg
    gs, gsc = ctx.singles()
    assert len(gs) == r["n_singles"]
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    pr, cl = ctx.coincidences()
    assert len(pr) == r["n_coinc"]


@pytest.mark.parametrize("ptype,prange", [(0, 1), (0, 0), (1, 0)])
def test_phase_space_source_bit_exact(ptype, prange, scene_positron, data_dir, gpet_lib, oracle_mod, tmp_path):
    """A phase-space file as the source (initialize.cu:76-115; setPosition-
    ForPhoton, gPET_kernals.cu:563-604): positron records (ptype 0, with and
    without positron range: each makes a pair, the second photon with its
    time set) and photon records (ptype 1: one photon each, records with
    t <= 0 dropped); histories, singles and coincidences against the oracle."""
    import copy
    from gpet_gb300 import formats as F
    rng = np.random.default_rng(21 + 3 * ptype + prange)
    n = 20000
    rec = np.zeros((n, 8))
    rec[:, 0:3] = rng.uniform(-1.0, 1.0, (n, 3))
    rec[:, 3] = rng.uniform(0.0, 1.0e6, n)
    if ptype == 1:
        rec[::50, 3] = 0.0                           # dropped by the reference's t > 0 test
    u = rng.standard_normal((n, 3))
    rec[:, 4:7] = u / np.linalg.norm(u, axis=1, keepdims=True)
    rec[:, 7] = rng.uniform(1.0e5, 6.0e5, n) if ptype == 0 else rng.choice([511.0e3, 350.0e3], n)
    psf_path = tmp_path / "psf.dat"
    rec.tofile(psf_path)
    cfg = F.read_config(scene_positron.config_path)
    cfg.usepsf, cfg.sourcefile, cfg.ptype, cfg.useprange, cfg.nparticle = 1, str(psf_path), ptype, prange, n
    path = tmp_path / "input_PET.in"
    F.write_config(str(path), cfg)
    sc = copy.copy(scene_positron)
    sc.config_path = str(path)
    ctx, st, r = _run_both(sc, data_dir)
    assert st["n_decays"] == n
    gx = ctx.exits()
    assert len(gx) == len(r["exits"]) == 2 * n
    msg = _first_diff(gx, r["exits"], ["status", "panel", "nscat", "E", "x", "y", "z", "ux", "uy", "uz", "t"])
    assert msg is None, msg
    if ptype == 1:
        assert (gx["status"][1::2] == 2).all()        # no second photon
        assert (gx["status"][0::2][::50] == 2).all()  # t = 0 records emit nothing
    gs, _ = ctx.singles()
    assert len(gs) == r["n_singles"] > 0
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    pr, cl = ctx.coincidences()
    assert np.array_equal(pr, r["coinc"]) and np.array_equal(cl, r["coinc_class"])
    if prange:
        # the same records through gpet_set_source_psf on a context loaded
        # with its decay source: the same run
        api_ctx = make_ctx(scene_positron, data_dir, record_exits=1)
        api_ctx.set_source_psf(rec, ptype)
        api_ctx.run()
        assert np.array_equal(api_ctx.singles()[0].view(np.uint8), gs.view(np.uint8))
