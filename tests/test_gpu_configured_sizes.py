"""The workloads at the sizes they are configured at, against the oracle.

small: 1e6 back-to-back 511 keV pairs from a point at the origin, 200^3
voxels over a 1 cm cube (water cylinder r = 0.4 cm in air), eight LYSO panels
of 8 x 8 crystals (1.5 x 1.5 x 10 mm) at 4 cm: the whole acquisition bit for
bit against the FP32 oracle (every photon's phantom exit state, pulses,
singles, coincidences), and an independent GPU realisation against the FP64
oracle (singles spectrum, per-crystal singles, coincidence classes, scatter
fraction; chi-square p > 0.01, totals within 3 sigma).

positron: F-18 in a 3 cm cylinder with positron range, the 128^3 x 0.5 mm
water/bone/lung phantom, the 8-panel ring at 8 cm, paralyzable dead time
0.3 us per block; 1e7 decays on the GPU and 1e7 on the FP64 oracle with
independent seeds, compared the same way.

These cover gPET_kernals.cu:256-345 (phantom transport), :347-604 (source,
positron range), :839-1279 (detector transport, adder, readout) and the
digitizer (:607-837) at the geometries the workloads name."""
import numpy as np
import pytest

from conftest import make_ctx, oracle_for, two_sample_chi2, within_sigma

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_full(tmp_path_factory, data_dir):
    from gpet_gb300 import scenes
    return scenes.small(str(tmp_path_factory.mktemp("small_full")))   # 1e6 decays, 200^3


@pytest.fixture(scope="module")
def positron_1e7(tmp_path_factory, data_dir):
    from gpet_gb300 import scenes
    return scenes.positron(str(tmp_path_factory.mktemp("positron_1e7")), n_decays=10_000_000)   # 128^3


def _first_diff(a, b, fields):
    for f in fields:
        bad = np.nonzero(a[f] != b[f])[0]
        if len(bad):
            i = bad[0]
            return "%s differs at %d (of %d): gpu %r oracle %r" % (f, i, len(bad), a[f][i], b[f][i])
    return None


def test_small_full_size_bit_exact(small_full, data_dir, gpet_lib, oracle_mod):
    ctx = make_ctx(small_full, data_dir, record_exits=1)
    st = ctx.run()
    assert st["n_decays"] == 1_000_000
    r = oracle_for(small_full, data_dir, panels=ctx.panels()).run(precision="fp32", exits=True)
    gx, ox = ctx.exits(), r["exits"]
    assert len(gx) == len(ox) == 2_000_000
    msg = _first_diff(gx, ox, ["status", "panel", "nscat", "E", "x", "y", "z", "ux", "uy", "uz", "t"])
    assert msg is None, msg
    gp, gsc, gsl = ctx.pulses()
    assert st["n_pulses"] == r["n_pulses"] == len(gp)
    assert np.array_equal(gp.view(np.uint8), r["pulses"].view(np.uint8))
    gs, gss = ctx.singles()
    assert st["n_singles"] == r["n_singles"] == len(gs) > 10000
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8)), _first_diff(
        gs, r["singles"], ["parn", "pann", "modn", "cryn", "siten", "eventid", "t", "E", "x", "y", "z"])
    assert np.array_equal(gss, r["single_scat"])
    pr, cl = ctx.coincidences()
    assert st["n_coinc"] == r["n_coinc"] == len(pr) > 1000
    assert np.array_equal(pr, r["coinc"]) and np.array_equal(cl, r["coinc_class"])


def _statistical(scene, data_dir, ncry):
    ctx = make_ctx(scene, data_dir, seed=1101)
    st = ctx.run()
    gs, _ = ctx.singles()
    gp, gc = ctx.coincidences()
    r = oracle_for(scene, data_dir, seed=2202).run(precision="fp64")
    # singles spectrum over the energy window, 5 keV bins
    edges = np.linspace(350e3, 650e3, 61)
    a, _ = np.histogram(gs["E"], edges)
    b, _ = np.histogram(r["singles"]["E"], edges)
    assert two_sample_chi2(a, b) > 0.01
    assert within_sigma(len(gs), r["n_singles"])
    # per-crystal singles over the ring
    key = lambda s: s["pann"] * ncry + s["cryn"]
    a = np.bincount(key(gs), minlength=8 * ncry)
    b = np.bincount(key(r["singles"]), minlength=8 * ncry)
    assert two_sample_chi2(a, b) > 0.01
    # coincidence classes and the scatter fraction
    for k in ("n_true", "n_scatter", "n_random"):
        assert within_sigma(st[k], r[k]), (k, st[k], r[k])
    a = np.bincount(gc, minlength=3)
    b = np.bincount(r["coinc_class"], minlength=3)
    assert two_sample_chi2(a, b) > 0.01
    sfa = st["n_scatter"] / max(st["n_true"] + st["n_scatter"], 1)
    sfb = r["n_scatter"] / max(r["n_true"] + r["n_scatter"], 1)
    n = st["n_true"] + st["n_scatter"]
    assert abs(sfa - sfb) < 3 * np.sqrt(2 * sfa * (1 - sfa) / max(n, 1)) + 1e-3
    for k in ("n_pairs", "n_entered", "n_pulses", "n_threshold", "n_deadtime", "n_singles", "n_coinc"):
        assert within_sigma(st[k], r[k]), (k, st[k], r[k])
    return st, r


def test_small_full_size_against_fp64_oracle(small_full, data_dir, gpet_lib, oracle_mod):
    st, r = _statistical(small_full, data_dir, 64)
    assert st["n_coinc"] > 3000 and r["n_coinc"] > 3000


def test_positron_128_1e7_against_fp64_oracle(positron_1e7, data_dir, gpet_lib, oracle_mod):
    st, r = _statistical(positron_1e7, data_dir, 64)
    assert st["n_decays"] == r["n_decays"] == 10_000_000
    assert st["n_singles"] > 300000 and st["n_coinc"] > 4000
    assert st["n_deadtime"] < st["n_threshold"]      # the paralyzable dead time removes pulses here
