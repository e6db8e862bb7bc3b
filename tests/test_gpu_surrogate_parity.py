"""The learned detector response against plain Monte Carlo, on the GPU.

The committed model (data/surrogate_positron_ring.npz, made by
data/make_surrogate.py with the library's own training kernels) replaces the
detector transport of photonde (gPET_kernals.cu:839-1233, with crystalSearch
:1236-1279 and adder/readout :737-813) for photons in its domain. Independent
acquisitions of the positron workload (F-18 cylinder, 128^3 water/bone/lung
phantom, 8-panel LYSO ring) with and without it must agree:
  - singles energy spectrum 350-650 keV: chi-square p > 0.01;
  - singles per crystal (the 64 crystals of a panel, pooled over panels):
    every crystal within 2 % at 2.3e8 decays per arm (about 1e7 singles,
    0.36 % statistical error per crystal), and chi-square p > 0.01 at about
    1e6 singles per arm;
  - singles, coincidences and their true / scatter / random classes: totals
    within 3 sigma.
What the trained network gains over the method without it: more than half
of the photons entering a panel skip the detector transport (the Monte
Carlo's detector Woodcock steps fall accordingly) with the observables above
at parity, while a network of the same shape that was never trained, given
the same domain and calibration, misses the energy spectrum."""
import os

import numpy as np
import pytest

from conftest import make_ctx, two_sample_chi2, within_sigma

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODEL = os.path.join(ROOT, "data", "surrogate_positron_ring.npz")
DECAYS = 230_000_000
DECAYS_SMALL = 23_000_000


@pytest.fixture(scope="module")
def positron128(tmp_path_factory, data_dir):
    from gpet_gb300 import scenes
    return scenes.positron(str(tmp_path_factory.mktemp("sur_parity")), n_decays=DECAYS)


def _acquire(scene, data_dir, seed, decays, sur=None):
    ctx = make_ctx(scene, data_dir, seed=seed, n_decays=decays)
    if sur is not None:
        ctx.set_surrogate(sur)
    st = ctx.run()
    s, _ = ctx.singles()
    out = {"st": st, "E": np.asarray(s["E"], np.float64), "cry": np.asarray(s["cryn"], np.int64)}
    ctx.set_surrogate(None)
    ctx.close()
    return out


@pytest.fixture(scope="module")
def model(positron128, data_dir, gpet_lib):
    from gpet_gb300 import api
    ctx = make_ctx(positron128, data_dir, n_decays=1000)
    sur = api.Surrogate(ctx, seed=1)
    meta = sur.load(MODEL)
    return sur, meta, ctx


@pytest.fixture(scope="module")
def arms(positron128, data_dir, model):
    sur = model[0]
    return {"mc": _acquire(positron128, data_dir, 101, DECAYS),
            "sur": _acquire(positron128, data_dir, 202, DECAYS, sur),
            "mc_small": _acquire(positron128, data_dir, 303, DECAYS_SMALL),
            "sur_small": _acquire(positron128, data_dir, 404, DECAYS_SMALL, sur)}


def _spectrum(E):
    return np.histogram(E, bins=60, range=(3.5e5, 6.5e5))[0]


def test_model_file_loads_with_its_domain(model):
    sur, meta, _ = model
    assert meta["train_records"] > 1e7 and meta["calibration_records"] > 1e7
    assert len(meta["loss_per_epoch"]) == meta["train"]["epochs"]
    assert meta["loss_per_epoch"][-1] < meta["loss_per_epoch"][0]


def test_energy_spectrum_at_parity(arms):
    mc, su = arms["mc"], arms["sur"]
    assert two_sample_chi2(_spectrum(mc["E"]), _spectrum(su["E"])) > 0.01
    assert within_sigma(len(mc["E"]), len(su["E"]))


def test_per_crystal_singles_within_two_percent(arms):
    mc, su = arms["mc"], arms["sur"]
    a = np.bincount(mc["cry"], minlength=64)[:64].astype(np.float64)
    b = np.bincount(su["cry"], minlength=64)[:64].astype(np.float64)
    assert a.sum() > 9e6 and b.sum() > 9e6
    rel = (b / b.sum()) / (a / a.sum()) - 1.0
    assert np.abs(rel).max() < 0.02, np.round(100 * rel, 2)


def test_per_crystal_chi2_at_1e6_singles(arms):
    mc, su = arms["mc_small"], arms["sur_small"]
    a = np.bincount(mc["cry"], minlength=64)[:64]
    b = np.bincount(su["cry"], minlength=64)[:64]
    assert a.sum() > 9e5 and b.sum() > 9e5
    assert two_sample_chi2(a, b) > 0.01


def test_coincidence_classes_within_three_sigma(arms):
    a, b = arms["mc"]["st"], arms["sur"]["st"]
    for k in ("n_singles", "n_coinc", "n_true", "n_scatter", "n_random"):
        assert within_sigma(a[k], b[k]), (k, a[k], b[k])


def test_what_the_trained_network_gains(positron128, data_dir, model, arms):
    """Work avoided at parity, against the plain Monte Carlo; accuracy,
    against a network of the same shape that was never trained."""
    from gpet_gb300 import api
    a, b = arms["mc"]["st"], arms["sur"]["st"]
    assert b["n_entered"] == pytest.approx(a["n_entered"], rel=0.01)
    assert b["n_surrogate"] > 0.5 * b["n_entered"]
    assert b["detector_steps"] < 0.6 * a["detector_steps"]
    # the same architecture, random weights, the same domain and calibration
    sur, meta, ctx = model
    gen = make_ctx(positron128, data_dir, seed=505, n_decays=20_000_000, record_entries=1)
    gen.run()
    rec = gen.entries()
    gen.close()
    raw = api.Surrogate(ctx, seed=77)
    raw.set_domain(1.0e5, 5.2e5, 0.3)
    raw.calibrate(rec, iters=meta["calibration"]["passes"])
    un = _acquire(positron128, data_dir, 606, DECAYS_SMALL, raw)
    mc = arms["mc_small"]
    assert two_sample_chi2(_spectrum(mc["E"]), _spectrum(un["E"])) < 1e-6
    raw.close()
