"""The learned detector response of the whole-body ring against plain Monte
Carlo, on the GPU.

The whole-body ring has 48 LYSO panels of 16 x 16 crystals (4 x 4 x 20 mm) at
49 cm, more crystals than one softmax of the fused head holds, so its model
(data/surrogate_wholebody_ring.npz, made by data/make_surrogate.py --ring
wholebody with the library's own training kernels) predicts each energy
class's crystal as a row and a column. It replaces photonde
(gPET_kernals.cu:839-1233) for photons in its domain. Two bed positions of
the whole-body acquisition (the 256 x 256 x 512 x 2 mm body shifted by
-3.2 and +3.2 cm), with and without it, on independent seeds:
  - singles per crystal (256, pooled over panels): every crystal within 2 %
    at 3e8 decays per bed and arm;
  - singles energy spectrum 350-650 keV and the crystal map: chi-square
    p > 0.01 at 1.5e7 decays per bed and arm;
  - singles, coincidences, true / scatter / random: within 3 sigma there.
"""
import os

import numpy as np
import pytest

from conftest import two_sample_chi2, within_sigma

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODEL = os.path.join(ROOT, "data", "surrogate_wholebody_ring.npz")
BEDS = (3, 4)


@pytest.fixture(scope="module")
def beds(tmp_path_factory, data_dir, gpet_lib):
    from gpet_gb300 import api, formats as F, scenes
    d = str(tmp_path_factory.mktemp("wholebody"))
    bl = scenes.large_beds(d)
    cfg = F.read_config(bl[0].config_path)
    mat, den = F.read_phantom(cfg.matfile, cfg.denfile, tuple(cfg.pdim))
    ctxs = []
    for k in BEDS:
        b = bl[k]
        c = api.Context(0)
        c.set_options(dict(b.options, data_dir=data_dir, base_dir=d))
        c.load_config(b.config_path)
        c.set_phantom(mat, den, b.dims, b.offset, b.size)
        c.set_source_file(b.source_path, 0.0, 120.0)
        ctxs.append(c)
    sur = api.Surrogate(ctxs[0], seed=1)
    meta = sur.load(MODEL)
    yield ctxs, sur, meta
    for c in ctxs:
        c.close()
    sur.close()


def _acquire(ctxs, sur, decays, seed):
    tot = {"E": [], "cry": []}
    st_sum = {}
    for i, c in enumerate(ctxs):
        c.set_options({"n_decays": decays, "seed": seed + 17 * i})
        c.set_surrogate(sur)
        st = c.run()
        s, _ = c.singles()
        tot["E"].append(np.asarray(s["E"], np.float64))
        tot["cry"].append(np.asarray(s["cryn"], np.int64))
        for k, v in st.items():
            st_sum[k] = st_sum.get(k, 0) + v
        c.set_surrogate(None)
    return {"E": np.concatenate(tot["E"]), "cry": np.concatenate(tot["cry"]), "st": st_sum}


@pytest.fixture(scope="module")
def arms(beds):
    ctxs, sur, _ = beds
    return {"mc": _acquire(ctxs, None, 300_000_000, 101), "sur": _acquire(ctxs, sur, 300_000_000, 202),
            "mc_small": _acquire(ctxs, None, 15_000_000, 303), "sur_small": _acquire(ctxs, sur, 15_000_000, 404)}


def test_model_is_factorised_for_the_ring(beds):
    ctxs, sur, meta = beds
    assert ctxs[0].counts() == (1, 1, 16, 256)
    assert meta["train_records"] > 1e7 and meta["calibration_records"] > 1e6
    assert meta["loss_per_epoch"][-1] < meta["loss_per_epoch"][0]


def test_per_crystal_singles_within_two_percent(arms):
    a = np.bincount(arms["mc"]["cry"], minlength=256)[:256].astype(np.float64)
    b = np.bincount(arms["sur"]["cry"], minlength=256)[:256].astype(np.float64)
    assert a.min() > 3e4
    rel = (b / b.sum()) / (a / a.sum()) - 1.0
    worst = int(np.argmax(np.abs(rel)))
    assert np.abs(rel).max() < 0.02, (worst, rel[worst], np.round(100 * rel, 2).tolist())


def test_spectrum_and_crystal_map_chi2(arms):
    mc, su = arms["mc_small"], arms["sur_small"]
    ea = np.histogram(mc["E"], bins=60, range=(3.5e5, 6.5e5))[0]
    eb = np.histogram(su["E"], bins=60, range=(3.5e5, 6.5e5))[0]
    assert two_sample_chi2(ea, eb) > 0.01
    a = np.bincount(mc["cry"], minlength=256)[:256]
    b = np.bincount(su["cry"], minlength=256)[:256]
    assert two_sample_chi2(a, b) > 0.01


def test_counts_within_three_sigma(arms):
    a, b = arms["mc_small"]["st"], arms["sur_small"]["st"]
    for k in ("n_singles", "n_coinc", "n_true", "n_scatter", "n_random"):
        assert within_sigma(a[k], b[k]), (k, a[k], b[k])
    s = arms["sur"]["st"]
    assert s["n_surrogate"] > 0.4 * s["n_entered"]
