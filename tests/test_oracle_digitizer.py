"""The oracle's digitizer and coincidence sorter on hand-built pulse lists with
answers worked out by hand from the reference's semantics (deadtime,
gPET_kernals.cu:657-698; energywindow :641-656; the coincidence policy)."""
import numpy as np
import pytest

from conftest import oracle_for
from gpet_gb300.formats import EVENT_DTYPE


def pulses(rows):
    """rows: (parn, pann, eventid, t, E[, scat])"""
    ev = np.zeros(len(rows), EVENT_DTYPE)
    scat = np.zeros(len(rows), np.uint8)
    for i, r in enumerate(rows):
        ev[i]["parn"], ev[i]["pann"], ev[i]["eventid"], ev[i]["t"], ev[i]["E"] = r[:5]
        ev[i]["siten"] = r[1] * 64
        scat[i] = r[5] if len(r) > 5 else 0
    return ev, scat, np.zeros(len(rows), np.uint8)


@pytest.fixture
def oracle_nodigiblur(scene_small, data_dir, tmp_path, oracle_mod):
    from gpet_gb300 import formats as F
    import copy

    def make(dlevel=1, dtype=0, dtime=1.0, policy=0, window_ns=4.0):
        cfg = F.read_config(scene_small.config_path)
        cfg.blurpolicy, cfg.rref, cfg.eslope, cfg.sblur = 1, 0.0, 0.0, 0.0   # no blur
        cfg.eth, cfg.ewin_lo, cfg.ewin_hi = 100e3, 350e3, 650e3
        cfg.dlevel, cfg.dtype, cfg.dtime = dlevel, dtype, dtime
        p = tmp_path / ("c%d%d%d.in" % (dlevel, dtype, policy))
        F.write_config(str(p), cfg)
        sc = copy.copy(scene_small)
        sc.config_path = str(p)
        return oracle_for(sc, data_dir, coinc_policy=policy, coinc_window_ns=window_ns)
    return make


def test_deadtime_paralyzable_vs_not(oracle_nodigiblur):
    # one site (panel 0), events at 0, 0.5, 1.2, 2.5, 3.0 us, tau = 1 us
    rows = [(2 * i, 0, i, t, 500e3) for i, t in enumerate([0.0, 0.5, 1.2, 2.5, 3.0])]
    ev, sc, sl = pulses(rows)
    # paralyzable: each event extends the dead period -> 0 kept, 0.5 lost (0.5<1),
    # 1.2 lost (1.2<1.5), 2.5 kept (2.5>=2.2), 3.0 lost (3.0<3.5)
    r = oracle_nodigiblur(dtype=0).digitize(ev, sc, sl)
    assert list(r["singles"]["t"]) == [0.0, 2.5]
    # non-paralyzable: dead until last survivor + tau -> 0, 1.2, 2.5 kept
    r = oracle_nodigiblur(dtype=1).digitize(ev, sc, sl)
    assert list(r["singles"]["t"]) == [0.0, 1.2, 2.5]


def test_deadtime_exactly_tau_apart_survives(oracle_nodigiblur):
    rows = [(0, 0, 0, 10.0, 500e3), (2, 0, 1, 11.0, 500e3)]      # t2 = t1 + tau exactly
    r = oracle_nodigiblur(dtype=0).digitize(*pulses(rows))
    assert r["n_deadtime"] == 2


def test_deadtime_is_per_site(oracle_nodigiblur):
    rows = [(0, 0, 0, 10.0, 500e3), (2, 1, 1, 10.1, 500e3)]       # different panels
    r = oracle_nodigiblur(dlevel=1).digitize(*pulses(rows))
    assert r["n_deadtime"] == 2
    r = oracle_nodigiblur(dlevel=0).digitize(*pulses(rows))        # one site for the world
    assert r["n_deadtime"] == 1


def test_threshold_and_window(oracle_nodigiblur):
    rows = [(0, 0, 0, 1.0, 99e3), (2, 1, 1, 5.0, 200e3), (4, 2, 2, 9.0, 650e3), (6, 3, 3, 13.0, 651e3)]
    r = oracle_nodigiblur(dtime=0.0).digitize(*pulses(rows))
    assert r["n_threshold"] == 3          # 99 keV below the 100 keV threshold
    assert list(r["singles"]["t"]) == [9.0]   # 650 keV is inside [350, 650]


def test_coincidence_policy_and_classes(oracle_nodigiblur):
    W = 0.004
    rows = [
        (0, 0, 7, 100.0, 500e3), (1, 4, 7, 100.0 + W / 2, 500e3),            # true pair
        (2, 1, 8, 200.0, 500e3), (3, 5, 8, 200.001, 500e3, 1),               # scatter (one scattered)
        (4, 2, 9, 300.0, 500e3), (6, 6, 10, 300.002, 500e3),                 # random
        (8, 3, 11, 400.0, 500e3), (10, 7, 12, 400.001, 500e3), (12, 1, 13, 400.002, 500e3),   # triple
        (14, 0, 14, 500.0, 500e3), (15, 0, 14, 500.001, 500e3),              # same panel
        (16, 2, 15, 600.0, 500e3), (18, 3, 16, 600.0 + W, 500e3),            # exactly W apart: no
    ]
    r = oracle_nodigiblur(dlevel=0, dtime=0.0).digitize(*pulses(rows))
    s = r["singles"]
    pairs = [(int(s["parn"][a]), int(s["parn"][b])) for a, b in r["coinc"]]
    assert pairs == [(0, 1), (2, 3), (4, 6)]
    assert list(r["coinc_class"]) == [0, 1, 2]
    assert r["n_multiple"] == 1
    r = oracle_nodigiblur(dlevel=0, dtime=0.0, policy=1).digitize(*pulses(rows))
    s = r["singles"]
    pairs = [(int(s["parn"][a]), int(s["parn"][b])) for a, b in r["coinc"]]
    assert pairs == [(0, 1), (2, 3), (4, 6), (8, 10), (8, 12), (10, 12)]


def test_empty_and_single(oracle_nodigiblur):
    o = oracle_nodigiblur()
    r = o.digitize(*pulses([]))
    assert r["n_singles"] == 0 and r["n_coinc"] == 0
    r = o.digitize(*pulses([(0, 0, 0, 1.0, 500e3)]))
    assert r["n_singles"] == 1 and r["n_coinc"] == 0


def test_ties_in_t_are_ordered_by_parn(oracle_nodigiblur):
    rows = [(8, 0, 0, 5.0, 500e3), (2, 1, 1, 5.0, 500e3), (4, 2, 2, 5.0, 500e3)]
    r = oracle_nodigiblur(dtime=0.0).digitize(*pulses(rows))
    assert list(r["singles"]["parn"]) == [2, 4, 8]


def test_fp32_and_fp64_oracles_agree_statistically(scene_positron, data_dir, oracle_mod):
    o = oracle_for(scene_positron, data_dir)
    a = o.run(precision="fp64")
    b = o.run(precision="fp32")
    for k in ("n_pairs", "n_entered", "n_pulses", "n_singles", "n_coinc"):
        sa, sb = a[k], b[k]
        assert abs(sa - sb) <= 4 * np.sqrt(max(sa, 1)) + 2, (k, sa, sb)


def test_background_singles_statistics(oracle_mod, scene_small, data_dir):
    """The oracle's background stream: Poisson count, Gaussian energy, uniform
    crystals, times inside the window."""
    from conftest import oracle_for
    from gpet_gb300.formats import EVENT_DTYPE
    o = oracle_for(scene_small, data_dir, noise_lambda_us=50.0, noise_emean_ev=400000.0, noise_sigma_ev=50000.0,
                   noise_interval_us=800.0, coinc_policy=1)
    o.s.ewin_lo, o.s.ewin_hi, o.s.Eth, o.s.dtime_us = 0.0, 2.0e6, 0.0, 0.0
    o.s.noise_t1_us = 2.0e6
    r = o.digitize(np.zeros(0, EVENT_DTYPE), np.zeros(0, np.uint8), np.zeros(0, np.uint8), precision="fp64")
    mean = 2.0e6 / 50.0
    assert abs(r["n_noise"] - mean) < 5 * np.sqrt(mean)
    s = r["singles"]
    assert len(s) == r["n_noise"]
    assert abs(s["E"].mean() - 400000.0) < 5 * 50000.0 / np.sqrt(len(s))
    assert abs(s["E"].std() - 50000.0) < 0.05 * 50000.0
    assert (s["t"] >= 0).all() and (s["t"] < 2.0e6).all() and (np.diff(s["t"]) >= 0).all()
    counts = np.bincount(s["cryn"], minlength=64)
    exp = len(s) / 64.0
    chi2 = ((counts - exp) ** 2 / exp).sum()
    assert chi2 < 63 + 5 * np.sqrt(2 * 63)
    assert (s["parn"] == -1).all() and (s["eventid"] == -1).all()
    assert (r["coinc_class"] == 2).all()
