"""Digitizer and coincidence sorter on the GPU vs the oracle on the same pulse
list: bit-exact, including the edge cases of gPET's digitizer (ties in t,
events exactly tau apart, site changes, empty input) and both dead-time
policies."""
import numpy as np
import pytest

from conftest import make_ctx, oracle_for
from gpet_gb300.formats import EVENT_DTYPE

pytestmark = pytest.mark.gpu


def synthetic_pulses(n, seed, npanels=8, moduleN=1, crystalN=64, t_span=1e5, ties=True):
    rng = np.random.default_rng(seed)
    ev = np.zeros(n, EVENT_DTYPE)
    ev["parn"] = rng.permutation(4 * n)[:n]
    ev["pann"] = rng.integers(0, npanels, n)
    ev["modn"] = rng.integers(0, moduleN, n)
    ev["cryn"] = rng.integers(0, crystalN, n)
    ev["siten"] = ev["pann"] * moduleN * crystalN + ev["modn"] * crystalN + ev["cryn"]
    ev["eventid"] = ev["parn"] // 2
    t = np.sort(rng.uniform(0, t_span, n))
    if ties and n > 10:
        k = rng.integers(1, n, n // 20)
        t[k] = t[k - 1]                              # exact ties
        k = rng.integers(1, n, n // 20)
        t[k] = t[k - 1] + 0.3                        # exactly tau apart (tau = 0.3 us)
        k = rng.integers(1, n, n // 20)
        t[k] = t[k - 1] + 0.004                      # exactly one coincidence window apart
    ev["t"] = rng.permutation(t)
    ev["E"] = rng.uniform(100e3, 700e3, n).astype(np.float32)
    ev["x"] = rng.uniform(-1, 0, n); ev["y"] = rng.uniform(-1, 1, n); ev["z"] = rng.uniform(-1, 1, n)
    scat = (rng.random(n) < 0.3).astype(np.uint8)
    slot = rng.integers(0, 3, n).astype(np.uint8)
    return ev, scat, slot


def _check(ctx, o, ev, scat, slot):
    st = ctx.digitize(ev, scat, slot)
    r = o.digitize(ev, scat, slot, precision="fp32")
    assert st["n_threshold"] == r["n_threshold"]
    assert st["n_deadtime"] == r["n_deadtime"]
    gs, gsc = ctx.singles()
    assert len(gs) == r["n_singles"]
    assert np.array_equal(gs.view(np.uint8), r["singles"].view(np.uint8))
    assert np.array_equal(gsc, r["single_scat"])
    pr, cl = ctx.coincidences()
    assert np.array_equal(pr, r["coinc"]) and np.array_equal(cl, r["coinc_class"])
    assert st["n_multiple"] == r["n_multiple"]
    return st


@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("policy", [0, 1])
@pytest.mark.parametrize("n", [0, 1, 2, 1000, 200000])
def test_digitizer_bit_exact(scene_positron, data_dir, gpet_lib, oracle_mod, tmp_path, n, dtype, policy):
    from gpet_gb300 import formats as F
    cfg = F.read_config(scene_positron.config_path)
    cfg.dtype = dtype
    cfg.dtime = 0.3
    cfg.dlevel = 3 if n % 2 else 2
    path = tmp_path / "input_PET.in"
    F.write_config(str(path), cfg)
    import copy
    sc = copy.copy(scene_positron)
    sc.config_path = str(path)
    ctx = make_ctx(sc, data_dir, coinc_policy=policy)
    o = oracle_for(sc, data_dir, coinc_policy=policy)
    ev, scat, slot = synthetic_pulses(n, seed=n + 7 * dtype + 3 * policy, t_span=max(1.0, n * 0.05))
    st = _check(ctx, o, ev, scat, slot)
    if n >= 1000:
        assert st["n_deadtime"] < st["n_threshold"]          # dead time did something
        assert st["n_coinc"] > 0


def test_digitizer_twice_same_context(scene_small, data_dir, gpet_lib, oracle_mod):
    ctx = make_ctx(scene_small, data_dir)
    o = oracle_for(scene_small, data_dir)
    for seed in (1, 2):
        ev, scat, slot = synthetic_pulses(5000, seed)
        _check(ctx, o, ev, scat, slot)


@pytest.mark.parametrize("n", [0, 5000])
def test_digitizer_with_background_singles(scene_positron, data_dir, gpet_lib, oracle_mod, tmp_path, n):
    """addnoise (gPET_kernals.cu:699-735): a Poisson stream of background
    singles joins the pulses before the digitizer; bit-exact against the
    oracle, never classed as the same decay."""
    from gpet_gb300 import formats as F
    cfg = F.read_config(scene_positron.config_path)
    cfg.tstart, cfg.tend = 0.0, 0.5
    path = tmp_path / "input_PET.in"
    F.write_config(str(path), cfg)
    import copy
    sc = copy.copy(scene_positron)
    sc.config_path = str(path)
    opts = dict(noise_lambda_us=20.0, noise_emean_ev=450000.0, noise_sigma_ev=60000.0, noise_interval_us=500.0,
                coinc_policy=1)
    ctx = make_ctx(sc, data_dir, **opts)
    o = oracle_for(sc, data_dir, **opts)
    ev, scat, slot = synthetic_pulses(n, seed=11, t_span=5e5)
    st = _check(ctx, o, ev, scat, slot)
    r = o.digitize(ev, scat, slot, precision="fp32")
    assert st["n_noise"] == r["n_noise"]
    mean = 5e5 / 20.0
    assert abs(st["n_noise"] - mean) < 5 * np.sqrt(mean)
    gs, _ = ctx.singles()
    noise = gs["parn"] == -1
    assert noise.sum() > 0 and (gs["eventid"][noise] == -1).all()
    pr, cl = ctx.coincidences()
    with_noise = noise[pr[:, 0]] | noise[pr[:, 1]]
    assert with_noise.any() and (cl[with_noise] == 2).all()


@pytest.mark.parametrize("case", ["one_instant", "ulp_apart_wide_span", "negative_times"])
def test_time_order_keys_edge_cases(scene_positron, data_dir, gpet_lib, oracle_mod, case):
    """The time order sorts 32-bit keys of (t - t_min) over the survivors'
    time span and puts runs of equal keys in (t, parn, slot) order: pulses
    at one instant (zero span: the IEEE bits of t are the keys), pulses a few
    ulps apart within a span of 1e12 us (many share a quantised key), and
    negative times; singles and coincidences bit for bit against the oracle."""
    ctx = make_ctx(scene_positron, data_dir)
    o = oracle_for(scene_positron, data_dir)
    n = 4000
    ev, scat, slot = synthetic_pulses(n, seed=99, ties=False)
    rng = np.random.default_rng(5)
    if case == "one_instant":
        ev["t"] = 1234.5
    elif case == "ulp_apart_wide_span":
        base = rng.uniform(0, 1e12, n // 8)
        t = np.repeat(base, 8)
        t = t + np.tile(np.arange(8), n // 8) * np.spacing(t)       # 8 times a few ulps apart
        ev["t"] = rng.permutation(t)
    else:
        ev["t"] = rng.uniform(-50.0, 50.0, n)
    _check(ctx, o, ev, scat, slot)
