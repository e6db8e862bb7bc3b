"""GPU transport vs the double-precision oracle: statistical equivalence on
independent realizations (different Philox seeds) of the same workload:
singles energy spectrum, per-crystal singles, coincidence classes and the
scatter fraction (chi-square p > 0.01, totals within 3 sigma)."""
import numpy as np
import pytest

from conftest import make_ctx, oracle_for, two_sample_chi2, within_sigma

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def runs(tmp_path_factory, data_dir, gpet_lib, oracle_mod):
    from gpet_gb300 import scenes
    d = tmp_path_factory.mktemp("stat")
    sc = scenes.positron(str(d), n_decays=3_000_000, nvox=64)
    ctx = make_ctx(sc, data_dir, seed=101)
    st = ctx.run()
    gs, _ = ctx.singles()
    gp, gc = ctx.coincidences()
    r = oracle_for(sc, data_dir, seed=202).run(precision="fp64")
    return st, gs, gc, r


def test_energy_spectrum(runs):
    st, gs, gc, r = runs
    edges = np.linspace(350e3, 650e3, 61)
    a, _ = np.histogram(gs["E"], edges)
    b, _ = np.histogram(r["singles"]["E"], edges)
    assert two_sample_chi2(a, b) > 0.01
    assert within_sigma(len(gs), r["n_singles"])


def test_per_crystal_singles(runs):
    st, gs, gc, r = runs
    key = lambda s: s["pann"] * 64 + s["cryn"]
    a = np.bincount(key(gs), minlength=512)
    b = np.bincount(key(r["singles"]), minlength=512)
    assert two_sample_chi2(a, b) > 0.01


def test_coincidence_classes_and_scatter_fraction(runs):
    st, gs, gc, r = runs
    assert within_sigma(st["n_true"], r["n_true"])
    assert within_sigma(st["n_scatter"], r["n_scatter"])
    assert within_sigma(st["n_random"], r["n_random"])
    a = np.bincount(gc, minlength=3)
    b = np.bincount(r["coinc_class"], minlength=3)
    assert two_sample_chi2(a, b) > 0.01
    sfa = st["n_scatter"] / max(st["n_true"] + st["n_scatter"], 1)
    sfb = r["n_scatter"] / max(r["n_true"] + r["n_scatter"], 1)
    n = st["n_true"] + st["n_scatter"]
    assert abs(sfa - sfb) < 3 * np.sqrt(2 * sfa * (1 - sfa) / max(n, 1)) + 1e-3


def test_intermediate_counts(runs):
    st, gs, gc, r = runs
    for k in ("n_pairs", "n_entered", "n_pulses", "n_threshold", "n_deadtime"):
        assert within_sigma(st[k], r[k]), (k, st[k], r[k])
