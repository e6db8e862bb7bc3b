"""Pins of the CPU oracle against known answers: Random123's Philox vectors,
the random streams seeded from them, the reference's own data files (tables
at 511 keV, isotope spectra, the example detector), and the physics the
samplers must reproduce."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

KAT = json.load(open(os.path.join(GOLDEN, "kat.json")))


def test_philox_random123_vectors(oracle_mod):
    ph = oracle_mod.philox
    assert ph([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert ph([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert ph([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def _xoshiro128ss(state, n):
    # xoshiro128** (Blackman & Vigna), restated from the paper in Python
    s = list(state)
    rotl = lambda x, k: ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF
    out = []
    for _ in range(n):
        out.append(rotl((s[1] * 5) & 0xFFFFFFFF, 7) * 9 & 0xFFFFFFFF)
        t = (s[1] << 9) & 0xFFFFFFFF
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = rotl(s[3], 11)
    return out


def test_stream_is_xoshiro_from_a_philox_block(oracle_mod):
    """A stream's words: xoshiro128** from the Philox4x32-10 block of counter
    (0, tag, id) under the key. The generator's first words from state
    (1, 2, 3, 4) worked by hand: 11520, 0, 5927040."""
    assert _xoshiro128ss([1, 2, 3, 4], 3) == [11520, 0, 5927040]
    for key, tag, ident in (([0, 0], 0, 0), ([20261203, 7], 2, 123456789), ([0xFFFFFFFF, 1], 9, (5 << 32) + 17)):
        seed = oracle_mod.philox([0, tag, ident & 0xFFFFFFFF, ident >> 32], key)
        assert oracle_mod.stream_words(key, tag, ident, 64) == _xoshiro128ss(seed, 64)
    # streams of neighbouring ids and tags share no words
    a = oracle_mod.stream_words([1, 2], 2, 1000, 4096)
    b = oracle_mod.stream_words([1, 2], 2, 1001, 4096)
    c = oracle_mod.stream_words([1, 2], 3, 1000, 4096)
    assert not (set(a) & set(b)) and not (set(a) & set(c))
    # the top 24 bits (what a uniform uses) are uniform: chi-square over 256 bins
    w = np.array(oracle_mod.stream_words([3, 4], 1, 42, 1 << 18), np.uint32) >> 24
    h = np.bincount(w, minlength=256)
    chi2 = float(((h - h.mean()) ** 2 / h.mean()).sum())
    assert 150 < chi2 < 380


def test_uniforms_stay_inside_the_unit_interval(oracle_mod):
    """Every word gives (k + 1/2) 2^-23 from its top 23 bits, exactly, never 0
    or 1 (a uniform of 1 made a Box-Muller normal exactly 0, and the
    positron-range walk's reciprocal of that displacement component a NaN
    position)."""
    L = oracle_mod.lib("fp32")
    L.oracle_u01.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
    w = np.concatenate([np.arange(0, 1 << 12, dtype=np.uint64), (1 << 32) - 1 - np.arange(1 << 12, dtype=np.uint64),
                        np.random.default_rng(3).integers(0, 1 << 32, 1 << 16, dtype=np.uint64)]).astype(np.uint32)
    u = np.zeros(len(w), np.float32)
    L.oracle_u01(len(w), w.ctypes.data, u.ctypes.data)
    assert u.min() == np.float32(2.0 ** -24) and u.max() == np.float32(1 - 2.0 ** -24)
    assert np.array_equal(u.astype(np.float64), ((w >> 9).astype(np.float64) + 0.5) * 2.0 ** -23)


def _dm(oracle_mod, which, x):
    L = oracle_mod.lib("fp32")
    L.oracle_detmath.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p]
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x)
    L.oracle_detmath(which, len(x), x.ctypes.data, y.ctypes.data)
    return y


def test_detmath_accuracy(oracle_mod):
    u = ((np.arange(1 << 20, dtype=np.float64) * 16 + 0.5) * 2.0 ** -24).astype(np.float32)
    rel = lambda a, b: np.max(np.abs(a.astype(np.float64) - b) / np.maximum(np.abs(b), 1e-30))
    assert rel(_dm(oracle_mod, 0, u), np.log(u.astype(np.float64))) < 4e-7
    xs = np.linspace(-80, 80, 100001).astype(np.float32)
    assert rel(_dm(oracle_mod, 1, xs), np.exp(xs.astype(np.float64))) < 2e-7
    tw = 2 * np.pi * u.astype(np.float64)
    assert np.max(np.abs(_dm(oracle_mod, 2, u) - np.sin(tw))) < 2e-7
    assert np.max(np.abs(_dm(oracle_mod, 3, u) - np.cos(tw))) < 2e-7
    assert rel(_dm(oracle_mod, 4, u), np.cbrt(u.astype(np.float64))) < 2e-7
    L = oracle_mod.lib("fp32")
    L.oracle_detmath_log.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
    xd = np.random.default_rng(0).random(100000) + 1e-300
    yd = np.zeros_like(xd)
    L.oracle_detmath_log(len(xd), xd.ctypes.data, yd.ctypes.data)
    assert np.max(np.abs(yd - np.log(xd)) / np.abs(np.log(xd))) < 1e-15


def test_tables_511keV(data_dir):
    from gpet_gb300 import formats as F
    T = F.read_tables(data_dir)
    for m, name in enumerate(T.names):
        k = KAT["mu_rho_511keV"][name]
        tot = np.interp(511e3, T.energy, T.lamph[m])
        assert tot == pytest.approx(k["total"], rel=1e-6)
        parts = sum(np.interp(511e3, T.energy, t[m]) for t in (T.compt, T.phote, T.rayle))
        assert parts == pytest.approx(tot, rel=1e-4)
    # pins quoted for the PET materials (cm^2/g)
    expect = {"Water": 0.09596, "LYSO": 0.11476, "LSO": 0.11676, "CorticalBone": 0.09047, "DryAir": 0.08630}
    for n, v in expect.items():
        assert KAT["mu_rho_511keV"][n]["total"] == pytest.approx(v, abs=6e-6)


def test_surfaces_shape_and_monotone(data_dir):
    from gpet_gb300 import formats as F
    T = F.read_tables(data_dir)
    for s in (T.cmpsf, T.rayff):
        assert s.shape == (10, 301, 151)
        assert np.all(np.diff(s, axis=1) >= -1e-6)          # cos rises with probability
        assert np.all(s[:, 0, :] == -1) and np.all(s[:, -1, :] == 1)
    # Rayleigh at 511 keV is forward peaked; Compton in water has mean cos ~0.3-0.4
    assert np.mean(T.rayff[1, :, 77]) > 0.9
    assert 0.25 < np.mean(T.cmpsf[1, :, 77]) < 0.5


def test_positron_spectrum_mean(oracle_mod, data_dir):
    from gpet_gb300 import formats as F
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    L = oracle_mod.lib("fp64")
    L.oracle_sample_ek.argtypes = [C.c_void_p, C.c_uint64, C.c_int64, C.c_void_p]
    for row in range(len(iso.halftime)):
        cf = np.ascontiguousarray(iso.coef[row], np.float32)
        out = np.zeros(200000)
        L.oracle_sample_ek(cf.ctypes.data, 7 + row, len(out), out.ctypes.data)
        mean = out.mean() / 1e6
        se = out.std() / 1e6 / np.sqrt(len(out))
        assert abs(mean - KAT["positron_mean_kinetic_MeV"][row]) < 4 * se + 1e-4
        assert out.min() >= 0 and out.max() <= (cf[0] - 0.511) * 1e6 + 1
    # F-18: the fitted spectrum's mean kinetic energy (0.276 MeV; the tabulated
    # F-18 mean is 0.25 MeV, the fit is what the reference samples)
    assert KAT["positron_mean_kinetic_MeV"][0] == pytest.approx(0.2756, abs=2e-3)


def test_positron_sampler_matches_reference_density(oracle_mod, data_dir):
    """The positron kinetic energies follow the reference's density
    min(polynomial, nmax) on [0.511, emax] MeV (its rejection against nmax,
    gPET_kernals.cu:420-443; for F-18 the fitted polynomial peaks slightly
    above nmax, so the top is clipped): chi-square of 400k draws."""
    from scipy import stats
    from gpet_gb300 import formats as F
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    L = oracle_mod.lib("fp64")
    L.oracle_sample_ek.argtypes = [C.c_void_p, C.c_uint64, C.c_int64, C.c_void_p]
    for row in range(len(iso.halftime)):
        cf32 = np.ascontiguousarray(iso.coef[row], np.float32)
        cf = cf32.astype(np.float64)
        emax, nmax = cf[0], cf[1]
        E = np.linspace(0.511, emax, 100001)
        target = np.clip(np.minimum(sum(cf[2 + i] * E ** (5 - i) for i in range(6)), nmax), 0.0, None)
        out = np.zeros(400000)
        L.oracle_sample_ek(cf32.ctypes.data, 99 + row, len(out), out.ctypes.data)
        edges = np.linspace(0.511, emax, 51)
        h, _ = np.histogram(out / 1e6 + 0.511, bins=edges)
        cdf = np.concatenate([[0.0], np.cumsum((target[1:] + target[:-1]) * 0.5 * np.diff(E))])
        p = np.diff(np.interp(edges, E, cdf))
        exp = p / p.sum() * len(out)
        keep = exp > 20
        chi2 = float((((h[keep] - exp[keep]) ** 2) / exp[keep]).sum())
        assert stats.chi2.sf(chi2, int(keep.sum()) - 1) > 1e-3, (row, chi2, int(keep.sum()))


@pytest.mark.parametrize("energy", [511e3, 300e3, 100e3])
def test_klein_nishina_chi2(oracle_mod, energy):
    from scipy import stats
    L = oracle_mod.lib("fp64")
    L.oracle_kn_sample.argtypes = [C.c_double, C.c_uint64, C.c_int64, C.c_void_p, C.c_void_p]
    n = 400000
    cost = np.zeros(n)
    ef = np.zeros(n)
    L.oracle_kn_sample(energy, 11, n, cost.ctypes.data, ef.ctypes.data)
    k = energy / 510999.1
    edges = np.linspace(-1, 1, 41)
    mu = np.linspace(-1, 1, 200001)
    r = 1 / (1 + k * (1 - mu))
    pdf = r * r * (r + 1 / r - (1 - mu * mu))
    cdf = np.concatenate([[0], np.cumsum((pdf[1:] + pdf[:-1]) / 2 * np.diff(mu))])
    cdf /= cdf[-1]
    expct = np.diff(np.interp(edges, mu, cdf)) * n
    obs, _ = np.histogram(cost, edges)
    chi2 = np.sum((obs - expct) ** 2 / expct)
    assert stats.chi2.sf(chi2, len(obs) - 1) > 1e-3
    # Compton kinematics: efrac = 1/(1 + k(1-cos))
    assert np.allclose(ef, 1 / (1 + k * (1 - cost)), rtol=1e-9, atol=1e-9)


def test_noncollinearity_sigma(oracle_mod):
    L = oracle_mod.lib("fp64")
    L.oracle_pair_angles.argtypes = [C.c_float, C.c_uint64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    n = 200000
    ang, e0, e1 = np.zeros(n), np.zeros(n), np.zeros(n)
    sigma = 0.0037056
    L.oracle_pair_angles(sigma, 5, n, ang.ctypes.data, e0.ctypes.data, e1.ctypes.data)
    dev = np.pi - ang                       # |theta|, theta ~ N(0, sigma)
    assert np.sqrt(np.mean(dev ** 2)) == pytest.approx(sigma, rel=0.01)
    # the reference's energy shift: E = MC2 +- theta*MC2/2 (sum is 2 MC2)
    assert np.allclose(e0 + e1, 2 * 510999.1, rtol=1e-12)
    assert np.std(e0) == pytest.approx(sigma * 510999.1 / 2, rel=0.02)


def test_geometry_counts_config8():
    from gpet_gb300 import formats as F
    g = F.read_geo(os.path.join(GOLDEN, "reference_inputs", "config8.geo"))
    assert g.counts == (9, 117, 8, 64)
    assert g.counts == tuple(KAT["config8_counts"][k] for k in ("moduleNy", "moduleN", "crystalNy", "crystalN"))
    assert np.allclose(g.panels[1], KAT["config8_panel1"], atol=1e-5)
    # panel 1 is panel 0 turned by 45 degrees about z
    assert np.allclose(g.panels[1][15:18], [15.909903, -15.909903, 0], atol=1e-4)


def test_event_record_layout():
    from gpet_gb300.formats import EVENT_DTYPE
    assert EVENT_DTYPE.itemsize == KAT["event_record"]["size"]
    assert EVENT_DTYPE.fields["t"][1] == KAT["event_record"]["t_offset"]
    assert EVENT_DTYPE.fields["E"][1] == KAT["event_record"]["E_offset"]


def test_example_config_parses():
    from gpet_gb300 import formats as F
    c = F.read_config(os.path.join(GOLDEN, "reference_inputs", "input_PET.in"))
    k = KAT["config"]
    assert list(c.pdim) == k["pdim"] == [200, 200, 200]
    assert c.rdepth == 2 and c.rpolicy == 1
    assert (c.dlevel, c.dtype) == (3, 0) and c.dtime == pytest.approx(2.2)
    assert (c.ewin_lo, c.ewin_hi) == (30000.0, 700000.0)
    assert c.surfaces == [[0, 0, 0, 0, 0, 0, 0, 0, 0, 1]]
    assert c.geofile == "input/config8.geo" and c.sourcefile == "input/pointsource.txt"


def test_detmath_double_helpers(oracle_mod):
    """The decay-time series and the 52-bit uniform of detmath.h."""
    L = oracle_mod.lib("fp32")
    L.oracle_detmath_d.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p]
    x = -np.linspace(1e-12, 2.0 ** -6, 200001)
    y = np.zeros_like(x)
    L.oracle_detmath_d(0, len(x), x.ctypes.data, y.ctypes.data)
    assert np.max(np.abs(y - np.log1p(x)) / np.abs(np.log1p(x))) < 8 * 2.0 ** -53
    # (hi, lo) as hi * 2^32 + lo; the top 12 bits of hi are not used
    hl = np.array([0, 1, 0xFFFFF00000000, 0xFFFFFFFFFFFFF, 0x123456789ABCD, 0x7FF0000000000000], np.float64)
    u = np.zeros_like(hl)
    L.oracle_detmath_d(1, len(hl), hl.ctypes.data, u.ctypes.data)
    k = np.array([0, 1, 0xFFFFF00000000, 0xFFFFFFFFFFFFF, 0x123456789ABCD, 0], np.float64)
    assert np.array_equal(u, (k + 0.5) * 2.0 ** -52)
    assert u.min() > 0 and u.max() < 1
