"""Pins of the oracle against the reference's own code (TEST
INFRASTRUCTURE, used by tests/test_oracle_reference_pins.py and
tests/golden/make_ref_vectors.py).

The reference's functions, built for the CPU by ref_build.py
(oracle/_ref/libgpet_ref.so), and the oracle's tape-driven entry points
(oracle/build/liboracle_fp32_tape.so) are run on the same inputs with the
same random words. `reference_outputs` collects what the reference computes
(the golden vectors); `oracle_outputs` what the oracle computes; `compare`
measures their agreement.

The pin workload: a 24^3 phantom of 2.5 mm voxels (water body, bone rod,
lung sphere, air outside), the positron workload's 8-panel LYSO ring at 8 cm
and its digitizer; photons start inside the phantom.
"""
import ctypes as C
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
sys.path.insert(0, ROOT)
sys.path.insert(0, ORACLE)

from gpet_gb300 import formats as F, scenes  # noqa: E402

TAPE = 256            # words per photon or sample
N_PHANTOM = 2000      # photons through the phantom
N_DETECTOR = 2000     # photons toward the ring
N_SAMPLER = 1000      # samples of each sampler
SEED = 20261204

_FP = C.POINTER(C.c_float)
_DP = C.POINTER(C.c_double)
_UP = C.POINTER(C.c_uint32)
_IP = C.POINTER(C.c_int32)
_LP = C.POINTER(C.c_int64)


def _p(a, t):
    return a.ctypes.data_as(t)


# ------------------------------------------------------------------ the scene
def write_scene(directory):
    """The pin workload in gPET's file formats; returns the Scene."""
    os.makedirs(directory, exist_ok=True)
    n, size = 24, 6.0
    c = scenes._base_config(directory, (n, n, n), (size, size, size), (-size / 2,) * 3)
    c.useprange = 1
    c.dlevel, c.dtype, c.dtime = 2, 0, 0.3
    x = scenes._voxel_centres(n, size, -size / 2)
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    mat = np.full((n, n, n), scenes.MAT_AIR, np.int32)
    den = np.full((n, n, n), scenes.RHO_AIR, np.float32)
    body = np.broadcast_to(X ** 2 + Y ** 2 < 2.6 ** 2, (n, n, n))
    mat[body] = scenes.MAT_WATER
    den[body] = 1.0
    rod = np.broadcast_to((X - 1.2) ** 2 + Y ** 2 < 0.6 ** 2, (n, n, n))
    mat[rod] = scenes.MAT_BONE
    den[rod] = 1.85
    lung = (X + 1.0) ** 2 + (Y - 0.5) ** 2 + Z ** 2 < 1.0
    mat[lung] = scenes.MAT_TISSUE
    den[lung] = 0.3
    F.write_phantom(c.matfile, c.denfile, mat, den)
    F.write_geo(c.geofile, 8, (0, 0, 1), 45.0, (scenes.MAT_LYSO, scenes.MAT_AIR), (7.1, 0.001025),
                scenes.ring_panel0(8.0, 8, 8, 0.298, 0.002, 2.0))
    F.write_sources(c.sourcefile, [4_000_000_000], [0], [1], [(0, 0, 0, 2.0, 5.0, 0)])
    F.write_config(os.path.join(directory, "input_PET.in"), c)
    return scenes.Scene(directory, os.path.join(directory, "input_PET.in"),
                        {"n_decays": 1000, "seed": SEED, "coinc_window_ns": 4.0}, "pin workload")


def philox_words(seed, tag, n):
    """n 32-bit words of Philox4x32-10 (the published algorithm; key = the
    seed's two halves, counter = (block, tag, 0, 0)), vectorised: a portable,
    version-independent source for the pin inputs and random words."""
    M0, M1, W0, W1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57), np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
    nb = (n + 3) // 4
    c0 = np.arange(nb, dtype=np.uint64).astype(np.uint32)
    c1 = np.full(nb, tag, np.uint32)
    c2 = np.zeros(nb, np.uint32)
    c3 = np.zeros(nb, np.uint32)
    k0, k1 = np.uint32(seed & 0xFFFFFFFF), np.uint32((seed >> 32) & 0xFFFFFFFF)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = c0.astype(np.uint64) * M0
            p1 = c2.astype(np.uint64) * M1
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), p0.astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), p1.astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0, k1 = np.uint32(k0 + W0), np.uint32(k1 + W1)
    return np.stack([c0, c1, c2, c3], 1).reshape(-1)[:n]


class _Draws:
    """Uniforms and integers from a Philox stream (tag) of the seed."""

    def __init__(self, seed):
        self.seed, self.tag = seed, 0

    def words(self, n):
        self.tag += 1
        return philox_words(self.seed, self.tag, n)

    def uniform(self, lo, hi, shape):
        n = int(np.prod(shape))
        u = (self.words(n).astype(np.float64) + 0.5) / 4294967296.0
        return (lo + (hi - lo) * u).reshape(shape)

    def random(self, n):
        return self.uniform(0.0, 1.0, (n,))

    def integers(self, lo, hi, n):
        return (lo + self.words(n).astype(np.int64) % (hi - lo)).astype(np.int64)


def inputs(seed=SEED):
    """Inputs and random words of every pin, deterministic in seed."""
    rng = _Draws(seed)

    def iso(n):
        c = rng.uniform(-1, 1, (n,))
        ph = rng.uniform(0, 2 * np.pi, (n,))
        s = np.sqrt(1 - c * c)
        return np.stack([s * np.cos(ph), s * np.sin(ph), c], 1)

    def words(n):
        return rng.words(n * TAPE).reshape(n, TAPE)

    I = {}
    # photons inside the phantom, 511 keV and below
    n = N_PHANTOM
    pos = np.stack([rng.uniform(-2.4, 2.4, (n,)), rng.uniform(-2.4, 2.4, (n,)), rng.uniform(-2.7, 2.7, (n,))], 1)
    r = rng.random(n)
    E = np.where(r < 0.5, 510999.1, np.where(r < 0.8, rng.uniform(2e4, 1.2e5, (n,)), rng.uniform(1.2e5, 5.2e5, (n,))))
    I["ph_in"] = np.concatenate([pos, iso(n), E[:, None]], 1).astype(np.float32)
    I["ph_t"] = rng.uniform(1.0, 1e6, (n,))
    I["ph_tape"] = words(n)
    # photons heading out toward the ring from near the centre
    n = N_DETECTOR
    pos = rng.uniform(-1.5, 1.5, (n, 3))
    d = iso(n)
    d[:, 2] *= 0.3
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    E = np.where(rng.random(n) < 0.8, 510999.1, rng.uniform(1.5e5, 5.2e5, (n,)))
    I["de_in"] = np.concatenate([pos, d, E[:, None]], 1).astype(np.float32)
    I["de_t"] = rng.uniform(1.0, 1e6, (n,))
    I["de_tape"] = words(n)
    # samplers
    n = N_SAMPLER
    I["kn_e"] = rng.uniform(2e4, 6e5, (n,)).astype(np.float32)
    I["kn_tape"] = words(n)
    I["sf_e"] = rng.uniform(2e4, 6e5, (n,)).astype(np.float32)
    I["sf_m"] = rng.integers(0, 9, n).astype(np.int32)
    I["sf_tape"] = words(n)
    I["ek_tape"] = words(n)
    I["shape_kind"] = rng.integers(0, 3, n).astype(np.int32)
    I["shape_coef"] = np.concatenate([rng.uniform(-1, 1, (n, 3)), rng.uniform(0.1, 2.0, (n, 3))], 1).astype(np.float32)
    I["shape_tape"] = words(n)
    I["pr_x"] = np.stack([rng.uniform(-2.8, 2.8, (n,)), rng.uniform(-2.8, 2.8, (n,)), rng.uniform(-2.8, 2.8, (n,))],
                         1).astype(np.float32)
    I["pr_v"] = np.concatenate([iso(n), rng.uniform(1e4, 1.6e6, (n, 1))], 1).astype(np.float32)
    I["pr_usedir"] = rng.integers(0, 2, n).astype(np.int32)
    I["pr_tape"] = words(n)
    I["pair_useprange"] = rng.integers(0, 2, n).astype(np.int32)
    I["pair_tape"] = words(n)
    # crystal search: points of the panel's local frame, over and beyond the face
    I["cs_panel"] = rng.integers(0, 8, n).astype(np.int32)
    I["cs_x"] = np.stack([rng.uniform(0, 2.1, (n,)), rng.uniform(-1.3, 1.3, (n,)), rng.uniform(-1.3, 1.3, (n,))],
                         1).astype(np.float32)
    # adder and readout: 1-6 deposits of one photon over a few crystals
    m = 600
    dep = np.zeros((m, 6), F.EVENT_DTYPE)
    ndep = rng.integers(1, 7, m).astype(np.int32)
    for i in range(m):
        k = ndep[i]
        pann = int(rng.integers(0, 2, 1)[0])
        cry = rng.integers(0, 4, k) + 8 * rng.integers(0, 2, k)
        dep[i, :k]["parn"] = 7
        dep[i, :k]["pann"] = pann
        dep[i, :k]["modn"] = 0
        dep[i, :k]["cryn"] = cry
        dep[i, :k]["siten"] = pann * 64 + cry
        dep[i, :k]["eventid"] = 3
        dep[i, :k]["t"] = 100.0 + np.cumsum(rng.uniform(0, 1e-3, (k,)))
        dep[i, :k]["E"] = rng.uniform(1e3, 3e5, (k,))
        dep[i, :k]["x"] = rng.uniform(0, 2, (k,))
        dep[i, :k]["y"] = rng.uniform(-1.2, 1.2, (k,))
        dep[i, :k]["z"] = rng.uniform(-1.2, 1.2, (k,))
    I["ar_dep"] = dep
    I["ar_n"] = ndep
    I["ar_mode"] = rng.integers(0, 4, m).astype(np.int32)    # (depth, policy) of READOUT_MODES
    # blur (policies 0 and 1, no spatial blur)
    ev = np.zeros(n, F.EVENT_DTYPE)
    ev["E"] = rng.uniform(5e4, 6e5, (n,))
    ev["x"] = rng.uniform(0, 2, (n,))
    I["bl_ev"] = ev
    I["bl_policy"] = rng.integers(0, 2, n).astype(np.int32)
    I["bl_tape"] = words(n)
    return I


READOUT_MODES = [(0, 0), (1, 0), (2, 0), (2, 1)]   # (rdepth, rpolicy)
BLUR = dict(Eref=511e3, Rref=0.12, slope=0.0)


# ---------------------------------------------------------------- the reference
def reference_lib(build=True):
    """The reference's functions built for the CPU, or None when the
    reference source is not at hand."""
    sys.path.insert(0, HERE)
    import ref_build
    path = ref_build.LIB
    if build:
        path = ref_build.build()
    if not path or not os.path.exists(path):
        return None
    L = C.CDLL(path)
    L.ref_load_tables.argtypes = [C.c_char_p, _FP, _FP]
    L.ref_get_table.argtypes = [C.c_int, _FP, C.c_int64]
    L.ref_get_scalars.argtypes = [_FP]
    L.ref_set_phantom.argtypes = [_IP, _FP, C.c_int, C.c_int, C.c_int, _FP, _FP, C.c_float]
    L.ref_set_detector.argtypes = [C.c_char_p]
    L.ref_get_panels.argtypes = [_FP, C.c_int, _IP, _IP, _FP]
    L.ref_set_surfaces.argtypes = [C.c_int, _FP]
    L.ref_get_majorant.argtypes = [C.c_int, _FP, _FP, _FP]
    L.ref_photon.argtypes = [_FP, C.c_double, _UP, C.c_int64, _FP, _DP, _LP]
    L.ref_photonde.argtypes = [_FP, C.c_double, C.c_int32, C.c_int, C.c_int, _UP, C.c_int64, C.c_void_p, C.c_int,
                               _LP]
    L.ref_comsam_kn.argtypes = [C.c_float, _UP, C.c_int64, _FP, _FP, _LP]
    L.ref_surface_sample.argtypes = [C.c_int, C.c_float, C.c_int, _UP, C.c_int64, _FP, _FP, _LP]
    L.ref_sample_ek.argtypes = [_FP, _UP, C.c_int64, _LP]
    L.ref_sample_ek.restype = C.c_float
    L.ref_shape.argtypes = [C.c_int, _FP, _UP, C.c_int64, _FP, _LP]
    L.ref_positron_range.argtypes = [_FP, _FP, C.c_int, _UP, C.c_int64, _FP, _LP]
    L.ref_psf_pair.argtypes = [_FP, _FP, C.c_int, C.c_float, _UP, C.c_int64, _FP, _LP]
    L.ref_crystal_search.argtypes = [C.c_int, _FP, _IP]
    L.ref_adder_readout.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
    L.ref_blur.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, _UP, C.c_int64, _LP]
    return L


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def reference_outputs(L, scene, data_dir, I):
    """Everything the reference computes for the pins (the golden vectors)."""
    cfg = F.read_config(scene.config_path)
    out = {}
    e0, e1 = C.c_float(), C.c_float()
    nmat = L.ref_load_tables(ROOT.encode(), C.byref(e0), C.byref(e1))
    out["nmat"] = np.int32(nmat)
    out["eminph_emax"] = np.array([e0.value, e1.value], np.float32)
    sizes = [10 * 4096] * 4 + [10 * 301 * 151] * 2 + [4096] * 4
    for k, n in enumerate(sizes):
        t = np.zeros(n, np.float32)
        assert L.ref_get_table(k, _p(t, _FP), n) == n
        out["table_sha256_%d" % k] = np.array(_digest(t))
        if k == 6:
            out["table_energy"] = t
    sc = np.zeros(8, np.float32)
    L.ref_get_scalars(_p(sc, _FP))
    out["table_scalars"] = sc
    # phantom, its majorant; the ring, its majorant
    mat, den = F.read_phantom(os.path.join(scene.directory, "phantom_mat.dat"),
                              os.path.join(scene.directory, "phantom_den.dat"), cfg.pdim)
    mat = np.ascontiguousarray(mat, np.int32)
    den = np.ascontiguousarray(den, np.float32)
    d = (np.float32(cfg.psize) / np.float32(cfg.pdim)).astype(np.float32)
    off = np.array(cfg.poffset, np.float32)
    L.ref_set_phantom(_p(mat, _IP), _p(den, _FP), *cfg.pdim, _p(d, _FP), _p(off, _FP), cfg.eabsph)
    for which, key in ((0, "majorant_phantom"),):
        tab = np.zeros(4096, np.float32)
        a, b = C.c_float(), C.c_float()
        L.ref_get_majorant(which, _p(tab, _FP), C.byref(a), C.byref(b))
        out[key] = tab
        out[key + "_grid"] = np.array([a.value, b.value], np.float32)
    for name, geo in (("ring", os.path.join(scene.directory, "ring.geo")),
                      ("config8", os.path.join(ROOT, "tests", "golden", "reference_inputs", "config8.geo"))):
        npan = L.ref_set_detector(geo.encode())
        P = np.zeros((npan, 31), np.float32)
        cnt = np.zeros(4, np.int32)
        m2 = np.zeros(2, np.int32)
        d2 = np.zeros(2, np.float32)
        L.ref_get_panels(_p(P, _FP), npan, _p(cnt, _IP), _p(m2, _IP), _p(d2, _FP))
        out["panels_" + name] = P
        out["counts_" + name] = cnt
        out["detmat_" + name] = m2
        out["detden_" + name] = d2
    # the ring again: it is the detector of the transport pins
    L.ref_set_detector(os.path.join(scene.directory, "ring.geo").encode())
    surf = np.array(cfg.surfaces, np.float32).reshape(-1)
    L.ref_set_surfaces(len(cfg.surfaces), _p(surf, _FP))
    tab = np.zeros(4096, np.float32)
    a, b = C.c_float(), C.c_float()
    L.ref_get_majorant(1, _p(tab, _FP), C.byref(a), C.byref(b))
    out["majorant_detector"] = tab
    out["majorant_detector_grid"] = np.array([a.value, b.value], np.float32)
    used = C.c_int64()
    # phantom transport
    n = len(I["ph_in"])
    o = np.zeros((n, 7), np.float32)
    t = np.zeros(n)
    u = np.zeros(n, np.int64)
    for i in range(n):
        tt = C.c_double()
        L.ref_photon(_p(I["ph_in"][i], _FP), float(I["ph_t"][i]), _p(I["ph_tape"][i], _UP), TAPE, _p(o[i], _FP),
                     C.byref(tt), C.byref(used))
        t[i] = tt.value
        u[i] = used.value
    out["ph_out"], out["ph_t_out"], out["ph_used"] = o, t, u
    # detector transport
    n = len(I["de_in"])
    pulses = np.zeros((n, 8), F.EVENT_DTYPE)
    npul = np.zeros(n, np.int32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        k = L.ref_photonde(_p(I["de_in"][i], _FP), float(I["de_t"][i]), 11, cfg.rdepth, cfg.rpolicy,
                           _p(I["de_tape"][i], _UP), TAPE, pulses[i].ctypes.data, 8, C.byref(used))
        npul[i] = k
        u[i] = used.value
    out["de_pulses"], out["de_npulses"], out["de_used"] = pulses, npul, u
    # samplers
    n = len(I["kn_e"])
    r = np.zeros((n, 2), np.float32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        a, b = C.c_float(), C.c_float()
        L.ref_comsam_kn(float(I["kn_e"][i]), _p(I["kn_tape"][i], _UP), TAPE, C.byref(a), C.byref(b), C.byref(used))
        r[i] = a.value, b.value
        u[i] = used.value
    out["kn_out"], out["kn_used"] = r, u
    r = np.zeros((n, 2, 2), np.float32)
    u = np.zeros((n, 2), np.int64)
    for i in range(n):
        for w in range(2):
            a, b = C.c_float(), C.c_float()
            L.ref_surface_sample(w, float(I["sf_e"][i]), int(I["sf_m"][i]), _p(I["sf_tape"][i], _UP), TAPE,
                                 C.byref(a), C.byref(b), C.byref(used))
            r[i, w] = a.value, b.value
            u[i, w] = used.value
    out["sf_out"], out["sf_used"] = r, u
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    coef = np.ascontiguousarray(iso.coef[0], np.float32)
    r = np.zeros(n, np.float32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        r[i] = L.ref_sample_ek(_p(coef, _FP), _p(I["ek_tape"][i], _UP), TAPE, C.byref(used))
        u[i] = used.value
    out["ek_out"], out["ek_used"] = r, u
    r = np.zeros((n, 3), np.float32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        L.ref_shape(int(I["shape_kind"][i]), _p(I["shape_coef"][i], _FP), _p(I["shape_tape"][i], _UP), TAPE,
                    _p(r[i], _FP), C.byref(used))
        u[i] = used.value
    out["shape_out"], out["shape_used"] = r, u
    r = np.zeros((n, 3), np.float32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        L.ref_positron_range(_p(I["pr_x"][i], _FP), _p(I["pr_v"][i], _FP), int(I["pr_usedir"][i]),
                             _p(I["pr_tape"][i], _UP), TAPE, _p(r[i], _FP), C.byref(used))
        u[i] = used.value
    out["pr_out"], out["pr_used"] = r, u
    r = np.zeros((n, 11), np.float32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        L.ref_psf_pair(_p(I["pr_x"][i], _FP), _p(I["pr_v"][i], _FP), int(I["pair_useprange"][i]),
                       cfg.noncol_sigma, _p(I["pair_tape"][i], _UP), TAPE, _p(r[i], _FP), C.byref(used))
        u[i] = used.value
    out["pair_out"], out["pair_used"] = r, u
    ids = np.zeros((n, 3), np.int32)
    for i in range(n):
        L.ref_crystal_search(int(I["cs_panel"][i]), _p(I["cs_x"][i], _FP), _p(ids[i], _IP))
    out["cs_ids"] = ids
    m = len(I["ar_n"])
    res = np.zeros((m, 8), F.EVENT_DTYPE)
    nres = np.zeros(m, np.int32)
    for i in range(m):
        dep = np.ascontiguousarray(I["ar_dep"][i])
        depth, pol = READOUT_MODES[int(I["ar_mode"][i])]
        nres[i] = L.ref_adder_readout(dep.ctypes.data, int(I["ar_n"][i]), depth, pol, res[i].ctypes.data, 8)
    out["ar_out"], out["ar_nout"] = res, nres
    ev = I["bl_ev"].copy()
    u = np.zeros(n, np.int64)
    for i in range(n):
        e = ev[i:i + 1]
        L.ref_blur(e.ctypes.data, int(I["bl_policy"][i]), BLUR["Eref"], BLUR["Rref"], BLUR["slope"], 0.0,
                   _p(I["bl_tape"][i], _UP), TAPE, C.byref(used))
        u[i] = used.value
    out["bl_out"], out["bl_used"] = ev, u
    return out


# ------------------------------------------------------------------ the oracle
def oracle_lib():
    import bridge
    bridge.build()
    L = C.CDLL(os.path.join(ORACLE, "build", "liboracle_fp32_tape.so"))
    S = C.POINTER(bridge._Scene)
    L.oracle_majorant.argtypes = [S, C.c_int, _FP, _FP, _FP]
    L.oracle_tape_phantom.argtypes = [S, _FP, C.c_float, C.c_float, _FP, C.c_double, _UP, C.c_int64, _DP, _DP,
                                      _IP, _LP]
    L.oracle_tape_detector.argtypes = [S, _FP, C.c_float, C.c_float, _FP, C.c_double, C.c_int32, _UP, C.c_int64,
                                       C.c_void_p, C.c_int, _IP, _LP]
    L.oracle_tape_kn.argtypes = [C.c_double, _UP, C.c_int64, _DP, _DP, _LP]
    L.oracle_tape_surface.argtypes = [S, C.c_int, C.c_double, C.c_int, _UP, C.c_int64, _DP, _DP, _LP]
    L.oracle_tape_sample_ek.argtypes = [_FP, _UP, C.c_int64, _LP]
    L.oracle_tape_sample_ek.restype = C.c_double
    L.oracle_tape_shape.argtypes = [C.c_int, _FP, _UP, C.c_int64, _DP, _LP]
    L.oracle_tape_positron_range.argtypes = [S, _FP, C.c_double, _FP, _UP, C.c_int64, _DP, _LP]
    L.oracle_tape_psf_pair.argtypes = [S, _FP, _FP, C.c_int, _UP, C.c_int64, _DP, _LP]
    L.oracle_crystal_search_at.argtypes = [S, C.c_int, _DP, _IP]
    L.oracle_adder_readout.argtypes = [S, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    L.oracle_tape_blur.argtypes = [S, C.c_void_p, _UP, C.c_int64, _LP]
    return L


def oracle_outputs(scene, data_dir, I, ref):
    """What the oracle computes for the pins. The transport pins use the
    reference's majorant tables (given in ref), so that they compare the
    transport itself; the oracle's own majorants are returned beside them."""
    import bridge
    L = oracle_lib()
    osc = bridge.OracleScene(scene.config_path, scene.options, data_dir, base_dir=scene.directory)
    S = C.byref(osc.s)
    out = {"tables": osc.tables, "geo": osc.geo}
    for which, key in ((0, "majorant_phantom"), (1, "majorant_detector")):
        tab = np.zeros(4096, np.float32)
        a, b = C.c_float(), C.c_float()
        assert L.oracle_majorant(S, which, _p(tab, _FP), C.byref(a), C.byref(b)) == 0
        out[key] = tab
        out[key + "_grid"] = np.array([a.value, b.value], np.float32)
    used = C.c_int64()
    wph = np.ascontiguousarray(ref["majorant_phantom"], np.float32)
    gph = ref["majorant_phantom_grid"]
    n = len(I["ph_in"])
    o = np.zeros((n, 7))
    t = np.zeros(n)
    st = np.zeros(n, np.int32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        tt = C.c_double()
        ns = C.c_int32()
        st[i] = L.oracle_tape_phantom(S, _p(wph, _FP), float(gph[0]), float(gph[1]), _p(I["ph_in"][i], _FP),
                                      float(I["ph_t"][i]), _p(I["ph_tape"][i], _UP), TAPE, _p(o[i], _DP),
                                      C.byref(tt), C.byref(ns), C.byref(used))
        t[i] = tt.value
        u[i] = used.value
    out["ph_out"], out["ph_t_out"], out["ph_status"], out["ph_used"] = o, t, st, u
    wde = np.ascontiguousarray(ref["majorant_detector"], np.float32)
    gde = ref["majorant_detector_grid"]
    n = len(I["de_in"])
    pulses = np.zeros((n, 8), F.EVENT_DTYPE)
    npul = np.zeros(n, np.int32)
    pan = np.zeros(n, np.int32)
    u = np.zeros(n, np.int64)
    for i in range(n):
        pp = C.c_int32()
        npul[i] = L.oracle_tape_detector(S, _p(wde, _FP), float(gde[0]), float(gde[1]), _p(I["de_in"][i], _FP),
                                         float(I["de_t"][i]), 11, _p(I["de_tape"][i], _UP), TAPE,
                                         pulses[i].ctypes.data, 8, C.byref(pp), C.byref(used))
        pan[i] = pp.value
        u[i] = used.value
    out["de_pulses"], out["de_npulses"], out["de_panel"], out["de_used"] = pulses, npul, pan, u
    n = len(I["kn_e"])
    r = np.zeros((n, 2))
    u = np.zeros(n, np.int64)
    for i in range(n):
        a, b = C.c_double(), C.c_double()
        L.oracle_tape_kn(float(I["kn_e"][i]), _p(I["kn_tape"][i], _UP), TAPE, C.byref(a), C.byref(b), C.byref(used))
        r[i] = a.value, b.value
        u[i] = used.value
    out["kn_out"], out["kn_used"] = r, u
    r = np.zeros((n, 2, 2))
    u = np.zeros((n, 2), np.int64)
    for i in range(n):
        for w in range(2):
            a, b = C.c_double(), C.c_double()
            L.oracle_tape_surface(S, w, float(I["sf_e"][i]), int(I["sf_m"][i]), _p(I["sf_tape"][i], _UP), TAPE,
                                  C.byref(a), C.byref(b), C.byref(used))
            r[i, w] = a.value, b.value
            u[i, w] = used.value
    out["sf_out"], out["sf_used"] = r, u
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    coef = np.ascontiguousarray(iso.coef[0], np.float32)
    r = np.zeros(n)
    u = np.zeros(n, np.int64)
    for i in range(n):
        r[i] = L.oracle_tape_sample_ek(_p(coef, _FP), _p(I["ek_tape"][i], _UP), TAPE, C.byref(used))
        u[i] = used.value
    out["ek_out"], out["ek_used"] = r, u
    r = np.zeros((n, 3))
    u = np.zeros(n, np.int64)
    for i in range(n):
        L.oracle_tape_shape(int(I["shape_kind"][i]), _p(I["shape_coef"][i], _FP), _p(I["shape_tape"][i], _UP), TAPE,
                            _p(r[i], _DP), C.byref(used))
        u[i] = used.value
    out["shape_out"], out["shape_used"] = r, u
    r = np.zeros((n, 3))
    u = np.zeros(n, np.int64)
    for i in range(n):
        v = I["pr_v"][i]
        dirp = _p(np.ascontiguousarray(v[:3]), _FP) if I["pr_usedir"][i] else None
        L.oracle_tape_positron_range(S, _p(I["pr_x"][i], _FP), float(v[3]), dirp, _p(I["pr_tape"][i], _UP), TAPE,
                                     _p(r[i], _DP), C.byref(used))
        u[i] = used.value
    out["pr_out"], out["pr_used"] = r, u
    r = np.zeros((n, 11))
    u = np.zeros(n, np.int64)
    for i in range(n):
        L.oracle_tape_psf_pair(S, _p(I["pr_x"][i], _FP), _p(I["pr_v"][i], _FP), int(I["pair_useprange"][i]),
                               _p(I["pair_tape"][i], _UP), TAPE, _p(r[i], _DP), C.byref(used))
        u[i] = used.value
    out["pair_out"], out["pair_used"] = r, u
    ids = np.zeros((n, 3), np.int32)
    for i in range(n):
        x = np.ascontiguousarray(I["cs_x"][i], np.float64)
        L.oracle_crystal_search_at(S, int(I["cs_panel"][i]), _p(x, _DP), _p(ids[i], _IP))
    out["cs_ids"] = ids
    m = len(I["ar_n"])
    res = np.zeros((m, 8), F.EVENT_DTYPE)
    nres = np.zeros(m, np.int32)
    for i in range(m):
        depth, pol = READOUT_MODES[int(I["ar_mode"][i])]
        osc.s.rdepth, osc.s.rpolicy = depth, pol
        dep = np.ascontiguousarray(I["ar_dep"][i])
        nres[i] = L.oracle_adder_readout(S, dep.ctypes.data, int(I["ar_n"][i]), res[i].ctypes.data, 8)
    out["ar_out"], out["ar_nout"] = res, nres
    ev = I["bl_ev"].copy()
    u = np.zeros(n, np.int64)
    osc.s.Eref, osc.s.Rref, osc.s.Eslope, osc.s.Sblur = BLUR["Eref"], BLUR["Rref"], BLUR["slope"], 0.0
    for i in range(n):
        osc.s.blurpolicy = int(I["bl_policy"][i])
        L.oracle_tape_blur(S, ev[i:i + 1].ctypes.data, _p(I["bl_tape"][i], _UP), TAPE, C.byref(used))
        u[i] = used.value
    out["bl_out"], out["bl_used"] = ev, u
    return out


# ------------------------------------------------------------ golden vectors
def pack(R):
    """The reference's outputs as stored in tests/golden/ref_vectors.npz:
    the detector pulses of the photons that made some, flattened."""
    out = {k: v for k, v in R.items() if k != "de_pulses"}
    n = R["de_npulses"]
    out["de_pulses_flat"] = np.concatenate([R["de_pulses"][i, :min(int(k), 8)] for i, k in enumerate(n)]) \
        if n.sum() else np.zeros(0, F.EVENT_DTYPE)
    for k in list(out):
        if k.endswith("_used"):
            out[k] = out[k].astype(np.int16)
    return out


def unpack(G):
    R = {k: G[k] for k in G.files} if hasattr(G, "files") else dict(G)
    n = R["de_npulses"]
    pulses = np.zeros((len(n), 8), F.EVENT_DTYPE)
    off = 0
    for i, k in enumerate(n):
        k = min(int(k), 8)
        pulses[i, :k] = R["de_pulses_flat"][off:off + k]
        off += k
    R["de_pulses"] = pulses
    for k in list(R):
        if k.endswith("_used"):
            R[k] = R[k].astype(np.int64)
    return R
