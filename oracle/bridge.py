"""ctypes bridge to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported by tests/ and by bench.py's CPU-baseline leg; the product never
imports it. Builds the oracle's scene from gPET input files (parsed with
gpet_gb300.formats, an implementation independent of the native loaders) and
returns results as numpy arrays.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np

from gpet_gb300 import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")


def build(quiet=True):
    """Compile both oracle builds with the Makefile beside this file."""
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if not quiet:
        print(r.stdout)


class _Event(C.Structure):
    _fields_ = [("parn", C.c_int32), ("pann", C.c_int32), ("modn", C.c_int32), ("cryn", C.c_int32),
                ("siten", C.c_int32), ("eventid", C.c_int32), ("t", C.c_double),
                ("E", C.c_float), ("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class _Exit(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("ux", C.c_float), ("uy", C.c_float),
                ("uz", C.c_float), ("E", C.c_float), ("nscat", C.c_int32), ("t", C.c_double),
                ("status", C.c_int32), ("panel", C.c_int32)]


EXIT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                       ("E", "<f4"), ("nscat", "<i4"), ("t", "<f8"), ("status", "<i4"), ("panel", "<i4")])
assert EXIT_DTYPE.itemsize == C.sizeof(_Exit)
# emitted-photon / phantom-exit phase-space record (40 bytes)
PSF_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                      ("E", "<f4"), ("eventid", "<i4"), ("t", "<f8")])

_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)
_LP = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)


class _Scene(C.Structure):
    _fields_ = [
        ("nmat", C.c_int32), ("ne", C.c_int32), ("e0", C.c_float), ("idle", C.c_float),
        ("lamph", _FP), ("compt", _FP), ("phote", _FP), ("rayle", _FP),
        ("ncp_c", C.c_int32), ("ne_c", C.c_int32), ("idcp_c", C.c_float), ("ide_c", C.c_float), ("cmpsf", _FP),
        ("ncp_r", C.c_int32), ("ne_r", C.c_int32), ("idcp_r", C.c_float), ("ide_r", C.c_float), ("rayff", _FP),
        ("eminph", C.c_float), ("emax", C.c_float),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
        ("offx", C.c_float), ("offy", C.c_float), ("offz", C.c_float),
        ("mat", _IP), ("den", _FP),
        ("npanels", C.c_int32), ("panels", _FP), ("det_mat", C.c_int32 * 2), ("det_den", C.c_float * 2),
        ("moduleN", C.c_int32), ("crystalN", C.c_int32), ("moduleNy", C.c_int32), ("crystalNy", C.c_int32),
        ("nsurface", C.c_int32), ("surface", C.c_float * 50),
        ("nsrc", C.c_int32), ("src_first", _LP), ("src_count", _LP), ("src_type", _IP), ("src_shape", _IP),
        ("src_coef", _FP), ("iso_halftime", _FP), ("iso_ratio", _FP), ("iso_coef", _FP),
        ("tstart_s", C.c_double), ("dt_s", C.c_double), ("useprange", C.c_int32),
        ("noncol_sigma", C.c_float), ("eabsph", C.c_float),
        ("npsf", C.c_int64), ("psf", _DP), ("psf_ptype", C.c_int32),
        ("rdepth", C.c_int32), ("rpolicy", C.c_int32), ("blurpolicy", C.c_int32),
        ("Eref", C.c_float), ("Rref", C.c_float), ("Eslope", C.c_float), ("Sblur", C.c_float), ("Eth", C.c_float),
        ("dlevel", C.c_int32), ("dtype", C.c_int32),
        ("dtime_us", C.c_float), ("ewin_lo", C.c_float), ("ewin_hi", C.c_float),
        ("coinc_window_us", C.c_double), ("coinc_policy", C.c_int32),
        ("seed", C.c_uint64), ("sim_id", C.c_uint32),
        ("noise_lambda_us", C.c_float), ("noise_emean", C.c_float), ("noise_sigma", C.c_float),
        ("noise_interval_us", C.c_double), ("noise_t0_us", C.c_double), ("noise_t1_us", C.c_double),
        ("nxdet", C.c_int32), ("xdet_mat", C.c_int32 * 6), ("xdet_den", C.c_float * 6),
        ("prmap", C.POINTER(C.c_int8)),
    ]


class _Result(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "n_decays", "n_pairs", "n_entered", "n_pulses", "n_hits", "n_threshold", "n_deadtime", "n_singles",
        "n_coinc", "n_true", "n_scatter", "n_random", "n_multiple", "n_overflow", "n_stepcap", "n_noise")] + [
        ("exits", C.POINTER(_Exit)), ("source", C.c_void_p), ("pulses", C.POINTER(_Event)),
        ("pulse_scat", C.POINTER(C.c_uint8)), ("pulse_slot", C.POINTER(C.c_uint8)),
        ("hit_id", _IP), ("hit_f", _FP),
        ("singles", C.POINTER(_Event)), ("single_scat", C.POINTER(C.c_uint8)), ("single_slot", C.POINTER(C.c_uint8)),
        ("coinc", _LP), ("coinc_class", C.POINTER(C.c_uint8)),
    ]


_LIBS = {}


def lib(precision="fp64"):
    if precision not in _LIBS:
        path = os.path.join(BUILD, "liboracle_%s.so" % precision)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.oracle_run.argtypes = [C.POINTER(_Scene), C.c_int64, C.c_int64, C.c_int, C.c_int, C.POINTER(_Result)]
        L.oracle_digitize.argtypes = [C.POINTER(_Scene), C.POINTER(_Event), C.POINTER(C.c_uint8),
                                      C.POINTER(C.c_uint8), C.c_int64, C.POINTER(_Result)]
        L.oracle_free_result.argtypes = [C.POINTER(_Result)]
        L.oracle_build_prmap.argtypes = [C.POINTER(_Scene), C.POINTER(C.c_int8)]
        L.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.oracle_stream_words.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_int64,
                                          C.POINTER(C.c_uint32)]
        _LIBS[precision] = L
    return _LIBS[precision]


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().oracle_philox4x32_10(c, k, o)
    return list(o)


def stream_words(key, tag, ident, n):
    """The first n words of the oracle's random stream (key, tag, id)."""
    o = (C.c_uint32 * n)()
    lib().oracle_stream_words(key[0], key[1], tag, ident, n, o)
    return list(o)


def source_layout(natom, types, halftime, tstart, dt, n_decays=None):
    """Decays per source: floor(N_t (1 - 2^(-dt/T))) with N_t = floor(natom
    2^(-tstart/T)) (gPET.cu:204-208, 264-272); with n_decays given, that total
    is split over the sources in proportion (largest remainder)."""
    exp_counts = []
    for n, t in zip(natom, types):
        th = float(halftime[t])
        nt = math.floor(float(n) * math.pow(2.0, -float(tstart) / th))
        exp_counts.append(math.floor(nt * (1.0 - math.pow(2.0, -float(dt) / th))))
    if n_decays is None:
        counts = exp_counts
    else:
        tot = float(sum(exp_counts))
        if tot <= 0:
            raise ValueError("no source decays in the window")
        quota = [n_decays * e / tot for e in exp_counts]
        counts = [math.floor(q) for q in quota]
        rest = n_decays - sum(counts)
        order = sorted(range(len(quota)), key=lambda i: (-(quota[i] - counts[i]), i))
        for i in order[:rest]:
            counts[i] += 1
    first = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    return first, np.array(counts, np.int64)


class OracleScene:
    """Holds the numpy arrays behind one or_scene."""

    def __init__(self, config_path, options=None, data_dir=None, panels=None, base_dir=None, psf=None):
        options = dict(options or {})
        base = base_dir or os.getcwd()

        def res(p):
            return p if os.path.isabs(p) else os.path.join(base, p)

        cfg = F.read_config(config_path)
        self.cfg = cfg
        data_dir = data_dir or os.path.join(os.path.dirname(HERE), "data")
        T = F.read_tables(data_dir)
        self.tables = T
        geo = F.read_geo(res(cfg.geofile))
        self.geo = geo
        self.panels = np.ascontiguousarray(panels if panels is not None else geo.panels, np.float32)
        mat, den = F.read_phantom(res(cfg.matfile), res(cfg.denfile), cfg.pdim)
        self.mat, self.den = np.ascontiguousarray(mat), np.ascontiguousarray(den)
        self.lamph = np.ascontiguousarray(T.lamph); self.compt = np.ascontiguousarray(T.compt)
        self.phote = np.ascontiguousarray(T.phote); self.rayle = np.ascontiguousarray(T.rayle)
        self.cmpsf = np.ascontiguousarray(T.cmpsf); self.rayff = np.ascontiguousarray(T.rayff)
        iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
        self.iso_ht, self.iso_ratio, self.iso_coef = iso.halftime, iso.ratio, np.ascontiguousarray(iso.coef)
        s = _Scene()
        s.nmat = len(T.names); s.ne = len(T.energy)
        s.e0 = float(T.energy[0]); s.idle = T.idle
        s.lamph = self.lamph.ctypes.data_as(_FP); s.compt = self.compt.ctypes.data_as(_FP)
        s.phote = self.phote.ctypes.data_as(_FP); s.rayle = self.rayle.ctypes.data_as(_FP)
        s.ncp_c, s.ne_c = self.cmpsf.shape[1], self.cmpsf.shape[2]
        s.idcp_c = F.f32(np.float32(1.0) / np.float32(T.cmpsf_dcp)); s.ide_c = F.f32(np.float32(1.0) / np.float32(T.cmpsf_de))
        s.cmpsf = self.cmpsf.ctypes.data_as(_FP)
        s.ncp_r, s.ne_r = self.rayff.shape[1], self.rayff.shape[2]
        s.idcp_r = F.f32(np.float32(1.0) / np.float32(T.rayff_dcp)); s.ide_r = F.f32(np.float32(1.0) / np.float32(T.rayff_de))
        s.rayff = self.rayff.ctypes.data_as(_FP)
        s.eminph, s.emax = T.eminph, T.emax
        s.nx, s.ny, s.nz = cfg.pdim
        s.dx = F.f32(np.float32(cfg.psize[0]) / np.float32(cfg.pdim[0]))
        s.dy = F.f32(np.float32(cfg.psize[1]) / np.float32(cfg.pdim[1]))
        s.dz = F.f32(np.float32(cfg.psize[2]) / np.float32(cfg.pdim[2]))
        s.offx, s.offy, s.offz = cfg.poffset
        s.mat = self.mat.ctypes.data_as(_IP); s.den = self.den.ctypes.data_as(_FP)
        # the uniform-density map of the positron range's closed form (the
        # same map the library builds at phantom upload)
        self.prmap = np.empty(int(np.prod(cfg.pdim)), np.int8)
        lib().oracle_build_prmap(C.byref(s), self.prmap.ctypes.data_as(C.POINTER(C.c_int8)))
        s.prmap = self.prmap.ctypes.data_as(C.POINTER(C.c_int8))
        s.npanels = geo.npanels; s.panels = self.panels.ctypes.data_as(_FP)
        s.det_mat[0], s.det_mat[1] = geo.det_mat[:2]
        s.det_den[0], s.det_den[1] = geo.det_den[:2]
        s.nxdet = len(geo.det_mat) - 2
        for k in range(s.nxdet):
            s.xdet_mat[k] = geo.det_mat[2 + k]
            s.xdet_den[k] = geo.det_den[2 + k]
        mny, mn, cny, cn = F.panel_counts(self.panels[0])
        s.moduleN, s.crystalN, s.moduleNy, s.crystalNy = mn, cn, mny, cny
        s.nsurface = len(cfg.surfaces)
        for k, surf in enumerate(cfg.surfaces):
            for j in range(10):
                s.surface[10 * k + j] = surf[j]
        s.tstart_s = float(cfg.tstart); s.dt_s = float(np.float32(cfg.tend) - np.float32(cfg.tstart))
        s.useprange = cfg.useprange
        s.noncol_sigma = cfg.noncol_sigma; s.eabsph = cfg.eabsph
        if cfg.usepsf or psf is not None:
            rec = psf if psf is not None else F.read_psf(res(cfg.sourcefile), cfg.nparticle or None)
            self.psf = np.ascontiguousarray(rec, np.float64)
            s.npsf = len(self.psf); s.psf = self.psf.ctypes.data_as(_DP); s.psf_ptype = cfg.ptype
            self.n_decays = len(self.psf)
            self.src_first = np.zeros(1, np.int64); self.src_count = np.zeros(1, np.int64)
            self.src_type = np.zeros(1, np.int32); self.src_shape = np.zeros(1, np.int32)
            self.src_coef = np.zeros((1, 6), np.float32)
            s.nsrc = 0
        else:
            src = F.read_sources(res(cfg.sourcefile))
            first, count = source_layout(src.natom, src.type, iso.halftime, cfg.tstart, s.dt_s,
                                         options.get("n_decays"))
            self.src_first, self.src_count = first, count
            self.src_type, self.src_shape = src.type.astype(np.int32), src.shape.astype(np.int32)
            self.src_coef = np.ascontiguousarray(src.coef, np.float32)
            s.nsrc = len(first)
            self.n_decays = int(count.sum())
        s.src_first = self.src_first.ctypes.data_as(_LP); s.src_count = self.src_count.ctypes.data_as(_LP)
        s.src_type = self.src_type.ctypes.data_as(_IP); s.src_shape = self.src_shape.ctypes.data_as(_IP)
        s.src_coef = self.src_coef.ctypes.data_as(_FP)
        s.iso_halftime = self.iso_ht.ctypes.data_as(_FP); s.iso_ratio = self.iso_ratio.ctypes.data_as(_FP)
        s.iso_coef = self.iso_coef.ctypes.data_as(_FP)
        s.rdepth, s.rpolicy, s.blurpolicy = cfg.rdepth, cfg.rpolicy, cfg.blurpolicy
        s.Eref, s.Rref, s.Eslope, s.Sblur, s.Eth = cfg.eref, cfg.rref, cfg.eslope, cfg.sblur, cfg.eth
        s.dlevel, s.dtype, s.dtime_us = cfg.dlevel, cfg.dtype, cfg.dtime
        s.ewin_lo, s.ewin_hi = cfg.ewin_lo, cfg.ewin_hi
        s.coinc_window_us = float(options.get("coinc_window_ns", 4.0)) * 1e-3
        s.coinc_policy = int(options.get("coinc_policy", 0))
        s.seed = int(options.get("seed", 20261203)); s.sim_id = int(options.get("sim_id", 0))
        s.noise_lambda_us = float(options.get("noise_lambda_us", 0.0))
        s.noise_emean = float(options.get("noise_emean_ev", 511000.0))
        s.noise_sigma = float(options.get("noise_sigma_ev", 0.0))
        s.noise_interval_us = float(options.get("noise_interval_us", 1000.0))
        s.noise_t0_us = float(np.float32(cfg.tstart)) * 1e6
        s.noise_t1_us = float(np.float32(cfg.tend)) * 1e6
        self.s = s

    def run(self, d_begin=0, d_end=None, precision="fp64", threads=0, exits=False, hits=False, source=False):
        d_end = self.n_decays if d_end is None else d_end
        r = _Result()
        L = lib(precision)
        rc = L.oracle_run(C.byref(self.s), d_begin, d_end, threads,
                          (1 if exits else 0) | (2 if hits else 0) | (4 if source else 0), C.byref(r))
        if rc != 0:
            raise RuntimeError("oracle_run failed: %d" % rc)
        try:
            out = _collect(r, exits)
            if source:
                out["source"] = _arr(r.source, 2 * r.n_decays, PSF_DTYPE)
            return out
        finally:
            L.oracle_free_result(C.byref(r))

    def digitize(self, pulses, scat, slot, precision="fp64"):
        pulses = np.ascontiguousarray(pulses, F.EVENT_DTYPE)
        scat = np.ascontiguousarray(scat, np.uint8)
        slot = np.ascontiguousarray(slot, np.uint8)
        r = _Result()
        L = lib(precision)
        L.oracle_digitize(C.byref(self.s), pulses.ctypes.data_as(C.POINTER(_Event)),
                          scat.ctypes.data_as(C.POINTER(C.c_uint8)), slot.ctypes.data_as(C.POINTER(C.c_uint8)),
                          len(pulses), C.byref(r))
        try:
            return _collect(r, False)
        finally:
            L.oracle_free_result(C.byref(r))


def _arr(ptr, n, dtype, shape=None):
    if n == 0 or not ptr:
        return np.zeros((0,) + (shape or ()), dtype)
    a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(n * np.dtype(dtype).itemsize *
                                                                        int(np.prod(shape or (1,))),))
    return a.view(dtype).reshape((n,) + (shape or ())).copy()


def _collect(r, exits):
    out = {k: int(getattr(r, k)) for k, _ in _Result._fields_[:16]}
    if exits:
        out["exits"] = _arr(r.exits, 2 * r.n_decays, EXIT_DTYPE)
    out["pulses"] = _arr(r.pulses, r.n_pulses, F.EVENT_DTYPE)
    out["pulse_scat"] = _arr(r.pulse_scat, r.n_pulses, np.uint8)
    out["pulse_slot"] = _arr(r.pulse_slot, r.n_pulses, np.uint8)
    out["hit_id"] = _arr(r.hit_id, r.n_hits, np.int32, (5,))
    out["hit_f"] = _arr(r.hit_f, r.n_hits, np.float32, (5,))
    out["singles"] = _arr(r.singles, r.n_singles, F.EVENT_DTYPE)
    out["single_scat"] = _arr(r.single_scat, r.n_singles, np.uint8)
    out["single_slot"] = _arr(r.single_slot, r.n_singles, np.uint8)
    out["coinc"] = _arr(r.coinc, r.n_coinc, np.int64, (2,))
    out["coinc_class"] = _arr(r.coinc_class, r.n_coinc, np.uint8)
    return out
