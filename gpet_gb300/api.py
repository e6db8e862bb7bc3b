"""Python mirror of the C ABI in include/gpet.h (ctypes over libgpet.so).

The native library is the product: every call here goes to the CUDA
implementation, and a missing or unloadable library raises GpetError instead
of falling back to anything else.
"""
import ctypes as C
import os

import numpy as np

from .formats import EVENT_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpet.so")

GPET_OK = 0
ERRORS = {-1: "bad argument or state", -2: "missing or malformed input file", -3: "CUDA runtime error",
          -4: "a bounded buffer overflowed", -5: "no CUDA device or kernels not built for it"}

ENTRY_DTYPE = np.dtype([("panel", "<i4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                        ("E", "<f4"), ("crystal", "<i4"), ("depth", "<f4"), ("Edep", "<f4")])

PSF_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                      ("E", "<f4"), ("eventid", "<i4"), ("t", "<f8")])

EXIT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                       ("E", "<f4"), ("nscat", "<i4"), ("t", "<f8"), ("status", "<i4"), ("panel", "<i4")])


class GpetError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gpet error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


class Tuning(C.Structure):
    _fields_ = [("sub_decays", C.c_int64), ("chunk_decays", C.c_int64), ("phantom_blocks_per_sm", C.c_int32),
                ("drain_period", C.c_int32), ("detector_threads", C.c_int32), ("source_threads", C.c_int32),
                ("candidates", C.c_int32), ("sample_decays", C.c_int64), ("ms_default", C.c_double),
                ("ms_tuned", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SinoParams(C.Structure):
    _fields_ = [("n_s", C.c_int32), ("n_phi", C.c_int32), ("n_z", C.c_int32), ("s_max", C.c_float),
                ("z_max", C.c_float), ("class_mask", C.c_int32)]


class RunStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "n_decays", "n_pairs", "n_entered", "n_pulses", "n_hits", "n_threshold", "n_deadtime", "n_singles",
        "n_coinc", "n_true", "n_scatter", "n_random", "n_multiple", "n_overflow", "n_stepcap")] + [
        (n, C.c_double) for n in ("ms_total", "ms_source_phantom", "ms_detector", "ms_digitizer",
                                  "ms_coincidence")] + [
        ("kernel_launches", C.c_int64), ("phantom_steps", C.c_int64), ("detector_steps", C.c_int64),
        ("ms_source", C.c_double), ("ms_phantom", C.c_double), ("n_surrogate", C.c_int64),
        ("ms_surrogate", C.c_double), ("n_noise", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_LIB = None


def load_library(path=None):
    """Load libgpet.so (built by gpet_gb300.build). Raises GpetError when absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise GpetError(-5, "%s is missing: run gpet_gb300.build.build() first" % p)
    L = C.CDLL(p)
    vp, i32, i64, u8p = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_uint8)
    L.gpet_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.gpet_destroy.argtypes = [vp]
    L.gpet_destroy.restype = None
    L.gpet_last_error.argtypes = [vp]
    L.gpet_last_error.restype = C.c_char_p
    L.gpet_set_option.argtypes = [vp, C.c_char_p, C.c_char_p]
    L.gpet_load_config.argtypes = [vp, C.c_char_p]
    L.gpet_load_tables.argtypes = [vp, C.c_char_p]
    L.gpet_set_phantom.argtypes = [vp, vp, vp, vp, vp, vp]
    L.gpet_load_geometry.argtypes = [vp, C.c_char_p]
    L.gpet_set_source_file.argtypes = [vp, C.c_char_p, C.c_float, C.c_float]
    L.gpet_set_source_psf.argtypes = [vp, vp, i64, C.c_int]
    L.gpet_run.argtypes = [vp, C.POINTER(RunStats)]
    L.gpet_run_batched.argtypes = [C.POINTER(vp), i32, C.POINTER(RunStats)]
    L.gpet_autotune.argtypes = [vp, i64, C.POINTER(Tuning)]
    f32p = C.POINTER(C.c_float)
    L.gpet_get_entries.argtypes = [vp, vp, i64, C.POINTER(i64)]
    L.gpet_get_source_records.argtypes = [vp, vp, i64, C.POINTER(i64)]
    L.gpet_sinogram.argtypes = [vp, C.POINTER(SinoParams), vp]
    L.gpet_get_phantom_records.argtypes = [vp, vp, i64, C.POINTER(i64)]
    L.gpet_surrogate_create.argtypes = [vp, C.c_uint64, C.POINTER(vp)]
    L.gpet_surrogate_destroy.argtypes = [vp]
    L.gpet_surrogate_destroy.restype = None
    L.gpet_surrogate_last_error.argtypes = [vp]
    L.gpet_surrogate_last_error.restype = C.c_char_p
    L.gpet_surrogate_param_count.argtypes = [vp]
    L.gpet_surrogate_param_count.restype = i64
    L.gpet_surrogate_get_params.argtypes = [vp, vp, i64]
    L.gpet_surrogate_set_params.argtypes = [vp, vp, i64]
    L.gpet_surrogate_set_domain.argtypes = [vp, C.c_float, C.c_float, C.c_float, vp, i32]
    L.gpet_surrogate_grad.argtypes = [vp, vp, i64, f32p, vp]
    L.gpet_surrogate_forward.argtypes = [vp, vp, i64, vp]
    L.gpet_surrogate_train.argtypes = [vp, vp, i64, i32, i32, C.c_float, C.c_uint64, vp]
    L.gpet_surrogate_calibrate.argtypes = [vp, vp, i64, i32, C.POINTER(C.c_float)]
    L.gpet_surrogate_get_cell_weights.argtypes = [vp, vp, i64]
    L.gpet_surrogate_set_cell_weights.argtypes = [vp, vp, i64]
    L.gpet_set_surrogate.argtypes = [vp, vp]
    L.gpet_umma_selftest.argtypes = [C.c_int, vp, vp, i32, i32, vp]
    L.gpet_digitize.argtypes = [vp, vp, vp, vp, i64, C.POINTER(RunStats)]
    L.gpet_get_singles.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    L.gpet_get_pulses.argtypes = [vp, vp, vp, vp, i64, C.POINTER(i64)]
    L.gpet_get_coincidences.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    L.gpet_get_singles_async.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    L.gpet_get_coincidences_async.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    L.gpet_wait_copies.argtypes = [vp]
    L.gpet_get_hits.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    L.gpet_get_exits.argtypes = [vp, vp, i64, C.POINTER(i64)]
    L.gpet_write_outputs.argtypes = [vp, C.c_char_p]
    L.gpet_get_panels.argtypes = [vp, vp, i32, C.POINTER(i32)]
    L.gpet_get_counts.argtypes = [vp, vp]
    L.gpet_get_source_layout.argtypes = [vp, vp, vp, i32, C.POINTER(i32)]
    L.gpet_get_majorant.argtypes = [vp, C.c_int, vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.gpet_get_table.argtypes = [vp, C.c_int, vp, i64, C.POINTER(i64)]
    if path is None:
        _LIB = L
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Context:
    """One simulation context on one GPU (gpet_create / gpet_destroy)."""

    def __init__(self, device=0, lib=None):
        self.L = lib or load_library()
        h = C.c_void_p()
        rc = self.L.gpet_create(device, C.byref(h))
        if rc != GPET_OK:
            raise GpetError(rc, "gpet_create(device=%d) failed" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.gpet_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != GPET_OK:
            raise GpetError(rc, self.L.gpet_last_error(self.h).decode(errors="replace"))

    # ---- inputs
    def set_option(self, key, value):
        self._ck(self.L.gpet_set_option(self.h, str(key).encode(), str(value).encode()))

    def set_options(self, opts):
        for k, v in opts.items():
            self.set_option(k, v)

    def load_config(self, path):
        self._ck(self.L.gpet_load_config(self.h, os.fspath(path).encode()))

    def load_tables(self, data_dir):
        self._ck(self.L.gpet_load_tables(self.h, os.fspath(data_dir).encode()))

    def set_phantom(self, mat, den, dims, offset, size):
        mat = np.ascontiguousarray(mat, np.int32)
        den = np.ascontiguousarray(den, np.float32)
        d = np.asarray(dims, np.int32)
        o = np.asarray(offset, np.float32)
        s = np.asarray(size, np.float32)
        self._ck(self.L.gpet_set_phantom(self.h, _ptr(mat), _ptr(den), _ptr(d), _ptr(o), _ptr(s)))

    def load_geometry(self, path):
        self._ck(self.L.gpet_load_geometry(self.h, os.fspath(path).encode()))

    def set_source_file(self, path, tstart, tend):
        self._ck(self.L.gpet_set_source_file(self.h, os.fspath(path).encode(), tstart, tend))

    def set_source_psf(self, records, ptype):
        r = np.ascontiguousarray(records, np.float64).reshape(-1, 8)
        self._ck(self.L.gpet_set_source_psf(self.h, _ptr(r), len(r), ptype))

    # ---- run
    def run(self):
        st = RunStats()
        self._ck(self.L.gpet_run(self.h, C.byref(st)))
        return st.as_dict()

    def autotune(self, sample_decays=0):
        """Time launch shapes on a sample of this workload and keep the fastest
        (gpet_autotune); returns the chosen shape and the sample's times."""
        t = Tuning()
        self._ck(self.L.gpet_autotune(self.h, int(sample_decays), C.byref(t)))
        return t.as_dict()

    def digitize(self, pulses, scat, slot):
        pulses = np.ascontiguousarray(pulses, EVENT_DTYPE)
        scat = np.ascontiguousarray(scat, np.uint8)
        slot = np.ascontiguousarray(slot, np.uint8)
        st = RunStats()
        self._ck(self.L.gpet_digitize(self.h, _ptr(pulses), _ptr(scat), _ptr(slot), len(pulses), C.byref(st)))
        return st.as_dict()

    # ---- outputs
    def _count(self, fn, *nulls):
        n = C.c_int64()
        self._ck(fn(self.h, *nulls, 0, C.byref(n)))
        return n.value

    def singles(self, out=None):
        """Singles in time order and their phantom-scatter flags. `out` may
        give (events, flags) arrays to fill (e.g. views of pinned memory); the
        returned arrays are then their first n entries."""
        n = self._count(self.L.gpet_get_singles, None, None)
        if out is not None and len(out[0]) >= n and len(out[1]) >= n:
            ev, sc = out[0][:n], out[1][:n]
        else:
            ev = np.zeros(n, EVENT_DTYPE)
            sc = np.zeros(n, np.uint8)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_singles(self.h, _ptr(ev), _ptr(sc), n, C.byref(m)))
        return ev, sc

    def pulses(self):
        n = self._count(self.L.gpet_get_pulses, None, None, None)
        ev = np.zeros(n, EVENT_DTYPE)
        sc = np.zeros(n, np.uint8)
        sl = np.zeros(n, np.uint8)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_pulses(self.h, _ptr(ev), _ptr(sc), _ptr(sl), n, C.byref(m)))
        return ev, sc, sl

    def coincidences(self, out=None):
        """Index pairs into the singles and class bytes; `out` as for singles()."""
        n = self._count(self.L.gpet_get_coincidences, None, None)
        if out is not None and len(out[0]) >= n and len(out[1]) >= n:
            pr, cl = out[0][:n], out[1][:n]
        else:
            pr = np.zeros((n, 2), np.int64)
            cl = np.zeros(n, np.uint8)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_coincidences(self.h, _ptr(pr), _ptr(cl), n, C.byref(m)))
        return pr, cl

    def singles_async(self, out):
        """As singles(out=...), but the records reach `out` (page-locked
        arrays, e.g. views of pinned memory, large enough) on the context's
        copy stream while the next run proceeds: the returned views hold them
        after wait_copies()."""
        n = self._count(self.L.gpet_get_singles_async, None, None)
        if len(out[0]) < n or len(out[1]) < n:
            raise ValueError("output arrays too small for %d singles" % n)
        ev, sc = out[0][:n], out[1][:n]
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_singles_async(self.h, _ptr(ev), _ptr(sc), n, C.byref(m)))
        return ev, sc

    def coincidences_async(self, out):
        """As coincidences(out=...), asynchronously as singles_async()."""
        n = self._count(self.L.gpet_get_coincidences_async, None, None)
        if len(out[0]) < n or len(out[1]) < n:
            raise ValueError("output arrays too small for %d coincidences" % n)
        pr, cl = out[0][:n], out[1][:n]
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_coincidences_async(self.h, _ptr(pr), _ptr(cl), n, C.byref(m)))
        return pr, cl

    def wait_copies(self):
        """Waits for the copies of singles_async / coincidences_async."""
        self._ck(self.L.gpet_wait_copies(self.h))

    def hits(self):
        n = self._count(self.L.gpet_get_hits, None, None)
        ids = np.zeros((n, 5), np.int32)
        f = np.zeros((n, 5), np.float32)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_hits(self.h, _ptr(ids), _ptr(f), n, C.byref(m)))
        return ids, f

    def exits(self):
        n = self._count(self.L.gpet_get_exits, None)
        out = np.zeros(n, EXIT_DTYPE)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_exits(self.h, _ptr(out), n, C.byref(m)))
        return out

    def entries(self):
        """Entry records of the last run (option record_entries=1)."""
        n = self._count(self.L.gpet_get_entries, None)
        out = np.zeros(n, ENTRY_DTYPE)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_entries(self.h, _ptr(out), n, C.byref(m)))
        return out

    def sinogram(self, n_s, n_phi, n_z, s_max, z_max, classes=(0, 1, 2)):
        """The last run's coincidences as a [n_z][n_phi][n_s] sinogram
        (gpet_sinogram); classes: 0 true, 1 scatter, 2 random."""
        p = SinoParams(n_s, n_phi, n_z, s_max, z_max, sum(1 << k for k in classes))
        out = np.zeros((n_z, n_phi, n_s), np.uint32)
        self._ck(self.L.gpet_sinogram(self.h, C.byref(p), _ptr(out)))
        return out

    def source_records(self):
        """Emitted photons of the last run (option record_source=1)."""
        n = self._count(self.L.gpet_get_source_records, None)
        out = np.zeros(n, PSF_DTYPE)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_source_records(self.h, _ptr(out), n, C.byref(m)))
        return out

    def phantom_records(self):
        """Photons leaving the phantom in the last run (option record_exits=1)."""
        n = self._count(self.L.gpet_get_phantom_records, None)
        out = np.zeros(n, PSF_DTYPE)
        m = C.c_int64()
        if n:
            self._ck(self.L.gpet_get_phantom_records(self.h, _ptr(out), n, C.byref(m)))
        return out

    def set_surrogate(self, sur):
        self._ck(self.L.gpet_set_surrogate(self.h, sur.h if sur is not None else None))
        self._sur = sur      # keeps it alive while attached

    def write_outputs(self, out_dir):
        self._ck(self.L.gpet_write_outputs(self.h, os.fspath(out_dir).encode()))

    # ---- introspection
    def panels(self):
        n = C.c_int32()
        self._ck(self.L.gpet_get_panels(self.h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 32), np.float32)
        self._ck(self.L.gpet_get_panels(self.h, _ptr(out), n.value, C.byref(n)))
        return out

    def counts(self):
        out = np.zeros(4, np.int32)
        self._ck(self.L.gpet_get_counts(self.h, _ptr(out)))
        return tuple(int(v) for v in out)

    def source_layout(self):
        n = C.c_int32()
        self._ck(self.L.gpet_get_source_layout(self.h, None, None, 0, C.byref(n)))
        first = np.zeros(n.value, np.int64)
        count = np.zeros(n.value, np.int64)
        if n.value:
            self._ck(self.L.gpet_get_source_layout(self.h, _ptr(first), _ptr(count), n.value, C.byref(n)))
        return first, count

    def majorant(self, which):
        tab = np.zeros(4096, np.float32)
        e0, ide = C.c_float(), C.c_float()
        self._ck(self.L.gpet_get_majorant(self.h, which, _ptr(tab), C.byref(e0), C.byref(ide)))
        return tab, e0.value, ide.value

    def table(self, which):
        n = C.c_int64()
        self._ck(self.L.gpet_get_table(self.h, which, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.float32)
        self._ck(self.L.gpet_get_table(self.h, which, _ptr(out), n.value, C.byref(n)))
        return out


def run_batched(contexts):
    """Run several loaded contexts (one device) as one job (gpet_run_batched);
    returns each simulation's stats. Each context then reads its own results."""
    ctxs = list(contexts)
    if not ctxs:
        return []
    L = ctxs[0].L
    arr = (C.c_void_p * len(ctxs))(*[c.h for c in ctxs])
    st = (RunStats * len(ctxs))()
    rc = L.gpet_run_batched(arr, len(ctxs), st)
    if rc != GPET_OK:
        msgs = "; ".join(sorted({c.L.gpet_last_error(c.h).decode(errors="replace") for c in ctxs} - {""}))
        raise GpetError(rc, msgs)
    return [s.as_dict() for s in st]


class Surrogate:
    """Learned detector response for a context's detector (gpet_surrogate_*)."""

    def __init__(self, ctx, seed=1):
        self.L = ctx.L
        h = C.c_void_p()
        rc = self.L.gpet_surrogate_create(ctx.h, seed, C.byref(h))
        if rc != GPET_OK:
            raise GpetError(rc, "gpet_surrogate_create failed (detector not supported or no GPU)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.gpet_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != GPET_OK:
            raise GpetError(rc, self.L.gpet_surrogate_last_error(self.h).decode(errors="replace"))

    @property
    def param_count(self):
        return int(self.L.gpet_surrogate_param_count(self.h))

    def params(self):
        out = np.zeros(self.param_count, np.float32)
        self._ck(self.L.gpet_surrogate_get_params(self.h, _ptr(out), len(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self.L.gpet_surrogate_set_params(self.h, _ptr(p), len(p)))

    def set_domain(self, e_lo, e_hi, margin, panel_ok=None):
        po = None if panel_ok is None else np.ascontiguousarray(panel_ok, np.uint8)
        self._ck(self.L.gpet_surrogate_set_domain(self.h, e_lo, e_hi, margin, _ptr(po),
                                                  0 if po is None else len(po)))

    def grad(self, rec):
        rec = np.ascontiguousarray(rec, ENTRY_DTYPE)
        g = np.zeros(self.param_count, np.float32)
        loss = C.c_float()
        self._ck(self.L.gpet_surrogate_grad(self.h, _ptr(rec), len(rec), C.byref(loss), _ptr(g)))
        return loss.value, g

    def forward(self, rec):
        rec = np.ascontiguousarray(rec, ENTRY_DTYPE)
        out = np.zeros((len(rec), 208), np.float32)
        self._ck(self.L.gpet_surrogate_forward(self.h, _ptr(rec), len(rec), _ptr(out)))
        return out

    def cell_weights(self):
        """Factorised head: the (energy class, row, column) cell weights [2, 32, 32]."""
        w = np.zeros(2048, np.float32)
        self._ck(self.L.gpet_surrogate_get_cell_weights(self.h, _ptr(w), 2048))
        return w.reshape(2, 32, 32)

    def set_cell_weights(self, w):
        w = np.ascontiguousarray(w, np.float32).reshape(-1)
        self._ck(self.L.gpet_surrogate_set_cell_weights(self.h, _ptr(w), len(w)))

    def calibrate(self, rec, iters=3):
        """Match the expected (energy class, crystal) and energy-bin counts of
        the records in the current domain (gpet_surrogate_calibrate); returns
        the last pass's largest |log(observed / expected)|."""
        rec = np.ascontiguousarray(rec, ENTRY_DTYPE)
        adj = C.c_float()
        self._ck(self.L.gpet_surrogate_calibrate(self.h, _ptr(rec), len(rec), int(iters), C.byref(adj)))
        return adj.value

    # layer shapes of the parameter vector (gpet_surrogate.h): weights [out][in], then biases
    LAYERS = ((16, 256), (256, 256), (256, 256), (256, 256), (256, 208))

    def save(self, path, domain, **meta):
        """Write the parameters for inference: the weight matrices rounded to
        bf16 (the precision the tensor-core forward uses, so inference is
        unchanged) as 16-bit patterns, biases and the panel embedding in
        float32, the cell weights of a factorised head, the validated domain
        (e_lo, e_hi, margin) and `meta`."""
        p = self.params()
        w_bits, rest, off = [], [], 0
        for fin, fout in self.LAYERS:
            w = np.ascontiguousarray(p[off:off + fin * fout], np.float32).view(np.uint32)
            w_bits.append(((w + 0x7FFF + ((w >> 16) & 1)) >> 16).astype(np.uint16))
            off += fin * fout
            rest.append(p[off:off + fout])
            off += fout
        np.savez_compressed(path, weights_bf16=np.concatenate(w_bits), biases=np.concatenate(rest),
                            embedding=p[off:], domain=np.array(domain, np.float32),
                            cell_weights=self.cell_weights(), meta=np.array(repr(meta)))

    def load(self, path):
        """Set the parameters and domain saved by save(); returns its meta."""
        import ast
        z = np.load(path)
        wb, b, emb = z["weights_bf16"], z["biases"], z["embedding"]
        parts, wo, bo = [], 0, 0
        for fin, fout in self.LAYERS:
            parts.append((wb[wo:wo + fin * fout].astype(np.uint32) << 16).view(np.float32))
            parts.append(b[bo:bo + fout])
            wo += fin * fout
            bo += fout
        parts.append(emb)
        self.set_params(np.concatenate(parts).astype(np.float32))
        d = z["domain"]
        self.set_domain(float(d[0]), float(d[1]), float(d[2]))
        if "cell_weights" in z.files:
            self.set_cell_weights(z["cell_weights"])
        return ast.literal_eval(str(z["meta"]))

    def train(self, rec, epochs=1, batch=8192, lr=1e-3, seed=7):
        rec = np.ascontiguousarray(rec, ENTRY_DTYPE)
        losses = np.zeros(epochs, np.float32)
        self._ck(self.L.gpet_surrogate_train(self.h, _ptr(rec), len(rec), epochs, batch, lr, seed, _ptr(losses)))
        return losses
