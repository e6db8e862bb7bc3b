"""gpet_digitize_static against gpet_digitize.

gpet_digitize_static is the digitizer for callers that cannot allocate device
memory (code running inside another framework's memory pool, or whose device
memory is fixed when it starts): its working memory is a file-scope device
array, and the caller hands over inputs and outputs in device memory it
already owns. Here that memory comes from torch. The test checks, on two calls
in a row, that it returns exactly what the allocating entry point returns for
the same pulses; the second call is smaller than the first, so anything left
over in the shared array from the first call would show. It also checks that
an input above the stated maximum is refused with a message."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_ctx
from gpet_gb300.formats import EVENT_DTYPE

pytestmark = pytest.mark.gpu

MAX_PULSES = 131072


class DigiParams(C.Structure):
    _fields_ = [("blurpolicy", C.c_int32), ("Eref", C.c_float), ("Rref", C.c_float), ("Eslope", C.c_float),
                ("Sblur", C.c_float), ("Eth", C.c_float), ("dlevel", C.c_int32), ("dtype", C.c_int32),
                ("dtime_us", C.c_float), ("ewin_lo", C.c_float), ("ewin_hi", C.c_float),
                ("coinc_window_ns", C.c_double), ("coinc_policy", C.c_int32), ("moduleN", C.c_int32),
                ("crystalN", C.c_int32), ("seed", C.c_uint64), ("sim_id", C.c_uint32)]


def pulses(n, seed):
    rng = np.random.default_rng(seed)
    ev = np.zeros(n, EVENT_DTYPE)
    ev["parn"] = rng.permutation(4 * n)[:n]
    ev["pann"] = rng.integers(0, 8, n)
    ev["cryn"] = rng.integers(0, 64, n)
    ev["siten"] = ev["pann"] * 64 + ev["cryn"]
    ev["eventid"] = ev["parn"] // 2
    t = np.sort(rng.uniform(0, n * 0.05, n))
    k = rng.integers(1, n, n // 20)
    t[k] = t[k - 1] + 0.002                     # pairs inside one coincidence window
    ev["t"] = rng.permutation(t)
    ev["E"] = rng.uniform(100e3, 700e3, n)
    ev["x"] = rng.uniform(-1, 0, n); ev["y"] = rng.uniform(-1, 1, n); ev["z"] = rng.uniform(-1, 1, n)
    return ev, (rng.random(n) < 0.3).astype(np.uint8), rng.integers(0, 3, n).astype(np.uint8)


def test_static_matches_allocating_entry_point(scene_positron, data_dir, gpet_lib):
    torch = pytest.importorskip("torch")
    from gpet_gb300 import formats as F
    L = gpet_lib
    L.gpet_digitize_static.argtypes = [C.POINTER(DigiParams)] + [C.c_void_p] * 3 + [C.c_int64] + [C.c_void_p] * 2 + \
        [C.c_int64] + [C.c_void_p] * 2 + [C.c_int64, C.POINTER(C.c_int64), C.c_void_p, C.c_char_p, C.c_int32]
    ctx = make_ctx(scene_positron, data_dir)
    cfg = F.read_config(scene_positron.config_path)
    _, mod_n, _, cry_n = ctx.counts()
    prm = DigiParams(cfg.blurpolicy, cfg.eref, cfg.rref, cfg.eslope, cfg.sblur, cfg.eth, cfg.dlevel, cfg.dtype,
                     cfg.dtime, cfg.ewin_lo, cfg.ewin_hi, float(scene_positron.options["coinc_window_ns"]), 0,
                     mod_n, cry_n, int(scene_positron.options["seed"]), 0)
    dev = torch.device("cuda:0")
    cap = MAX_PULSES
    d_singles = torch.zeros(cap * 48, dtype=torch.uint8, device=dev)
    d_sscat = torch.zeros(cap, dtype=torch.uint8, device=dev)
    d_pairs = torch.zeros(cap * 2, dtype=torch.int64, device=dev)
    d_class = torch.zeros(cap, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for n, seed in ((60000, 1), (9000, 2)):
        ev, scat, slot = pulses(n, seed)
        st = ctx.digitize(ev, scat, slot)
        ref_s, ref_sc = ctx.singles()
        ref_p, ref_c = ctx.coincidences()
        d_ev = torch.from_numpy(ev.view(np.uint8).copy()).to(dev)
        d_scat = torch.from_numpy(scat).to(dev)
        d_slot = torch.from_numpy(slot).to(dev)
        counts = (C.c_int64 * 8)()
        err = C.create_string_buffer(256)
        rc = L.gpet_digitize_static(C.byref(prm), d_ev.data_ptr(), d_scat.data_ptr(), d_slot.data_ptr(), n,
                                    d_singles.data_ptr(), d_sscat.data_ptr(), cap, d_pairs.data_ptr(),
                                    d_class.data_ptr(), cap, counts, stream, err, 256)
        assert rc == 0, err.value
        ns, nc = counts[2], counts[3]
        assert (counts[0], counts[1], ns, nc) == (st["n_threshold"], st["n_deadtime"], st["n_singles"], st["n_coinc"])
        assert (counts[4], counts[5], counts[6], counts[7]) == (st["n_true"], st["n_scatter"], st["n_random"],
                                                                st["n_multiple"])
        got = d_singles[: ns * 48].cpu().numpy().view(EVENT_DTYPE)
        assert np.array_equal(got.view(np.uint8), ref_s.view(np.uint8))
        assert np.array_equal(d_sscat[:ns].cpu().numpy(), ref_sc)
        assert np.array_equal(d_pairs[: 2 * nc].cpu().numpy().reshape(-1, 2), ref_p)
        assert np.array_equal(d_class[:nc].cpu().numpy(), ref_c)
        assert nc > 0
    # above the stated maximum: refused, with a message
    n = MAX_PULSES + 1
    d_big = torch.zeros(n * 48, dtype=torch.uint8, device=dev)
    d_b1 = torch.zeros(n, dtype=torch.uint8, device=dev)
    counts = (C.c_int64 * 8)()
    err = C.create_string_buffer(256)
    rc = L.gpet_digitize_static(C.byref(prm), d_big.data_ptr(), d_b1.data_ptr(), d_b1.data_ptr(), n,
                                d_singles.data_ptr(), d_sscat.data_ptr(), cap, d_pairs.data_ptr(), d_class.data_ptr(),
                                cap, counts, stream, err, 256)
    assert rc == -1 and b"exceed the maximum" in err.value
