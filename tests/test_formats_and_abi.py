"""File-format round trips, scene generators, and the C ABI of libgpet.so
(loads and exports every declared symbol; without a GPU it refuses to create
a context instead of falling back to anything)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_config_round_trip(tmp_path):
    from gpet_gb300 import formats as F
    c = F.read_config(os.path.join(ROOT, "tests", "golden", "reference_inputs", "input_PET.in"))
    p = tmp_path / "in.in"
    F.write_config(str(p), c)
    assert F.read_config(str(p)) == c


def test_geo_round_trip(tmp_path):
    from gpet_gb300 import formats as F, scenes
    p0 = scenes.ring_panel0(8.0, 8, 8, 0.298, 0.002, 2.0)
    F.write_geo(str(tmp_path / "r.geo"), 8, (0, 0, 1), 45.0, (8, 0), (7.1, 0.001025), p0)
    g = F.read_geo(str(tmp_path / "r.geo"))
    assert g.counts == (1, 1, 8, 64)
    assert g.det_mat == (8, 0)
    # the ring: panel i's face centre sits at radius 8 cm, i*45 degrees on
    for i in range(8):
        o = g.panels[i][15:18]
        assert np.hypot(o[0], o[1]) == pytest.approx(8.0, abs=1e-5)
        ux = g.panels[i][21:24]
        # local x points at the ring centre; the crystals extend along -x (outward)
        assert np.dot(ux, -o / 8.0) == pytest.approx(1.0, abs=1e-5)
        assert g.panels[i][18] == -1.0


def test_sources_and_isotopes(tmp_path, data_dir):
    from gpet_gb300 import formats as F
    s = F.read_sources(os.path.join(ROOT, "tests", "golden", "reference_inputs", "source.txt"))
    assert len(s.natom) == 7 and s.natom[0] == 9000000 and s.shape[0] == 1
    assert np.allclose(s.coef[6], [0, 0, 1.15, 1.5, 3, 0])
    F.write_sources(str(tmp_path / "s.txt"), s.natom, s.type, s.shape, s.coef)
    s2 = F.read_sources(str(tmp_path / "s.txt"))
    assert np.array_equal(s2.natom, s.natom) and np.array_equal(s2.coef, s.coef)
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    assert iso.halftime[0] == pytest.approx(6586.26) and iso.ratio[0] == pytest.approx(0.97)


def test_scene_generators(tmp_path):
    from gpet_gb300 import formats as F, scenes
    sc = scenes.positron(str(tmp_path), n_decays=1000, nvox=32)
    c = F.read_config(sc.config_path)
    mat, den = F.read_phantom(c.matfile, c.denfile, c.pdim)
    assert set(np.unique(mat)) == {1, 2, 3}
    assert den[mat == 3].min() == pytest.approx(1.85) and den[mat == 2].max() == pytest.approx(0.3)
    assert c.useprange == 1 and (c.dlevel, c.dtype) == (2, 0) and c.dtime == pytest.approx(0.3)
    sm = scenes.small(str(tmp_path / "s"), n_decays=1000, nvox=20)
    c = F.read_config(sm.config_path)
    mat, den = F.read_phantom(c.matfile, c.denfile, c.pdim)
    assert set(np.unique(mat)) == {0, 1}


def test_psf_and_event_readers(tmp_path):
    from gpet_gb300 import formats as F
    rec = np.arange(80, dtype="<f8").reshape(10, 8)
    rec.tofile(tmp_path / "psf.dat")
    assert np.array_equal(F.read_psf(str(tmp_path / "psf.dat")), rec)
    assert len(F.read_psf(str(tmp_path / "psf.dat"), 4)) == 4
    ev = np.zeros(3, F.EVENT_DTYPE)
    ev["t"] = [1.5, 2.5, 3.5]
    ev.tofile(tmp_path / "singles.dat")
    assert np.array_equal(F.read_events(str(tmp_path / "singles.dat"))["t"], ev["t"])


def _declared_symbols():
    syms = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            syms |= set(re.findall(r"\b(gpet_[a-z0-9_]+)\s*\(", txt))
    return sorted(syms)


def test_library_exports_every_declared_symbol(gpet_lib):
    syms = _declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(gpet_lib, s), s


def test_no_gpu_refuses_context(gpet_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = gpet_lib.gpet_create(0, C.byref(h))
    assert rc == -5 and not h.value


def test_null_context_is_an_error(gpet_lib):
    assert gpet_lib.gpet_run(None, None) == -1
    assert gpet_lib.gpet_set_option(None, b"seed", b"1") == -1
    assert gpet_lib.gpet_last_error(None) == b"null context"


def test_phase_space_reader(tmp_path):
    from gpet_gb300 import formats as F
    rng = np.random.default_rng(2)
    st = rng.standard_normal((5, 7)).astype("<f4")
    ids = np.arange(5, dtype="<i4") * 3
    t = rng.uniform(1, 2, 5)
    st.tofile(str(tmp_path / "outphantom.dat"))
    ids.tofile(str(tmp_path / "idphantom.dat"))
    t.tofile(str(tmp_path / "timephantom.dat"))
    r = F.read_phase_space(str(tmp_path), "phantom")
    assert np.array_equal(r["uy"], st[:, 4]) and np.array_equal(r["eventid"], ids) and np.array_equal(r["t"], t)
    (tmp_path / "timephantom.dat").write_bytes(b"\0" * 8)
    with pytest.raises(ValueError):
        F.read_phase_space(str(tmp_path), "phantom")
