"""The native loaders (C++) and the Python readers are independent
implementations of gPET's parsers; both must see the same numbers."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, make_ctx

pytestmark = pytest.mark.gpu


def test_tables_identical(scene_small, data_dir, gpet_lib):
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_small, data_dir)
    T = F.read_tables(data_dir)
    for which, arr in enumerate((T.lamph, T.compt, T.phote, T.rayle, T.cmpsf, T.rayff)):
        assert np.array_equal(ctx.table(which), arr.ravel()), which


def test_geometry_and_counts(scene_positron, data_dir, gpet_lib):
    from gpet_gb300 import formats as F
    ctx = make_ctx(scene_positron, data_dir)
    g = F.read_geo(os.path.join(scene_positron.directory, "ring.geo"))
    assert np.allclose(ctx.panels(), g.panels, atol=2e-6)
    assert ctx.counts() == g.counts


def test_config8_geometry(data_dir, gpet_lib, tmp_path):
    from gpet_gb300 import api
    ctx = api.Context(0)
    ctx.load_tables(data_dir)
    ctx.load_geometry(os.path.join(GOLDEN, "reference_inputs", "config8.geo"))
    assert ctx.counts() == (9, 117, 8, 64)


def test_source_layout_matches(data_dir, gpet_lib, tmp_path):
    import bridge
    from gpet_gb300 import api, formats as F
    ctx = api.Context(0)
    ctx.load_tables(data_dir)
    src = os.path.join(GOLDEN, "reference_inputs", "source.txt")
    ctx.set_source_file(src, 0.0, 120.0)
    first, count = ctx.source_layout()
    s = F.read_sources(src)
    iso = F.read_isotopes(os.path.join(data_dir, "isotopes.txt"))
    f2, c2 = bridge.source_layout(s.natom, s.type, iso.halftime, 0.0, 120.0)
    assert np.array_equal(first, f2) and np.array_equal(count, c2)
    ctx.set_option("n_decays", 1000003)
    first, count = ctx.source_layout()
    f2, c2 = bridge.source_layout(s.natom, s.type, iso.halftime, 0.0, 120.0, 1000003)
    assert count.sum() == 1000003 and np.array_equal(count, c2)


def test_bad_inputs_fail_cleanly(data_dir, gpet_lib, tmp_path):
    from gpet_gb300 import api
    ctx = api.Context(0)
    with pytest.raises(api.GpetError) as e:
        ctx.load_tables(str(tmp_path))
    assert e.value.code == -2
    with pytest.raises(api.GpetError):
        ctx.run()
    with pytest.raises(api.GpetError):
        ctx.set_option("no_such_option", "1")
    ctx.load_tables(data_dir)
    with pytest.raises(api.GpetError):
        ctx.set_phantom(np.full(8, 99, np.int32), np.ones(8, np.float32), (2, 2, 2), (0, 0, 0), (1, 1, 1))
    (tmp_path / "bad.geo").write_text("panel repetition times\n")
    with pytest.raises(api.GpetError):
        ctx.load_geometry(str(tmp_path / "bad.geo"))
