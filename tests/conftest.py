import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

DATA = os.path.join(ROOT, "data")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgpet.so")


def _ensure_surfaces():
    if not (os.path.exists(os.path.join(DATA, "input4gPET.cmpsf")) and
            os.path.exists(os.path.join(DATA, "input4gPET.rayff"))):
        import subprocess
        subprocess.check_call([sys.executable, os.path.join(DATA, "make_surfaces.py"), DATA])


@pytest.fixture(scope="session")
def data_dir():
    _ensure_surfaces()
    return DATA


@pytest.fixture(scope="session")
def oracle_mod(data_dir):
    import bridge
    bridge.build()
    return bridge


@pytest.fixture(scope="session")
def gpet_lib(data_dir):
    """The native library, built for sm_103a; GPU tests fail loudly without it."""
    from gpet_gb300 import build as B
    B.build()
    from gpet_gb300 import api
    return api.load_library()


@pytest.fixture(scope="session")
def scene_small(tmp_path_factory, data_dir):
    from gpet_gb300 import scenes
    d = tmp_path_factory.mktemp("small")
    return scenes.small(str(d), n_decays=20000, nvox=40)


@pytest.fixture(scope="session")
def scene_positron(tmp_path_factory, data_dir):
    from gpet_gb300 import scenes
    d = tmp_path_factory.mktemp("positron")
    return scenes.positron(str(d), n_decays=20000, nvox=48)


@pytest.fixture(scope="session")
def scene_large(tmp_path_factory, data_dir):
    """The whole-body configuration (48 panels at 49 cm, body phantom) on a
    coarse 64 x 64 x 128 grid of 0.8 cm voxels."""
    from gpet_gb300 import scenes
    d = tmp_path_factory.mktemp("large")
    return scenes.large(str(d), n_decays=300000, dims=(64, 64, 128), voxel_cm=0.8)


def make_ctx(scene, data_dir, **extra):
    from gpet_gb300 import api
    ctx = api.Context(0)
    opts = dict(scene.options)
    opts.update(extra)
    opts["data_dir"] = data_dir
    opts["base_dir"] = scene.directory
    ctx.set_options(opts)
    ctx.load_config(scene.config_path)
    return ctx


def oracle_for(scene, data_dir, panels=None, **extra):
    import bridge
    opts = dict(scene.options)
    opts.update(extra)
    return bridge.OracleScene(scene.config_path, opts, data_dir, panels=panels, base_dir=scene.directory)


def two_sample_chi2(a, b):
    """p-value of the two-sample chi-square of histograms a and b (same bins,
    empty bins of both dropped)."""
    from scipy import stats
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    m = (a + b) > 0
    a, b = a[m], b[m]
    ka = np.sqrt(b.sum() / a.sum())
    kb = np.sqrt(a.sum() / b.sum())
    chi2 = np.sum((ka * a - kb * b) ** 2 / (a + b))
    return stats.chi2.sf(chi2, max(len(a) - 1, 1))


def within_sigma(x, y, k=3.0):
    """Two Poisson counts agree within k standard deviations of their difference."""
    return abs(x - y) <= k * np.sqrt(x + y + 1.0)


def event_key_sort(ev, slot):
    order = np.lexsort((slot, ev["parn"]))
    return ev[order], slot[order], order
