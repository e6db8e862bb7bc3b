"""The positron range at its edges, GPU against the FP32 oracle bit for bit.

setPositronRange (gPET_kernals.cu:347-418) is taken three ways on the GPU:
the closed form where the start voxel's neighbourhood is of one density, a
jump through that neighbourhood followed by the voxel walk in k_walk, and
the walk alone (k_walk's four lists by estimated length). This scene puts
positrons of a long-range isotope (O-15, 1.7 MeV end point) into every
case: decays outside the phantom and in its index-0 layer (the source
cylinder is wider and longer than the phantom), a slab of zero density
(the walk crosses it without covering range), a bone plate one voxel thick,
a lung block, isolated voxels of another density and the phantom's far
faces. The emitted photons' phase-space records hold each positron's end
point; they, the singles and the coincidences must equal the oracle's.
"""
import os

import numpy as np
import pytest

from conftest import make_ctx, oracle_for

pytestmark = pytest.mark.gpu


def _edge_scene(d, n_decays):
    from gpet_gb300 import formats as F, scenes
    n, size = 32, 3.2
    c = scenes._base_config(d, (n, n, n), (size, size, size), (-size / 2, -size / 2, -size / 2))
    c.useprange = 1
    c.dlevel, c.dtype, c.dtime = 2, 0, 0.3
    mat = np.full((n, n, n), scenes.MAT_WATER, np.int32)    # [z][y][x]
    den = np.full((n, n, n), 1.0, np.float32)
    den[:, :, 10:12] = 0.0                                   # zero density, two voxels along x
    mat[:, 20, :] = scenes.MAT_BONE                          # bone plate one voxel thick
    den[:, 20, :] = 1.85
    mat[5:12, 5:12, 20:28] = scenes.MAT_TISSUE               # lung block
    den[5:12, 5:12, 20:28] = 0.3
    rng = np.random.default_rng(5)
    iv = rng.integers(0, n, size=(60, 3))
    den[iv[:, 0], iv[:, 1], iv[:, 2]] = 1.2                  # isolated voxels
    F.write_phantom(c.matfile, c.denfile, mat, den)
    F.write_geo(c.geofile, 8, (0, 0, 1), 45.0, (scenes.MAT_LYSO, scenes.MAT_AIR), (7.1, 0.001025),
                scenes.ring_panel0(4.0, 8, 8, 0.15, 0.001, 1.0))
    # isotope row 2 (O-15: half-life 122 s, 1.74 MeV end point), cylinder
    # r = 2.0 cm, 3.6 cm long around a phantom of half-width 1.6 cm
    F.write_sources(c.sourcefile, [1_000_000_000], [2], [1], [(0, 0, 0, 2.0, 3.6, 0)])
    F.write_config(os.path.join(d, "input_PET.in"), c)
    return scenes.Scene(d, os.path.join(d, "input_PET.in"),
                        {"n_decays": n_decays, "seed": 7, "coinc_window_ns": 4.0}, "positron-range edges")


def test_positron_walk_edges_bit_exact(data_dir, gpet_lib, oracle_mod, tmp_path):
    scene = _edge_scene(str(tmp_path), 400000)
    ctx = make_ctx(scene, data_dir, record_source=1)
    st = ctx.run()
    o = oracle_for(scene, data_dir, panels=ctx.panels())
    r = o.run(precision="fp32", source=True)
    src = ctx.source_records()
    osrc = r["source"][r["source"]["t"] > 0]
    assert len(src) == len(osrc) > 700000
    assert np.array_equal(src.view(np.uint8), osrc.view(np.uint8))
    singles, _ = ctx.singles()
    pairs, cls = ctx.coincidences()
    assert np.array_equal(singles.view(np.uint8), r["singles"].view(np.uint8))
    assert np.array_equal(pairs, r["coinc"]) and np.array_equal(cls, r["coinc_class"])
    assert st["n_coinc"] > 0
    # every case was taken: end points outside the phantom (a positron that
    # leaves it finishes its range in air), in the zero slab
    x, y, z = src["x"], src["y"], src["z"]
    assert np.mean(np.abs(x) > 1.6) > 0.01 and np.mean(np.abs(z) > 1.6) > 0.01
    zero_slab = (x >= -0.6) & (x < -0.4) & (np.abs(y) < 1.6) & (np.abs(z) < 1.6)
    assert zero_slab.sum() > 0
    prange = o.prmap.reshape(32, 32, 32)
    assert (prange >= 2).mean() > 0.15 and (prange == 0).mean() > 0.05


def test_positron_walk_anisotropic_voxels_bit_exact(data_dir, gpet_lib, oracle_mod, tmp_path):
    """Voxels of 0.5 x 0.5 x 2 mm: the uniform-density map's reach bound in
    units of the smallest side, the closed form, the jump and the walk give
    the FP32 oracle's end points, singles and coincidences bit for bit."""
    from test_positron_range_map import _anisotropic_scene
    scene = _anisotropic_scene(str(tmp_path))
    scene.options["n_decays"] = 300000
    ctx = make_ctx(scene, data_dir, record_source=1)
    st = ctx.run()
    o = oracle_for(scene, data_dir, panels=ctx.panels())
    r = o.run(precision="fp32", source=True)
    src = ctx.source_records()
    osrc = r["source"][r["source"]["t"] > 0]
    assert len(src) == len(osrc) > 500000
    assert np.array_equal(src.view(np.uint8), osrc.view(np.uint8))
    singles, _ = ctx.singles()
    pairs, cls = ctx.coincidences()
    assert np.array_equal(singles.view(np.uint8), r["singles"].view(np.uint8))
    assert np.array_equal(pairs, r["coinc"]) and np.array_equal(cls, r["coinc_class"])
    assert st["n_singles"] > 1000
