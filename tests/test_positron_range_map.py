"""The positron range's closed form for walks in voxels of one density.

setPositronRange (gPET_kernals.cu:347-418) walks a positron through the
voxels until the density-weighted path length reaches the sampled range r.
Where every voxel the walk reads has one density rho, its end point is
x + (r / rho) * d / r, and both the oracle and the CUDA kernels take that
closed form instead of the walk when a per-voxel map says the voxels within
reach are uniform. These CPU tests check the map against its definition by
brute force and the closed form against the full walk on the same random
words (the oracle's FP32 build, which the kernels match bit for bit)."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))

PRMAX = 6


def _map_by_definition(den):
    """R = the largest radius <= PRMAX such that every voxel within that
    Chebyshev distance has the voxel's density bits and lies in [1, n-2] on
    every axis; -1 where the voxel itself is outside that range."""
    nz, ny, nx = den.shape
    bits = den.view(np.uint32)
    out = np.full(den.shape, -1, np.int8)
    for z in range(1, nz - 1):
        for y in range(1, ny - 1):
            for x in range(1, nx - 1):
                r = 0
                for k in range(1, PRMAX + 1):
                    if x - k < 1 or y - k < 1 or z - k < 1 or x + k > nx - 2 or y + k > ny - 2 or z + k > nz - 2:
                        break
                    cube = bits[z - k:z + k + 1, y - k:y + k + 1, x - k:x + k + 1]
                    if not np.all(cube == bits[z, y, x]):
                        break
                    r = k
                out[z, y, x] = r
    return out


@pytest.mark.parametrize("shape", [(17, 19, 23), (1, 1, 1), (2, 3, 4), (5, 5, 5), (3, 40, 7)])
def test_map_matches_its_definition(oracle_mod, shape):
    rng = np.random.default_rng(7)
    nz, ny, nx = shape
    den = np.ones((nz, ny, nx), np.float32)
    for _ in range(5):   # boxes of other densities
        z0, y0, x0 = rng.integers(0, [nz, ny, nx])
        dz, dy, dx = rng.integers(1, 7, 3)
        den[z0:z0 + dz, y0:y0 + dy, x0:x0 + dx] = rng.choice([0.3, 1.85, 1.0000001])
    if shape == (17, 19, 23):
        den[3, 17, 5] = -0.0   # same value as 0.0, other bits: not uniform with a 0.0 neighbour
    s = oracle_mod._Scene()
    s.nx, s.ny, s.nz = nx, ny, nz
    s.den = den.ctypes.data_as(C.POINTER(C.c_float))
    got = np.empty(den.size, np.int8)
    oracle_mod.lib().oracle_build_prmap(C.byref(s), got.ctypes.data_as(C.POINTER(C.c_int8)))
    want = _map_by_definition(den)
    assert np.array_equal(got.reshape(den.shape), want)
    if shape == (17, 19, 23):
        assert (want >= 2).sum() > 100 and (want == 0).sum() > 100
    if min(shape) < 3:
        assert (want == -1).all()   # no voxel in [1, n-2] on every axis


def _anisotropic_scene(d):
    """Voxels of 0.5 x 0.5 x 2 mm (x, y, z): water with a bone slab across z
    and a lung ball, so that the closed form's reach bound (in units of the
    smallest voxel side) is tried where one axis is four times coarser."""
    import os
    from gpet_gb300 import formats as F, scenes
    nx, ny, nz = 96, 96, 24
    c = scenes._base_config(d, (nx, ny, nz), (4.8, 4.8, 4.8), (-2.4, -2.4, -2.4))
    c.useprange = 1
    z = -2.4 + (np.arange(nz) + 0.5) * 0.2
    y = -2.4 + (np.arange(ny) + 0.5) * 0.05
    x = -2.4 + (np.arange(nx) + 0.5) * 0.05
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    mat = np.full((nz, ny, nx), scenes.MAT_WATER, np.int32)
    den = np.full((nz, ny, nx), 1.0, np.float32)
    slab = np.abs(Z - 0.5) < 0.3
    mat[slab], den[slab] = scenes.MAT_BONE, 1.85
    ball = X ** 2 + (Y - 0.6) ** 2 + (Z + 0.8) ** 2 < 0.7 ** 2
    mat[ball], den[ball] = scenes.MAT_TISSUE, 0.3
    F.write_phantom(c.matfile, c.denfile, mat, den)
    F.write_geo(c.geofile, 8, (0, 0, 1), 45.0, (scenes.MAT_LYSO, scenes.MAT_AIR), (7.1, 0.001025),
                scenes.ring_panel0(8.0, 8, 8, 0.298, 0.002, 2.0))
    F.write_sources(c.sourcefile, [1_000_000_000], [0], [1], [(0, 0, 0, 2.2, 4.6, 0)])
    F.write_config(os.path.join(d, "input_PET.in"), c)
    return scenes.Scene(d, os.path.join(d, "input_PET.in"), {"n_decays": 1000, "seed": 3}, "anisotropic voxels")


@pytest.mark.parametrize("nvox", [48, 128, "anisotropic"])
def test_closed_form_equals_walk(oracle_mod, data_dir, tmp_path, nvox):
    """On the positron workload's phantom (water, bone rods, lung sphere),
    and on one of anisotropic voxels, positrons of the F-18 range started all
    over the source cylinder end where the full walk ends them, to the
    rounding of the walk's steps, with the same random words; most of them
    take the closed form."""
    import pins
    from gpet_gb300 import scenes
    if nvox == "anisotropic":
        sc = _anisotropic_scene(str(tmp_path))
    else:
        sc = scenes.positron(str(tmp_path), n_decays=1000, nvox=nvox)
    o = oracle_mod.OracleScene(sc.config_path, sc.options, data_dir, base_dir=sc.directory)
    with_map = o.s
    without = oracle_mod._Scene.from_buffer_copy(o.s)
    without.prmap = C.POINTER(C.c_int8)()
    L = pins.oracle_lib()
    rng = np.random.default_rng(11)
    n = 4000
    rr = 3.0 * np.sqrt(rng.random(n))
    ph = 2 * np.pi * rng.random(n)
    x = np.stack([rr * np.cos(ph), rr * np.sin(ph), 4.4 * (rng.random(n) - 0.5)], 1).astype(np.float32)
    ek = rng.random(n) * 633e3
    tape = rng.integers(1, 2 ** 32 - 1, size=(n, pins.TAPE), dtype=np.uint64).astype(np.uint32)
    ends = {}
    for name, S in (("map", with_map), ("walk", without)):
        out = np.zeros((n, 3))
        used = np.zeros(n, np.int64)
        u = C.c_int64()
        for i in range(n):
            L.oracle_tape_positron_range(C.byref(S), pins._p(np.ascontiguousarray(x[i]), pins._FP), float(ek[i]),
                                         None, pins._p(np.ascontiguousarray(tape[i]), pins._UP), pins.TAPE,
                                         pins._p(out[i], pins._DP), C.byref(u))
            used[i] = u.value
        ends[name] = (out, used)
    assert np.array_equal(ends["map"][1], ends["walk"][1])
    dist = np.linalg.norm(ends["map"][0] - ends["walk"][0], axis=1)
    assert dist.max() < 2e-6
    moved = np.linalg.norm(ends["walk"][0] - x, axis=1)
    assert np.median(moved) > 0.01                    # ranges of a fraction of a millimetre
    exact = dist == 0.0
    assert exact.mean() < 0.9                          # most positrons took the closed form (not bit-equal)
    assert (o.prmap >= 2).mean() > 0.3
