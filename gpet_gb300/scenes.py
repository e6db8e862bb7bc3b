"""Seeded synthetic workloads written in gPET's own input formats.

The reference ships no benchmark inputs (its example phantom and PSF are
missing blobs), so each workload is generated here and written as the files a
gPET user would have: input_PET.in, mat.dat/den.dat, a .geo ring and a
source.txt. Options that the reference format has no key for (exact decay
count, seed, coincidence window) are returned separately and passed through
gpet_set_option.

Workloads (materials are row indices of data/input4gPET.matter):
  small    : 1e6 back-to-back pairs from a point at the origin; 200^3 voxels
             over a 1 cm cube, water cylinder r=0.4 cm along z in air; ring of
             8 LYSO panels at 4 cm, 8x8 crystals of 1.5x1.5x10 mm.
  positron : F-18 uniform in a 3 cm-radius cylinder, 128^3 voxels of 0.5 mm;
             water with four bone rods (r 3 mm) and a lung sphere (rho 0.3,
             r 8 mm); 1e8 decays, positron range on; the ring scaled by 2
             (8 cm, 3 mm crystals, 20 mm deep); paralyzable dead time 300 ns
             per block.
  large    : 1e9 F-18 decays in 256x256x512 voxels of 2 mm (30x20 cm body
             ellipse, lungs, spine); 48 panels of 16x16 4x4x20 mm crystals.
  batched  : 64 simulations of uneven size for one batched job (phantoms
             64^3-256^3, 1e5-1e7 decays each, point or cylinder sources).
  beds     : the large acquisition in 8 bed positions (the body shifted
             along z by 6.4 cm steps), one simulation each, for one batched
             job.
"""
import os
from dataclasses import dataclass, field

import numpy as np

from . import formats as F

MAT_AIR, MAT_WATER, MAT_TISSUE, MAT_BONE, MAT_LYSO = 0, 1, 2, 3, 8
RHO_AIR = 0.0012048
DEFAULT_SEED = 20261203


@dataclass
class Scene:
    directory: str
    config_path: str
    options: dict = field(default_factory=dict)
    description: str = ""


def ring_panel0(radius, ncry_y, ncry_z, crystal, gap, depth):
    """One flat panel facing the origin from -y, one module of ncry_y x ncry_z
    crystals; its local x runs along global +y (depth grows outward)."""
    pitch = crystal + gap
    mody = ncry_y * pitch - gap
    modz = ncry_z * pitch - gap
    return {
        "start": 0,
        "len": (depth, mody, modz), "MOD": (depth, mody, modz), "Ms": (0.0, gap, gap),
        "LSO": (depth, crystal, crystal), "s": (0.0, gap, gap),
        "dir": (-1.0, 1.0, 1.0), "o": (0.0, -radius, 0.0),
        "UX": (0.0, 1.0, 0.0), "UY": (1.0, 0.0, 0.0), "UZ": (0.0, 0.0, -1.0),
    }


def _base_config(d, pdim, psize, poffset):
    c = F.Config()
    c.device = 0
    c.noncol_sigma = 0.0037056
    c.pdim, c.psize, c.poffset = pdim, psize, poffset
    c.matfile = os.path.join(d, "phantom_mat.dat")
    c.denfile = os.path.join(d, "phantom_den.dat")
    c.nparticle = 0
    c.usepsf = 0
    c.sourcefile = os.path.join(d, "source.txt")
    c.ptype = 0
    c.useprange = 0
    c.tstart, c.tend = 0.0, 120.0
    c.recordsphere = (0.0, 0.0, 0.0, 5.0)
    c.eabsph = 1.0e3
    c.geofile = os.path.join(d, "ring.geo")
    c.surfaces = [[0, 0, 0, 0, 0, 0, 0, 0, 0, 1]]
    c.rdepth, c.rpolicy = 2, 1
    c.eth = 50.0e3
    c.blurpolicy, c.eref, c.rref, c.eslope, c.sblur = 1, 511.0e3, 0.12, 0.0, 0.0
    c.dlevel, c.dtype, c.dtime = 3, 0, 0.0
    c.ewin_lo, c.ewin_hi = 350.0e3, 650.0e3
    return c


def _voxel_centres(n, size, off):
    d = size / n
    return off + (np.arange(n, dtype=np.float64) + 0.5) * d


def small(directory, n_decays=1_000_000, nvox=200, seed=DEFAULT_SEED):
    os.makedirs(directory, exist_ok=True)
    c = _base_config(directory, (nvox, nvox, nvox), (1.0, 1.0, 1.0), (-0.5, -0.5, -0.5))
    x = _voxel_centres(nvox, 1.0, -0.5)
    r2 = x[None, :] ** 2 + x[:, None] ** 2          # [y][x]
    cyl = np.broadcast_to(r2 < 0.4 ** 2, (nvox, nvox, nvox))   # [z][y][x]
    mat = np.where(cyl, MAT_WATER, MAT_AIR).astype(np.int32)
    den = np.where(cyl, 1.0, RHO_AIR).astype(np.float32)
    F.write_phantom(c.matfile, c.denfile, mat, den)
    F.write_geo(c.geofile, 8, (0, 0, 1), 45.0, (MAT_LYSO, MAT_AIR), (7.1, 0.001025),
                ring_panel0(4.0, 8, 8, 0.15, 0.001, 1.0))
    # a pure annihilation-pair emitter: isotope row 3 has branching ratio 1
    F.write_sources(c.sourcefile, [1_000_000_000], [3], [2], [(0, 0, 0, 0.0, 0, 0)])
    F.write_config(os.path.join(directory, "input_PET.in"), c)
    return Scene(directory, os.path.join(directory, "input_PET.in"),
                 {"n_decays": n_decays, "seed": seed, "coinc_window_ns": 4.0},
                 "point source, %d^3 water cylinder, 8-panel ring at 4 cm" % nvox)


def positron_phantom(n):
    """128^3-style phantom of the positron workload scaled to n voxels."""
    size = 6.4
    x = _voxel_centres(n, size, -size / 2)
    X = x[None, None, :]
    Y = x[None, :, None]
    Z = x[:, None, None]
    mat = np.full((n, n, n), MAT_WATER, np.int32)
    den = np.full((n, n, n), 1.0, np.float32)
    for a in (0.0, 0.5 * np.pi, np.pi, 1.5 * np.pi):
        cx, cy = 1.5 * np.cos(a), 1.5 * np.sin(a)
        rod = np.broadcast_to((X - cx) ** 2 + (Y - cy) ** 2 < 0.3 ** 2, (n, n, n))
        mat[rod] = MAT_BONE
        den[rod] = 1.85
    lung = X ** 2 + Y ** 2 + Z ** 2 < 0.8 ** 2
    mat[lung] = MAT_TISSUE
    den[lung] = 0.3
    return mat, den


def positron(directory, n_decays=100_000_000, nvox=128, seed=DEFAULT_SEED):
    os.makedirs(directory, exist_ok=True)
    c = _base_config(directory, (nvox, nvox, nvox), (6.4, 6.4, 6.4), (-3.2, -3.2, -3.2))
    c.useprange = 1
    c.dlevel, c.dtype, c.dtime = 2, 0, 0.3
    mat, den = positron_phantom(nvox)
    F.write_phantom(c.matfile, c.denfile, mat, den)
    F.write_geo(c.geofile, 8, (0, 0, 1), 45.0, (MAT_LYSO, MAT_AIR), (7.1, 0.001025),
                ring_panel0(8.0, 8, 8, 0.298, 0.002, 2.0))
    F.write_sources(c.sourcefile, [4_000_000_000], [0], [1], [(0, 0, 0, 3.0, 6.4, 0)])
    F.write_config(os.path.join(directory, "input_PET.in"), c)
    return Scene(directory, os.path.join(directory, "input_PET.in"),
                 {"n_decays": n_decays, "seed": seed, "coinc_window_ns": 4.0},
                 "F-18 cylinder r=3 cm, %d^3 water/bone/lung, 8-panel ring at 8 cm" % nvox)


def large(directory, n_decays=1_000_000_000, dims=(256, 256, 512), seed=DEFAULT_SEED, voxel_cm=0.2):
    """Whole-body acquisition: F-18 cylinder r=10 cm, h=60 cm in a 30 x 20 cm
    elliptic water body with lungs (rho 0.3) and a spine (bone), 48-panel
    ring of 16 x 16 LYSO crystals (4 x 4 x 20 mm). voxel_cm coarsens the grid
    (the body keeps its size) for cases the oracle finishes in seconds."""
    os.makedirs(directory, exist_ok=True)
    nx, ny, nz = dims
    sx, sy, sz = voxel_cm * nx, voxel_cm * ny, voxel_cm * nz
    c = _base_config(directory, dims, (sx, sy, sz), (-sx / 2, -sy / 2, -sz / 2))
    c.useprange = 1
    c.dlevel, c.dtype, c.dtime = 2, 0, 0.3
    X = _voxel_centres(nx, sx, -sx / 2)[None, None, :]
    Y = _voxel_centres(ny, sy, -sy / 2)[None, :, None]
    Z = _voxel_centres(nz, sz, -sz / 2)[:, None, None]
    body = np.broadcast_to((X / 15.0) ** 2 + (Y / 10.0) ** 2 < 1.0, (nz, ny, nx))
    mat = np.where(body, MAT_WATER, MAT_AIR).astype(np.int32)
    den = np.where(body, 1.0, RHO_AIR).astype(np.float32)
    for cx in (-5.5, 5.5):
        lung = ((X - cx) / 3.5) ** 2 + ((Y + 0.5) / 5.0) ** 2 + (Z / 12.0) ** 2 < 1.0
        mat[lung] = MAT_TISSUE
        den[lung] = 0.3
    spine = np.broadcast_to(X ** 2 + (Y + 6.5) ** 2 < 1.5 ** 2, (nz, ny, nx))
    mat[spine] = MAT_BONE
    den[spine] = 1.85
    F.write_phantom(c.matfile, c.denfile, mat, den)
    # 48 panels of 6.4 cm: the smallest radius at which they do not overlap
    F.write_geo(c.geofile, 48, (0, 0, 1), 7.5, (MAT_LYSO, MAT_AIR), (7.1, 0.001025),
                ring_panel0(49.0, 16, 16, 0.4, 0.001, 2.0))
    F.write_sources(c.sourcefile, [4_000_000_000], [0], [1], [(0, 0, 0, 10.0, 60.0, 0)])
    F.write_config(os.path.join(directory, "input_PET.in"), c)
    return Scene(directory, os.path.join(directory, "input_PET.in"),
                 {"n_decays": n_decays, "seed": seed, "coinc_window_ns": 4.0},
                 "F-18 body phantom 256x256x512, 48-panel ring")


@dataclass
class BedPosition:
    """One bed position of the whole-body acquisition: the body and its
    source moved along z by `shift` cm through the ring (the configuration
    and phantom of `large`, offset), with its own decays and seed."""
    config_path: str
    directory: str
    source_path: str
    shift: float
    offset: tuple
    size: tuple
    dims: tuple
    options: dict


def large_beds(directory, n_beds=8, decays_per_bed=125_000_000, dims=(256, 256, 512), voxel_cm=0.2,
               seed=DEFAULT_SEED):
    """Whole-body acquisition in n_beds bed positions: the body of `large`
    (its source, a cylinder r=10 cm h=60 cm, moving with it) shifted along z
    so that consecutive positions put adjacent 6.4 cm slabs (the ring's axial
    extent) in the ring. Returns the BedPosition list; the phantom is
    written once (phantom_mat.dat / phantom_den.dat of the `large` scene)."""
    sc = large(directory, n_decays=decays_per_bed, dims=dims, seed=seed, voxel_cm=voxel_cm)
    nx, ny, nz = dims
    size = (voxel_cm * nx, voxel_cm * ny, voxel_cm * nz)
    beds = []
    for k in range(n_beds):
        shift = (k - 0.5 * (n_beds - 1)) * 6.4
        src = os.path.join(directory, "source_bed%d.txt" % k)
        F.write_sources(src, [4_000_000_000], [0], [1], [(0, 0, shift, 10.0, 60.0, 0)])
        off = (-size[0] / 2, -size[1] / 2, -size[2] / 2 + shift)
        beds.append(BedPosition(sc.config_path, directory, src, shift, off, size, dims,
                                {"n_decays": decays_per_bed, "seed": seed + 7919 * (k + 1), "sim_id": k,
                                 "coinc_window_ns": 4.0}))
    return beds


@dataclass
class BatchSim:
    """One simulation of a batch: the shared configuration plus its own
    phantom (made on demand), source file and options."""
    config_path: str
    directory: str
    nvox: int
    source_path: str
    options: dict
    phantom_seed: int

    def phantom(self):
        return batch_phantom(self.nvox, self.phantom_seed)


def batch_phantom(n, seed):
    """n^3 voxels over a 6.4 cm cube: air, a water body ellipsoid and three to
    six seeded ellipsoids of water, bone or air inside it."""
    rng = np.random.default_rng(seed)
    size = 6.4
    x = _voxel_centres(n, size, -size / 2).astype(np.float32)
    X = x[None, None, :]
    Y = x[None, :, None]
    Z = x[:, None, None]
    mat = np.full((n, n, n), MAT_AIR, np.int32)
    den = np.full((n, n, n), RHO_AIR, np.float32)
    a = rng.uniform(2.2, 3.1, 3)
    body = (X / a[0]) ** 2 + (Y / a[1]) ** 2 + (Z / a[2]) ** 2 < 1.0
    mat[body] = MAT_WATER
    den[body] = 1.0
    for _ in range(int(rng.integers(3, 7))):
        c = rng.uniform(-1.2, 1.2, 3)
        r = rng.uniform(0.2, 0.9, 3)
        e = ((X - c[0]) / r[0]) ** 2 + ((Y - c[1]) / r[1]) ** 2 + ((Z - c[2]) / r[2]) ** 2 < 1.0
        kind = int(rng.integers(0, 3))
        mat[e], den[e] = ((MAT_WATER, 1.0), (MAT_BONE, 1.85), (MAT_AIR, RHO_AIR))[kind]
    return mat, den


def batched(directory, n_sims=64, seed=DEFAULT_SEED, min_vox=64, max_vox=256, min_decays=100_000,
            max_decays=10_000_000):
    """Many uneven simulations for one batched job: phantom sizes log-uniform
    in [min_vox, max_vox]^3 over the same 6.4 cm cube, decays log-uniform in
    [min_decays, max_decays], F-18 (positron range on) from a point or a
    cylinder (r 1-3 cm) with equal odds, each with its own seed; the ring,
    digitizer and window of the positron workload. Returns the BatchSim list;
    the seeds it drew are in each entry's options."""
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(seed)
    c = _base_config(directory, (8, 8, 8), (6.4, 6.4, 6.4), (-3.2, -3.2, -3.2))
    c.useprange = 1
    c.dlevel, c.dtype, c.dtime = 2, 0, 0.3
    mat, den = batch_phantom(8, seed)
    F.write_phantom(c.matfile, c.denfile, mat, den)
    F.write_geo(c.geofile, 8, (0, 0, 1), 45.0, (MAT_LYSO, MAT_AIR), (7.1, 0.001025),
                ring_panel0(8.0, 8, 8, 0.298, 0.002, 2.0))
    F.write_sources(c.sourcefile, [4_000_000_000], [0], [1], [(0, 0, 0, 3.0, 6.4, 0)])
    cfg = os.path.join(directory, "input_PET.in")
    F.write_config(cfg, c)
    sims = []
    for i in range(n_sims):
        nvox = int(round(np.exp(rng.uniform(np.log(min_vox), np.log(max_vox)))))
        nd = int(round(np.exp(rng.uniform(np.log(min_decays), np.log(max_decays)))))
        src = os.path.join(directory, "source_%02d.txt" % i)
        if rng.uniform() < 0.5:
            F.write_sources(src, [4_000_000_000], [0], [2], [(0, 0, 0, 0.0, 0, 0)])
        else:
            F.write_sources(src, [4_000_000_000], [0], [1], [(0, 0, 0, float(rng.uniform(1.0, 3.0)), 6.4, 0)])
        sims.append(BatchSim(cfg, directory, nvox, src,
                             {"n_decays": nd, "seed": int(rng.integers(1, 2 ** 62)), "sim_id": i,
                              "coinc_window_ns": 4.0},
                             int(rng.integers(1, 2 ** 31))))
    return sims


WORKLOADS = {"small": small, "positron": positron, "large": large}
