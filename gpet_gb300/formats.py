"""Readers and writers for gPET's on-disk formats (the drop-in surface).

Each reader follows the reference's own parser; the native library has its own
C++ implementation of the same parsers and the tests check that both agree.

  input_PET.in   positional text config             main.cu:50-182
  *.geo          one panel + rotation copies         detector.cu:64-285
  source.txt     natom type shape cx cy cz c1 c2 c3  initialize.cu:116-144
  isotopes.txt   T1/2 ratio Emax nmax c0..c5         initialize.cu:10-31
  *.matter       table header (Emin_ph, Emax, nmat)  initialize.cu:279-368
  *.lamph/.compt/.phote/.rayle   4096-point tables   initialize.cu:370-662
  *.cmpsf/.rayff inverse-CDF surfaces                 initialize.cu:483-566, 664-748
  mat.dat/den.dat int32 / float32 voxels, x fastest  initialize.cu:32-74
  psf.dat        float64 x,y,z,t,vx,vy,vz,E           initialize.cu:76-115
  singles.dat    Event records, 48 bytes             gPET.h:87-92, detector.cu:287-307
  HitsID.dat / Hits.dat  int32 x5 / float32 x5       gPET_kernals.cu:1062-1080
"""
import math
import os
import re
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

EVENT_DTYPE = np.dtype([
    ("parn", "<i4"), ("pann", "<i4"), ("modn", "<i4"), ("cryn", "<i4"),
    ("siten", "<i4"), ("eventid", "<i4"), ("t", "<f8"),
    ("E", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4"),
])
assert EVENT_DTYPE.itemsize == 48 and EVENT_DTYPE.fields["t"][1] == 24

PANEL_STRIDE = 32
PANEL_FIELDS = ["lenx", "leny", "lenz", "MODx", "MODy", "MODz", "Msx", "Msy", "Msz",
                "LSOx", "LSOy", "LSOz", "sx", "sy", "sz", "ox", "oy", "oz",
                "dirx", "diry", "dirz", "UXx", "UXy", "UXz", "UYx", "UYy", "UYz",
                "UZx", "UZy", "UZz", "panel"]


class _Lines:
    """Header-line / value-token reader mirroring the fgets+fscanf pairs."""

    def __init__(self, text):
        self.lines = text.split("\n")
        self.i = 0

    def header(self):
        self.i += 1

    def values(self, n):
        out = []
        while len(out) < n:
            if self.i >= len(self.lines):
                raise ValueError("unexpected end of file")
            out.extend(self.lines[self.i].split())
            self.i += 1
        if len(out) != n:
            raise ValueError("expected %d values, got %r" % (n, out))
        return out


@dataclass
class Config:
    device: int = 0
    noncol_sigma: float = 0.0
    pdim: tuple = (0, 0, 0)
    poffset: tuple = (0.0, 0.0, 0.0)
    psize: tuple = (0.0, 0.0, 0.0)
    matfile: str = ""
    denfile: str = ""
    nparticle: int = 0
    usepsf: int = 0
    sourcefile: str = ""
    ptype: int = 0
    useprange: int = 0
    tstart: float = 0.0
    tend: float = 1.0
    recordsphere: tuple = (0.0, 0.0, 0.0, 0.0)
    eabsph: float = 0.0
    geofile: str = ""
    surfaces: List[List[float]] = field(default_factory=list)
    rdepth: int = 2
    rpolicy: int = 1
    eth: float = 0.0
    blurpolicy: int = 1
    eref: float = 0.0
    rref: float = 0.0
    eslope: float = 0.0
    sblur: float = 0.0
    dlevel: int = 3
    dtype: int = 0
    dtime: float = 0.0
    ewin_lo: float = 0.0
    ewin_hi: float = 0.0


def f32(v):
    return float(np.float32(v))


def read_config(path):
    """input_PET.in, main.cu:50-182 (positional; header line then values)."""
    r = _Lines(open(path).read())
    c = Config()
    r.header(); c.device = int(r.values(1)[0])
    r.header(); c.noncol_sigma = f32(r.values(1)[0])
    r.header(); c.pdim = tuple(int(v) for v in r.values(3))
    r.header(); c.poffset = tuple(f32(v) for v in r.values(3))
    r.header(); c.psize = tuple(f32(v) for v in r.values(3))
    r.header(); c.matfile = r.values(1)[0]
    r.header(); c.denfile = r.values(1)[0]
    r.header(); c.nparticle = int(r.values(1)[0])
    r.header(); c.usepsf = int(r.values(1)[0])
    r.header(); c.sourcefile = r.values(1)[0]
    r.header(); c.ptype = int(r.values(1)[0])
    r.header(); c.useprange = int(r.values(1)[0])
    r.header(); c.tstart, c.tend = (f32(v) for v in r.values(2))
    r.header(); c.recordsphere = tuple(f32(v) for v in r.values(4))
    r.header(); c.eabsph = f32(r.values(1)[0])
    r.header(); c.geofile = r.values(1)[0]
    r.header()
    ns = int(r.values(1)[0])
    c.surfaces = [[f32(v) for v in r.values(10)] for _ in range(ns)]
    r.header(); c.rdepth, c.rpolicy = (int(v) for v in r.values(2))
    r.header(); c.eth = f32(r.values(1)[0])
    r.header()
    v = r.values(5)
    c.blurpolicy, c.eref, c.rref, c.eslope, c.sblur = int(v[0]), f32(v[1]), f32(v[2]), f32(v[3]), f32(v[4])
    r.header()
    v = r.values(3)
    c.dlevel, c.dtype, c.dtime = int(v[0]), int(v[1]), f32(v[2])
    r.header(); c.ewin_lo, c.ewin_hi = (f32(v) for v in r.values(2))
    return c


def write_config(path, c: Config):
    def fl(x):
        return repr(float(x))
    lines = [
        "device number:", str(c.device),
        "noncolinear angle (sigma of Gaussian in rad):", fl(c.noncol_sigma),
        "phantom dimension", " ".join(str(int(v)) for v in c.pdim),
        "phantom offset in global coordinate (in cm):", " ".join(fl(v) for v in c.poffset),
        "phantom size (in cm):", " ".join(fl(v) for v in c.psize),
        "phantom material data file:", c.matfile,
        "phantom density data file:", c.denfile,
        "simulation history:", str(c.nparticle),
        "use phase space file as source (0 for no, 1 for yes):", str(c.usepsf),
        "source file:", c.sourcefile,
        "particle type of phase-space file for source (0 for positron, 1 for photon):", str(c.ptype),
        "positron range consideration (0 for no, 1 for yes):", str(c.useprange),
        "start time, end time for the radioactive decay process (in seconds):", "%s %s" % (fl(c.tstart), fl(c.tend)),
        "center (x, y, z) and radius for the photon-PSF-recording spherical surface in the global coordinate (in cm):",
        " ".join(fl(v) for v in c.recordsphere),
        "photon absorption energy (in eV):", fl(c.eabsph),
        "detector geometry file:", c.geofile,
        "total number of quadratic surfaces and the TEN parameters (x2 y2 z2 xy xz yz x y z constant) to define "
        "each quadratic surface in the local coordinate (in cm):",
        str(len(c.surfaces)),
    ]
    for s in c.surfaces:
        lines.append(" ".join(fl(v) for v in s))
    lines += [
        "readout depth (1 to 3), policy (1 and 2):", "%d %d" % (c.rdepth, c.rpolicy),
        "thresholder energy before deadtime (in eV):", fl(c.eth),
        "policy, reference energy (in eV), reference resolution (in eV) and slope for energy blurring, and "
        "resolution for space blurring (in cm):",
        "%d %s %s %s %s" % (c.blurpolicy, fl(c.eref), fl(c.rref), fl(c.eslope), fl(c.sblur)),
        "deadtime level (1 to 3), deadtime policy (0 for paralyzable, 1 for nonparalyzable), and deadtime "
        "duration (in micro-second):",
        "%d %d %s" % (c.dlevel, c.dtype, fl(c.dtime)),
        "thresholder and upholder for energy window (in eV):", "%s %s" % (fl(c.ewin_lo), fl(c.ewin_hi)),
    ]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


@dataclass
class Geometry:
    npanels: int
    axis: tuple
    angle_deg: float
    det_mat: tuple
    det_den: tuple
    panels: np.ndarray            # [npanels][PANEL_STRIDE] float32

    @property
    def counts(self):
        return panel_counts(self.panels[0])


def panel_counts(p):
    """moduleNy, moduleN, crystalNy, crystalN as iniPanel computes them
    (initialize.cu:1074-1086), in float arithmetic."""
    p = np.asarray(p, np.float32)
    ly, lz = p[1], p[2]
    my_, mz_ = p[4], p[5]
    msy, msz = p[7], p[8]
    cy, cz = p[10], p[11]
    sy, sz = p[13], p[14]
    mny = int(np.floor(np.float32(ly / np.float32(my_ + msy)))) + 1
    cny = int(np.floor(np.float32(my_ / np.float32(cy + sy)))) + 1
    mn = mny * (int(np.floor(np.float32(lz / np.float32(mz_ + msz)))) + 1)
    cn = cny * (int(np.floor(np.float32(mz_ / np.float32(cz + sz)))) + 1)
    return mny, mn, cny, cn


def read_geo(path):
    """read_file_ro, detector.cu:64-285: one panel given, N-1 copies rotated
    about an axis by i*angle with Rodrigues' formula (float arithmetic)."""
    r = _Lines(open(path).read())
    r.header(); n = int(r.values(1)[0])
    r.header(); axis = tuple(f32(v) for v in r.values(3))
    r.header(); ang = f32(r.values(1)[0])
    r.header()
    # (material, density) pairs up to the separator: the reference's two,
    # more for crystal regions marked by the quadratic surfaces
    v = []
    while r.i < len(r.lines):
        t = r.lines[r.i].split()
        if not t:
            r.i += 1
            continue
        try:
            float(t[0])
        except ValueError:
            break
        v += t
        r.i += 1
    if len(v) < 4 or len(v) % 2 or len(v) // 2 > 8:
        raise ValueError("%s: 2 to 8 (material, density) pairs expected" % path)
    det_mat = tuple(int(v[2 * k]) for k in range(len(v) // 2))
    det_den = tuple(f32(v[2 * k + 1]) for k in range(len(v) // 2))
    r.header()                      # separator line
    r.header(); pane = int(r.values(1)[0])
    vals = {}
    for key in ("len", "MOD", "Ms", "LSO", "s", "dir", "o", "UX", "UY", "UZ"):
        r.header()
        vals[key] = [f32(x) for x in r.values(3)]
    P = np.zeros((n, PANEL_STRIDE), np.float32)
    base = np.zeros(PANEL_STRIDE, np.float32)
    base[0:3] = vals["len"]; base[3:6] = vals["MOD"]; base[6:9] = vals["Ms"]
    base[9:12] = vals["LSO"]; base[12:15] = vals["s"]; base[15:18] = vals["o"]
    base[18:21] = vals["dir"]; base[21:24] = vals["UX"]; base[24:27] = vals["UY"]; base[27:30] = vals["UZ"]
    base[30] = pane
    rot = np.array(axis, np.float32)
    for i in range(n):
        P[i] = base
        if i == 0:
            continue
        P[i, 30] = i
        a = np.float32(np.float32(np.float32(ang) * np.float32(math.pi)) / np.float32(180.0)) * np.float32(i)
        ca, sa = np.float32(np.cos(a, dtype=np.float32)), np.float32(np.sin(a, dtype=np.float32))
        for off in (15, 21, 24, 27):
            vec = base[off:off + 3].astype(np.float32)
            P[i, off + 0] = (1 - ca) * (vec[0] * rot[0]) * rot[0] + ca * vec[0] + sa * (rot[1] * vec[2] - rot[2] * vec[1])
            P[i, off + 1] = (1 - ca) * (vec[1] * rot[1]) * rot[1] + ca * vec[1] + sa * (rot[2] * vec[0] - rot[0] * vec[2])
            P[i, off + 2] = (1 - ca) * (vec[2] * rot[2]) * rot[2] + ca * vec[2] + sa * (rot[0] * vec[1] - rot[1] * vec[0])
    return Geometry(n, axis, ang, det_mat, det_den, P)


def write_geo(path, npanels, axis, angle_deg, det_mat, det_den, panel0):
    """panel0: dict with keys len, MOD, Ms, LSO, s, dir, o, UX, UY, UZ (3-vectors) and start."""
    def v3(x):
        return " ".join(repr(float(t)) for t in x)
    lines = [
        "panel repetition times", str(npanels),
        "panel rotational axis in the global coordinate", v3(axis),
        "panel rotational angle (in degree, plus: counterclockwise, minus: clockwise)", repr(float(angle_deg)),
        "material density (in the order of crystal material, air)",
    ] + ["%d %s" % (m, repr(float(d))) for m, d in zip(det_mat, det_den)] + [
        "%" * 49,
        "starting panel index", str(panel0.get("start", 0)),
        "dimension(cm)", v3(panel0["len"]),
        "module size", v3(panel0["MOD"]),
        "module space", v3(panel0["Ms"]),
        "crystal size (cm)", v3(panel0["LSO"]),
        "crystal space(cm)", v3(panel0["s"]),
        "panel expansion direction in the local coordinate (x y z)", v3(panel0["dir"]),
        "offset of the panel surface center facing the phantom (cm)", v3(panel0["o"]),
        "unit vector along the local x direction in the global coordinate", v3(panel0["UX"]),
        "unit vector along the local y direction in the global coordinate", v3(panel0["UY"]),
        "unit vector along the local z direction in the global coordinate", v3(panel0["UZ"]),
        "%" * 49,
    ]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


@dataclass
class Sources:
    natom: np.ndarray      # uint32
    type: np.ndarray       # int32
    shape: np.ndarray      # int32
    coef: np.ndarray       # [n][6] float32


def _skip_to_hash(text):
    """`infile >> n; infile.ignore(512,'#')` (initialize.cu:16-17, 123-125)."""
    s = text.lstrip()
    m = re.match(r"[+-]?\d+", s)
    if not m:
        raise ValueError("expected a count at the start of the file")
    rest = s[m.end():]
    k = rest.find("#", 0, 512)
    rest = rest[k + 1:] if k >= 0 else rest[512:]
    return int(m.group(0)), rest.split()


def read_sources(path):
    n, tok = _skip_to_hash(open(path).read())
    natom = np.zeros(n, np.uint32); typ = np.zeros(n, np.int32); shp = np.zeros(n, np.int32)
    coef = np.zeros((n, 6), np.float32)
    for i in range(n):
        natom[i] = int(tok[9 * i]); typ[i] = int(tok[9 * i + 1]); shp[i] = int(tok[9 * i + 2])
        coef[i] = [f32(t) for t in tok[9 * i + 3: 9 * i + 9]]
    return Sources(natom, typ, shp, coef)


def write_sources(path, natom, types, shapes, coefs):
    with open(path, "w") as f:
        f.write("%d\n" % len(natom))
        f.write("Natoms(equal to activity times lamda) type(from isotope file, start from 0), shape type, "
                "centerx(cm) centery(cm) centerz(cm) Threecoefftodefineshape#\n")
        for n, t, s, c in zip(natom, types, shapes, coefs):
            f.write("%d %d %d %s\n" % (n, t, s, " ".join(repr(float(v)) for v in c)))


@dataclass
class Isotopes:
    halftime: np.ndarray
    ratio: np.ndarray
    coef: np.ndarray       # [n][8]: Emax, nmax, c0..c5


def read_isotopes(path):
    n, tok = _skip_to_hash(open(path).read())
    ht = np.zeros(n, np.float32); ra = np.zeros(n, np.float32); cf = np.zeros((n, 8), np.float32)
    for i in range(n):
        ht[i] = f32(tok[10 * i]); ra[i] = f32(tok[10 * i + 1])
        cf[i] = [f32(t) for t in tok[10 * i + 2: 10 * i + 10]]
    return Isotopes(ht, ra, cf)


@dataclass
class Tables:
    names: List[str]
    eminph: float
    emax: float
    energy: np.ndarray            # [ne] float32
    lamph: np.ndarray             # [nmat][ne]
    compt: np.ndarray
    phote: np.ndarray
    rayle: np.ndarray
    cmpsf: np.ndarray             # [nmat][ncp][ne_s]
    cmpsf_dcp: float = 0.0
    cmpsf_de: float = 0.0
    rayff: Optional[np.ndarray] = None
    rayff_dcp: float = 0.0
    rayff_de: float = 0.0

    @property
    def idle(self):
        n = len(self.energy)
        return f32(np.float32(n - 1) / np.float32(self.energy[-1] - self.energy[0]))


def read_matter(path):
    """rmater, initialize.cu:279-368: [Emin_ph, Emin, Emax] and material names."""
    lines = open(path).read().split("\n")
    k = 4
    while not lines[k].split():   # fscanf skips the blank line after 4 fgets
        k += 1
    e = lines[k].split()
    names = [ln.split(":", 1)[1].strip() for ln in lines if ln.strip().startswith("MATERIAL:")]
    return f32(e[0]), f32(e[2]), names


def read_table_1d(path, nmat):
    """rlamph / rcompt / rphote / rrayle: per material 'ndata' header, count
    line, column header, then (energy, value) rows."""
    lines = open(path).read().split("\n")
    i = 0
    energies = None
    vals = []
    while len(vals) < nmat:
        while not lines[i].strip().startswith("ndata"):
            i += 1
        nd = int(lines[i + 1].split()[0])
        arr = np.array([ln.split() for ln in lines[i + 3:i + 3 + nd]], dtype=np.float32)
        energies = arr[:, 0]
        vals.append(arr[:, 1])
        i += 3 + nd
    return energies, np.stack(vals)


def read_surface(path, nmat):
    """rcmpsf / rrayff: per material a q-table (skipped) then the surface."""
    lines = open(path).read().split("\n")
    i = 0
    out = []
    dcp = de = None
    while len(out) < nmat:
        while not lines[i].strip().startswith("nCP"):
            i += 1
        h = lines[i + 1].split()
        ncp, ne = int(h[0]), int(h[4])
        dcp, de = f32(h[3]), f32(h[7])
        rows = np.array([ln.split() for ln in lines[i + 4:i + 4 + ncp]], dtype=np.float32)
        assert rows.shape == (ncp, ne), rows.shape
        out.append(rows)
        i += 4 + ncp
    return np.stack(out), dcp, de


def read_tables(data_dir, prefix="input4gPET"):
    base = os.path.join(data_dir, prefix)
    eminph, emax, names = read_matter(base + ".matter")
    nmat = len(names)
    e, lamph = read_table_1d(base + ".lamph", nmat)
    _, compt = read_table_1d(base + ".compt", nmat)
    _, phote = read_table_1d(base + ".phote", nmat)
    _, rayle = read_table_1d(base + ".rayle", nmat)
    cm, cdcp, cde = read_surface(base + ".cmpsf", nmat)
    rf, rdcp, rde = read_surface(base + ".rayff", nmat)
    return Tables(names, eminph, emax, e, lamph, compt, phote, rayle, cm, cdcp, cde, rf, rdcp, rde)


def read_phantom(matfile, denfile, dims):
    n = int(dims[0]) * int(dims[1]) * int(dims[2])
    mat = np.fromfile(matfile, dtype="<i4", count=n)
    den = np.fromfile(denfile, dtype="<f4", count=n)
    if mat.size != n or den.size != n:
        raise ValueError("phantom files hold fewer than %d voxels" % n)
    return mat, den


def write_phantom(matfile, denfile, mat, den):
    np.asarray(mat, "<i4").tofile(matfile)
    np.asarray(den, "<f4").tofile(denfile)


def read_psf(path, n=None):
    a = np.fromfile(path, dtype="<f8")
    a = a[: (a.size // 8) * 8].reshape(-1, 8)
    return a if n is None else a[:n]


def read_events(path):
    return np.fromfile(path, dtype=EVENT_DTYPE)


def read_hits(id_path, f_path):
    ids = np.fromfile(id_path, dtype="<i4").reshape(-1, 5)
    fs = np.fromfile(f_path, dtype="<f4").reshape(-1, 5)
    return ids, fs


def read_coincidences(path):
    """coincidences.dat: pairs of Event records (96 bytes per coincidence);
    coincidences_class.dat: uint8 class per pair (0 true, 1 scatter, 2 random)."""
    ev = np.fromfile(path, dtype=EVENT_DTYPE).reshape(-1, 2)
    cls_path = path.replace(".dat", "_class.dat")
    cls = np.fromfile(cls_path, dtype=np.uint8) if os.path.exists(cls_path) else None
    return ev, cls


# ---------------------------------------------------------------- phase space
PSF_STATE_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"),
                            ("E", "<f4")])


def read_phase_space(directory, stem):
    """out<stem>.dat (float3 position + float4 direction/energy per photon),
    id<stem>.dat (int32 event id) and time<stem>.dat (double, us) as written
    by gPET with OUTPUTPSF (gPET.cu:63-114); stem is "source" or "phantom"."""
    st = np.fromfile(os.path.join(directory, "out%s.dat" % stem), PSF_STATE_DTYPE)
    ids = np.fromfile(os.path.join(directory, "id%s.dat" % stem), "<i4")
    t = np.fromfile(os.path.join(directory, "time%s.dat" % stem), "<f8")
    if not (len(st) == len(ids) == len(t)):
        raise ValueError("phase-space files of %s disagree in length" % stem)
    out = np.zeros(len(st), [(n, st.dtype[n]) for n in st.dtype.names] + [("eventid", "<i4"), ("t", "<f8")])
    for n in st.dtype.names:
        out[n] = st[n]
    out["eventid"] = ids
    out["t"] = t
    return out
