"""Regenerate the two inverse-CDF angular surfaces of the PET table set that the
reference lists as missing blobs: data/input4gPET.cmpsf (Compton) and
data/input4gPET.rayff (Rayleigh).

What the surfaces are (read by rcmpsf/rrayff, initialize.cu:483-566, 664-748;
sampled by comsam(matid) gPET_kernals.cu:66-88 and rylsam :128-146):
  for material m, photon energy E_j = j*dE (j = 0..NE-1) and cumulative
  probability CP_i = i*dCP (i = 0..NCP-1), the surface holds cos(theta) such that
  P(cos <= value) = CP_i under the differential cross section at E_j.
  Layout on disk: per material, NCP rows of NE values ([m][icp][ie]).

Physics used (stated choices; parity against gPET's own PET surfaces is
unpinned because those files are not in the reference tree):
  Compton : Klein-Nishina x S(q) / Z shape, q = (E/mc^2) sqrt(2(1-cos))
  Rayleigh: Thomson (1+cos^2)/2 x F(q)^2, same q
  E = 0 column: Thomson (the gCTD surfaces shipped with the reference do this).
S(q), F(q) come from ctd_sf_ff.txt (extracted from the gCTD tables). PET
materials without their own S/F table use the shape of a stand-in:
TissueICRU, MuscleStriated, Brain -> TissueICRP; CorticalBone -> Water;
Pb -> LSO.  Regenerating gCTD's own shipped surfaces with this recipe
reproduces them to a mean |d cos| of 0.005 (Compton) and 0.004-0.025
(Rayleigh, water-LYSO).

usage: python data/make_surfaces.py [data_dir]
"""
import os
import sys

import numpy as np

MC2 = 510.9991e3
NCP = 301
NE = 151
EMAX = 1.0e6
STANDIN = {
    "DryAir": "DryAir", "Water": "Water", "TissueICRU": "TissueICRP",
    "CorticalBone": "Water", "MuscleStriated": "TissueICRP", "Brain": "TissueICRP",
    "PMMA": "PMMA", "LSO": "LSO", "LYSO": "LYSO", "Pb": "LSO",
}


def read_sf_ff(path):
    tabs = {}
    cur = None
    for ln in open(path):
        if ln.startswith("#"):
            continue
        if ln.startswith("material"):
            cur = ln.split()[1]
            tabs[cur] = []
        elif ln.strip():
            tabs[cur].append([float(v) for v in ln.split()])
    return {k: np.array(v) for k, v in tabs.items()}


def material_names(matter_path):
    return [ln.split(":", 1)[1].strip() for ln in open(matter_path) if ln.strip().startswith("MATERIAL:")]


def _loglog(qtab, vtab, q, low_power):
    """Log-log interpolation; below the table v ~ q^low_power, above it the
    last log-log slope is continued."""
    lq, lv = np.log(qtab), np.log(np.maximum(vtab, 1e-300))
    x = np.log(np.maximum(q, 1e-300))
    out = np.interp(x, lq, lv)
    lo = x < lq[0]
    out[lo] = lv[0] + low_power * (x[lo] - lq[0])
    hi = x > lq[-1]
    slope = (lv[-1] - lv[-2]) / (lq[-1] - lq[-2])
    out[hi] = lv[-1] + slope * (x[hi] - lq[-1])
    return np.exp(out)


def surface(tab, kind):
    """Return the [NCP][NE] surface of cos(theta) for one material."""
    w = np.linspace(0.0, 1.0, 40001)
    mu = 1.0 - 2.0 * w * w            # dense near cos = 1 (forward peak)
    dmu = 4.0 * w                     # |d mu / d w|
    cp = np.arange(NCP) / (NCP - 1.0)
    out = np.empty((NCP, NE))
    for j in range(NE):
        e = j * EMAX / (NE - 1)
        if j == 0:
            pdf = 0.5 * (1.0 + mu * mu)
        else:
            k = e / MC2
            q = k * np.sqrt(2.0 * (1.0 - mu))
            if kind == "compton":
                r = 1.0 / (1.0 + k * (1.0 - mu))
                pdf = r * r * (r + 1.0 / r - (1.0 - mu * mu)) * _loglog(tab[:, 0], tab[:, 1], q, 2.0)
            else:
                f = _loglog(tab[:, 0], tab[:, 2], q, 0.0)
                pdf = 0.5 * (1.0 + mu * mu) * f * f
        g = pdf * dmu                 # density in w; w runs from cos=1 down to cos=-1
        cdf_w = np.concatenate([[0.0], np.cumsum(0.5 * (g[1:] + g[:-1]) * np.diff(w))])
        cdf_mu = 1.0 - cdf_w / cdf_w[-1]  # P(cos <= mu(w))
        # cdf_mu decreases with w; invert on the reversed (increasing) arrays
        out[:, j] = np.interp(cp, cdf_mu[::-1], mu[::-1])
    out[0, :] = -1.0
    out[-1, :] = 1.0
    return out


def write_surface_file(path, set_name, names, tabs, kind):
    col = "sf" if kind == "compton" else "ff"
    with open(path, "w") as f:
        f.write(" This file is part of set:\n %s\n" % set_name)
        for name in names:
            tab = tabs[STANDIN[name]]
            n = len(tab)
            lq = np.log(tab[:, 0])
            f.write(" ndata, logqmin, logqmax, dlogq:\n")
            f.write("  %d  %.6e  %.6e  %.6e\n" % (n, lq[0], lq[-1], (lq[-1] - lq[0]) / (n - 1)))
            f.write("  q(m_e*c) -- logq -- %s\n" % col)
            vals = tab[:, 1] if kind == "compton" else tab[:, 2]
            for q, l, v in zip(tab[:, 0], lq, vals):
                f.write(" %.6e  %.6e  %.6e\n" % (q, l, v))
            f.write("\n nCP, CPmin, CPmax, dCP, nE, Emin, Emax, dE:\n")
            f.write("  %d %.9e %.9e %.9e %d %.9e %.9e %.9e\n"
                    % (NCP, 0.0, 1.0, 1.0 / (NCP - 1), NE, 0.0, EMAX, EMAX / (NE - 1)))
            f.write(" " + " ".join("%.9e" % (i / (NCP - 1.0)) for i in range(NCP)) + "\n")
            f.write(" " + " ".join("%.9e" % (j * EMAX / (NE - 1)) for j in range(NE)) + "\n")
            s = surface(tab, kind)
            for i in range(NCP):
                f.write(" " + " ".join("%.7e" % v for v in s[i]) + "\n")
            f.write("\n")


def main():
    ddir = sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__))
    here = os.path.dirname(os.path.abspath(__file__))
    tabs = read_sf_ff(os.path.join(here, "ctd_sf_ff.txt"))
    names = material_names(os.path.join(ddir, "input4gPET.matter"))
    for name in names:
        if name not in STANDIN:
            raise SystemExit("no S(q)/F(q) stand-in for material %s" % name)
    write_surface_file(os.path.join(ddir, "input4gPET.cmpsf"), "input4gPET", names, tabs, "compton")
    write_surface_file(os.path.join(ddir, "input4gPET.rayff"), "input4gPET", names, tabs, "rayleigh")


if __name__ == "__main__":
    main()
