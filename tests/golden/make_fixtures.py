"""Generate the golden fixtures of the test suite from the reference tree.

The reference ships no tests or golden vectors, so the pins are its own
example inputs and numbers derived from its own data files:
  reference_inputs/  the example input_PET.in, config8.geo, source.txt and
                     pointsource.txt, copied as files (they are inputs)
  kat.json           values the reference's code computes from them:
                     - input_PET.in fields as main.cu:50-182 reads them
                     - module/crystal counts of config8.geo (initialize.cu:1074-1086)
                     - mu/rho at 511 keV by linear interpolation of
                       data/input4gPET.{lamph,compt,phote,rayle} (the textures
                       of gPET_kernals.cu:45-64)
                     - mean positron kinetic energy of each isotope from its
                       fitted spectrum (sampleEkPositron, gPET_kernals.cu:420-443)

usage: python tests/golden/make_fixtures.py <reference_root>
"""
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from gpet_gb300 import formats as F  # noqa: E402


def main():
    ref = sys.argv[1]
    out = os.path.join(HERE, "reference_inputs")
    os.makedirs(out, exist_ok=True)
    for src, dst in (("input_PET.in", "input_PET.in"), ("input/config8.geo", "config8.geo"),
                     ("input/source.txt", "source.txt"), ("input/pointsource.txt", "pointsource.txt")):
        shutil.copyfile(os.path.join(ref, src), os.path.join(out, dst))
    kat = {}
    c = F.read_config(os.path.join(out, "input_PET.in"))
    kat["config"] = {k: (list(v) if isinstance(v, tuple) else v) for k, v in c.__dict__.items()}
    g = F.read_geo(os.path.join(out, "config8.geo"))
    kat["config8_counts"] = {"moduleNy": g.counts[0], "moduleN": g.counts[1],
                             "crystalNy": g.counts[2], "crystalN": g.counts[3]}
    kat["config8_panel1"] = [float(v) for v in g.panels[1]]
    data = os.path.join(ref, "data")
    eminph, emax, names = F.read_matter(os.path.join(data, "input4gPET.matter"))
    e, lam = F.read_table_1d(os.path.join(data, "input4gPET.lamph"), len(names))
    _, cmp_ = F.read_table_1d(os.path.join(data, "input4gPET.compt"), len(names))
    _, pho = F.read_table_1d(os.path.join(data, "input4gPET.phote"), len(names))
    _, ray = F.read_table_1d(os.path.join(data, "input4gPET.rayle"), len(names))
    kat["mu_rho_511keV"] = {n: {"total": float(np.interp(511e3, e, lam[m])),
                                "compton": float(np.interp(511e3, e, cmp_[m])),
                                "photo": float(np.interp(511e3, e, pho[m])),
                                "rayleigh": float(np.interp(511e3, e, ray[m]))}
                            for m, n in enumerate(names)}
    iso = F.read_isotopes(os.path.join(data, "isotopes.txt"))
    means = []
    for i in range(len(iso.halftime)):
        cf = iso.coef[i].astype(np.float64)
        E = np.linspace(0.511, cf[0], 200001)
        p = np.polyval(cf[2:], E)
        p = np.clip(p, 0, cf[1])
        means.append(float(np.trapezoid((E - 0.511) * p, E) / np.trapezoid(p, E)))
    kat["positron_mean_kinetic_MeV"] = means
    kat["event_record"] = {"size": 48, "t_offset": 24, "E_offset": 32}
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kat, f, indent=1, sort_keys=True)
    print("wrote", out, "and kat.json")


if __name__ == "__main__":
    main()
