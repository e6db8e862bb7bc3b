"""Extract the incoherent scattering functions S(q) and atomic form factors F(q)
that ship inside the gCTD table set of the reference (data/input4gCTD.cmpsf and
data/input4gCTD.rayff, 64-point tables per material, q in units of m_e*c).

The PET table set of the reference lists data/input4gPET.cmpsf and
data/input4gPET.rayff as missing blobs, so the inverse-CDF surfaces the photon
samplers need (gPET_kernals.cu:66-88 comsam(matid), :128-146 rylsam) are
regenerated by make_surfaces.py from these S(q)/F(q) tables.

Runs only where the reference tree is mounted; its output ctd_sf_ff.txt is
committed beside this script.

usage: python data/extract_ctd_sf.py <reference_root> [out]
"""
import os
import sys


def _read_blocks(path):
    """Yield (q, logq, value) rows per material, following the per-material
    block layout read by rcmpsf/rrayff (initialize.cu:496-507, 677-688)."""
    lines = open(path).read().split("\n")
    i = 0
    blocks = []
    while i < len(lines):
        if lines[i].strip().startswith("ndata"):
            nd = int(lines[i + 1].split()[0])
            rows = [tuple(float(v) for v in lines[i + 3 + k].split()) for k in range(nd)]
            blocks.append(rows)
            i += 3 + nd
        else:
            i += 1
    return blocks


def _material_names(path):
    return [ln.split(":", 1)[1].strip() for ln in open(path) if ln.strip().startswith("MATERIAL:")]


def main():
    ref = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(__file__), "ctd_sf_ff.txt")
    names = _material_names(os.path.join(ref, "data", "input4gCTD.matter"))
    sblocks = _read_blocks(os.path.join(ref, "data", "input4gCTD.cmpsf"))
    fblocks = _read_blocks(os.path.join(ref, "data", "input4gCTD.rayff"))
    assert len(names) == len(sblocks) == len(fblocks), (len(names), len(sblocks), len(fblocks))
    with open(out, "w") as f:
        f.write("# S(q) (incoherent scattering function) and F(q) (atomic form factor) per material,\n")
        f.write("# q in units of m_e*c, extracted from the gCTD tables input4gCTD.cmpsf / input4gCTD.rayff.\n")
        for name, s, ff in zip(names, sblocks, fblocks):
            assert len(s) == len(ff)
            f.write("material %s %d\n" % (name, len(s)))
            for (q, _, sv), (q2, _, fv) in zip(s, ff):
                assert abs(q - q2) <= 1e-6 * q
                f.write("%.6e %.6e %.6e\n" % (q, sv, fv))
    print("wrote", out)


if __name__ == "__main__":
    main()
