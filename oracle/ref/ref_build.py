"""Build the reference's own host and kernel functions for the CPU
(TEST INFRASTRUCTURE: the library it makes is used only by the pins in
tests/ and by tests/golden/make_ref_vectors.py).

Recipe: the named functions are cut, as they are, out of the reference's
source files (gPET_kernals.cu, initialize.cu, detector.cu; the types of
gPET.h) into oracle/_ref/gen/ref_sources.cpp, and compiled with g++ behind
oracle/ref/ref_prelude.h (CPU stand-ins for the CUDA runtime, textures and
curand) together with oracle/ref/ref_harness.cpp into
oracle/_ref/libgpet_ref.so. Everything it writes goes to oracle/_ref/, which
is not part of the repository. Two mechanical edits are made to the cut
text, both in photonde (gPET_kernals.cu:839-1233):
  - `extern __shared__ float s[];` becomes a pointer to a host buffer
    (dynamic shared memory has no host counterpart);
  - `Event events[4];` becomes `Event events[64];`: the reference's adder
    (:737-755) appends without a bound check, which on the host would write
    past the array for a photon that deposits in more than four crystals.

The reference must be present (at REF_DIR or the path given); the build is
skipped otherwise: the pins then run on the committed golden vectors only.

  python oracle/ref/ref_build.py [REF_DIR]
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libgpet_ref.so")
REF_DIR = "/root/reference"

# (file, function name, how many definitions of that name in file order)
FUNCTIONS = [
    ("gPET_kernals.cu", "getAbsVox", 1), ("gPET_kernals.cu", "lamwck", 1), ("gPET_kernals.cu", "lamwckde", 1),
    ("gPET_kernals.cu", "itphip_G", 1), ("gPET_kernals.cu", "irylip", 1), ("gPET_kernals.cu", "icptip", 1),
    ("gPET_kernals.cu", "comsam", 2), ("gPET_kernals.cu", "rylsam", 1), ("gPET_kernals.cu", "getDistance", 1),
    ("gPET_kernals.cu", "rotate", 1), ("gPET_kernals.cu", "photon", 1), ("gPET_kernals.cu", "setPositronRange", 1),
    ("gPET_kernals.cu", "sampleEkPositron", 1), ("gPET_kernals.cu", "getPositionFromShape", 1),
    ("gPET_kernals.cu", "setPositionForPhoton", 1), ("gPET_kernals.cu", "adder", 1),
    ("gPET_kernals.cu", "readout", 1), ("gPET_kernals.cu", "blur", 1), ("gPET_kernals.cu", "crystalSearch", 1),
    ("gPET_kernals.cu", "photonde", 1),
    ("initialize.cu", "spline", 1), ("initialize.cu", "rmater", 1), ("initialize.cu", "rlamph", 1),
    ("initialize.cu", "rcompt", 1), ("initialize.cu", "rcmpsf", 1), ("initialize.cu", "rphote", 1),
    ("initialize.cu", "rrayle", 1), ("initialize.cu", "rrayff", 1), ("initialize.cu", "itphip", 1),
    ("initialize.cu", "iniwck", 2), ("initialize.cu", "initPhantom", 1), ("initialize.cu", "iniPanel", 1),
    ("detector.cu", "InitializeObject", 1), ("detector.cu", "read_file_ro", 1),
]
EDITS = [
    ("extern __shared__ float s[];", "float* s = ref_dyn_smem;"),
    ("Event events[4];", "Event events[64];"),
]


def _code_mask(text):
    """Per character: True where it is code (not a comment or a literal)."""
    mask = [True] * len(text)
    i, n = 0, len(text)
    while i < n:
        c = text[i]
        if text.startswith("//", i):
            j = text.find("\n", i)
            j = n if j < 0 else j
            for k in range(i, j):
                mask[k] = False
            i = j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            for k in range(i, j):
                mask[k] = False
            i = j
        elif c in "\"'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            for k in range(i, min(j + 1, n)):
                mask[k] = False
            i = j + 1
        else:
            i += 1
    return mask


def _definitions(text, name):
    """(start, signature end, body end) of every definition of `name`."""
    mask = _code_mask(text)
    out = []
    for m in re.finditer(r"(?m)^[A-Za-z_][^\n;{}()]*\b%s\s*\(" % re.escape(name), text):
        if not mask[m.start()]:
            continue
        # the parameter list
        depth, i = 0, m.end() - 1
        while True:
            if mask[i]:
                depth += text[i] == "("
                depth -= text[i] == ")"
            i += 1
            if depth == 0:
                break
        sig_end = i
        # a definition: the next code character that is not space is '{'
        # (comments may come between)
        j = i
        while j < len(text) and (not mask[j] or text[j].isspace()):
            j += 1
        if j >= len(text) or text[j] != "{":
            continue
        depth = 0
        while True:
            if mask[j]:
                depth += text[j] == "{"
                depth -= text[j] == "}"
            j += 1
            if depth == 0:
                break
        out.append((m.start(), sig_end, j))
    return out


def _types(ref_dir):
    """The types and the inline helper of gPET.h (its CUDA includes left out)."""
    text = open(os.path.join(ref_dir, "gPET.h")).read()
    a = text.index("#define FILEEXIST")
    b = text.index("/***************************************************\nthe following are declaration")
    types = text[a:b]
    (s, _, e), = _definitions(text, "ind2To1")
    return types + "\n" + text[s:e] + "\n"


def generate(ref_dir=REF_DIR):
    os.makedirs(os.path.join(OUT, "gen"), exist_ok=True)
    protos, bodies = [], []
    cache = {}
    for fname, name, count in FUNCTIONS:
        if fname not in cache:
            cache[fname] = open(os.path.join(ref_dir, fname)).read()
        text = cache[fname]
        defs = _definitions(text, name)
        if len(defs) != count:
            raise RuntimeError("%s: %d definitions of %s, expected %d" % (fname, len(defs), name, count))
        for s, sig_end, e in defs:
            line = text.count("\n", 0, s) + 1
            protos.append(text[s:sig_end].strip() + ";")
            body = text[s:e]
            for old, new in EDITS:
                body = body.replace(old, new)
            bodies.append("// %s:%d\n%s\n" % (fname, line, body))
    src = ["// generated by oracle/ref/ref_build.py from the reference's source files; not part of the repository",
           _types(ref_dir), "\n".join(protos), ""] + bodies
    path = os.path.join(OUT, "gen", "ref_sources.cpp")
    with open(path, "w") as f:
        f.write("\n".join(src))
    return path


def build(ref_dir=REF_DIR, quiet=True):
    """Generate and compile oracle/_ref/libgpet_ref.so; returns its path, or
    None when the reference is not present."""
    if not os.path.exists(os.path.join(ref_dir, "gPET_kernals.cu")):
        return None
    generate(ref_dir)
    cmd = ["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-I", HERE, "-I", os.path.join(OUT, "gen"), "-I", ref_dir,
           "-I", os.path.join(ROOT, "gpet_gb300", "csrc"),
           os.path.join(HERE, "ref_harness.cpp"), "-o", LIB, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference CPU build failed:\n" + r.stdout + r.stderr)
    if not quiet:
        print(LIB)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else REF_DIR, quiet=False))
