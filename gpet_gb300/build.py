"""Build libgpet.so and the gpet CLI in-tree (gpet_gb300/_build/) with nvcc
for sm_103a. Device code is compiled with -fmad=false: the kernels use explicit
fma where they want one, so their arithmetic is reproducible on the CPU.

usage: python -m gpet_gb300.build [--verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                     "-I" + os.path.join(ROOT, "include")]
LIB_SOURCES = ["transport.cu", "digitizer.cu", "gpet_api.cu", "loaders.cpp", "digitize_static.cu", "surrogate.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr)
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_flags=()):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    objs = []
    jobs = []
    for src in LIB_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers + [__file__]):
            lang = [] if src.endswith(".cu") else ["-x", "c++"]
            jobs.append([cc] + NVCC_FLAGS + list(extra_flags) + lang + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    lib = os.path.join(OUT, "libgpet.so")
    if _stale(lib, objs):
        _run([cc] + ARCH + ["-shared", "-o", lib] + objs, verbose)
    cli_src = os.path.join(CSRC, "gpet_cli.cpp")
    cli = os.path.join(OUT, "gpet")
    if _stale(cli, [cli_src, lib]):
        _run([cc, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-x", "c++", cli_src, "-o", cli,
              "-L" + OUT, "-lgpet", "-Xlinker", "-rpath,$ORIGIN"], verbose)
    return lib


def ptxas_report():
    """Registers / spills / shared memory per kernel (-Xptxas -v)."""
    cc = nvcc()
    out = []
    for src in ("transport.cu", "digitizer.cu", "surrogate.cu"):
        r = subprocess.run([cc] + NVCC_FLAGS + ["-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", os.devnull],
                           capture_output=True, text=True)
        out.append(r.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv)
    if "--ptxas" in sys.argv:
        print(ptxas_report())
