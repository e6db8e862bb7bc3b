"""Benchmark: detected coincidences/s of the plain Monte Carlo on one GB300.

Workload (one step = one full acquisition, simulated and digitized):
  F-18 uniform in a 3 cm-radius cylinder (positron range on), 128^3 voxels of
  0.5 mm (water, four bone rods, lung sphere), 1e8 decays in [0, 120] s,
  8-panel LYSO ring at 8 cm (8x8 crystals of 3x3x20 mm), energy blur 12%,
  paralyzable dead time 300 ns per block, window 350-650 keV, coincidence
  window 4 ns. Seeded synthetic inputs written in gPET's own file formats.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). `value` = coincidences / device time with the
scene resident on the GPU (CUDA events on the library's stream); `e2e` = the
same metric through the C ABI with host buffers (phantom upload, run, singles
and coincidence copy-out, the copy-out of one step overlapping the next step)
timed on the host clock. `surrogate_batched` = the
metric's second form: 64 uneven simulations batched in one job with the
learned detector response (committed model), against the plain form (each
simulation its own plain Monte Carlo run) and plain batched, with the
chi-square of the singles spectrum and crystal map. The reference arm
(--impl reference) times the CPU oracle, the restatement of the reference's
algorithm, on all host cores (the reference's own GPU build does not compile
with CUDA 13).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "detected coincidences/s on 1 GB300 (plain MC)"
SUB_DECAYS = 1 << 20      # decays per k_source/k_phantom launch (library default)
UNIT = "coincidences/s"
WORKLOAD = ("positron: F-18 cylinder r=3 cm (positron range on), 128^3 x 0.5 mm water/bone/lung phantom, "
            "1e8 decays per step, 8-panel LYSO ring at 8 cm (8x8 crystals 3x3x20 mm), blur 12%, "
            "paralyzable dead time 0.3 us per block, window 350-650 keV, coincidence window 4 ns")

# Algorithmic bytes of the phantom-transport kernel (the dominant one), from
# the byte model of the gPET path: per photon 88 B of phantom state read and
# written, 5 B per Woodcock step for the voxel it lands in (u8 material + f32
# density), 44 B per photon handed to the detector queue.
def algorithmic_bytes_phantom(n_photons, ph_steps, entered):
    return 88 * n_photons + 5 * ph_steps + 44 * entered


# DRAM bytes per photon slot of k_phantom measured by ncu (dram__bytes_read.sum
# + dram__bytes_write.sum of one launch of 4,194,304 decays of this workload,
# 8,388,608 photon slots: 311.1 MB + 36.1 MB; profiles/k_phantom_positron_4M.md)
MEASURED_DRAM_BYTES_PER_PHOTON = (311.065088e6 + 36.134656e6) / 8388608


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def combine_ranks(ms, coincidences, dist=None, device="cpu"):
    """Whole-job numbers over ranks: the slowest rank's device time and the
    sum of all ranks' coincidences (each rank simulates its own acquisition
    with its own Philox key; there is no data exchange)."""
    if dist is None:
        return float(ms), float(coincidences)
    import torch
    mx = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    sm = torch.tensor([float(coincidences)], dtype=torch.float64, device=device)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx.item()), float(sm.item())


def make_scene(directory, n_decays, workload="positron"):
    from gpet_gb300 import scenes
    if workload == "large":
        return scenes.large(directory, n_decays=n_decays)
    return scenes.positron(directory, n_decays=n_decays)


def cpu_baseline(scene, seconds, threads=0, max_decays=200_000_000, with_hists=False):
    """The oracle (FP64, OpenMP over decays) on a bounded sample of the workload
    (with_hists: also its singles histograms and counts, for the parity check)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bridge
    bridge.build()
    o = bridge.OracleScene(scene.config_path, scene.options, os.path.join(ROOT, "data"), base_dir=scene.directory)
    if with_hists:
        o.s.seed = 4242   # a key no GPU step of the bench uses: independent samples
    n0 = min(200_000, o.n_decays)
    t0 = time.perf_counter()
    o.run(0, n0, precision="fp64", threads=threads)
    rate = n0 / max(time.perf_counter() - t0, 1e-6)
    n = int(min(max(n0, rate * seconds), max_decays, o.n_decays))
    t0 = time.perf_counter()
    r = o.run(0, n, precision="fp64", threads=threads)
    dt = time.perf_counter() - t0
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    out = {"value": r["n_coinc"] / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "%d of the %d decays (oracle FP64, %d threads, %.1f s)" % (n, o.n_decays, cores, dt),
           "decays_per_s": n / dt, "coincidences": r["n_coinc"]}
    if with_hists:
        out["_parity"] = (_singles_hists(r["singles"]),
                          {"n_decays": n, "n_singles": r["n_singles"], "n_coinc": r["n_coinc"],
                           "n_true": r["n_true"], "n_scatter": r["n_scatter"], "n_random": r["n_random"]},
                          int(o.s.seed))
    return out


def _singles_hists(ev):
    """Singles energy spectrum (60 bins over the 350-650 keV window) and
    singles per crystal (pooled over panels and modules)."""
    import numpy as np
    he = np.histogram(ev["E"], bins=60, range=(3.5e5, 6.5e5))[0]
    hc = np.bincount(ev["cryn"], minlength=64) if len(ev) else np.zeros(64, np.int64)
    return he, hc


def _parity_vs_oracle(gpu_hist, gpu_counts, gpu_seed, oracle_part):
    """Plain Monte Carlo on the GPU against the FP64 oracle on the same
    workload with independent seeds: two-sample chi-square of the singles
    spectrum and crystal map, and per-decay rates with the difference in
    standard deviations of the two Poisson counts."""
    import numpy as np
    (oe, oc), ocounts, oseed = oracle_part
    ge, gc = gpu_hist
    nc = max(len(gc), len(oc))
    gc = np.pad(gc, (0, nc - len(gc)))
    oc = np.pad(oc, (0, nc - len(oc)))
    rates = {}
    for k in ("n_singles", "n_coinc", "n_true", "n_scatter", "n_random"):
        a, na = float(gpu_counts[k]), float(gpu_counts["n_decays"])
        b, nb = float(ocounts[k]), float(ocounts["n_decays"])
        ra, rb = a / na, b / nb
        sd = np.sqrt(a / na ** 2 + b / nb ** 2)
        rates[k[2:]] = {"gpu_per_decay": ra, "oracle_per_decay": rb, "sigma": (ra - rb) / sd if sd > 0 else 0.0}
    return {"gpu": {"seed": gpu_seed, "decays": int(gpu_counts["n_decays"])},
            "oracle": {"seed": oseed, "decays": int(ocounts["n_decays"]), "precision": "fp64"},
            "singles_energy_350_650keV": _chi2(ge, oe), "singles_per_crystal": _chi2(gc, oc), "rates": rates}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), or None."""
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as d:
        sc = make_scene(d, args.decays, args.workload)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import bridge
        bridge.build()
        o = bridge.OracleScene(sc.config_path, sc.options, os.path.join(ROOT, "data"), base_dir=d)
        n0 = min(200_000, o.n_decays)
        t0 = time.perf_counter()
        o.run(0, n0, precision="fp64")
        rate = n0 / max(time.perf_counter() - t0, 1e-6)
        # each timed step is the whole acquisition unless a bounded sample is asked for
        n = o.n_decays if args.ref_step_seconds <= 0 else int(min(o.n_decays, max(n0, rate * args.ref_step_seconds)))
        for w in range(args.warmup):
            o.run(0, min(n, n0), precision="fp64")
        tot_c, tot_t, tot_d = 0, 0.0, 0
        for k in range(args.steps):
            b = (k * n) % max(1, o.n_decays - n + 1)
            o.s.seed = 20261203 + k      # the seeds of the GPU arm's timed steps
            t0 = time.perf_counter()
            r = o.run(b, b + n, precision="fp64")
            tot_t += time.perf_counter() - t0
            tot_c += r["n_coinc"]
            tot_d += n
        value = tot_c / tot_t
        cores = os.cpu_count() or 1
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": WORKLOAD, "decays_per_step": n, "sample_of": o.n_decays},
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": "%d decays per step of the %d-decay workload, oracle FP64, %d threads"
                                           % (n, o.n_decays, cores)},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "decays_per_s": tot_d / tot_t}
        print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if not args.gloo else "gloo")
    import torch
    from gpet_gb300 import api, formats as F
    torch.cuda.set_device(local)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda:%d" % local)   # 512 MB > L2

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    with tempfile.TemporaryDirectory() as d:
        sc = make_scene(d, args.decays, args.workload)
        data = os.path.join(ROOT, "data")
        t_setup = time.perf_counter()
        ctx = api.Context(local)
        opts = dict(sc.options, data_dir=data, base_dir=d, sim_id=rank)
        opts.update(args.set)
        ctx.set_options(opts)
        ctx.load_config(sc.config_path)
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t_setup
        tuning = ctx.autotune(args.tune_decays) if args.autotune else None
        # decays per k_source / k_phantom launch of this run
        sub_decays = int(tuning["sub_decays"]) if tuning else int(args.set.get("sub_decays", SUB_DECAYS))
        for w in range(args.warmup):
            flush.zero_()
            ctx.set_option("seed", 1000 + w)
            ctx.run()
        sampler = ClockSampler(local)
        barrier()
        sampler.start()
        t_wall0 = time.perf_counter()
        tot = {"coinc": 0, "ms": 0.0, "ms_sp": 0.0, "ms_src": 0.0, "ms_ph": 0.0, "ms_det": 0.0, "ms_dig": 0.0, "launches": 0, "ph_steps": 0,
               "entered": 0, "decays": 0, "singles": 0, "true": 0, "scatter": 0, "random": 0, "chunks": 0,
               "pairs": 0}
        t_flush, t_run = 0.0, 0.0
        for k in range(args.steps):
            t0 = time.perf_counter()
            flush.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            ctx.set_option("seed", 20261203 + k)
            st = ctx.run()
            t_run += time.perf_counter() - t1
            t_flush += t1 - t0
            tot["coinc"] += st["n_coinc"]; tot["ms"] += st["ms_total"]; tot["ms_sp"] += st["ms_source_phantom"]
            tot["ms_src"] += st["ms_source"]; tot["ms_ph"] += st["ms_phantom"]
            tot["ms_det"] += st["ms_detector"]; tot["ms_dig"] += st["ms_digitizer"]
            tot["launches"] += st["kernel_launches"]; tot["ph_steps"] += st["phantom_steps"]
            tot["entered"] += st["n_entered"]; tot["decays"] += st["n_decays"]; tot["singles"] += st["n_singles"]
            tot["true"] += st["n_true"]; tot["scatter"] += st["n_scatter"]; tot["random"] += st["n_random"]
            tot["chunks"] += -(-st["n_decays"] // sub_decays)
            tot["pairs"] += st["n_pairs"]
        barrier()
        wall = time.perf_counter() - t_wall0
        clocks = sampler.stop()
        # the last timed acquisition's singles, for the parity check against
        # the oracle's own acquisition (independent seeds) below
        last_seed = 20261203 + args.steps - 1
        last_hist, last_counts = None, None
        if world == 1 and not args.no_cpu_baseline:
            last_ev, _ = ctx.singles()
            last_hist = _singles_hists(last_ev)
            last_counts = {k: st[k] for k in ("n_decays", "n_singles", "n_coinc", "n_true", "n_scatter", "n_random")}
        ms_max, coinc_all = combine_ranks(tot["ms"], tot["coinc"], dist,
                                          "cpu" if args.gloo else "cuda:%d" % local)
        value = coinc_all / (ms_max * 1e-3)
        # e2e through the C ABI with host buffers: the phantom goes up from
        # pinned host memory, singles and coincidences come back into pinned
        # host memory, every step
        cfg = F.read_config(sc.config_path)
        mat0, den0 = F.read_phantom(os.path.join(d, "phantom_mat.dat"), os.path.join(d, "phantom_den.dat"),
                                    tuple(cfg.pdim))

        def pinned(shape, dtype):
            nb = int(np.prod(shape)) * np.dtype(dtype).itemsize
            return torch.empty(nb, dtype=torch.uint8, pin_memory=True).numpy().view(dtype).reshape(shape)

        mat = pinned(mat0.shape, np.int32)
        den = pinned(den0.shape, np.float32)
        mat[...] = mat0
        den[...] = den0
        cap_s = int(2 * tot["singles"] / max(1, args.steps)) + 1024
        cap_c = int(2 * tot["coinc"] / max(1, args.steps)) + 1024
        # two sets of host buffers: a step's records are copied (on the
        # library's copy stream) while the next step's phantom upload and run
        # proceed, and read on the host once the next run has returned
        outs = [((pinned((cap_s,), F.EVENT_DTYPE), pinned((cap_s,), np.uint8)),
                 (pinned((cap_c, 2), np.int64), pinned((cap_c,), np.uint8))) for _ in range(2)]
        e2e_steps = max(2, args.steps // 2) if args.e2e_steps < 0 else args.e2e_steps

        def host_read(singles, pairs):
            # the step's result read on the host: time order of its first and
            # last single, its last pair's indices within the singles
            ok = len(singles) == 0 or singles["t"][-1] >= singles["t"][0]
            return ok and (len(pairs) == 0 or int(pairs[-1].max()) < len(singles))

        # one untimed step first: the library's staging buffers and copy
        # stream are set up there, as in a stream of acquisitions
        if e2e_steps > 0:
            ctx.set_option("seed", 776)
            ctx.set_phantom(mat, den, cfg.pdim, cfg.poffset, cfg.psize)
            ctx.run()
            ctx.singles_async(outs[1][0])
            ctx.coincidences_async(outs[1][1])
            ctx.wait_copies()
        barrier()
        t0 = time.perf_counter()
        e_coinc, h2d, d2h, e_ok, pend = 0, 0, 0, True, None
        e_host = {"set_phantom": 0.0, "gpet_run": 0.0, "wait_and_read": 0.0, "singles_async": 0.0,
                  "coincidences_async": 0.0}
        for k in range(e2e_steps):
            ta = time.perf_counter()
            ctx.set_option("seed", 777 + k)
            ctx.set_phantom(mat, den, cfg.pdim, cfg.poffset, cfg.psize)
            tb = time.perf_counter()
            st = ctx.run()
            tc = time.perf_counter()
            ctx.wait_copies()
            if pend is not None:
                e_ok = e_ok and host_read(*pend)
            td = time.perf_counter()
            singles, scat = ctx.singles_async(outs[k % 2][0])
            te = time.perf_counter()
            pairs, cls = ctx.coincidences_async(outs[k % 2][1])
            tf = time.perf_counter()
            for key, dt in zip(e_host, (tb - ta, tc - tb, td - tc, te - td, tf - te)):
                e_host[key] += dt
            pend = (singles, pairs)
            e_coinc += len(pairs)
            h2d += mat.nbytes + den.nbytes
            d2h += singles.nbytes + scat.nbytes + pairs.nbytes + cls.nbytes
        ctx.wait_copies()
        e_ok = e_ok and (pend is None or host_read(*pend))
        barrier()
        e_wall = time.perf_counter() - t0
        if not e_ok:
            raise RuntimeError("end-to-end results read back inconsistent")
        ctx.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = _peaks()
    n_launch = max(1, tot["chunks"])
    photons = 2 * tot["pairs"]
    bytes_ph = algorithmic_bytes_phantom(photons, tot["ph_steps"], tot["entered"])
    dur_ph = tot["ms_ph"] * 1e-3 / n_launch
    achieved = (bytes_ph / n_launch) / dur_ph / 1e9
    # the ncu capture is of the positron workload's k_phantom
    traffic = MEASURED_DRAM_BYTES_PER_PHOTON * photons / n_launch if args.workload == "positron" else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded, written in gPET input formats)",
        "config": {"workload": WORKLOAD if args.workload == "positron" else LARGE_WORKLOAD,
                   "decays_per_step": args.decays, "l2": "flushed between steps (512 MB write)",
                   "per_rank": "independent acquisitions (disjoint Philox keys)"},
        "gpu_launches": tot["launches"],
        "breakdown_ms_per_step": {"source": tot["ms_src"] / args.steps, "phantom": tot["ms_ph"] / args.steps,
                                  "detector": tot["ms_det"] / args.steps,
                                  "digitizer_and_coincidences": tot["ms_dig"] / args.steps},
        "counts_per_step": {"decays": tot["decays"] / args.steps, "singles": tot["singles"] / args.steps,
                            "coincidences": tot["coinc"] / args.steps, "true": tot["true"] / args.steps,
                            "scatter": tot["scatter"] / args.steps, "random": tot["random"] / args.steps},
        "decays_per_s": tot["decays"] * world / (ms_max * 1e-3),
        "roofline": {"kernel": "k_phantom", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes_per_launch": bytes_ph / n_launch, "launch_ms": dur_ph * 1e3,
                     "launches": n_launch,
                     "note": "issue/latency-bound (RNG, transcendental math, dependent L2 gathers); "
                             "HBM per the path's byte model"},
        "e2e": {"value": e_coinc / e_wall, "unit": UNIT, "h2d_bytes_per_step": h2d // e2e_steps,
                "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps,
                "host_ms_per_step": {k: 1e3 * v / e2e_steps for k, v in e_host.items()},
                "copies": "each step's singles and coincidences are gathered on the device and copied into "
                          "pinned host memory on the library's copy stream while the next step's phantom "
                          "upload and run proceed (gpet_get_*_async); the timed region ends after the last "
                          "step's copies have landed"} if e2e_steps > 0 else None,
        "clocks": clocks,
        "wall_s_timed_region": wall,
        # host clock per step: the L2 flush (512 MB write + sync) and gpet_run
        # (device time plus the host's per-chunk count reads and launches)
        "wall_ms_per_step": {"l2_flush": 1e3 * t_flush / args.steps, "gpet_run": 1e3 * t_run / args.steps},
        "launch_shape": tuning if tuning else "library defaults",
        "setup_s": setup_s,
    }
    if world == 1 and args.surrogate_steps > 0 and args.workload == "positron":
        line["surrogate_batched"] = measure_surrogate_batched(args.surrogate_steps, 2)
    if world == 1 and not args.no_cpu_baseline:
        with tempfile.TemporaryDirectory() as d2:
            sc2 = make_scene(d2, args.decays, args.workload)
            line["cpu_baseline"] = cpu_baseline(sc2, args.cpu_seconds, with_hists=True)
            line["cpu_baseline"]["cpu_model"] = cpu_model()
            line["parity_vs_oracle"] = _parity_vs_oracle(last_hist, last_counts, last_seed,
                                                         line["cpu_baseline"].pop("_parity"))
            one = cpu_baseline(sc2, args.cpu_seconds / 4, threads=1)
            line["cpu_baseline_1core"] = {k: one[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


LARGE_WORKLOAD = ("large: F-18 cylinder r=10 cm h=60 cm (positron range on) in a 256x256x512 x 2 mm body phantom "
                  "(30x20 cm water ellipse, lungs rho 0.3, bone spine), 1e9 decays per step, 48-panel LYSO ring "
                  "at 49 cm (16x16 crystals 4x4x20 mm), blur 12%, paralyzable dead time 0.3 us per block, "
                  "window 350-650 keV, coincidence window 4 ns")

BATCH_WORKLOAD = ("batched64: 64 simulations of uneven size in one job - phantoms 64^3-256^3 voxels (log-uniform) "
                  "over a 6.4 cm cube of seeded water/bone/air ellipsoids, 1e5-1e7 F-18 decays each "
                  "(log-uniform, positron range on), point or cylinder sources, the positron workload's ring "
                  "and digitizer")


SURROGATE_MODEL = os.path.join(ROOT, "data", "surrogate_positron_ring.npz")


def _three_arms(ctxs, seeds, sur, steps, warmup, ncry):
    """One job of several loaded contexts in three forms: each its own plain
    Monte Carlo run (the plain form), plain Monte Carlo batched, and batched
    with the surrogate `sur`; device time per job (CUDA events), L2 flushed
    before each; the pooled singles of the two batched arms (independent
    seeds) compared by two-sample chi-square."""
    import numpy as np
    import torch
    from gpet_gb300 import api
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda:0")

    def reseed(k):
        for c, sd in zip(ctxs, seeds):
            c.set_option("seed", sd + 1000003 * k)

    def arm(kind, k0):
        for c in ctxs:
            c.set_surrogate(sur if kind == "surrogate_batched" else None)
        tot = {"ms": 0.0, "det": 0.0, "coinc": 0, "decays": 0, "nsur": 0, "entered": 0, "launches": 0,
               "true": 0, "scatter": 0, "random": 0, "singles": 0}
        he, hc = np.zeros(60), np.zeros(ncry)
        for k in range(-warmup, steps):
            flush.zero_()
            torch.cuda.synchronize()
            reseed(k0 + k)
            if kind == "plain_separate":
                st = [c.run() for c in ctxs]
                ms = sum(x["ms_total"] for x in st)
                det = sum(x["ms_detector"] for x in st)
                launches = sum(x["kernel_launches"] for x in st)
            else:
                st = api.run_batched(ctxs)
                ms, det, launches = st[0]["ms_total"], st[0]["ms_detector"], st[0]["kernel_launches"]
            if k < 0:
                continue
            tot["ms"] += ms; tot["det"] += det; tot["launches"] += launches
            for key, f in (("coinc", "n_coinc"), ("decays", "n_decays"), ("nsur", "n_surrogate"),
                           ("entered", "n_entered"), ("true", "n_true"), ("scatter", "n_scatter"),
                           ("random", "n_random"), ("singles", "n_singles")):
                tot[key] += sum(x[f] for x in st)
            if kind != "plain_separate":
                for c in ctxs:
                    s_ev, _ = c.singles()
                    he += np.histogram(s_ev["E"], bins=60, range=(3.5e5, 6.5e5))[0]
                    hc += np.bincount(s_ev["cryn"], minlength=ncry)[:ncry]
        r = {"value": tot["coinc"] / (tot["ms"] * 1e-3), "unit": UNIT, "ms_per_job": tot["ms"] / steps,
             "detector_ms_per_job": tot["det"] / steps, "coincidences_per_job": tot["coinc"] / steps,
             "singles_per_job": tot["singles"] / steps, "gpu_launches_per_job": tot["launches"] / steps,
             "classes_per_job": {"true": tot["true"] / steps, "scatter": tot["scatter"] / steps,
                                 "random": tot["random"] / steps}}
        if kind == "surrogate_batched":
            r["fraction_of_entered_photons"] = tot["nsur"] / max(1, tot["entered"])
        return r, he, hc, tot

    plain_sep, _, _, _ = arm("plain_separate", 0)
    plain_bat, mc_e, mc_c, t_bat = arm("plain_batched", 0)
    sur_bat, su_e, su_c, _ = arm("surrogate_batched", 50000)
    for c in ctxs:
        c.set_surrogate(None)
    big = mc_c >= 1000
    rel = (su_c[big] / su_c.sum()) / (mc_c[big] / mc_c.sum()) - 1.0
    det_share = plain_bat["detector_ms_per_job"] / plain_bat["ms_per_job"]
    return {
        "decays_per_job": t_bat["decays"] / steps, "steps": steps, "warmup": warmup,
        "l2": "flushed before each job (512 MB write)",
        "plain_separate": plain_sep, "plain_batched": plain_bat, "surrogate_batched": sur_bat,
        "speedup_vs_plain_separate": sur_bat["value"] / plain_sep["value"],
        "speedup_vs_plain_batched": sur_bat["value"] / plain_bat["value"],
        "batching_speedup_plain": plain_bat["value"] / plain_sep["value"],
        "parity_vs_plain_batched": {"singles_energy_350_650keV": _chi2(mc_e, su_e),
                                    "singles_per_crystal": _chi2(mc_c, su_c),
                                    "per_crystal_max_rel_dev": float(np.abs(rel).max()),
                                    "per_crystal_within_2pct": bool(np.abs(rel).max() < 0.02),
                                    "singles_plain": float(mc_c.sum()), "singles_surrogate": float(su_c.sum())},
        "amdahl": {"detector_share_of_plain_batched_job": det_share,
                   "bound_free_detector_vs_plain_batched": 1.0 / max(1e-9, 1.0 - det_share),
                   "bound_free_detector_vs_plain_separate":
                       plain_bat["value"] / plain_sep["value"] / max(1e-9, 1.0 - det_share)},
    }


SURROGATE_ARCH = ("16 inputs (entry y, z; direction; E; 6-wide panel embedding; 4 in-crystal offsets) -> "
                  "4 x 256 SiLU -> 204 outputs (two crystal sets of 64 logits by energy class, factorised into "
                  "32 row + 32 column logits above 64 crystals; MoG-4 depth; 64 energy bins); BASELINE's "
                  "surrogate configuration names 14 inputs with an 8-wide embedding and 140 outputs")


def _model_meta(path, meta, domain="entry energy 100-520 keV, >= 3 mm inside the panel edges, all panels"):
    return {"file": os.path.relpath(path, ROOT), "architecture": SURROGATE_ARCH,
            "train_records": meta.get("train_records"), "epochs": meta.get("train", {}).get("epochs"),
            "calibration_records": meta.get("calibration_records"), "domain": domain}


def measure_surrogate_batched(steps, warmup, model_path=SURROGATE_MODEL):
    """The metric's second form: the 64-simulation job (BATCH_WORKLOAD) with
    the learned detector response (the committed model, trained by
    data/make_surrogate.py with the library's kernels), batched in one job,
    against the plain form and plain batched (_three_arms)."""
    from gpet_gb300 import api, scenes
    data = os.path.join(ROOT, "data")
    with tempfile.TemporaryDirectory() as d:
        sims = scenes.batched(d)
        ctxs = []
        for bs in sims:
            c = api.Context(0)
            c.set_options(dict(bs.options, data_dir=data, base_dir=d))
            c.load_config(bs.config_path)
            mat, den = bs.phantom()
            c.set_phantom(mat, den, (bs.nvox,) * 3, (-3.2,) * 3, (6.4,) * 3)
            c.set_source_file(bs.source_path, 0.0, 120.0)
            ctxs.append(c)
        sur = api.Surrogate(ctxs[0], seed=1)
        meta = sur.load(model_path)
        res = _three_arms(ctxs, [bs.options["seed"] for bs in sims], sur, steps, warmup, 64)
        for c in ctxs:
            c.close()
        sur.close()
    return dict({"workload": BATCH_WORKLOAD, "simulations": len(sims)}, **res,
                model=_model_meta(model_path, meta))


WHOLEBODY_MODEL = os.path.join(ROOT, "data", "surrogate_wholebody_ring.npz")
BEDS_WORKLOAD = ("whole-body in 8 bed positions: the large workload's body (256x256x512 x 2 mm) and source "
                 "shifted along z in 6.4 cm steps through the 48-panel ring (16x16 crystals 4x4x20 mm), "
                 "1e9 F-18 decays in all (1.25e8 per bed), one simulation per bed")


def run_beds_workload(args):
    """BASELINE's whole-body configuration as plain Monte Carlo and as
    surrogate + batched (8 bed positions batched): the three arms of
    _three_arms with the committed whole-body model."""
    import torch
    from gpet_gb300 import api, formats as F, scenes
    torch.cuda.set_device(0)
    data = os.path.join(ROOT, "data")
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        beds = scenes.large_beds(d, decays_per_bed=args.decays // 8)
        cfg = F.read_config(beds[0].config_path)
        mat, den = F.read_phantom(cfg.matfile, cfg.denfile, tuple(cfg.pdim))
        ctxs = []
        for b in beds:
            c = api.Context(0)
            c.set_options(dict(b.options, data_dir=data, base_dir=d))
            c.load_config(b.config_path)
            c.set_phantom(mat, den, b.dims, b.offset, b.size)
            c.set_source_file(b.source_path, 0.0, 120.0)
            ctxs.append(c)
        setup_s = time.perf_counter() - t0
        sur = api.Surrogate(ctxs[0], seed=1)
        meta = sur.load(args.model or WHOLEBODY_MODEL)
        sampler = ClockSampler(0)
        sampler.start()
        res = _three_arms(ctxs, [b.options["seed"] for b in beds], sur, args.steps, args.warmup, 256)
        clocks = sampler.stop()
        for c in ctxs:
            c.close()
        sur.close()
    sb = res["surrogate_batched"]
    line = {"metric": METRIC.replace("(plain MC)", "(whole-body: surrogate detector response, 8 bed positions "
                                                   "batched)"),
            "value": sb["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sb["ms_per_job"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 (MLP), f32 (transport)", "data": "synthetic (seeded)",
            "config": {"workload": BEDS_WORKLOAD, "decays_per_step": args.decays, "beds": len(beds),
                       "l2": "flushed between steps (512 MB write)"},
            "setup_s": setup_s, "clocks": clocks,
            "model": _model_meta(args.model or WHOLEBODY_MODEL, meta)}
    line.update(res)
    print(json.dumps(line), flush=True)


def run_batched_workload(args, surrogate=False):
    """The 64-simulation job, once batched (gpet_run_batched) and once as 64
    separate runs, on the same contexts. surrogate: instead, the batched job
    with and without a learned detector response (trained, untimed, on entry
    records of the positron workload, whose ring the 64 simulations share),
    on independent seeds, with the two-sample chi-square of the pooled
    singles spectra and crystal maps."""
    import numpy as np
    import torch
    from gpet_gb300 import api, scenes
    torch.cuda.set_device(0)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda:0")
    with tempfile.TemporaryDirectory() as d:
        sims = scenes.batched(d, n_sims=args.batch_sims)
        data = os.path.join(ROOT, "data")
        ctxs = []
        t0 = time.perf_counter()
        for bs in sims:
            ctx = api.Context(0)
            ctx.set_options(dict(bs.options, data_dir=data, base_dir=d))
            ctx.load_config(bs.config_path)
            mat, den = bs.phantom()
            ctx.set_phantom(mat, den, (bs.nvox,) * 3, (-3.2,) * 3, (6.4,) * 3)
            ctx.set_source_file(bs.source_path, 0.0, 120.0)
            ctxs.append(ctx)
        setup_s = time.perf_counter() - t0
        seeds = [bs.options["seed"] for bs in sims]
        sur, train = None, None
        if surrogate:
            t0 = time.perf_counter()
            ps = scenes.positron(os.path.join(d, "train"), n_decays=args.train_decays)
            gen = api.Context(0)
            gen.set_options(dict(ps.options, data_dir=data, base_dir=ps.directory, record_entries=1, seed=555))
            gen.load_config(ps.config_path)
            gen.run()
            rec = gen.entries()
            sur = api.Surrogate(gen, seed=9)
            losses = sur.train(rec, epochs=args.train_epochs, batch=8192, lr=2e-3)
            sur.set_domain(1.0e5, 5.2e5, 0.3)
            calib = sur.calibrate(rec, iters=args.calib_iters) if args.calib_iters > 0 else None
            gen.close()
            train = {"decays": args.train_decays, "records": int(len(rec)), "epochs": args.train_epochs,
                     "loss_last_epoch": float(losses[-1]), "calibration_passes": args.calib_iters,
                     "calibration_last_max_log_ratio": calib, "seconds": time.perf_counter() - t0}

        def reseed(k):
            for c, sd in zip(ctxs, seeds):
                c.set_option("seed", sd + 1000003 * k)

        def batched_arm(k0, with_sur):
            for c in ctxs:
                c.set_surrogate(sur if with_sur else None)
            for w in range(args.warmup):
                reseed(k0 + 100 + w)
                api.run_batched(ctxs)
            sampler = ClockSampler(0)
            torch.cuda.synchronize()
            sampler.start()
            tot = {"ms": 0.0, "coinc": 0, "decays": 0, "launches": 0, "wall": 0.0, "nsur": 0, "entered": 0,
                   "det": 0.0}
            hist_e, hist_c = np.zeros(60), np.zeros(64)
            for k in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                reseed(k0 + k)
                t0 = time.perf_counter()
                st = api.run_batched(ctxs)
                tot["wall"] += time.perf_counter() - t0
                tot["ms"] += st[0]["ms_total"]
                tot["det"] += st[0]["ms_detector"]
                tot["coinc"] += sum(x["n_coinc"] for x in st)
                tot["decays"] += sum(x["n_decays"] for x in st)
                tot["nsur"] += sum(x["n_surrogate"] for x in st)
                tot["entered"] += sum(x["n_entered"] for x in st)
                tot["launches"] += st[0]["kernel_launches"]
                if surrogate:
                    for c in ctxs:
                        s_ev, _ = c.singles()
                        hist_e += np.histogram(s_ev["E"], bins=60, range=(3.5e5, 6.5e5))[0]
                        hist_c += np.bincount(s_ev["cryn"], minlength=64)[:64]
            return tot, sampler.stop(), hist_e, hist_c

        mc, clocks, mc_e, mc_c = batched_arm(0, False)
        if surrogate:
            su, clocks, su_e, su_c = batched_arm(50000, True)
        else:
            # the same simulations one after another
            ms_s, coinc_s, wall_s, launches_s = 0.0, 0, 0.0, 0
            for k in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                reseed(k)
                for c in ctxs:
                    t0 = time.perf_counter()
                    st = c.run()
                    wall_s += time.perf_counter() - t0
                    ms_s += st["ms_total"]
                    coinc_s += st["n_coinc"]
                    launches_s += st["kernel_launches"]
        for c in ctxs:
            c.close()
    base = {"unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "data": "synthetic (seeded)",
            "config": {"workload": BATCH_WORKLOAD, "simulations": len(sims),
                       "decays_per_step": mc["decays"] // max(1, args.steps),
                       "l2": "flushed between steps (512 MB write)"},
            "setup_s": setup_s, "clocks": clocks}
    if surrogate:
        line = dict(base, metric=METRIC.replace("(plain MC)", "(surrogate detector response, batched simulations)"),
                    value=su["coinc"] / (su["ms"] * 1e-3), ms_per_step=su["ms"] / args.steps,
                    dtype="bf16 (MLP), f32 (transport)", gpu_launches=su["launches"],
                    decays_per_s=su["decays"] / (su["ms"] * 1e-3))
        line["config"] = dict(base["config"], training=train,
                              domain="entry energy 100-520 keV, >= 3 mm inside the panel edges, all panels")
        line["plain_mc_batched"] = {"value": mc["coinc"] / (mc["ms"] * 1e-3), "ms_per_step": mc["ms"] / args.steps,
                                    "detector_ms_per_step": mc["det"] / args.steps}
        line["surrogate"] = {"detector_ms_per_step": su["det"] / args.steps,
                             "photons_per_step": su["nsur"] / args.steps,
                             "fraction_of_entered": su["nsur"] / max(1, su["entered"])}
        line["parity"] = {"singles_energy_350_650keV": _chi2(mc_e, su_e), "singles_per_crystal": _chi2(mc_c, su_c),
                          "singles_mc": float(mc_e.sum()), "singles_surrogate": float(su_e.sum()),
                          "coincidences_mc": mc["coinc"], "coincidences_surrogate": su["coinc"]}
    else:
        line = dict(base, metric=METRIC.replace("(plain MC)", "(plain MC, batched simulations)"),
                    value=mc["coinc"] / (mc["ms"] * 1e-3), ms_per_step=mc["ms"] / args.steps, dtype="f32",
                    gpu_launches=mc["launches"], decays_per_s=mc["decays"] / (mc["ms"] * 1e-3),
                    host_wall_per_step_s=mc["wall"] / args.steps,
                    separate_runs={"value": coinc_s / (ms_s * 1e-3), "ms_per_step": ms_s / args.steps,
                                   "host_wall_per_step_s": wall_s / args.steps,
                                   "gpu_launches": launches_s, "same_coincidences": coinc_s == mc["coinc"]})
    print(json.dumps(line), flush=True)


def _chi2(a, b):
    """Two-sample chi-square of histograms with counts a and b (same bins)."""
    import numpy as np
    from scipy import stats
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    keep = (a + b) > 0
    a, b = a[keep], b[keep]
    ka = np.sqrt(b.sum() / a.sum())
    kb = 1.0 / ka
    chi2 = float((((ka * a - kb * b) ** 2) / (a + b)).sum())
    ndf = int(keep.sum()) - 1
    # relative deviations over the bins holding at least 1000 counts in each
    big = (a >= 1000) & (b >= 1000)
    rel = np.abs(b[big] / b.sum() - a[big] / a.sum()) / (a[big] / a.sum())
    return {"chi2": chi2, "ndf": ndf, "p": float(stats.chi2.sf(chi2, ndf)),
            "max_rel_dev": float(rel.max()) if big.any() else None,
            "mean_rel_dev": float(rel.mean()) if big.any() else None}


def run_surrogate_workload(args):
    """The headline workload with the learned detector response: training on
    entry records of independent Monte Carlo runs (untimed), then acquisitions
    with and without the surrogate (independent seeds), timed like the
    headline, and the two-sample chi-square of their singles spectra and
    crystal maps."""
    import numpy as np
    import torch
    from gpet_gb300 import api
    torch.cuda.set_device(0)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda:0")
    peak_t = 1917.6
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak_t = float(json.load(f)["bf16_tflops"])
    except Exception:
        pass
    with tempfile.TemporaryDirectory() as d:
        sc = make_scene(d, args.decays, args.workload)
        data = os.path.join(ROOT, "data")

        def ctx_for(**extra):
            c = api.Context(0)
            c.set_options(dict(sc.options, data_dir=data, base_dir=d, **extra))
            c.load_config(sc.config_path)
            return c

        t0 = time.perf_counter()
        if args.model:
            # the committed model (data/make_surrogate.py)
            gen = ctx_for(n_decays=1000)
            sur = api.Surrogate(gen, seed=9)
            meta = sur.load(args.model)
            rec, losses, calib = np.zeros(meta["train_records"]), meta["loss_per_epoch"], \
                meta["calibration_last_max_log_ratio"]
        else:
            gen = ctx_for(record_entries=1, n_decays=args.train_decays, seed=555)
            gen.run()
            rec = gen.entries()
            sur = api.Surrogate(gen, seed=9)
            losses = sur.train(rec, epochs=args.train_epochs, batch=8192, lr=2e-3)
            sur.set_domain(1.0e5, 5.2e5, 0.3)
            calib = sur.calibrate(rec, iters=args.calib_iters) if args.calib_iters > 0 else None
            gen.close()
        train_s = time.perf_counter() - t0
        res = {}
        for mode in ("mc", "surrogate"):
            ctx = ctx_for()
            ctx.autotune(1 << 23)
            if mode == "surrogate":
                ctx.set_surrogate(sur)
            for w in range(args.warmup):
                ctx.set_option("seed", 1000 + w)
                ctx.run()
            tot = {"ms": 0.0, "det": 0.0, "sur": 0.0, "coinc": 0, "nsur": 0, "entered": 0}
            hist_e = np.zeros(60)
            hist_c = np.zeros(64)
            for k in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                ctx.set_option("seed", (20261203 if mode == "mc" else 40261203) + k)
                st = ctx.run()
                tot["ms"] += st["ms_total"]; tot["det"] += st["ms_detector"]; tot["sur"] += st["ms_surrogate"]
                tot["coinc"] += st["n_coinc"]; tot["nsur"] += st["n_surrogate"]; tot["entered"] += st["n_entered"]
                s_ev, _ = ctx.singles()
                hist_e += np.histogram(s_ev["E"], bins=60, range=(3.5e5, 6.5e5))[0]
                hist_c += np.bincount(s_ev["cryn"], minlength=64)[:64]
            res[mode] = (tot, hist_e, hist_c)
            ctx.close()
    mc, su = res["mc"][0], res["surrogate"][0]
    flops = 2 * 252928 * su["nsur"]
    ach = flops / max(su["sur"] * 1e-3, 1e-12) / 1e12
    line = {"metric": METRIC.replace("(plain MC)", "(surrogate detector response)"),
            "value": su["coinc"] / (su["ms"] * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": su["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (MLP), f32 (transport)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "decays_per_step": args.decays,
                       "training": {"decays": args.train_decays, "records": int(len(rec)),
                                    "epochs": args.train_epochs, "loss_per_epoch": [float(x) for x in losses],
                                    "calibration_passes": args.calib_iters,
                                    "calibration_last_max_log_ratio": calib, "seconds": train_s},
                       "domain": "entry energy 100-520 keV, >= 3 mm inside the panel edges, all panels"},
            "plain_mc": {"value": mc["coinc"] / (mc["ms"] * 1e-3), "ms_per_step": mc["ms"] / args.steps,
                         "detector_ms_per_step": mc["det"] / args.steps},
            "surrogate": {"detector_ms_per_step": su["det"] / args.steps,
                          "mlp_ms_per_step": su["sur"] / args.steps,
                          "photons_per_step": su["nsur"] / args.steps,
                          "fraction_of_entered": su["nsur"] / max(1, su["entered"])},
            "roofline_mlp": {"kernel": "k_mlp_fwd<false>", "bound": "tensor", "achieved": ach, "peak": peak_t,
                             "unit": "TFLOP/s", "frac": ach / peak_t,
                             "flops_per_photon": 2 * 252928},
            "parity": {"singles_energy_350_650keV": _chi2(res["mc"][1], res["surrogate"][1]),
                       "singles_per_crystal": _chi2(res["mc"][2], res["surrogate"][2]),
                       "singles_mc": float(res["mc"][1].sum()), "singles_surrogate": float(res["surrogate"][1].sum()),
                       "coincidences_mc": mc["coinc"], "coincidences_surrogate": su["coinc"]}}
    print(json.dumps(line), flush=True)


WIDEN_WORKLOAD = ("widen: the positron workload with one optional feature at a time - phase-space records of "
                  "the emitted and escaped photons, a quadric exclusion (cylinder r=6 mm along each crystal "
                  "block's depth axis), two-material crystals (back 10 mm LSO), background singles (Poisson, "
                  "mean gap 270 us, 511 +- 60 keV), and the sinogram of the run's coincidences")


def run_widen_workload(args):
    """Cost of each widened feature on the positron workload: per variant W
    untimed and K timed acquisitions (device time of the run's CUDA events,
    host wall time beside it, L2 flushed before each), with the launch shape
    the tuner picks for the plain run. Phase-space records are kept for
    args.psf_decays decays per step (host memory: 80 B per decay)."""
    import numpy as np
    import torch
    from gpet_gb300 import api, formats as F, scenes
    torch.cuda.set_device(0)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda:0")
    data = os.path.join(ROOT, "data")
    res = {}
    with tempfile.TemporaryDirectory() as d:
        sc = make_scene(d, args.decays, "positron")

        def variant_config(name, surfaces=None, geo=None):
            cfg = F.read_config(sc.config_path)
            if surfaces is not None:
                cfg.surfaces = surfaces
            if geo is not None:
                cfg.geofile = geo
            path = os.path.join(d, "input_%s.in" % name)
            F.write_config(path, cfg)
            return path

        geo3 = os.path.join(d, "ring3.geo")
        F.write_geo(geo3, 8, (0, 0, 1), 45.0, (scenes.MAT_LYSO, scenes.MAT_AIR, 9), (7.1, 0.001025, 7.4),
                    scenes.ring_panel0(8.0, 8, 8, 0.298, 0.002, 2.0))
        variants = [
            ("plain", sc.config_path, {}, args.decays),
            ("phase_space", sc.config_path, {"record_source": 1, "record_exits": 1}, args.psf_decays),
            ("quadric_exclusion", variant_config("quadric", [[0, 1, 1, 0, 0, 0, 0, 0, 0, -0.6 ** 2]]), {},
             args.decays),
            ("two_material_crystals", variant_config("lso", [[0, 0, 0, 0, 0, 0, 1, 0, 0, 1.0]], geo3), {},
             args.decays),
            ("background_singles", sc.config_path,
             {"noise_lambda_us": 270.0, "noise_emean_ev": 511000.0, "noise_sigma_ev": 60000.0}, args.decays),
        ]
        shape = None
        for name, cfg_path, extra, nd in variants:
            ctx = api.Context(0)
            opts = dict(sc.options, data_dir=data, base_dir=d, n_decays=nd)
            opts.update(args.set)
            opts.update(extra)
            ctx.set_options(opts)
            ctx.load_config(cfg_path)
            if shape is None:
                shape = ctx.autotune(args.tune_decays) if args.autotune else None
            elif shape:
                ctx.set_options({"sub_decays": shape["sub_decays"], "chunk_decays": shape["chunk_decays"],
                                 "source_threads": shape["source_threads"],
                                 "detector_threads": shape["detector_threads"],
                                 "drain_period": shape["drain_period"]})
            for w in range(args.warmup):
                ctx.set_option("seed", 1000 + w)
                ctx.run()
            tot = {"ms": 0.0, "wall": 0.0, "src": 0.0, "ph": 0.0, "det": 0.0, "dig": 0.0, "coinc": 0, "singles": 0,
                   "hits": 0, "noise": 0, "records": 0}
            for k in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                ctx.set_option("seed", 20261203 + k)
                t0 = time.perf_counter()
                st = ctx.run()
                tot["wall"] += time.perf_counter() - t0
                tot["ms"] += st["ms_total"]; tot["src"] += st["ms_source"]; tot["ph"] += st["ms_phantom"]
                tot["det"] += st["ms_detector"]; tot["dig"] += st["ms_digitizer"] + st["ms_coincidence"]
                tot["coinc"] += st["n_coinc"]; tot["singles"] += st["n_singles"]; tot["hits"] += st["n_hits"]
                tot["noise"] += st["n_noise"]
                if name == "phase_space":
                    tot["records"] += ctx._count(ctx.L.gpet_get_source_records, None)
                    tot["records"] += ctx._count(ctx.L.gpet_get_phantom_records, None)
            K = args.steps
            r = {"decays_per_step": nd, "ms_per_step": tot["ms"] / K, "wall_ms_per_step": 1e3 * tot["wall"] / K,
                 "decays_per_s": nd / (tot["ms"] / K * 1e-3),
                 "stage_ms": {"source": tot["src"] / K, "phantom": tot["ph"] / K, "detector": tot["det"] / K,
                              "digitizer_and_coincidences": tot["dig"] / K},
                 "coincidences_per_step": tot["coinc"] / K, "singles_per_step": tot["singles"] / K,
                 "coincidences_per_s": tot["coinc"] / (tot["ms"] * 1e-3)}
            if name == "phase_space":
                r["records_per_step"] = tot["records"] / K
                r["records_per_s_wall"] = tot["records"] / tot["wall"]
            if name == "background_singles":
                r["background_singles_per_step"] = tot["noise"] / K
            if name == "plain":
                # sinogram of the last run's coincidences (host clock: launch, binning, copy-back)
                ts = []
                for _ in range(5):
                    t0 = time.perf_counter()
                    sino = ctx.sinogram(128, 96, 8, 6.0, 1.2)
                    ts.append(time.perf_counter() - t0)
                t_s = statistics.median(ts)
                r["sinogram"] = {"bins": [8, 96, 128], "ms": 1e3 * t_s, "coincidences": int(st["n_coinc"]),
                                 "binned": int(sino.sum()), "coincidences_per_s": st["n_coinc"] / t_s}
            res[name] = r
            ctx.close()
    base = res["plain"]["ms_per_step"]
    for name, r in res.items():
        r["ms_vs_plain"] = r["ms_per_step"] / base * (res["plain"]["decays_per_step"] / r["decays_per_step"])
    line = {"metric": "cost of the widened features (device ms per acquisition)", "workload": "widen",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WIDEN_WORKLOAD, "base": WORKLOAD, "l2": "flushed before each acquisition"},
            "launch_shape": shape if shape else "library defaults", "variants": res}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--decays", type=int, default=None,
                    help="decays per step (default 1e8; 1e9 for the large workload)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=0.0,
                    help="reference arm: decays per step sized to about this many seconds (0: the whole workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--autotune", action=argparse.BooleanOptionalAction, default=True,
                    help="time launch shapes on a sample before the warm-up (results do not depend on the shape)")
    ap.add_argument("--tune-decays", type=int, default=1 << 24)
    ap.add_argument("--set", action="append", default=[], metavar="KEY=VALUE",
                    help="context option for the headline workload (e.g. a fixed launch shape for profiling)")
    ap.add_argument("--e2e-steps", type=int, default=-1,
                    help="steps of the end-to-end leg (default max(2, steps/2); 0 skips it: profiling only)")
    ap.add_argument("--surrogate-steps", type=int, default=3,
                    help="jobs per arm of the surrogate+batched measurement in the default line (0: skip)")
    ap.add_argument("--gloo", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--workload", choices=["positron", "batched64", "surrogate", "surrogate_batched64", "large", "widen",
                                           "beds"],
                    default="positron",
                    help="positron: the headline workload; batched64: 64 uneven simulations in one job; "
                         "surrogate: the headline workload with the learned detector response; "
                         "surrogate_batched64: the 64-simulation job with and without it; "
                         "large: the whole-body configuration (48 panels, 256x256x512 phantom); "
                         "beds: the whole-body configuration in 8 bed positions, plain and surrogate + batched")
    ap.add_argument("--train-decays", type=int, default=200_000_000, help=argparse.SUPPRESS)
    ap.add_argument("--train-epochs", type=int, default=12, help=argparse.SUPPRESS)
    ap.add_argument("--batch-sims", type=int, default=64, help=argparse.SUPPRESS)
    ap.add_argument("--psf-decays", type=int, default=10_000_000, help=argparse.SUPPRESS)
    ap.add_argument("--calib-iters", type=int, default=10, help=argparse.SUPPRESS)
    ap.add_argument("--model", default=None,
                    help="surrogate workload: load this model (e.g. data/surrogate_positron_ring.npz) instead of "
                         "training one")
    args = ap.parse_args()
    args.set = dict(kv.split("=", 1) for kv in args.set)
    if args.decays is None:
        args.decays = 1_000_000_000 if args.workload in ("large", "beds") else 100_000_000
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched64":
        run_batched_workload(args)
    elif args.workload == "surrogate_batched64":
        run_batched_workload(args, surrogate=True)
    elif args.workload == "surrogate":
        run_surrogate_workload(args)
    elif args.workload == "widen":
        run_widen_workload(args)
    elif args.workload == "beds":
        run_beds_workload(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
