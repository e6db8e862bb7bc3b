"""Train a learned detector response and write it to data/ (needs a GB300:
the training and the records come from the library's own kernels).

  positron ring (default) -> data/surrogate_positron_ring.npz
  --ring wholebody        -> data/surrogate_wholebody_ring.npz

The positron ring:

Training records: photons entering a panel, from plain Monte Carlo of the
positron workload (F-18 cylinder in the 128^3 water/bone/lung phantom) and of
the 64-simulation batched workload (point and cylinder sources in seeded
water/bone/air phantoms), which share the 8-panel LYSO ring; both kinds of
entry distribution are in the training set. Calibration (iterative
proportional fitting of the head's crystal and energy-bin biases) runs on an
independent record set of the same two workloads. The weights are saved at
the bf16 precision the tensor-core forward uses (inference is unchanged).

The whole-body ring (48 LYSO panels at 49 cm, 16 x 16 crystals of 4 x 4 x
20 mm, whose crystal head is factorised into rows and columns): records from
plain Monte Carlo of the whole-body workload at its eight bed positions (the
body shifted along z in 6.4 cm steps), training and calibration records from
independent seeds.

  python data/make_surrogate.py [out.npz] [--ring positron|wholebody] [--quick]
"""
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

OUT = os.path.join(HERE, "surrogate_positron_ring.npz")
OUT_WB = os.path.join(HERE, "surrogate_wholebody_ring.npz")
DOMAIN = (1.0e5, 5.2e5, 0.3)        # entry energy (eV), edge margin (cm)
TRAIN = dict(positron_decays=400_000_000, batched_jobs=2, epochs=10, batch=8192, lr=2e-3, seed=9)
CALIB = dict(positron_decays=200_000_000, batched_jobs=1, passes=16)
TRAIN_WB = dict(decays_per_bed=75_000_000, epochs=18, batch=8192, lr=2e-3, seed=9)
CALIB_WB = dict(decays_per_bed=40_000_000, passes=40)


def records_positron(sc, data, decays, seed):
    from gpet_gb300 import api
    out = []
    left, k = decays, 0
    while left > 0:
        n = min(left, 200_000_000)
        c = api.Context(0)
        c.set_options(dict(sc.options, data_dir=data, base_dir=sc.directory, record_entries=1, n_decays=n,
                           seed=seed + k))
        c.load_config(sc.config_path)
        c.run()
        out.append(c.entries())
        c.close()
        left -= n
        k += 1
    return np.concatenate(out)


def records_batched(ctxs, seeds, job):
    """Entry records of each simulation of the batched workload (one job,
    seeds offset by job), run one at a time (records are per context)."""
    out = []
    for c, sd in zip(ctxs, seeds):
        c.set_option("record_entries", 1)
        c.set_option("seed", sd + 7777777 * (job + 1))
        c.run()
        out.append(c.entries())
        c.set_option("record_entries", 0)
    return np.concatenate(out)


def batched_contexts(directory, data):
    from gpet_gb300 import api, scenes
    sims = scenes.batched(directory)
    ctxs = []
    for bs in sims:
        c = api.Context(0)
        c.set_options(dict(bs.options, data_dir=data, base_dir=directory))
        c.load_config(bs.config_path)
        mat, den = bs.phantom()
        c.set_phantom(mat, den, (bs.nvox,) * 3, (-3.2,) * 3, (6.4,) * 3)
        c.set_source_file(bs.source_path, 0.0, 120.0)
        ctxs.append(c)
    return ctxs, [bs.options["seed"] for bs in sims]


def bed_contexts(directory, data):
    """One context per bed position of the whole-body acquisition."""
    from gpet_gb300 import api, formats as F, scenes
    beds = scenes.large_beds(directory)
    cfg = F.read_config(beds[0].config_path)
    mat, den = F.read_phantom(cfg.matfile, cfg.denfile, tuple(cfg.pdim))
    ctxs = []
    for b in beds:
        c = api.Context(0)
        c.set_options(dict(b.options, data_dir=data, base_dir=directory))
        c.load_config(b.config_path)
        c.set_phantom(mat, den, b.dims, b.offset, b.size)
        c.set_source_file(b.source_path, 0.0, 120.0)
        ctxs.append(c)
    return ctxs, [b.options["seed"] for b in beds]


def records_beds(ctxs, seeds, decays, job):
    out = []
    for c, sd in zip(ctxs, seeds):
        c.set_options({"record_entries": 1, "n_decays": decays, "seed": sd + 7777777 * (job + 1)})
        c.run()
        out.append(c.entries())
        c.set_option("record_entries", 0)
    return np.concatenate(out)


def main_wholebody(out, quick):
    from gpet_gb300 import api
    train, calib = dict(TRAIN_WB), dict(CALIB_WB)
    if quick:
        train.update(decays_per_bed=5_000_000, epochs=2)
        calib.update(decays_per_bed=5_000_000, passes=4)
    data = os.path.join(ROOT, "data")
    t0 = time.perf_counter()
    with tempfile.TemporaryDirectory() as d:
        ctxs, seeds = bed_contexts(d, data)
        rec = records_beds(ctxs, seeds, train["decays_per_bed"], 0)
        sur = api.Surrogate(ctxs[0], seed=train["seed"])
        losses = sur.train(rec, epochs=train["epochs"], batch=train["batch"], lr=train["lr"])
        n_train = len(rec)
        del rec
        sur.set_domain(*DOMAIN)
        cal = records_beds(ctxs, seeds, calib["decays_per_bed"], 1)
        adj = sur.calibrate(cal, iters=calib["passes"])
        meta = {"ring": "whole-body workload: 48 LYSO panels at 49 cm, 16x16 crystals of 4x4x20 mm "
                        "(factorised crystal head), 8 bed positions",
                "train_records": int(n_train), "train": train, "loss_per_epoch": [float(x) for x in losses],
                "calibration_records": int(len(cal)), "calibration": calib,
                "calibration_last_max_log_ratio": float(adj), "seconds": time.perf_counter() - t0}
        sur.save(out, DOMAIN, **meta)
        sur.close()
        for c in ctxs:
            c.close()
    print(out, meta)


def main():
    from gpet_gb300 import api, scenes
    out = OUT
    if "--ring" in sys.argv and sys.argv[sys.argv.index("--ring") + 1] == "wholebody":
        args = [a for i, a in enumerate(sys.argv[1:], 1)
                if not a.startswith("--") and sys.argv[i - 1] != "--ring"]
        return main_wholebody(args[0] if args else OUT_WB, "--quick" in sys.argv)
    train, calib = dict(TRAIN), dict(CALIB)
    args = [a for i, a in enumerate(sys.argv[1:], 1) if not a.startswith("--") and sys.argv[i - 1] != "--ring"]
    if args:
        out = args[0]
    if "--quick" in sys.argv:   # a small run of the recipe (for checking it)
        train.update(positron_decays=20_000_000, batched_jobs=1, epochs=2)
        calib.update(positron_decays=20_000_000, batched_jobs=1, passes=4)
    data = os.path.join(ROOT, "data")
    t0 = time.perf_counter()
    with tempfile.TemporaryDirectory() as d:
        sc = scenes.positron(os.path.join(d, "positron"))
        ctxs, seeds = batched_contexts(os.path.join(d, "batched"), data)
        rec = np.concatenate([records_positron(sc, data, train["positron_decays"], 555)] +
                             [records_batched(ctxs, seeds, j) for j in range(train["batched_jobs"])])
        gen = api.Context(0)
        gen.set_options(dict(sc.options, data_dir=data, base_dir=sc.directory, n_decays=1000))
        gen.load_config(sc.config_path)
        sur = api.Surrogate(gen, seed=train["seed"])
        losses = sur.train(rec, epochs=train["epochs"], batch=train["batch"], lr=train["lr"])
        n_train = len(rec)
        del rec
        sur.set_domain(*DOMAIN)
        cal = np.concatenate([records_positron(sc, data, calib["positron_decays"], 10_555)] +
                             [records_batched(ctxs, seeds, 100 + j) for j in range(calib["batched_jobs"])])
        adj = sur.calibrate(cal, iters=calib["passes"])
        meta = {"ring": "positron workload: 8 LYSO panels at 8 cm, 8x8 crystals of 3x3x20 mm",
                "train_records": int(n_train), "train": train, "loss_per_epoch": [float(x) for x in losses],
                "calibration_records": int(len(cal)), "calibration": calib,
                "calibration_last_max_log_ratio": float(adj), "seconds": time.perf_counter() - t0}
        sur.save(out, DOMAIN, **meta)
        for c in ctxs:
            c.close()
    print(out, meta)


if __name__ == "__main__":
    main()
