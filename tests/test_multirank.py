"""The multi-GPU form of the path is independent acquisitions per rank
(disjoint Philox keys, no data exchange); only the timing and the totals are
reduced. Covered here with two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, oracle_for


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, c = bench.combine_ranks(10.0 + rank, 100 * (rank + 1), dist, "cpu")
    out[rank] = (ms, c)
    dist.destroy_process_group()


def test_combine_ranks_gloo_two_ranks():
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == (11.0, 300.0)


def test_single_rank_combine():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(5.0, 7) == (5.0, 7.0)


def test_ranks_draw_disjoint_streams(scene_small, data_dir, oracle_mod):
    a = oracle_for(scene_small, data_dir, sim_id=0).run(0, 4000, exits=True)["exits"]
    b = oracle_for(scene_small, data_dir, sim_id=1).run(0, 4000, exits=True)["exits"]
    esc = (a["status"] == 1) & (b["status"] == 1)
    assert np.mean(a["x"][esc] == b["x"][esc]) < 0.01


def test_bench_reference_arm_json_line():
    """`bench.py --impl reference` (the CPU arm the GPU arm is compared
    with) prints one JSON line with the contract's keys, on a small sample."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--decays", "30000", "--ref-step-seconds", "0.2"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["value"] > 0 and j["steps"] == 2 and j["warmup"] == 1
    for k in ("metric", "unit", "ms_per_step", "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert k in j, k
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["e2e"]["d2h_bytes_per_step"] == 0
    assert j["cpu_baseline"]["kind"] == "port"


def test_bench_reference_arm_under_torchrun_two_ranks():
    """Launched as the two-rank job of the bench contract (torchrun, one
    process per rank), the reference arm prints exactly one JSON line, from
    rank 0, and every rank exits 0."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(root, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1", "--decays", "30000",
           "--ref-step-seconds", "0.2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["n_gpus"] == 2 and j["value"] > 0


def test_bench_parity_vs_oracle_helper(data_dir, oracle_mod, tmp_path):
    """The bench line's parity object: two independent acquisitions of one
    scene agree (spectrum and crystal map chi-square p-values, per-decay
    rates in standard deviations), and the oracle's seed is none the GPU
    steps use."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    from gpet_gb300 import scenes
    sc = scenes.positron(str(tmp_path), n_decays=400_000, nvox=48)
    o = oracle_mod.OracleScene(sc.config_path, dict(sc.options, seed=99), data_dir, base_dir=sc.directory)
    r = o.run(precision="fp32")
    counts = {"n_decays": 400_000, **{k: r[k] for k in ("n_singles", "n_coinc", "n_true", "n_scatter", "n_random")}}
    cb = bench.cpu_baseline(sc, 1.0, with_hists=True)
    part = cb.pop("_parity")
    assert part[2] == 4242 and "_parity" not in cb
    p = bench._parity_vs_oracle(bench._singles_hists(r["singles"]), counts, 99, part)
    assert p["singles_energy_350_650keV"]["ndf"] > 30 and p["singles_per_crystal"]["ndf"] == 63
    assert p["singles_energy_350_650keV"]["p"] > 1e-4 and p["singles_per_crystal"]["p"] > 1e-4
    assert set(p["rates"]) == {"singles", "coinc", "true", "scatter", "random"}
    assert abs(p["rates"]["singles"]["sigma"]) < 5
