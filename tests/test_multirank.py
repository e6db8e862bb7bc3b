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
