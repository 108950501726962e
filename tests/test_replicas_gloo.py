"""Multi-GPU form of the path = independent replicas (no collective on the data
path).  Covered here on CPU with two gloo ranks: each rank builds its own
seeded instance, solves it with the oracle, and the ranks agree on the
throughput aggregation bench.py reports (all ranks' units / max rank time)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from oracle import oracle as O
    from theses_code_gb300 import workloads
    p, V2, C0 = workloads.convection_2d(24, 20, seed=11 + rank)  # one replica per rank
    C, _ = O.tg_solve(p, V2, C0, 8)
    t_ms = 100.0 + 50.0 * rank  # the slower rank sets the job time
    tt = torch.tensor([t_ms], dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    value = bench.aggregate_value(world, 24 * 24 * 8, 3, float(tt.item()))
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([[value, tt.item()], C]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r0 = np.load(tmp_path / "rank0.npy")
    r1 = np.load(tmp_path / "rank1.npy")
    # both ranks report the same job throughput: 2 * units * steps / max time
    assert r0[0] == r1[0] == pytest.approx(2 * 24 * 24 * 8 * 3 / 0.150)
    assert r0[1] == r1[1] == 150.0
    # the replicas solved different seeded instances
    assert not np.allclose(r0[2:], r1[2:])
