"""The sharded path on CPU ranks (gloo, world size 2): each rank runs its
block of the neutron index range and the tallies are summed with one
all-reduce; the result equals the single-process run (Philox counters make
neutron i the same neutron on any rank).  Per-rank compute uses the CPU
oracle, the collective is the same torch.distributed all-reduce
acc_gb300.sharding.reduce_tallies issues between GPUs."""

import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

NEUTRONS = 60_001


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from acc_gb300 import instruments
    from acc_gb300.sharding import reduce_tallies, shard_range
    from helpers import oracle_run
    first, count = shard_range(NEUTRONS, rank, world)
    tallies, stats, _, _ = oracle_run(instruments.guide_chain(), count,
                                      seed=17, first=first, nthreads=1)
    assert stats["processed"] == count
    ts = [torch.from_numpy(np.ascontiguousarray(t)) for t in tallies.values()]
    reduce_tallies(ts)
    if rank == 0:
        np.savez(os.path.join(out_dir, "reduced.npz"),
                 *[t.numpy() for t in ts])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_sum_to_single_run(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import oracle_run
    from acc_gb300 import instruments
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path)))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    got = np.load(tmp_path / "reduced.npz")
    ref, _, _, _ = oracle_run(instruments.guide_chain(), NEUTRONS, seed=17,
                              nthreads=1)
    for k, r in enumerate(ref.values()):
        g = got[f"arr_{k}"].reshape(r.shape)
        np.testing.assert_array_equal(g[0], r[0])
        np.testing.assert_allclose(g[1:], r[1:], rtol=1e-12, atol=1e-300)
        assert r[0].sum() > 0
