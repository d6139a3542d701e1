"""The sharded path on CPU ranks (gloo, world size 2): each rank runs its
block of the neutron index range through acc_gb300.sharding.run_sharded
(the product's entry point) and the tallies are summed with one
all-reduce; the result equals the single-process run (Philox counters make
neutron i the same neutron on any rank).  run_sharded's runner is the CPU
oracle here (the GPU's is the fused kernel); the collective is the same
torch.distributed all-reduce it issues between GPUs.  The gradient
reduction (sharding.reduce_gradients, used by a sharded GradRun) is checked
the same way: per-rank gradients of per-rank neutron blocks sum to the
gradient of the whole run."""

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
    from acc_gb300.sharding import run_sharded, shard_range
    from helpers import oracle_run
    ts = []

    def oracle_runner(ins, first, count):
        tallies, stats, _, _ = oracle_run(ins, count, seed=17, first=first,
                                          nthreads=1)
        ts.extend(torch.from_numpy(np.ascontiguousarray(t))
                  for t in tallies.values())
        return stats["processed"], ts

    processed = run_sharded(instruments.guide_chain(), NEUTRONS, rank, world,
                            runner=oracle_runner)
    assert processed == shard_range(NEUTRONS, rank, world)[1]
    if rank == 0:
        np.savez(os.path.join(out_dir, "reduced.npz"),
                 *[t.numpy() for t in ts])
    dist.barrier()
    dist.destroy_process_group()


def _grad_rank_main(rank, world, port, out_dir):
    """Each rank's 'gradient' of L = sum over its neutron block of a weight
    function (the exit weights of the oracle's run, a stand-in for the
    replayed d p / d theta), reduced with sharding.reduce_gradients."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from acc_gb300 import instruments
    from acc_gb300.sharding import reduce_gradients, shard_range
    from helpers import oracle_run
    first, count = shard_range(NEUTRONS, rank, world)
    _, _, out, last = oracle_run(instruments.guide_chain(), count, seed=17,
                                 first=first, nthreads=1, record=True)
    alive = out[:, 9] > 0
    grads = {"p": torch.tensor(out[alive, 9].sum(), dtype=torch.float64),
             "pv": torch.from_numpy((out[alive, 3:6] * out[alive, 9:10])
                                    .sum(axis=0))}
    reduce_gradients(grads)
    if rank == 0:
        np.savez(os.path.join(out_dir, "grads.npz"), p=grads["p"].numpy(),
                 pv=grads["pv"].numpy())
    dist.barrier()
    dist.destroy_process_group()


def _spawn(target, tmp_path, world=2):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, str(tmp_path)))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0


def test_two_rank_gradients_sum_to_single_run(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import oracle_run
    from acc_gb300 import instruments
    _spawn(_grad_rank_main, tmp_path)
    got = np.load(tmp_path / "grads.npz")
    _, _, out, _ = oracle_run(instruments.guide_chain(), NEUTRONS, seed=17,
                              nthreads=1, record=True)
    alive = out[:, 9] > 0
    np.testing.assert_allclose(got["p"], out[alive, 9].sum(), rtol=1e-12)
    np.testing.assert_allclose(
        got["pv"], (out[alive, 3:6] * out[alive, 9:10]).sum(axis=0),
        rtol=1e-12)


def test_two_rank_shards_sum_to_single_run(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from helpers import oracle_run
    from acc_gb300 import instruments
    _spawn(_rank_main, tmp_path)
    got = np.load(tmp_path / "reduced.npz")
    ref, _, _, _ = oracle_run(instruments.guide_chain(), NEUTRONS, seed=17,
                              nthreads=1)
    for k, r in enumerate(ref.values()):
        g = got[f"arr_{k}"].reshape(r.shape)
        np.testing.assert_array_equal(g[0], r[0])
        np.testing.assert_allclose(g[1:], r[1:], rtol=1e-12, atol=1e-300)
        assert r[0].sum() > 0
