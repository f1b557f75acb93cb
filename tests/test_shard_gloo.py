"""Replicas over several ranks: partition, local scoring, host gather (gloo, world size 2, CPU).

Each rank scores its share with the CPU oracle (a stand-in for its own GPU
engine; no GPU is used), and the gathered results must equal a single-process
run region for region.
"""
import os

import numpy as np
import pytest

from phylocsf_gb300 import shard


def test_partition_longest_first_balances():
    lengths = [100, 5, 80, 60, 7, 40, 3]
    parts = shard.partition_longest_first(lengths, 2)
    assert sorted(np.concatenate(parts).tolist()) == list(range(len(lengths)))
    loads = [sum(lengths[i] for i in p) for p in parts]
    assert abs(loads[0] - loads[1]) <= max(lengths)
    assert [p.tolist() for p in shard.partition_longest_first(lengths, 1)] == [list(range(len(lengths)))]


def _oracle_scorer():
    from oracle import oracle as O
    from tests import helpers as H
    O.set_sparse_leaves(True)
    mc, mn, ot, tree = H.oracle_models("12flies")
    dt = np.dtype([("score", "f8"), ("anc", "f8"), ("status", "i4")])

    def score(offs, lv):
        out = np.zeros(len(offs) - 1, dt)
        for r in range(len(offs) - 1):
            res = O.score_region(mc, mn, ot, O.FIXED, H.u8_to_oracle(lv[offs[r]:offs[r + 1]]))
            out[r] = (res.score, res.anc, res.status)
        return out
    return score


def _data():
    from phylocsf_gb300 import synth
    ps = synth.load_params("12flies")
    rng = np.random.default_rng(5)
    lengths = rng.integers(0, 60, size=9)
    return synth.simulate(ps, lengths, (np.arange(9) % 2).astype(np.int32), None, 5)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    offs, lv = _data()
    res = shard.score_sharded(offs, lv, _oracle_scorer(), rank, world)
    q.put((rank, res))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process():
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    offs, lv = _data()
    ref = _oracle_scorer()(offs, lv)
    for rank, res in got:
        assert np.array_equal(res["score"], ref["score"]), rank
        assert np.array_equal(res["status"], ref["status"])
