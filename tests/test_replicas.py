"""Replica host logic on CPU with two gloo ranks (no GPU).

Each rank evaluates its shard of the golden emission case's parameter sets with
the FP64 oracle; the gathered log-likelihoods must equal the reference's golden
values in the global order on both ranks, and the max-over-ranks timing must be
the slowest rank's."""

import os
import socket

import numpy as np
import pytest

from bear_gb300.replicas import shard

HERE = os.path.dirname(os.path.abspath(__file__))


def test_shard_is_a_balanced_partition():
    for n in (0, 1, 7, 512, 1023):
        for world in (1, 2, 3, 8):
            rows = [list(range(n))[shard(n, r, world)] for r in range(world)]
            assert sum(rows, []) == list(range(n))
            sizes = [len(r) for r in rows]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case_path, out_dir):
    import sys
    sys.path[:0] = [os.path.dirname(HERE), os.path.join(os.path.dirname(HERE), "oracle"), HERE]
    import torch
    import torch.distributed as dist

    import goldenlib
    import oracle
    from bear_gb300.replicas import ReplicaBatch, max_over_ranks

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle.set_threads(1)
        c = goldenlib.Case(case_path)
        om = oracle.OracleModel(c.config_text(), c.observations())

        def evaluate(p):
            ll = torch.tensor([om.loglike(row) for row in p.numpy()], dtype=torch.float64)
            neg = torch.tensor([om.forward(row)[2] for row in p.numpy()], dtype=torch.uint8)
            return ll, neg

        ll, neg = ReplicaBatch(evaluate, dist)(torch.tensor(c.params))
        slowest = max_over_ranks(1.0 + rank, dist)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), ll=ll.numpy(), neg=neg.numpy(), slowest=slowest,
                 ref=c.arrays["ref_loglike"], ref_neg=c.arrays["ref_neglect"])
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_global_batch(tmp_path):
    import torch.multiprocessing as mp

    import goldenlib

    case = [p for p in goldenlib.golden_cases() if p.endswith("emission_edges.npz")][0]
    goldenlib.Case(case).table_root()  # tables written once, before the ranks start
    mp.spawn(_rank_main, args=(2, _free_port(), case, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        r = np.load(tmp_path / f"rank{rank}.npz")
        assert r["slowest"] == 2.0
        assert np.array_equal(r["neg"].astype(bool), r["ref_neg"].astype(bool))
        keep = ~r["ref_neg"].astype(bool)
        ref = r["ref"][keep]
        assert np.all(np.abs(r["ll"][keep] - ref) <= 1e-8 + 1e-14 * np.abs(ref))
