"""Sharding of chain batches over ranks: the split and the FP64 reduction of
per-group sums, run as world_size-2 gloo process groups on the CPU (no GPU).
The chain results are synthetic stand-ins (ChainRun with seeded samples), so
this covers the host logic only; the per-rank Batch runs on one GPU each."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from suqa_gb300.batch import ChainRun, TfimChain
from suqa_gb300 import shard


def _chains(n=37):
    rng = np.random.default_rng(4)
    return [TfimChain(spins=int(rng.integers(4, 11)), ene_qbits=int(rng.integers(4, 7)),
                      steps=int(rng.integers(5, 40)), beta=1.0, h=1.0, seed=i) for i in range(n)]


def _runs(chains):
    out = []
    for i, c in enumerate(chains):
        r = np.random.default_rng(100 + i)
        k = c.steps // 2
        out.append(ChainRun(0, 0, r.normal(-3, 1, k), r.normal(0, 2, k), np.arange(k, dtype=np.uint32)))
    return out


def test_partition_is_a_balanced_split():
    ch = _chains()
    for world in (1, 2, 3, 4):
        parts = shard.partition(ch, world)
        assert sorted(i for p in parts for i in p) == list(range(len(ch)))
        loads = [sum(shard.chain_cost(ch[i]) for i in p) for p in parts]
        biggest = max(shard.chain_cost(c) for c in ch)
        assert max(loads) - min(loads) <= biggest  # LPT bound
    assert shard.partition(ch, 2) == shard.partition(list(ch), 2)  # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ch = _chains()
    runs = _runs(ch)
    mine = shard.partition(ch, world)[rank]
    keys = sorted({c.spins for c in ch})
    acc = np.zeros((len(keys), len(shard.FIELDS)))
    k2, a2 = shard.group_sums([ch[i] for i in mine], [runs[i] for i in mine], lambda c: c.spins)
    pos = {k: i for i, k in enumerate(keys)}
    for k, row in zip(k2, a2):
        acc[pos[k]] += row
    tot = shard.reduce_sums(acc)
    q.put((rank, keys, tot))
    dist.destroy_process_group()


def test_two_rank_reduction_equals_one_rank():
    ch = _chains()
    keys1, acc1 = shard.group_sums(ch, _runs(ch), lambda c: c.spins)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, keys, tot in got:
        assert keys == keys1
        assert np.allclose(tot, acc1, rtol=1e-13, atol=1e-9)
    av = shard.averages(keys1, acc1)
    assert sum(v["samples"] for v in av.values()) == sum(len(r.E) for r in _runs(ch))


def _walks(n=29):
    from suqa_gb300.walk import QsaWalk
    rng = np.random.default_rng(6)
    return [QsaWalk(int(rng.integers(3, 11)), [1] * 12, 1.0, int(rng.integers(2, 9)), 5, 6, seed=i)
            for i in range(n)]


def _walk_runs(walks):
    from suqa_gb300.walk import QsaWalkRun
    out = []
    for i, w in enumerate(walks):
        r = np.random.default_rng(300 + i)
        out.append(QsaWalkRun(bool(i % 5), 0, w.cap, 0, float(r.integers(-10, 11)), float(r.integers(0, 11)), 1.0))
    return out


def test_walk_partition_balances_state_size_times_steps():
    ws = _walks()
    for world in (2, 3):
        parts = shard.partition(ws, world, shard.walk_cost)
        assert sorted(i for p in parts for i in p) == list(range(len(ws)))
        loads = [sum(shard.walk_cost(ws[i]) for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(shard.walk_cost(w) for w in ws)


def _walk_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws = _walks()
    runs = _walk_runs(ws)
    mine = shard.partition(ws, world, shard.walk_cost)[rank]
    keys = sorted({w.spins for w in ws})
    acc = np.zeros((len(keys), len(shard.FIELDS)))
    k2, a2 = shard.walk_sums([ws[i] for i in mine], [runs[i] for i in mine], lambda w: w.spins)
    pos = {k: i for i, k in enumerate(keys)}
    for k, row in zip(k2, a2):
        acc[pos[k]] += row
    q.put((rank, keys, shard.reduce_sums(acc)))
    dist.destroy_process_group()


def test_two_rank_walk_reduction_equals_one_rank():
    ws = _walks()
    keys1, acc1 = shard.walk_sums(ws, _walk_runs(ws), lambda w: w.spins)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_walk_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for rank, keys, tot in got:
        assert keys == keys1
        assert np.allclose(tot, acc1, rtol=0, atol=1e-9)
    assert acc1[:, 0].sum() == sum(1 for i in range(len(ws)) if i % 5)
