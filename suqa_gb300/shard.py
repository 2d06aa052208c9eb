"""Sharding a chain batch over ranks (one GPU per rank).

Chains (and annealed walks) are independent, so a batch splits by id with no
exchange while it runs; the only collective is one final FP64 reduction of the
per-group sums {count, sum E, sum E^2, sum A, sum A^2} (A = |M| for walks).  Ranks are balanced by the
estimated cost of their chains: steps x 2^n amplitudes per chain (the state
size sets the cost of every sweep).  torch.distributed carries the reduction
(gloo on CPU, nccl on GPUs); without an initialised process group everything
runs as one rank.
"""
from __future__ import annotations

import numpy as np

FIELDS = ("count", "sum_E", "sum_E2", "sum_A", "sum_A2")


def chain_cost(c) -> float:
    return float(c.steps) * float(1 << c.nqubits)


def walk_cost(w) -> float:
    """Annealed Szegedy walk: its step cap x 2^(2s+1) amplitudes per step."""
    return float(w.cap) * float(1 << (2 * w.spins + 1))


def partition(chains, world: int, cost=chain_cost) -> list[list[int]]:
    """Item indices per rank: longest-processing-time-first greedy on `cost`,
    ties broken by index, so every rank computes the same split."""
    order = sorted(range(len(chains)), key=lambda i: (-cost(chains[i]), i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += cost(chains[i])
    return [sorted(p) for p in parts]


def group_sums(chains, runs, key) -> tuple[list, np.ndarray]:
    """Per-group FP64 sums over the samples of `runs` (ChainRun per chain);
    key(chain) names the group.  Returns (sorted group keys, array [groups, 5])."""
    keys = sorted({key(c) for c in chains})
    pos = {k: i for i, k in enumerate(keys)}
    acc = np.zeros((len(keys), len(FIELDS)), dtype=np.float64)
    for c, r in zip(chains, runs):
        g = pos[key(c)]
        E = np.asarray(r.E, dtype=np.float64)
        A = np.asarray(r.A, dtype=np.float64)
        acc[g] += (len(E), E.sum(), (E * E).sum(), A.sum(), (A * A).sum())
    return keys, acc


def walk_sums(walks, runs, key) -> tuple[list, np.ndarray]:
    """Per-group FP64 sums over completed walks (one readout each): the fields of
    FIELDS with A = |M|."""
    keys = sorted({key(w) for w in walks})
    pos = {k: i for i, k in enumerate(keys)}
    acc = np.zeros((len(keys), len(FIELDS)), dtype=np.float64)
    for w, r in zip(walks, runs):
        if r.done:
            acc[pos[key(w)]] += (1.0, r.E, r.E * r.E, r.absM, r.absM * r.absM)
    return keys, acc


def reduce_sums(acc: np.ndarray) -> np.ndarray:
    """Sum the per-group sums over all ranks (FP64 all-reduce)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return acc
    backend = dist.get_backend()
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.from_numpy(np.ascontiguousarray(acc)).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def averages(keys, acc: np.ndarray) -> dict:
    """<E>, <A> and their standard errors (samples treated as independent) per group."""
    out = {}
    for k, (n, se, se2, sa, sa2) in zip(keys, acc):
        if n == 0:
            continue
        mE, mA = se / n, sa / n
        vE, vA = max(se2 / n - mE * mE, 0.0), max(sa2 / n - mA * mA, 0.0)
        out[k] = {"samples": int(n), "E": mE, "E_err": (vE / n) ** 0.5, "A": mA, "A_err": (vA / n) ** 0.5}
    return out


def run_sharded(chains, precision: str = "f32", key=lambda c: c.spins, rank: int | None = None,
                world: int | None = None, **batch_opts):
    """Runs this rank's share of `chains` as one Batch on the current GPU and
    returns the all-rank per-group averages (identical on every rank)."""
    import torch.distributed as dist
    from .batch import Batch
    if rank is None or world is None:
        init = dist.is_available() and dist.is_initialized()
        rank = dist.get_rank() if init else 0
        world = dist.get_world_size() if init else 1
    mine = partition(chains, world)[rank]
    sub = [chains[i] for i in mine]
    keys = sorted({key(c) for c in chains})
    acc = np.zeros((len(keys), len(FIELDS)), dtype=np.float64)
    if sub:
        b = Batch(sub, precision, **batch_opts)
        b.run(max(c.steps for c in sub))
        k2, a2 = group_sums(sub, b.results(), key)
        b.close()
        pos = {k: i for i, k in enumerate(keys)}
        for k, row in zip(k2, a2):
            acc[pos[k]] += row
    return averages(keys, reduce_sums(acc))


def run_sharded_walks(walks, precision: str = "f32", key=lambda w: w.spins, rank: int | None = None,
                      world: int | None = None):
    """Runs this rank's share of the annealed walks on the current GPU and
    returns the all-rank per-group <E>, <|M|> (identical on every rank)."""
    import torch.distributed as dist
    from .walk import run_qsa_walks
    if rank is None or world is None:
        init = dist.is_available() and dist.is_initialized()
        rank = dist.get_rank() if init else 0
        world = dist.get_world_size() if init else 1
    mine = partition(walks, world, walk_cost)[rank]
    keys = sorted({key(w) for w in walks})
    acc = np.zeros((len(keys), len(FIELDS)), dtype=np.float64)
    if mine:
        sub = [walks[i] for i in mine]
        runs, _ = run_qsa_walks(sub, precision)
        k2, a2 = walk_sums(sub, runs, key)
        pos = {k: i for i, k in enumerate(keys)}
        for k, row in zip(k2, a2):
            acc[pos[k]] += row
    return averages(keys, reduce_sums(acc))
