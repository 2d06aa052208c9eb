"""Batched quantum Metropolis sampling of transverse-field Ising rings on the GPU
(libsq sq_qms_tfim_batch / sq_batch_*): thousands of independent chains, one
PCG32 stream each, run in persistent kernels; a Batch can be advanced in
segments (replayed from a captured CUDA graph), checkpointed and resumed."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import SQ_F32, SQ_F64, SqBatchClass, SqBatchOpts, SqChainResult, SqTfimChain, SqTfimEvolution, check


@dataclass
class TfimChain:
    spins: int
    ene_qbits: int
    steps: int
    beta: float
    h: float
    J: float = 1.0
    ene_min: float | None = None
    ene_max: float | None = None
    thermalization: int = 20
    reset_each: int = 1
    max_reverse: int = 100
    dt: float = 0.1
    seed: int = 1
    warm_angles: list | None = None  # per-spin RY angles of a learned warm start

    def window(self):
        """Phase-estimation window; by default +-s(|J|+|h|), a bound of the spectrum."""
        b = self.spins * (abs(self.J) + abs(self.h))
        lo = -b if self.ene_min is None else self.ene_min
        hi = b if self.ene_max is None else self.ene_max
        return lo, hi

    @property
    def nqubits(self):
        return self.spins + self.ene_qbits + 1


@dataclass
class ChainRun:
    accepted: int
    failures: int
    E: np.ndarray
    A: np.ndarray
    step: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))
    phase_estimations: int = 0
    cycles: int = 0
    evolution_cycles: int = 0

    def reference_rows(self, steps: int):
        """Rows the reference qms driver would have written to its output file: it
        appends the samples at steps s with s % ceil(steps/20) == 0, so samples
        after the last such step are never written (src/qms.cu:145-148)."""
        every = (steps + 19) // 20
        last = ((steps - 1) // every) * every
        keep = self.step <= last
        return self.E[keep], self.A[keep]


def _chain_array(chains):
    n = len(chains)
    arr = (SqTfimChain * n)()
    for i, c in enumerate(chains):
        lo, hi = c.window()
        arr[i] = SqTfimChain(c.spins, c.ene_qbits, c.steps, c.thermalization, c.reset_each, c.max_reverse,
                             c.J, c.h, c.beta, lo, hi, c.dt, c.seed)
        if c.warm_angles is not None:
            arr[i].warm_start = 1
            for k, a in enumerate(c.warm_angles[:20]):
                arr[i].ry[k] = float(a)
    return arr


def _precision(p):
    return SQ_F64 if p in ("f64", "fp64") else SQ_F32


def _split_runs(chains, res, E, A, S):
    out = []
    off = 0
    for i, c in enumerate(chains):
        k = res[i].samples
        out.append(ChainRun(res[i].accepted, res[i].failures, E[off:off + k].copy(), A[off:off + k].copy(),
                            S[off:off + k].copy(), res[i].phase_estimations, res[i].cycles,
                            res[i].evolution_cycles))
        off += c.steps
    return out


def run_tfim_batch(chains: list[TfimChain], precision: str = "f32", stream: int | None = None):
    """Runs all chains; returns ([ChainRun], device milliseconds)."""
    L = _lib.load()
    n = len(chains)
    arr = _chain_array(chains)
    res = (SqChainResult * n)()
    total = sum(c.steps for c in chains)
    E = np.zeros(max(total, 1), dtype=np.float64)
    A = np.zeros(max(total, 1), dtype=np.float64)
    S = np.zeros(max(total, 1), dtype=np.uint32)
    ms = C.c_float()
    check(L.sq_qms_tfim_batch(arr, n, _precision(precision), res, E.ctypes.data_as(C.c_void_p),
                              A.ctypes.data_as(C.c_void_p), S.ctypes.data_as(C.c_void_p),
                              C.c_void_p(stream) if stream else None, C.byref(ms)))
    return _split_runs(chains, res, E, A, S), ms.value


MODES = {0: "shared", 1: "cluster-shared", 2: "cluster-global"}


class Batch:
    """A resumable batch of chains (sq_batch_*).

    segment_steps / use_graph: run() advances in segments of that many steps,
    replaying one captured CUDA graph per segment; autotune: time the CTA sizes
    per chain-width class on a sample of its chains and keep the fastest."""

    def __init__(self, chains: list[TfimChain], precision: str = "f32", segment_steps: int = 0,
                 use_graph: bool = False, autotune: bool = False, threads: int = 0, l2_budget_bytes: int = 0,
                 cta_qubits: int = 0, global_qubits: int = 0):
        self._L = _lib.load()
        self.chains = list(chains)
        self._arr = _chain_array(self.chains)
        opts = SqBatchOpts(segment_steps, 1 if use_graph else 0, 1 if autotune else 0, threads, l2_budget_bytes,
                           cta_qubits, global_qubits)
        h = C.c_void_p()
        check(self._L.sq_batch_create(C.byref(h), self._arr, len(self.chains), _precision(precision), C.byref(opts)))
        self._h = h

    def close(self):
        if self._h:
            self._L.sq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, steps: int) -> float:
        """Advance every unfinished chain by up to `steps` steps; returns device ms."""
        ms = C.c_float()
        check(self._L.sq_batch_run(self._h, steps, C.byref(ms)))
        return ms.value

    def results(self):
        n = len(self.chains)
        res = (SqChainResult * n)()
        total = max(sum(c.steps for c in self.chains), 1)
        E = np.zeros(total, dtype=np.float64)
        A = np.zeros(total, dtype=np.float64)
        S = np.zeros(total, dtype=np.uint32)
        check(self._L.sq_batch_results(self._h, res, E.ctypes.data_as(C.c_void_p), A.ctypes.data_as(C.c_void_p),
                                       S.ctypes.data_as(C.c_void_p)))
        return _split_runs(self.chains, res, E, A, S)

    def progress(self) -> np.ndarray:
        out = np.zeros(len(self.chains), dtype=np.uint32)
        check(self._L.sq_batch_progress(self._h, out.ctypes.data_as(C.c_void_p)))
        return out

    def state(self, chain: int) -> np.ndarray:
        N = 1 << self.chains[chain].nqubits
        re = np.zeros(N, dtype=np.float64)
        im = np.zeros(N, dtype=np.float64)
        check(self._L.sq_batch_state(self._h, chain, re.ctypes.data_as(C.c_void_p), im.ctypes.data_as(C.c_void_p)))
        return re + 1j * im

    def checkpoint(self) -> bytes:
        size = C.c_uint64()
        check(self._L.sq_batch_checkpoint_size(self._h, C.byref(size)))
        buf = (C.c_char * size.value)()
        check(self._L.sq_batch_checkpoint(self._h, buf, size.value))
        return bytes(buf)

    def restore(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        check(self._L.sq_batch_restore(self._h, buf, len(blob)))

    def plan(self) -> list[dict]:
        cnt = C.c_uint32()
        check(self._L.sq_batch_plan(self._h, None, 0, C.byref(cnt)))
        info = (SqBatchClass * max(cnt.value, 1))()
        check(self._L.sq_batch_plan(self._h, info, cnt.value, C.byref(cnt)))
        return [{"n": c.n, "chains": c.count, "mode": MODES.get(c.mode, c.mode), "cluster": c.cluster,
                 "threads": c.threads, "grid": c.grid, "smem_bytes": c.smem_bytes,
                 "probe_ms": round(float(c.probe_ms), 3)} for c in info[:cnt.value]]


@dataclass
class TfimEvolution:
    """A ring evolved by `steps` Trotter steps of width dt (see sq_tfim_evolve_batch)."""
    spins: int
    steps: int
    dt: float
    h: float
    J: float = 1.0
    warm_angles: list | None = None


def run_tfim_evolution(jobs: list[TfimEvolution], precision: str = "f64"):
    """Returns ([array (steps+1, 2^spins) of probabilities per job], device ms)."""
    L = _lib.load()
    n = len(jobs)
    arr = (SqTfimEvolution * n)()
    total = 0
    for i, j in enumerate(jobs):
        arr[i] = SqTfimEvolution(j.spins, j.steps, j.J, j.h, j.dt)
        if j.warm_angles is not None:
            arr[i].warm_start = 1
            for k, a in enumerate(j.warm_angles[:20]):
                arr[i].ry[k] = float(a)
        total += (j.steps + 1) << j.spins
    out = np.zeros(total, dtype=np.float64)
    ms = C.c_float()
    check(L.sq_tfim_evolve_batch(arr, n, _precision(precision), out.ctypes.data_as(C.c_void_p), C.byref(ms)))
    res, off = [], 0
    for j in jobs:
        k = (j.steps + 1) << j.spins
        res.append(out[off:off + k].reshape(j.steps + 1, 1 << j.spins).copy())
        off += k
    return res, ms.value


def tfim_config3(n_chains: int = 4096, steps: int = 500, seed: int = 2024):
    """The 4096-chain TFIM workload: spins ~ U{4..10}, energy register ~ U{4..6}
    qubits, J = 1, h ~ U[0.5, 1.5], beta ~ U[0.2, 2.0], dt = 0.1, window
    +-s(|J|+|h|), chain k seeded base + k."""
    rng = np.random.default_rng(seed)
    return [TfimChain(spins=int(rng.integers(4, 11)), ene_qbits=int(rng.integers(4, 7)), steps=steps,
                      beta=float(rng.uniform(0.2, 2.0)), h=float(rng.uniform(0.5, 1.5)), thermalization=20,
                      seed=1 + i) for i in range(n_chains)]


def config3_study(n_chains=4096, steps=500, segment=50, f64_chains=128):
    """Runs the full workload in FP32 as one resumable batch (graph-replayed
    segments, checkpointed half-way and resumed in a fresh batch), then the
    first f64_chains chains in FP64, and compares their trajectories; returns
    the throughput and per-ring-length energies."""
    import time
    from . import shard
    chains = tfim_config3(n_chains, steps)
    out = {"chains": n_chains, "steps": steps}
    t0 = time.perf_counter()
    b = Batch(chains, "f32", segment_steps=segment, use_graph=True, autotune=True)
    out["f32_setup_s"] = time.perf_counter() - t0
    ms1 = b.run(steps // 2)
    blob = b.checkpoint()
    b.close()
    b = Batch(chains, "f32", segment_steps=segment, use_graph=True, autotune=True)
    b.restore(blob)
    ms2 = b.run(steps - steps // 2)
    r32 = b.results()
    b.close()
    out["f32_device_s"] = (ms1 + ms2) / 1e3
    out["f32_chain_steps_per_s"] = n_chains * steps / ((ms1 + ms2) / 1e3)
    out["checkpoint_bytes"] = len(blob)
    keys, acc = shard.group_sums(chains, r32, lambda c: c.spins)
    out["f32_energy_by_ring_length"] = shard.averages(keys, acc)
    sub = chains[:f64_chains]
    b = Batch(sub, "f64", segment_steps=segment, use_graph=True)
    ms = b.run(steps)
    r64 = b.results()
    b.close()
    out["f64_chains"] = f64_chains
    out["f64_chain_steps_per_s"] = f64_chains * steps / (ms / 1e3)
    out["f64_trajectories_identical_to_f32"] = int(sum(
        1 for a, c in zip(r32[:f64_chains], r64)
        if a.accepted == c.accepted and np.array_equal(a.E, c.E) and np.array_equal(a.A, c.A)))
    return out


def evolution_study(n_rings=2048, steps=50, seed=3):
    """Throughput of the batched evolution: rings of 8-12 spins (h ~ U[0.5, 1.5],
    dt = 0.1) evolved `steps` Trotter steps with every step's probabilities
    recorded, in FP32 and FP64."""
    rng = np.random.default_rng(seed)
    jobs = [TfimEvolution(spins=int(rng.integers(8, 13)), steps=steps, dt=0.1, h=float(rng.uniform(0.5, 1.5)))
            for _ in range(n_rings)]
    out = {"rings": n_rings, "steps": steps, "spins": "8-12"}
    for prec in ("f32", "f64"):
        rows, ms = run_tfim_evolution(jobs, prec)
        amps = sum((1 << j.spins) * j.steps for j in jobs)
        out[prec] = {"device_ms": ms, "ring_steps_per_s": n_rings * steps / (ms / 1e3),
                     "amplitude_steps_per_s": amps / (ms / 1e3),
                     "probability_bytes": int(sum(r.nbytes for r in rows))}
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="batched-chain studies")
    ap.add_argument("--evolution", action="store_true", help="time the batched evolution instead")
    a = ap.parse_args()
    print(json.dumps(evolution_study() if a.evolution else config3_study()))
