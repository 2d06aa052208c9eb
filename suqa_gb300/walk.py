"""Batched Szegedy-walk annealing (QSA) on Ising rings (sq_qsa_walk_batch).

The reference's QSA driver (src/qsa.cu:159-268) anneals one walk on the 3-spin
triangle; this runs thousands of walks on rings of s spins with integer
couplings and no field, every walk with its own PCG32 stream, on the GPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import SQ_F32, SQ_F64, SqQsaWalk, SqQsaWalkResult, check


@dataclass
class QsaWalk:
    """One annealed walk: beta_k = (k+1) beta / stages for k < stages,
    steps_per_stage walk steps at each, a phase_qbits walk-phase register."""
    spins: int
    J: list
    beta: float = 1.0
    stages: int = 50
    steps_per_stage: int = 20
    phase_qbits: int = 6
    seed: int = 1
    max_steps: int = 0
    algo: int = 0  # 0: iterate W per orbit; 1: per orbit class; 2: 1 prepared per step (see sq_qsa_walk)

    @property
    def cap(self) -> int:
        return self.max_steps or 8 * self.stages * self.steps_per_stage


@dataclass
class QsaWalkRun:
    done: bool
    restarts: int
    steps: int
    readout: int
    E: float
    absM: float
    last_p0: float
    p0: np.ndarray = field(default_factory=lambda: np.zeros(0))


def _precision(p):
    return SQ_F64 if p in ("f64", "fp64") else SQ_F32


def run_qsa_walks(walks: list[QsaWalk], precision: str = "f32", trace: bool = False):
    """Runs all walks; returns ([QsaWalkRun], device milliseconds)."""
    L = _lib.load()
    n = len(walks)
    arr = (SqQsaWalk * n)()
    for i, w in enumerate(walks):
        J = list(w.J) + [0] * (12 - len(w.J))
        arr[i] = SqQsaWalk(w.spins, w.phase_qbits, w.stages, w.steps_per_stage, w.max_steps,
                           (C.c_int32 * 12)(*J), w.algo, w.beta, w.seed)
    res = (SqQsaWalkResult * n)()
    caps = [w.cap for w in walks]
    tr = np.zeros(sum(caps) if trace else 0, dtype=np.float64)
    ms = C.c_float()
    check(L.sq_qsa_walk_batch(arr, n, _precision(precision), res,
                              tr.ctypes.data_as(C.c_void_p) if trace else None, C.byref(ms)))
    out = []
    off = 0
    for i, w in enumerate(walks):
        r = res[i]
        p0 = tr[off:off + r.steps].copy() if trace else np.zeros(0)
        off += caps[i]
        out.append(QsaWalkRun(bool(r.done), r.restarts, r.steps, r.readout, r.E, r.absM, r.last_p0, p0))
    return out, ms.value


def ising_ring_walks(n: int, spins: int = 10, beta: float = 1.0, stages: int = 50, steps_per_stage: int = 20,
                     phase_qbits: int = 6, seed: int = 2025, max_steps: int = 0, algo: int = 0) -> list[QsaWalk]:
    """n walks on periodic Ising rings with couplings +-1 drawn uniformly and no
    field; walk k has seed seed + k and its own couplings."""
    rng = np.random.default_rng(seed)
    return [QsaWalk(spins, [int(v) for v in rng.choice([-1, 1], spins)], beta, stages, steps_per_stage,
                    phase_qbits, seed + k, max_steps, algo) for k in range(n)]


def summarize(runs: list[QsaWalkRun]) -> dict:
    """<E> and <|M|> (standard errors, walks independent) over the completed walks."""
    done = [r for r in runs if r.done]
    out = {"walks": len(runs), "completed": len(done), "restarts": int(sum(r.restarts for r in runs)),
           "steps": int(sum(r.steps for r in runs))}
    if done:
        E = np.array([r.E for r in done])
        M = np.array([r.absM for r in done])
        k = len(done)
        out.update({"E": float(E.mean()), "E_err": float(E.std(ddof=1) / np.sqrt(k)) if k > 1 else 0.0,
                    "absM": float(M.mean()), "absM_err": float(M.std(ddof=1) / np.sqrt(k)) if k > 1 else 0.0})
    return out


def config4_study(n_walks: int = 1024, f64_walks: int = 64, spins: int = 10, stages: int = 50,
                  steps_per_stage: int = 20, phase_qbits: int = 6, seed: int = 2025, algo: int = 1):
    """1024 annealed walks on 10-spin rings (J = +-1, h = 0), beta 0 -> 1 over
    50 stages x 20 walk steps, 6-qubit walk-phase register, in FP32; the first
    f64_walks of them again in FP64, walk by walk."""
    walks = ising_ring_walks(n_walks, spins, 1.0, stages, steps_per_stage, phase_qbits, seed, algo=algo)
    r32, ms32 = run_qsa_walks(walks, "f32")
    out = {"config": f"{n_walks} walks, {spins}-spin Ising rings J=+-1 h=0, beta 0->1 over {stages} stages x "
                     f"{steps_per_stage} walk steps, {phase_qbits}-qubit walk-phase register, algorithm {algo}",
           "f32": summarize(r32), "f32_device_s": ms32 / 1e3,
           "f32_walk_steps_per_s": sum(r.steps for r in r32) / (ms32 / 1e3)}
    if f64_walks:
        sub = walks[:f64_walks]
        r64, ms64 = run_qsa_walks(sub, "f64")
        same = sum(1 for a, b in zip(r32[:f64_walks], r64)
                   if (a.done, a.restarts, a.steps, a.readout) == (b.done, b.restarts, b.steps, b.readout))
        out.update({"f64": summarize(r64), "f32_same_walks": summarize(r32[:f64_walks]),
                    "f64_device_s": ms64 / 1e3, "f64_walk_steps_per_s": sum(r.steps for r in r64) / (ms64 / 1e3),
                    "identical_walks": same, "compared_walks": f64_walks})
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="Batched Szegedy-walk annealing on Ising rings")
    ap.add_argument("--walks", type=int, default=1024)
    ap.add_argument("--f64-walks", type=int, default=64)
    ap.add_argument("--stages", type=int, default=50)
    ap.add_argument("--steps-per-stage", type=int, default=20)
    ap.add_argument("--algo", type=int, default=1, help="0: iterate W per orbit; 1: per orbit class; 2: classes prepared per step")
    a = ap.parse_args()
    print(json.dumps(config4_study(a.walks, a.f64_walks, stages=a.stages, steps_per_stage=a.steps_per_stage,
                                   algo=a.algo)))
