"""Batched quantum Metropolis sampling of transverse-field Ising rings on the GPU
(libsq sq_qms_tfim_batch): thousands of independent chains, one PCG32 stream
each, run to completion in persistent kernels."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import SQ_F32, SQ_F64, SqChainResult, SqTfimChain, check


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

    def reference_rows(self, steps: int):
        """Rows the reference qms driver would have written to its output file: it
        appends the samples at steps s with s % ceil(steps/20) == 0, so samples
        after the last such step are never written (src/qms.cu:145-148)."""
        every = (steps + 19) // 20
        last = ((steps - 1) // every) * every
        keep = self.step <= last
        return self.E[keep], self.A[keep]


def run_tfim_batch(chains: list[TfimChain], precision: str = "f32", stream: int | None = None):
    """Runs all chains; returns ([ChainRun], device milliseconds)."""
    L = _lib.load()
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
    res = (SqChainResult * n)()
    total = sum(c.steps for c in chains)
    E = np.zeros(max(total, 1), dtype=np.float64)
    A = np.zeros(max(total, 1), dtype=np.float64)
    S = np.zeros(max(total, 1), dtype=np.uint32)
    ms = C.c_float()
    prec = SQ_F64 if precision in ("f64", "fp64") else SQ_F32
    check(L.sq_qms_tfim_batch(arr, n, prec, res, E.ctypes.data_as(C.c_void_p), A.ctypes.data_as(C.c_void_p),
                              S.ctypes.data_as(C.c_void_p), C.c_void_p(stream) if stream else None, C.byref(ms)))
    out = []
    off = 0
    for i, c in enumerate(chains):
        k = res[i].samples
        out.append(ChainRun(res[i].accepted, res[i].failures, E[off:off + k].copy(), A[off:off + k].copy(),
                            S[off:off + k].copy(), res[i].phase_estimations, res[i].cycles))
        off += c.steps
    return out, ms.value
