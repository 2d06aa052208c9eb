"""Per-gate pass timing: every gate type applied alone (fusion off) as one pass
over an n-qubit state, timed with the engine's per-launch CUDA events, plus the
fused random circuit of the benchmark.

    python -m suqa_gb300.gate_timing [n] [precision]
    python -m suqa_gb300.gate_timing --kind h|u1|ptp|x|cx|mcx [n] [precision]

Prints one JSON object: per case (ms per pass, launches, bytes per launch, GB/s).
The --kind form applies H to every qubit, then 60 gates of one type drawn by the
benchmark's generator (fusion on): the workload for counting the floating-point
instructions of one gate type under a profiler.
"""
from __future__ import annotations

import json
import sys

from .state import State
from .workloads import apply_circuit, random_circuit


def _time(st, fn, reps=10):
    st.flush()
    st.synchronize()
    st.set_timing(True)
    st.kernel_time()
    for _ in range(reps):
        fn()
    ms, nl, by = st.kernel_time()
    st.set_timing(False)
    nl = max(nl, 1)
    return {"ms_per_pass": ms / nl, "launches": nl, "bytes_per_launch": by / nl, "gbs": by / (ms / 1e3) / 1e9}


def run(n: int = 28, precision: str = "f64"):
    st = State(n, precision)
    st.set_fusion(False)
    st.apply_h(list(range(n)))
    out = {
        "x0": _time(st, lambda: st.apply_x(0)),
        f"x{n - 1}": _time(st, lambda: st.apply_x(n - 1)),
        "h3": _time(st, lambda: st.apply_h(3)),
        "h20": _time(st, lambda: st.apply_h(min(20, n - 1))),
        "u1": _time(st, lambda: st.apply_u1(5, 0.3)),
        "cx": _time(st, lambda: st.apply_cx(2, min(17, n - 1))),
        "mcx3": _time(st, lambda: st.apply_mcx([1, 9, min(22, n - 2)], min(14, n - 1))),
        "pauli3": _time(st, lambda: st.apply_pauli_rotation([2, 11, min(25, n - 1)], [1, 2, 3], 0.4)),
        "pauli6": _time(st, lambda: st.apply_pauli_rotation([0, 4, 9, 13, min(21, n - 2), min(26, n - 1)],
                                                            [1, 2, 3, 1, 2, 3], 0.4)),
        "measure": _time(st, lambda: st.measure_qbit(7, 0.5), reps=5),
    }
    st.set_fusion(True)
    gates = random_circuit(n, 1000, seed=7)
    apply_circuit(st, gates)
    out["fused_circuit_pass"] = _time(st, lambda: apply_circuit(st, gates), reps=1)
    st.close()
    return out


def single_kind(kind: str, n: int = 22, precision: str = "f64", count: int = 60):
    gates = [g for g in random_circuit(n, 10 * count, seed=3, measure_every=0) if g[0] == kind][:count]
    st = State(n, precision)
    st.apply_h(list(range(n)))
    st.flush()
    apply_circuit(st, gates)
    st.flush()
    st.synchronize()
    out = {"kind": kind, "gates": len(gates), "stats": st.stats()}
    st.close()
    return out


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] == "--kind":
        kind = args[1]
        n = int(args[2]) if len(args) > 2 else 22
        prec = args[3] if len(args) > 3 else "f64"
        print(json.dumps({"n": n, "precision": prec, **single_kind(kind, n, prec)}))
    else:
        n = int(args[0]) if args else 28
        prec = args[1] if len(args) > 1 else "f64"
        print(json.dumps({"n": n, "precision": prec, "passes": run(n, prec)}))
