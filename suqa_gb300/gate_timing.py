"""Per-gate pass timing: every gate type applied alone (fusion off) as one pass
over an n-qubit state, timed with the engine's per-launch CUDA events, plus the
fused random circuit of the benchmark.

    python -m suqa_gb300.gate_timing [n] [precision]

Prints one JSON object: per case (ms per pass, launches, bytes per launch, GB/s).
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


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 28
    prec = sys.argv[2] if len(sys.argv) > 2 else "f64"
    print(json.dumps({"n": n, "precision": prec, "passes": run(n, prec)}))
