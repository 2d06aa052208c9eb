"""Synthetic workloads of the benchmark configurations (seeded, no datasets).

random_circuit: the gate-engine microbenchmark — gates drawn uniformly from
{X, H, CX, MCX with 2-4 controls, U1 with theta ~ U[0, 2pi), Pauli
tensor-product rotation on 2-6 qubits with Paulis uniform over X/Y/Z}, distinct
qubits per gate, and a measure_qbit on a random qubit every 100 gates with r
from the same stream."""
from __future__ import annotations

import math

import numpy as np

KINDS = ("x", "h", "cx", "mcx", "u1", "ptp")


def random_circuit(n: int, ngates: int = 1000, seed: int = 7, measure_every: int = 100):
    rng = np.random.default_rng(seed)
    gates = []
    for g in range(ngates):
        kind = KINDS[int(rng.integers(len(KINDS)))]
        if kind in ("x", "h"):
            gates.append((kind, int(rng.integers(n))))
        elif kind == "cx":
            c, t = (int(q) for q in rng.choice(n, size=2, replace=False))
            gates.append(("cx", c, t))
        elif kind == "mcx":
            k = int(rng.integers(2, 5))
            qs = [int(q) for q in rng.choice(n, size=k + 1, replace=False)]
            gates.append(("mcx", qs[:k], qs[k]))
        elif kind == "u1":
            gates.append(("u1", int(rng.integers(n)), float(rng.uniform(0.0, 2.0 * math.pi))))
        else:
            k = int(rng.integers(2, 7))
            qs = [int(q) for q in rng.choice(n, size=k, replace=False)]
            ps = [int(p) for p in rng.integers(1, 4, size=k)]
            gates.append(("ptp", qs, ps, float(rng.uniform(0.0, 2.0 * math.pi))))
        if measure_every and (g + 1) % measure_every == 0:
            gates.append(("measure", int(rng.integers(n)), float(rng.random())))
    return gates


def random_state(n: int, seed: int = 7, dtype=np.float64):
    """re, im ~ N(0, 1), normalised in FP64; returned as two arrays of dtype."""
    rng = np.random.default_rng(seed)
    N = 1 << n
    re = rng.standard_normal(N)
    im = rng.standard_normal(N)
    nrm = math.sqrt(float(np.dot(re, re)) + float(np.dot(im, im)))
    re /= nrm
    im /= nrm
    return re.astype(dtype, copy=False), im.astype(dtype, copy=False)


def apply_circuit(st, gates):
    """Applies a circuit through the suqa:: mirror; returns the measured bits."""
    bits = []
    for g in gates:
        k = g[0]
        if k == "x":
            st.apply_x(g[1])
        elif k == "h":
            st.apply_h(g[1])
        elif k == "cx":
            st.apply_cx(g[1], g[2])
        elif k == "mcx":
            st.apply_mcx(g[1], g[2])
        elif k == "u1":
            st.apply_u1(g[1], g[2])
        elif k == "ptp":
            st.apply_pauli_rotation(g[1], g[2], g[3])
        elif k == "measure":
            bits.append(st.measure_qbit(g[1], g[2]))
    return bits


def algorithmic_bytes(gates, n: int, bytes_per_amp: int) -> int:
    """Sum over gates of 2 * B * N * f (f = fraction of amplitudes a gate must
    read and write): 1 for X, H and Pauli rotations, 2^-c for c controls, 1/2
    for U1; a measurement counts 2 * B * N (probability read of half, zero-write
    of half, rescale of the kept half)."""
    N = 1 << n
    tot = 0.0
    for g in gates:
        k = g[0]
        if k in ("x", "h", "ptp"):
            f = 1.0
        elif k == "cx":
            f = 0.5
        elif k == "mcx":
            f = 2.0 ** -len(g[1])
        elif k == "u1":
            f = 0.5
        else:  # measure
            f = 1.0
        tot += 2.0 * bytes_per_amp * N * f
    return int(tot)


def fp64_instructions(gates, n: int) -> int:
    """FP64 instructions the tile pass needs for an uncontrolled circuit of the
    benchmark's gate set, per amplitude: H 2 (sum and difference, 1/sqrt2 in the
    global scale), U1 4 on the half it phases, a Pauli rotation 2 (one fused
    multiply-add per component, c or s in the global scale), X/CX/MCX 0, a
    measurement 2 (the squared-magnitude reduction; the collapse is a select)."""
    cost = {"h": 2, "u1": 2, "ptp": 2, "measure": 2}
    return sum(cost.get(g[0], 0) for g in gates) * (1 << n)


def single_kind_circuit(n: int, kind: str, ngates: int = 60, seed: int = 11):
    """H on every qubit, then ngates gates of one kind of the benchmark's set
    (drawn as random_circuit draws them, without measurements): the per-gate
    instruction and time costs of the tile pass are read off such circuits."""
    if kind not in KINDS:
        raise ValueError(f"kind must be one of {KINDS}")
    rng = np.random.default_rng(seed)
    gates = [("h", q) for q in range(n)]
    while len(gates) < n + ngates:
        g = random_circuit(n, 1, seed=int(rng.integers(1 << 31)), measure_every=0)[0]
        if g[0] == kind:
            gates.append(g)
    return gates


def qft_blocks(n: int, pairs: int = 40, seed: int = 3):
    """QFT / inverse-QFT pairs on random 5-qubit registers (the dense-block
    workload): a list of registers, each applied as QFT then inverse QFT."""
    rng = np.random.default_rng(seed)
    return [sorted(int(q) for q in rng.choice(n, size=5, replace=False)) for _ in range(pairs)]


def _main(argv=None):
    """Runs one workload through libsq on the current GPU (the commands the
    committed profiles were captured with):

        python -m suqa_gb300.workloads random --n 24 --gates 300 --precision f64 [--double-float]
        python -m suqa_gb300.workloads qft-blocks --n 24 --pairs 40 --precision f32 --dense-fusion 4
        python -m suqa_gb300.workloads single --gate u1 --n 22 --gates 60 --precision f64 --repeat 1
    """
    import argparse
    from . import State
    ap = argparse.ArgumentParser(prog="python -m suqa_gb300.workloads")
    ap.add_argument("kind", choices=["random", "qft-blocks", "single"])
    ap.add_argument("--gate", default="h", choices=list(KINDS))
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--gates", type=int, default=300)
    ap.add_argument("--pairs", type=int, default=40)
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"])
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--dense-fusion", type=int, default=0)
    ap.add_argument("--double-float", action="store_true")
    ap.add_argument("--staging", type=int, default=None)
    args = ap.parse_args(argv)
    dt = np.float64 if args.precision == "f64" else np.float32
    re, im = random_state(args.n, 7, dt)
    with State(args.n, args.precision) as st:
        st.upload(re.ctypes.data, im.ctypes.data)
        st.set_dense_fusion(args.dense_fusion)
        st.set_double_float(args.double_float)
        if args.staging is not None:
            st.set_staging(args.staging)
        for _ in range(args.repeat):
            if args.kind == "random":
                apply_circuit(st, random_circuit(args.n, args.gates, seed=7))
            elif args.kind == "single":
                apply_circuit(st, single_kind_circuit(args.n, args.gate, args.gates))
            else:
                for r in qft_blocks(args.n, args.pairs):
                    st.apply_qft(r)
                    st.apply_qft_inverse(r[::-1])
        st.synchronize()
        print(st.stats())


if __name__ == "__main__":
    _main()
