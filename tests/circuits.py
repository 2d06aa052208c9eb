"""Seeded random gate scripts in the dumper grammar (oracle/ref_dump.cpp), shared by
the parity tests and the golden-fixture generator."""
from __future__ import annotations

import math

import numpy as np

PAULI_X, PAULI_Y, PAULI_Z = 1, 2, 3


def hx(v: float) -> str:
    return float(v).hex()


def random_state_line(rng: np.random.Generator, n: int):
    N = 1 << n
    a = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    a /= np.linalg.norm(a)
    return ["setstate", " ".join(hx(v) for v in np.concatenate([a.real, a.imag]))]


def _ref_supported_ptp(ps):
    if len(ps) in (1, 2):
        return True
    if len(ps) == 3:
        s = sorted(ps)
        return s[2] == PAULI_Z and s[0] == s[1]
    return False


def random_script(seed: int, n: int, ngates: int, *, reference_only: bool = True,
                  with_gc: bool = True, measure_every: int = 7, random_init: bool = True,
                  dump_every: int = 5, overlap: str = "none"):
    """A script over n qubits.  reference_only keeps to the gate patterns the
    reference supports (its CPU build throws on other Pauli strings and has no
    phase-list symbol).  overlap="all" lets gate qubits fall inside the global
    control mask (the reference then follows its loops' aliasing semantics);
    overlap="engine" restricts that to the patterns libsq reproduces."""
    rng = np.random.default_rng(seed)
    lines = [f"setup {n}"]
    if random_init:
        lines += random_state_line(rng, n)
    else:
        # a layer of Hadamards and phases so the state is dense from the start
        for q in range(n):
            lines += [f"h {q}", f"u1 {q} {hx(rng.uniform(-math.pi, math.pi))}"]
    gc_on = []
    kinds = ["x", "y", "z", "h", "s", "t", "tdg", "u1", "u1m", "cx", "mcx", "mcxm", "cu1",
             "mcu1", "mcu1m", "swap", "ptp", "qft", "iqft"]
    if not reference_only:
        kinds += ["ptpg", "plist"]
    for g in range(ngates):
        # occasionally toggle a global control
        if with_gc and n >= 3 and rng.random() < 0.08:
            if gc_on:
                lines.append(f"gc_off {len(gc_on)} " + " ".join(map(str, gc_on)))
                gc_on = []
            else:
                k = int(rng.integers(1, 3))
                gc_on = [int(q) for q in rng.choice(n, size=k, replace=False)]
                lines.append(f"gc_on {len(gc_on)} " + " ".join(map(str, gc_on)))
        free = [q for q in range(n) if q not in gc_on]
        if len(free) < 2:
            continue
        kind = kinds[int(rng.integers(len(kinds)))]
        if overlap != "none" and gc_on and rng.random() < 0.5:
            # a gate acting on a qubit of the global control mask
            q0 = int(rng.choice(gc_on))
            other = int(rng.choice(free))
            ph = hx(rng.uniform(-2 * math.pi, 2 * math.pi))
            opts = ["x", "y", "h", "u1", "cx", "swap", "ptp1", "xx"]
            if overlap == "all":
                opts += ["ptp2"]
            k = opts[int(rng.integers(len(opts)))]
            if k in ("x", "y", "h"):
                lines.append(f"{k} {q0}")
            elif k == "u1":
                lines.append(f"u1m {q0} {int(rng.integers(2))} {ph}")
            elif k == "cx":
                lines.append(f"cx {other} {q0} 1")
            elif k == "swap":
                lines.append(f"swap {q0} {other}" if rng.random() < 0.5 else f"swap {other} {q0}")
            elif k == "ptp1":
                pz = int(rng.integers(1, 4)) if overlap == "all" else [1, 3][int(rng.integers(2))]
                lines.append(f"ptp 1 {q0} {pz} {ph}")
            elif k == "xx":
                pair = [q0, other] if rng.random() < 0.5 else [other, q0]
                if len(gc_on) > 1 and rng.random() < 0.3:
                    pair = list(gc_on[:2])
                lines.append(f"ptp 2 {pair[0]} {pair[1]} 1 1 {ph}")
            else:
                lines.append(f"ptp 2 {q0} {other} {int(rng.integers(1, 4))} {int(rng.integers(1, 4))} {ph}")
            continue
        ph = hx(rng.uniform(-2 * math.pi, 2 * math.pi))
        pick = lambda k: [int(q) for q in rng.choice(free, size=k, replace=False)]
        if kind in ("x", "y", "z", "h", "s", "t", "tdg"):
            lines.append(f"{kind} {pick(1)[0]}")
        elif kind == "u1":
            lines.append(f"u1 {pick(1)[0]} {ph}")
        elif kind == "u1m":
            lines.append(f"u1m {pick(1)[0]} {int(rng.integers(2))} {ph}")
        elif kind == "cx":
            c, t = pick(2)
            lines.append(f"cx {c} {t} {int(rng.integers(2))}")
        elif kind in ("mcx", "mcxm", "mcu1", "mcu1m"):
            k = int(rng.integers(1, min(4, len(free) - 1) + 1))
            qs = pick(k + 1)
            cs, t = qs[:k], qs[k]
            s = f"{kind} {k} " + " ".join(map(str, cs))
            if kind.endswith("m"):
                s += " " + " ".join(str(int(rng.integers(2))) for _ in cs)
            s += f" {t}"
            if kind.startswith("mcu1"):
                s += f" {ph}"
            lines.append(s)
        elif kind == "cu1":
            c, t = pick(2)
            lines.append(f"cu1 {c} {t} {ph} {int(rng.integers(2))}")
        elif kind == "swap":
            a, b = pick(2)
            lines.append(f"swap {a} {b}")
        elif kind in ("ptp", "ptpg"):
            while True:
                k = int(rng.integers(1, min(6, len(free)) + 1)) if kind == "ptpg" else int(rng.integers(1, min(3, len(free)) + 1))
                ps = [int(x) for x in rng.integers(1, 4, size=k)]
                if kind == "ptpg" or _ref_supported_ptp(ps):
                    break
            qs = pick(k)
            lines.append(f"{kind} {k} " + " ".join(map(str, qs)) + " " + " ".join(map(str, ps)) + f" {ph}")
        elif kind in ("qft", "iqft"):
            # fixed register width per script: the reference sizes its QFT phase
            # table on the first call (src/suqa.cu:620-625)
            k = 2 if n < 6 else 3
            if len(free) < k:
                continue
            qs = pick(k)
            lines.append(f"{kind} {k} " + " ".join(map(str, qs)))
        elif kind == "plist":
            qsz = int(rng.integers(1, min(4, n) + 1))
            q0 = int(rng.integers(0, n - qsz + 1))
            phs = " ".join(hx(v) for v in rng.uniform(-math.pi, math.pi, size=1 << qsz))
            lines.append(f"plist {q0} {qsz} {phs}")
        if measure_every and (g + 1) % measure_every == 0:
            q = int(rng.choice(free))
            op = ["measure", "reset", "prob"][int(rng.integers(3))]
            if op == "prob":
                k = int(rng.integers(1, min(3, n) + 1))
                qs = [int(x) for x in rng.choice(n, size=k, replace=False)]
                ms = [int(rng.integers(2)) for _ in qs]
                lines.append(f"prob {k} " + " ".join(map(str, qs)) + " " + " ".join(map(str, ms)))
            else:
                lines.append(f"{op} {q} {hx(rng.random())}")
        if dump_every and (g + 1) % dump_every == 0:
            lines.append("dump")
    if gc_on:
        lines.append(f"gc_off {len(gc_on)} " + " ".join(map(str, gc_on)))
    lines += ["vnorm", "dump"]
    return lines


def test_suqa_sequence():
    """The gate sequence of the reference's src/test_suqa.cu:21-111, with a dump
    after every gate (the reference prints them only in debug builds)."""
    L = ["setup 5"]
    for g in ["x 3", "x 3", "h 1", "x 3", "h 1", "cx 3 0 1", "cx 3 0 1", "h 0", "h 1", "h 2", "h 4",
              "cx 0 4 1", f"u1 3 {hx(math.pi / 3.0)}"]:
        L += [g, "dump"]
    L += ["setup 1"]
    for _ in range(4):
        L += [f"ptp 1 0 1 {hx(math.pi / 4.0)}", "dump"]
    L += ["setup 2"]
    for _ in range(4):
        L += [f"ptp 2 0 1 1 1 {hx(math.pi / 4.0)}", "dump"]
    return L
