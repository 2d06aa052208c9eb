"""Python access to the CPU oracle (liboracle.so, the C restatement in sq_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
CPU-baseline leg of bench.py, never by the product package.

Gate scripts are lists of text lines in the grammar of oracle/ref_dump.cpp (the
golden dumper that replays the same script through the reference build).  The
host-side mask construction below restates the reference dispatcher
(src/suqa.cu:45-61 gc mask, :267-416 gate masks, :705-727 prob_filter).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DUMP = os.path.join(HERE, "_ref", "ref_dump")


class _OrState(C.Structure):
    _fields_ = [("n", C.c_uint32), ("N", C.c_uint64), ("data", C.POINTER(C.c_double)),
                ("re", C.POINTER(C.c_double)), ("im", C.POINTER(C.c_double))]


class _OrPcg(C.Structure):
    _fields_ = [("state", C.c_uint64), ("inc", C.c_uint64)]


_lib = None


def build():
    """Compile liboracle.so (plain C, no reference sources needed)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = C.CDLL(LIB_PATH)
    P = C.POINTER(_OrState)
    u32, u64, dbl = C.c_uint32, C.c_uint64, C.c_double
    sig = {
        "or_set_threads": (None, [C.c_int]),
        "or_create": (P, [u32]),
        "or_destroy": (None, [P]),
        "or_init_state": (None, [P]),
        "or_vnorm": (dbl, [P]),
        "or_vnormalize": (None, [P]),
        "or_apply_x": (None, [P, u32, u64]),
        "or_apply_y": (None, [P, u32, u64]),
        "or_apply_h": (None, [P, u32, u64]),
        "or_apply_u1": (None, [P, u32, u32, dbl, u64]),
        "or_apply_mcx": (None, [P, u64, u64, u32]),
        "or_apply_mcu1": (None, [P, u64, u64, dbl]),
        "or_apply_swap": (None, [P, u32, u32, u64]),
        "or_apply_phase_list": (C.c_int, [P, u32, u32, C.POINTER(dbl), u64]),
        "or_apply_pauli": (C.c_int, [P, u32, C.POINTER(u32), C.POINTER(u32), dbl, u64, C.c_int]),
        "or_apply_qft": (None, [P, u32, C.POINTER(u32), u64]),
        "or_apply_qft_inverse": (None, [P, u32, C.POINTER(u32), u64]),
        "or_prob1": (dbl, [P, u32]),
        "or_measure_qbit": (u32, [P, u32, dbl]),
        "or_apply_reset": (None, [P, u32, dbl, u64]),
        "or_prob_filter": (dbl, [P, u64, u64]),
        "or_apply_qms_w": (None, [P, u32, u64, u32, u32, dbl]),
        "or_pcg_seed": (None, [C.POINTER(_OrPcg), u64, u64]),
        "or_pcg_next": (u32, [C.POINTER(_OrPcg)]),
        "or_pcg_doub": (dbl, [C.POINTER(_OrPcg)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _u32arr(xs):
    return (C.c_uint32 * len(xs))(*xs)


class OracleState:
    """A dense FP64 state held by the C oracle, plus the reference's gc mask."""

    def __init__(self, n: int):
        self.L = load()
        self.n = n
        self.p = self.L.or_create(n)
        if not self.p:
            raise MemoryError("oracle state allocation failed")
        self.gc = 0

    def close(self):
        if self.p:
            self.L.or_destroy(self.p)
            self.p = None

    __del__ = close

    @property
    def N(self):
        return 1 << self.n

    def array(self) -> np.ndarray:
        """Copy of the state as complex128."""
        N = self.N
        buf = np.ctypeslib.as_array(self.p.contents.data, shape=(2 * N,))
        return buf[:N] + 1j * buf[N:]

    def set_array(self, a: np.ndarray):
        N = self.N
        buf = np.ctypeslib.as_array(self.p.contents.data, shape=(2 * N,))
        buf[:N] = a.real
        buf[N:] = a.imag


def run_script(lines, threads: int = 1):
    """Execute a gate script on the C oracle.  Returns a list of results in the
    dumper's output order: ("M", c), ("P", p), ("N", norm), ("S", complex array),
    ("E", msg)."""
    L = load()
    L.or_set_threads(threads)
    st = None
    out = []
    it = iter(lines)
    for line in it:
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        tok = line.split()
        cmd, a = tok[0], tok[1:]
        if cmd == "setup":
            if st is not None:
                st.close()
            st = OracleState(int(a[0]))
            continue
        if cmd == "setstate":
            vals = np.array([float.fromhex(v) for v in next(it).split()])
            N = st.N
            st.set_array(vals[:N] + 1j * vals[N:])
            continue
        out_item = _apply(L, st, cmd, a)
        if out_item is not None:
            out.append(out_item)
    if st is not None:
        st.close()
    L.or_set_threads(1)
    return out


def _lst(a, i):
    k = int(a[i])
    return [int(x) for x in a[i + 1:i + 1 + k]], i + 1 + k


def _ph(x):
    return float.fromhex(x) if ("0x" in x or "0X" in x) else float(x)


def _apply(L, st, cmd, a):
    p, gc = st.p, st.gc
    if cmd == "init":
        L.or_init_state(p)
    elif cmd == "vnorm":
        return ("N", L.or_vnorm(p))
    elif cmd == "normalize":
        L.or_vnormalize(p)
    elif cmd == "dump":
        return ("S", st.array().copy())
    elif cmd == "gc_on":
        qs, _ = _lst(a, 0)
        for q in qs:
            st.gc |= 1 << q
    elif cmd == "gc_off":
        qs, _ = _lst(a, 0)
        for q in qs:
            st.gc &= ~(1 << q)
    elif cmd == "x":
        L.or_apply_x(p, int(a[0]), gc)
    elif cmd == "y":
        L.or_apply_y(p, int(a[0]), gc)
    elif cmd == "h":
        L.or_apply_h(p, int(a[0]), gc)
    elif cmd in ("z", "s", "t", "tdg"):
        ph = {"z": math.pi, "s": math.pi / 2.0, "t": math.pi / 4.0, "tdg": -math.pi / 4.0}[cmd]
        L.or_apply_u1(p, int(a[0]), 1, ph, gc)
    elif cmd == "u1":
        L.or_apply_u1(p, int(a[0]), 1, _ph(a[1]), gc)
    elif cmd == "u1m":
        L.or_apply_u1(p, int(a[0]), int(a[1]), _ph(a[2]), gc)
    elif cmd == "cx":
        c, t, m = int(a[0]), int(a[1]), int(a[2])
        mask_qs = gc | ((1 << c) if m else 0)
        L.or_apply_mcx(p, gc | (1 << c), mask_qs, t)
    elif cmd in ("mcx", "mcxm"):
        cs, i = _lst(a, 0)
        ms = [int(x) for x in a[i:i + len(cs)]] if cmd == "mcxm" else [1] * len(cs)
        if cmd == "mcxm":
            i += len(cs)
        t = int(a[i])
        mask = gc
        mask_qs = gc
        for c, m in zip(cs, ms):
            mask |= 1 << c
            if m:
                mask_qs |= 1 << c
        L.or_apply_mcx(p, mask, mask_qs, t)
    elif cmd == "cu1":
        c, t, ph, m = int(a[0]), int(a[1]), _ph(a[2]), int(a[3])
        mask_qs = (1 << t) | gc
        mask = mask_qs | (1 << c)
        if m:
            mask_qs |= 1 << c
        L.or_apply_mcu1(p, mask, mask_qs, ph)
    elif cmd in ("mcu1", "mcu1m"):
        cs, i = _lst(a, 0)
        ms = [int(x) for x in a[i:i + len(cs)]] if cmd == "mcu1m" else [1] * len(cs)
        if cmd == "mcu1m":
            i += len(cs)
        t, ph = int(a[i]), _ph(a[i + 1])
        mask = (1 << t) | gc
        mask_qs = (1 << t) | gc
        for c, m in zip(cs, ms):
            mask |= 1 << c
            if m:
                mask_qs |= 1 << c
        L.or_apply_mcu1(p, mask, mask_qs, ph)
    elif cmd == "swap":
        L.or_apply_swap(p, int(a[0]), int(a[1]), gc)
    elif cmd == "ptp":
        qs, i = _lst(a, 0)
        ps = [int(x) for x in a[i:i + len(qs)]]
        ph = _ph(a[i + len(qs)])
        rc = L.or_apply_pauli(p, len(qs), _u32arr(qs), _u32arr(ps), ph, gc, 1)
        if rc != 0:
            return ("E", "unsupported pauli rotation")
    elif cmd == "ptpg":  # any Pauli string (no reference counterpart beyond its subset)
        qs, i = _lst(a, 0)
        ps = [int(x) for x in a[i:i + len(qs)]]
        L.or_apply_pauli(p, len(qs), _u32arr(qs), _u32arr(ps), _ph(a[i + len(qs)]), gc, 0)
    elif cmd == "plist":  # phase list: q0 q_size phases...
        q0, qsz = int(a[0]), int(a[1])
        phs = [_ph(x) for x in a[2:2 + (1 << qsz)]]
        arr = (C.c_double * len(phs))(*phs)
        L.or_apply_phase_list(p, q0, qsz, arr, gc)
    elif cmd == "qft":
        qs, _ = _lst(a, 0)
        L.or_apply_qft(p, len(qs), _u32arr(qs), gc)
    elif cmd == "iqft":
        qs, _ = _lst(a, 0)
        L.or_apply_qft_inverse(p, len(qs), _u32arr(qs), gc)
    elif cmd == "measure":
        return ("M", int(L.or_measure_qbit(p, int(a[0]), _ph(a[1]))))
    elif cmd == "reset":
        L.or_apply_reset(p, int(a[0]), _ph(a[1]), gc)
    elif cmd == "prob":
        qs, i = _lst(a, 0)
        ms = [int(x) for x in a[i:i + len(qs)]]
        mask_qs = 0
        mask = 0
        for q, m in zip(qs, ms):
            mask_qs |= 1 << q
            if m:
                mask |= m << q
        return ("P", L.or_prob_filter(p, mask_qs, mask))
    else:
        raise ValueError(f"unknown command {cmd}")
    return None


def run_reference(lines, workdir):
    """Run a script through the reference build's golden dumper (only where
    oracle/_ref exists, i.e. where the reference sources were compiled)."""
    out_path = os.path.join(workdir, "ref_out.txt")
    subprocess.run([REF_DUMP, out_path], input="\n".join(lines) + "\n", text=True,
                   check=True, stdout=subprocess.DEVNULL)
    return parse_dump(open(out_path).read().splitlines())


def parse_dump(lines):
    res = []
    it = iter(lines)
    for line in it:
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "M":
            res.append(("M", int(tok[1])))
        elif tok[0] == "P":
            res.append(("P", float.fromhex(tok[1])))
        elif tok[0] == "N":
            res.append(("N", float.fromhex(tok[1])))
        elif tok[0] == "E":
            res.append(("E", " ".join(tok[1:])))
        elif tok[0] == "S":
            re_ = np.array([float.fromhex(v) for v in next(it).split()])
            im_ = np.array([float.fromhex(v) for v in next(it).split()])
            res.append(("S", re_ + 1j * im_))
    return res


class Pcg32:
    """PCG32 through the oracle (pcg32.h:53-68 and :121-130 of the reference)."""

    def __init__(self, seed: int, initseq: int = 1):
        self.L = load()
        self.g = _OrPcg()
        self.L.or_pcg_seed(C.byref(self.g), seed, initseq)

    def next_u32(self) -> int:
        return int(self.L.or_pcg_next(C.byref(self.g)))

    def doub(self) -> float:
        return float(self.L.or_pcg_doub(C.byref(self.g)))


def apply_circuit(ost: "OracleState", gates):
    """Applies a benchmark circuit (suqa_gb300.workloads.random_circuit form) on the
    oracle (CPU-baseline timing, parity of the full-size benchmark circuit);
    returns the measured bits."""
    L = load()
    p = ost.p
    bits = []
    for g in gates:
        k = g[0]
        if k == "x":
            L.or_apply_x(p, g[1], 0)
        elif k == "h":
            L.or_apply_h(p, g[1], 0)
        elif k == "cx":
            L.or_apply_mcx(p, 1 << g[1], 1 << g[1], g[2])
        elif k == "mcx":
            m = sum(1 << q for q in g[1])
            L.or_apply_mcx(p, m, m, g[2])
        elif k == "u1":
            L.or_apply_u1(p, g[1], 1, g[2], 0)
        elif k == "ptp":
            L.or_apply_pauli(p, len(g[1]), _u32arr(g[1]), _u32arr(g[2]), g[3], 0, 0)
        elif k == "measure":
            bits.append(int(L.or_measure_qbit(p, g[1], g[2])))
    return bits
