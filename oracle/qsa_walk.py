"""CPU oracle for the batched Szegedy-walk annealer (QSA on Ising rings).

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
CPU-baseline leg of bench.py, never by the product package.

The reference QSA (include/qsa.cuh, src/qsa.cu) is written for the 3-spin
triangle only: its rotation and reflection are hard-wired to one energy level
(qsa.cuh:421-474) and its energy register aliases the copy register
(qsa.cuh:107-115 against system.cuh:33).  This module restates the walk in the
general form its own commented-out code describes (qsa.cuh:372-418: a rotation
for every level with a positive energy difference, a reflection for every level
with a zero difference) on a ring of s spins with integer couplings and no
field, H(x) = -sum_i J_i s_i s_{i+1 mod s}, s_i = 1 - 2 x_i.

Registers: system x (s qubits), copy x~ (s qubits), the energy-difference
register, the walk-phase register (q qubits), the acceptance qubit.  Because H is
diagonal with integer spectrum, phase estimation of exp(-it(H(x~)-H(x))) on a
grid that contains every difference is exact, so each block "estimate, act on
the level, un-estimate" (qsa.cuh:616-709) equals the action applied directly as
a function of dE = H(x~) - H(x); the energy register always returns to zero and
is not stored.  `gate_level_step` below simulates the uncompressed registers
gate by gate (qsa.cuh:251-295 phase estimation, :421-474 rotation/reflection,
:616-756 walk) so the test suite can check this equivalence.

Compressed state: real amplitudes psi[acc, d, x] with d = x XOR x~ (every gate
of the walk is real and the initial state is real).  One walk operator W for the
move C (qsa.cuh:711-718, in application order):
    L1, H_C, R, S0, R^T, H_C, L1, H_C, R, S0, R^T, H_C
  L1   : -1 on acc = 0 where dE = 0                      (universal_reflection)
  H_C  : Hadamard on copy bit C                          (qsa_apply_C)
  R    : RY on acc where dE > 0, ptp(Y, -acos(e)) with e = exp(-beta dE / 2)
         = [[e, -r], [r, e]], r = sqrt(1 - e^2)           (universal_rotation)
  S0   : swap x <-> x~ where acc = 0                     (apply_uy's swaps)
One walk step (qsa.cu:181-205): H on the q walk-phase qubits, controlled
W^(2^(q-1-j)) on walk-phase qubit j, inverse QFT (qsa.cuh:732-756), measure the
q qubits one by one.  The branches of the walk-phase register are independent,
so with v_k = W^k psi the register value m has amplitude
    w_m = L^-2 sum_k exp(-2 pi i m k / L) v_k,   L = 2^q
(the reference's bit order turns its inverse QFT into exactly this DFT), whence
    P(m) = L^-2 sum_{|j|<L} (L - |j|) g_|j| cos(2 pi m j / L),  g_j = <psi, W^j psi>
and the state after reading m = 0 is sum_k v_k normalised.  A nonzero reading
restarts the anneal from the initial state sum_x |x>|x>|acc 0> (qsa.cu:199-205).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def ring_energies(s: int, J) -> np.ndarray:
    """Integer energies H(x) for x in [0, 2^s), bond i joins spins i and i+1 mod s."""
    x = np.arange(1 << s)
    sig = 1 - 2 * ((x[:, None] >> np.arange(s)[None, :]) & 1)
    E = np.zeros(1 << s, dtype=np.int64)
    for i in range(s):
        E -= int(J[i]) * sig[:, i] * sig[:, (i + 1) % s]
    return E


def draw_move(rng, s: int) -> int:
    """Move choice as qsa::draw_C (qsa.cuh:334-343) with weight sums (i+1)/s."""
    u = rng.doub()
    for i in range(s):
        if u < (i + 1) / s:
            return i
    return s


class CompressedWalk:
    """W on psi[acc, d, x] (FP64) for one ring."""

    def __init__(self, s: int, J):
        self.s = s
        self.N = 1 << s
        self.E = ring_energies(s, J)
        d = np.arange(self.N)[:, None]
        x = np.arange(self.N)[None, :]
        self.xt = x ^ d                                   # copy register value x~
        self.dE = self.E[self.xt] - self.E[x]             # [d, x]
        self.zero = self.dE == 0
        self.swap_src = np.broadcast_to(x ^ d, (self.N, self.N))

    def coeffs(self, beta: float):
        pos = self.dE > 0
        e = np.where(pos, np.exp(-0.5 * beta * np.where(pos, self.dE, 0)), 1.0)
        r = np.where(pos, np.sqrt(1.0 - e * e), 0.0)
        return e, r

    def apply(self, p: np.ndarray, C: int, e: np.ndarray, r: np.ndarray) -> np.ndarray:
        N = self.N
        rows = np.arange(N)
        partner = rows ^ (1 << C)
        tbit = (self.xt >> C) & 1
        h = math.sqrt(0.5)

        def L1(p):
            p = p.copy()
            p[0][self.zero] *= -1.0
            return p

        def HC(p):
            q = p[:, partner, :]
            return np.where(tbit[None] == 0, (p + q) * h, (q - p) * h)

        def R(p, sign):
            p0, p1 = p[0], p[1]
            if sign > 0:
                return np.stack([e * p0 - r * p1, r * p0 + e * p1])
            return np.stack([e * p0 + r * p1, -r * p0 + e * p1])

        def S0(p):
            p = p.copy()
            p[0] = np.take_along_axis(p[0], self.swap_src, axis=1)
            return p

        p = L1(p)
        p = HC(p)
        p = R(p, +1)
        p = S0(p)
        p = R(p, -1)
        p = HC(p)
        p = L1(p)
        p = HC(p)
        p = R(p, +1)
        p = S0(p)
        p = R(p, -1)
        p = HC(p)
        return p

    def initial(self) -> np.ndarray:
        p = np.zeros((2, self.N, self.N))
        p[0, 0, :] = 1.0 / math.sqrt(self.N)
        return p


def phase_probs(g: np.ndarray) -> np.ndarray:
    """P(m) of the walk-phase register from g_j = <psi, W^j psi>, j < L."""
    L = len(g)
    j = np.arange(1, L)
    out = np.empty(L)
    for m in range(L):
        out[m] = (L * g[0] + 2.0 * np.sum((L - j) * g[1:] * np.cos(2 * np.pi * ((m * j) % L) / L))) / (L * L)
    return out


def walk_step(cw: CompressedWalk, psi: np.ndarray, C: int, beta: float, q: int):
    """Returns (P[m], S = sum_k W^k psi, |S|^2)."""
    L = 1 << q
    e, r = cw.coeffs(beta)
    v = psi
    S = np.zeros_like(psi)
    g = np.zeros(L)
    for k in range(L):
        g[k] = float(np.sum(psi * v))
        S += v
        if k < L - 1:
            v = cw.apply(v, C, e, r)
    n2 = L * g[0] + 2.0 * float(np.sum((L - np.arange(1, L)) * g[1:]))
    return phase_probs(g), S, n2


def measure_register(P: np.ndarray, rands) -> int:
    """Qubit-by-qubit readout (suqa measure_qbits; c = r < p1) of a register
    whose value distribution is P."""
    L = len(P)
    m = 0
    alive = np.ones(L, dtype=bool)
    vals = np.arange(L)
    for j, r in enumerate(rands):
        den = float(np.sum(P[alive]))
        num = float(np.sum(P[alive & (((vals >> j) & 1) == 1)]))
        p1 = num / den if den > 0 else 0.0
        c = 1 if r < p1 else 0
        m |= c << j
        alive &= ((vals >> j) & 1) == c
    return m


@dataclass
class WalkResult:
    done: int
    restarts: int
    steps: int
    readout: int
    E: float
    absM: float
    last_p0: float
    p0: list = field(default_factory=list)


def run_walk(s: int, J, beta: float, stages: int, steps_per_stage: int, q: int, seed: int,
             max_steps: int = 0, rng=None) -> WalkResult:
    """One annealed walk: beta_k = (k+1) beta / stages for k = 0..stages-1,
    steps_per_stage walk steps at each; draws per step: the move, then q
    readout values; a completed anneal reads the s spins with s draws."""
    if rng is None:
        from oracle import Pcg32
        rng = Pcg32(seed)
    cw = CompressedWalk(s, J)
    nominal = stages * steps_per_stage
    cap = max_steps or 8 * nominal
    C = draw_move(rng, s)
    psi = cw.initial()
    att = 0
    total = 0
    restarts = 0
    trace = []
    while True:
        beta_k = (att // steps_per_stage + 1) * beta / stages
        P, S, n2 = walk_step(cw, psi, C, beta_k, q)
        rands = [rng.doub() for _ in range(q)]
        m = measure_register(P, rands)
        total += 1
        trace.append(float(P[0] / np.sum(P)))
        if m == 0:
            psi = S / math.sqrt(n2)
            att += 1
            if att == nominal:
                break
        else:
            restarts += 1
            psi = cw.initial()
            att = 0
        if total >= cap:
            return WalkResult(0, restarts, total, 0, 0.0, 0.0, trace[-1], trace)
        C = draw_move(rng, s)
    Px = np.sum(psi * psi, axis=(0, 1))
    x = measure_register(Px, [rng.doub() for _ in range(s)])
    M = abs(sum(1 - 2 * ((x >> i) & 1) for i in range(s)))
    return WalkResult(1, restarts, total, x, float(cw.E[x]), float(M), trace[-1], trace)


# ---------------------------------------------------------------------------
# Gate-level walk step on the uncompressed registers (checks the compression).

class _Reg:
    def __init__(self, s, e, q):
        self.s, self.e, self.q = s, e, q
        self.sys = list(range(s))
        self.cpy = list(range(s, 2 * s))
        self.ene = list(range(2 * s, 2 * s + e))
        self.szg = list(range(2 * s + e, 2 * s + e + q))
        self.acc = 2 * s + e + q
        self.n = self.acc + 1
        self.idx = np.arange(1 << self.n)


class _Gates:
    def __init__(self, reg: _Reg, E: np.ndarray):
        self.r = reg
        i = reg.idx
        s = reg.s
        x = i & ((1 << s) - 1)
        xt = (i >> s) & ((1 << s) - 1)
        self.dE = (E[xt] - E[x]).astype(np.float64)

    def _sel(self, ctrl):
        return (self.r.idx & ctrl) == ctrl

    def h(self, st, qb, ctrl=0):
        i = self.r.idx
        lo = ((i >> qb) & 1 == 0) & self._sel(ctrl)
        a = st[lo].copy()
        b = st[i[lo] | (1 << qb)].copy()
        c = 0.7071067811865475
        st[lo] = (a + b) * c
        st[i[lo] | (1 << qb)] = (a - b) * c

    def x(self, st, qb, ctrl=0):
        i = self.r.idx
        lo = ((i >> qb) & 1 == 0) & self._sel(ctrl)
        a = st[lo].copy()
        st[lo] = st[i[lo] | (1 << qb)]
        st[i[lo] | (1 << qb)] = a

    def u1(self, st, qb, ph, ctrl=0):
        m = self._sel(ctrl | (1 << qb))
        st[m] *= np.exp(1j * ph)

    def ry(self, st, qb, th, ctrl=0):
        """suqa apply_pauli_TP_rotation({qb}, {PAULI_Y}, th) = [[c, s], [-s, c]]."""
        i = self.r.idx
        lo = ((i >> qb) & 1 == 0) & self._sel(ctrl)
        a = st[lo].copy()
        b = st[i[lo] | (1 << qb)].copy()
        c, sn = math.cos(th), math.sin(th)
        st[lo] = c * a + sn * b
        st[i[lo] | (1 << qb)] = -sn * a + c * b

    def swap(self, st, q1, q2, ctrl=0):
        i = self.r.idx
        m = (((i >> q1) & 1) == 1) & (((i >> q2) & 1) == 0) & self._sel(ctrl)
        j = i[m] ^ (1 << q1) ^ (1 << q2)
        a = st[m].copy()
        st[m] = st[j]
        st[j] = a

    def evo(self, st, t, ctrl):
        """evolution_szegedy(t) = exp(-i t (H(x~) - H(x))), under ctrl."""
        m = self._sel(ctrl)
        st[m] *= np.exp(-1j * t * self.dE[m])


def gate_level_step(s, J, beta, C, q, e, emin, spacing, psi_c):
    """One walk step on the uncompressed registers from the compressed state
    psi_c[acc, d, x]; returns (P[m] of the walk-phase register, the state after
    reading m = 0 mapped back to [acc, d, x], the largest amplitude left in
    nonzero energy-register values)."""
    reg = _Reg(s, e, q)
    E = ring_energies(s, J)
    G = _Gates(reg, E)
    N = 1 << s
    st = np.zeros(1 << reg.n, dtype=np.complex128)
    for a in range(2):
        for d in range(N):
            for x in range(N):
                st[x | ((x ^ d) << s) | (a << reg.acc)] = psi_c[a, d, x]
    Le = 1 << e
    factor = 1.0 / (Le * spacing)            # t_PE_factor: level = factor L (dE - emin)
    t = factor * 8.0 * math.atan(1.0)
    levels = [emin + k * spacing for k in range(Le)]
    ene_all = sum(1 << b for b in reg.ene)

    def qft_inv(st, regq, ctrl):
        for o in range(len(regq)):
            for inn in range(o):
                G.u1(st, regq[o], -2 * math.pi / (1 << (1 + o - inn)), ctrl | (1 << regq[inn]))
            G.h(st, regq[o], ctrl)

    def qft(st, regq, ctrl):
        for o in range(len(regq) - 1, -1, -1):
            G.h(st, regq[o], ctrl)
            for inn in range(o - 1, -1, -1):
                G.u1(st, regq[o], 2 * math.pi / (1 << (1 + o - inn)), ctrl | (1 << regq[inn]))

    def pe(st, ctrl):
        for b in reg.ene:
            G.h(st, b, ctrl)
        for trg in range(e - 1, -1, -1):
            pw = float(1 << (e - 1 - trg))
            G.evo(st, -pw * t, ctrl | (1 << reg.ene[trg]))
            G.u1(st, reg.ene[trg], -pw * t * emin, ctrl)
        qft_inv(st, reg.ene, ctrl)

    def pe_inv(st, ctrl):
        qft(st, reg.ene, ctrl)
        for trg in range(e):
            pw = float(1 << (e - 1 - trg))
            G.evo(st, pw * t, ctrl | (1 << reg.ene[trg]))
            G.u1(st, reg.ene[trg], pw * t * emin, ctrl)
        for b in reg.ene:
            G.h(st, b, ctrl)

    def ctrl_x(st, lvl, ctrl):
        for i, b in enumerate(reg.ene):
            if not (lvl >> i) & 1:
                G.x(st, b, ctrl)

    def rot(st, sign, ctrl):
        for k, dE in enumerate(levels):
            if dE > 0:
                ctrl_x(st, k, ctrl)
                G.ry(st, reg.acc, -sign * math.acos(math.exp(-0.5 * beta * dE)), ctrl | ene_all)
                ctrl_x(st, k, ctrl)

    def refl(st, ctrl):
        for k, dE in enumerate(levels):
            if dE == 0:
                ctrl_x(st, k, ctrl)
                G.x(st, reg.acc, ctrl | ene_all)
                G.u1(st, reg.acc, math.pi, ctrl | ene_all)
                G.x(st, reg.acc, ctrl | ene_all)
                ctrl_x(st, k, ctrl)

    def lam1(st, ctrl):
        pe(st, ctrl)
        refl(st, ctrl)
        pe_inv(st, ctrl)

    def ux(st, ctrl):
        G.h(st, reg.cpy[C], ctrl)
        pe(st, ctrl)
        rot(st, +1, ctrl)
        pe_inv(st, ctrl)

    def ux_inv(st, ctrl):
        pe(st, ctrl)
        rot(st, -1, ctrl)
        pe_inv(st, ctrl)
        G.h(st, reg.cpy[C], ctrl)

    def swaps(st, ctrl):
        G.x(st, reg.acc, ctrl)
        for j in range(s):
            G.swap(st, reg.sys[j], reg.cpy[j], ctrl | (1 << reg.acc))
        G.x(st, reg.acc, ctrl)

    def W(st, ctrl):
        lam1(st, ctrl)
        ux(st, ctrl)
        swaps(st, ctrl)      # uy^-1 = swaps then ux^-1
        ux_inv(st, ctrl)
        lam1(st, ctrl)
        ux(st, ctrl)         # uy = ux then swaps
        swaps(st, ctrl)
        ux_inv(st, ctrl)

    for b in reg.szg:
        G.h(st, b, 0)
    for trg in range(q - 1, -1, -1):
        for _ in range(1 << (q - 1 - trg)):
            W(st, 1 << reg.szg[trg])
    qft_inv(st, reg.szg, 0)

    i = reg.idx
    m_of = np.zeros_like(i)
    for j, b in enumerate(reg.szg):
        m_of |= ((i >> b) & 1) << j
    P = np.array([float(np.sum(np.abs(st[m_of == m]) ** 2)) for m in range(1 << q)])
    ene_of = (i >> reg.ene[0]) & (Le - 1)
    leak = float(np.max(np.abs(st[ene_of != 0]))) if np.any(ene_of != 0) else 0.0
    out = np.zeros((2, N, N), dtype=np.complex128)
    keep = (m_of == 0) & (ene_of == 0)
    for a in range(2):
        for d in range(N):
            for x in range(N):
                out[a, d, x] = st[x | ((x ^ d) << s) | (a << reg.acc)]
    out /= math.sqrt(P[0])
    return P, out, leak
