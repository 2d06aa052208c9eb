"""Exact thermal energies of transverse-field Ising rings (test infrastructure).

H = -J sum_i Z_i Z_{i+1} - h sum_i X_i on a periodic ring of s spins (the
system of oracle/systems/tfim/system.cuh), diagonalised densely (s <= 12).
Used to state how far the QMS chains of a given configuration (energy window,
register width, Trotter step) sit from the Gibbs ensemble they approximate.
"""
import numpy as np


def hamiltonian(s, J, h):
    N = 1 << s
    idx = np.arange(N)
    diag = np.zeros(N)
    for i in range(s):
        j = (i + 1) % s
        zi = 1 - 2 * ((idx >> i) & 1)
        zj = 1 - 2 * ((idx >> j) & 1)
        diag -= J * zi * zj
    H = np.diag(diag)
    for i in range(s):
        H[idx, idx ^ (1 << i)] -= h
    return H


def spectrum(s, J, h):
    return np.linalg.eigvalsh(hamiltonian(s, J, h))


def thermal_energy(s, J, h, beta):
    w = spectrum(s, J, h)
    p = np.exp(-beta * (w - w.min()))
    return float(np.dot(p, w) / p.sum())
