"""Batched real-time evolution of TFIM rings (sq_tfim_evolve_batch) against the
CPU oracle: the same first-order Trotter gate sequence (exp(i J dt ZZ) on every
bond, then exp(i h dt X) on every spin) applied by the oracle's exact Pauli
rotations, probabilities compared after every step."""
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

PAULI_X, PAULI_Z = 1, 3


def oracle_rows(spins, steps, J, h, dt, warm=None):
    L = oracle.load()
    st = oracle.OracleState(spins)
    if warm is not None:
        a = np.array([1.0 + 0j])
        for i in range(spins):  # qubit 0 is the least significant
            v = np.array([math.cos(warm[i] / 2), math.sin(warm[i] / 2)], dtype=complex)
            a = np.kron(v, a)
        st.set_array(a)
    rows = [np.abs(st.array()) ** 2]
    for _ in range(steps):
        for i in range(spins):
            q = oracle._u32arr([i, (i + 1) % spins])
            L.or_apply_pauli(st.p, 2, q, oracle._u32arr([PAULI_Z, PAULI_Z]), J * dt, 0, 0)
        for i in range(spins):
            L.or_apply_pauli(st.p, 1, oracle._u32arr([i]), oracle._u32arr([PAULI_X]), h * dt, 0, 0)
        rows.append(np.abs(st.array()) ** 2)
    st.close()
    return np.array(rows)


JOBS = [(3, 6, 1.0, 0.7, 0.1), (4, 8, 1.0, 1.2, 0.1), (5, 5, 0.8, 1.0, 0.05), (7, 4, 1.0, 0.9, 0.1),
        (9, 3, 1.0, 1.1, 0.1), (10, 3, 1.0, 0.6, 0.08), (12, 2, 1.0, 1.0, 0.1)]


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 2e-5)])
def test_evolution_rows_match_oracle(precision, tol):
    from suqa_gb300.batch import TfimEvolution, run_tfim_evolution
    jobs = [TfimEvolution(spins=s, steps=k, J=J, h=h, dt=dt) for (s, k, J, h, dt) in JOBS]
    jobs.append(TfimEvolution(spins=6, steps=4, J=1.0, h=1.0, dt=0.1, warm_angles=[0.3, -0.2, 0.5, 0.1, -0.4, 0.7]))
    got, _ = run_tfim_evolution(jobs, precision)
    for j, g in zip(jobs, got):
        want = oracle_rows(j.spins, j.steps, j.J, j.h, j.dt, j.warm_angles)
        assert g.shape == want.shape
        assert np.max(np.abs(g - want)) < tol, (j, np.max(np.abs(g - want)))
        assert np.allclose(g.sum(axis=1), 1.0, atol=10 * tol)


def test_evolution_of_a_classical_ring_is_trivial():
    """h = 0: |0...0> is an eigenstate (probability 1 stays on it)."""
    from suqa_gb300.batch import TfimEvolution, run_tfim_evolution
    got, _ = run_tfim_evolution([TfimEvolution(spins=8, steps=5, J=1.0, h=0.0, dt=0.1)], "f64")
    assert np.allclose(got[0][:, 0], 1.0, atol=1e-13)
