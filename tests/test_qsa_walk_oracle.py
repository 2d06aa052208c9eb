"""The Szegedy-walk oracle: its compressed walk (closed-form energy register,
branch-decomposed walk-phase register) against a gate-by-gate simulation of the
uncompressed registers in the reference's QSA structure."""
import math

import numpy as np
import pytest

import qsa_walk as qw


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_compressed_step_equals_gate_level_step(seed):
    rng = np.random.default_rng(seed)
    s, q, e = 3, 3, 3
    J = [int(v) for v in rng.choice([-1, 1], s)]
    cw = qw.CompressedWalk(s, J)
    psi = cw.initial()
    for _ in range(seed):  # start from a state the walk has already moved
        P, S, n2 = qw.walk_step(cw, psi, int(rng.integers(s)), 0.8, q)
        psi = S / math.sqrt(n2)
    C, beta = int(rng.integers(s)), float(rng.uniform(0.3, 2.0))
    # energy differences of a 3-spin ring with |J| = 1 lie in -6..6: an exact grid of spacing 2
    Pg, out, leak = qw.gate_level_step(s, J, beta, C, q, e, -6, 2, psi)
    P, S, n2 = qw.walk_step(cw, psi, C, beta, q)
    assert np.max(np.abs(Pg - P)) < 1e-12
    assert leak < 1e-12  # the energy register returns to zero
    assert np.max(np.abs(out.imag)) < 1e-12  # the walk is real
    assert np.max(np.abs(out.real - S / math.sqrt(n2))) < 1e-12


def test_initial_state_is_a_fixed_point_at_infinite_temperature():
    cw = qw.CompressedWalk(4, [1, -1, 1, 1])
    P, S, n2 = qw.walk_step(cw, cw.initial(), 2, 0.0, 4)
    assert abs(P[0] - 1.0) < 1e-12 and np.all(np.abs(P[1:]) < 1e-12)


def test_phase_probabilities_sum_to_the_norm():
    rng = np.random.default_rng(4)
    g = rng.normal(size=16)
    g[0] = 1.0
    assert abs(qw.phase_probs(g).sum() - 1.0) < 1e-12


def test_register_readout_follows_the_conditional_probabilities():
    P = np.array([0.1, 0.2, 0.3, 0.4])
    # bit 0: p1 = 0.6; r = 0.5 < 0.6 -> 1; bit 1 given bit0=1: p1 = 0.4/0.6; r = 0.7 >= 0.667 -> 0
    assert qw.measure_register(P, [0.5, 0.7]) == 1
    assert qw.measure_register(P, [0.7, 0.1]) == 2


def test_walk_driver_cap_and_completion():
    import oracle
    a = qw.run_walk(3, [1, 1, -1], 1.0, 2, 3, 3, seed=11, rng=oracle.Pcg32(11))
    assert a.done == 1 and a.steps >= 6 + a.restarts  # last attempt: 6 steps; each abandoned one >= 1
    assert a.E == float(qw.ring_energies(3, [1, 1, -1])[a.readout])
    b = qw.run_walk(3, [1, 1, -1], 1.0, 2, 3, 3, seed=11, max_steps=2, rng=oracle.Pcg32(11))
    assert b.done == 0 and b.steps == 2
