"""Bloch data of chain states for the equilibrium-angle warm-start targets
(suqa_gb300.warmstart.spin_bloch), on states whose values are known in closed
form; numpy only."""
import numpy as np

from suqa_gb300.warmstart import spin_bloch


def _product(theta, spins, extra_qubits):
    one = np.array([np.cos(theta / 2), np.sin(theta / 2)])
    psi = np.array([1.0])
    for _ in range(spins):
        psi = np.kron(one, psi)  # spin i on bit i
    reg = np.zeros(1 << extra_qubits)
    reg[3 % len(reg)] = 1.0  # the registers above the spins in some basis state
    return np.kron(reg, psi)


def test_product_state_gives_its_angle():
    for theta in (0.3, 0.9, 1.4):
        X, zz = spin_bloch(_product(theta, 5, 3), 5)
        assert np.allclose(X, np.sin(theta))
        assert np.allclose(zz, np.cos(theta) ** 2)
        assert np.allclose(np.arctan2(X, np.sqrt(zz)), theta)


def test_parity_eigenstate_has_no_x_and_full_bonds():
    s = 4
    psi = np.zeros(1 << (s + 2), dtype=complex)
    psi[0] = psi[(1 << s) - 1] = 1 / np.sqrt(2)  # (|0000> + |1111>) / sqrt 2, registers in |0>
    X, zz = spin_bloch(psi, s)
    assert np.allclose(X, 0.0) and np.allclose(zz, 1.0)


def test_registers_are_traced_out():
    """A spin state entangled with the register: the reduced state is mixed."""
    s = 3
    a = _product(0.0, s, 1)        # |000>, register |1>
    b = _product(np.pi, s, 1)      # |111>, register |1>
    b = np.roll(b, -(1 << s))      # register |0> instead
    psi = (a + b) / np.sqrt(2)
    X, zz = spin_bloch(psi, s)
    assert np.allclose(X, 0.0) and np.allclose(zz, 1.0)


def test_energy_target_angle_inverts_the_product_energy():
    """angle_for_energy returns the product-state angle of an energy inside the
    product states' range on [-pi/2, theta*], and clamps outside it."""
    import math
    from suqa_gb300.warmstart import angle_for_energy, product_energy
    for spins, J, h in ((6, 1.0, 0.7), (12, 1.0, 1.4), (4, 1.0, 2.5)):
        tmin = math.asin(min(1.0, h / (2.0 * J)))
        for th in np.linspace(-math.pi / 2 + 1e-3, tmin - 1e-3, 7):
            E = product_energy(th, spins, J, h)
            assert abs(angle_for_energy(E, spins, J, h) - th) < 1e-9
        assert angle_for_energy(1e9, spins, J, h) == -math.pi / 2
        assert abs(angle_for_energy(-1e9, spins, J, h) - tmin) < 1e-12
