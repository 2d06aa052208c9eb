"""The CPU oracle (oracle/sq_oracle.c) pinned against the reference build: the
committed golden fixtures (made by the reference itself) and, where the reference
sources are compiled here, fresh random scripts through the golden dumper."""
import tempfile

import numpy as np
import pytest

import circuits
import golden_io
import oracle
from conftest import has_reference_build


def test_oracle_matches_golden_fixtures_bit_exact():
    n_cases = 0
    for name, lines, want in golden_io.gate_cases():
        got = oracle.run_script(lines)
        golden_io.compare_results(got, want, exact=True)
        n_cases += 1
    assert n_cases >= 30


@pytest.mark.skipif(not has_reference_build(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", range(100, 140))
def test_oracle_matches_reference_dumper(seed):
    n = 2 + seed % 9
    lines = circuits.random_script(seed, n, 50)
    with tempfile.TemporaryDirectory() as d:
        want = oracle.run_reference(lines, d)
    golden_io.compare_results(oracle.run_script(lines), want, exact=True)


def test_general_pauli_is_exact_exponential():
    """strict=0 Pauli strings (beyond the reference's subset) equal expm(i t P)."""
    from scipy.linalg import expm
    mats = {1: np.array([[0, 1], [1, 0]], complex), 2: np.array([[0, -1j], [1j, 0]]),
            3: np.diag([1.0, -1.0]).astype(complex)}
    rng = np.random.default_rng(3)
    n = 5
    for trial in range(12):
        k = int(rng.integers(1, 6))
        qs = [int(q) for q in rng.choice(n, size=k, replace=False)]
        ps = [int(p) for p in rng.integers(1, 4, size=k)]
        th = float(rng.uniform(-3, 3))
        lines = ["setup 5"] + circuits.random_state_line(rng, n)
        psi0 = np.array([float.fromhex(v) for v in lines[2].split()])
        psi0 = psi0[:32] + 1j * psi0[32:]
        lines += [f"ptpg {k} " + " ".join(map(str, qs)) + " " + " ".join(map(str, ps)) + f" {th.hex()}", "dump"]
        got = oracle.run_script(lines)[0][1]
        P = np.eye(1, dtype=complex)
        for q in reversed(range(n)):
            P = np.kron(P, mats[ps[qs.index(q)]] if q in qs else np.eye(2))
        want = expm(1j * th * P) @ psi0
        assert np.max(np.abs(got - want)) < 1e-12


def test_reference_xy_quirk_reproduced():
    """The reference's two-qubit X/Y rotation is exp(i t Y(x)X) on the same qubits."""
    rng = np.random.default_rng(5)
    lines = ["setup 3"] + circuits.random_state_line(rng, 3)
    a = oracle.run_script(lines + ["ptp 2 0 2 1 2 0x1.0p-1", "dump"])[0][1]
    b = oracle.run_script(lines + ["ptpg 2 0 2 2 1 0x1.0p-1", "dump"])[0][1]
    assert np.array_equal(a, b)


def test_pcg32_matches_reference_draws():
    import os
    path = os.path.join(golden_io.GOLDEN, "pcg32_draws.txt")
    for line in open(path):
        tok = line.split()
        g = oracle.Pcg32(int(tok[0]))
        assert [g.doub() for _ in tok[1:]] == [float.fromhex(v) for v in tok[1:]]


def test_tfim_exact_energies():
    """Exact TFIM ring spectra: h = 0 is the classical ring (ground energy -J s),
    J = 0 the free field (+-h per spin), and the 2-spin ring's ground energy is
    -sqrt(4J^2 + 4h^2) (two bonds between the same pair)."""
    import math
    from tfim_exact import spectrum, thermal_energy
    assert abs(spectrum(6, 1.0, 0.0)[0] + 6.0) < 1e-12
    w = spectrum(4, 0.0, 0.7)
    assert abs(w[0] + 2.8) < 1e-12 and abs(w[-1] - 2.8) < 1e-12
    assert abs(spectrum(2, 1.0, 0.5)[0] + math.sqrt(4.0 + 1.0)) < 1e-12
    assert abs(thermal_energy(4, 1.0, 1.0, 0.0)) < 1e-12  # traceless


def test_threaded_oracle_matches_single_thread_on_the_benchmark_circuit():
    """The threaded oracle (the CPU baseline, and the checker of the full-size
    benchmark circuit) splits every loop into contiguous index ranges.  Gate
    loops are elementwise, but a measurement's probability is summed as
    per-thread partials, so its renormalisation can differ from the single-thread
    oracle's (the reference CPU build's) in the last bits: the measured bits
    agree and the amplitudes within 1e-13 of the largest."""
    import numpy as np
    import oracle
    from suqa_gb300.workloads import random_circuit, random_state
    n = 16
    gates = random_circuit(n, 400, seed=11, measure_every=40)
    re, im = random_state(n, 11)
    L = oracle.load()
    out = []
    for threads in (1, 8):
        L.or_set_threads(threads)
        ost = oracle.OracleState(n)
        buf = np.ctypeslib.as_array(ost.p.contents.data, shape=(2 << n,))
        buf[:1 << n] = re
        buf[1 << n:] = im
        bits = oracle.apply_circuit(ost, gates)
        out.append((bits, buf.copy()))
        ost.close()
    L.or_set_threads(1)
    assert out[0][0] == out[1][0]
    a, b = out[0][1], out[1][1]
    assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(a))
