"""Gate-engine parity on the GPU (libsq through the suqa:: mirror) against the
committed reference fixtures and the CPU oracle.  FP64 tolerance: 1e-12 of the
state's largest amplitude per amplitude; measured bits identical."""
import math

import numpy as np
import pytest

import circuits
import golden_io
import gpu_script
import oracle

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12
RTOL32 = 2e-5


@pytest.mark.parametrize("fusion", [True, False])
def test_golden_fixtures_fp64(fusion):
    worst = 0.0
    n = 0
    for name, lines, want in golden_io.gate_cases():
        got = gpu_script.run_script(lines, "f64", fusion)
        worst = max(worst, golden_io.compare_results(got, want, rtol=RTOL64))
        n += 1
    assert n >= 30
    print("worst relative amplitude error", worst)


@pytest.mark.parametrize("seed", range(20))
def test_random_scripts_vs_oracle_fp64(seed):
    n = [3, 5, 8, 11, 12, 13, 14, 15, 16, 17][seed % 10]
    lines = circuits.random_script(1000 + seed, n, 70, reference_only=False, random_init=n <= 12,
                                   dump_every=10 if n <= 12 else 35)
    want = oracle.run_script(lines)
    got = gpu_script.run_script(lines, "f64")
    golden_io.compare_results(got, want, rtol=RTOL64)


@pytest.mark.parametrize("seed", range(10))
def test_random_scripts_vs_oracle_double_float(seed):
    """FP64 states with the double-float arithmetic option: multi-tile passes
    compute in hi + lo FP32 pairs (48 significand bits); the FP64 bar holds."""
    n = [13, 14, 15, 16, 17][seed % 5]
    lines = circuits.random_script(1300 + seed, n, 70, reference_only=False, random_init=False,
                                   dump_every=35)
    want = oracle.run_script(lines)
    got = gpu_script.run_script(lines, "f64", dfloat=True)
    golden_io.compare_results(got, want, rtol=RTOL64)


@pytest.mark.parametrize("n", [18, 20, 22])
def test_large_random_vs_oracle_fp64(n):
    lines = circuits.random_script(77 + n, n, 40, reference_only=False, random_init=False,
                                   dump_every=0, measure_every=9)
    want = oracle.run_script(lines, threads=8)
    got = gpu_script.run_script(lines, "f64")
    golden_io.compare_results(got, want, rtol=RTOL64)


@pytest.mark.parametrize("n", [4, 10, 14, 18])
def test_fp32_vs_oracle(n):
    # no projective measurement: an FP32 rounding can legitimately flip a draw
    lines = circuits.random_script(500 + n, n, 60, reference_only=False, random_init=n <= 10,
                                   measure_every=0, dump_every=15)
    lines += ["prob 2 0 1 1 0", "vnorm", "dump"]
    want = oracle.run_script(lines)
    got = gpu_script.run_script(lines, "f32")
    golden_io.compare_results(got, want, rtol=RTOL32)


def test_fp32_measurement_far_from_threshold():
    lines = ["setup 12"] + [f"h {q}" for q in range(12)] + [f"u1 {q} {circuits.hx(0.3 * q)}" for q in range(12)]
    lines += ["measure 3 0x1.0p-3", "measure 7 0x1.cp-1", "dump", "vnorm"]
    golden_io.compare_results(gpu_script.run_script(lines, "f32"), oracle.run_script(lines), rtol=RTOL32)


def test_qms_w_vs_oracle():
    from suqa_gb300 import State
    rng = np.random.default_rng(9)
    for n, ene in [(8, 4), (10, 6), (15, 5)]:
        N = 1 << n
        a = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        a /= np.linalg.norm(a)
        o = oracle.OracleState(n)
        o.set_array(a)
        mask = ((1 << ene) - 1) << 3
        for e_old, cf in [(0, 0.7), (5, 1.3), ((1 << ene) - 1, 0.05)]:
            oracle.load().or_apply_qms_w(o.p, n - 1, mask, 3, e_old, cf)
        with State(n) as s:
            s.set_state(a)
            for e_old, cf in [(0, 0.7), (5, 1.3), ((1 << ene) - 1, 0.05)]:
                s.apply_qms_w(n - 1, mask, 3, e_old, cf)
            got = s.get_state()
        want = o.array()
        assert np.max(np.abs(got - want)) <= RTOL64 * np.max(np.abs(want))


def test_errors_and_edge_cases():
    from suqa_gb300 import SqError, SqUnsupported, State
    with State(4) as s:
        with pytest.raises(SqError):
            s.apply_x(4)
        s.apply_h([0, 1, 2, 3])
        s.activate_gc_mask([1])
        s.apply_h(1)  # target inside the global control mask: the reference zeroes that subspace
        s.deactivate_gc_mask([1])
        st = s.get_state()
        assert np.all(st[[i for i in range(16) if i & 2]] == 0)
        s.init_state()
        with pytest.raises(SqUnsupported):
            s.apply_pauli_TP_rotation([0, 1, 2], [1, 2, 3], 0.3)
        with pytest.raises(RuntimeError):
            s.apply_phase_list(0, 2, [0.1, 0.2, 0.3])
        before = s.get_state()
        s.apply_phase_list(0, 2, [0.1, 0.2, 0.3, 0.4])  # gc == 0: reference no-op
        assert np.array_equal(s.get_state(), before)
        assert abs(s.vnorm() - 1.0) < 1e-15
    for n in (1, 2):
        for prec in ("f64", "f32"):
            with State(n, prec) as s:
                s.apply_h(0)
                s.apply_pauli_rotation([0], [2], 0.4)
                st = s.get_state()
                assert abs(np.linalg.norm(st) - 1.0) < 1e-6


def test_wide_pauli_strings_cross_tiles():
    """Pauli strings with 6-11 flipped qubits spread over a 20-qubit state."""
    rng = np.random.default_rng(21)
    lines = ["setup 20"] + [f"h {q}" for q in range(20)] + [f"u1 {q} {circuits.hx(0.1 * q + 0.05)}" for q in range(20)]
    for k in (6, 8, 11):
        qs = [int(q) for q in rng.choice(20, size=k, replace=False)]
        ps = [int(p) for p in rng.integers(1, 3, size=k)]
        lines.append(f"ptpg {k} " + " ".join(map(str, qs)) + " " + " ".join(map(str, ps)) + f" {circuits.hx(0.37 * k)}")
        lines.append("dump")
    golden_io.compare_results(gpu_script.run_script(lines), oracle.run_script(lines, threads=8), rtol=RTOL64)


def test_fusion_counts_fewer_passes():
    from suqa_gb300 import State
    with State(22) as s:
        rng = np.random.default_rng(1)
        for _ in range(200):
            s.apply_h(int(rng.integers(0, 22)))
        s.synchronize()
        st = s.stats()
    assert st["gates"] == 200
    assert st["passes"] < 60


@pytest.mark.parametrize("seed", range(12))
def test_overlapping_global_control_vs_oracle(seed):
    """Gates acting on qubits of the global control mask follow the reference
    loops' semantics (the oracle restates them literally)."""
    n = 4 + seed % 9
    lines = circuits.random_script(2000 + seed, n, 80, overlap="engine", dump_every=8)
    golden_io.compare_results(gpu_script.run_script(lines), oracle.run_script(lines), rtol=RTOL64)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_tile_size_does_not_change_results(precision):
    """The fused-pass tile size is a tuning knob: the same circuit at several
    tile sizes gives the same measured bits and amplitudes to rounding."""
    from suqa_gb300 import State
    from suqa_gb300.workloads import apply_circuit, random_circuit
    n = 16
    gates = random_circuit(n, 200, seed=11, measure_every=50)
    results = []
    for k in (0, 8, 10, 12):
        with State(n, precision) as st:
            st.set_tile_qubits(k)
            st.apply_h(list(range(n)))
            bits = apply_circuit(st, gates)
            results.append((bits, st.get_state()))
    tol = 1e-12 if precision == "f64" else 2e-5
    for bits, amp in results[1:]:
        assert bits == results[0][0]
        assert np.max(np.abs(amp - results[0][1])) < tol
    with State(n, precision) as st:
        with pytest.raises(Exception):
            st.set_tile_qubits(3)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n,k", [(16, 10), (18, 12), (21, 0), (23, 11)])
def test_bulk_staging_is_bit_identical_to_register_staging(precision, n, k):
    """Multi-tile passes move tiles by bulk asynchronous copies (runs of 2^L
    amplitudes, completion on an mbarrier) or through registers; the arithmetic
    is the same, so the measured bits and every amplitude must be identical
    (modes 0 and 1).
    The circuits hold X gates on low and high qubits (index frames with and
    without a part below L), controlled gates and measurements."""
    from suqa_gb300 import State
    from suqa_gb300.workloads import apply_circuit, random_circuit
    gates = random_circuit(n, 160, seed=40 + n, measure_every=40)
    results = []
    for mode in (0, 1, 2):
        with State(n, precision) as st:
            st.set_tile_qubits(k)
            st.set_staging(mode)
            st.apply_h(list(range(n)))
            bits = apply_circuit(st, gates)
            st.synchronize()
            results.append((bits, st.get_state()))
    assert results[0][0] == results[1][0]
    assert np.array_equal(results[0][1], results[1][1])
    # double-buffered staging uses its own tile size (2^12 FP32, 2^11 FP64): the same
    # results to rounding
    tol = 1e-12 if precision == "f64" else 2e-5
    assert results[2][0] == results[0][0]
    assert np.max(np.abs(results[2][1] - results[0][1])) <= tol * np.max(np.abs(results[0][1]))


def test_fp64_fma_rate_probe_reports_a_rate():
    """The benchmark's FP64 FMA-rate probe (libsq_probe.so, the tile pass's
    ceiling in bench.py) runs and gives a plausible rate: more than 50 G
    instructions/s, less than the nominal SM count x clock x 2 per SM per cycle
    bound with room (1 T/s)."""
    import ctypes
    import os
    from suqa_gb300 import _lib
    lib = ctypes.CDLL(os.path.join(os.path.dirname(_lib.LIB_PATH), "libsq_probe.so"))
    lib.sqb_fp64_fma_rate.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)]
    g = ctypes.c_double()
    ms = ctypes.c_float()
    assert lib.sqb_fp64_fma_rate(ctypes.byref(g), ctypes.byref(ms)) == 0
    assert 50.0 < g.value < 1000.0 and ms.value > 0
