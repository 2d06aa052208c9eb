"""Dense k-qubit blocks (OP_DENSE): sq_apply_unitary against a numpy
application of the same matrix, on the tensor-core path (FP32 states with tiles
of 2^12 amplitudes or more: tcgen05, TF32 high/remainder split, four products) and the CUDA-core
path (FP64 states, small FP32 states), with global controls inside and outside
the tile; and automatic fusion of gate runs on at most five qubits against the
CPU oracle, which applies the same gates one by one.  FP32 tolerance 2e-5 of
the largest amplitude (the FP32 bar of the other tests), FP64 1e-12."""
import numpy as np
import pytest

import circuits
import golden_io
import gpu_script
import oracle

pytestmark = pytest.mark.gpu


def _apply_ref(psi, n, qubits, U, gc=0):
    """U on qubits (index bit b <-> qubits[b]) where every bit of gc is set."""
    k = len(qubits)
    t = psi.reshape([2] * n)  # tensor axis a <-> qubit n-1-a
    axes = [n - 1 - q for q in qubits]
    Ut = U.reshape([2] * (2 * k))  # (out bit k-1 .. 0, in bit k-1 .. 0)
    res = np.tensordot(Ut, t, axes=([k + (k - 1 - b) for b in range(k)], axes))
    res = np.moveaxis(res, [k - 1 - b for b in range(k)], axes).reshape(-1)
    if gc:
        idx = np.arange(1 << n)
        res = np.where((idx & gc) == gc, res, psi)
    return res


def _random_unitary(k, rng):
    z = rng.standard_normal((1 << k, 1 << k)) + 1j * rng.standard_normal((1 << k, 1 << k))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _random_state(n, rng):
    a = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return a / np.linalg.norm(a)


@pytest.mark.parametrize("precision,n,engine", [("f32", 14, 0), ("f32", 12, 0), ("f32", 17, 0), ("f32", 14, 1),
                                                ("f32", 8, 0), ("f64", 14, 0), ("f64", 9, 0)])
def test_apply_unitary_matches_numpy(precision, n, engine):
    from suqa_gb300 import State
    rng = np.random.default_rng(100 + n + engine)
    psi = _random_state(n, rng)
    want = psi.copy()
    cases = []
    for k in (5, 3, 1, 4, 2, 5):
        qs = [int(q) for q in rng.choice(n, size=k, replace=False)]
        cases.append((qs, _random_unitary(k, rng), 0))
    # global controls: one low qubit (inside every tile) and one high qubit
    free = [q for q in range(n) if q not in cases[-1][0]]
    gc_q = [free[0], free[-1]]
    cases.append(([q for q in range(n) if q not in gc_q][:5], _random_unitary(5, rng),
                  sum(1 << q for q in gc_q)))
    with State(n, precision) as st:
        st.set_dense_engine(engine)
        st.set_state(psi)
        for qs, U, gc in cases:
            if gc:
                st.activate_gc_mask([q for q in range(n) if gc >> q & 1])
            st.apply_unitary(qs, U)
            if gc:
                st.deactivate_gc_mask([q for q in range(n) if gc >> q & 1])
            want = _apply_ref(want, n, qs, U, gc)
        got = st.get_state()
    tol = 2e-5 if precision == "f32" else 1e-12
    err = float(np.max(np.abs(got - want)) / np.max(np.abs(want)))
    print(f"\n{precision} n={n} engine={engine}: max error / max amplitude {err:.2e}")
    assert err <= tol


def test_tensor_and_cuda_core_engines_agree():
    """The same dense blocks on both engines of an FP32 state: the TF32
    high/remainder split on the tensor cores against FP64 arithmetic rounded to
    FP32 (12 blocks; the FP32 bar of the other tests)."""
    from suqa_gb300 import State
    rng = np.random.default_rng(5)
    n = 16
    psi = _random_state(n, rng)
    out = []
    blocks = [([int(q) for q in rng.choice(n, size=5, replace=False)], _random_unitary(5, rng)) for _ in range(12)]
    for engine in (0, 1):
        with State(n, "f32") as st:
            st.set_dense_engine(engine)
            st.set_state(psi)
            for qs, U in blocks:
                st.apply_unitary(qs, U)
            out.append(st.get_state())
    err = float(np.max(np.abs(out[0] - out[1])) / np.max(np.abs(out[1])))
    print(f"\ntensor vs CUDA cores after 12 blocks: {err:.2e} of the largest amplitude")
    assert err <= 2e-5


@pytest.mark.parametrize("n", [13, 16, 20])
def test_dense_fusion_matches_the_oracle(n):
    """FP32 with automatic dense blocks (runs of >= 2 gates on <= 5 qubits) on
    random scripts with QFTs on small registers: the oracle applies the gates one
    by one."""
    lines = circuits.random_script(700 + n, n, 80, reference_only=False, random_init=False, measure_every=0,
                                   dump_every=20)
    rng = np.random.default_rng(n)
    for _ in range(3):
        reg = sorted(int(q) for q in rng.choice(n, size=5, replace=False))
        lines.append("qft " + " ".join(str(q) for q in [len(reg)] + reg))
        lines.append("iqft " + " ".join(str(q) for q in [len(reg)] + reg[::-1]))
    lines += ["prob 2 0 1 1 0", "vnorm", "dump"]
    want = oracle.run_script(lines)
    got = gpu_script.run_script(lines, "f32", dense_fusion=2)
    golden_io.compare_results(got, want, rtol=2e-5)


def test_dense_fusion_counts_fewer_sweeps_on_a_qft():
    """A QFT on five qubits (5 H + 10 controlled phases) becomes one dense block."""
    from suqa_gb300 import State
    n = 16
    with State(n, "f32") as st:
        st.set_dense_fusion(4)
        st.apply_h(list(range(n)))
        st.flush()
        st.reset_stats()
        st.apply_qft([3, 5, 8, 11, 14])
        st.flush()
        fused = st.stats()
    assert fused["passes"] == 1
