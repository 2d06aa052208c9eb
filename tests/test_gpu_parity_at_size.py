"""Parity at the benchmark's own size: the gate-engine microbenchmark circuit
(1000 random gates, a measurement every 100; seed 7) on a 28-qubit FP64 state,
and once on 30 qubits, through libsq on the GPU and through the CPU oracle
(threaded: its gate loops are the single-thread oracle's element for element,
its measurement sums are per-thread partials, within 1e-13 of the single-thread
oracle, which is bit-identical to the reference CPU build).

Checked: identical measured bits, and the amplitude error both normwise
(||a - b|| / ||b||) and elementwise relative (|a_i - b_i| / |b_i|).  The
elementwise bar is 1e-12 on every amplitude whose magnitude is at least 1e-4 of
the state's root-mean-square amplitude; below that, an amplitude is the small
remainder of a cancellation and its relative error says nothing about the
engine (the two sides round the same sums in different orders).  The test prints
the figures, including the largest relative error over all amplitudes."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _host_bytes_available():
    try:
        return os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError):
        return 0


@pytest.mark.parametrize("n", [28, 30])
def test_benchmark_circuit_at_full_size_matches_the_oracle(n):
    import oracle
    from suqa_gb300 import State
    from suqa_gb300.workloads import apply_circuit, random_circuit, random_state

    N = 1 << n
    # initial state, oracle state, GPU result: three complex FP64 copies, plus slack
    if _host_bytes_available() < 4 * 16 * N:
        pytest.skip(f"not enough host memory for a {n}-qubit comparison")
    gates = random_circuit(n, 1000, seed=7)
    re, im = random_state(n, 7)

    with State(n, "f64") as st:
        st.upload(re.ctypes.data, im.ctypes.data)
        st.synchronize()
        bits_gpu = apply_circuit(st, gates)
        gre = np.empty(N)
        gim = np.empty(N)
        st.download(gre.ctypes.data, gim.ctypes.data)

    L = oracle.load()
    L.or_set_threads(os.cpu_count() or 1)
    ost = oracle.OracleState(n)
    buf = np.ctypeslib.as_array(ost.p.contents.data, shape=(2 * N,))
    buf[:N] = re
    buf[N:] = im
    del re, im
    bits_ref = oracle.apply_circuit(ost, gates)
    L.or_set_threads(1)
    assert bits_gpu == bits_ref

    ore, oim = buf[:N], buf[N:]
    dre = gre - ore
    dim = gim - oim
    err2 = dre * dre + dim * dim
    del dre, dim, gre, gim
    ref2 = ore * ore + oim * oim
    normwise = float(np.sqrt(err2.sum() / ref2.sum()))
    rms2 = float(ref2.mean())
    sig = ref2 >= (1e-4) ** 2 * rms2
    rel_sig = float(np.sqrt(np.max(err2[sig] / ref2[sig])))
    nz = ref2 > 0
    rel_all = float(np.sqrt(np.max(err2[nz] / ref2[nz])))
    max_abs = float(np.sqrt(err2.max() / ref2.max()))
    print(f"\nn={n}: bits {len(bits_gpu)} identical; normwise {normwise:.3e}; max |a-b| / max |b| {max_abs:.3e}; "
          f"elementwise relative {rel_sig:.3e} over {int(sig.sum())} of {N} amplitudes (|b| >= 1e-4 rms), "
          f"{rel_all:.3e} over all nonzero")
    ost.close()
    assert normwise <= TOL
    assert max_abs <= TOL
    assert rel_sig <= TOL
