"""Parity at the benchmark's own size: the gate-engine microbenchmark circuit
(1000 random gates, a measurement every 100; seed 7) on a 28-qubit FP64 state,
and once on 30 qubits, through libsq on the GPU and through the CPU oracle
(threaded: its gate loops are the single-thread oracle's element for element,
its measurement sums are per-thread partials, within 1e-13 of the single-thread
oracle, which is bit-identical to the reference CPU build).

Checked: identical measured bits, and the amplitude error normwise
(||a - b|| / ||b|| <= 1e-13), against the largest amplitude (<= 1e-13) and
elementwise relative (|a_i - b_i| / |b_i|): at least 99 % of the nonzero
amplitudes within 1e-12.  The rest are small remainders of cancellations, whose
relative error no FP64 evaluation order controls (an absolute error of 1e-14 of
the largest amplitude is a large fraction of an amplitude near zero); the test
prints the magnitude, as a fraction of the root-mean-square amplitude, above
which every amplitude is within 1e-12, and the worst relative error."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_NORM = 1e-13
TOL_REL = 1e-12
TOL_NORM_DF = 1e-12  # double-float arithmetic: 48 significand bits per operation


def _host_bytes_available():
    try:
        return os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError):
        return 0


@pytest.mark.parametrize("n,dfloat", [(28, False), (30, False), (28, True)])
def test_benchmark_circuit_at_full_size_matches_the_oracle(n, dfloat):
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
        st.set_double_float(dfloat)
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
    max_abs = float(np.sqrt(err2.max() / ref2.max()))
    nz = ref2 > 0
    rel2 = err2[nz] / ref2[nz]
    within = float(np.mean(rel2 <= TOL_REL ** 2))
    rms = float(np.sqrt(ref2.mean()))
    bad = ref2[nz][rel2 > TOL_REL ** 2]
    threshold = float(np.sqrt(bad.max()) / rms) if bad.size else 0.0
    worst = float(np.sqrt(rel2.max()))
    print(f"\nn={n}{' double-float' if dfloat else ''}: {len(bits_gpu)} measured bits identical; normwise {normwise:.3e}; max |a-b| / max |b| "
          f"{max_abs:.3e}; {100 * within:.4f} % of {int(nz.sum())} nonzero amplitudes within {TOL_REL:g} relative; "
          f"all amplitudes above {threshold:.3e} x rms within it; worst relative {worst:.3e}")
    ost.close()
    tol = TOL_NORM_DF if dfloat else TOL_NORM
    assert normwise <= tol
    assert max_abs <= tol
    if not dfloat:
        assert within >= 0.99
