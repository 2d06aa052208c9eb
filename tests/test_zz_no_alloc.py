"""The allocation-free entry point sq_qubit_probs_noalloc (include/sq.h).

It serves callers that must not allocate device memory on the call path; its
scratch is a static device array instead of per-state buffers.  Called here
through the C ABI on a state owned by libsq's regular API, on two calls in a
row, and compared with the regular entry point sq_prob_filter (same 1e-12
tolerance as the other FP64 parity tests).  This file is collected last so a
failure here does not hide any other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_noalloc_probs_match_prob_filter(precision):
    import torch
    from suqa_gb300 import State, _lib

    L = _lib.load()
    n = 20
    rng = np.random.default_rng(4)
    with State(n, precision) as st:
        st.apply_h(list(range(n)))
        for _ in range(40):
            q = int(rng.integers(n))
            st.apply_u1(q, float(rng.uniform(0, 6.28)))
            st.apply_pauli_rotation([q, (q + 5) % n], [1, 2], float(rng.uniform(0, 6.28)))
        re_ptr, im_ptr = st.device_ptrs()  # applies queued gates
        st.synchronize()
        # the caller owns the output buffer; the entry point allocates nothing
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream()
        code = _lib.SQ_F64 if precision == "f64" else _lib.SQ_F32
        for q in (3, 17):  # two calls in a row share the static scratch
            rc = L.sq_qubit_probs_noalloc(ctypes.c_void_p(re_ptr), ctypes.c_void_p(im_ptr), n, code, q,
                                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, L.sq_last_error()
            stream.synchronize()
            p0, p1 = (float(x) for x in out.cpu())
            want1 = st.prob_filter([q], [1])
            want0 = st.prob_filter([q], [0])
            assert abs(p1 - want1) <= TOL * max(1.0, want1), (p1, want1)
            assert abs(p0 - want0) <= TOL * max(1.0, want0), (p0, want0)
            assert abs(p0 + p1 - 1.0) < 1e-6


def test_noalloc_rejects_bad_sizes():
    from suqa_gb300 import _lib
    L = _lib.load()
    rc = L.sq_qubit_probs_noalloc(ctypes.c_void_p(1), ctypes.c_void_p(1), 40, _lib.SQ_F64, 0,
                                  ctypes.c_void_p(1), None)
    assert rc == _lib.SQ_ERR_ARG
    assert "1..33" in L.sq_last_error().decode()
