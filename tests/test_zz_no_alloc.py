"""The allocation-free entry point sq_qubit_probs_noalloc (include/sq.h).

It serves callers that must not allocate device memory on the call path; its
scratch is a static device array instead of per-state buffers.  Called here
through the C ABI on a state owned by libsq's regular API, on two calls in a
row, and compared with the regular entry point sq_prob_filter (same 1e-12
tolerance as the other FP64 parity tests), over single-tile sizes (one CTA,
scalar loads for the narrowest FP32 state) and multi-tile sizes.  After the
one-time set-up of the first call, the device's free memory must not change
across calls.  This file is collected last so a failure here does not hide any
other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32": 1e-12}


def _prepare(st, n, rng):
    st.apply_h(list(range(n)))
    for _ in range(4 * n):
        q = int(rng.integers(n))
        st.apply_u1(q, float(rng.uniform(0, 6.28)))
        if n > 1:
            st.apply_pauli_rotation([q, (q + 1 + int(rng.integers(n - 1))) % n], [1, 2], float(rng.uniform(0, 6.28)))
        else:
            st.apply_pauli_rotation([q], [2], float(rng.uniform(0, 6.28)))


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", [1, 2, 5, 10, 11, 20])
def test_noalloc_probs_match_prob_filter(precision, n):
    import torch
    from suqa_gb300 import State, _lib

    L = _lib.load()
    rng = np.random.default_rng(4 + n)
    with State(n, precision) as st:
        _prepare(st, n, rng)
        re_ptr, im_ptr = st.device_ptrs()  # applies queued gates
        st.synchronize()
        # the caller owns the output buffer; the entry point allocates nothing
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream()
        code = _lib.SQ_F64 if precision == "f64" else _lib.SQ_F32

        def call(q):
            rc = L.sq_qubit_probs_noalloc(ctypes.c_void_p(re_ptr), ctypes.c_void_p(im_ptr), n, code, q,
                                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, L.sq_last_error()
            stream.synchronize()
            return [float(x) for x in out.cpu()]

        call(0)  # the first call on a device may do the one-time set-up
        free_before = torch.cuda.mem_get_info()[0]
        qs = sorted({0, n - 1})
        for q in qs + qs:  # calls in a row share the static scratch
            p0, p1 = call(q)
            want1 = st.prob_filter([q], [1])
            want0 = st.prob_filter([q], [0])
            assert abs(p1 - want1) <= TOL[precision] * max(1.0, want1), (n, q, p1, want1)
            assert abs(p0 - want0) <= TOL[precision] * max(1.0, want0), (n, q, p0, want0)
            assert abs(p0 + p1 - 1.0) < 1e-6
        assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_rejects_bad_sizes_and_misaligned_pointers():
    import torch
    from suqa_gb300 import _lib
    L = _lib.load()
    rc = L.sq_qubit_probs_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 40, _lib.SQ_F64, 0,
                                  ctypes.c_void_p(16), None)
    assert rc == _lib.SQ_ERR_ARG
    assert "1..33" in L.sq_last_error().decode()
    # a view one element into a buffer: 8-byte aligned, not 16; refused on the host
    buf = torch.zeros(2 * (1 << 12) + 2, dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    base = buf.data_ptr()
    assert base % 16 == 0
    rc = L.sq_qubit_probs_noalloc(ctypes.c_void_p(base + 8), ctypes.c_void_p(base + 8 + 8 * (1 << 12)), 12,
                                  _lib.SQ_F64, 3, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.SQ_ERR_ARG
    assert "aligned" in L.sq_last_error().decode()
    rc = L.sq_qubit_probs_noalloc(ctypes.c_void_p(base), ctypes.c_void_p(base + 8 * (1 << 12)), 12,
                                  _lib.SQ_F64, 3, ctypes.c_void_p(out.data_ptr() + 4), None)
    assert rc == _lib.SQ_ERR_ARG
    torch.cuda.synchronize()
    assert float(out.abs().sum()) == 0.0  # nothing ran
