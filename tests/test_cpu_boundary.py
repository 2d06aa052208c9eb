"""CPU-side checks of the boundary: the C-ABI library exports every symbol that
include/sq.h declares, and the Python mirror binds them (no compute calls)."""
import os
import re
import ctypes

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sq_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_api():
    syms = declared_symbols("sq.h")
    for s in ["sq_state_create", "sq_apply_h", "sq_apply_pauli_rotation", "sq_measure_qbit", "sq_prob_filter",
              "sq_apply_qms_w", "sq_apply_phase_list"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    from suqa_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libsq not built")
    L = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in declared_symbols("sq.h") if not hasattr(L, s)]
    assert not missing, missing
    # the Python binding covers every declared entry point
    assert set(declared_symbols("sq.h")) <= set(_lib.EXPORTED)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from suqa_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError):
        _lib.load()


def test_batch_entry_points_reject_bad_arguments_before_any_device_call():
    """Argument checks of the batched entry points run on the host first (no
    GPU needed): out-of-range rings, a bad precision, empty lists."""
    from suqa_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libsq not built")
    L = _lib.load()
    ev = (_lib.SqTfimEvolution * 1)()
    ev[0] = _lib.SqTfimEvolution(13, 2, 1.0, 1.0, 0.1)  # 13 spins: beyond 12
    ms = ctypes.c_float()
    buf = (ctypes.c_double * 8)()
    assert L.sq_tfim_evolve_batch(ev, 1, _lib.SQ_F64, buf, ctypes.byref(ms)) == _lib.SQ_ERR_ARG
    assert b"ring length" in L.sq_last_error()
    ev[0] = _lib.SqTfimEvolution(4, 2, 1.0, 1.0, 0.0)  # dt = 0
    assert L.sq_tfim_evolve_batch(ev, 1, _lib.SQ_F64, buf, ctypes.byref(ms)) == _lib.SQ_ERR_ARG
    assert L.sq_tfim_evolve_batch(ev, 0, _lib.SQ_F64, buf, ctypes.byref(ms)) == _lib.SQ_ERR_ARG
    ch = (_lib.SqTfimChain * 1)()
    ch[0] = _lib.SqTfimChain(4, 4, 10, 0, 1, 100, 1.0, 1.0, 1.0, -8.0, 8.0, 0.1, 1)
    h = ctypes.c_void_p()
    opts = _lib.SqBatchOpts(0, 0, 0, 384, 0, 0, 0)  # 384 threads: not a supported CTA size
    assert L.sq_batch_create(ctypes.byref(h), ch, 1, _lib.SQ_F32, ctypes.byref(opts)) == _lib.SQ_ERR_ARG
    assert L.sq_batch_create(ctypes.byref(h), ch, 1, 7, None) == _lib.SQ_ERR_ARG  # unknown precision
    ch[0].spins = 21
    assert L.sq_batch_create(ctypes.byref(h), ch, 1, _lib.SQ_F32, None) == _lib.SQ_ERR_ARG
    ch[0].spins, ch[0].ene_qbits = 16, 7  # 24 qubits
    assert L.sq_batch_create(ctypes.byref(h), ch, 1, _lib.SQ_F32, None) == _lib.SQ_ERR_ARG


def test_walk_batch_rejects_bad_arguments_before_any_device_call():
    from suqa_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libsq not built")
    L = _lib.load()
    w = (_lib.SqQsaWalk * 1)()
    res = (_lib.SqQsaWalkResult * 1)()
    ms = ctypes.c_float()

    def walk(**kw):
        a = dict(spins=4, phase_qbits=3, stages=2, steps_per_stage=2, max_steps=0, beta=1.0, seed=1)
        a.update(kw)
        J = kw.get("J", [1] * 12)
        return _lib.SqQsaWalk(a["spins"], a["phase_qbits"], a["stages"], a["steps_per_stage"], a["max_steps"],
                              (ctypes.c_int32 * 12)(*J), kw.get("algo", 0), a["beta"], a["seed"])

    for bad, msg in ((dict(spins=13), b"ring length"), (dict(spins=1), b"ring length"),
                     (dict(phase_qbits=7), b"walk-phase"), (dict(phase_qbits=0), b"walk-phase"),
                     (dict(stages=0), b"schedule"), (dict(beta=-1.0), b"beta"),
                     (dict(J=[9] + [1] * 11), b"couplings"), (dict(algo=3), b"algorithm")):
        w[0] = walk(**bad)
        assert L.sq_qsa_walk_batch(w, 1, _lib.SQ_F32, res, None, ctypes.byref(ms)) == _lib.SQ_ERR_ARG, bad
        assert msg in L.sq_last_error(), (bad, L.sq_last_error())
    w[0] = walk()
    assert L.sq_qsa_walk_batch(w, 0, _lib.SQ_F32, res, None, ctypes.byref(ms)) == _lib.SQ_ERR_ARG
    assert L.sq_qsa_walk_batch(w, 1, 7, res, None, ctypes.byref(ms)) == _lib.SQ_ERR_ARG


def test_walk_pass_switches_validate_their_arguments():
    """The process-wide switches of the FP32 orbit pass (warps per CTA, the orbit
    order table, tensor-core products) accept their documented values and refuse
    others on the host, with no device call."""
    from suqa_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libsq not built")
    L = _lib.load()
    try:
        for fn, good, bad in ((L.sq_set_walk_orbit_warps, (8, 16), (0, 4, 32)),
                              (L.sq_set_walk_presort, (0, 1), (-1, 2)),
                              (L.sq_set_walk_mma, (0, 1), (-1, 2))):
            for v in good:
                assert fn(v) == _lib.SQ_OK, (fn, v)
            for v in bad:
                assert fn(v) == _lib.SQ_ERR_ARG, (fn, v)
    finally:
        L.sq_set_walk_orbit_warps(16)
        L.sq_set_walk_presort(1)
        L.sq_set_walk_mma(1)
