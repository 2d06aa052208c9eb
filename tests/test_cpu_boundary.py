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
