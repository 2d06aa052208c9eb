"""suqa_gb300: GB300 (sm_103a) state-vector engine with SUQA's gate API.

The compute path is libsq (include/sq.h), hand-written CUDA kernels loaded
through ctypes; there is no CPU fallback.  `State` mirrors the reference's
suqa:: functions on one state; `suqa` mirrors the namespace-level singleton
(suqa::setup / suqa::apply_x / ...).
"""
from ._lib import SqError, SqUnsupported  # noqa: F401
from .state import PAULI_ID, PAULI_X, PAULI_Y, PAULI_Z, TWOSQINV, State  # noqa: F401

__all__ = ["State", "SqError", "SqUnsupported", "PAULI_ID", "PAULI_X", "PAULI_Y", "PAULI_Z", "TWOSQINV"]
