"""Namespace-level mirror of the reference's suqa:: API (include/suqa.cuh:94-176):
one global state, set up with setup(nq) and freed with clear(), exactly as the
reference drivers use it (src/qms.cu:105, :159)."""
from __future__ import annotations

from .state import PAULI_ID, PAULI_X, PAULI_Y, PAULI_Z, TWOSQINV, State  # noqa: F401

state: State | None = None
nq = 0


def setup(num_qubits: int, precision: str = "f64"):
    global state, nq
    clear()
    nq = int(num_qubits)
    state = State(nq, precision)


def clear():
    global state
    if state is not None:
        state.close()
    state = None


def __getattr__(name):
    # suqa::apply_x, suqa::measure_qbit, ... forward to the global state
    if state is not None and hasattr(state, name):
        return getattr(state, name)
    raise AttributeError(name)
