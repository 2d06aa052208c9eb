"""Python host mirror of the reference's suqa:: gate API (include/suqa.cuh:94-176).

A State owns one device state vector in libsq plus the reference's global
control mask (suqa::gc_mask, src/suqa.cu:36).  Method names, argument meaning,
overloads and error behaviour follow the reference: invalid Pauli patterns in
apply_pauli_TP_rotation raise (the reference throws std::runtime_error,
src/suqa.cu:477-579), apply_phase_list raises on a bad size
(src/suqa.cu:420-422).  Every method runs on the GPU through libsq.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import SQ_F32, SQ_F64, SQ_PAULI_EXACT, SQ_PAULI_REFERENCE, check

PAULI_ID, PAULI_X, PAULI_Y, PAULI_Z = 0, 1, 2, 3
TWOSQINV = 0.7071067811865475


def _u32(xs):
    xs = list(xs)
    return (C.c_uint32 * len(xs))(*xs)


class State:
    """A 2^n-amplitude state (FP64 by default, or FP32 amplitudes with FP64
    reductions) in the split re/im layout of the reference ComplexVec."""

    def __init__(self, nq: int, precision: str = "f64"):
        self.L = _lib.load()
        self.nq = int(nq)
        self.precision = precision
        prec = SQ_F64 if precision in ("f64", "fp64", "double") else SQ_F32
        h = C.c_void_p()
        check(self.L.sq_state_create(C.byref(h), self.nq, prec))
        self.h = h
        self.gc_mask = 0
        self.rphase_m: list[float] = []

    # -- lifecycle ---------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.sq_state_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def size(self) -> int:
        return 1 << self.nq

    # -- suqa:: state utilities (src/suqa.cu:45-111) -------------------------------
    def activate_gc_mask(self, q_controls: Iterable[int]):
        for q in q_controls:
            self.gc_mask |= 1 << int(q)

    def deactivate_gc_mask(self, q_controls: Iterable[int]):
        for q in q_controls:
            self.gc_mask &= ~(1 << int(q))

    def init_state(self):
        check(self.L.sq_init_state(self.h))

    def vnorm(self) -> float:
        out = C.c_double()
        check(self.L.sq_vnorm(self.h, C.byref(out)))
        return out.value

    def vnormalize(self):
        check(self.L.sq_vnormalize(self.h))

    def flush(self):
        check(self.L.sq_flush(self.h))

    def synchronize(self):
        check(self.L.sq_synchronize(self.h))

    def set_fusion(self, enabled: bool):
        check(self.L.sq_set_fusion(self.h, 1 if enabled else 0))

    def set_tile_qubits(self, k: int):
        """Tile size of the fused passes (0: default)."""
        check(self.L.sq_set_tile_qubits(self.h, k))

    def apply_unitary(self, qubits, u):
        """A 2^k x 2^k complex matrix on qubits (index bit b <-> qubits[b]), k <= 5,
        under the current global control mask."""
        u = np.asarray(u, dtype=np.complex128)
        k = len(qubits)
        if u.shape != (1 << k, 1 << k):
            raise ValueError("matrix shape does not match the qubit count")
        re = np.ascontiguousarray(u.real)
        im = np.ascontiguousarray(u.imag)
        qs = (C.c_uint32 * k)(*qubits)
        check(self.L.sq_apply_unitary(self.h, k, qs, re.ctypes.data_as(C.POINTER(C.c_double)),
                                      im.ctypes.data_as(C.POINTER(C.c_double)), self.gc_mask))

    def set_double_float(self, enabled: bool):
        """FP64 states: arithmetic of multi-tile passes in double-float on the FP32 pipe."""
        check(self.L.sq_set_double_float(self.h, 1 if enabled else 0))

    def set_dense_fusion(self, min_gates: int):
        """FP32: fuse runs of >= min_gates gates on <= 5 qubits into dense blocks (0 off)."""
        check(self.L.sq_set_dense_fusion(self.h, min_gates))

    def set_dense_engine(self, engine: int):
        """Dense blocks on the tensor cores (0, default) or the CUDA cores (1)."""
        check(self.L.sq_set_dense_engine(self.h, engine))

    def set_staging(self, mode: int):
        """Tile staging of multi-tile passes: 0 vector loads and stores through
        registers (default), 1 bulk asynchronous copies, 2 bulk copies
        double-buffered."""
        check(self.L.sq_set_staging(self.h, mode))

    def get_state(self) -> np.ndarray:
        N = self.size()
        re = np.empty(N, dtype=np.float64)
        im = np.empty(N, dtype=np.float64)
        check(self.L.sq_get_state(self.h, re.ctypes.data_as(C.c_void_p), im.ctypes.data_as(C.c_void_p)))
        return re + 1j * im

    def set_state(self, a: np.ndarray):
        a = np.asarray(a, dtype=np.complex128)
        if a.shape != (self.size(),):
            raise ValueError("state has the wrong length")
        re = np.ascontiguousarray(a.real)
        im = np.ascontiguousarray(a.imag)
        check(self.L.sq_set_state(self.h, re.ctypes.data_as(C.c_void_p), im.ctypes.data_as(C.c_void_p)))

    def upload(self, re_ptr: int, im_ptr: int):
        """Copy host buffers (state element type, ideally page-locked) into the state."""
        check(self.L.sq_upload(self.h, C.c_void_p(re_ptr), C.c_void_p(im_ptr)))

    def download(self, re_ptr: int, im_ptr: int):
        check(self.L.sq_download(self.h, C.c_void_p(re_ptr), C.c_void_p(im_ptr)))

    def device_ptrs(self):
        re, im = C.c_void_p(), C.c_void_p()
        check(self.L.sq_state_ptrs(self.h, C.byref(re), C.byref(im)))
        return re.value, im.value

    def stats(self) -> dict:
        st = _lib.SqStats()
        check(self.L.sq_get_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def reset_stats(self):
        check(self.L.sq_reset_stats(self.h))

    def set_timing(self, enabled: bool):
        check(self.L.sq_set_timing(self.h, 1 if enabled else 0))

    def kernel_time(self):
        """(device ms, launches, bytes moved) of the passes since the last call."""
        ms, n, b = C.c_double(), C.c_uint64(), C.c_uint64()
        check(self.L.sq_kernel_time(self.h, C.byref(ms), C.byref(n), C.byref(b)))
        return ms.value, n.value, b.value

    def set_stream(self, cuda_stream: int | None):
        """Run on a caller's CUDA stream, e.g. torch.cuda.Stream().cuda_stream.  A handle
        of 0 or None (also what the legacy default stream reports) selects the state's
        own non-blocking stream, which does not order with the default stream."""
        check(self.L.sq_set_stream(self.h, C.c_void_p(cuda_stream) if cuda_stream else None))

    # -- single-qubit gates (src/suqa.cu:115-285) ------------------------------------
    def _each(self, qs, fn):
        if isinstance(qs, (list, tuple)):
            for q in qs:
                fn(int(q))
        else:
            fn(int(qs))

    def apply_x(self, qs):
        self._each(qs, lambda q: check(self.L.sq_apply_x(self.h, q, self.gc_mask)))

    def apply_y(self, qs):
        self._each(qs, lambda q: check(self.L.sq_apply_y(self.h, q, self.gc_mask)))

    def apply_h(self, qs):
        self._each(qs, lambda q: check(self.L.sq_apply_h(self.h, q, self.gc_mask)))

    def apply_z(self, qs):
        self._each(qs, lambda q: self.apply_u1(q, math.pi))

    def apply_s(self, qs):
        self._each(qs, lambda q: self.apply_u1(q, math.pi / 2.0))

    def apply_t(self, qs):
        self._each(qs, lambda q: self.apply_u1(q, math.pi / 4.0))

    def apply_tdg(self, qs):
        self._each(qs, lambda q: self.apply_u1(q, -math.pi / 4.0))

    def apply_u1(self, q, a, b=None):
        """apply_u1(q, phase) or apply_u1(q, q_mask, phase)."""
        q_mask, phase = (1, a) if b is None else (a, b)
        check(self.L.sq_apply_u1(self.h, int(q), int(q_mask), float(phase), self.gc_mask))

    # -- multi-qubit gates (src/suqa.cu:289-416) -------------------------------------
    def apply_cx(self, q_control, q_target, q_mask=1):
        mask_qs = self.gc_mask
        mask = mask_qs | (1 << q_control)
        if q_mask:
            mask_qs |= 1 << q_control
        check(self.L.sq_apply_mcx(self.h, mask, mask_qs, int(q_target)))

    def apply_mcx(self, q_controls: Sequence[int], a, b=None):
        """apply_mcx(controls, target) or apply_mcx(controls, q_mask, target)."""
        q_mask, q_target = ([1] * len(q_controls), a) if b is None else (a, b)
        mask = self.gc_mask
        mask_qs = self.gc_mask
        for q, m in zip(q_controls, q_mask):
            mask |= 1 << q
            if m:
                mask_qs |= 1 << q
        check(self.L.sq_apply_mcx(self.h, mask, mask_qs, int(q_target)))

    def apply_cu1(self, q_control, q_target, phase, q_mask=1):
        mask_qs = (1 << q_target) | self.gc_mask
        mask = mask_qs | (1 << q_control)
        if q_mask:
            mask_qs |= 1 << q_control
        check(self.L.sq_apply_mcu1(self.h, mask, mask_qs, float(phase)))

    def apply_mcu1(self, q_controls: Sequence[int], a, b, c=None):
        """apply_mcu1(controls, target, phase) or apply_mcu1(controls, q_mask, target, phase)."""
        q_mask, q_target, phase = ([1] * len(q_controls), a, b) if c is None else (a, b, c)
        mask = (1 << q_target) | self.gc_mask
        mask_qs = (1 << q_target) | self.gc_mask
        for q, m in zip(q_controls, q_mask):
            mask |= 1 << q
            if m:
                mask_qs |= 1 << q
        check(self.L.sq_apply_mcu1(self.h, mask, mask_qs, float(phase)))

    def apply_swap(self, q1, q2):
        check(self.L.sq_apply_swap(self.h, int(q1), int(q2), self.gc_mask))

    def apply_phase_list(self, q0: int, q_size: int, phases: Sequence[float]):
        if not (q_size > 0 and len(phases) == (1 << q_size)):
            raise RuntimeError("ERROR: in suqa::apply_phase_list(): invalid q_size or phases.size()")
        arr = (C.c_double * len(phases))(*[float(x) for x in phases])
        check(self.L.sq_apply_phase_list(self.h, int(q0), int(q_size), arr, self.gc_mask))

    def apply_pauli_TP_rotation(self, q_apply: Sequence[int], pauli_TPtype: Sequence[int], phase: float):
        """Reference semantics (supported patterns only, its X/Y quirk)."""
        if len(q_apply) != len(pauli_TPtype):
            raise RuntimeError("ERROR: in suqa::apply_pauli_TP_rotation(): mismatch between qubits number "
                               "and pauli types specified")
        check(self.L.sq_apply_pauli_rotation(self.h, len(q_apply), _u32(q_apply), _u32(pauli_TPtype),
                                             float(phase), self.gc_mask, SQ_PAULI_REFERENCE))

    def apply_pauli_rotation(self, q_apply: Sequence[int], paulis: Sequence[int], phase: float):
        """exp(i phase P) for any Pauli string (no reference counterpart beyond its subset)."""
        check(self.L.sq_apply_pauli_rotation(self.h, len(q_apply), _u32(q_apply), _u32(paulis),
                                             float(phase), self.gc_mask, SQ_PAULI_EXACT))

    # -- QFT (src/suqa.cu:611-661) ----------------------------------------------------
    def _crm(self, q_control, q_target, m, nqubits):
        if not self.rphase_m:
            # sized by the first call, like the reference table (src/suqa.cu:620-625);
            # larger registers later are computed directly instead of read past the end
            self.rphase_m = [2.0 * math.pi / float(1 << i) for i in range(nqubits + 1)]
        am = m if m > 0 else -m
        rphase = self.rphase_m[am] if am < len(self.rphase_m) else 2.0 * math.pi / float(1 << am)
        if m <= 0:
            rphase *= -1
        self.apply_cu1(q_control, q_target, rphase)

    def apply_qft(self, qact: Sequence[int]):
        k = len(qact)
        for o in range(k - 1, -1, -1):
            self.apply_h(qact[o])
            for i in range(o - 1, -1, -1):
                self._crm(qact[i], qact[o], 1 + (o - i), k)

    def apply_qft_inverse(self, qact: Sequence[int]):
        k = len(qact)
        for o in range(k):
            for i in range(o):
                self._crm(qact[i], qact[o], -1 - (o - i), k)
            self.apply_h(qact[o])

    # -- measurement (src/suqa.cu:673-757) -----------------------------------------------
    def measure_qbit(self, q: int, rdoub: float) -> int:
        c = C.c_uint32()
        check(self.L.sq_measure_qbit(self.h, int(q), float(rdoub), C.byref(c)))
        return int(c.value)

    def measure_qbits(self, qs: Sequence[int], rdoubs: Sequence[float]) -> list[int]:
        return [self.measure_qbit(q, r) for q, r in zip(qs, rdoubs)]

    def apply_reset(self, qs, rdoubs):
        if isinstance(qs, (list, tuple)):
            for q, r in zip(qs, rdoubs):
                self.apply_reset(q, r)
            return
        if self.measure_qbit(qs, rdoubs):
            self.apply_x(qs)

    def prob_filter(self, qs: Sequence[int], q_mask: Sequence[int]) -> float:
        mask_qs = 0
        for q in qs:
            mask_qs |= 1 << q
        mask = 0
        for q, m in zip(qs, q_mask):
            if m:
                mask |= int(m) << q
        out = C.c_double()
        check(self.L.sq_prob_filter(self.h, mask_qs, mask, C.byref(out)))
        return out.value

    # -- QMS acceptance oracle (include/qms.cuh:220-329) ---------------------------------
    def apply_qms_w(self, q_acc: int, mask_enew: int, shift: int, E_old: int, c_factor: float):
        check(self.L.sq_apply_qms_w(self.h, int(q_acc), int(mask_enew), int(shift), int(E_old), float(c_factor)))
