"""ctypes binding of libsq (include/sq.h).  Loading fails loudly: there is no
CPU fallback for any engine call."""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libsq.so")

SQ_OK, SQ_ERR_ARG, SQ_ERR_CUDA, SQ_ERR_UNSUPPORTED, SQ_ERR_NOMEM, SQ_ERR_NODEVICE = range(6)
SQ_F64, SQ_F32 = 0, 1
SQ_PAULI_EXACT, SQ_PAULI_REFERENCE = 0, 1


class SqError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libsq error {code}: {msg}")
        self.code = code


class SqUnsupported(SqError):
    pass


class SqStats(C.Structure):
    _fields_ = [("gates", C.c_uint64), ("passes", C.c_uint64), ("launches", C.c_uint64),
                ("reductions", C.c_uint64), ("bytes_moved", C.c_uint64), ("flops", C.c_uint64)]


class SqTfimChain(C.Structure):
    _fields_ = [("spins", C.c_uint32), ("ene_qbits", C.c_uint32), ("steps", C.c_uint32),
                ("thermalization", C.c_uint32), ("reset_each", C.c_uint32), ("max_reverse", C.c_uint32),
                ("J", C.c_double), ("h", C.c_double), ("beta", C.c_double), ("ene_min", C.c_double),
                ("ene_max", C.c_double), ("dt", C.c_double), ("seed", C.c_uint64),
                ("warm_start", C.c_uint32), ("pad", C.c_uint32), ("ry", C.c_double * 20)]


class SqChainResult(C.Structure):
    _fields_ = [("accepted", C.c_uint32), ("failures", C.c_uint32), ("samples", C.c_uint32),
                ("phase_estimations", C.c_uint32), ("cycles", C.c_uint64), ("evolution_cycles", C.c_uint64)]


class SqTfimEvolution(C.Structure):
    _fields_ = [("spins", C.c_uint32), ("steps", C.c_uint32), ("J", C.c_double), ("h", C.c_double),
                ("dt", C.c_double), ("warm_start", C.c_uint32), ("pad", C.c_uint32), ("ry", C.c_double * 20)]


class SqQsaWalk(C.Structure):
    _fields_ = [("spins", C.c_uint32), ("phase_qbits", C.c_uint32), ("stages", C.c_uint32),
                ("steps_per_stage", C.c_uint32), ("max_steps", C.c_uint32), ("J", C.c_int32 * 12),
                ("algo", C.c_uint32), ("beta", C.c_double), ("seed", C.c_uint64)]


class SqQsaWalkResult(C.Structure):
    _fields_ = [("done", C.c_uint32), ("restarts", C.c_uint32), ("steps", C.c_uint32), ("readout", C.c_uint32),
                ("E", C.c_double), ("absM", C.c_double), ("last_p0", C.c_double)]


class SqBatchOpts(C.Structure):
    _fields_ = [("segment_steps", C.c_uint32), ("use_graph", C.c_uint32), ("autotune", C.c_uint32),
                ("threads", C.c_uint32), ("l2_budget_bytes", C.c_uint64), ("cta_qubits", C.c_uint32),
                ("global_qubits", C.c_uint32)]


class SqBatchClass(C.Structure):
    _fields_ = [("n", C.c_uint32), ("count", C.c_uint32), ("mode", C.c_uint32), ("cluster", C.c_uint32),
                ("threads", C.c_uint32), ("grid", C.c_uint32), ("smem_bytes", C.c_uint32), ("probe_ms", C.c_float)]


_lib = None

_SIGS = {
    "sq_last_error": (C.c_char_p, []),
    "sq_version": (C.c_char_p, []),
    "sq_state_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.c_int]),
    "sq_state_destroy": (C.c_int, [C.c_void_p]),
    "sq_state_ptrs": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "sq_state_nqubits": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_int)]),
    "sq_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sq_flush": (C.c_int, [C.c_void_p]),
    "sq_synchronize": (C.c_int, [C.c_void_p]),
    "sq_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sq_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sq_set_fusion": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_set_tile_qubits": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_set_staging": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_upload": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sq_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sq_init_state": (C.c_int, [C.c_void_p]),
    "sq_vnorm": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "sq_vnormalize": (C.c_int, [C.c_void_p]),
    "sq_apply_x": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64]),
    "sq_apply_y": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64]),
    "sq_apply_h": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64]),
    "sq_apply_u1": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_uint64]),
    "sq_apply_mcx": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint32]),
    "sq_apply_mcu1": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_double]),
    "sq_apply_swap": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64]),
    "sq_apply_phase_list": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_double), C.c_uint64]),
    "sq_apply_pauli_rotation": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                          C.c_double, C.c_uint64, C.c_int]),
    "sq_apply_unitary": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.c_uint64]),
    "sq_set_dense_fusion": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_set_double_float": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_set_dense_engine": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_measure_qbit": (C.c_int, [C.c_void_p, C.c_uint32, C.c_double, C.POINTER(C.c_uint32)]),
    "sq_prob_filter": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.POINTER(C.c_double)]),
    "sq_apply_qms_w": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_double]),
    "sq_get_stats": (C.c_int, [C.c_void_p, C.POINTER(SqStats)]),
    "sq_reset_stats": (C.c_int, [C.c_void_p]),
    "sq_set_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "sq_kernel_time": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "sq_set_walk_orbit_warps": (C.c_int, [C.c_int]),
    "sq_set_walk_presort": (C.c_int, [C.c_int]),
    "sq_set_walk_mma": (C.c_int, [C.c_int]),
    "sq_qms_tfim_batch": (C.c_int, [C.POINTER(SqTfimChain), C.c_uint32, C.c_int, C.POINTER(SqChainResult),
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    "sq_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(SqTfimChain), C.c_uint32, C.c_int,
                                  C.POINTER(SqBatchOpts)]),
    "sq_batch_destroy": (C.c_int, [C.c_void_p]),
    "sq_batch_run": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_float)]),
    "sq_batch_results": (C.c_int, [C.c_void_p, C.POINTER(SqChainResult), C.c_void_p, C.c_void_p, C.c_void_p]),
    "sq_batch_progress": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sq_batch_state": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "sq_batch_checkpoint_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "sq_batch_checkpoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "sq_batch_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "sq_batch_plan": (C.c_int, [C.c_void_p, C.POINTER(SqBatchClass), C.c_uint32, C.POINTER(C.c_uint32)]),
    "sq_tfim_evolve_batch": (C.c_int, [C.POINTER(SqTfimEvolution), C.c_uint32, C.c_int, C.c_void_p,
                                       C.POINTER(C.c_float)]),
    "sq_qsa_walk_batch": (C.c_int, [C.POINTER(SqQsaWalk), C.c_uint32, C.c_int, C.POINTER(SqQsaWalkResult),
                                    C.c_void_p, C.POINTER(C.c_float)]),
    "sq_mlp_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64]),
    "sq_mlp_destroy": (C.c_int, [C.c_void_p]),
    "sq_mlp_num_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    "sq_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sq_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sq_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "sq_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                   C.POINTER(C.c_float)]),
    "sq_mlp_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_float,
                                    C.POINTER(C.c_float)]),
    "sq_qubit_probs_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_uint32, C.c_void_p,
                                         C.c_void_p]),
}

EXPORTED = tuple(_SIGS)


def load():
    """Load libsq.so.  Raises RuntimeError when the native library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libsq not built ({LIB_PATH} missing): run `python -m suqa_gb300.build`; "
                           "suqa_gb300 has no CPU fallback")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != SQ_OK:
        msg = _lib.sq_last_error().decode(errors="replace")
        if rc == SQ_ERR_UNSUPPORTED:
            raise SqUnsupported(rc, msg)
        raise SqError(rc, msg)
    return rc
