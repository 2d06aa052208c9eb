/* libsq — C ABI of the GB300 (sm_103a) state-vector engine.
 *
 * Drop-in boundary for the gate engine of SUQA: every entry point below
 * replaces one function of the reference's suqa:: API (include/suqa.cuh:94-176,
 * implemented in src/suqa.cu) or of the QMS algorithm header
 * (include/qms.cuh), as cited beside it.  The C++ header-compatible shim in
 * suqa_gb300/include/ re-exports the exact suqa:: names on top of this ABI.
 *
 * Conventions
 *  - Plain C types only.  Qubit masks are 64-bit; a state holds n <= 33 qubits.
 *  - Layout: one device allocation of 2*2^n elements, re block then im block,
 *    as the reference ComplexVec (include/complex_defines.cuh:22-45).
 *    Elements are double (SQ_F64) or float (SQ_F32).
 *  - Every call returns SQ_OK (0) or an error code; sq_last_error() gives text.
 *  - Gates are queued and applied lazily: consecutive gates are fused into as
 *    few passes over the state as their qubits allow.  Any call that observes
 *    the state (measure, prob_filter, vnorm, get_state, state_ptrs) first applies
 *    everything queued.  sq_flush() forces it.
 *  - Trigonometric and exponential coefficients are computed on the host in
 *    double precision, as the reference does (src/suqa.cu:274, include/qms.cuh:232).
 *  - One state is used by one host thread at a time; calls are stream-ordered
 *    on the state's stream.
 */
#ifndef SQ_H
#define SQ_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sq_state sq_state;

enum {
    SQ_OK = 0,
    SQ_ERR_ARG = 1,         /* invalid argument (qubit out of range, overlap, size) */
    SQ_ERR_CUDA = 2,        /* CUDA runtime error */
    SQ_ERR_UNSUPPORTED = 3, /* pattern the reference rejects (Pauli string, phase list) */
    SQ_ERR_NOMEM = 4,       /* device or host allocation failed */
    SQ_ERR_NODEVICE = 5     /* no usable CUDA device */
};

enum { SQ_F64 = 0, SQ_F32 = 1 };

/* Pauli rotation flags */
enum {
    SQ_PAULI_EXACT = 0,     /* exp(i phase P) for any Pauli string */
    SQ_PAULI_REFERENCE = 1  /* reference semantics: only its supported patterns
                               (1 qubit, 2 qubits, Z(x)A(x)A; others -> SQ_ERR_UNSUPPORTED),
                               and its two-qubit X/Y case as exp(i phase Y(x)X) */
};

const char* sq_last_error(void);
const char* sq_version(void);

/* --- state lifecycle: src/suqa.cu:760-866 (allocate_state, setup, clear) --- */
/* Allocates 2^n amplitudes in the given precision and sets |0...0>. */
int sq_state_create(sq_state** out, uint32_t n, int precision);
int sq_state_destroy(sq_state* s);
/* Device pointers of the re and im blocks (data_re/data_im of the reference
 * ComplexVec); applies queued gates first. */
int sq_state_ptrs(sq_state* s, void** data_re, void** data_im);
int sq_state_nqubits(const sq_state* s, uint32_t* n, int* precision);
/* Use a caller's CUDA stream (cudaStream_t) for all later work; NULL = the state's own. */
int sq_set_stream(sq_state* s, void* cuda_stream);
int sq_flush(sq_state* s);
int sq_synchronize(sq_state* s);
/* Host <-> device copies of the whole state as doubles (FP32 states convert). */
int sq_get_state(sq_state* s, double* re, double* im);
int sq_set_state(sq_state* s, const double* re, const double* im);
/* Raw copies in the state's own element type (double for SQ_F64, float for
 * SQ_F32); with page-locked host buffers these run at full link bandwidth and
 * are stream-ordered (sq_download returns after the copy completed). */
int sq_upload(sq_state* s, const void* host_re, const void* host_im);
int sq_download(sq_state* s, void* host_re, void* host_im);
/* Gate fusion on/off (default on); off applies every gate as its own pass. */
int sq_set_fusion(sq_state* s, int enabled);
/* Tile size of the fused passes in qubits (0: the default for the state's size
 * and precision; else 6 .. 13 in FP64, 6 .. 14 in FP32).  A tuning knob: results
 * do not depend on it beyond floating-point summation order. */
int sq_set_tile_qubits(sq_state* s, int k);
/* How multi-tile passes move tiles between HBM and shared memory (no
 * counterpart in the reference; a tuning knob, results are identical):
 * 0 (default) = 16-byte vector loads and stores through registers; 1 = bulk asynchronous
 * copies (cp.async.bulk on the TMA engine), one per run of contiguous
 * amplitudes, completion on an mbarrier whose waits are bounded (a pass that
 * gives up sets an error word that the next synchronising call reports as
 * SQ_ERR_CUDA); 2 = the same with two tile buffers, the next tile's copies in
 * flight while the current tile is worked on (tiles of 2^12 FP32 / 2^11 FP64
 * amplitudes). */
int sq_set_staging(sq_state* s, int mode);

/* --- state utilities: src/suqa.cu:70-111 --- */
int sq_init_state(sq_state* s);                   /* suqa::init_state */
int sq_vnorm(sq_state* s, double* norm);          /* suqa::vnorm */
int sq_vnormalize(sq_state* s);                   /* suqa::vnormalize (multiply by 1./norm) */

/* --- gates; gc = the global control mask (suqa::gc_mask, src/suqa.cu:36) --- */
int sq_apply_x(sq_state* s, uint32_t q, uint64_t gc);      /* suqa::apply_x, src/suqa.cu:115 */
int sq_apply_y(sq_state* s, uint32_t q, uint64_t gc);      /* suqa::apply_y, src/suqa.cu:136 */
int sq_apply_h(sq_state* s, uint32_t q, uint64_t gc);      /* suqa::apply_h, src/suqa.cu:207 */
/* suqa::apply_u1(q, q_mask, phase), src/suqa.cu:271: phase on the |q_mask> branch of q */
int sq_apply_u1(sq_state* s, uint32_t q, uint32_t q_mask, double phase, uint64_t gc);
/* multi-controlled X with per-control polarity, masks as the reference builds
 * them (src/suqa.cu:289-344): flips q_target where (i & control_mask) == mask_qs
 * (control_mask/mask_qs include gc; the target bit is added internally) */
int sq_apply_mcx(sq_state* s, uint64_t control_mask, uint64_t mask_qs, uint32_t q_target);
/* controlled phase, src/suqa.cu:346-393: phase where (i & control_mask) == mask_qs */
int sq_apply_mcu1(sq_state* s, uint64_t control_mask, uint64_t mask_qs, double phase);
int sq_apply_swap(sq_state* s, uint32_t q1, uint32_t q2, uint64_t gc);  /* src/suqa.cu:396 */
/* suqa::apply_phase_list, src/suqa.cu:418-455 (the reference's GPU-only API): 2^q_size
 * phases on qubits q0..q0+q_size-1; keeps the reference's guard (i & gc) != 0,
 * so it is a no-op when gc == 0.  q_size in 1..7. */
int sq_apply_phase_list(sq_state* s, uint32_t q0, uint32_t q_size, const double* phases, uint64_t gc);
/* suqa::apply_pauli_TP_rotation, src/suqa.cu:467-604: exp(i phase P),
 * P = (x)_k paulis[k] on qubits[k], paulis 1=X 2=Y 3=Z; k in 1..32 */
int sq_apply_pauli_rotation(sq_state* s, uint32_t k, const uint32_t* qubits, const uint32_t* paulis,
                            double phase, uint64_t gc, int flags);

/* --- dense blocks (no counterpart in the reference: its gates are applied one
 * kernel at a time, include/suqa_kernels.cuh:82-526) ---
 * Applies a 2^k x 2^k complex matrix U (row-major, u_re[r * 2^k + c]) to qubits
 * qubits[0..k-1] (index bit b of U <-> qubits[b]), k in 1..5, on the elements
 * where every bit of gc is set (gc disjoint from the qubits).  U is applied as
 * given (no unitarity check).  FP32 states of 2^12 amplitudes or more run it on
 * the tensor cores (tcgen05, TF32 high/remainder split of both operands, four
 * products: ~2^-24 relative per product), otherwise on the CUDA cores in FP64
 * arithmetic.  States need at least 5 qubits. */
int sq_apply_unitary(sq_state* s, uint32_t k, const uint32_t* qubits, const double* u_re, const double* u_im,
                     uint64_t gc);
/* FP64 states: run the arithmetic of multi-tile passes (gates without tables or
 * dense blocks) in double-float on the FP32 pipe instead of the FP64 pipe (no
 * counterpart in the reference).  Amplitudes stay IEEE doubles in memory; each
 * pass converts them to hi + lo FP32 pairs (48 significand bits) and back with
 * integer operations.  Rounding differs from FP64 arithmetic at the 1e-14 level
 * per operation.  Default 0. */
int sq_set_double_float(sq_state* s, int enabled);
/* Automatic dense blocks (FP32 states): runs of consecutive gates on at most
 * five qubits with at least min_gates gates (uncontrolled X gates not counted)
 * are multiplied into one matrix on the host (FP64) and applied as one dense
 * block.  0 (default) disables it. */
int sq_set_dense_fusion(sq_state* s, int min_gates);
/* Engine for dense blocks: 0 (default) tensor cores where the state allows,
 * 1 CUDA cores. */
int sq_set_dense_engine(sq_state* s, int engine);

/* --- measurement: src/suqa.cu:673-727 --- */
/* p1 = sum |a_i|^2 over bit q set; c = (r < p1); zero the other branch; rescale
 * the kept one by 1/sqrt(p_c) */
int sq_measure_qbit(sq_state* s, uint32_t q, double r, uint32_t* c);
/* sum |a_i|^2 over (i & mask_qs) == mask */
int sq_prob_filter(sq_state* s, uint64_t mask_qs, uint64_t mask, double* prob);

/* --- QMS acceptance oracle W: include/qms.cuh:220-329 --- */
/* Rotation on the acceptance qubit q_acc (pairs i with bit q_acc set and
 * i without it) with f1 = exp(-dE/2), f2 = sqrt(1-f1^2) for dE > 0 (else 1, 0),
 * dE = Enew*c - E_old*c, Enew = (i & mask_enew) >> shift.  Like the reference,
 * it ignores the global control mask.  (mask_enew >> shift) < 128. */
int sq_apply_qms_w(sq_state* s, uint32_t q_acc, uint64_t mask_enew, uint32_t shift,
                   uint32_t E_old, double c_factor);

/* --- counters (gate-cost reporting) --- */
typedef struct sq_stats {
    uint64_t gates;        /* gates queued */
    uint64_t passes;       /* passes over the state executed */
    uint64_t launches;     /* kernel launches */
    uint64_t reductions;   /* measurement / filter reductions */
    uint64_t bytes_moved;  /* bytes read + written by executed passes (algorithmic) */
    uint64_t flops;        /* floating-point operations of the executed gates and reductions
                              (reference formulas: 4/amplitude for H, 6 for a phase or a
                              Pauli rotation on the amplitudes it touches, 0 for X/CX/MCX/SWAP) */
} sq_stats;
int sq_get_stats(const sq_state* s, sq_stats* out);
int sq_reset_stats(sq_state* s);
/* Kernel timing: when enabled, every pass launch is bracketed by CUDA events on
 * the state's stream; sq_kernel_time() synchronizes and returns the summed
 * device time (ms), the launch count and the bytes those launches moved since
 * the last call (then clears them). */
int sq_set_timing(sq_state* s, int enabled);
int sq_kernel_time(sq_state* s, double* ms, uint64_t* launches, uint64_t* bytes);

/* --- batched quantum Metropolis sampling: many independent chains on the device ---
 * No single reference function: each chain is one run of the reference's qms
 * driver (src/qms.cu:51-178, include/qms.cuh:373-545) for a transverse-field
 * Ising ring plugin, H = -J sum Z_i Z_{i+1} - h sum X_i (ring of `spins`),
 * exp(-iHt) by ceil(|t|/dt) first-order Trotter steps (bond phases, then X
 * rotations), moves = Hadamard on a uniformly drawn spin, observable = Z-basis
 * magnetisation.  Register layout: spins, energy register, acceptance qubit. */
typedef struct sq_tfim_chain {
    uint32_t spins;           /* ring length s (system qubits) */
    uint32_t ene_qbits;       /* energy register width e */
    uint32_t steps;           /* Metropolis steps */
    uint32_t thermalization;  /* sampling starts after this many steps */
    uint32_t reset_each;      /* sample every reset_each steps */
    uint32_t max_reverse;     /* restoration attempts (the reference default is 100) */
    double J, h, beta;
    double ene_min, ene_max;  /* phase-estimation window */
    double dt;                /* Trotter step width */
    uint64_t seed;            /* PCG32 seed, stream 1 (as pcg::set_seed) */
    uint32_t warm_start;      /* 1: the initial state is RY(ry[i]) on spin i applied to |0...0>
                                 (also after a failed restoration); 0: |0...0> */
    uint32_t pad;
    double ry[20];
} sq_tfim_chain;

typedef struct sq_chain_result {
    uint32_t accepted;        /* steps returning 1 or 2 */
    uint32_t failures;        /* failed restorations (state re-initialised) */
    uint32_t samples;         /* (E, A) samples written */
    uint32_t phase_estimations; /* energy phase estimations (forward and inverse) applied */
    uint64_t cycles;          /* SM clock cycles the chain took */
    uint64_t evolution_cycles; /* ... of which in the controlled time evolutions (Trotter steps) */
} sq_chain_result;

/* Runs every chain to completion on the current device (one persistent launch per
 * chain-size class).  Host arrays: results[nchains]; samples_E/A/step (may be
 * NULL) hold sum(steps) entries, chain i's samples starting at the sum of the
 * steps of chains 0..i-1 (E = energy reading, A = magnetisation, step = step
 * index).  kernel_ms (may be NULL) receives the device time of the launches. */
int sq_qms_tfim_batch(const sq_tfim_chain* chains, uint32_t nchains, int precision, sq_chain_result* results,
                      double* samples_E, double* samples_A, uint32_t* samples_step, void* stream, float* kernel_ms);

/* --- resumable chain batches ---
 * A batch keeps every chain's amplitudes, random stream (PCG32 state and
 * increment) and counters on the device between calls, so a run can be
 * advanced in pieces, read out, checkpointed to host memory and resumed; the
 * results are identical to one uninterrupted run.  Calls are blocking and use
 * the batch's own stream on the device current at creation. */
typedef struct sq_batch sq_batch;

typedef struct sq_batch_opts {
    uint32_t segment_steps;    /* steps per segment (0: a run call is one segment) */
    uint32_t use_graph;        /* 1 (with segment_steps > 0): the launches of one segment are
                                  captured once in a CUDA graph and replayed */
    uint32_t autotune;         /* 1 (with threads == 0): per chain-width class, time one step of
                                  a sample of its chains at each CTA size and keep the fastest */
    uint32_t threads;          /* CTA size 128, 256 or 512 (FP64: at most 256); 0: 256 or tuned */
    uint64_t l2_budget_bytes;  /* live-state bound for chains run from global memory (0: 64 MiB) */
    uint32_t cta_qubits;       /* most qubits one CTA holds in shared memory (0: as many as fit);
                                  wider chains are spread over a cluster */
    uint32_t global_qubits;    /* chains of at least this many qubits run from global memory
                                  (0: only chains too wide for a 16-CTA cluster) */
} sq_batch_opts;

typedef struct sq_batch_class {
    uint32_t n, count;         /* qubits per chain, chains of this width */
    uint32_t mode;             /* 0: one CTA, state in shared memory; 1: cluster, state in the
                                  CTAs' shared memory; 2: cluster, state in global memory */
    uint32_t cluster, threads, grid, smem_bytes;
    float probe_ms;            /* autotuner's time for the chosen size (-1: not tuned) */
} sq_batch_class;

int sq_batch_create(sq_batch** out, const sq_tfim_chain* chains, uint32_t nchains, int precision,
                    const sq_batch_opts* opts);
int sq_batch_destroy(sq_batch* b);
/* advance every unfinished chain by up to `steps` steps; kernel_ms (may be NULL) = device time */
int sq_batch_run(sq_batch* b, uint32_t steps, float* kernel_ms);
/* counters and all samples written so far (layout as sq_qms_tfim_batch) */
int sq_batch_results(sq_batch* b, sq_chain_result* results, double* samples_E, double* samples_A,
                     uint32_t* samples_step);
/* steps completed per chain (host array of nchains) */
int sq_batch_progress(sq_batch* b, uint32_t* steps_done);
/* current amplitudes of one chain (2^n each, converted to double) */
int sq_batch_state(sq_batch* b, uint32_t chain, double* re, double* im);
int sq_batch_checkpoint_size(const sq_batch* b, uint64_t* bytes);
int sq_batch_checkpoint(sq_batch* b, void* host, uint64_t bytes);
/* only into a batch created with the same chains and precision */
int sq_batch_restore(sq_batch* b, const void* host, uint64_t bytes);
/* the launch plan: one entry per chain-width class (widest first) */
int sq_batch_plan(const sq_batch* b, sq_batch_class* info, uint32_t max, uint32_t* nclasses);

/* --- batched time evolution with probability read-out ---
 * The reference's evo driver (src/evo.cu:51-98) for many transverse-field
 * Ising rings at once: job j evolves its ring (H = -J sum Z_i Z_{i+1} - h sum X_i)
 * from |0...0> (or RY(ry_i) per spin) by `steps` first-order Trotter steps of
 * width dt (ZZ bond phases, then the X rotations) and records, after 0, 1, ...,
 * steps steps, the 2^spins basis probabilities in FP64 (prob_filter of every
 * pattern).  probs receives, job after job, (steps + 1) rows of 2^spins values.
 * spins 2..12. */
typedef struct sq_tfim_evolution {
    uint32_t spins, steps;
    double J, h, dt;
    uint32_t warm_start, pad;
    double ry[20];
} sq_tfim_evolution;
int sq_tfim_evolve_batch(const sq_tfim_evolution* jobs, uint32_t njobs, int precision, double* probs,
                         float* kernel_ms);

/* --- batched Szegedy-walk annealing (QSA) on Ising rings ---
 * Generalises the reference's triangle-only QSA (include/qsa.cuh:616-756 walk,
 * src/qsa.cu:159-268 annealing loop) to a ring of s spins with integer couplings
 * and no field, H(x) = -sum_i J_i s_i s_{i+1 mod s}, with the rotation and
 * reflection of the reference's commented general form (qsa.cuh:372-418).
 * Each walk anneals beta_k = (k+1) beta / stages, k < stages, with
 * steps_per_stage walk steps at each; a step draws the move (qsa::draw_C with
 * weights 1/s), runs the walk-phase estimation with a phase_qbits register and
 * reads it (phase_qbits draws); a nonzero value restarts the anneal
 * (qsa.cu:199-205).  A completed anneal reads the s spins (s draws).  The
 * energy-difference register is exact for integer couplings and is applied in
 * closed form.  p0_trace (optional) receives, walk after walk, one slot per
 * allowed step (max_steps, or 8 x stages x steps_per_stage when 0): the
 * probability of the zero walk phase at each step run. */
typedef struct sq_qsa_walk {
    uint32_t spins;           /* ring length, 2..12 */
    uint32_t phase_qbits;     /* walk-phase register, 1..6 qubits */
    uint32_t stages;          /* annealing stages */
    uint32_t steps_per_stage; /* walk steps at each temperature */
    uint32_t max_steps;       /* cap on steps over all attempts (0: 8 x stages x steps_per_stage) */
    int32_t J[12];            /* bond couplings, bond i joins spins i and i+1 mod s; -8..8 */
    uint32_t algo;            /* 0: iterate W per orbit; 1: per orbit class (W, eigenvectors of
                                 (W + W^T)/2, sum of powers), at most 96 classes per move, the
                                 class data prepared once per batch for every (class, stage
                                 temperature) when that table fits (4 GiB), else per step;
                                 2: as 1, always prepared per walk and step;
                                 one value for the whole batch */
    double beta;              /* final inverse temperature */
    uint64_t seed;            /* PCG32 seed (pcg32::seed(seed, 1)) */
} sq_qsa_walk;
typedef struct sq_qsa_walk_result {
    uint32_t done;     /* 1: the anneal completed and the spins were read; 0: capped */
    uint32_t restarts; /* attempts abandoned on a nonzero walk phase */
    uint32_t steps;    /* walk steps run over all attempts */
    uint32_t readout;  /* spin configuration read (bit i = spin i) */
    double E, absM;    /* energy and |magnetisation| of the readout */
    double last_p0;    /* probability of the zero walk phase at the last step */
} sq_qsa_walk_result;
/* FP32 walks by orbit classes: the class-sorted orbit pass with 16 warps per
 * CTA (default, where the batch's classes fit its shared memory) or the 8-warp
 * pass (per-warp class sums).  Process-wide; results agree to FP32 rounding (the
 * class sums are added in different orders).  No counterpart in the reference. */
int sq_set_walk_orbit_warps(int warps);
/* FP32 walks by orbit classes with the 16-warp pass: 1 (default) records where
 * the per-chunk sort by class puts every orbit, the first time a part of a walk
 * runs a move (2 bytes per orbit and move, when that table fits 8 GiB and a
 * quarter of the free device memory), and later steps with that move take the
 * places from the table instead of sorting; 0 sorts at every step.  Results are
 * bit-identical.  Process-wide.  No counterpart in the reference. */
int sq_set_walk_presort(int on);
/* FP32 walks by orbit classes with the 16-warp pass: the 16 x 16 class products
 * on the tensor cores (1, default: mma.sync m16n8k8 TF32 with the three-product
 * split hi/lo of both operands, ~2^-22 relative per product) or on the CUDA cores
 * in FP32 (0).  Process-wide.  No counterpart in the reference. */
int sq_set_walk_mma(int on);
int sq_qsa_walk_batch(const sq_qsa_walk* walks, uint32_t nwalks, int precision, sq_qsa_walk_result* results,
                      double* p0_trace, float* kernel_ms);

/* --- learned warm start: a small MLP with BF16 weights/activations, FP32 sums ---
 * No reference counterpart.  in -> `layers` hidden layers of `hidden` GELU units
 * -> out.  Parameters are one flat FP32 array (W_l row-major, then b_l, layer by
 * layer).  Host arrays throughout: x[batch][in], y/targets/mask[batch][out].
 * Loss: mean over rows of sum_k mask*(y - t)^2.  train_step = forward, backward
 * and one Adam update (beta 0.9/0.999, eps 1e-8) on the FP32 master weights. */
typedef struct sq_mlp sq_mlp;
int sq_mlp_create(sq_mlp** out, uint32_t in, uint32_t hidden, uint32_t layers, uint32_t out_dim, uint64_t seed);
int sq_mlp_destroy(sq_mlp* n);
int sq_mlp_num_params(const sq_mlp* n, uint32_t* count);
int sq_mlp_get_params(sq_mlp* n, float* flat);
int sq_mlp_set_params(sq_mlp* n, const float* flat);
int sq_mlp_forward(sq_mlp* n, const float* x, uint32_t batch, float* y);
/* gradient of the loss w.r.t. the flat parameters (for checks against a CPU reference) */
int sq_mlp_gradients(sq_mlp* n, const float* x, const float* targets, const float* mask, uint32_t batch,
                     float* grad, float* loss);
int sq_mlp_train_step(sq_mlp* n, const float* x, const float* targets, const float* mask, uint32_t batch, float lr,
                      float* loss);

/* --- allocation-free measurement probabilities (no counterpart in the reference) ---
 * For callers that may not allocate device memory on the call path: their host
 * application's memory manager owns all device buffers, or they are a plugin
 * handed raw device pointers by another runtime, or an allocation's latency and
 * implicit synchronisation are unacceptable.  Computes p0 and p1 of qubit q
 * (sum of |a_i|^2 over i with bit q clear / set, reduced in FP64) of a state the
 * caller owns (re, im: device arrays of 2^n doubles for SQ_F64 or floats for
 * SQ_F32) and writes them to out_p01 (device memory, 2 doubles), on the given
 * CUDA stream (NULL = legacy default stream), without allocating anything.
 * The scratch is one static device array (partial sums of at most 4096 CTAs,
 * 64 KiB + 256 B, resident on every GPU that loads the library until exit);
 * launches needing more are rejected with SQ_ERR_ARG.  All calls share it:
 * calls whose kernels overlap on the GPU race; calls ordered on one stream are
 * safe.  The first call on a device performs a one-time set-up on it and
 * should come before any stream capture.  re and im must be 16-byte aligned
 * (element-aligned for states narrower than one 16-byte vector) and out_p01
 * 8-byte aligned; misaligned pointers are rejected with SQ_ERR_ARG before any
 * launch. */
int sq_qubit_probs_noalloc(const void* re, const void* im, uint32_t n, int precision, uint32_t q,
                           double* out_p01, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SQ_H */
