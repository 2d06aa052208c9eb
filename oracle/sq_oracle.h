/* CPU oracle for the suqa state-vector engine: a plain-C restatement of the
 * reference's dense CPU path (include/suqa_cpu.hpp non-SPARSE branches and the
 * dispatch in src/suqa.cu), plus the QMS acceptance rotation W
 * (include/qms.cuh:245-309) and the PCG32 generator (include/pcg32.h:40-130).
 *
 * TEST INFRASTRUCTURE ONLY.  Only the test suite, the smoke check and the
 * CPU-baseline leg of the benchmark may load this library; the product
 * (libsq) never calls it.
 *
 * Parity: pinned against the reference CPU build itself (oracle/_ref/ref_dump,
 * compiled from the reference sources) by tests/test_oracle_vs_reference.py and
 * by the committed fixtures in tests/golden/.
 *
 * Layout: one allocation of 2N doubles, re block then im block, as the
 * reference's ComplexVec (include/complex_defines.cuh:22-45, src/suqa.cu:779-785).
 */
#ifndef SQ_ORACLE_H
#define SQ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_state {
    uint32_t n;
    uint64_t N;
    double* data; /* 2N doubles: re[0..N), im[0..N) */
    double* re;
    double* im;
} or_state;

/* Threads used by gate loops and reductions (default 1).  With >1 thread the
 * reductions are summed per contiguous chunk, so their rounding differs from
 * the sequential reference; parity tests keep the default. */
void or_set_threads(int k);
int or_get_threads(void);

or_state* or_create(uint32_t n);
void or_destroy(or_state* s);
void or_init_state(or_state* s);
double or_vnorm(or_state* s);
void or_vnormalize(or_state* s);

void or_apply_x(or_state* s, uint32_t q, uint64_t gc);
void or_apply_y(or_state* s, uint32_t q, uint64_t gc);
void or_apply_h(or_state* s, uint32_t q, uint64_t gc);
void or_apply_u1(or_state* s, uint32_t q, uint32_t qmask, double phase, uint64_t gc);
void or_apply_mcx(or_state* s, uint64_t control_mask, uint64_t mask_qs, uint32_t q_target);
void or_apply_mcu1(or_state* s, uint64_t control_mask, uint64_t mask_qs, double phase);
void or_apply_swap(or_state* s, uint32_t q1, uint32_t q2, uint64_t gc);
/* returns 0, or -1 on an invalid size (the reference throws) */
int or_apply_phase_list(or_state* s, uint32_t q0, uint32_t q_size, const double* phases, uint64_t gc);
/* exp(i phase P), P = tensor product of paulis[k] (1=X,2=Y,3=Z) on qubits[k].
 * strict=1 reproduces the reference's supported set (1 qubit, 2 qubits, Z(x)A(x)A)
 * and returns -1 where the reference throws; strict=0 accepts any string. */
int or_apply_pauli(or_state* s, uint32_t k, const uint32_t* qubits, const uint32_t* paulis,
                   double phase, uint64_t gc, int strict);
void or_apply_qft(or_state* s, uint32_t k, const uint32_t* qs, uint64_t gc);
void or_apply_qft_inverse(or_state* s, uint32_t k, const uint32_t* qs, uint64_t gc);

double or_prob1(or_state* s, uint32_t q);
uint32_t or_measure_qbit(or_state* s, uint32_t q, double r);
void or_apply_reset(or_state* s, uint32_t q, double r, uint64_t gc);
double or_prob_filter(or_state* s, uint64_t mask_qs, uint64_t mask);

/* QMS acceptance rotation on the acceptance qubit (assumed the most significant),
 * conditioned on the energy register bits (i & mask_enew) >> shift against the
 * classical E_old: c_factor = beta / (t_PE_factor * ene_levels). */
void or_apply_qms_w(or_state* s, uint32_t q_acc, uint64_t mask_enew, uint32_t shift,
                    uint32_t E_old, double c_factor);

/* PCG32 (state, inc), seeded like pcg32::seed(initstate, initseq=1). */
typedef struct or_pcg { uint64_t state, inc; } or_pcg;
void or_pcg_seed(or_pcg* g, uint64_t initstate, uint64_t initseq);
uint32_t or_pcg_next(or_pcg* g);
double or_pcg_doub(or_pcg* g);

#ifdef __cplusplus
}
#endif
#endif
