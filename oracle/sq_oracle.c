/* CPU oracle: plain-C restatement of the reference's dense CPU state-vector
 * engine.  TEST INFRASTRUCTURE ONLY (see sq_oracle.h): the product never calls
 * it.  Every function names the reference lines it restates; element-wise
 * arithmetic keeps the reference's operation order so that, compiled without
 * floating-point contraction (-ffp-contract=off), results are bit-identical to
 * the reference CPU build.  Parity pinned by tests/test_oracle_vs_reference.py
 * (reference built from its sources) and the fixtures in tests/golden/.
 */
#define _GNU_SOURCE
#include "sq_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define TWOSQINV 0.7071067811865475 /* reference include/suqa.cuh:57 */
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int g_threads = 1;
void or_set_threads(int k) { g_threads = k < 1 ? 1 : (k > 256 ? 256 : k); }
int or_get_threads(void) { return g_threads; }

/* ---- range-parallel helper: splits [0,N) into contiguous chunks ------------- */
typedef void (*range_fn)(void* ctx, uint64_t lo, uint64_t hi, int tid);
typedef struct { range_fn fn; void* ctx; uint64_t lo, hi; int tid; } range_job;
static void* range_tramp(void* p) {
    range_job* j = (range_job*)p;
    j->fn(j->ctx, j->lo, j->hi, j->tid);
    return NULL;
}
static void run_range(uint64_t N, range_fn fn, void* ctx) {
    int T = g_threads;
    if (T <= 1 || N < 4096) { fn(ctx, 0, N, 0); return; }
    pthread_t th[256];
    range_job jobs[256];
    uint64_t chunk = (N + (uint64_t)T - 1) / (uint64_t)T;
    for (int t = 0; t < T; ++t) {
        uint64_t lo = chunk * (uint64_t)t, hi = lo + chunk;
        if (lo > N) lo = N;
        if (hi > N) hi = N;
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].lo = lo; jobs[t].hi = hi; jobs[t].tid = t;
        pthread_create(&th[t], NULL, range_tramp, &jobs[t]);
    }
    for (int t = 0; t < T; ++t) pthread_join(th[t], NULL);
}

/* ---- state --------------------------------------------------------------- */
or_state* or_create(uint32_t n) {
    or_state* s = (or_state*)calloc(1, sizeof(or_state));
    if (!s) return NULL;
    s->n = n;
    s->N = 1ULL << n;
    s->data = (double*)malloc(2 * s->N * sizeof(double));
    if (!s->data) { free(s); return NULL; }
    s->re = s->data;
    s->im = s->data + s->N;
    or_init_state(s);
    return s;
}

void or_destroy(or_state* s) {
    if (!s) return;
    free(s->data);
    free(s);
}

/* include/suqa_cpu.hpp:5-13 */
void or_init_state(or_state* s) {
    memset(s->data, 0, 2 * s->N * sizeof(double));
    s->data[0] = 1.0;
}

/* include/suqa_cpu.hpp:15-28 (sum over the 2N doubles in order), src/suqa.cu:90 */
typedef struct { const double* d; double part[256]; } sumsq_ctx;
static void sumsq_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    sumsq_ctx* x = (sumsq_ctx*)c;
    double r = 0.0;
    for (uint64_t i = lo; i < hi; ++i) r += x->d[i] * x->d[i];
    x->part[tid] = r;
}
double or_vnorm(or_state* s) {
    sumsq_ctx x;
    x.d = s->data;
    memset(x.part, 0, sizeof(x.part));
    run_range(2 * s->N, sumsq_range, &x);
    double r = 0.0;
    for (int t = 0; t < g_threads; ++t) r += x.part[t];
    return sqrt(r);
}

/* src/suqa.cu:97-111 and include/suqa_cpu.hpp:30-40: multiply by 1./norm */
typedef struct { double* d; double v; } scale_ctx;
static void scale_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    scale_ctx* x = (scale_ctx*)c;
    for (uint64_t i = lo; i < hi; ++i) x->d[i] *= x->v;
}
void or_vnormalize(or_state* s) {
    scale_ctx x;
    x.d = s->data;
    x.v = 1. / or_vnorm(s);
    run_range(2 * s->N, scale_range, &x);
}

/* ---- gates ----------------------------------------------------------------- */
typedef struct {
    double *re, *im;
    uint64_t m0, m1, m2;
    uint32_t q;
    double c, s;
} gate_ctx;

/* include/suqa_cpu.hpp:69-94 (dense X), dispatch src/suqa.cu:115-120 */
static void x_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    gate_ctx* g = (gate_ctx*)c;
    const uint64_t gm = g->m0, b = 1ULL << g->q;
    for (uint64_t i = lo; i < hi; ++i) {
        if ((i & gm) == gm) {
            uint64_t j = i & ~b;
            double t = g->re[i]; g->re[i] = g->re[j]; g->re[j] = t;
            t = g->im[i]; g->im[i] = g->im[j]; g->im[j] = t;
        }
    }
}
void or_apply_x(or_state* s, uint32_t q, uint64_t gc) {
    gate_ctx g = {s->re, s->im, gc | (1ULL << q), 0, 0, q, 0, 0};
    run_range(s->N, x_range, &g);
}

/* include/suqa_cpu.hpp:96-122 (dense Y) */
static void y_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    gate_ctx* g = (gate_ctx*)c;
    const uint64_t gm = g->m0, b = 1ULL << g->q;
    for (uint64_t i = lo; i < hi; ++i) {
        if ((i & gm) == gm) {
            uint64_t j = i & ~b;
            double t = g->re[i];
            g->re[i] = g->im[j] * -1.0;
            g->im[j] = t * -1.0;
            t = g->im[i];
            g->im[i] = g->re[j];
            g->re[j] = t;
        }
    }
}
void or_apply_y(or_state* s, uint32_t q, uint64_t gc) {
    gate_ctx g = {s->re, s->im, gc | (1ULL << q), 0, 0, q, 0, 0};
    run_range(s->N, y_range, &g);
}

/* include/suqa_cpu.hpp:150-206 (dense H, literal TWOSQINV) */
static void h_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    gate_ctx* g = (gate_ctx*)c;
    const uint64_t gc = g->m0, b = 1ULL << g->q, lm = gc | b;
    for (uint64_t i0 = lo; i0 < hi; ++i0) {
        if ((i0 & lm) == gc) {
            const uint64_t i1 = i0 | b;
            double a0r = g->re[i0], a0i = g->im[i0], a1r = g->re[i1], a1i = g->im[i1];
            g->re[i0] = TWOSQINV * (a0r + a1r);
            g->im[i0] = TWOSQINV * (a0i + a1i);
            g->re[i1] = TWOSQINV * (a0r - a1r);
            g->im[i1] = TWOSQINV * (a0i - a1i);
        }
    }
}
void or_apply_h(or_state* s, uint32_t q, uint64_t gc) {
    gate_ctx g = {s->re, s->im, gc, 0, 0, q, 0, 0};
    run_range(s->N, h_range, &g);
}

/* diagonal phase on (i & m1) == m0: util_rotate2 of include/suqa_cpu.hpp:49-54 */
static void phase_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    gate_ctx* g = (gate_ctx*)c;
    for (uint64_t i = lo; i < hi; ++i) {
        if ((i & g->m1) == g->m0) {
            double a = g->re[i];
            g->re[i] = a * g->c - g->im[i] * g->s;
            g->im[i] = g->im[i] * g->c + a * g->s;
        }
    }
}

/* src/suqa.cu:271-285 (mask build, host sincos) + include/suqa_cpu.hpp:208-221 */
void or_apply_u1(or_state* s, uint32_t q, uint32_t qmask, double phase, uint64_t gc) {
    double sn, cs;
    sincos(phase, &sn, &cs);
    gate_ctx g = {s->re, s->im, gc | ((uint64_t)qmask << q), gc | (1ULL << q), 0, q, cs, sn};
    run_range(s->N, phase_range, &g);
}

/* include/suqa_cpu.hpp:223-253 (dense MCX); masks as built in src/suqa.cu:289-344 */
static void mcx_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    gate_ctx* g = (gate_ctx*)c;
    const uint64_t b = 1ULL << g->q;
    for (uint64_t i = lo; i < hi; ++i) {
        if ((i & g->m1) == g->m0) {
            uint64_t j = i & ~b;
            double t = g->re[i]; g->re[i] = g->re[j]; g->re[j] = t;
            t = g->im[i]; g->im[i] = g->im[j]; g->im[j] = t;
        }
    }
}
void or_apply_mcx(or_state* s, uint64_t control_mask, uint64_t mask_qs, uint32_t q_target) {
    const uint64_t b = 1ULL << q_target;
    gate_ctx g = {s->re, s->im, mask_qs | b, control_mask | b, 0, q_target, 0, 0};
    run_range(s->N, mcx_range, &g);
}

/* include/suqa_cpu.hpp:255-266; masks as built in src/suqa.cu:346-393 */
void or_apply_mcu1(or_state* s, uint64_t control_mask, uint64_t mask_qs, double phase) {
    double sn, cs;
    sincos(phase, &sn, &cs);
    gate_ctx g = {s->re, s->im, mask_qs, control_mask, 0, 0, cs, sn};
    run_range(s->N, phase_range, &g);
}

/* include/suqa_cpu.hpp:268-319 (dense SWAP), masks src/suqa.cu:396-408 */
static void swap_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    gate_ctx* g = (gate_ctx*)c;
    for (uint64_t i = lo; i < hi; ++i) {
        if ((i & g->m1) == g->m0) {
            uint64_t i1 = i | g->m2, i2 = i | (1ULL << g->q);
            double t = g->re[i1]; g->re[i1] = g->re[i2]; g->re[i2] = t;
            t = g->im[i1]; g->im[i1] = g->im[i2]; g->im[i2] = t;
        }
    }
}
void or_apply_swap(or_state* s, uint32_t q1, uint32_t q2, uint64_t gc) {
    const uint64_t b1 = 1ULL << q1, b2 = 1ULL << q2;
    gate_ctx g = {s->re, s->im, gc, gc | b1 | b2, b1, q2, 0, 0};
    run_range(s->N, swap_range, &g);
}

/* GPU-only reference API: src/suqa.cu:418-455 + kernel include/suqa_kernels.cuh:246-259.
 * Quirk kept: the guard is (i & gc) != 0, so the call is a no-op when gc == 0. */
typedef struct { double *re, *im; uint64_t gc; uint32_t q0; uint64_t size_mask; double* cph; } plist_ctx;
static void plist_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    plist_ctx* x = (plist_ctx*)c;
    for (uint64_t i = lo; i < hi; ++i) {
        if (i & x->gc) {
            uint64_t k = (i >> x->q0) & x->size_mask;
            double cx = x->cph[2 * k], cy = x->cph[2 * k + 1];
            double t = x->re[i];
            x->re[i] = x->re[i] * cx - x->im[i] * cy;
            x->im[i] = t * cy + x->im[i] * cx;
        }
    }
}
int or_apply_phase_list(or_state* s, uint32_t q0, uint32_t q_size, const double* phases, uint64_t gc) {
    if (q_size == 0 || q_size > 7) return -1;
    const uint32_t L = 1U << q_size;
    double cph[2 * 128];
    for (uint32_t k = 0; k < L; ++k) sincos(phases[k], &cph[2 * k + 1], &cph[2 * k]);
    plist_ctx x = {s->re, s->im, gc, q0, (uint64_t)L - 1, cph};
    run_range(s->N, plist_range, &x);
    return 0;
}

/* Pauli tensor-product rotation exp(i phase P).
 * Reference: src/suqa.cu:467-604 (dispatch, host sincos, supported patterns) and
 * include/suqa_cpu.hpp:338-527 (element updates).  Restated from the algebra
 * P|j> = w(j)|j ^ m>, m = X/Y qubits, w(j) = i^{#Y} (-1)^{popcount(j & (Y|Z qubits))},
 * so that a'[j] = c a[j] + i s w(j^m) a[j^m].  The update is written as
 * re' = re*c -/+ x*s, im' = im*c +/- y*s with x, y an exact permutation/negation of
 * the partner, the same floating-point operations as the reference's
 * util_rotate2, which makes the supported cases bit-identical to it. */
typedef struct {
    double *re, *im;
    uint64_t gc, flip, zy, pairbit;
    uint32_t ny;
    double c, s;
} pauli_ctx;

/* Apply out = c*a + s*(i*w*b) where i*w = i^(ny+1) * sign, written in the
 * reference's rotate2 form. */
static inline void rot_one(double* ar, double* ai, double br, double bi, int k, double c, double s,
                           double* outr, double* outi) {
    /* k = power of i in the factor (i * w), mod 4, sign included */
    switch (k & 3) {
    case 0: /* +1 */ *outr = *ar * c + br * s; *outi = *ai * c + bi * s; break;
    case 1: /* +i */ *outr = *ar * c - bi * s; *outi = *ai * c + br * s; break;
    case 2: /* -1 */ *outr = *ar * c - br * s; *outi = *ai * c - bi * s; break;
    default: /* -i */ *outr = *ar * c + bi * s; *outi = *ai * c - br * s; break;
    }
}

static void pauli_range(void* cx, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    pauli_ctx* p = (pauli_ctx*)cx;
    const uint64_t req = p->gc | p->pairbit;
    for (uint64_t j0 = lo; j0 < hi; ++j0) {
        if ((j0 & req) != p->gc) continue;
        if (p->flip == 0) {
            /* diagonal: a' = (c + i s w(j)) a, w = (-1)^parity (no Y when flip == 0) */
            int k = 1 + 2 * (__builtin_popcountll(j0 & p->zy) & 1);
            double r, i;
            rot_one(&p->re[j0], &p->im[j0], p->re[j0], p->im[j0], k, p->c, p->s, &r, &i);
            p->re[j0] = r;
            p->im[j0] = i;
        } else {
            const uint64_t j1 = j0 ^ p->flip;
            double a0r = p->re[j0], a0i = p->im[j0], a1r = p->re[j1], a1i = p->im[j1];
            /* factor for the update of j0 uses w(j1), and vice versa */
            int k0 = 1 + (int)p->ny + 2 * (__builtin_popcountll(j1 & p->zy) & 1);
            int k1 = 1 + (int)p->ny + 2 * (__builtin_popcountll(j0 & p->zy) & 1);
            double r0, i0, r1, i1;
            rot_one(&a0r, &a0i, a1r, a1i, k0, p->c, p->s, &r0, &i0);
            rot_one(&a1r, &a1i, a0r, a0i, k1, p->c, p->s, &r1, &i1);
            p->re[j0] = r0; p->im[j0] = i0;
            p->re[j1] = r1; p->im[j1] = i1;
        }
    }
}


/* Literal restatement of the reference's dense Pauli loops
 * (include/suqa_cpu.hpp:338-527, dispatch src/suqa.cu:467-581), used in strict
 * mode so that the oracle also reproduces the reference when the global control
 * mask overlaps the rotated qubits (the loops then alias elements). */
static inline void rot2(double* a, double* b, double c, double s) {
    double cpy = *a;
    *a = cpy * c - (*b) * s;
    *b = (*b) * c + cpy * s;
}
static inline void rot4(double* a, double* b, double* c2, double* d, double c, double s) {
    rot2(a, b, c, s);
    rot2(c2, d, c, s);
}
static void ref_pauli1(uint32_t p1, double* re, double* im, uint64_t m0, uint64_t m1, uint64_t mq1, double c,
                       double s, uint64_t N) {
    for (uint64_t i0 = 0; i0 < N; ++i0) {
        if ((i0 & m1) != m0) continue;
        uint64_t i[2] = {i0, i0 | mq1};
        switch (p1) {
        case 1: rot4(&re[i[0]], &im[i[1]], &re[i[1]], &im[i[0]], c, s); break;
        case 2: rot4(&re[i[0]], &re[i[1]], &im[i[0]], &im[i[1]], c, -s); break;
        case 3: rot4(&re[i[0]], &im[i[0]], &im[i[1]], &re[i[1]], c, s); break;
        }
    }
}
static void ref_pauli2(uint32_t p1, uint32_t p2, double* re, double* im, uint64_t m0, uint64_t m1, uint64_t mq1,
                       uint64_t mq2, double c, double s, uint64_t N) {
    for (uint64_t i0 = 0; i0 < N; ++i0) {
        if ((i0 & m1) != m0) continue;
        uint64_t i[4];
        i[0] = i0; i[1] = i0 | mq1; i[2] = i0 | mq2; i[3] = i[2] | i[1];
        if (p1 == 1 && p2 == 1) {
            rot4(&re[i[0]], &im[i[3]], &re[i[3]], &im[i[0]], c, s);
            rot4(&re[i[1]], &im[i[2]], &re[i[2]], &im[i[1]], c, s);
        } else if (p1 == 2 && p2 == 2) {
            rot4(&re[i[0]], &im[i[3]], &re[i[3]], &im[i[0]], c, -s);
            rot4(&re[i[1]], &im[i[2]], &re[i[2]], &im[i[1]], c, s);
        } else if (p1 == 3 && p2 == 3) {
            rot4(&re[i[0]], &im[i[0]], &re[i[3]], &im[i[3]], c, s);
            rot4(&re[i[1]], &im[i[1]], &re[i[2]], &im[i[2]], c, -s);
        } else if (p1 == 1 && p2 == 2) {
            rot4(&re[i[0]], &re[i[3]], &im[i[0]], &im[i[3]], c, -s);
            rot4(&re[i[2]], &re[i[1]], &im[i[2]], &im[i[1]], c, -s);
        } else if (p1 == 1 && p2 == 3) {
            rot4(&re[i[0]], &im[i[1]], &re[i[1]], &im[i[0]], c, s);
            rot4(&re[i[2]], &im[i[3]], &re[i[3]], &im[i[2]], c, -s);
        } else if (p1 == 2 && p2 == 3) {
            rot4(&re[i[0]], &re[i[1]], &im[i[0]], &im[i[1]], c, -s);
            rot4(&re[i[2]], &re[i[3]], &im[i[2]], &im[i[3]], c, s);
        }
    }
}
static void ref_pauli3(uint32_t p2, double* re, double* im, uint64_t m0, uint64_t m1, uint64_t mq1,
                       uint64_t mq2, uint64_t mq3, double c, double s, uint64_t N) {
    for (uint64_t i0 = 0; i0 < N; ++i0) {
        if ((i0 & m1) != m0) continue;
        uint64_t i[8];
        i[0] = i0; i[1] = i0 | mq1; i[2] = i0 | mq2; i[3] = i[2] | i[1];
        i[4] = i0 | mq3; i[5] = i[4] | i[1]; i[6] = i[4] | i[2]; i[7] = i[4] | i[3];
        if (p2 == 1) {
            rot4(&re[i[0]], &im[i[3]], &re[i[3]], &im[i[0]], c, s);
            rot4(&re[i[1]], &im[i[2]], &re[i[2]], &im[i[1]], c, s);
            rot4(&re[i[4]], &im[i[7]], &re[i[7]], &im[i[4]], c, -s);
            rot4(&re[i[5]], &im[i[6]], &re[i[6]], &im[i[5]], c, -s);
        } else if (p2 == 2) {
            rot4(&re[i[0]], &im[i[3]], &re[i[3]], &im[i[0]], c, -s);
            rot4(&re[i[1]], &im[i[2]], &re[i[2]], &im[i[1]], c, s);
            rot4(&re[i[4]], &im[i[7]], &re[i[7]], &im[i[4]], c, s);
            rot4(&re[i[5]], &im[i[6]], &re[i[6]], &im[i[5]], c, -s);
        } else {
            rot4(&re[i[0]], &im[i[0]], &re[i[3]], &im[i[3]], c, s);
            rot4(&re[i[5]], &im[i[5]], &re[i[6]], &im[i[6]], c, s);
            rot4(&re[i[1]], &im[i[1]], &re[i[2]], &im[i[2]], c, -s);
            rot4(&re[i[4]], &im[i[4]], &re[i[7]], &im[i[7]], c, -s);
        }
    }
}
static int ref_pauli(or_state* st, uint32_t k, const uint32_t* qubits, const uint32_t* paulis, double phase,
                     uint64_t gc) {
    double sph, cph;
    sincos(phase, &sph, &cph);
    uint64_t m0 = gc, m1 = gc;
    for (uint32_t t = 0; t < k; ++t) m1 |= 1ULL << qubits[t];
    uint32_t p[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    for (uint32_t t = 0; t < k; ++t) { p[t] = paulis[t]; q[t] = qubits[t]; }
    uint32_t tt;
#define OR_SWAP2(a, b) do { tt = p[a]; p[a] = p[b]; p[b] = tt; tt = q[a]; q[a] = q[b]; q[b] = tt; } while (0)
    if (k == 1) {
        ref_pauli1(p[0], st->re, st->im, m0, m1, 1ULL << q[0], cph, sph, st->N);
    } else if (k == 2) {
        if (p[0] > p[1]) OR_SWAP2(0, 1);
        ref_pauli2(p[0], p[1], st->re, st->im, m0, m1, 1ULL << q[0], 1ULL << q[1], cph, sph, st->N);
    } else {
        if (p[0] > p[1]) OR_SWAP2(0, 1);
        if (p[1] > p[2]) OR_SWAP2(1, 2);
        if (p[0] > p[1]) OR_SWAP2(0, 1);
        ref_pauli3(p[0], st->re, st->im, m0, m1, 1ULL << q[0], 1ULL << q[1], 1ULL << q[2], cph, sph, st->N);
    }
#undef OR_SWAP2
    return 0;
}

/* supported set of the reference: src/suqa.cu:484-581 */
static int ref_supported(uint32_t k, const uint32_t* ps) {
    if (k == 1 || k == 2) return 1;
    if (k == 3) {
        uint32_t a[3] = {ps[0], ps[1], ps[2]}, t;
        if (a[0] > a[1]) { t = a[0]; a[0] = a[1]; a[1] = t; }
        if (a[1] > a[2]) { t = a[1]; a[1] = a[2]; a[2] = t; }
        if (a[0] > a[1]) { t = a[0]; a[0] = a[1]; a[1] = t; }
        return a[2] == 3 && a[0] == a[1];
    }
    return 0;
}

int or_apply_pauli(or_state* s, uint32_t k, const uint32_t* qubits, const uint32_t* paulis,
                   double phase, uint64_t gc, int strict) {
    if (k == 0 || k > 64) return -1;
    if (strict && !ref_supported(k, paulis)) return -1;
    if (strict) {
        uint64_t qm = 0;
        for (uint32_t t = 0; t < k; ++t) qm |= 1ULL << qubits[t];
        if (qm & gc) return ref_pauli(s, k, qubits, paulis, phase, gc);
    }
    pauli_ctx p;
    memset(&p, 0, sizeof(p));
    p.re = s->re; p.im = s->im; p.gc = gc;
    /* Reference quirk: for a two-qubit string of one X and one Y, its XY kernel
     * (include/suqa_cpu.hpp:408-411, include/suqa_kernels.cuh:379-396) applies
     * exp(i phase Y(x)X) with the roles of the two qubits exchanged.  The strict
     * (reference-compatible) mode reproduces that; strict=0 is the exact form. */
    uint32_t pl[64];
    for (uint32_t t = 0; t < k && t < 64; ++t) pl[t] = paulis[t];
    if (strict && k == 2 && ((pl[0] == 1 && pl[1] == 2) || (pl[0] == 2 && pl[1] == 1))) {
        uint32_t t = pl[0]; pl[0] = pl[1]; pl[1] = t;
    }
    for (uint32_t t = 0; t < k; ++t) {
        const uint64_t b = 1ULL << qubits[t];
        if (pl[t] < 1 || pl[t] > 3) return -1;
        if (pl[t] == 1 || pl[t] == 2) p.flip |= b;
        if (pl[t] == 2 || pl[t] == 3) p.zy |= b;
        if (pl[t] == 2) p.ny++;
    }
    p.pairbit = p.flip & (~p.flip + 1ULL); /* lowest flipped bit */
    sincos(phase, &p.s, &p.c);
    run_range(s->N, pauli_range, &p);
    return 0;
}

/* src/suqa.cu:611-661: QFT as H + CU1(+-2pi/2^m) under the current gc mask */
static void qft_crm(or_state* s, uint32_t qc, uint32_t qt, int m, uint64_t gc) {
    int am = m > 0 ? m : -m;
    double rphase = 2.0 * M_PI / (double)(1U << am);
    if (m <= 0) rphase *= -1;
    const uint64_t mask_qs = (1ULL << qt) | gc | (1ULL << qc);
    or_apply_mcu1(s, mask_qs, mask_qs, rphase);
}
void or_apply_qft(or_state* s, uint32_t k, const uint32_t* q, uint64_t gc) {
    for (int o = (int)k - 1; o >= 0; o--) {
        or_apply_h(s, q[o], gc);
        for (int in = o - 1; in >= 0; in--) qft_crm(s, q[in], q[o], 1 + (o - in), gc);
    }
}
void or_apply_qft_inverse(or_state* s, uint32_t k, const uint32_t* q, uint64_t gc) {
    for (int o = 0; o < (int)k; o++) {
        for (int in = 0; in < o; in++) qft_crm(s, q[in], q[o], -1 - (o - in), gc);
        or_apply_h(s, q[o], gc);
    }
}

/* ---- measurement ------------------------------------------------------------ */
/* include/suqa_cpu.hpp:554-573 (sequential sum, re^2 then im^2 per index) */
typedef struct { const double *re, *im; uint64_t m, v; double part[256]; } filt_ctx;
static void filt_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    filt_ctx* f = (filt_ctx*)c;
    double r = 0.0, t;
    for (uint64_t i = lo; i < hi; ++i) {
        if ((i & f->m) == f->v) {
            t = f->re[i]; r += t * t;
            t = f->im[i]; r += t * t;
        }
    }
    f->part[tid] = r;
}
static double filtered_sum(or_state* s, uint64_t m, uint64_t v) {
    filt_ctx f;
    f.re = s->re; f.im = s->im; f.m = m; f.v = v;
    memset(f.part, 0, sizeof(f.part));
    run_range(s->N, filt_range, &f);
    double r = 0.0;
    for (int t = 0; t < g_threads; ++t) r += f.part[t];
    return r;
}
double or_prob1(or_state* s, uint32_t q) { return filtered_sum(s, 1ULL << q, 1ULL << q); }

/* include/suqa_cpu.hpp:532-551 */
typedef struct { double *re, *im; uint32_t q; uint64_t val; } zero_ctx;
static void zero_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    zero_ctx* z = (zero_ctx*)c;
    for (uint64_t i = lo; i < hi; ++i)
        if (((i >> z->q) & 1ULL) == z->val) { z->re[i] = 0.0; z->im[i] = 0.0; }
}

/* src/suqa.cu:673-696: c = r < prob1; zero the other branch; vnormalize */
uint32_t or_measure_qbit(or_state* s, uint32_t q, double r) {
    double p1 = or_prob1(s, q);
    uint32_t c = (uint32_t)(r < p1);
    zero_ctx z = {s->re, s->im, q, (uint64_t)(c ^ 1U)};
    run_range(s->N, zero_range, &z);
    or_vnormalize(s);
    return c;
}

/* src/suqa.cu:730-738: the flip after a 1 outcome is an apply_x, so it runs
 * under the current global control mask */
void or_apply_reset(or_state* s, uint32_t q, double r, uint64_t gc) {
    if (or_measure_qbit(s, q, r)) or_apply_x(s, q, gc);
}

/* src/suqa.cu:705-727 + include/suqa_cpu.hpp:575-591 */
double or_prob_filter(or_state* s, uint64_t mask_qs, uint64_t mask) {
    return filtered_sum(s, mask_qs, mask);
}

/* ---- QMS W oracle: include/qms.cuh:245-309 (dense CPU branch) ---------------- */
typedef struct { double *re, *im; uint32_t q_acc; uint64_t me; uint32_t sh, eold; double cf; } w_ctx;
static void w_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    (void)tid;
    w_ctx* w = (w_ctx*)c;
    for (uint64_t i = lo; i < hi; ++i) {
        uint64_t j = i & ~(1ULL << w->q_acc);
        uint32_t Enew = (uint32_t)((i & w->me) >> w->sh);
        double dE = (Enew * w->cf - w->eold * w->cf);
        double fs1, fs2;
        if (dE > 0) {
            fs1 = exp(-dE / 2.0);
            fs2 = sqrt(1.0 - fs1 * fs1);
        } else {
            fs1 = 1.0;
            fs2 = 0.0;
        }
        double t = w->re[j];
        w->re[j] = fs2 * w->re[j] + fs1 * w->re[i];
        w->re[i] = fs1 * t - fs2 * w->re[i];
        t = w->im[j];
        w->im[j] = fs2 * w->im[j] + fs1 * w->im[i];
        w->im[i] = fs1 * t - fs2 * w->im[i];
    }
}
typedef struct { w_ctx w; uint64_t base; } w_off_ctx;
static void w_off_range(void* c, uint64_t lo, uint64_t hi, int tid) {
    w_off_ctx* o = (w_off_ctx*)c;
    w_range(&o->w, lo + o->base, hi + o->base, tid);
}
void or_apply_qms_w(or_state* s, uint32_t q_acc, uint64_t mask_enew, uint32_t shift,
                    uint32_t E_old, double c_factor) {
    w_off_ctx o;
    o.w.re = s->re; o.w.im = s->im; o.w.q_acc = q_acc; o.w.me = mask_enew;
    o.w.sh = shift; o.w.eold = E_old; o.w.cf = c_factor;
    o.base = s->N / 2; /* loop over the upper half: the acceptance qubit is the MSB */
    run_range(s->N / 2, w_off_range, &o);
}

/* ---- PCG32: include/pcg32.h:53-68 (seed, nextUInt), :121-130 (nextDouble) ---- */
#define OR_PCG_MULT 0x5851f42d4c957f2dULL
uint32_t or_pcg_next(or_pcg* g) {
    uint64_t old = g->state;
    g->state = old * OR_PCG_MULT + g->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31));
}
void or_pcg_seed(or_pcg* g, uint64_t initstate, uint64_t initseq) {
    g->state = 0U;
    g->inc = (initseq << 1u) | 1u;
    or_pcg_next(g);
    g->state += initstate;
    or_pcg_next(g);
}
double or_pcg_doub(or_pcg* g) {
    union { uint64_t u; double d; } x;
    x.u = ((uint64_t)or_pcg_next(g) << 20) | 0x3ff0000000000000ULL;
    return x.d - 1.0;
}
