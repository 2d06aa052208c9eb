// Batched Szegedy-walk annealing (QSA) on Ising rings with integer couplings
// and no field: the reference's walk (include/qsa.cuh:616-756, driver loop
// src/qsa.cu:159-268) in the general form of its own commented-out rotation and
// reflection (qsa.cuh:372-418), for many walks at once.
//
// Registers per walk: system x and copy x~ (s qubits each), the acceptance
// qubit, the q-qubit walk-phase register and an energy-difference register.  The
// ring's Hamiltonian is diagonal with integer spectrum, so phase estimation of
// the energy difference is exact and every "estimate, act on the level,
// un-estimate" block equals its action applied directly as a function of
// dE = H(x~) - H(x): the energy register is never stored.  The walk-phase
// register's branches are independent: branch k carries W^k psi, so a walk step
// needs v_k = W^k psi for k < L = 2^q, the overlaps g_k = <psi, v_k> (which give
// the register's readout distribution after the inverse QFT) and sum_k v_k
// (the state after reading zero).
//
// State: real amplitudes psi[acc][d][x], d = x XOR x~, 2^(2s+1) per walk.  For
// the step's move C the operator W (L1 H_C R S0 R^T H_C L1 H_C R S0 R^T H_C)
// only ever mixes the 16 amplitudes
//     x in {x0, x0^d', x0^e_C, x0^d'^e_C},  d in {d', d'^e_C},  acc in {0, 1}
// (d' = d without bit C), so one thread keeps such an orbit in registers and
// applies W L-1 times without touching memory.  Orbits with d' = 0 have 8
// amplitudes; they run duplicated in the 16 registers and count half.
//
// Per step (algo 0: one launch of k_walk_step and one of k_walk_measure):
//   k_walk_step     every orbit: load psi (scaled by the last normalisation, or
//                   the initial state), L-1 applications of W, per-k warp sums
//                   of <psi, v_k> accumulated in FP64, store sum_k v_k;
//   k_walk_measure  per walk: g_k, P(m), the register readout with q draws,
//                   restart on a nonzero value, the next move and temperature.
// algo 1 and 2 work per orbit class instead (the section "Orbit classes" below):
// k_cls_keys and k_cls_table once per batch (or k_cls_prep every step), then
// per step one orbit pass -- k_walk_step_sorted2 (FP32, 16 warps, orbit order
// table, class products on the tensor cores), k_walk_step_sorted (FP32, 8
// warps) or k_walk_step_cls (FP64, and batches with too many classes) -- and
// k_walk_measure.  k_walk_readout reads the spins of every completed walk.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "sq.h"

namespace sqi {
void set_error(const char* msg);
}

namespace sqw {

constexpr int kThreads = 256;
constexpr int kOrbitsPerThread = 4;
constexpr int kOrbitsPerCta = kThreads * kOrbitsPerThread;
constexpr int kMaxL = 64;
constexpr int kMaxJ = 8;
constexpr int kMaxD = 2 * 12 * kMaxJ;  // largest |dE|

struct WalkDev {
    int s, q, stages, per;
    uint32_t nominal, cap;
    double beta;
    uint64_t seed;
    uint64_t state_off;  // first element of psi[acc][d][x]
    uint64_t trace_off;  // first p0 trace slot
    uint32_t e_off;      // first entry of the energy table (2^s int32)
    uint32_t cta0, ncta; // CTAs of the walk in the step grid
    int dmax;            // largest |dE| of the ring
    uint32_t slot0;      // class-table temperature slot of stage 0 (algo 1)
    uint32_t jplane[5];  // bit planes of J_b + joff over the bonds b < s
    int joff, jnp;       // offset making every J_b + joff >= 0; planes in use
    uint64_t ord_off;    // first entry of the walk's orbit order table (16-warp orbit pass)
};

struct WalkRec {
    uint64_t rng_state, rng_inc;
    double beta_k;   // inverse temperature of the next step
    double scale;    // factor of the stored state
    double last_p0;  // P(zero walk phase) at the last step
    uint32_t C;      // move of the next step
    uint32_t fresh;  // the next step starts from the initial state
    uint32_t att;    // completed steps of the current attempt
    uint32_t total, restarts;
    uint32_t status; // 0 running, 1 capped, 2 completed, 3 read out
    uint32_t readout, pad;
};

__host__ __device__ inline uint32_t ins0(uint32_t p, int b) {
    return ((p >> b) << (b + 1)) | (p & ((1u << b) - 1u));
}

__host__ __device__ inline uint32_t norbits(int s) {
    return (1u << (s - 1)) + ((1u << (s - 1)) - 1u) * (1u << (s - 2));
}

__device__ __forceinline__ uint32_t pcg_next(uint64_t& st, uint64_t inc) {
    const uint64_t old = st;
    st = old * 6364136223846793005ULL + inc;
    const uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (x >> rot) | (x << ((0u - rot) & 31u));
}

__device__ __forceinline__ double pcg_doub(uint64_t& st, uint64_t inc) {
    const uint64_t bits = ((uint64_t)pcg_next(st, inc) << 20) | 0x3ff0000000000000ULL;
    return __longlong_as_double((long long)bits) - 1.0;
}

// qsa::draw_C (qsa.cuh:334-343) with weight sums (i+1)/s.  The last sum is exactly
// 1 and u < 1, so the loop always returns; the fallback keeps C a valid spin.
__device__ __forceinline__ uint32_t draw_move(uint64_t& st, uint64_t inc, int s) {
    const double u = pcg_doub(st, inc);
    for (int i = 0; i < s; ++i)
        if (u < (double)(i + 1) / (double)s) return (uint32_t)i;
    return (uint32_t)(s - 1);
}

// register slot of orbit coordinates (a: x ^= d', b: x ^= e_C, c: d ^= e_C, acc)
#define SLOT(a, b, c, acc) (((a) << 3) | ((b) << 2) | ((c) << 1) | (acc))

// The walk W on one orbit, scalar form (FP64).  The Hadamards run unnormalised;
// the first rotation of each H R S0 R^T H group carries their factor 1/2.
template <typename T>
struct Orbit {
    T v[16];
    T e[8], r[8], he[8], hr[8];  // rotation per position (a, b, c)
    uint32_t zmask;              // positions with dE = 0

    __device__ __forceinline__ void setup(const T (&ce)[8], const T (&cr)[8], uint32_t z) {
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            e[p] = ce[p];
            r[p] = cr[p];
            he[p] = (T)0.5 * ce[p];
            hr[p] = (T)0.5 * cr[p];
        }
        zmask = z;
    }
    __device__ __forceinline__ void lam() {
#pragma unroll
        for (int p = 0; p < 8; ++p)
            if ((zmask >> p) & 1u) v[2 * p] = -v[2 * p];
    }
    // Hadamard on copy bit C, unnormalised: the copy bit is b ^ c
    __device__ __forceinline__ void hc() {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int acc = 0; acc < 2; ++acc) {
                    const T A = v[SLOT(a, b, 0, acc)], B = v[SLOT(a, b, 1, acc)];
                    if (b == 0) {
                        v[SLOT(a, b, 0, acc)] = A + B;
                        v[SLOT(a, b, 1, acc)] = A - B;
                    } else {
                        v[SLOT(a, b, 1, acc)] = A + B;
                        v[SLOT(a, b, 0, acc)] = B - A;
                    }
                }
    }
    // ptp(Y, -acos e) on acc = [[e, -r], [r, e]], times 1/2
    __device__ __forceinline__ void rot_half() {
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const T p0 = v[2 * p], p1 = v[2 * p + 1];
            v[2 * p] = he[p] * p0 - hr[p] * p1;
            v[2 * p + 1] = hr[p] * p0 + he[p] * p1;
        }
    }
    __device__ __forceinline__ void rot_inv() {
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const T p0 = v[2 * p], p1 = v[2 * p + 1];
            v[2 * p] = e[p] * p0 + r[p] * p1;
            v[2 * p + 1] = e[p] * p1 - r[p] * p0;
        }
    }
    // swap x <-> x~ on acc = 0: (a, b, c) <-> (a ^ 1, b ^ c, c)
    __device__ __forceinline__ void sw0() {
        T t;
        t = v[SLOT(0, 0, 0, 0)]; v[SLOT(0, 0, 0, 0)] = v[SLOT(1, 0, 0, 0)]; v[SLOT(1, 0, 0, 0)] = t;
        t = v[SLOT(0, 1, 0, 0)]; v[SLOT(0, 1, 0, 0)] = v[SLOT(1, 1, 0, 0)]; v[SLOT(1, 1, 0, 0)] = t;
        t = v[SLOT(0, 0, 1, 0)]; v[SLOT(0, 0, 1, 0)] = v[SLOT(1, 1, 1, 0)]; v[SLOT(1, 1, 1, 0)] = t;
        t = v[SLOT(0, 1, 1, 0)]; v[SLOT(0, 1, 1, 0)] = v[SLOT(1, 0, 1, 0)]; v[SLOT(1, 0, 1, 0)] = t;
    }
    __device__ __forceinline__ void walk() {
        lam(); hc(); rot_half(); sw0(); rot_inv(); hc();
        lam(); hc(); rot_half(); sw0(); rot_inv(); hc();
    }
    // v = psi on entry; returns with v = sum_{k<L} W^k psi, red[k] += <psi, W^k psi>
    __device__ __forceinline__ void run(int L, T wgt, int lane, double* red) {
        T psi[16], S[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            psi[j] = v[j];
            S[j] = (T)0;
        }
        for (int k = 0; k < L; ++k) {
            T dot = (T)0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                dot += psi[j] * v[j];
                S[j] += v[j];
            }
            dot *= wgt;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, off);
            if (lane == 0) red[k] += (double)dot;
            if (k < L - 1) walk();
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = S[j];
    }
};

// FP32 form on Blackwell's packed f32x2 arithmetic: each 64-bit register holds
// the pair (b = 0, b = 1) of one (a, c, acc).  The Hadamard on the copy bit is
// then two packed FMAs with sign vectors, the swap renames pairs (c = 0) or
// swaps their halves (c = 1), and both rotations use (e, r) / sqrt(2), which
// carries the factor 1/2 of the two unnormalised Hadamards around them.
typedef unsigned long long f2;

__device__ __forceinline__ f2 pk2(float x, float y) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ void up2(f2 v, float& x, float& y) { asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v)); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 swap2(f2 v) {
    float x, y;
    up2(v, x, y);
    return pk2(y, x);
}

struct OrbitF2 {
    f2 P[2][2][2];      // [a][c][acc], halves b = 0, 1
    f2 A[2][2], B[2][2], NB[2][2], SG[2][2];  // per (a, c): e/sqrt2, r/sqrt2, -r/sqrt2, L1 sign on acc = 0

    __device__ __forceinline__ void setup(const float (&ce)[8], const float (&cr)[8], uint32_t z) {
        const float h = 0.70710678118654752f;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int p0 = (a << 2) | c, p1 = (a << 2) | 2 | c;  // positions (a, b = 0, c), (a, b = 1, c)
                A[a][c] = pk2(h * ce[p0], h * ce[p1]);
                B[a][c] = pk2(h * cr[p0], h * cr[p1]);
                NB[a][c] = pk2(-h * cr[p0], -h * cr[p1]);
                SG[a][c] = pk2(((z >> p0) & 1u) ? -1.f : 1.f, ((z >> p1) & 1u) ? -1.f : 1.f);
            }
    }
    __device__ __forceinline__ void load(const float (&v)[16]) {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int acc = 0; acc < 2; ++acc) P[a][c][acc] = pk2(v[SLOT(a, 0, c, acc)], v[SLOT(a, 1, c, acc)]);
    }
    __device__ __forceinline__ void lam() {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c) P[a][c][0] = mul2(P[a][c][0], SG[a][c]);
    }
    // copy bit = b ^ c: new c0 = (A + B, B - A), new c1 = (A - B, A + B) over the halves b = 0, 1
    __device__ __forceinline__ void hc(f2 pm, f2 mp) {
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int acc = 0; acc < 2; ++acc) {
                const f2 X = P[a][0][acc], Y = P[a][1][acc];
                P[a][0][acc] = fma2(X, pm, Y);
                P[a][1][acc] = fma2(Y, mp, X);
            }
    }
    __device__ __forceinline__ void rot() {  // [[e, -r], [r, e]] / sqrt2
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const f2 p0 = P[a][c][0], p1 = P[a][c][1];
                P[a][c][0] = fma2(NB[a][c], p1, mul2(A[a][c], p0));
                P[a][c][1] = fma2(B[a][c], p0, mul2(A[a][c], p1));
            }
    }
    __device__ __forceinline__ void rot_t() {  // [[e, r], [-r, e]] / sqrt2
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const f2 p0 = P[a][c][0], p1 = P[a][c][1];
                P[a][c][0] = fma2(B[a][c], p1, mul2(A[a][c], p0));
                P[a][c][1] = fma2(NB[a][c], p0, mul2(A[a][c], p1));
            }
    }
    __device__ __forceinline__ void sw0() {
        f2 t = P[0][0][0];
        P[0][0][0] = P[1][0][0];
        P[1][0][0] = t;
        t = P[0][1][0];
        P[0][1][0] = swap2(P[1][1][0]);
        P[1][1][0] = swap2(t);
    }
    __device__ __forceinline__ void walk(f2 pm, f2 mp) {
        lam(); hc(pm, mp); rot(); sw0(); rot_t(); hc(pm, mp);
        lam(); hc(pm, mp); rot(); sw0(); rot_t(); hc(pm, mp);
    }
    // v = psi on entry; returns with v = sum_{k<L} W^k psi; red32[k] = the warp's
    // FP32 sum of <psi, W^k psi> (summed over warps and orbits in FP64 later)
    __device__ __forceinline__ void run(float (&v)[16], int L, float wgt, int lane, float* red32) {
        load(v);
        const f2 pm = pk2(1.f, -1.f), mp = pk2(-1.f, 1.f);
        f2 psi[2][2][2], S[2][2][2];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int acc = 0; acc < 2; ++acc) {
                    psi[a][c][acc] = P[a][c][acc];
                    S[a][c][acc] = 0ull;
                }
        for (int k = 0; k < L; ++k) {
            f2 d2 = 0ull;
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int acc = 0; acc < 2; ++acc) {
                        d2 = fma2(psi[a][c][acc], P[a][c][acc], d2);
                        S[a][c][acc] = add2(S[a][c][acc], P[a][c][acc]);
                    }
            float x, y;
            up2(d2, x, y);
            float dot = (x + y) * wgt;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, off);
            if (lane == 0) red32[k] = dot;
            if (k < L - 1) walk(pm, mp);
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int acc = 0; acc < 2; ++acc) up2(S[a][c][acc], v[SLOT(a, 0, c, acc)], v[SLOT(a, 1, c, acc)]);
    }
};

template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 8 ? 1 : 2)
k_walk_step(const WalkDev* __restrict__ walks, const int* __restrict__ cta_walk, const WalkRec* __restrict__ recs,
            const int* __restrict__ energies, T* __restrict__ states, double* __restrict__ partial) {
    const int w = cta_walk[blockIdx.x];
    const WalkDev& W = walks[w];
    const WalkRec& R = recs[w];
    if (R.status != 0) return;  // uniform over the CTA
    __shared__ double red[kThreads / 32][kMaxL];                    // FP64 path
    __shared__ float red32[kThreads / 32][kOrbitsPerThread][kMaxL];  // FP32 path
    __shared__ T tab_e[kMaxD + 1], tab_r[kMaxD + 1];
    const int s = W.s, C = (int)R.C, L = 1 << W.q;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (kThreads / 32) * kMaxL; i += blockDim.x) (&red[0][0])[i] = 0.0;
    for (int i = threadIdx.x; i < (kThreads / 32) * kOrbitsPerThread * kMaxL; i += blockDim.x)
        (&red32[0][0][0])[i] = 0.f;
    for (int k = threadIdx.x; k <= W.dmax; k += blockDim.x) {
        double e = 1.0, r = 0.0;
        if (k > 0) {
            e = exp(-0.5 * R.beta_k * (double)k);
            r = sqrt(1.0 - e * e);
        }
        tab_e[k] = (T)e;
        tab_r[k] = (T)r;
    }
    __syncthreads();
    const uint32_t N = 1u << s;
    const uint64_t NN = (uint64_t)N * N;
    const uint32_t norb = norbits(s);
    const uint32_t eC = 1u << C;
    const int* E = energies + W.e_off;
    T* st = states + W.state_off;
    const bool fresh = R.fresh != 0;
    const T scale = (T)R.scale;
    const T init = (T)(1.0 / sqrt((double)N));
    const uint32_t first = (blockIdx.x - W.cta0) * (uint32_t)kOrbitsPerCta;
    for (int it = 0; it < kOrbitsPerThread; ++it) {
        const uint32_t o = first + (uint32_t)(it * kThreads) + threadIdx.x;
        const bool active = o < norb;
        if (!__any_sync(0xffffffffu, active)) continue;  // warp-uniform
        uint32_t dp = 0, x0 = 0;
        bool single = true;
        if (active) {
            const uint32_t nb = 1u << (s - 1);
            if (o < nb) {
                x0 = ins0(o, C);
            } else {
                single = false;
                const uint32_t o2 = o - nb;
                const uint32_t di = 1u + (o2 >> (s - 2)), ri = o2 & ((1u << (s - 2)) - 1u);
                dp = ins0(di, C);
                const int p = __ffs((int)dp) - 1;
                x0 = ins0(ins0(ri, min(p, C)), max(p, C));
            }
        }
        T v[16], ce[8], cr[8];
        uint32_t zmask = 0;
#pragma unroll
        for (int pos = 0; pos < 8; ++pos) {
            const int a = pos >> 2, b = (pos >> 1) & 1, c = pos & 1;
            const uint32_t x = x0 ^ (a ? dp : 0u) ^ (b ? eC : 0u);
            const uint32_t d = dp ^ (c ? eC : 0u);
            int dE = 0;
            if (active) dE = E[x ^ d] - E[x];
            const int k = dE > 0 ? dE : 0;
            ce[pos] = tab_e[k];
            cr[pos] = tab_r[k];
            if (dE == 0) zmask |= 1u << pos;
#pragma unroll
            for (int acc = 0; acc < 2; ++acc) {
                T val = (T)0;
                if (active) {
                    if (fresh) {
                        val = (single && c == 0 && acc == 0) ? init : (T)0;
                    } else if (!(single && a == 1)) {
                        val = st[(uint64_t)acc * NN + (uint64_t)d * N + x] * scale;
                    }
                }
                v[SLOT(a, b, c, acc)] = val;
            }
        }
        if (single) {
#pragma unroll
            for (int j = 0; j < 8; ++j) v[8 + j] = v[j];
        }
        const T wgt = single ? (T)0.5 : (T)1;
        if constexpr (sizeof(T) == 4) {
            OrbitF2 ob;
            ob.setup(ce, cr, zmask);
            ob.run(v, L, wgt, lane, red32[warp][it]);
        } else {
            Orbit<T> ob;
            ob.setup(ce, cr, zmask);
#pragma unroll
            for (int j = 0; j < 16; ++j) ob.v[j] = v[j];
            ob.run(L, wgt, lane, red[warp]);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = ob.v[j];
        }
        if (active) {
#pragma unroll
            for (int pos = 0; pos < 8; ++pos) {
                const int a = pos >> 2, b = (pos >> 1) & 1, c = pos & 1;
                if (single && a == 1) continue;
                const uint32_t x = x0 ^ (a ? dp : 0u) ^ (b ? eC : 0u);
                const uint32_t d = dp ^ (c ? eC : 0u);
#pragma unroll
                for (int acc = 0; acc < 2; ++acc) st[(uint64_t)acc * NN + (uint64_t)d * N + x] = v[SLOT(a, b, c, acc)];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < L) {
        double sum = 0.0;
        for (int wp = 0; wp < kThreads / 32; ++wp) {
            sum += red[wp][threadIdx.x];
            for (int it = 0; it < kOrbitsPerThread; ++it) sum += (double)red32[wp][it][threadIdx.x];
        }
        partial[(uint64_t)blockIdx.x * kMaxL + threadIdx.x] = sum;
    }
}

// ---------------------------------------------------------------------------
// Orbit classes (algo 1).  W on an orbit depends only on the energy differences
// at its four a = 0 positions (the a = 1 ones are their negatives), and a step
// has few distinct such signatures (62-71 among 131,328 orbits of a 10-spin
// ring).  Per class: W (16 x 16), A = (W + W^T)/2 = V diag(lambda) V^T,
// Q = sum_{k<L} W^k and d_{k,i} = v_i^T W^k v_i.  W is real orthogonal, so
// <psi, W^k psi> = psi^T T_k(A) psi (T_k: Chebyshev) and T_k(lambda_i) = d_{k,i}:
// an orbit adds the 16 values (V^T psi)_i^2 to its class, g_k = sum_{c,i} N_{c,i}
// d_{c,k,i}, and the state after reading zero is Q psi per orbit.  The d table
// comes from the powers of W themselves (errors grow with k, not with k^2 as
// T_k(lambda) evaluated from an approximate lambda would).  The class data depend
// only on (key, beta_k, q): algo 1 prepares them once per batch for every distinct
// key and stage temperature (k_cls_table; rings with couplings +-1 have a few dozen
// keys in all), algo 2 (and algo 1 when that table would not fit) per walk and step
// (k_cls_prep).

constexpr int kMaxCls = 96;
constexpr int kClsOrbitsPerThread = 32;
constexpr int kClsOrbitsPerCta = kThreads * kClsOrbitsPerThread;
constexpr int kClsStride = 16 * 16 + 16 * 16 + kMaxL * 16;  // V^T, Q, d[k][i]
constexpr int kMaxMoves = 12;
constexpr uint64_t kTableBudget = 4ull << 30;  // largest batch class table (bytes)

__device__ __forceinline__ bool orbit_decode(uint32_t o, int s, int C, uint32_t& dp, uint32_t& x0) {
    const uint32_t nb = 1u << (s - 1);
    if (o < nb) {
        dp = 0;
        x0 = ins0(o, C);
        return true;
    }
    const uint32_t o2 = o - nb;
    const uint32_t di = 1u + (o2 >> (s - 2)), ri = o2 & ((1u << (s - 2)) - 1u);
    dp = ins0(di, C);
    const int p = __ffs((int)dp) - 1;
    x0 = ins0(ins0(ri, min(p, C)), max(p, C));
    return false;
}

// signature key: dE at positions (a, b, c) = (0, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1),
// each + 256 in 9 bits (never 0)
__device__ __forceinline__ uint64_t orbit_key(const int* E, uint32_t x0, uint32_t dp, uint32_t eC) {
    uint64_t key = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t x = x0 ^ ((j & 1) ? eC : 0u);
        const uint32_t d = dp ^ ((j & 2) ? eC : 0u);
        key |= (uint64_t)(E[x ^ d] - E[x] + 256) << (9 * j);
    }
    return key;
}

// One CTA per (walk, move): the sorted distinct keys of the walk's orbits for that move.
__global__ void k_cls_keys(const WalkDev* __restrict__ walks, const int* __restrict__ energies,
                           const int* __restrict__ job_walk, const int* __restrict__ job_move,
                           unsigned long long* __restrict__ keys, uint32_t* __restrict__ ncls) {
    const int w = job_walk[blockIdx.x], C = job_move[blockIdx.x];
    const WalkDev& W = walks[w];
    __shared__ unsigned long long table[512];
    __shared__ unsigned long long arr[512];
    __shared__ unsigned int count, overflow;
    for (int i = threadIdx.x; i < 512; i += blockDim.x) table[i] = 0ull;
    if (threadIdx.x == 0) {
        count = 0;
        overflow = 0;
    }
    __syncthreads();
    const int s = W.s;
    const uint32_t norb = norbits(s), eC = 1u << C;
    const int* E = energies + W.e_off;
    for (uint32_t o = threadIdx.x; o < norb; o += blockDim.x) {
        uint32_t dp, x0;
        orbit_decode(o, s, C, dp, x0);
        const unsigned long long key = orbit_key(E, x0, dp, eC);
        uint32_t h = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 55);
        bool done = false;
        for (int probe = 0; probe < 512 && !done; ++probe) {  // bounded: 512 slots
            const unsigned long long prev = atomicCAS(&table[h], 0ull, key);
            if (prev == 0ull || prev == key) done = true;
            h = (h + 1u) & 511u;
        }
        if (!done) overflow = 1;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x)
        if (table[i] != 0ull) arr[atomicAdd(&count, 1u)] = table[i];
    __syncthreads();
    const uint32_t n = count;
    unsigned long long* out = keys + ((uint64_t)w * kMaxMoves + C) * kMaxCls;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t rank = 0;
        for (uint32_t j = 0; j < n; ++j) rank += arr[j] < arr[i] ? 1u : 0u;
        if (rank < (uint32_t)kMaxCls) out[rank] = arr[i];
    }
    if (threadIdx.x == 0) ncls[(uint64_t)w * kMaxMoves + C] = overflow ? 0xffffffffu : n;
}

// 16 x 16 product by one warp: Z = X Y (row-major, padded rows of 17); each lane
// computes 8 entries of one row
template <typename T>
__device__ __forceinline__ void warp_matmul(T (*Z)[17], const T (*X)[17], const T (*Y)[17], int lane) {
    const int row = lane >> 1, c0 = (lane & 1) * 8;
    T acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = (T)0;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const T xv = X[row][m];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] += xv * Y[m][c0 + j];
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 8; ++j) Z[row][c0 + j] = acc[j];
    __syncwarp();
}

// One class, by one warp: W (its columns are W applied to the unit vectors), the
// eigen-decomposition of A = (W + W^T)/2 (cyclic Jacobi), the d table and Q, written
// to out[kClsStride] as V^T, Q, d[k][i].  mats: the warp's five 16 x 17 scratch
// matrices.  The result depends only on (key, beta_k, q).
constexpr int kPrepThreads = 512;

template <typename T>
__device__ void prep_class(unsigned long long key, double beta_k, int q, T* __restrict__ out, T (*mats)[16][17],
                           int lane) {
    T(*Wp)[17] = mats[0];
    T(*A)[17] = mats[1];
    T(*V)[17] = mats[2];
    T(*Q)[17] = mats[3];
    T(*Tm)[17] = mats[4];
    int dE0[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) dE0[j] = (int)((key >> (9 * j)) & 511ull) - 256;
    T ce[8], cr[8];
    uint32_t zmask = 0;
#pragma unroll
    for (int pos = 0; pos < 8; ++pos) {
        const int a = pos >> 2, b = (pos >> 1) & 1, cc = pos & 1;
        // a = 1 positions are the swap partners of (0, b ^ c, c): negated differences
        const int dE = a == 0 ? dE0[b + 2 * cc] : -dE0[(b ^ cc) + 2 * cc];
        double e = 1.0, r = 0.0;
        if (dE > 0) {
            e = exp(-0.5 * beta_k * (double)dE);
            r = sqrt(1.0 - e * e);
        }
        ce[pos] = (T)e;
        cr[pos] = (T)r;
        if (dE == 0) zmask |= 1u << pos;
    }
    // W column by column: W applied to the unit vectors
    if (lane < 16) {
        Orbit<T> ob;
        ob.setup(ce, cr, zmask);
#pragma unroll
        for (int j = 0; j < 16; ++j) ob.v[j] = j == lane ? (T)1 : (T)0;
        ob.walk();
#pragma unroll
        for (int i = 0; i < 16; ++i) Wp[i][lane] = ob.v[i];
    }
    __syncwarp();
    for (int idx = lane; idx < 256; idx += 32) {
        const int i = idx >> 4, j = idx & 15;
        A[i][j] = (T)0.5 * (Wp[i][j] + Wp[j][i]);
        V[i][j] = i == j ? (T)1 : (T)0;
    }
    __syncwarp();
    // cyclic Jacobi: A' = J^T A J zeroes A[p][q]; V' = V J; stops when the
    // off-diagonal mass is at rounding level (at most 10 sweeps)
    const T tol = sizeof(T) == 8 ? (T)1e-28 : (T)1e-12;
    for (int sweep = 0; sweep < 10; ++sweep) {
        T off = (T)0;
        for (int idx = lane; idx < 256; idx += 32) {
            const int i = idx >> 4, j = idx & 15;
            if (i < j) off += A[i][j] * A[i][j];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
        if (off < tol) break;  // uniform over the warp
        for (int p = 0; p < 15; ++p) {
            for (int qq = p + 1; qq < 16; ++qq) {
                const T apq = A[p][qq];
                if (fabs((double)apq) < 1e-300) continue;  // uniform: every lane reads the same value
                const T app = A[p][p], aqq = A[qq][qq];
                const T tau = (aqq - app) / ((T)2 * apq);
                const T t = (tau >= (T)0 ? (T)1 : (T)-1) / (fabs(tau) + sqrt((T)1 + tau * tau));
                const T c1 = (T)1 / sqrt((T)1 + t * t), s1 = t * c1;
                __syncwarp();
                if (lane < 16) {
                    const T akp = A[lane][p], akq = A[lane][qq];
                    A[lane][p] = c1 * akp - s1 * akq;
                    A[lane][qq] = s1 * akp + c1 * akq;
                }
                __syncwarp();
                if (lane < 16) {
                    const T apk = A[p][lane], aqk = A[qq][lane];
                    A[p][lane] = c1 * apk - s1 * aqk;
                    A[qq][lane] = s1 * apk + c1 * aqk;
                    const T vkp = V[lane][p], vkq = V[lane][qq];
                    V[lane][p] = c1 * vkp - s1 * vkq;
                    V[lane][qq] = s1 * vkp + c1 * vkq;
                }
                __syncwarp();
            }
        }
    }
    // d[k][i] = v_i^T U_k with U_k = W U_{k-1} = W^k V (A is free again: it holds U)
    T(*U)[17] = A;
    for (int idx = lane; idx < 256; idx += 32) U[idx >> 4][idx & 15] = V[idx >> 4][idx & 15];
    if (lane < 16) out[512 + lane] = (T)1;  // d[0][i] = |v_i|^2 = 1
    __syncwarp();
    for (int k = 1; k < (1 << q); ++k) {
        warp_matmul<T>(Tm, Wp, U, lane);  // U_k = W U_{k-1}
        for (int idx = lane; idx < 256; idx += 32) U[idx >> 4][idx & 15] = Tm[idx >> 4][idx & 15];
        __syncwarp();
        if (lane < 16) {
            T dk = (T)0;
#pragma unroll
            for (int j = 0; j < 16; ++j) dk += V[j][lane] * U[j][lane];
            out[512 + k * 16 + lane] = dk;
        }
        __syncwarp();
    }
    // Q = sum_{k<L} W^k = prod_{j<q} (I + W^(2^j)); Wp becomes the running square
    for (int idx = lane; idx < 256; idx += 32) {
        const int i = idx >> 4, j = idx & 15;
        Q[i][j] = Wp[i][j] + (i == j ? (T)1 : (T)0);
    }
    __syncwarp();
    for (int j = 1; j < q; ++j) {
        warp_matmul<T>(Tm, Wp, Wp, lane);
        for (int idx = lane; idx < 256; idx += 32) Wp[idx >> 4][idx & 15] = Tm[idx >> 4][idx & 15];
        __syncwarp();
        warp_matmul<T>(Tm, Q, Wp, lane);
        for (int idx = lane; idx < 256; idx += 32) Q[idx >> 4][idx & 15] += Tm[idx >> 4][idx & 15];
        __syncwarp();
    }
    for (int idx = lane; idx < 256; idx += 32) {
        const int i = idx >> 4, j = idx & 15;
        out[idx] = V[j][i];  // V^T, row i = eigenvector i
        out[256 + idx] = Q[i][j];
    }
    __syncwarp();
}

// Per walk and step, one warp per class of the current move (classes at the walk's
// current temperature; used when the batch's class table does not fit).
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_cls_prep(const WalkDev* __restrict__ walks, const WalkRec* __restrict__ recs,
                                                      const unsigned long long* __restrict__ keys,
                                                      const uint32_t* __restrict__ ncls, T* __restrict__ cls) {
    const int w = blockIdx.x;
    const WalkDev& W = walks[w];
    const WalkRec& R = recs[w];
    if (R.status != 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typedef T Mat[16][17];
    Mat* mats = reinterpret_cast<Mat*>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nc = ncls[(uint64_t)w * kMaxMoves + R.C];
    const unsigned long long* kk = keys + ((uint64_t)w * kMaxMoves + R.C) * kMaxCls;
    for (uint32_t c = warp; c < nc; c += kPrepThreads / 32)
        prep_class<T>(kk[c], R.beta_k, W.q, cls + ((uint64_t)w * kMaxCls + c) * kClsStride, mats + warp * 5, lane);
}

// The batch's class table, once: entry e = key index * nslot + temperature slot, one
// warp per entry.  Slot j holds (beta_j, q_j); a walk's stage k at slot slot0 + k.
template <typename T>
__global__ void __launch_bounds__(kPrepThreads) k_cls_table(const unsigned long long* __restrict__ gkeys,
                                                       const double* __restrict__ slot_beta, const int* __restrict__ slot_q,
                                                       uint32_t nslot, uint32_t nentry, T* __restrict__ tab) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typedef T Mat[16][17];
    Mat* mats = reinterpret_cast<Mat*>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t e = blockIdx.x * (kPrepThreads / 32) + warp;
    if (e >= nentry) return;  // warp-uniform; no block-wide barrier follows
    const uint32_t slot = e % nslot;
    prep_class<T>(gkeys[e / nslot], slot_beta[slot], slot_q[slot], tab + (uint64_t)e * kClsStride, mats + warp * 5, lane);
}

// Class data of class c of the walk's current move: per-step preparation (gid null)
// keeps it per walk; the table indexes it by key and temperature slot.
__device__ __forceinline__ uint64_t cls_entry(const WalkDev& W, const WalkRec& R, const uint32_t* __restrict__ gid, int w,
                                              uint32_t c) {
    if (!gid) return (uint64_t)w * kMaxCls + c;
    return (uint64_t)gid[((uint64_t)w * kMaxMoves + R.C) * kMaxCls + c] + W.slot0 + R.att / (uint32_t)W.per;
}

// Orbit pass of algo 1: per orbit its class, y = V^T psi, the class sums of
// y_i^2 (per warp, in a fixed order), S = Q psi written back.  STAGED: the
// classes' V^T and Q are copied to shared memory first (rows of kStagedStride
// elements, an odd number of 16-byte units, so lanes reading different classes
// fall into different bank groups); otherwise they are read through L1.
constexpr int kStagedStride = 516;

template <typename T, bool STAGED>
__global__ void __launch_bounds__(kThreads) k_walk_step_cls(const WalkDev* __restrict__ walks, const int* __restrict__ cta_walk,
                                                           const WalkRec* __restrict__ recs, const int* __restrict__ energies,
                                                           const unsigned long long* __restrict__ keys,
                                                           const uint32_t* __restrict__ ncls, const T* __restrict__ cls,
                                                           const uint32_t* __restrict__ gid, T* __restrict__ states,
                                                           double* __restrict__ npart, int nslot) {
    const int w = cta_walk[blockIdx.x];
    const WalkDev& W = walks[w];
    const WalkRec& R = recs[w];
    if (R.status != 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // nslot: classes per warp slot array (the batch's largest class count)
    T* cls_s = reinterpret_cast<T*>(smem_raw);                                // STAGED: [nslot][kStagedStride]
    T* slots = cls_s + (STAGED ? nslot * kStagedStride : 0);                  // [warps][nslot][16]
    T* stage_n = slots + (kThreads / 32) * nslot * 16;                        // [warps][32][16]
    int* stage_c = reinterpret_cast<int*>(stage_n + (kThreads / 32) * 32 * 16);  // [warps][32]
    unsigned long long* skeys = reinterpret_cast<unsigned long long*>(
        (reinterpret_cast<uintptr_t>(stage_c + (kThreads / 32) * 32) + 15) & ~(uintptr_t)15);
    unsigned long long* sent = skeys + kMaxCls;  // class data entry of each class
    const int s = W.s, C = (int)R.C;
    const uint32_t nc = ncls[(uint64_t)w * kMaxMoves + C];
    for (int i = threadIdx.x; i < (kThreads / 32) * nslot * 16; i += blockDim.x) slots[i] = (T)0;
    for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) skeys[i] = keys[((uint64_t)w * kMaxMoves + C) * kMaxCls + i];
    // entry 0 always set: lanes without a class read (and discard) class 0's data
    for (uint32_t i = threadIdx.x; i < max(nc, 1u); i += blockDim.x) sent[i] = cls_entry(W, R, gid, w, i);
    __syncthreads();
    if (STAGED) {
        typedef typename std::conditional<sizeof(T) == 4, float4, double2>::type VecS;
        constexpr int VS = sizeof(VecS) / sizeof(T);
        for (uint32_t i = threadIdx.x; i < nc * (512 / VS); i += blockDim.x) {
            const uint32_t c = i / (512 / VS), e = (i % (512 / VS)) * VS;
            *reinterpret_cast<VecS*>(cls_s + c * kStagedStride + e) =
                __ldg(reinterpret_cast<const VecS*>(cls + sent[c] * kClsStride + e));
        }
        __syncthreads();
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t N = 1u << s;
    const uint64_t NN = (uint64_t)N * N;
    const uint32_t norb = norbits(s), eC = 1u << C;
    const int* E = energies + W.e_off;
    T* st = states + W.state_off;
    const bool fresh = R.fresh != 0;
    const T scale = (T)R.scale;
    const T init = (T)(1.0 / sqrt((double)N));
    T* myslots = slots + warp * nslot * 16;
    const uint32_t first = (blockIdx.x - W.cta0) * (uint32_t)kClsOrbitsPerCta;
    for (int it = 0; it < kClsOrbitsPerThread; ++it) {
        const uint32_t o = first + (uint32_t)(it * kThreads) + threadIdx.x;
        const bool active = o < norb;
        if (!__any_sync(0xffffffffu, active)) continue;  // warp-uniform
        uint32_t dp = 0, x0 = 0;
        bool single = true;
        int ci = -1;
        if (active) {
            single = orbit_decode(o, s, C, dp, x0);
            const unsigned long long key = orbit_key(E, x0, dp, eC);
            int lo = 0, hi = (int)nc - 1;  // binary search in the sorted class keys
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (skeys[mid] < key) lo = mid + 1;
                else hi = mid;
            }
            ci = (nc > 0 && skeys[lo] == key) ? lo : -1;
        }
        T v[16];
#pragma unroll
        for (int pos = 0; pos < 8; ++pos) {
            const int a = pos >> 2, b = (pos >> 1) & 1, c = pos & 1;
            const uint32_t x = x0 ^ (a ? dp : 0u) ^ (b ? eC : 0u);
            const uint32_t d = dp ^ (c ? eC : 0u);
#pragma unroll
            for (int acc = 0; acc < 2; ++acc) {
                T val = (T)0;
                if (ci >= 0) {
                    if (fresh) val = (single && c == 0 && acc == 0) ? init : (T)0;
                    else if (!(single && a == 1)) val = st[(uint64_t)acc * NN + (uint64_t)d * N + x] * scale;
                }
                v[SLOT(a, b, c, acc)] = val;
            }
        }
        if (single) {
#pragma unroll
            for (int j = 0; j < 8; ++j) v[8 + j] = v[j];
        }
        const T wgt = single ? (T)0.5 : (T)1;
        const T* cb = STAGED ? cls_s + (ci >= 0 ? ci : 0) * kStagedStride : cls + sent[ci >= 0 ? ci : 0] * kClsStride;
        T S[16];
        typedef typename std::conditional<sizeof(T) == 4, float4, double2>::type VecL;
        constexpr int VW = sizeof(VecL) / sizeof(T);  // elements per vector load
        const VecL* cv = reinterpret_cast<const VecL*>(cb);  // class rows are 16-byte aligned
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            T y = (T)0, sq = (T)0;
#pragma unroll
            for (int j = 0; j < 16; j += VW) {
                const VecL a = STAGED ? cv[(i * 16 + j) / VW] : __ldg(cv + (i * 16 + j) / VW);
                const VecL b = STAGED ? cv[(256 + i * 16 + j) / VW] : __ldg(cv + (256 + i * 16 + j) / VW);
                const T* av = reinterpret_cast<const T*>(&a);
                const T* bv = reinterpret_cast<const T*>(&b);
#pragma unroll
                for (int u = 0; u < VW; ++u) {
                    y += av[u] * v[j + u];
                    sq += bv[u] * v[j + u];
                }
            }
            S[i] = sq;
            stage_n[(warp * 32 + lane) * 16 + i] = wgt * y * y;
        }
        stage_c[warp * 32 + lane] = ci;
        if (ci >= 0) {
#pragma unroll
            for (int pos = 0; pos < 8; ++pos) {
                const int a = pos >> 2, b = (pos >> 1) & 1, c = pos & 1;
                if (single && a == 1) continue;
                const uint32_t x = x0 ^ (a ? dp : 0u) ^ (b ? eC : 0u);
                const uint32_t d = dp ^ (c ? eC : 0u);
#pragma unroll
                for (int acc = 0; acc < 2; ++acc) st[(uint64_t)acc * NN + (uint64_t)d * N + x] = S[SLOT(a, b, c, acc)];
            }
        }
        __syncwarp();
        if (lane < 16) {  // fixed order: lanes of the warp one after the other
            for (int l = 0; l < 32; ++l) {
                const int cl = stage_c[warp * 32 + l];
                if (cl >= 0) myslots[cl * 16 + lane] += stage_n[(warp * 32 + l) * 16 + lane];
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < nc * 16u; e += blockDim.x) {
        double sum = 0.0;
        for (int wp = 0; wp < kThreads / 32; ++wp) sum += (double)slots[wp * nslot * 16 + e];
        npart[(uint64_t)blockIdx.x * kMaxCls * 16 + e] = sum;
    }
}

// FP32 orbit pass of algo 1 with the orbits sorted by class.  The CTA takes its
// orbits in chunks of kSortChunk, one orbit per thread: coalesced loads (the next
// chunk's in flight while this chunk's products run), a stable counting sort in
// shared memory by q = 2 class + (8-amplitude orbit) (per-warp counts from
// __match_any_sync, offsets over keys then warps), then each warp walks a
// contiguous range of the sorted chunk run by run, with the run's class rows in
// registers: lane l < 16 holds row l of V^T (y_l = v_l^T psi), lane 16 + i row i
// of Q (S_i).  The 16 amplitudes of an orbit are one broadcast read; lanes < 16
// keep the class sums of w y^2 in a register until the class changes (w = 1/2 for
// 8-amplitude orbits, constant over a run).  Each class row is read once per run
// instead of once per orbit.  S returns to the thread that loaded the orbit and
// is stored coalesced.  Orbit classes come from a 256-slot hash of the class keys.
constexpr int kSortChunk = kThreads;
constexpr int kWarps = kThreads / 32;
constexpr int kHash = 256;
constexpr int kRow = 20;  // floats per sorted row: 16 amplitudes, rows 5 bank groups apart

__device__ __forceinline__ uint32_t cls_hash(unsigned long long key) {
    return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 56);
}

// Orbit o of the chunk in two halves, so that no instruction waits on the loads
// before this chunk's products have run: sorted_issue decodes the orbit and
// issues its loads (its 16 amplitudes, read even on a fresh start and for orbits
// past the walk's end, whose indices stay inside the walk's state, and then
// dropped) after forming its class key, sorted_finish looks up the class (-1 past
// the end) and scales the amplitudes.  State index of amplitude
// (a, b, c, acc): b0 ^ (a ? dp) ^ (b ? e_C) ^ (c ? e_C << s) ^ (acc ? 1 << 2s),
// the bits of (acc, d, x).
struct SortedLoad {
    uint32_t b0, dp;
    bool active, single;
    unsigned long long key;
    float raw[16];
};

// The ring's bonds for the class keys without the energy table: flipping the spins
// of d changes the sign of s_b s_{b+1} exactly on the bonds that cross the border of
// d, m = d ^ rot(d), so E(x ^ d) - E(x) = 2 sum_{b in m} J_b s_b s_{b+1}(x)
//   = 2 J(m) - 4 J(m & (x ^ rot(x))),  J(mask) = sum of J_b over the bonds in mask,
// from bit planes of J_b + joff: sum_k 2^k popc(mask & plane_k) - joff popc(mask).
struct RingBonds {
    uint32_t plane[5];
    int np, off, s;
    uint32_t smask;
};

__device__ __forceinline__ int bond_sum(uint32_t m, const RingBonds& B) {
    int t = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k)
        if (k < B.np) t += __popc(m & B.plane[k]) << k;
    return t - B.off * __popc(m);
}

__device__ __forceinline__ int ring_dE(uint32_t x, uint32_t d, const RingBonds& B) {
    const uint32_t m = (d ^ ((d >> 1) | (d << (B.s - 1)))) & B.smask;
    const uint32_t bx = (x ^ ((x >> 1) | (x << (B.s - 1)))) & B.smask;
    return 2 * bond_sum(m, B) - 4 * bond_sum(m & bx, B);
}

__device__ __forceinline__ void sorted_issue(uint32_t o, uint32_t norb, int s, int C, uint32_t eC, const RingBonds& B,
                                             const float* __restrict__ st, SortedLoad& L) {
    uint32_t x0 = 0, dp = 0;
    L.active = o < norb;
    L.single = true;
    if (L.active) L.single = orbit_decode(o, s, C, dp, x0);
    L.b0 = (dp << s) | x0;
    L.dp = dp;
    L.key = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {  // orbit_key's terms: dE at x = x0 ^ (j&1 ? e_C), d = dp ^ (j&2 ? e_C)
        const uint32_t x = x0 ^ ((j & 1) ? eC : 0u);
        const uint32_t d = dp ^ ((j & 2) ? eC : 0u);
        L.key |= (unsigned long long)(ring_dE(x, d, B) + 256) << (9 * j);
    }
    const uint32_t mc = eC << s, macc = 1u << (2 * s);
#pragma unroll
    for (int pos = 0; pos < 8; ++pos) {
        const int a = pos >> 2, b = (pos >> 1) & 1, c = pos & 1;
        const uint32_t i0 = L.b0 ^ (a ? dp : 0u) ^ (b ? eC : 0u) ^ (c ? mc : 0u);
#pragma unroll
        for (int acc = 0; acc < 2; ++acc) L.raw[SLOT(a, b, c, acc)] = st[i0 ^ (acc ? macc : 0u)];
    }
}

__device__ __forceinline__ int sorted_finish(const SortedLoad& L, const unsigned long long* htab, bool fresh, float scale,
                                             float init, float (&v)[16]) {
    int ci = -1;
    if (L.active) {
        const unsigned long long key = L.key;
        uint32_t h = cls_hash(key);
        for (int probe = 0; probe < kHash; ++probe) {  // bounded; the table is at most 3/8 full
            const unsigned long long e = htab[h];
            if (e == 0ull) break;
            if ((e >> 8) == key) {
                ci = (int)(e & 255ull);
                break;
            }
            h = (h + 1u) & (kHash - 1);
        }
    }
#pragma unroll
    for (int pos = 0; pos < 8; ++pos) {
        const int a = pos >> 2, c = pos & 1;
#pragma unroll
        for (int acc = 0; acc < 2; ++acc) {
            const int j = SLOT(a, (pos >> 1) & 1, c, acc);
            float val;
            if (fresh) val = (L.single && c == 0 && acc == 0) ? init : 0.f;
            else val = (L.single && a == 1) ? 0.f : L.raw[j] * scale;
            v[j] = val;
        }
    }
    if (L.single) {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[8 + j] = v[j];
    }
    return ci;
}

__device__ __forceinline__ void sorted_row(const float* vrow, f2 (&v)[8]) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const ulonglong2 q = *reinterpret_cast<const ulonglong2*>(vrow + 4 * u);
        v[2 * u] = q.x;
        v[2 * u + 1] = q.y;
    }
}

// row . v with the pairs (2m, 2m+1) in packed f32x2: two chains of four, then the halves
__device__ __forceinline__ float sorted_dot(const f2 (&r)[8], const f2 (&v)[8]) {
    f2 ea = mul2(r[0], v[0]), eb = mul2(r[1], v[1]);
#pragma unroll
    for (int m = 1; m < 4; ++m) {
        ea = fma2(r[2 * m], v[2 * m], ea);
        eb = fma2(r[2 * m + 1], v[2 * m + 1], eb);
    }
    float x, y;
    up2(add2(ea, eb), x, y);
    return x + y;
}

__global__ void __launch_bounds__(kThreads, 1) k_walk_step_sorted(const WalkDev* __restrict__ walks, const int* __restrict__ cta_walk,
                                                               const WalkRec* __restrict__ recs,
                                                               const unsigned long long* __restrict__ keys,
                                                               const uint32_t* __restrict__ ncls, const float* __restrict__ cls,
                                                               const uint32_t* __restrict__ gid, float* __restrict__ states,
                                                               double* __restrict__ npart, int nslot) {
    const int w = cta_walk[blockIdx.x];
    const WalkDev& W = walks[w];
    const WalkRec& R = recs[w];
    if (R.status != 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // nslot: classes per slot array (the batch's largest class count, <= kMaxCls = 96);
    // nk = 2 nslot sort keys, at most 6 per lane of one warp
    const int nk = 2 * nslot;
    float* cls_s = reinterpret_cast<float*>(smem_raw);              // [nslot][512]: V^T rows, then Q rows
    float* slots = cls_s + nslot * 512;                              // [warps][nslot][16]
    float* vbuf = slots + kWarps * nslot * 16;                       // [kSortChunk][kRow] amplitudes, sorted
    float* sbuf = vbuf + kSortChunk * kRow;                          // [kSortChunk][kRow] S, sorted
    unsigned long long* htab = reinterpret_cast<unsigned long long*>(sbuf + kSortChunk * kRow);  // [kHash] key << 8 | class
    unsigned long long* sent = htab + kHash;                         // [kMaxCls] class data entries
    int* wcnt = reinterpret_cast<int*>(sent + kMaxCls);              // [warps][nk] counts, then offsets within a key
    int* kstart = wcnt + kWarps * nk;                                // [nk] start of each key's run
    int* kend = kstart + nk;                                         // [nk] end of each key's run
    int* wsum = kend + nk;                                           // [warps] key totals per warp of the scan
    int* nact_s = wsum + kWarps;
    unsigned char* csort = reinterpret_cast<unsigned char*>(nact_s + 4);  // [kSortChunk] key of each sorted orbit
    const int s = W.s, C = (int)R.C;
    const uint32_t nc = ncls[(uint64_t)w * kMaxMoves + C];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * nslot * 16; i += kThreads) slots[i] = 0.f;
    for (int i = threadIdx.x; i < kHash; i += kThreads) htab[i] = 0ull;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nc; i += kThreads) {
        const unsigned long long key = keys[((uint64_t)w * kMaxMoves + C) * kMaxCls + i];
        uint32_t h = cls_hash(key);
        for (int probe = 0; probe < kHash; ++probe) {  // distinct keys, nc <= 96 < kHash: always placed
            if (atomicCAS(&htab[h], 0ull, (key << 8) | (unsigned long long)i) == 0ull) break;
            h = (h + 1u) & (kHash - 1);
        }
    }
    // entry 0 always set: lanes without a class never read class data, but keep it valid
    for (uint32_t i = threadIdx.x; i < max(nc, 1u); i += kThreads) sent[i] = cls_entry(W, R, gid, w, i);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nc * 128u; i += kThreads) {
        const uint32_t c = i >> 7, e = (i & 127u) * 4u;
        *reinterpret_cast<float4*>(cls_s + c * 512 + e) = __ldg(reinterpret_cast<const float4*>(cls + sent[c] * kClsStride + e));
    }
    const uint32_t norb = norbits(s), eC = 1u << C;
    const uint32_t mc = eC << s, macc = 1u << (2 * s);
    RingBonds bonds;
#pragma unroll
    for (int k = 0; k < 5; ++k) bonds.plane[k] = W.jplane[k];
    bonds.np = W.jnp;
    bonds.off = W.joff;
    bonds.s = s;
    bonds.smask = (1u << s) - 1u;
    const int kslot = threadIdx.x;  // the sort key this thread scans
    float* st = states + W.state_off;
    const bool fresh = R.fresh != 0;
    const float scale = (float)R.scale;
    const float init = (float)(1.0 / sqrt((double)(1u << s)));
    float* myslots = slots + warp * nslot * 16;
    const uint32_t first = (blockIdx.x - W.cta0) * (uint32_t)kClsOrbitsPerCta;
    constexpr int kChunks = kClsOrbitsPerCta / kSortChunk;
    const int row = lane & 15, part = lane >> 4;  // part 0: V^T row, 1: Q row

    SortedLoad ld;
    sorted_issue(first + threadIdx.x, norb, s, C, eC, bonds, st, ld);
    for (int k = 0; k < kChunks; ++k) {
        const uint32_t cbase = first + (uint32_t)(k * kSortChunk);
        if (cbase >= norb) break;  // uniform over the CTA
        float vn[16];
        const int ci = sorted_finish(ld, htab, fresh, scale, init, vn);
        const bool single = ld.single;
        const uint32_t b0 = ld.b0, dp = ld.dp;
        const int q = ci >= 0 ? 2 * ci + (single ? 1 : 0) : -1;
        // per-warp key counts; the first lane of each key group writes its size
        for (int c = lane; c < nk; c += 32) wcnt[warp * nk + c] = 0;
        __syncwarp();
        const unsigned grp = __match_any_sync(0xffffffffu, q);
        const int rank = __popc(grp & ((1u << lane) - 1u));
        if (q >= 0 && rank == 0) wcnt[warp * nk + q] = __popc(grp);
        __syncthreads();
        // positions: keys in order, warps in order within a key; thread t scans key t
        int tot = 0;
        if (kslot < nk) {
            for (int wp = 0; wp < kWarps; ++wp) {
                const int t = wcnt[wp * nk + kslot];
                wcnt[wp * nk + kslot] = tot;
                tot += t;
            }
        }
        int incl = tot;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (kslot < nk) {
            int base = incl - tot;
            for (int wp = 0; wp < warp; ++wp) base += wsum[wp];
            kstart[kslot] = base;
            kend[kslot] = base + tot;
        }
        if (threadIdx.x == 0) {
            int n = 0;
            for (int wp = 0; wp < kWarps; ++wp) n += wsum[wp];
            *nact_s = n;
        }
        __syncthreads();
        int pos = -1;
        if (q >= 0) {
            pos = kstart[q] + wcnt[warp * nk + q] + rank;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                *reinterpret_cast<float4*>(vbuf + pos * kRow + 4 * u) = make_float4(vn[4 * u], vn[4 * u + 1], vn[4 * u + 2], vn[4 * u + 3]);
            csort[pos] = (unsigned char)q;
        }
        __syncthreads();
        if (k + 1 < kChunks)  // the next chunk's loads overlap this chunk's products
            sorted_issue(cbase + kSortChunk + threadIdx.x, norb, s, C, eC, bonds, st, ld);
        {
            const int nact = *nact_s;
            const int p1 = nact * (warp + 1) / kWarps;
            int p = nact * warp / kWarps;
            int cur = -1;
            float nacc = 0.f;
            f2 r[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) r[m] = 0ull;
            while (p < p1) {  // one run (one key) per iteration; uniform over the warp
                const int qq = csort[p];
                const int e = max(min(kend[qq], p1), p + 1);  // p lies in its key's run: kend[qq] > p
                const float wt = (qq & 1) ? 0.5f : 1.f;
                if ((qq >> 1) != cur) {
                    if (cur >= 0 && part == 0) myslots[cur * 16 + row] += nacc;
                    nacc = 0.f;
                    cur = qq >> 1;
                    const ulonglong2* rp = reinterpret_cast<const ulonglong2*>(cls_s + cur * 512 + lane * 16);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const ulonglong2 t = rp[u];
                        r[2 * u] = t.x;
                        r[2 * u + 1] = t.y;
                    }
                }
                for (; p + 4 <= e; p += 4) {
                    f2 v0[8], v1[8], v2[8], v3[8];
                    sorted_row(vbuf + p * kRow, v0);
                    sorted_row(vbuf + (p + 1) * kRow, v1);
                    sorted_row(vbuf + (p + 2) * kRow, v2);
                    sorted_row(vbuf + (p + 3) * kRow, v3);
                    const float y0 = sorted_dot(r, v0), y1 = sorted_dot(r, v1);
                    const float y2 = sorted_dot(r, v2), y3 = sorted_dot(r, v3);
                    if (part == 0) {
                        nacc += wt * y0 * y0;
                        nacc += wt * y1 * y1;
                        nacc += wt * y2 * y2;
                        nacc += wt * y3 * y3;
                    } else {
                        sbuf[p * kRow + row] = y0;
                        sbuf[(p + 1) * kRow + row] = y1;
                        sbuf[(p + 2) * kRow + row] = y2;
                        sbuf[(p + 3) * kRow + row] = y3;
                    }
                }
                for (; p < e; ++p) {
                    f2 v0[8];
                    sorted_row(vbuf + p * kRow, v0);
                    const float y0 = sorted_dot(r, v0);
                    if (part == 0) nacc += wt * y0 * y0;
                    else sbuf[p * kRow + row] = y0;
                }
            }
            if (cur >= 0 && part == 0) myslots[cur * 16 + row] += nacc;
        }
        __syncthreads();
        if (q >= 0) {
            float S[16];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float4 t = *reinterpret_cast<const float4*>(sbuf + pos * kRow + 4 * u);
                S[4 * u] = t.x;
                S[4 * u + 1] = t.y;
                S[4 * u + 2] = t.z;
                S[4 * u + 3] = t.w;
            }
#pragma unroll
            for (int pp = 0; pp < 8; ++pp) {
                const int a = pp >> 2, b = (pp >> 1) & 1, c = pp & 1;
                if (single && a == 1) continue;
                const uint32_t i0 = b0 ^ (a ? dp : 0u) ^ (b ? eC : 0u) ^ (c ? mc : 0u);
                st[i0] = S[SLOT(a, b, c, 0)];
                st[i0 ^ macc] = S[SLOT(a, b, c, 1)];
            }
        }
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < nc * 16u; e += blockDim.x) {
        double sum = 0.0;
        for (int wp = 0; wp < kWarps; ++wp) sum += (double)slots[wp * nslot * 16 + e];
        npart[(uint64_t)blockIdx.x * kMaxCls * 16 + e] = sum;
    }
}

// The same orbit pass with 16 warps per CTA (one CTA per SM, twice the warps of
// k_walk_step_sorted): chunks of 512 orbits, the class sums in one CTA-level slot
// array instead of one per warp, and the sorted amplitudes overwritten in place by
// S.  A warp's sorted range holds whole runs of the classes strictly inside it, so
// it adds those classes' sums directly; the classes at the two ends of its range
// may continue in the neighbouring warps, so their partial sums go to a per-warp
// edge buffer that is added in warp order after the chunk (the sums stay
// deterministic).  Sorted rows of 20 floats (16 amplitudes, then S in place; the
// padding spreads the scattered row stores of a quarter-warp over the banks).
//
// Orbit order table.  An orbit's class depends only on the ring's couplings and
// the move, not on the state, so the chunk's counting sort puts every orbit at the
// same place at every step with that move.  With a table (`order`: per walk, move
// and orbit the 16-bit entry place | class << 9), the first step of a CTA with a
// move sorts as usual and records the places; its flag in `ready` (per CTA and
// move) then lets every later step with that move take the places from the table
// and skip the class keys, the hash lookups and the sort with its two extra CTA
// barriers per chunk.  Either way the places, and so the sums, are the same.
// process-wide choice of the FP32 class-sorted orbit pass (sq_set_walk_orbit_warps)
std::atomic<int> g_orbit_warps{16};
// process-wide use of the orbit order table where it fits (sq_set_walk_presort)
std::atomic<int> g_presort{1};
// process-wide choice of the 16-warp pass's products: tensor cores (1) or CUDA cores (0) (sq_set_walk_mma)
std::atomic<int> g_walk_mma{1};
constexpr uint64_t kOrderBudget = 8ull << 30;  // largest batch orbit order table (bytes)

constexpr int kS2Threads = 512;
constexpr int kS2Warps = kS2Threads / 32;
constexpr int kS2Chunk = kS2Threads;
constexpr int kS2Row = 20;  // floats per sorted row: 16 amplitudes, rows 5 bank groups apart
constexpr int kS2Chunks = kClsOrbitsPerCta / kS2Chunk;

// entries of a walk's order table: every move, every orbit slot of its CTAs
__host__ __device__ inline uint64_t order_entries(int s, uint32_t ncta) {
    return (uint64_t)s * ncta * (uint64_t)kClsOrbitsPerCta;
}

// dynamic shared memory of k_walk_step_sorted2 for nslot classes
__host__ __device__ inline size_t sorted2_smem_bytes(int nslot) {
    const size_t nk = 2 * (size_t)nslot;
    return sizeof(float) * ((size_t)nslot * 512 + (size_t)nslot * 16 + (size_t)kS2Warps * 2 * 16 +
                            (size_t)kS2Chunk * kS2Row) +
           sizeof(unsigned long long) * (kHash + kMaxCls) + sizeof(int) * ((size_t)kS2Warps * nk + nk + kS2Warps +
                                                                          2 * kS2Warps + 4) +
           kS2Chunk;
}

// One orbit of the chunk: its 16 amplitudes and either its order entry (table) or
// its class key (sort), issued before the products of the previous chunk.
struct S2Load {
    uint32_t b0, dp;
    bool active, single;
    uint16_t ord;
    unsigned long long key;
    float raw[16];
};

__device__ __forceinline__ void s2_issue(uint32_t o, uint32_t norb, int s, int C, uint32_t eC, const RingBonds& B,
                                         bool have, const float* __restrict__ st, const uint16_t* __restrict__ ord,
                                         S2Load& L) {
    uint32_t x0 = 0, dp = 0;
    L.active = o < norb;
    L.single = true;
    L.ord = 0xffff;
    L.key = 0;
    if (L.active) {
        L.single = orbit_decode(o, s, C, dp, x0);
        if (have) L.ord = ord[o];
    }
    L.b0 = (dp << s) | x0;
    L.dp = dp;
    if (!have) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {  // orbit_key's terms: dE at x = x0 ^ (j&1 ? e_C), d = dp ^ (j&2 ? e_C)
            const uint32_t x = x0 ^ ((j & 1) ? eC : 0u);
            const uint32_t d = dp ^ ((j & 2) ? eC : 0u);
            L.key |= (unsigned long long)(ring_dE(x, d, B) + 256) << (9 * j);
        }
    }
    const uint32_t mc = eC << s, macc = 1u << (2 * s);
#pragma unroll
    for (int pos = 0; pos < 8; ++pos) {
        const int a = pos >> 2, b = (pos >> 1) & 1, c = pos & 1;
        const uint32_t i0 = L.b0 ^ (a ? dp : 0u) ^ (b ? eC : 0u) ^ (c ? mc : 0u);
#pragma unroll
        for (int acc = 0; acc < 2; ++acc) L.raw[SLOT(a, b, c, acc)] = st[i0 ^ (acc ? macc : 0u)];
    }
}

__device__ __forceinline__ void s2_finish(const S2Load& L, bool fresh, float scale, float init, float (&v)[16]) {
#pragma unroll
    for (int pos = 0; pos < 8; ++pos) {
        const int a = pos >> 2, c = pos & 1;
#pragma unroll
        for (int acc = 0; acc < 2; ++acc) {
            const int j = SLOT(a, (pos >> 1) & 1, c, acc);
            float val;
            if (fresh) val = (L.single && c == 0 && acc == 0) ? init : 0.f;
            else val = (L.single && a == 1) ? 0.f : L.raw[j] * scale;
            v[j] = val;
        }
    }
    if (L.single) {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[8 + j] = v[j];
    }
}

// ---- the products of a run on the tensor cores (mma.sync m16n8k8, TF32) ----
// For a run of orbits of one class, [V^T; Q] (32 x 16) times the run's amplitude
// rows (16 x 8 orbits per tile): the class rows are the A operand (two 16-row
// tiles, two 8-column k-steps), eight orbits the B operand.  FP32 accuracy from
// TF32 inputs by the three-product split x = hi + lo (hi = x rounded to TF32,
// lo = x - hi, whose bits below TF32 the tensor cores drop): A_hi B_hi + A_hi B_lo
// + A_lo B_hi, each product exact and summed in FP32; the dropped A_lo B_lo and
// the truncation of lo are ~2^-22 of the product.  Fragment layout (PTX ISA,
// m16n8k8 .tf32): g = lane / 4, t = lane % 4; A: a0 (g, t), a1 (g + 8, t),
// a2 (g, t + 4), a3 (g + 8, t + 4); B: b0 (k = t, n = g), b1 (t + 4, g);
// D: d0 (g, 2t), d1 (g, 2t + 1), d2 (g + 8, 2t), d3 (g + 8, 2t + 1).
__device__ __forceinline__ uint32_t tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The class's A fragments (hi and lo) for this lane from the staged class rows
// (row l's 16-byte chunk u at u ^ ((l >> 1) & 3)): [m-tile][k-step][4].
__device__ __forceinline__ void mma_class_frags(const float* crow, int lane, uint32_t (&ahi)[2][2][4],
                                                uint32_t (&alo)[2][2][4]) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int l = 16 * mt + g + ((j & 1) ? 8 : 0);
                const int chunk = 2 * ks + ((j & 2) ? 1 : 0);  // columns 8 ks + t (+ 4)
                const float x = crow[l * 16 + 4 * (chunk ^ ((l >> 1) & 3)) + t];
                const uint32_t h = tf32_hi(x);
                ahi[mt][ks][j] = h;
                alo[mt][ks][j] = __float_as_uint(x - __uint_as_float(h));
            }
}

template <bool MMA>
__global__ void __launch_bounds__(kS2Threads, 1) k_walk_step_sorted2(
    const WalkDev* __restrict__ walks, const int* __restrict__ cta_walk, const WalkRec* __restrict__ recs,
    const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ ncls, const float* __restrict__ cls,
    const uint32_t* __restrict__ gid, uint16_t* __restrict__ order, unsigned char* __restrict__ ready,
    float* __restrict__ states, double* __restrict__ npart, int nslot) {
    const int w = cta_walk[blockIdx.x];
    const WalkDev& W = walks[w];
    const WalkRec& R = recs[w];
    if (R.status != 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nk = 2 * nslot;
    float* cls_s = reinterpret_cast<float*>(smem_raw);               // [nslot][512]: V^T rows, then Q rows
    float* slots = cls_s + nslot * 512;                               // [nslot][16] class sums of the CTA
    float* edge = slots + nslot * 16;                                 // [warps][2][16] end-of-range partial sums
    float* vbuf = edge + kS2Warps * 2 * 16;                           // [kS2Chunk][kS2Row] amplitudes, then S
    unsigned long long* htab = reinterpret_cast<unsigned long long*>(vbuf + kS2Chunk * kS2Row);  // [kHash]
    unsigned long long* sent = htab + kHash;                          // [kMaxCls] class data entries
    int* wcnt = reinterpret_cast<int*>(sent + kMaxCls);               // [warps][nk]
    int* kstart = wcnt + kS2Warps * nk;                               // [nk]
    int* wsum = kstart + nk;                                          // [warps]
    int* ecls = wsum + kS2Warps;                                      // [warps][2] class of each edge sum (-1: none)
    unsigned char* csort = reinterpret_cast<unsigned char*>(ecls + 2 * kS2Warps + 4);  // [kS2Chunk]
    const int s = W.s, C = (int)R.C;
    const uint32_t nc = ncls[(uint64_t)w * kMaxMoves + C];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the order table's places for this CTA and move (uniform over the CTA)
    uint16_t* ord = order ? order + W.ord_off + (uint64_t)C * W.ncta * kClsOrbitsPerCta : nullptr;
    const bool have = ord != nullptr && ready[(uint64_t)blockIdx.x * kMaxMoves + C] != 0;
    for (int i = threadIdx.x; i < nslot * 16; i += kS2Threads) slots[i] = 0.f;
    for (int i = threadIdx.x; i < kS2Chunk; i += kS2Threads) csort[i] = 0;  // every key read stays a class of the CTA
    if (!have)
        for (int i = threadIdx.x; i < kHash; i += kS2Threads) htab[i] = 0ull;
    __syncthreads();
    if (!have)
        for (uint32_t i = threadIdx.x; i < nc; i += kS2Threads) {
            const unsigned long long key = keys[((uint64_t)w * kMaxMoves + C) * kMaxCls + i];
            uint32_t h = cls_hash(key);
            for (int probe = 0; probe < kHash; ++probe) {  // distinct keys, nc <= 96 < kHash: always placed
                if (atomicCAS(&htab[h], 0ull, (key << 8) | (unsigned long long)i) == 0ull) break;
                h = (h + 1u) & (kHash - 1);
            }
        }
    for (uint32_t i = threadIdx.x; i < max(nc, 1u); i += kS2Threads) sent[i] = cls_entry(W, R, gid, w, i);
    __syncthreads();
    // class rows with their 16-byte chunks swizzled by row (chunk u of row l at u ^ ((l >> 1) & 3)): the
    // eight lanes of a quarter-warp loading eight consecutive rows then hit eight different bank groups
    for (uint32_t i = threadIdx.x; i < nc * 128u; i += kS2Threads) {
        const uint32_t c = i >> 7, e = (i & 127u) * 4u, l = e >> 4, u = (e >> 2) & 3u;
        *reinterpret_cast<float4*>(cls_s + c * 512 + l * 16 + 4 * (u ^ ((l >> 1) & 3u))) =
            __ldg(reinterpret_cast<const float4*>(cls + sent[c] * kClsStride + e));
    }
    const uint32_t norb = norbits(s), eC = 1u << C;
    const uint32_t mc = eC << s, macc = 1u << (2 * s);
    RingBonds bonds;
#pragma unroll
    for (int k = 0; k < 5; ++k) bonds.plane[k] = W.jplane[k];
    bonds.np = W.jnp;
    bonds.off = W.joff;
    bonds.s = s;
    bonds.smask = (1u << s) - 1u;
    const int kslot = threadIdx.x;
    float* st = states + W.state_off;
    const bool fresh = R.fresh != 0;
    const float scale = (float)R.scale;
    const float init = (float)(1.0 / sqrt((double)(1u << s)));
    const uint32_t first = (blockIdx.x - W.cta0) * (uint32_t)kClsOrbitsPerCta;
    const int row = lane & 15, part = lane >> 4;

    S2Load ld;
    s2_issue(first + threadIdx.x, norb, s, C, eC, bonds, have, st, ord, ld);
    for (int k = 0; k < kS2Chunks; ++k) {
        const uint32_t cbase = first + (uint32_t)(k * kS2Chunk);
        if (cbase >= norb) break;  // uniform over the CTA
        float vn[16];
        s2_finish(ld, fresh, scale, init, vn);
        const bool single = ld.single;
        const uint32_t b0 = ld.b0, dp = ld.dp;
        int pos = -1, q = -1;
        if (have) {
            // the recorded place; an orbit whose class was not found keeps the table's fill 0xffff
            if (ld.active && (uint32_t)(ld.ord >> 9) < nc) {
                pos = (int)(ld.ord & 511u);
                q = 2 * (int)(ld.ord >> 9) + (single ? 1 : 0);
            }
        } else {
            int ci = -1;
            if (ld.active) {
                const unsigned long long key = ld.key;
                uint32_t h = cls_hash(key);
                for (int probe = 0; probe < kHash; ++probe) {  // bounded; the table is at most 3/8 full
                    const unsigned long long e = htab[h];
                    if (e == 0ull) break;
                    if ((e >> 8) == key) {
                        ci = (int)(e & 255ull);
                        break;
                    }
                    h = (h + 1u) & (kHash - 1);
                }
            }
            q = ci >= 0 ? 2 * ci + (single ? 1 : 0) : -1;
            // stable counting sort by q: place = orbits of smaller q + orbits of equal q
            // in earlier warps + in earlier lanes of this warp
            for (int c = lane; c < nk; c += 32) wcnt[warp * nk + c] = 0;
            __syncwarp();
            const unsigned grp = __match_any_sync(0xffffffffu, q);
            const int rank = __popc(grp & ((1u << lane) - 1u));
            if (q >= 0 && rank == 0) wcnt[warp * nk + q] = __popc(grp);
            __syncthreads();
            int tot = 0;
            if (kslot < nk) {
                for (int wp = 0; wp < kS2Warps; ++wp) {
                    const int t = wcnt[wp * nk + kslot];
                    wcnt[wp * nk + kslot] = tot;
                    tot += t;
                }
            }
            int incl = tot;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += y;
            }
            if (lane == 31) wsum[warp] = incl;
            __syncthreads();
            if (kslot < nk) {
                int base = incl - tot;
                for (int wp = 0; wp < warp; ++wp) base += wsum[wp];
                kstart[kslot] = base;
            }
            __syncthreads();
            if (q >= 0) {
                pos = kstart[q] + wcnt[warp * nk + q] + rank;
                if (ord) ord[cbase + threadIdx.x] = (uint16_t)(pos | (ci << 9));
            }
        }
        if (pos >= 0) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
                *reinterpret_cast<float4*>(vbuf + pos * kS2Row + 4 * u) =
                    make_float4(vn[4 * u], vn[4 * u + 1], vn[4 * u + 2], vn[4 * u + 3]);
            csort[pos] = (unsigned char)q;
        }
        const int nact = __syncthreads_count(pos >= 0);  // the placed orbits fill places 0 .. nact-1
        if (k + 1 < kS2Chunks)  // the next chunk's loads overlap this chunk's products
            s2_issue(cbase + kS2Chunk + threadIdx.x, norb, s, C, eC, bonds, have, st, ord, ld);
        if constexpr (MMA) {
            const int p1 = nact * (warp + 1) / kS2Warps;
            int p = nact * warp / kS2Warps;
            // the classes at the two ends of this warp's range
            const int cfirst = p < p1 ? (int)(csort[p] >> 1) : -1;
            const int clast = p < p1 ? (int)(csort[p1 - 1] >> 1) : -1;
            if (lane < 2) ecls[warp * 2 + lane] = lane == 0 ? cfirst : (clast != cfirst ? clast : -1);
            const int g = lane >> 2, t = lane & 3;
            int cur = -1;
            float nacc0 = 0.f, nacc1 = 0.f;  // class sums of rows g and g + 8 (this lane's columns)
            uint32_t ahi[2][2][4], alo[2][2][4];
            auto close_class = [&](int c) {
                if (c < 0) return;
                // rows g and g + 8: the four lanes of group g hold columns 2t, 2t + 1 of each tile
                nacc0 += __shfl_xor_sync(0xffffffffu, nacc0, 1);
                nacc1 += __shfl_xor_sync(0xffffffffu, nacc1, 1);
                nacc0 += __shfl_xor_sync(0xffffffffu, nacc0, 2);
                nacc1 += __shfl_xor_sync(0xffffffffu, nacc1, 2);
                if (t != 0) return;
                float* dst = c == cfirst ? edge + (warp * 2) * 16
                             : c == clast ? edge + (warp * 2 + 1) * 16
                                          : slots + c * 16;  // only this warp holds class c in this chunk
                if (c == cfirst || c == clast) {
                    dst[g] = nacc0;
                    dst[g + 8] = nacc1;
                } else {
                    dst[g] += nacc0;
                    dst[g + 8] += nacc1;
                }
            };
            while (p < p1) {  // one run (one key) per iteration; uniform over the warp
                const int qq = csort[p];
                // the run ends at the first place past p with another key (the keys ascend)
                int e = p + 1;
                for (;;) {
                    const int idx = e + lane;
                    const unsigned same = __ballot_sync(0xffffffffu, idx < p1 && csort[idx] == qq);
                    if (same != 0xffffffffu) {
                        e += __ffs(~same) - 1;
                        break;
                    }
                    e += 32;
                }
                const float wt = (qq & 1) ? 0.5f : 1.f;
                if ((qq >> 1) != cur) {
                    close_class(cur);
                    nacc0 = 0.f;
                    nacc1 = 0.f;
                    cur = qq >> 1;
                    mma_class_frags(cls_s + cur * 512, lane, ahi, alo);
                }
                for (; p < e; p += 8) {  // tiles of eight orbits; columns past the run are zero
                    const bool in = p + g < e;
                    const float* vr = vbuf + (p + g) * kS2Row + t;
                    uint32_t bhi[4], blo[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {  // k = t + 4 j: b0, b1 of k-step 0, then of k-step 1
                        const float x = in ? vr[4 * j] : 0.f;
                        const uint32_t h = tf32_hi(x);
                        bhi[j] = h;
                        blo[j] = __float_as_uint(x - __uint_as_float(h));
                    }
                    float dy[4] = {0.f, 0.f, 0.f, 0.f}, ds[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int ks = 0; ks < 2; ++ks) {
                        mma_tf32(dy, ahi[0][ks], bhi[2 * ks], bhi[2 * ks + 1]);
                        mma_tf32(dy, ahi[0][ks], blo[2 * ks], blo[2 * ks + 1]);
                        mma_tf32(dy, alo[0][ks], bhi[2 * ks], bhi[2 * ks + 1]);
                        mma_tf32(ds, ahi[1][ks], bhi[2 * ks], bhi[2 * ks + 1]);
                        mma_tf32(ds, ahi[1][ks], blo[2 * ks], blo[2 * ks + 1]);
                        mma_tf32(ds, alo[1][ks], bhi[2 * ks], bhi[2 * ks + 1]);
                    }
                    nacc0 += wt * (dy[0] * dy[0] + dy[1] * dy[1]);
                    nacc1 += wt * (dy[2] * dy[2] + dy[3] * dy[3]);
                    __syncwarp();  // every lane has read these rows before S overwrites them
                    // S of orbits 2t, 2t + 1 of the tile, rows g and g + 8
                    if (p + 2 * t < e) {
                        vbuf[(p + 2 * t) * kS2Row + g] = ds[0];
                        vbuf[(p + 2 * t) * kS2Row + g + 8] = ds[2];
                    }
                    if (p + 2 * t + 1 < e) {
                        vbuf[(p + 2 * t + 1) * kS2Row + g] = ds[1];
                        vbuf[(p + 2 * t + 1) * kS2Row + g + 8] = ds[3];
                    }
                    __syncwarp();
                }
                p = e;
            }
            close_class(cur);
        } else
        {
            const int p1 = nact * (warp + 1) / kS2Warps;
            int p = nact * warp / kS2Warps;
            // the classes at the two ends of this warp's range
            const int cfirst = p < p1 ? (int)(csort[p] >> 1) : -1;
            const int clast = p < p1 ? (int)(csort[p1 - 1] >> 1) : -1;
            if (lane < 2) ecls[warp * 2 + lane] = lane == 0 ? cfirst : (clast != cfirst ? clast : -1);
            int cur = -1;
            float nacc = 0.f;
            f2 r[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) r[m] = 0ull;
            auto close_class = [&](int c) {
                if (c < 0 || part != 0) return;
                if (c == cfirst) edge[(warp * 2) * 16 + row] = nacc;
                else if (c == clast) edge[(warp * 2 + 1) * 16 + row] = nacc;
                else slots[c * 16 + row] += nacc;  // only this warp holds class c in this chunk
            };
            while (p < p1) {  // one run (one key) per iteration; uniform over the warp
                const int qq = csort[p];
                // the run ends at the first place past p with another key (the keys ascend)
                int e = p + 1;
                for (;;) {
                    const int idx = e + lane;
                    const unsigned same = __ballot_sync(0xffffffffu, idx < p1 && csort[idx] == qq);
                    if (same != 0xffffffffu) {
                        e += __ffs(~same) - 1;
                        break;
                    }
                    e += 32;
                }
                const float wt = (qq & 1) ? 0.5f : 1.f;
                if ((qq >> 1) != cur) {
                    close_class(cur);
                    nacc = 0.f;
                    cur = qq >> 1;
                    const ulonglong2* rp = reinterpret_cast<const ulonglong2*>(cls_s + cur * 512 + lane * 16);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const ulonglong2 t = rp[u ^ ((lane >> 1) & 3)];
                        r[2 * u] = t.x;
                        r[2 * u + 1] = t.y;
                    }
                }
                for (; p + 4 <= e; p += 4) {
                    f2 v0[8], v1[8], v2[8], v3[8];
                    sorted_row(vbuf + p * kS2Row, v0);
                    sorted_row(vbuf + (p + 1) * kS2Row, v1);
                    sorted_row(vbuf + (p + 2) * kS2Row, v2);
                    sorted_row(vbuf + (p + 3) * kS2Row, v3);
                    const float y0 = sorted_dot(r, v0), y1 = sorted_dot(r, v1);
                    const float y2 = sorted_dot(r, v2), y3 = sorted_dot(r, v3);
                    __syncwarp();  // every lane has read these rows before S overwrites them
                    if (part == 0) {
                        nacc += wt * y0 * y0;
                        nacc += wt * y1 * y1;
                        nacc += wt * y2 * y2;
                        nacc += wt * y3 * y3;
                    } else {
                        vbuf[p * kS2Row + row] = y0;
                        vbuf[(p + 1) * kS2Row + row] = y1;
                        vbuf[(p + 2) * kS2Row + row] = y2;
                        vbuf[(p + 3) * kS2Row + row] = y3;
                    }
                    __syncwarp();
                }
                for (; p < e; ++p) {
                    f2 v0[8];
                    sorted_row(vbuf + p * kS2Row, v0);
                    const float y0 = sorted_dot(r, v0);
                    __syncwarp();
                    if (part == 0) nacc += wt * y0 * y0;
                    else vbuf[p * kS2Row + row] = y0;
                    __syncwarp();
                }
            }
            close_class(cur);
        }
        __syncthreads();
        // the end-of-range sums, warp by warp (a fixed order)
        if (threadIdx.x < 16) {
            for (int wp = 0; wp < kS2Warps; ++wp)
                for (int e2 = 0; e2 < 2; ++e2) {
                    const int c = ecls[wp * 2 + e2];
                    if (c >= 0) slots[c * 16 + threadIdx.x] += edge[(wp * 2 + e2) * 16 + threadIdx.x];
                }
        }
        if (pos >= 0) {
            float S[16];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float4 t = *reinterpret_cast<const float4*>(vbuf + pos * kS2Row + 4 * u);
                S[4 * u] = t.x;
                S[4 * u + 1] = t.y;
                S[4 * u + 2] = t.z;
                S[4 * u + 3] = t.w;
            }
#pragma unroll
            for (int pp = 0; pp < 8; ++pp) {
                const int a = pp >> 2, b = (pp >> 1) & 1, c = pp & 1;
                if (single && a == 1) continue;
                const uint32_t i0 = b0 ^ (a ? dp : 0u) ^ (b ? eC : 0u) ^ (c ? mc : 0u);
                st[i0] = S[SLOT(a, b, c, 0)];
                st[i0 ^ macc] = S[SLOT(a, b, c, 1)];
            }
        }
        __syncthreads();  // S read back and edges added before the next chunk reuses the buffers
    }
    // this CTA's places for the move are recorded: later steps take them from the table
    if (ord && !have && threadIdx.x == 0) ready[(uint64_t)blockIdx.x * kMaxMoves + C] = 1;
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < nc * 16u; e += blockDim.x) npart[(uint64_t)blockIdx.x * kMaxCls * 16 + e] = (double)slots[e];
}

// g_k of a walk from its class sums (algo 1): g_k = sum_{c,i} N_{c,i} d_{c,k,i}, with
// N_{c,i} the class sums added over the walk's CTAs (first, into shared memory).  A
// class's d block is [k][i] (16 i per k, at offset 512 of its class-data entry):
// thread t takes k = t / 4 and i = 4 (t % 4) .. +3, so a warp reads eight k rows of
// the block contiguously, and the four threads of a k are combined by shuffles
// (a fixed order: the sums are deterministic).  kMeasThreads = 4 kMaxL threads.
constexpr int kMeasThreads = 4 * kMaxL;

template <typename T>
__device__ void cls_overlaps(const WalkDev& W, const WalkRec& R, uint32_t nc, const double* __restrict__ npart,
                             const T* __restrict__ cls, const uint32_t* __restrict__ gid, int w, int L, double* g,
                             double* Nsh) {
    const int t = threadIdx.x;
    for (uint32_t e = t; e < nc * 16u; e += kMeasThreads) {
        double Nv = 0.0;
        for (uint32_t c = 0; c < W.ncta; ++c) Nv += npart[(uint64_t)(W.cta0 + c) * kMaxCls * 16 + e];
        Nsh[e] = Nv;
    }
    __syncthreads();
    const int k = t >> 2, q4 = t & 3;
    double acc = 0.0;
    if (k < L) {
        for (uint32_t c = 0; c < nc; ++c) {
            const T* d = cls + cls_entry(W, R, gid, w, c) * kClsStride + 512 + k * 16 + 4 * q4;
            const double* Nc = Nsh + c * 16 + 4 * q4;
            acc += Nc[0] * (double)d[0] + Nc[1] * (double)d[1] + Nc[2] * (double)d[2] + Nc[3] * (double)d[3];
        }
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    if (k < L && q4 == 0) g[k] = acc;
}

// One CTA of kMeasThreads threads per walk.
__global__ void __launch_bounds__(kMeasThreads) k_walk_measure(const WalkDev* __restrict__ walks, WalkRec* __restrict__ recs,
                               const double* __restrict__ partial, const double* __restrict__ cos64,
                               double* __restrict__ trace, unsigned int* __restrict__ running, int algo,
                               const uint32_t* __restrict__ ncls, const void* __restrict__ cls,
                               const uint32_t* __restrict__ gid, int cls_f64) {
    const int w = blockIdx.x;
    const WalkDev& W = walks[w];
    WalkRec& R = recs[w];
    if (R.status != 0) return;
    __shared__ double g[kMaxL], P[kMaxL];
    __shared__ double Nsh[kMaxCls * 16];
    __shared__ double n2;
    const int L = 1 << W.q;
    const int t = threadIdx.x;
    if (algo == 1) {
        const uint32_t nc = ncls[(uint64_t)w * kMaxMoves + R.C];
        if (cls_f64) cls_overlaps<double>(W, R, nc, partial, (const double*)cls, gid, w, L, g, Nsh);
        else cls_overlaps<float>(W, R, nc, partial, (const float*)cls, gid, w, L, g, Nsh);
    } else if (t < L) {
        double sum = 0.0;
        for (uint32_t c = 0; c < W.ncta; ++c) sum += partial[(uint64_t)(W.cta0 + c) * kMaxL + t];
        g[t] = sum;
    }
    __syncthreads();
    if (t < L) {
        double acc = 0.0;
        const int stride = kMaxL / L;
        for (int j = 1; j < L; ++j) acc += (double)(L - j) * g[j] * cos64[((t * j) % L) * stride];
        P[t] = ((double)L * g[0] + 2.0 * acc) / ((double)L * L);
        if (t == 0) {
            double a2 = 0.0;
            for (int j = 1; j < L; ++j) a2 += (double)(L - j) * g[j];
            n2 = (double)L * g[0] + 2.0 * a2;
        }
    }
    __syncthreads();
    if (t != 0) return;
    uint64_t rs = R.rng_state;
    const uint64_t ri = R.rng_inc;
    // walk-phase readout, qubit by qubit (c = r < p1)
    uint32_t m = 0;
    for (int j = 0; j < W.q; ++j) {
        const double r = pcg_doub(rs, ri);
        double num = 0.0, den = 0.0;
        const uint32_t lowmask = (1u << j) - 1u;
        for (int v = 0; v < L; ++v) {
            if (((uint32_t)v & lowmask) != m) continue;
            den += P[v];
            if ((v >> j) & 1) num += P[v];
        }
        const double p1 = den > 0.0 ? num / den : 0.0;
        if (r < p1) m |= 1u << j;
    }
    double ptot = 0.0;
    for (int v = 0; v < L; ++v) ptot += P[v];
    const double p0 = ptot > 0.0 ? P[0] / ptot : 0.0;
    if (trace) trace[W.trace_off + R.total] = p0;
    R.last_p0 = p0;
    R.total += 1;
    if (m == 0) {
        R.scale = 1.0 / sqrt(n2);
        R.fresh = 0;
        R.att += 1;
        if (R.att == W.nominal) R.status = 2;
    } else {
        R.restarts += 1;
        R.fresh = 1;
        R.att = 0;
        R.scale = 1.0;
    }
    if (R.status == 0 && R.total >= W.cap) R.status = 1;
    if (R.status == 0) {
        R.C = draw_move(rs, ri, W.s);
        R.beta_k = (double)(R.att / (uint32_t)W.per + 1) * W.beta / (double)W.stages;
    } else {
        atomicSub(running, 1u);
    }
    R.rng_state = rs;
}

__global__ void k_walk_init(const WalkDev* __restrict__ walks, WalkRec* __restrict__ recs, int n) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n) return;
    const WalkDev& W = walks[w];
    WalkRec R;
    // pcg32::seed(initstate, initseq = 1)
    R.rng_state = 0;
    R.rng_inc = (1ull << 1u) | 1u;
    pcg_next(R.rng_state, R.rng_inc);
    R.rng_state += W.seed;
    pcg_next(R.rng_state, R.rng_inc);
    R.C = draw_move(R.rng_state, R.rng_inc, W.s);
    R.beta_k = W.beta / (double)W.stages;
    R.scale = 1.0;
    R.last_p0 = 0.0;
    R.fresh = 1;
    R.att = 0;
    R.total = 0;
    R.restarts = 0;
    R.status = 0;
    R.readout = 0;
    R.pad = 0;
    recs[w] = R;
}

// Spin readout of completed walks: P(x) = sum over (acc, d) of psi^2, then the
// s spins measured one by one.  One CTA per walk.
template <typename T>
__global__ void __launch_bounds__(1024) k_walk_readout(const WalkDev* __restrict__ walks, WalkRec* __restrict__ recs,
                                                       const T* __restrict__ states) {
    const int w = blockIdx.x;
    const WalkDev& W = walks[w];
    WalkRec& R = recs[w];
    if (R.status != 2) return;
    extern __shared__ double px[];
    const uint32_t N = 1u << W.s;
    const T* st = states + W.state_off;
    for (uint32_t x = threadIdx.x; x < N; x += blockDim.x) {
        double acc = 0.0;
        for (uint32_t row = 0; row < 2 * N; ++row) {
            const double v = (double)st[(uint64_t)row * N + x];
            acc += v * v;
        }
        px[x] = acc;
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    uint64_t rs = R.rng_state;
    const uint64_t ri = R.rng_inc;
    uint32_t m = 0;
    for (int j = 0; j < W.s; ++j) {
        double r = 0.0;
        if (lane == 0) r = pcg_doub(rs, ri);
        const uint32_t lowmask = (1u << j) - 1u;
        double num = 0.0, den = 0.0;
        for (uint32_t x = lane; x < N; x += 32) {
            if ((x & lowmask) != m) continue;
            den += px[x];
            if ((x >> j) & 1u) num += px[x];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            num += __shfl_xor_sync(0xffffffffu, num, off);
            den += __shfl_xor_sync(0xffffffffu, den, off);
        }
        int c = 0;
        if (lane == 0) c = r < (den > 0.0 ? num / den : 0.0) ? 1 : 0;
        c = __shfl_sync(0xffffffffu, c, 0);
        m |= (uint32_t)c << j;
    }
    if (lane == 0) {
        R.readout = m;
        R.status = 3;
        R.rng_state = rs;
    }
}

}  // namespace sqw

namespace {
int wfail(int code, const std::string& m) {
    sqi::set_error(m.c_str());
    return code;
}
}  // namespace

extern "C" int sq_set_walk_orbit_warps(int warps) {
    if (warps != 8 && warps != 16) return wfail(SQ_ERR_ARG, "orbit-pass warps must be 8 or 16");
    sqw::g_orbit_warps.store(warps);
    return SQ_OK;
}

extern "C" int sq_set_walk_mma(int on) {
    if (on != 0 && on != 1) return wfail(SQ_ERR_ARG, "walk mma must be 0 or 1");
    sqw::g_walk_mma.store(on);
    return SQ_OK;
}

extern "C" int sq_set_walk_presort(int on) {
    if (on != 0 && on != 1) return wfail(SQ_ERR_ARG, "presort must be 0 or 1");
    sqw::g_presort.store(on);
    return SQ_OK;
}

extern "C" int sq_qsa_walk_batch(const sq_qsa_walk* walks, uint32_t nwalks, int precision,
                                 sq_qsa_walk_result* results, double* p0_trace, float* kernel_ms) {
    using namespace sqw;
    if (kernel_ms) *kernel_ms = 0.f;
    if (!walks || nwalks == 0 || !results) return wfail(SQ_ERR_ARG, "null or empty walk list");
    if (precision != SQ_F64 && precision != SQ_F32) return wfail(SQ_ERR_ARG, "unknown precision");
    const size_t esz = precision == SQ_F64 ? 8 : 4;
    const uint32_t algo = walks[0].algo;
    if (algo > 2)
        return wfail(SQ_ERR_ARG, "unknown walk algorithm (0: per-orbit iteration, 1: orbit classes, 2: orbit classes "
                                 "prepared per step)");
    for (uint32_t i = 1; i < nwalks; ++i)
        if (walks[i].algo != algo) return wfail(SQ_ERR_ARG, "all walks of a batch use one algorithm");
    const bool classes = algo >= 1;
    const uint32_t orbits_per_cta = classes ? (uint32_t)kClsOrbitsPerCta : (uint32_t)kOrbitsPerCta;
    std::vector<WalkDev> wd(nwalks);
    std::vector<int> energies;
    std::vector<int> cta_walk;
    uint64_t state_elems = 0, trace_len = 0, order_len = 0;
    uint32_t max_cap = 0;
    for (uint32_t i = 0; i < nwalks; ++i) {
        const sq_qsa_walk& a = walks[i];
        if (a.spins < 2 || a.spins > 12) return wfail(SQ_ERR_ARG, "ring length out of range (2..12 spins)");
        if (a.phase_qbits < 1 || a.phase_qbits > 6) return wfail(SQ_ERR_ARG, "walk-phase register out of range (1..6 qubits)");
        if (a.stages == 0 || a.steps_per_stage == 0) return wfail(SQ_ERR_ARG, "empty annealing schedule");
        if ((uint64_t)a.stages * a.steps_per_stage > (1u << 24)) return wfail(SQ_ERR_ARG, "annealing schedule too long");
        if (!(a.beta >= 0.0) || !std::isfinite(a.beta)) return wfail(SQ_ERR_ARG, "beta must be finite and non-negative");
        int sumJ = 0;
        for (uint32_t b = 0; b < a.spins; ++b) {
            if (a.J[b] < -kMaxJ || a.J[b] > kMaxJ) return wfail(SQ_ERR_ARG, "couplings must lie in -8..8");
            sumJ += std::abs(a.J[b]);
        }
        WalkDev& d = wd[i];
        d.s = (int)a.spins;
        d.q = (int)a.phase_qbits;
        d.stages = (int)a.stages;
        d.per = (int)a.steps_per_stage;
        d.nominal = a.stages * a.steps_per_stage;
        const uint64_t cap = a.max_steps ? (uint64_t)a.max_steps : 8ull * d.nominal;
        d.cap = (uint32_t)std::min<uint64_t>(cap, 0xffffffffu);
        d.beta = a.beta;
        d.seed = a.seed;
        d.state_off = state_elems;
        d.trace_off = trace_len;
        d.e_off = (uint32_t)energies.size();
        d.dmax = 2 * sumJ;
        int jmin = 0, jmax = 0;
        for (uint32_t b = 0; b < a.spins; ++b) jmin = std::min(jmin, (int)a.J[b]);
        d.joff = -jmin;
        for (uint32_t b = 0; b < a.spins; ++b) jmax = std::max(jmax, (int)a.J[b] + d.joff);
        d.jnp = 0;
        while (d.jnp < 5 && (jmax >> d.jnp) != 0) ++d.jnp;  // J_b + joff <= 16: 5 planes at most
        for (int k = 0; k < 5; ++k) {
            d.jplane[k] = 0;
            for (uint32_t b = 0; b < a.spins; ++b)
                if ((((int)a.J[b] + d.joff) >> k) & 1) d.jplane[k] |= 1u << b;
        }
        const uint32_t N = 1u << a.spins;
        for (uint32_t x = 0; x < N; ++x) {
            int E = 0;
            for (uint32_t b = 0; b < a.spins; ++b) {
                const int sb = 1 - 2 * (int)((x >> b) & 1u);
                const uint32_t b2 = (b + 1) % a.spins;
                const int sb2 = 1 - 2 * (int)((x >> b2) & 1u);
                E -= a.J[b] * sb * sb2;
            }
            energies.push_back(E);
        }
        const uint32_t ncta = (norbits(d.s) + orbits_per_cta - 1) / orbits_per_cta;
        d.cta0 = (uint32_t)cta_walk.size();
        d.ncta = ncta;
        d.ord_off = order_len;
        order_len += order_entries(d.s, ncta);
        for (uint32_t c = 0; c < ncta; ++c) cta_walk.push_back((int)i);
        state_elems += 2ull << (2 * a.spins);
        trace_len += d.cap;
        max_cap = std::max(max_cap, d.cap);
    }
    std::vector<double> cos64(kMaxL);
    for (int t = 0; t < kMaxL; ++t) cos64[t] = std::cos(2.0 * M_PI * (double)t / (double)kMaxL);

    WalkDev* d_walks = nullptr;
    WalkRec* d_recs = nullptr;
    int* d_cta = nullptr;
    int* d_E = nullptr;
    void* d_states = nullptr;
    double* d_partial = nullptr;
    double* d_cos = nullptr;
    double* d_trace = nullptr;
    unsigned int* d_running = nullptr;
    unsigned long long* d_keys = nullptr;
    uint32_t* d_ncls = nullptr;
    void* d_cls = nullptr;
    int* d_jobs = nullptr;
    uint32_t* d_gid = nullptr;
    unsigned long long* d_gkeys = nullptr;
    double* d_sbeta = nullptr;
    int* d_sq = nullptr;
    uint16_t* d_order = nullptr;
    unsigned char* d_ready = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_order);
        cudaFree(d_ready);
        cudaFree(d_gid);
        cudaFree(d_gkeys);
        cudaFree(d_sbeta);
        cudaFree(d_sq);
        cudaFree(d_keys);
        cudaFree(d_ncls);
        cudaFree(d_cls);
        cudaFree(d_jobs);
        cudaFree(d_walks);
        cudaFree(d_recs);
        cudaFree(d_cta);
        cudaFree(d_E);
        cudaFree(d_states);
        cudaFree(d_partial);
        cudaFree(d_cos);
        cudaFree(d_trace);
        cudaFree(d_running);
    };
    const size_t nct = cta_walk.size();
    bool ok = cudaMalloc(&d_walks, sizeof(WalkDev) * nwalks) == cudaSuccess &&
              cudaMalloc(&d_recs, sizeof(WalkRec) * nwalks) == cudaSuccess &&
              cudaMalloc(&d_cta, sizeof(int) * nct) == cudaSuccess &&
              cudaMalloc(&d_E, sizeof(int) * energies.size()) == cudaSuccess &&
              cudaMalloc(&d_states, esz * state_elems) == cudaSuccess &&
              cudaMalloc(&d_partial, sizeof(double) * (classes ? (size_t)kMaxCls * 16 : (size_t)kMaxL) * nct) ==
                  cudaSuccess &&
              (!classes ||
               (cudaMalloc(&d_keys, sizeof(unsigned long long) * nwalks * kMaxMoves * kMaxCls) == cudaSuccess &&
                cudaMalloc(&d_ncls, sizeof(uint32_t) * nwalks * kMaxMoves) == cudaSuccess &&
                cudaMalloc(&d_jobs, sizeof(int) * 2 * nwalks * kMaxMoves) == cudaSuccess)) &&
              cudaMalloc(&d_cos, sizeof(double) * kMaxL) == cudaSuccess &&
              cudaMalloc(&d_running, sizeof(unsigned int)) == cudaSuccess &&
              (!p0_trace || cudaMalloc(&d_trace, sizeof(double) * trace_len) == cudaSuccess);
    if (!ok) {
        cudaGetLastError();
        cleanup();
        return wfail(SQ_ERR_NOMEM, "device allocation for the walk batch failed");
    }
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    const unsigned int nrun = nwalks;
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_walks, wd.data(), sizeof(WalkDev) * nwalks, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_cta, cta_walk.data(), sizeof(int) * nct, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_E, energies.data(), sizeof(int) * energies.size(), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_cos, cos64.data(), sizeof(double) * kMaxL, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_running, &nrun, sizeof(unsigned int), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess && d_trace) err = cudaMemsetAsync(d_trace, 0, sizeof(double) * trace_len, st);
    if (err == cudaSuccess) err = cudaEventRecord(e0, st);
    if (err == cudaSuccess) {
        k_walk_init<<<(nwalks + 127) / 128, 128, 0, st>>>(d_walks, d_recs, (int)nwalks);
        err = cudaGetLastError();
    }
    size_t prep_smem = 0, cls_smem = 0;
    int nslot = 1;
    bool staged = false, sorted = false, sorted2 = false;
    const bool use_mma = g_walk_mma.load() == 1;
    bool tabled = false;
    uint32_t tab_entries = 0, tab_slots = 0;
    if (err == cudaSuccess && classes) {
        // the orbit classes of every (walk, move), once per batch
        std::vector<int> jw, jm;
        for (uint32_t i = 0; i < nwalks; ++i)
            for (uint32_t c = 0; c < walks[i].spins; ++c) {
                jw.push_back((int)i);
                jm.push_back((int)c);
            }
        const size_t nj = jw.size();
        std::vector<int> jobs(jw);
        jobs.insert(jobs.end(), jm.begin(), jm.end());
        err = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(int) * 2 * nj, cudaMemcpyHostToDevice, st);
        if (err == cudaSuccess) {
            k_cls_keys<<<(unsigned)nj, kThreads, 0, st>>>(d_walks, d_E, d_jobs, d_jobs + nj, d_keys, d_ncls);
            err = cudaGetLastError();
        }
        std::vector<uint32_t> nc(nwalks * kMaxMoves, 0u);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(nc.data(), d_ncls, sizeof(uint32_t) * nc.size(), cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
        if (err == cudaSuccess) {
            for (size_t j = 0; j < nj; ++j)
                if (nc[(size_t)jw[j] * kMaxMoves + jm[j]] > (uint32_t)kMaxCls) {
                    cudaStreamDestroy(st);
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    cleanup();
                    return wfail(SQ_ERR_UNSUPPORTED, "more orbit classes than algorithm 1 holds (96); use algorithm 0");
                }
            // The class data depend only on (key, beta_k, q): one table for the batch,
            // entry = key index * nslot + temperature slot, when it fits; otherwise
            // (and for algo 2) per walk, prepared every step.
            std::vector<unsigned long long> hk((size_t)nwalks * kMaxMoves * kMaxCls);
            err = cudaMemcpyAsync(hk.data(), d_keys, sizeof(unsigned long long) * hk.size(), cudaMemcpyDeviceToHost, st);
            if (err == cudaSuccess) err = cudaStreamSynchronize(st);
            std::vector<unsigned long long> gkeys;
            std::unordered_map<unsigned long long, uint32_t> kid;
            std::vector<uint32_t> gk((size_t)nwalks * kMaxMoves * kMaxCls, 0u);
            std::map<std::tuple<uint64_t, uint32_t, int>, uint32_t> sched;  // (beta bits, stages, q) -> slot0
            std::vector<double> sbeta;
            std::vector<int> sq;
            for (uint32_t i = 0; err == cudaSuccess && i < nwalks; ++i) {
                for (uint32_t c = 0; c < walks[i].spins; ++c) {
                    const size_t base = ((size_t)i * kMaxMoves + c) * kMaxCls;
                    for (uint32_t k = 0; k < nc[(size_t)i * kMaxMoves + c]; ++k) {
                        auto it = kid.find(hk[base + k]);
                        if (it == kid.end()) {
                            it = kid.emplace(hk[base + k], (uint32_t)gkeys.size()).first;
                            gkeys.push_back(hk[base + k]);
                        }
                        gk[base + k] = it->second;
                    }
                }
                uint64_t bbits;
                std::memcpy(&bbits, &walks[i].beta, sizeof bbits);
                const auto key = std::make_tuple(bbits, walks[i].stages, (int)walks[i].phase_qbits);
                auto it = sched.find(key);
                if (it == sched.end()) {
                    it = sched.emplace(key, (uint32_t)sbeta.size()).first;
                    // the stage temperatures exactly as the step loop forms them
                    for (uint32_t j = 0; j < walks[i].stages; ++j) {
                        sbeta.push_back((double)(j + 1) * walks[i].beta / (double)walks[i].stages);
                        sq.push_back((int)walks[i].phase_qbits);
                    }
                }
                wd[i].slot0 = it->second;
            }
            const uint64_t nslot_t = sbeta.size(), nentry = gkeys.size() * nslot_t;
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            const uint64_t tab_bytes = nentry * kClsStride * esz;
            tabled = err == cudaSuccess && algo == 1 && nentry > 0 && nentry < (1ull << 31) &&
                     tab_bytes <= std::min<uint64_t>(kTableBudget, free_b / 4);
            if (err == cudaSuccess && tabled) {
                for (size_t j = 0; j < gk.size(); ++j) gk[j] *= (uint32_t)nslot_t;
                const bool aok = cudaMalloc(&d_cls, tab_bytes) == cudaSuccess &&
                                 cudaMalloc(&d_gid, sizeof(uint32_t) * gk.size()) == cudaSuccess &&
                                 cudaMalloc(&d_gkeys, sizeof(unsigned long long) * gkeys.size()) == cudaSuccess &&
                                 cudaMalloc(&d_sbeta, sizeof(double) * nslot_t) == cudaSuccess &&
                                 cudaMalloc(&d_sq, sizeof(int) * nslot_t) == cudaSuccess;
                if (!aok) {
                    cudaGetLastError();
                    err = cudaErrorMemoryAllocation;
                }
                if (err == cudaSuccess)
                    err = cudaMemcpyAsync(d_gid, gk.data(), sizeof(uint32_t) * gk.size(), cudaMemcpyHostToDevice, st);
                if (err == cudaSuccess)
                    err = cudaMemcpyAsync(d_gkeys, gkeys.data(), sizeof(unsigned long long) * gkeys.size(),
                                          cudaMemcpyHostToDevice, st);
                if (err == cudaSuccess)
                    err = cudaMemcpyAsync(d_sbeta, sbeta.data(), sizeof(double) * nslot_t, cudaMemcpyHostToDevice, st);
                if (err == cudaSuccess) err = cudaMemcpyAsync(d_sq, sq.data(), sizeof(int) * nslot_t, cudaMemcpyHostToDevice, st);
                // slot0 joins the walk records on the device
                if (err == cudaSuccess)
                    err = cudaMemcpyAsync(d_walks, wd.data(), sizeof(WalkDev) * nwalks, cudaMemcpyHostToDevice, st);
                tab_entries = (uint32_t)nentry;
                tab_slots = (uint32_t)nslot_t;
            } else if (err == cudaSuccess) {
                if (cudaMalloc(&d_cls, esz * nwalks * kMaxCls * kClsStride) != cudaSuccess) {
                    cudaGetLastError();
                    err = cudaErrorMemoryAllocation;
                }
            }
            nslot = 1;
            for (size_t j = 0; j < nj; ++j) nslot = std::max<int>(nslot, (int)nc[(size_t)jw[j] * kMaxMoves + jm[j]]);
            prep_smem = esz * (kPrepThreads / 32) * 5 * 16 * 17;
            const size_t base_smem = esz * ((kThreads / 32) * (size_t)nslot * 16 + (kThreads / 32) * 32 * 16) +
                                     sizeof(int) * (kThreads / 32) * 32 + 16 + 2 * sizeof(unsigned long long) * kMaxCls;
            const size_t staged_smem = base_smem + esz * (size_t)nslot * kStagedStride;
            const size_t sorted_smem =
                sizeof(float) * ((size_t)nslot * 512 + (size_t)kWarps * nslot * 16 + 2 * (size_t)kSortChunk * kRow) +
                sizeof(unsigned long long) * (kHash + kMaxCls) +
                sizeof(int) * ((size_t)(kWarps + 2) * 2 * nslot + kWarps + 4) + kSortChunk;
            int optin = 0, cur_dev = 0;
            if (err == cudaSuccess) err = cudaGetDevice(&cur_dev);  // the device the walks run on
            if (err == cudaSuccess)
                err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, cur_dev);
            const size_t sorted2_smem = sorted2_smem_bytes(nslot);
            sorted2 = precision == SQ_F32 && g_orbit_warps.load() == 16 && sorted2_smem <= (size_t)optin;
            sorted = !sorted2 && precision == SQ_F32 && sorted_smem <= (size_t)optin;
            staged = !sorted2 && !sorted && precision == SQ_F32 && staged_smem <= (size_t)optin;
            cls_smem = sorted2 ? sorted2_smem : sorted ? sorted_smem : staged ? staged_smem : base_smem;
            // the 16-warp pass records each CTA's orbit places per move where the batch's table fits
            const uint64_t order_bytes = order_len * sizeof(uint16_t);
            if (err == cudaSuccess && sorted2 && g_presort.load() == 1 &&
                order_bytes <= std::min<uint64_t>(kOrderBudget, free_b / 4)) {
                if (cudaMalloc(&d_order, order_bytes) == cudaSuccess &&
                    cudaMalloc(&d_ready, nct * kMaxMoves) == cudaSuccess) {
                    err = cudaMemsetAsync(d_order, 0xff, order_bytes, st);
                    if (err == cudaSuccess) err = cudaMemsetAsync(d_ready, 0, nct * kMaxMoves, st);
                } else {
                    cudaGetLastError();  // no room: the 16-warp pass sorts every chunk at every step
                    cudaFree(d_order);
                    cudaFree(d_ready);
                    d_order = nullptr;
                    d_ready = nullptr;
                }
            }
            if (err == cudaSuccess && precision == SQ_F64) {
                err = tabled ? cudaFuncSetAttribute(k_cls_table<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)prep_smem)
                             : cudaFuncSetAttribute(k_cls_prep<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)prep_smem);
                if (err == cudaSuccess)
                    err = cudaFuncSetAttribute(k_walk_step_cls<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)cls_smem);
            } else if (err == cudaSuccess) {
                err = tabled ? cudaFuncSetAttribute(k_cls_table<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)prep_smem)
                             : cudaFuncSetAttribute(k_cls_prep<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)prep_smem);
                if (err == cudaSuccess)
                    err = sorted2  ? (use_mma ? cudaFuncSetAttribute(k_walk_step_sorted2<true>,
                                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                                     (int)cls_smem)
                                              : cudaFuncSetAttribute(k_walk_step_sorted2<false>,
                                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                                     (int)cls_smem))
                          : sorted ? cudaFuncSetAttribute(k_walk_step_sorted, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)cls_smem)
                          : staged ? cudaFuncSetAttribute(k_walk_step_cls<float, true>,
                                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cls_smem)
                                   : cudaFuncSetAttribute(k_walk_step_cls<float, false>,
                                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cls_smem);
            }
            if (err == cudaSuccess && tabled) {
                const unsigned grid = (tab_entries + kPrepThreads / 32 - 1) / (kPrepThreads / 32);
                if (precision == SQ_F64)
                    k_cls_table<double><<<grid, kPrepThreads, prep_smem, st>>>(d_gkeys, d_sbeta, d_sq, tab_slots,
                                                                               tab_entries, (double*)d_cls);
                else
                    k_cls_table<float><<<grid, kPrepThreads, prep_smem, st>>>(d_gkeys, d_sbeta, d_sq, tab_slots,
                                                                              tab_entries, (float*)d_cls);
                err = cudaGetLastError();
            }
        }
    }
    // advance every running walk one step per iteration; poll the running count
    // every `chunk` iterations
    const uint32_t chunk = 16;
    uint32_t iter = 0;
    unsigned int left = nrun;
    while (err == cudaSuccess && left > 0 && iter < max_cap) {
        const uint32_t q = std::min(chunk, max_cap - iter);
        for (uint32_t k = 0; k < q && err == cudaSuccess; ++k) {
            if (classes) {
                if (precision == SQ_F64) {
                    if (!tabled)
                        k_cls_prep<double><<<nwalks, kPrepThreads, prep_smem, st>>>(d_walks, d_recs, d_keys, d_ncls,
                                                                                    (double*)d_cls);
                    k_walk_step_cls<double, false><<<(unsigned)nct, kThreads, cls_smem, st>>>(
                        d_walks, d_cta, d_recs, d_E, d_keys, d_ncls, (const double*)d_cls, d_gid, (double*)d_states,
                        d_partial, nslot);
                } else {
                    if (!tabled)
                        k_cls_prep<float><<<nwalks, kPrepThreads, prep_smem, st>>>(d_walks, d_recs, d_keys, d_ncls,
                                                                                   (float*)d_cls);
                    if (sorted2 && use_mma)
                        k_walk_step_sorted2<true><<<(unsigned)nct, kS2Threads, cls_smem, st>>>(
                            d_walks, d_cta, d_recs, d_keys, d_ncls, (const float*)d_cls, d_gid, d_order, d_ready,
                            (float*)d_states, d_partial, nslot);
                    else if (sorted2)
                        k_walk_step_sorted2<false><<<(unsigned)nct, kS2Threads, cls_smem, st>>>(
                            d_walks, d_cta, d_recs, d_keys, d_ncls, (const float*)d_cls, d_gid, d_order, d_ready,
                            (float*)d_states, d_partial, nslot);
                    else if (sorted)
                        k_walk_step_sorted<<<(unsigned)nct, kThreads, cls_smem, st>>>(
                            d_walks, d_cta, d_recs, d_keys, d_ncls, (const float*)d_cls, d_gid, (float*)d_states,
                            d_partial, nslot);
                    else if (staged)
                        k_walk_step_cls<float, true><<<(unsigned)nct, kThreads, cls_smem, st>>>(
                            d_walks, d_cta, d_recs, d_E, d_keys, d_ncls, (const float*)d_cls, d_gid, (float*)d_states,
                            d_partial, nslot);
                    else
                        k_walk_step_cls<float, false><<<(unsigned)nct, kThreads, cls_smem, st>>>(
                            d_walks, d_cta, d_recs, d_E, d_keys, d_ncls, (const float*)d_cls, d_gid, (float*)d_states,
                            d_partial, nslot);
                }
            } else if (precision == SQ_F64) {
                k_walk_step<double><<<(unsigned)nct, kThreads, 0, st>>>(d_walks, d_cta, d_recs, d_E,
                                                                        (double*)d_states, d_partial);
            } else {
                k_walk_step<float><<<(unsigned)nct, kThreads, 0, st>>>(d_walks, d_cta, d_recs, d_E,
                                                                       (float*)d_states, d_partial);
            }
            err = cudaGetLastError();
            if (err != cudaSuccess) break;
            k_walk_measure<<<nwalks, kMeasThreads, 0, st>>>(d_walks, d_recs, d_partial, d_cos, d_trace, d_running,
                                                     classes ? 1 : 0, d_ncls, d_cls, d_gid, precision == SQ_F64 ? 1 : 0);
            err = cudaGetLastError();
        }
        iter += q;
        if (err == cudaSuccess) err = cudaMemcpyAsync(&left, d_running, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    }
    if (err == cudaSuccess) {
        uint32_t smax = 0;
        for (uint32_t i = 0; i < nwalks; ++i) smax = std::max<uint32_t>(smax, walks[i].spins);
        const size_t smem = sizeof(double) << smax;
        if (precision == SQ_F64) {
            err = cudaFuncSetAttribute(k_walk_readout<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (err == cudaSuccess) k_walk_readout<double><<<nwalks, 1024, smem, st>>>(d_walks, d_recs, (const double*)d_states);
        } else {
            err = cudaFuncSetAttribute(k_walk_readout<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (err == cudaSuccess) k_walk_readout<float><<<nwalks, 1024, smem, st>>>(d_walks, d_recs, (const float*)d_states);
        }
        if (err == cudaSuccess) err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    std::vector<WalkRec> rec(nwalks);
    if (err == cudaSuccess) err = cudaMemcpyAsync(rec.data(), d_recs, sizeof(WalkRec) * nwalks, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess && p0_trace)
        err = cudaMemcpyAsync(p0_trace, d_trace, sizeof(double) * trace_len, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    float ms = 0.f;
    if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    if (kernel_ms) *kernel_ms = ms;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cleanup();
    if (err == cudaErrorMemoryAllocation)
        return wfail(SQ_ERR_NOMEM, "device allocation for the walk batch's class data failed");
    if (err != cudaSuccess) return wfail(SQ_ERR_CUDA, std::string("walk batch: ") + cudaGetErrorString(err));
    for (uint32_t i = 0; i < nwalks; ++i) {
        const WalkRec& R = rec[i];
        sq_qsa_walk_result& o = results[i];
        const uint32_t s = walks[i].spins;
        o.done = R.status == 3 ? 1u : 0u;
        o.restarts = R.restarts;
        o.steps = R.total;
        o.readout = o.done ? R.readout : 0u;
        o.last_p0 = R.last_p0;
        o.E = 0.0;
        o.absM = 0.0;
        if (o.done) {
            o.E = (double)energies[wd[i].e_off + R.readout];
            int M = 0;
            for (uint32_t b = 0; b < s; ++b) M += 1 - 2 * (int)((R.readout >> b) & 1u);
            o.absM = (double)std::abs(M);
        }
    }
    return SQ_OK;
}
