// Batched quantum Metropolis sampling of transverse-field Ising rings, one chain
// per CTA, entirely on the device.
//
// System: H = -J sum_i Z_i Z_{i+1} - h sum_i X_i on a ring of s spins; exp(-iHt)
// as ceil(|t|/dt) first-order Trotter steps of width d = t/steps, each the ZZ
// bond phases exp(i J d Z_i Z_{i+1}) then exp(i h d X_i) on every spin; moves:
// Hadamard on spin i with probability 1/s; observable: magnetisation read in
// the Z basis.  The register layout, the QMS step (reset, phase estimation,
// move, acceptance oracle W, accept / restore loop, sampling branch) and the
// order of every PCG32 draw restate the reference's include/qms.cuh:128-545 and
// the driver loop of src/qms.cu:114-149, so each chain reproduces the reference
// CPU `qms` binary built with the same system (measured outcomes identical,
// amplitudes to rounding).
//
// GB300 mapping: a persistent grid of CTAs pulls chains from an atomic work
// counter (largest first); a chain's 2^n amplitudes stay in shared memory for
// its whole run (n <= 13 FP64 / 14 FP32; larger chains use a per-CTA buffer in
// global memory that stays L2-resident); gates are CTA-wide sweeps with no
// kernel launches and no host round trips; measurement probabilities are FP64
// block reductions; the bond phases of a Trotter step are applied as one
// diagonal (their product depends only on the number of domain walls).
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <cooperative_groups.h>

#include "sq.h"

namespace cg = cooperative_groups;

namespace sqi {
void set_error(const char* msg);
}

namespace sqb {

constexpr int kThreads = 256;

struct DevChain {
    int s, e, n, steps, therm, reset_each, max_reverse;
    double J, h, beta, dt;
    double t_pe, t_shift, pe_factor, c_factor;  // as the reference driver computes them
    uint64_t seed;
    int out_offset;  // first sample slot of this chain
    int warm;
    double ry[20];   // warm-start RY angles per spin
};

struct Shared {
    double red[2][32];
    double bcast_d[4];
    int bcast_i[4];
    uint64_t rng_state, rng_inc;
};

__device__ __forceinline__ uint32_t pcg_next(Shared& sh) {
    const uint64_t old = sh.rng_state;
    sh.rng_state = old * 6364136223846793005ULL + sh.rng_inc;
    const uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (x >> rot) | (x << ((0u - rot) & 31u));
}

__device__ __forceinline__ double pcg_doub(Shared& sh) {
    const uint64_t bits = ((uint64_t)pcg_next(sh) << 20) | 0x3ff0000000000000ULL;
    return __longlong_as_double((long long)bits) - 1.0;
}

__device__ __forceinline__ void pcg_seed(Shared& sh, uint64_t s) {
    sh.rng_state = 0U;
    sh.rng_inc = (1ull << 1u) | 1u;
    pcg_next(sh);
    sh.rng_state += s;
    pcg_next(sh);
}

__device__ __forceinline__ uint32_t ins0(uint32_t p, uint32_t b) {
    return ((p >> b) << (b + 1u)) | (p & ((1u << b) - 1u));
}

// index p of the subspace with bit q = 0 and (if c >= 0) bit c = 1
__device__ __forceinline__ uint32_t pair_idx(uint32_t p, int q, int c) {
    if (c < 0) return ins0(p, (uint32_t)q);
    const uint32_t lo = q < c ? (uint32_t)q : (uint32_t)c, hi = q < c ? (uint32_t)c : (uint32_t)q;
    return ins0(ins0(p, lo), hi) | (1u << c);
}

// Shared-memory layout: element i lives at i + i/32 (one pad word per 32), which
// makes the strided group loads of the fused Trotter sweeps bank-conflict free.
__device__ __forceinline__ uint32_t pad(uint32_t i) { return i + (i >> 5); }

// A chain's state.  Chains wider than one CTA's shared memory run on a cluster
// of 2^k CTAs: the k most significant qubits (the acceptance qubit and the top
// energy qubits) are distributed, CTA rank r holding the slice whose top bits
// equal r.  Gates on local qubits never leave the CTA; a distributed qubit used
// as a control is a per-CTA predicate; only H/X/W on a distributed qubit and the
// measurement reductions exchange data through distributed shared memory.
// Rank 0 owns the chain's random stream and broadcasts every decision, so all
// ranks follow the same control flow.
template <typename T, bool CL>
struct Ctx {
    T* re;
    T* im;
    int n, k, nl;      // total, distributed, local qubits
    uint32_t Nl;       // local amplitudes
    uint32_t rank;
    Shared* sh;

    __device__ void sync() const { __syncthreads(); }
    __device__ void csync() const {
        if (CL) cg::this_cluster().sync(); else __syncthreads();
    }
    __device__ bool dist(int q) const { return q >= nl; }
    __device__ uint32_t rbit(int q) const { return (rank >> (q - nl)) & 1u; }
    __device__ T* peer_re(uint32_t r) const { return cg::this_cluster().map_shared_rank(re, r); }
    __device__ T* peer_im(uint32_t r) const { return cg::this_cluster().map_shared_rank(im, r); }
    __device__ Shared* peer_sh(uint32_t r) const { return cg::this_cluster().map_shared_rank(sh, r); }

    __device__ void init() {
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            re[pad(i)] = (T)0;
            im[pad(i)] = (T)0;
        }
        sync();
        if (threadIdx.x == 0 && rank == 0) re[pad(0)] = (T)1;
        csync();
    }

    // 2x2 update of a pair across the cluster: this CTA holds the element with
    // bit value `mine` of the distributed qubit q, the partner CTA the other.
    // op: 0 = X (swap), 1 = H
    __device__ void cross_pair(int q, int op) {
        const uint32_t partner = rank ^ (1u << (q - nl));
        const uint32_t mine = rbit(q);
        T* pre = peer_re(partner);
        T* pim = peer_im(partner);
        csync();  // partner's previous writes are visible
        const T kh = (T)0.7071067811865475;
        // read phase into registers (at most Nl/blockDim elements per thread)
        for (uint32_t base = 0; base < Nl; base += blockDim.x * 8u) {
            T nr[8], ni[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t i = base + threadIdx.x + u * blockDim.x;
                if (i < Nl) {
                    const T ar = re[pad(i)], ai = im[pad(i)], br = pre[pad(i)], bi = pim[pad(i)];
                    if (op == 0) {
                        nr[u] = br;
                        ni[u] = bi;
                    } else if (mine == 0) {
                        nr[u] = kh * (ar + br);
                        ni[u] = kh * (ai + bi);
                    } else {
                        nr[u] = kh * (br - ar);
                        ni[u] = kh * (bi - ai);
                    }
                }
            }
            csync();  // everyone has read before anyone writes
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t i = base + threadIdx.x + u * blockDim.x;
                if (i < Nl) {
                    re[pad(i)] = nr[u];
                    im[pad(i)] = ni[u];
                }
            }
            csync();
        }
    }

    // Hadamard on q (uncontrolled)
    __device__ void h(int q) {
        if (CL && dist(q)) { cross_pair(q, 1); return; }
        const T kk = (T)0.7071067811865475;
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i0 = ins0(p, (uint32_t)q), i1 = i0 | (1u << q);
            const T a0r = re[pad(i0)], a0i = im[pad(i0)], a1r = re[pad(i1)], a1i = im[pad(i1)];
            re[pad(i0)] = kk * (a0r + a1r);
            im[pad(i0)] = kk * (a0i + a1i);
            re[pad(i1)] = kk * (a0r - a1r);
            im[pad(i1)] = kk * (a0i - a1i);
        }
        sync();
    }

    __device__ void x(int q) {
        if (CL && dist(q)) { cross_pair(q, 0); return; }
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i0 = ins0(p, (uint32_t)q), i1 = i0 | (1u << q);
            const T r = re[pad(i0)], i = im[pad(i0)];
            re[pad(i0)] = re[pad(i1)];
            im[pad(i0)] = im[pad(i1)];
            re[pad(i1)] = r;
            im[pad(i1)] = i;
        }
        sync();
    }

    // RY(theta) on a local qubit: a0' = c a0 - s a1, a1' = s a0 + c a1 (c, s of theta/2)
    __device__ void ry(int q, T cs, T sn) {
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i0 = ins0(p, (uint32_t)q), i1 = i0 | (1u << q);
            const T a0r = re[pad(i0)], a0i = im[pad(i0)], a1r = re[pad(i1)], a1i = im[pad(i1)];
            re[pad(i0)] = cs * a0r - sn * a1r;
            im[pad(i0)] = cs * a0i - sn * a1i;
            re[pad(i1)] = sn * a0r + cs * a1r;
            im[pad(i1)] = sn * a0i + cs * a1i;
        }
        sync();
    }

    // phase (cs + i sn) on the elements with bit q == val (U1 with q_mask = val)
    __device__ void u1(int q, int val, T cs, T sn) {
        if (CL && dist(q)) {
            if (rbit(q) == (uint32_t)val) {
                for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
                    const T a = re[pad(i)];
                    re[pad(i)] = a * cs - im[pad(i)] * sn;
                    im[pad(i)] = im[pad(i)] * cs + a * sn;
                }
            }
            sync();
            return;
        }
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i = ins0(p, (uint32_t)q) | ((uint32_t)val << q);
            const T a = re[pad(i)];
            re[pad(i)] = a * cs - im[pad(i)] * sn;
            im[pad(i)] = im[pad(i)] * cs + a * sn;
        }
        sync();
    }

    // controlled phase: both bits set
    __device__ void cu1(int qc, int qt, T cs, T sn) {
        int fixed[2];
        int nf = 0;
        bool skip = false;
        for (int q : {qc, qt}) {
            if (CL && dist(q)) {
                if (!rbit(q)) skip = true;
            } else {
                fixed[nf++] = q;
            }
        }
        if (!skip) {
            const uint32_t cnt = Nl >> nf;
            for (uint32_t p = threadIdx.x; p < cnt; p += blockDim.x) {
                uint32_t i = p;
                if (nf == 2) {
                    const int lo = fixed[0] < fixed[1] ? fixed[0] : fixed[1], hi = fixed[0] < fixed[1] ? fixed[1] : fixed[0];
                    i = ins0(ins0(i, lo), hi);
                } else if (nf == 1) {
                    i = ins0(i, fixed[0]);
                }
                for (int f = 0; f < nf; ++f) i |= 1u << fixed[f];
                const T a = re[pad(i)];
                re[pad(i)] = a * cs - im[pad(i)] * sn;
                im[pad(i)] = im[pad(i)] * cs + a * sn;
            }
        }
        sync();
    }

    // One Trotter step on the half with bit c set: the ZZ bond phases (a diagonal
    // indexed by the number of domain walls), then exp(i h d X_i) on every spin.
    // Spins are processed M at a time: a thread loads the 2^M amplitudes that
    // differ only in those spins into registers, applies the M rotations there
    // (they commute) and stores them back, so a step costs ceil(s/4) sweeps.
    template <int M>
    __device__ void trotter_group(int s, int g0, int c, bool with_zz, const T* tc, const T* ts, T xc, T xs) {
        constexpr int G = 1 << M;
        const uint32_t smask = (1u << s) - 1u;
        const bool local_c = !(CL && dist(c));
        if (!local_c && !rbit(c)) { sync(); return; }
        const uint32_t ngroups = local_c ? (Nl >> (M + 1)) : (Nl >> M);
        for (uint32_t gi = threadIdx.x; gi < ngroups; gi += blockDim.x) {
            // insert M zero bits at g0, then the control bit (c > every spin bit)
            uint32_t base = ((gi >> g0) << (g0 + M)) | (gi & ((1u << g0) - 1u));
            if (local_c) base = ins0(base, (uint32_t)c) | (1u << c);
            T ar[G], ai[G];
#pragma unroll
            for (int r = 0; r < G; ++r) {
                const uint32_t i = base | ((uint32_t)r << g0);
                ar[r] = re[pad(i)];
                ai[r] = im[pad(i)];
            }
            if (with_zz) {
#pragma unroll
                for (int r = 0; r < G; ++r) {
                    const uint32_t xsb = (base | ((uint32_t)r << g0)) & smask;
                    const uint32_t rot = ((xsb >> 1) | ((xsb & 1u) << (s - 1))) & smask;
                    const int w = __popc(xsb ^ rot);
                    const T cs = tc[w], sn = ts[w];
                    const T a = ar[r];
                    ar[r] = a * cs - ai[r] * sn;
                    ai[r] = ai[r] * cs + a * sn;
                }
            }
#pragma unroll
            for (int kq = 0; kq < M; ++kq) {
#pragma unroll
                for (int r = 0; r < G; ++r) {
                    if (r & (1 << kq)) continue;
                    const int r1 = r | (1 << kq);
                    const T a0r = ar[r], a0i = ai[r], a1r = ar[r1], a1i = ai[r1];
                    ar[r] = a0r * xc - a1i * xs;
                    ai[r] = a0i * xc + a1r * xs;
                    ar[r1] = a1r * xc - a0i * xs;
                    ai[r1] = a1i * xc + a0r * xs;
                }
            }
#pragma unroll
            for (int r = 0; r < G; ++r) {
                const uint32_t i = base | ((uint32_t)r << g0);
                re[pad(i)] = ar[r];
                im[pad(i)] = ai[r];
            }
        }
        sync();
    }

    __device__ void trotter_step(int s, int c, const T* tc, const T* ts, T xc, T xs) {
        for (int g0 = 0; g0 < s; g0 += 4) {
            const int m = s - g0 < 4 ? s - g0 : 4;
            const bool zz = (g0 == 0);
            switch (m) {
                case 4: trotter_group<4>(s, g0, c, zz, tc, ts, xc, xs); break;
                case 3: trotter_group<3>(s, g0, c, zz, tc, ts, xc, xs); break;
                case 2: trotter_group<2>(s, g0, c, zz, tc, ts, xc, xs); break;
                default: trotter_group<1>(s, g0, c, zz, tc, ts, xc, xs); break;
            }
        }
    }

    // QMS acceptance rotation W on the acceptance qubit (the MSB), factors per
    // energy reading Enew = (j >> shift) & (L-1), j the element with acc = 0
    __device__ void w_oracle(int qacc, int shift, uint32_t L, const double* f1, const double* f2) {
        if (CL && dist(qacc)) {
            const uint32_t accbit = 1u << (qacc - nl);
            const uint32_t partner = rank ^ accbit;
            const bool is_j = (rank & accbit) == 0u;
            const uint32_t jrank = rank & ~accbit;
            T* pre = peer_re(partner);
            T* pim = peer_im(partner);
            csync();
            for (uint32_t base = 0; base < Nl; base += blockDim.x * 8u) {
                T nr[8], ni[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const uint32_t l = base + threadIdx.x + u * blockDim.x;
                    if (l < Nl) {
                        const uint32_t gj = l | (jrank << nl);
                        const uint32_t e = (gj >> shift) & (L - 1u);
                        const T a = (T)f1[e], b = (T)f2[e];
                        const T mr = re[pad(l)], mi = im[pad(l)], pr = pre[pad(l)], pi = pim[pad(l)];
                        if (is_j) {
                            nr[u] = b * mr + a * pr;
                            ni[u] = b * mi + a * pi;
                        } else {
                            nr[u] = a * pr - b * mr;
                            ni[u] = a * pi - b * mi;
                        }
                    }
                }
                csync();
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const uint32_t l = base + threadIdx.x + u * blockDim.x;
                    if (l < Nl) {
                        re[pad(l)] = nr[u];
                        im[pad(l)] = ni[u];
                    }
                }
                csync();
            }
            return;
        }
        const uint32_t half = 1u << qacc;
        for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) {
            const uint32_t i = j | half;
            const uint32_t e = (j >> shift) & (L - 1u);
            const T a = (T)f1[e], b = (T)f2[e];
            const T jr = re[pad(j)], ji = im[pad(j)], ir = re[pad(i)], ii = im[pad(i)];
            re[pad(j)] = b * jr + a * ir;
            im[pad(j)] = b * ji + a * ii;
            re[pad(i)] = a * jr - b * ir;
            im[pad(i)] = a * ji - b * ii;
        }
        sync();
    }

    // projective measurement of q with the draw r: returns c = (r < p1)
    __device__ int measure(int q, double r) {
        double p0 = 0.0, p1 = 0.0;
        const bool dq = CL && dist(q);
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            const double w = (double)re[pad(i)] * (double)re[pad(i)] + (double)im[pad(i)] * (double)im[pad(i)];
            const uint32_t bit = dq ? rbit(q) : ((i >> q) & 1u);
            if (bit) p1 += w; else p0 += w;
        }
        for (int o = 16; o > 0; o >>= 1) {
            p0 += __shfl_down_sync(0xffffffffu, p0, o);
            p1 += __shfl_down_sync(0xffffffffu, p1, o);
        }
        const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0) {
            sh->red[0][wid] = p0;
            sh->red[1][wid] = p1;
        }
        sync();
        if (threadIdx.x == 0) {
            double a = 0.0, b = 0.0;
            for (int kk = 0; kk < (int)(blockDim.x >> 5); ++kk) {
                a += sh->red[0][kk];
                b += sh->red[1][kk];
            }
            sh->bcast_d[2] = a;
            sh->bcast_d[3] = b;
        }
        if (CL) {
            csync();
            if (rank == 0 && threadIdx.x == 0) {
                double a = 0.0, b = 0.0;
                const uint32_t nr = 1u << k;
                for (uint32_t rr = 0; rr < nr; ++rr) {
                    Shared* ps = peer_sh(rr);
                    a += ps->bcast_d[2];
                    b += ps->bcast_d[3];
                }
                const int cc = (int)(r < b);
                const double sc = 1. / sqrt(cc ? b : a);
                for (uint32_t rr = 0; rr < nr; ++rr) {
                    Shared* ps = peer_sh(rr);
                    ps->bcast_i[0] = cc;
                    ps->bcast_d[0] = sc;
                }
            }
            csync();
        } else {
            if (threadIdx.x == 0) {
                const double a = sh->bcast_d[2], b = sh->bcast_d[3];
                const int cc = (int)(r < b);
                sh->bcast_i[0] = cc;
                sh->bcast_d[0] = 1. / sqrt(cc ? b : a);
            }
            sync();
        }
        const int cc = sh->bcast_i[0];
        const T sc = (T)sh->bcast_d[0];
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            const uint32_t bit = dq ? rbit(q) : ((i >> q) & 1u);
            const bool keep = (int)bit == cc;
            re[pad(i)] = (keep ? re[pad(i)] : (T)0) * sc;
            im[pad(i)] = (keep ? im[pad(i)] : (T)0) * sc;
        }
        sync();
        return cc;
    }

    // one draw from the chain's stream (rank 0, thread 0), broadcast to every thread
    __device__ double draw() {
        csync();
        if (threadIdx.x == 0 && rank == 0) {
            const double v = pcg_doub(*sh);
            if (CL) {
                for (uint32_t rr = 0; rr < (1u << k); ++rr) peer_sh(rr)->bcast_d[1] = v;
            } else {
                sh->bcast_d[1] = v;
            }
        }
        csync();
        return sh->bcast_d[1];
    }
};

template <typename T, bool CL>
struct Qms {
    Ctx<T, CL> cx;
    const DevChain* P;
    int s, e, acc;
    uint32_t L;
    uint32_t E_old;
    int gCi;
    uint32_t nphi = 0;

    // exp(-iHt) on the spins, controlled on bit c (a phase-estimation target)
    __device__ void evolution(double t, int c) {
        const double at = fabs(t);
        int steps = (int)ceil(at / P->dt - 1e-9);
        if (steps < 1) steps = 1;
        const double d = t / (double)steps;
        __shared__ T tc[24], ts[24];
        __shared__ T xc, xs;
        if (threadIdx.x <= (unsigned)s) {
            double sn, cs;
            sincos(P->J * d * (double)(s - 2 * (int)threadIdx.x), &sn, &cs);
            tc[threadIdx.x] = (T)cs;
            ts[threadIdx.x] = (T)sn;
        }
        if (threadIdx.x == 32) {
            double sn, cs;
            sincos(P->h * d, &sn, &cs);
            xc = (T)cs;
            xs = (T)sn;
        }
        __syncthreads();
        for (int kk = 0; kk < steps; ++kk) cx.trotter_step(s, c, tc, ts, xc, xs);
    }

    __device__ void u1(int q, double phase) {
        double sn, cs;
        sincos(phase, &sn, &cs);
        cx.u1(q, 1, (T)cs, (T)sn);
    }

    __device__ void cu1(int qc, int qt, double phase) {
        double sn, cs;
        sincos(phase, &sn, &cs);
        cx.cu1(qc, qt, (T)cs, (T)sn);
    }

    // QFT over the energy register (phases 2 pi / 2^m, the reference's table)
    __device__ void qft(bool inverse) {
        if (!inverse) {
            for (int o = e - 1; o >= 0; o--) {
                cx.h(s + o);
                for (int i = o - 1; i >= 0; i--) cu1(s + i, s + o, 2.0 * M_PI / (double)(1u << (1 + (o - i))));
            }
        } else {
            for (int o = 0; o < e; o++) {
                for (int i = 0; i < o; i++) cu1(s + i, s + o, -(2.0 * M_PI / (double)(1u << (1 + (o - i)))));
                cx.h(s + o);
            }
        }
    }

    __device__ void phi() {
        nphi++;
        const double t = P->t_pe;
        for (int kk = 0; kk < e; ++kk) cx.h(s + kk);
        for (int trg = e - 1; trg > -1; --trg) {
            const double powr = (double)(1u << (e - 1 - trg));
            evolution(-powr * t, s + trg);
            u1(s + trg, -powr * t * P->t_shift);
        }
        qft(true);
    }

    __device__ void phi_inverse() {
        nphi++;
        const double t = P->t_pe;
        qft(false);
        for (int trg = 0; trg < e; ++trg) {
            const double powr = (double)(1u << (e - 1 - trg));
            evolution(powr * t, s + trg);
            u1(s + trg, powr * t * P->t_shift);
        }
        for (int kk = 0; kk < e; ++kk) cx.h(s + kk);
    }

    __device__ void w() {
        __shared__ double f1[128], f2[128];
        for (uint32_t en = threadIdx.x; en < L; en += blockDim.x) {
            const double dE = (en * P->c_factor - E_old * P->c_factor);
            if (dE > 0) {
                f1[en] = exp(-dE / 2.0);
                f2[en] = sqrt(1.0 - f1[en] * f1[en]);
            } else {
                f1[en] = 1.0;
                f2[en] = 0.0;
            }
        }
        __syncthreads();
        cx.w_oracle(acc, s, L, f1, f2);
    }

    __device__ void apply_U() {
        cx.h(gCi);
        phi();
        w();
    }

    __device__ void apply_U_inverse() {
        w();
        phi_inverse();
        cx.h(gCi);
    }

    __device__ void reset(int q) {
        const double r = cx.draw();
        if (cx.measure(q, r)) cx.x(q);
    }

    __device__ uint32_t read_energy() {
        double r[8];
        for (int kk = 0; kk < e; ++kk) r[kk] = cx.draw();
        uint32_t v = 0;
        for (int kk = 0; kk < e; ++kk) v += (uint32_t)cx.measure(s + kk, r[kk]) << kk;
        return v;
    }

    __device__ double energy_of(uint32_t v) const { return P->t_shift + v / (double)(P->pe_factor * L); }

    // the system's initial state: |0...0>, or the learned warm start RY(ry_i) per spin
    __device__ void init_state() {
        cx.init();
        if (P->warm) {
            for (int i = 0; i < s; ++i) {
                double sn, cs;
                sincos(0.5 * P->ry[i], &sn, &cs);
                cx.ry(i, (T)cs, (T)sn);
            }
            cx.csync();
        }
    }

    __device__ double measure_magnetisation() {
        double r[24];
        for (int i = 0; i < s; ++i) r[i] = cx.draw();
        double m = 0.0;
        for (int i = 0; i < s; ++i) m += cx.measure(i, r[i]) ? -1.0 : 1.0;
        return m;
    }

    __device__ int draw_C() {
        const double xr = cx.draw();
        for (int i = 0; i < s; ++i) {
            const double wsum = (i + 1 == s) ? 1.0 : (double)(i + 1) / (double)s;
            if (xr < wsum) return i;
        }
        return s;
    }

    // one Metropolis step; returns 1/2 accepted (not/sampled), 3/4 restored, -1 failed
    __device__ int metro_step(bool take, double* Eout, double* Aout, bool* sampled) {
        *sampled = false;
        for (int kk = 0; kk < e; ++kk) reset(s + kk);
        reset(acc);
        phi();
        const uint32_t eo = read_energy();
        E_old = eo;
        for (int kk = 0; kk < e; ++kk)
            if ((eo >> kk) & 1u) cx.x(s + kk);
        gCi = draw_C();
        apply_U();
        const int c_acc = cx.measure(acc, cx.draw());
        if (c_acc == 1) {
            const uint32_t en = read_energy();
            phi_inverse();
            if (!take) return 1;
            *Eout = energy_of(en);
            for (int kk = 0; kk < e; ++kk)
                if ((en >> kk) & 1u) cx.x(s + kk);
            *Aout = measure_magnetisation();
            *sampled = true;
            for (int kk = 0; kk < e; ++kk) reset(s + kk);
            phi();
            read_energy();
            phi_inverse();
            return 2;
        }
        apply_U_inverse();
        int ret = 0;
        int iters = 0;
        while (iters < P->max_reverse) {
            phi();
            const uint32_t en = read_energy();
            phi_inverse();
            if (E_old == en) {
                if (take) {
                    *Eout = energy_of(E_old);
                    for (int kk = 0; kk < e; ++kk) reset(s + kk);
                    *Aout = measure_magnetisation();
                    *sampled = true;
                    for (int kk = 0; kk < e; ++kk) reset(s + kk);
                    phi();
                    read_energy();
                    phi_inverse();
                    ret = 4;
                } else {
                    ret = 3;
                }
                break;
            }
            apply_U();
            cx.measure(acc, cx.draw());
            apply_U_inverse();
            iters++;
        }
        if (iters == P->max_reverse) return -1;
        return ret;
    }
};

// Persistent chain loop.  CL = cluster mode (one chain per cluster of 2^k CTAs).
template <typename T, bool CL>
__global__ void __launch_bounds__(kThreads, 2) k_qms_tfim(const DevChain* __restrict__ chains,
                                                          const int* __restrict__ order, int nchains,
                                                          unsigned int* next, sq_chain_result* res, double* sE,
                                                          double* sA, uint32_t* sStep, int kdist) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ Shared sh;
    __shared__ int cur;
    const uint32_t rank = CL ? cg::this_cluster().block_rank() : 0u;
    for (;;) {
        if (CL) cg::this_cluster().sync(); else __syncthreads();
        if (threadIdx.x == 0 && rank == 0) {
            const int c = (int)atomicAdd(next, 1u);
            if (CL) {
                for (uint32_t rr = 0; rr < (1u << kdist); ++rr) *cg::this_cluster().map_shared_rank(&cur, rr) = c;
            } else {
                cur = c;
            }
        }
        if (CL) cg::this_cluster().sync(); else __syncthreads();
        if (cur >= nchains) return;
        const int ci = order[cur];
        const DevChain& P = chains[ci];
        Qms<T, CL> q;
        q.P = &P;
        q.s = P.s;
        q.e = P.e;
        q.acc = P.s + P.e;
        q.L = 1u << P.e;
        q.cx.n = P.n;
        q.cx.k = CL ? kdist : 0;
        q.cx.nl = P.n - q.cx.k;
        q.cx.Nl = 1u << q.cx.nl;
        q.cx.rank = rank;
        q.cx.sh = &sh;
        q.cx.re = reinterpret_cast<T*>(smem_raw);
        q.cx.im = q.cx.re + (q.cx.Nl + q.cx.Nl / 32 + 1);
        if (threadIdx.x == 0 && rank == 0) pcg_seed(sh, P.seed);
        const long long t_start = clock64();
        q.init_state();
        uint32_t s0 = 0, accepted = 0, failures = 0, ns = 0;
        for (uint32_t st = 0; st < (uint32_t)P.steps; ++st) {
            const bool take = (st > s0 + (uint32_t)P.therm) && ((st - s0) % (uint32_t)P.reset_each == 0u);
            double E = 0.0, A = 0.0;
            bool sampled = false;
            const int ret = q.metro_step(take, &E, &A, &sampled);
            if (threadIdx.x == 0 && rank == 0 && sampled) {
                const size_t o = (size_t)P.out_offset + ns;
                sE[o] = E;
                sA[o] = A;
                sStep[o] = st;
            }
            if (sampled) ns++;
            if (ret < 0) {
                q.init_state();
                s0 = st + 1;
                failures++;
            }
            if (ret == 1 || ret == 2) accepted++;
        }
        if (threadIdx.x == 0 && rank == 0) {
            res[ci].accepted = accepted;
            res[ci].failures = failures;
            res[ci].samples = ns;
            res[ci].phase_estimations = q.nphi;
            res[ci].cycles = (uint64_t)(clock64() - t_start);
        }
    }
}

}  // namespace sqb

namespace {
int fail(int code, const std::string& m) {
    sqi::set_error(m.c_str());
    return code;
}
#define SQB_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(SQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
}  // namespace

extern "C" int sq_qms_tfim_batch(const sq_tfim_chain* chains, uint32_t nchains, int precision, sq_chain_result* results,
                                 double* samples_E, double* samples_A, uint32_t* samples_step, void* stream,
                                 float* kernel_ms) {
    using namespace sqb;
    if (!chains || !results || nchains == 0) return fail(SQ_ERR_ARG, "null or empty chain list");
    if (precision != SQ_F64 && precision != SQ_F32) return fail(SQ_ERR_ARG, "unknown precision");
    std::vector<DevChain> dc(nchains);
    size_t total = 0;
    int nmax = 0;
    for (uint32_t i = 0; i < nchains; ++i) {
        const sq_tfim_chain& c = chains[i];
        if (c.spins < 2 || c.spins > 20 || c.ene_qbits < 1 || c.ene_qbits > 7)
            return fail(SQ_ERR_ARG, "chain sizes out of range (spins 2..20, energy qubits 1..7)");
        if (c.spins + c.ene_qbits + 1 > 22) return fail(SQ_ERR_ARG, "chain wider than 22 qubits");
        if (c.reset_each == 0 || c.max_reverse == 0 || !(c.ene_max > c.ene_min) || !(c.dt > 0))
            return fail(SQ_ERR_ARG, "invalid chain parameters");
        DevChain& d = dc[i];
        d.s = (int)c.spins;
        d.e = (int)c.ene_qbits;
        d.n = d.s + d.e + 1;
        d.steps = (int)c.steps;
        d.therm = (int)c.thermalization;
        d.reset_each = (int)c.reset_each;
        d.max_reverse = (int)c.max_reverse;
        d.J = c.J;
        d.h = c.h;
        d.beta = c.beta;
        d.dt = c.dt;
        const uint32_t L = 1u << c.ene_qbits;
        // the reference driver's derived constants (src/qms.cu:82-84, qms.cuh:96-103)
        d.t_shift = c.ene_min;
        d.pe_factor = (L - 1) / (double)(L * (c.ene_max - c.ene_min));
        d.t_pe = d.pe_factor * 8. * atan(1.0);
        d.c_factor = c.beta / (d.pe_factor * L);
        d.seed = c.seed;
        d.out_offset = (int)total;
        d.warm = c.warm_start ? 1 : 0;
        for (int k = 0; k < 20; ++k) d.ry[k] = c.ry[k];
        total += c.steps;
        if (d.n > nmax) nmax = d.n;
    }
    // chains grouped by width; each class is one persistent launch sized for it
    int dev = 0, nsm = 1, optin = 0;
    SQB_CUDA(cudaGetDevice(&dev));
    SQB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    SQB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t esz = precision == SQ_F64 ? 8 : 4;
    const size_t static_smem = 4096;
    int smem_q = 0;
    auto padded = [](int q) { return (size_t)(((size_t)1 << q) + ((size_t)1 << q) / 32 + 1); };
    while (smem_q < 22 && 2 * padded(smem_q + 1) * esz + static_smem <= (size_t)optin) ++smem_q;

    std::vector<int> order(nchains);
    for (uint32_t i = 0; i < nchains; ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return dc[a].n > dc[b].n; });
    struct Class { int n, first, count; };
    std::vector<Class> classes;
    for (uint32_t k = 0; k < nchains; ++k) {
        const int n = dc[order[k]].n;
        if (classes.empty() || classes.back().n != n) classes.push_back({n, (int)k, 0});
        classes.back().count++;
    }
    cudaStream_t st = (cudaStream_t)stream;
    DevChain* d_ch = nullptr;
    int* d_order = nullptr;
    unsigned int* d_next = nullptr;
    sq_chain_result* d_res = nullptr;
    double *d_E = nullptr, *d_A = nullptr;
    uint32_t* d_step = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_ch); cudaFree(d_order); cudaFree(d_next); cudaFree(d_res);
        cudaFree(d_E); cudaFree(d_A); cudaFree(d_step);
    };
    if (nmax > smem_q + 4) return fail(SQ_ERR_ARG, "chain too wide for a 16-CTA cluster");
    if (cudaMalloc(&d_ch, sizeof(DevChain) * nchains) != cudaSuccess ||
        cudaMalloc(&d_order, sizeof(int) * nchains) != cudaSuccess ||
        cudaMalloc(&d_next, sizeof(unsigned int) * classes.size()) != cudaSuccess ||
        cudaMalloc(&d_res, sizeof(sq_chain_result) * nchains) != cudaSuccess ||
        cudaMalloc(&d_E, sizeof(double) * (total + 1)) != cudaSuccess ||
        cudaMalloc(&d_A, sizeof(double) * (total + 1)) != cudaSuccess ||
        cudaMalloc(&d_step, sizeof(uint32_t) * (total + 1)) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return fail(SQ_ERR_NOMEM, "device allocation for the chain batch failed");
    }
    cudaMemcpyAsync(d_ch, dc.data(), sizeof(DevChain) * nchains, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_order, order.data(), sizeof(int) * nchains, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_next, 0, sizeof(unsigned int) * classes.size(), st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    cudaError_t err = cudaSuccess;
    for (size_t ci = 0; ci < classes.size() && err == cudaSuccess; ++ci) {
        const Class& c = classes[ci];
        const int kd = c.n > smem_q ? c.n - smem_q : 0;  // distributed qubits
        const int nl = c.n - kd;
        const int csize = 1 << kd;
        const size_t smem = 2 * padded(nl) * esz;
        int per_sm = (int)((size_t)(228 * 1024) / (smem + static_smem + 1024));
        per_sm = std::max(1, std::min(per_sm, 8));
        int groups = std::max(1, (nsm * per_sm) / csize);
        groups = std::min(groups, c.count);
        const unsigned grid = (unsigned)(groups * csize);
        const int* ord = d_order + c.first;
        unsigned int* nxt = d_next + ci;
        if (kd == 0) {
            if (precision == SQ_F64) {
                cudaFuncSetAttribute(k_qms_tfim<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                k_qms_tfim<double, false><<<grid, kThreads, smem, st>>>(d_ch, ord, c.count, nxt, d_res, d_E, d_A, d_step, 0);
            } else {
                cudaFuncSetAttribute(k_qms_tfim<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                k_qms_tfim<float, false><<<grid, kThreads, smem, st>>>(d_ch, ord, c.count, nxt, d_res, d_E, d_A, d_step, 0);
            }
        } else {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(grid, 1, 1);
            cfg.blockDim = dim3(kThreads, 1, 1);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)csize;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            if (precision == SQ_F64) {
                auto kf = k_qms_tfim<double, true>;
                cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (csize > 8) cudaFuncSetAttribute(kf, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
                err = cudaLaunchKernelEx(&cfg, kf, (const DevChain*)d_ch, ord, c.count, nxt, d_res, d_E, d_A, d_step, kd);
            } else {
                auto kf = k_qms_tfim<float, true>;
                cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (csize > 8) cudaFuncSetAttribute(kf, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
                err = cudaLaunchKernelEx(&cfg, kf, (const DevChain*)d_ch, ord, c.count, nxt, d_res, d_E, d_A, d_step, kd);
            }
        }
        if (err == cudaSuccess) err = cudaGetLastError();
    }
    cudaEventRecord(e1, st);
    if (err == cudaSuccess) {
        cudaMemcpyAsync(results, d_res, sizeof(sq_chain_result) * nchains, cudaMemcpyDeviceToHost, st);
        if (samples_E) cudaMemcpyAsync(samples_E, d_E, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
        if (samples_A) cudaMemcpyAsync(samples_A, d_A, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
        if (samples_step) cudaMemcpyAsync(samples_step, d_step, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost, st);
        err = cudaStreamSynchronize(st);
    }
    float ms = 0.f;
    if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    if (kernel_ms) *kernel_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (err != cudaSuccess) return fail(SQ_ERR_CUDA, std::string("chain batch: ") + cudaGetErrorString(err));
    return SQ_OK;
}
