// Device side of the batched QMS engine (transverse-field Ising rings).
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
// Storage modes of a chain's 2^n amplitudes (re block, then im block):
//   MODE 0  one CTA, the whole state in its shared memory;
//   MODE 1  a thread-block cluster of 2^k CTAs, the k most significant qubits
//           distributed, each CTA's slice in its own shared memory (gates on a
//           distributed qubit exchange through distributed shared memory);
//   MODE 2  a cluster of 2^k CTAs working in place on the chain's state in
//           global memory (kept L2-resident by bounding the number of live
//           chains), for chains wider than 16 CTAs' shared memory.
// Rank 0 of a cluster owns the chain's random stream and broadcasts every
// decision, so all ranks follow the same control flow.
//
// Chains are resumable: a launch advances each chain by at most `quota` steps,
// reading its saved amplitudes, random stream and counters from global memory
// and writing them back at the end, so a run can be split into segments,
// replayed from a captured CUDA graph, checkpointed and resumed.
#pragma once
#include <cmath>
#include <cstdint>

#include <cooperative_groups.h>

namespace sqb {
namespace cg = cooperative_groups;

struct DevChain {
    int s, e, n, steps, therm, reset_each, max_reverse;
    double J, h, beta, dt;
    double t_pe, t_shift, pe_factor, c_factor;  // as the reference driver computes them
    uint64_t seed;
    uint64_t state_off;  // element offset of the chain's saved state (re block then im block)
    int out_offset;      // first sample slot of this chain
    int warm;
    double ry[20];       // warm-start RY angles per spin
};

// Per-chain progress between launches.
struct ChainRec {
    uint64_t rng_state, rng_inc;
    uint64_t cycles, evo_cycles;
    uint32_t step;       // next Metropolis step
    uint32_t s0;         // step of the last (re-)initialisation
    uint32_t accepted, failures, samples, nphi;
    uint32_t started, pad;
};

struct KArgs {
    const DevChain* chains;
    const int* order;     // chain indices of this width class
    int count;
    unsigned int* next;   // work counter of this class
    ChainRec* recs;
    double* sE;
    double* sA;
    uint32_t* sStep;
    void* states;         // saved states (T elements)
    uint32_t quota;       // steps per chain in this launch
    int kdist;            // distributed qubits (MODE 1, 2)
    uint32_t stage_elems; // MODE 2: elements of dynamic shared memory for the Trotter exchange
};

// Longer rings than this keep their top spin bits across a warp group
// (evolve_regs); the staging area of mode 2 then needs kStageR elements per
// thread for re and for im.
constexpr int kChunkSpins = 9;
constexpr int kStageR = 1 << (kChunkSpins - 5);

struct Shared {
    double red[2][32];
    double bcast_d[4];
    int bcast_i[4];
    uint64_t rng_state, rng_inc;
};

// Per-chain coefficients, computed once when a chain starts (FP64 transcendentals
// on the device, one entry per thread), indexed by direction (0: the forward
// phase estimation, 1: its inverse) and energy qubit / QFT distance.
template <typename T>
struct Tables {
    T tz[2][8][24], sz[2][8][24];  // ZZ phase by domain-wall count (cos(hd)^s folded in on the register path)
    T tn[2][8], xc[2][8], xs[2][8];  // tan(hd), cos(hd), sin(hd) of the X rotations
    int steps[2][8], regs[2][8];   // Trotter steps of the controlled power; register path usable
    T rtc[128], rts[128];          // e^{i 2 pi k / 2^e}
    T u1v_c[2][128], u1v_s[2][128];  // all phase-estimation shifts as one phase per register value
    T dc[128], ds[128];            // the diagonal of the current fused QFT step
    double hist[256];              // register histogram (measurements)
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

// kernel entry of a storage mode for element type T; defined in
// sq_batch_{f32,f64}_m{0,1,2}.cu
template <typename T, int MODE>
const void* kernel_for();

template <typename T>
__device__ __forceinline__ T shfl_x(T v, int m) {
    return __shfl_xor_sync(0xffffffffu, v, m);
}

template <typename T, int MODE>
struct Ctx {
    static constexpr bool CL = MODE != 0;
    T* re;        // this CTA's slice (MODE 0, 1: shared memory; MODE 2: global)
    T* im;
    T* gre;       // MODE 2: the whole state's re / im blocks
    T* gim;
    T* stage;     // MODE 2: shared-memory staging for the Trotter exchange
    uint32_t stage_elems;
    int n, k, nl;      // total, distributed, local qubits
    uint32_t Nl;       // local amplitudes
    uint32_t rank;
    Shared* sh;

    // Shared-memory slices use the layout i + i/32 (one pad word per 32), which
    // makes the strided group loads of the Trotter sweeps bank-conflict free;
    // global-memory slices are dense.
    __device__ __forceinline__ uint32_t at(uint32_t i) const { return MODE == 2 ? i : i + (i >> 5); }

    __device__ void sync() const { __syncthreads(); }
    __device__ void csync() const {
        if (CL) cg::this_cluster().sync(); else __syncthreads();
    }
    __device__ bool dist(int q) const { return CL && q >= nl; }
    __device__ uint32_t rbit(int q) const { return (rank >> (q - nl)) & 1u; }
    __device__ T* peer_re(uint32_t r) const {
        if (MODE == 2) return gre + (size_t)r * Nl;
        return cg::this_cluster().map_shared_rank(re, r);
    }
    __device__ T* peer_im(uint32_t r) const {
        if (MODE == 2) return gim + (size_t)r * Nl;
        return cg::this_cluster().map_shared_rank(im, r);
    }
    __device__ Shared* peer_sh(uint32_t r) const { return cg::this_cluster().map_shared_rank(sh, r); }

    __device__ void init() {
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            re[at(i)] = (T)0;
            im[at(i)] = (T)0;
        }
        sync();
        if (threadIdx.x == 0 && rank == 0) re[at(0)] = (T)1;
        csync();
    }

    // saved state <-> working slice (MODE 0, 1; MODE 2 works in place)
    __device__ void load(const T* sre, const T* sim) {
        if (MODE == 2) return;
        const size_t o = (size_t)rank * Nl;
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            re[at(i)] = sre[o + i];
            im[at(i)] = sim[o + i];
        }
        csync();
    }
    __device__ void save(T* sre, T* sim) {
        if (MODE == 2) { csync(); return; }
        const size_t o = (size_t)rank * Nl;
        sync();
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            sre[o + i] = re[at(i)];
            sim[o + i] = im[at(i)];
        }
        csync();
    }

    // 2x2 update of a pair across the cluster: this CTA holds the element with
    // bit value `mine` of the distributed qubit q, the partner CTA the other.
    // op: 0 = X (swap), 1 = H
    __device__ __noinline__ void cross_pair(int q, int op) {
        const uint32_t partner = rank ^ (1u << (q - nl));
        const uint32_t mine = rbit(q);
        T* pre = peer_re(partner);
        T* pim = peer_im(partner);
        csync();  // partner's previous writes are visible
        const T kh = (T)0.7071067811865475;
        for (uint32_t base = 0; base < Nl; base += blockDim.x * 8u) {
            T nr[8], ni[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t i = base + threadIdx.x + u * blockDim.x;
                if (i < Nl) {
                    const T ar = re[at(i)], ai = im[at(i)], br = pre[at(i)], bi = pim[at(i)];
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
                    re[at(i)] = nr[u];
                    im[at(i)] = ni[u];
                }
            }
            csync();
        }
    }

    // Hadamard on q (uncontrolled)
    __device__ __noinline__ void h(int q) {
        if (dist(q)) { cross_pair(q, 1); return; }
        const T kk = (T)0.7071067811865475;
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i0 = ins0(p, (uint32_t)q), i1 = i0 | (1u << q);
            const T a0r = re[at(i0)], a0i = im[at(i0)], a1r = re[at(i1)], a1i = im[at(i1)];
            re[at(i0)] = kk * (a0r + a1r);
            im[at(i0)] = kk * (a0i + a1i);
            re[at(i1)] = kk * (a0r - a1r);
            im[at(i1)] = kk * (a0i - a1i);
        }
        sync();
    }

    // RY(theta) on a local qubit: a0' = c a0 - s a1, a1' = s a0 + c a1 (c, s of theta/2)
    __device__ __noinline__ void ry(int q, T cs, T sn) {
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i0 = ins0(p, (uint32_t)q), i1 = i0 | (1u << q);
            const T a0r = re[at(i0)], a0i = im[at(i0)], a1r = re[at(i1)], a1i = im[at(i1)];
            re[at(i0)] = cs * a0r - sn * a1r;
            im[at(i0)] = cs * a0i - sn * a1i;
            re[at(i1)] = sn * a0r + cs * a1r;
            im[at(i1)] = sn * a0i + cs * a1i;
        }
        sync();
    }

    // One Trotter step on the half with bit c set, through shared memory: the ZZ
    // bond phases (a diagonal indexed by the number of domain walls), then
    // exp(i h d X_i) on every spin, M spins per sweep held in registers.  Used
    // for rings too long for the register-resident evolution below.
    template <int M>
    __device__ void trotter_group(int s, int g0, int c, bool with_zz, const T* tc, const T* ts, T xc, T xs) {
        constexpr int G = 1 << M;
        const uint32_t smask = (1u << s) - 1u;
        // c < 0: uncontrolled (the whole slice)
        const bool local_c = c >= 0 && !dist(c);
        if (c >= 0 && !local_c && !rbit(c)) { sync(); return; }
        const uint32_t ngroups = local_c ? (Nl >> (M + 1)) : (Nl >> M);
        for (uint32_t gi = threadIdx.x; gi < ngroups; gi += blockDim.x) {
            uint32_t base = ((gi >> g0) << (g0 + M)) | (gi & ((1u << g0) - 1u));
            if (local_c) base = ins0(base, (uint32_t)c) | (1u << c);
            T ar[G], ai[G];
#pragma unroll
            for (int r = 0; r < G; ++r) {
                const uint32_t i = base | ((uint32_t)r << g0);
                ar[r] = re[at(i)];
                ai[r] = im[at(i)];
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
                re[at(i)] = ar[r];
                im[at(i)] = ai[r];
            }
        }
        sync();
    }

    __device__ __noinline__ void trotter_step_smem(int s, int c, const T* tc, const T* ts, T xc, T xs) {
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

    // Register-resident evolution: `steps` Trotter steps on the half with bit c
    // set.  The controlled half is cut into chunks of 32*R consecutive indices
    // (of the index space with bit c removed); a warp loads a chunk once (lane =
    // index bits 0-4, register r = bits 5..m-1), applies every Trotter step
    // there and stores it once.  Spin bits 0-4 rotate across lanes by shuffles,
    // spin bits 5..m-1 across registers, and spin bits m..s-1 (rings longer than
    // the chunk) across the G = 2^(s-m) warps of a group that hold the chunks
    // differing in those bits, through shared memory (the chunks' own slots of
    // the state, or a staging area when the state is in global memory) between
    // named barriers.  The X rotation is applied as cos(hd) (a + i tan(hd) b),
    // with cos(hd)^s folded into the ZZ phase table (tz, sz), so a spin costs
    // two FMAs per amplitude.
    template <int R, bool XG>
    __device__ __noinline__ void evolve_regs(int s, int c, int steps, int G, const T* tz, const T* sz, T tn) {
        // c < 0: uncontrolled (the whole slice)
        const bool local_c = c >= 0 && !dist(c);
        if (c >= 0 && !local_c && !rbit(c)) { sync(); return; }
        constexpr int LR = R == 1 ? 0 : R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : R == 16 ? 4 : 5;
        constexpr int m = 5 + LR;
        const int lg = s > m ? s - m : 0;  // log2 G
        const uint32_t nbits = local_c ? (uint32_t)nl - 1u : (uint32_t)nl;
        const uint32_t ngroups = 1u << (nbits - m - lg);
        const uint32_t smask = (1u << s) - 1u;
        const int lane = threadIdx.x & 31;
        const uint32_t w = threadIdx.x >> 5;
        const uint32_t g = w & (uint32_t)(G - 1), gid = w / (uint32_t)G;
        const uint32_t gstep = (blockDim.x >> 5) / (uint32_t)G;
        const uint32_t stride = (local_c && c < 5) ? 64u : 32u;
        const uint32_t astep = MODE == 2 ? stride : stride + (stride >> 5);
        // exchange slots (G > 1): MODE 0/1 the state's own slots, MODE 2 the staging area
        T* xre = MODE == 2 ? stage : re;
        T* xim = MODE == 2 ? stage + (blockDim.x >> 5) * (uint32_t)R * 32u : im;
        for (uint32_t cg_ = gid; cg_ < ngroups; cg_ += gstep) {
            const uint32_t ch = (cg_ << lg) | g;
            T ar[R], ai[R];
            // domain-wall counts (<= 15) of the R amplitudes, 4 bits each
            constexpr int NW = (R + 7) / 8;
            uint32_t wz[NW];
#pragma unroll
            for (int u = 0; u < NW; ++u) wz[u] = 0u;
            // element r of the chunk sits at a0 + r * astep: bit c is either below
            // the lane bits' top (c < 5) or above the chunk (c >= m)
            const uint32_t xl0 = (ch << m) | (uint32_t)lane;
            const uint32_t i0 = local_c ? (ins0(xl0, (uint32_t)c) | (1u << c)) : xl0;
            const uint32_t a0 = at(i0);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const uint32_t xl = xl0 | ((uint32_t)r << 5);
                ar[r] = re[a0 + r * astep];
                ai[r] = im[a0 + r * astep];
                const uint32_t xsb = xl & smask;
                const uint32_t rot = ((xsb >> 1) | ((xsb & 1u) << (s - 1))) & smask;
                wz[r >> 3] |= (uint32_t)__popc(xsb ^ rot) << (4 * (r & 7));
            }
            // my exchange slot base and step
            const uint32_t xa0 = MODE == 2 ? w * (uint32_t)R * 32u + (uint32_t)lane : a0;
            const uint32_t xas = MODE == 2 ? 32u : astep;
            for (int st = 0; st < steps; ++st) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t wv = (wz[r >> 3] >> (4 * (r & 7))) & 15u;
                    const T cs = tz[wv], sn = sz[wv];
                    const T a = ar[r];
                    ar[r] = a * cs - ai[r] * sn;
                    ai[r] = ai[r] * cs + a * sn;
                }
                const int sl = s < 5 ? s : 5;
                for (int b = 0; b < sl; ++b) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const T pr = shfl_x(ar[r], 1 << b), pi = shfl_x(ai[r], 1 << b);
                        ar[r] = fma(-tn, pi, ar[r]);
                        ai[r] = fma(tn, pr, ai[r]);
                    }
                }
#pragma unroll
                for (int kb = 0; kb < LR; ++kb) {
                    if (5 + kb >= s) break;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        if (r & (1 << kb)) continue;
                        const int r1 = r | (1 << kb);
                        const T a0r = ar[r], a0i = ai[r], a1r = ar[r1], a1i = ai[r1];
                        ar[r] = fma(-tn, a1i, a0r);
                        ai[r] = fma(tn, a1r, a0i);
                        ar[r1] = fma(-tn, a0i, a1r);
                        ai[r1] = fma(tn, a0r, a1i);
                    }
                }
                for (int j = 0; XG && j < lg; ++j) {
                    // partner chunk differs in spin bit m + j
                    uint32_t pa0;
                    if (MODE == 2) {
                        pa0 = (w ^ (1u << j)) * (uint32_t)R * 32u + (uint32_t)lane;
                    } else {
                        const uint32_t pxl = xl0 ^ (1u << (m + j));
                        pa0 = at(local_c ? (ins0(pxl, (uint32_t)c) | (1u << c)) : pxl);
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        xre[xa0 + r * xas] = ar[r];
                        xim[xa0 + r * xas] = ai[r];
                    }
                    asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(32 * G) : "memory");
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const T pr = xre[pa0 + r * xas], pi = xim[pa0 + r * xas];
                        ar[r] = fma(-tn, pi, ar[r]);
                        ai[r] = fma(tn, pr, ai[r]);
                    }
                    asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(32 * G) : "memory");
                }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
                re[a0 + r * astep] = ar[r];
                im[a0 + r * astep] = ai[r];
            }
        }
        sync();
    }

    // value of the k-qubit register starting at q0 for local element i (the
    // distributed top qubits come from the CTA's rank)
    __device__ __forceinline__ uint32_t regval(uint32_t i, int q0, int k) const {
        const uint32_t g = CL ? (i | (rank << nl)) : i;
        return (g >> q0) & ((1u << k) - 1u);
    }

    // Hadamards on the local qubits q0..q0+CNT-1 in one sweep (groups of 2^CNT
    // amplitudes in registers), each the reference's H: sum and difference
    // times 0.7071067811865475
    template <int CNT>
    __device__ __noinline__ void h_group(int q0) {
        constexpr int G = 1 << CNT;
        const T kk = (T)0.7071067811865475;
        const uint32_t ng = Nl >> CNT;
        for (uint32_t gi = threadIdx.x; gi < ng; gi += blockDim.x) {
            const uint32_t base = ((gi >> q0) << (q0 + CNT)) | (gi & ((1u << q0) - 1u));
            T ar[G], ai[G];
#pragma unroll
            for (int r = 0; r < G; ++r) {
                ar[r] = re[at(base | ((uint32_t)r << q0))];
                ai[r] = im[at(base | ((uint32_t)r << q0))];
            }
#pragma unroll
            for (int b = 0; b < CNT; ++b) {
#pragma unroll
                for (int r = 0; r < G; ++r) {
                    if (r & (1 << b)) continue;
                    const int r1 = r | (1 << b);
                    const T xr = ar[r], xi = ai[r], yr = ar[r1], yi = ai[r1];
                    ar[r] = kk * (xr + yr);
                    ai[r] = kk * (xi + yi);
                    ar[r1] = kk * (xr - yr);
                    ai[r1] = kk * (xi - yi);
                }
            }
#pragma unroll
            for (int r = 0; r < G; ++r) {
                re[at(base | ((uint32_t)r << q0))] = ar[r];
                im[at(base | ((uint32_t)r << q0))] = ai[r];
            }
        }
        sync();
    }

    // H on every qubit of q0..q0+k-1: local ones up to four per sweep, distributed
    // ones through the cluster
    __device__ void h_layer(int q0, int k) {
        int q = q0;
        const int qe = q0 + k;
        while (q < qe && !dist(q)) {
            int cnt = qe - q;
            int room = nl - q;
            if (cnt > room) cnt = room;
            if (cnt > 4) cnt = 4;
            switch (cnt) {
                case 4: h_group<4>(q); break;
                case 3: h_group<3>(q); break;
                case 2: h_group<2>(q); break;
                default: h_group<1>(q); break;
            }
            q += cnt;
        }
        for (; q < qe; ++q) cross_pair(q, 1);
    }

    // element phase (dc, ds)[v], v the value of the e-qubit register at q0
    __device__ __noinline__ void diag(int q0, int e, const T* dcr, const T* dsr) {
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            const uint32_t v = regval(i, q0, e);
            const T cs = dcr[v], sn = dsr[v];
            const T a = re[at(i)];
            re[at(i)] = a * cs - im[at(i)] * sn;
            im[at(i)] = im[at(i)] * cs + a * sn;
        }
        sync();
    }

    // the diagonal and H on the local qubit q in one sweep (DIAG_FIRST: diagonal
    // then H, else H then diagonal)
    template <bool DIAG_FIRST>
    __device__ __noinline__ void diag_h_local(int q, int q0, int e, const T* dcr, const T* dsr) {
        const T kk = (T)0.7071067811865475;
        for (uint32_t p = threadIdx.x; p < Nl / 2; p += blockDim.x) {
            const uint32_t i0 = ins0(p, (uint32_t)q), i1 = i0 | (1u << q);
            T a0r = re[at(i0)], a0i = im[at(i0)], a1r = re[at(i1)], a1i = im[at(i1)];
            const uint32_t v0 = regval(i0, q0, e), v1 = regval(i1, q0, e);
            if (DIAG_FIRST) {
                T c = dcr[v0], sn = dsr[v0], t = a0r;
                a0r = t * c - a0i * sn;
                a0i = a0i * c + t * sn;
                c = dcr[v1], sn = dsr[v1], t = a1r;
                a1r = t * c - a1i * sn;
                a1i = a1i * c + t * sn;
            }
            T b0r = kk * (a0r + a1r), b0i = kk * (a0i + a1i), b1r = kk * (a0r - a1r), b1i = kk * (a0i - a1i);
            if (!DIAG_FIRST) {
                T c = dcr[v0], sn = dsr[v0], t = b0r;
                b0r = t * c - b0i * sn;
                b0i = b0i * c + t * sn;
                c = dcr[v1], sn = dsr[v1], t = b1r;
                b1r = t * c - b1i * sn;
                b1i = b1i * c + t * sn;
            }
            re[at(i0)] = b0r;
            im[at(i0)] = b0i;
            re[at(i1)] = b1r;
            im[at(i1)] = b1i;
        }
        sync();
    }

    __device__ void diag_h(bool diag_first, int q, int q0, int e, const T* dcr, const T* dsr) {
        if (!dist(q)) {
            if (diag_first) diag_h_local<true>(q, q0, e, dcr, dsr);
            else diag_h_local<false>(q, q0, e, dcr, dsr);
            return;
        }
        if (diag_first) {
            diag(q0, e, dcr, dsr);
            cross_pair(q, 1);
        } else {
            cross_pair(q, 1);
            diag(q0, e, dcr, dsr);
        }
    }

    // X on the register qubits set in c: element i takes the value of i ^ (c << q0).
    // The local qubits swap pairs inside the CTA; the distributed ones then swap
    // whole slices with the partner CTA at equal local indices (so the batched
    // exchange below never reads an element the partner has already rewritten).
    __device__ __noinline__ void xor_register(int q0, int k, uint32_t c) {
        if (c == 0u) return;
        const uint32_t full = c << q0;
        const uint32_t mloc = full & (Nl - 1u);
        const uint32_t rx = CL ? (full >> nl) : 0u;
        if (mloc != 0u) {
            for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
                const uint32_t j = i ^ mloc;
                if (j > i) {
                    const T r = re[at(i)], m = im[at(i)];
                    re[at(i)] = re[at(j)];
                    im[at(i)] = im[at(j)];
                    re[at(j)] = r;
                    im[at(j)] = m;
                }
            }
            sync();
        }
        if (rx == 0u) return;
        const uint32_t partner = rank ^ rx;
        T* pre = peer_re(partner);
        T* pim = peer_im(partner);
        csync();
        for (uint32_t base = 0; base < Nl; base += blockDim.x * 8u) {
            T nr[8], ni[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t i = base + threadIdx.x + u * blockDim.x;
                if (i < Nl) {
                    nr[u] = pre[at(i)];
                    ni[u] = pim[at(i)];
                }
            }
            csync();
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t i = base + threadIdx.x + u * blockDim.x;
                if (i < Nl) {
                    re[at(i)] = nr[u];
                    im[at(i)] = ni[u];
                }
            }
            csync();
        }
    }

    // Measures the k-qubit register at q0 (k <= 8) qubit by qubit, lowest first,
    // with k fresh draws of the chain's stream, exactly as k successive
    // measure_qbit calls of the reference (each outcome c_j = r_j < p1 given the
    // earlier outcomes), but with one histogram pass and one collapse pass:
    // the histogram P[v] (FP64, each warp summing whole bins in a fixed order)
    // gives every conditional p1; the collapse keeps the elements of the outcome
    // v = c scaled by 1/sqrt(P[c]), and with `flip` also applies X to every qubit
    // read as 1 (moves them to v = 0), as the reference's apply_reset.
    __device__ __noinline__ uint32_t measure_register(int q0, int k, bool flip, double* hist) {
        const uint32_t nb = 1u << k;
        // register qubits held locally, and the rank bits of the distributed ones
        int kl = nl - q0;
        if (kl > k) kl = k;
        if (kl < 0) kl = 0;
        const uint32_t nbl = 1u << kl;
        const uint32_t vhi = (CL && kl < k) ? ((rank >> (q0 + kl - nl)) & ((1u << (k - kl)) - 1u)) : 0u;
        const int lane = threadIdx.x & 31;
        const uint32_t nw = blockDim.x >> 5;
        // local bins: warp w sums bins w, w + nw, ...; bin vl holds the elements
        // (low q0 bits) | vl << q0 | (high bits) << (q0 + kl)
        const uint32_t per = Nl >> kl;
        for (uint32_t vl = threadIdx.x >> 5; vl < nbl; vl += nw) {
            double acc = 0.0;
            for (uint32_t j = lane; j < per; j += 32) {
                const uint32_t i = (j & ((1u << q0) - 1u)) | (vl << q0) | ((j >> q0) << (q0 + kl));
                acc += (double)re[at(i)] * (double)re[at(i)] + (double)im[at(i)] * (double)im[at(i)];
            }
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) hist[vl] = acc;
        }
        csync();
        if (threadIdx.x == 0 && rank == 0) {
            double P[256];
            for (uint32_t v = 0; v < nb; ++v) P[v] = 0.0;
            const uint32_t nr = CL ? (1u << this->k) : 1u;
            for (uint32_t rr = 0; rr < nr; ++rr) {
                const double* hr = CL ? cg::this_cluster().map_shared_rank(hist, rr) : hist;
                const uint32_t vh = (CL && kl < k) ? ((rr >> (q0 + kl - nl)) & ((1u << (k - kl)) - 1u)) : 0u;
                for (uint32_t vl = 0; vl < nbl; ++vl) P[vl | (vh << kl)] += hr[vl];
            }
            // sequential decisions with the reference's draws and comparisons
            uint32_t c = 0;
            for (int j = 0; j < k; ++j) {
                const double r = pcg_doub(*sh);
                // candidates: the values agreeing with the outcomes so far
                double s0 = 0.0, s1 = 0.0;
                for (uint32_t t = 0; t < (nb >> j); t += 2) {
                    s0 += P[c | (t << j)];
                    s1 += P[c | ((t + 1) << j)];
                }
                const double p1 = s1 / (s0 + s1);
                if (r < p1) c |= 1u << j;
            }
            const double sc = 1. / sqrt(P[c]);
            for (uint32_t rr = 0; rr < nr; ++rr) {
                Shared* ps = CL ? peer_sh(rr) : sh;
                ps->bcast_i[1] = (int)c;
                ps->bcast_d[0] = sc;
            }
        }
        csync();
        const uint32_t c = (uint32_t)sh->bcast_i[1];
        const T sc = (T)sh->bcast_d[0];
        const uint32_t chi = c >> kl, clo = c & (nbl - 1u);
        if (!flip) {
            const bool mine = chi == vhi;
            for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
                const bool keep = mine && ((i >> q0) & (nbl - 1u)) == clo;
                re[at(i)] = (keep ? re[at(i)] : (T)0) * sc;
                im[at(i)] = (keep ? im[at(i)] : (T)0) * sc;
            }
            sync();
            return c;
        }
        // reset: the outcome's elements move to register value 0, all else is zero.
        // Targets are this CTA's elements with local register bits 0 when its
        // distributed register bits are 0; the source CTA is rank ^ (chi << ...).
        if (vhi == 0u) {
            const uint32_t src = CL && kl < k ? (rank ^ (chi << (q0 + kl - nl))) : rank;
            const T* sre = (src == rank) ? re : peer_re(src);
            const T* sim = (src == rank) ? im : peer_im(src);
            for (uint32_t gi = threadIdx.x; gi < per; gi += blockDim.x) {
                const uint32_t b = (gi & ((1u << q0) - 1u)) | ((gi >> q0) << (q0 + kl));
                const uint32_t isrc = b | (clo << q0);
                const T vr = sre[at(isrc)] * sc, vi = sim[at(isrc)] * sc;
                for (uint32_t vl = 1; vl < nbl; ++vl) {
                    re[at(b | (vl << q0))] = (T)0;
                    im[at(b | (vl << q0))] = (T)0;
                }
                re[at(b)] = vr;
                im[at(b)] = vi;
            }
        }
        csync();
        if (vhi != 0u) {
            for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
                re[at(i)] = (T)0;
                im[at(i)] = (T)0;
            }
        }
        csync();
        return c;
    }

    // QMS acceptance rotation W on the acceptance qubit (the MSB), factors per
    // energy reading Enew = (j >> shift) & (L-1), j the element with acc = 0
    __device__ __noinline__ void w_oracle(int qacc, int shift, uint32_t L, const double* f1, const double* f2) {
        if (dist(qacc)) {
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
                        const T mr = re[at(l)], mi = im[at(l)], pr = pre[at(l)], pi = pim[at(l)];
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
                        re[at(l)] = nr[u];
                        im[at(l)] = ni[u];
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
            const T jr = re[at(j)], ji = im[at(j)], ir = re[at(i)], ii = im[at(i)];
            re[at(j)] = b * jr + a * ir;
            im[at(j)] = b * ji + a * ii;
            re[at(i)] = a * jr - b * ir;
            im[at(i)] = a * ji - b * ii;
        }
        sync();
    }

    // projective measurement of q with the draw r: returns c = (r < p1)
    __device__ __noinline__ int measure(int q, double r) {
        double p0 = 0.0, p1 = 0.0;
        const bool dq = dist(q);
        for (uint32_t i = threadIdx.x; i < Nl; i += blockDim.x) {
            const double w = (double)re[at(i)] * (double)re[at(i)] + (double)im[at(i)] * (double)im[at(i)];
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
            re[at(i)] = (keep ? re[at(i)] : (T)0) * sc;
            im[at(i)] = (keep ? im[at(i)] : (T)0) * sc;
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

template <typename T, int MODE>
struct Qms {
    Ctx<T, MODE> cx;
    const DevChain* P;
    int s, e, acc;
    uint32_t L;
    uint32_t E_old;
    int gCi;
    uint32_t nphi = 0;

    Tables<T>* tb;
    uint64_t evo_cycles = 0;  // thread 0 of rank 0 only

    // chunk geometry of the register path for control qubit c
    __device__ bool chunking(int c, int* m_out, int* G_out) const {
        const int nbits = cx.dist(c) ? cx.nl : cx.nl - 1;
        const int nw = (int)(blockDim.x >> 5);
        int m = 0, G = 1;
        if (s <= kChunkSpins) {
            // at least 5 (a warp), up to 8 for register-level parallelism while
            // leaving a chunk per warp; when c is local and >= 5 the chunk stays
            // below it, so a chunk's elements are equally spaced
            const int lw = nw >= 16 ? 4 : nw >= 8 ? 3 : 2;
            m = nbits - lw;
            if (m > 8) m = 8;
            if (!cx.dist(c) && c >= 5 && m > c) m = c;
            if (m < 5) m = 5;
            if (m < s) m = s;
            if (m > nbits) m = nbits;
        } else {
            // longer rings: chunks of kChunkSpins spin bits, the rest across a warp group
            m = kChunkSpins;
            G = 1 << (s - kChunkSpins);
        }
        *m_out = m;
        *G_out = G;
        // the exchange needs equally spaced chunk elements (modes 0, 1) or a
        // staging area large enough for every warp's chunk (mode 2)
        const bool xok = G == 1 || (MODE == 2 ? cx.stage_elems >= 2u * blockDim.x * (uint32_t)kStageR
                                              : (cx.dist(c) || c >= m));
        return nbits >= 5 && nbits >= s && m >= 5 && G <= 8 && G <= nw && xok;
    }

    // the coefficient tables of this chain (exp(-iHt) = Trotter steps of width
    // d = t / ceil(|t|/dt); t = -+2^(e-1-trg) t_pe for the forward / inverse
    // phase estimation, as the reference's apply_phase_estimation[_inverse])
    __device__ void fill_tables() {
        const int ne = 2 * e * (s + 1);
        for (int idx = threadIdx.x; idx < ne; idx += blockDim.x) {
            const int w = idx % (s + 1);
            const int trg = (idx / (s + 1)) % e;
            const int dir = idx / ((s + 1) * e);
            const double powr = (double)(1u << (e - 1 - trg));
            const double t = dir == 0 ? -powr * P->t_pe : powr * P->t_pe;
            int steps = (int)ceil(fabs(t) / P->dt - 1e-9);
            if (steps < 1) steps = 1;
            const double d = t / (double)steps;
            const double hd = P->h * d;
            int m, G;
            const bool regs = chunking(s + trg, &m, &G) && fabs(hd) < 0.78;  // |h d| < pi/4: tan well conditioned
            double shd, chd;
            sincos(hd, &shd, &chd);
            const double ch = regs ? pow(chd, (double)s) : 1.0;
            double sn, cs;
            sincos(P->J * d * (double)(s - 2 * w), &sn, &cs);
            tb->tz[dir][trg][w] = (T)(cs * ch);
            tb->sz[dir][trg][w] = (T)(sn * ch);
            if (w == 0) {
                tb->tn[dir][trg] = (T)(shd / chd);
                tb->xc[dir][trg] = (T)chd;
                tb->xs[dir][trg] = (T)shd;
                tb->steps[dir][trg] = steps;
                tb->regs[dir][trg] = regs ? 1 : 0;
            }
        }
        const int L = 1 << e;
        for (int idx = threadIdx.x; idx < 3 * L; idx += blockDim.x) {
            const int v = idx % L, which = idx / L;
            double ang;
            if (which == 0) {
                ang = 2.0 * M_PI * (double)v / (double)L;
            } else {
                // all phase-estimation shifts U1(-+2^(e-1-trg) t_pe E_min) on the
                // energy qubits set in v, as one phase
                ang = 0.0;
                for (int trg = 0; trg < e; ++trg)
                    if ((v >> trg) & 1) ang += (double)(1u << (e - 1 - trg)) * P->t_pe * P->t_shift;
                if (which == 1) ang = -ang;
            }
            double sa, ca;
            sincos(ang, &sa, &ca);
            if (which == 0) {
                tb->rtc[v] = (T)ca;
                tb->rts[v] = (T)sa;
            } else {
                tb->u1v_c[which - 1][v] = (T)ca;
                tb->u1v_s[which - 1][v] = (T)sa;
            }
        }
        __syncthreads();
    }

    // exp(-iHt) on the spins for energy qubit trg (controlled on it)
    __device__ void evolution(int dir, int trg) {
        const long long t0 = clock64();
        evolution_(dir, trg);
        if (threadIdx.x == 0) evo_cycles += (uint64_t)(clock64() - t0);
    }

    __device__ void evolution_(int dir, int trg) {
        const int c = s + trg;
        const T* tz = tb->tz[dir][trg];
        const T* sz = tb->sz[dir][trg];
        const int steps = tb->steps[dir][trg];
        if (!tb->regs[dir][trg]) {
            const T xc = tb->xc[dir][trg], xs = tb->xs[dir][trg];
            for (int kk = 0; kk < steps; ++kk) cx.trotter_step_smem(s, c, tz, sz, xc, xs);
            return;
        }
        int m, G;
        chunking(c, &m, &G);
        const T tn = tb->tn[dir][trg];
        switch (m) {
            case 5: cx.template evolve_regs<1, false>(s, c, steps, G, tz, sz, tn); break;
            case 6: cx.template evolve_regs<2, false>(s, c, steps, G, tz, sz, tn); break;
            case 7: cx.template evolve_regs<4, false>(s, c, steps, G, tz, sz, tn); break;
            case 8: cx.template evolve_regs<8, false>(s, c, steps, G, tz, sz, tn); break;
            default:
                if (G > 1) cx.template evolve_regs<16, true>(s, c, steps, G, tz, sz, tn);
                else cx.template evolve_regs<16, false>(s, c, steps, G, tz, sz, tn);
                break;
        }
    }

    // One fused step of a QFT over the energy register: the controlled phases
    // onto qubit o (reference: cu1(s+i, s+o, -+2 pi / 2^(1+o-i)) for i < o, whose
    // product is the phase -+2 pi v_low / 2^(o+1) on elements with bit o set,
    // v_low the lower register bits) as one diagonal, optionally times the
    // phase-estimation shifts (dir's U1 table), fused with H on qubit o.
    __device__ void qft_step(int o, bool inverse, int u1dir) {
        const int L = 1 << e;
        for (int v = threadIdx.x; v < L; v += blockDim.x) {
            T c = (T)1, sn = (T)0;
            if ((v >> o) & 1) {
                const int kx = (v & ((1 << o) - 1)) << (e - o - 1);
                c = tb->rtc[kx];
                sn = inverse ? -tb->rts[kx] : tb->rts[kx];
            }
            if (u1dir >= 0) {
                const T uc = tb->u1v_c[u1dir][v], us = tb->u1v_s[u1dir][v];
                const T t = c;
                c = t * uc - sn * us;
                sn = sn * uc + t * us;
            }
            tb->dc[v] = c;
            tb->ds[v] = sn;
        }
        __syncthreads();
        // inverse QFT: phases then H(o); forward: H(o) then phases
        cx.diag_h(inverse, s + o, s, e, tb->dc, tb->ds);
    }

    // the reference's apply_phase_estimation: H on the energy register, the
    // controlled powers of exp(-iHt) with their U1(-2^k t E_min) shifts (the
    // shifts are diagonal and commute with the evolutions, so they join the
    // first QFT step), then the inverse QFT
    __device__ void phi() {
        nphi++;
        cx.h_layer(s, e);
        for (int trg = e - 1; trg > -1; --trg) evolution(0, trg);
        for (int o = 0; o < e; o++) qft_step(o, true, o == 0 ? 0 : -1);
    }

    // apply_phase_estimation_inverse: the QFT (its last step also carries the
    // U1 shifts), the evolutions, H on the energy register
    __device__ void phi_inverse() {
        nphi++;
        for (int o = e - 1; o >= 0; o--) qft_step(o, false, o == 0 ? 1 : -1);
        for (int trg = 0; trg < e; ++trg) evolution(1, trg);
        cx.h_layer(s, e);
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

    // measure_qbits on the energy register with e fresh draws
    __device__ uint32_t read_energy() { return cx.measure_register(s, e, false, tb->hist); }
    // apply_reset on the energy register (and the acceptance qubit above it)
    __device__ void reset_energy(bool with_acc) { cx.measure_register(s, with_acc ? e + 1 : e, true, tb->hist); }

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
        double mg = 0.0;
        for (int i = 0; i < s; ++i) mg += cx.measure(i, r[i]) ? -1.0 : 1.0;
        return mg;
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
        reset_energy(true);
        phi();
        const uint32_t eo = read_energy();
        E_old = eo;
        cx.xor_register(s, e, eo);
        gCi = draw_C();
        apply_U();
        const int c_acc = cx.measure(acc, cx.draw());
        if (c_acc == 1) {
            const uint32_t en = read_energy();
            phi_inverse();
            if (!take) return 1;
            *Eout = energy_of(en);
            cx.xor_register(s, e, en);
            *Aout = measure_magnetisation();
            *sampled = true;
            reset_energy(false);
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
                    reset_energy(false);
                    *Aout = measure_magnetisation();
                    *sampled = true;
                    reset_energy(false);
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

// Persistent chain loop of one width class: CTAs (or clusters) pull chains from
// the class's work counter and advance each by at most a.quota steps.
// CTA size is chosen at launch (128-512 threads for FP32, 128-256 for FP64; the
// FP64 bound leaves room for 32 register-resident complex doubles per thread).
template <typename T, int MODE>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 256 : 512, 1) k_qms_tfim(const KArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ Shared sh;
    __shared__ Tables<T> tbl;
    __shared__ int cur;
    constexpr bool CL = MODE != 0;
    const uint32_t rank = CL ? cg::this_cluster().block_rank() : 0u;
    const uint32_t csz = CL ? (1u << a.kdist) : 1u;
    for (;;) {
        if (CL) cg::this_cluster().sync(); else __syncthreads();
        if (threadIdx.x == 0 && rank == 0) {
            const int c = (int)atomicAdd(a.next, 1u);
            if (CL) {
                for (uint32_t rr = 0; rr < csz; ++rr) *cg::this_cluster().map_shared_rank(&cur, rr) = c;
            } else {
                cur = c;
            }
        }
        if (CL) cg::this_cluster().sync(); else __syncthreads();
        if (cur >= a.count) return;
        const int ci = a.order[cur];
        const DevChain& P = a.chains[ci];
        ChainRec& R = a.recs[ci];
        const uint32_t first = R.step;
        if (first >= (uint32_t)P.steps) continue;  // uniform across the cluster
        uint32_t last = first + a.quota;
        if (last > (uint32_t)P.steps) last = (uint32_t)P.steps;
        Qms<T, MODE> q;
        q.P = &P;
        q.s = P.s;
        q.e = P.e;
        q.acc = P.s + P.e;
        q.L = 1u << P.e;
        q.cx.n = P.n;
        q.cx.k = CL ? a.kdist : 0;
        q.cx.nl = P.n - q.cx.k;
        q.cx.Nl = 1u << q.cx.nl;
        q.cx.rank = rank;
        q.cx.sh = &sh;
        T* sre = reinterpret_cast<T*>(a.states) + P.state_off;
        T* sim = sre + ((size_t)1 << P.n);
        q.cx.gre = sre;
        q.cx.gim = sim;
        q.cx.stage = reinterpret_cast<T*>(smem_raw);
        q.cx.stage_elems = a.stage_elems;
        q.tb = &tbl;
        q.fill_tables();
        if (MODE == 2) {
            q.cx.re = sre + (size_t)rank * q.cx.Nl;
            q.cx.im = sim + (size_t)rank * q.cx.Nl;
        } else {
            q.cx.re = reinterpret_cast<T*>(smem_raw);
            q.cx.im = q.cx.re + (q.cx.Nl + q.cx.Nl / 32 + 1);
        }
        const long long t_start = clock64();
        uint32_t s0, accepted, failures, ns;
        if (!R.started) {
            if (threadIdx.x == 0 && rank == 0) pcg_seed(sh, P.seed);
            q.init_state();
            s0 = 0;
            accepted = failures = ns = 0;
        } else {
            if (threadIdx.x == 0 && rank == 0) {
                sh.rng_state = R.rng_state;
                sh.rng_inc = R.rng_inc;
            }
            q.cx.load(sre, sim);
            s0 = R.s0;
            accepted = R.accepted;
            failures = R.failures;
            ns = R.samples;
            q.nphi = R.nphi;
        }
        for (uint32_t st = first; st < last; ++st) {
            const bool take = (st > s0 + (uint32_t)P.therm) && ((st - s0) % (uint32_t)P.reset_each == 0u);
            double E = 0.0, A = 0.0;
            bool sampled = false;
            const int ret = q.metro_step(take, &E, &A, &sampled);
            if (threadIdx.x == 0 && rank == 0 && sampled) {
                const size_t o = (size_t)P.out_offset + ns;
                a.sE[o] = E;
                a.sA[o] = A;
                a.sStep[o] = st;
            }
            if (sampled) ns++;
            if (ret < 0) {
                q.init_state();
                s0 = st + 1;
                failures++;
            }
            if (ret == 1 || ret == 2) accepted++;
        }
        q.cx.save(sre, sim);
        if (threadIdx.x == 0 && rank == 0) {
            R.rng_state = sh.rng_state;
            R.rng_inc = sh.rng_inc;
            R.step = last;
            R.s0 = s0;
            R.accepted = accepted;
            R.failures = failures;
            R.samples = ns;
            R.nphi = q.nphi;
            R.started = 1;
            R.cycles += (uint64_t)(clock64() - t_start);
            R.evo_cycles += q.evo_cycles;
        }
    }
}

}  // namespace sqb
