// Tile-pass kernel of the state-vector engine (sm_103a).
//
// One pass = one read and one write of (part of) the state.  The state index
// space is split into tiles of 2^K amplitudes: the tile holds the L lowest
// qubits (contiguous in memory, so loads are 16-byte vectors in runs of 2^L
// elements) plus K-L "high" qubits chosen by the host planner so that every
// non-diagonal qubit of every gate in the pass lies inside the tile.  A CTA
// stages a tile's re and im blocks in shared memory, applies the pass's gate
// list (each gate is one sweep of the tile with a barrier in between), folds in
// an optional reduction (measurement probabilities or a filtered norm) and
// writes the tile back.  Gates whose controls sit on qubits outside the tile
// are resolved per tile: a tile whose fixed bits fail a gate's controls skips
// that gate, and a tile that no gate touches is neither loaded nor stored.
//
// Element formulas restate the reference kernels (include/suqa_kernels.cuh and
// include/suqa_cpu.hpp of SUQA); each case names its source below.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "sq_df64.cuh"

namespace sqk {

constexpr int kMaxOps = 48;   // gates per launch (kernel parameters, ~6.4 KB)
constexpr int kMaxTab = 128;  // complex table entries per launch (W factors, phase lists)
constexpr int kMaxHigh = 16;  // tile qubits above the contiguous low block

enum OpKind : uint8_t {
    OP_SWAPP = 0,     // a0 <-> a1 over pairs (X, CX, MCX, SWAP)
    OP_YP = 1,        // Y: a0' = -i a1, a1' = i a0
    OP_HP = 2,        // Hadamard with the literal 0.7071067811865475
    OP_PAULI = 3,     // exp(i theta P) (pair form, or diagonal when no X/Y)
    OP_PHASE = 4,     // a *= c + i s on (g & cmask) == cval  (U1, CU1, MCU1)
    OP_PLIST = 5,     // a *= tab[(g >> shift) & zy] where (g & cmask) != 0
    OP_W = 6,         // QMS acceptance rotation, (f1, f2) = tab[(g0 & zy) >> shift]
    OP_COLLAPSE = 7,  // keep (g & cmask) == cval scaled by s, zero the rest
    OP_SCALE = 8,     // a *= s everywhere
    OP_DENSE = 9      // 32 x 32 complex matrix on the five tile bits of lflip (sq_dense.cuh)
};

// Optional parts of a pass-kernel instantiation (the template argument F of k_pass)
enum PassFeat : int {
    PF_BULK = 1,   // bulk asynchronous tile staging
    PF_DENSE = 2,  // OP_DENSE blocks
    PF_TC = 4      // OP_DENSE blocks on the tensor cores (with PF_DENSE)
};

// One gate in tile-local form (144 bytes).  For pair operations the pairs are
// (t0, t0 ^ lflip) with t0 the tile index whose bit lpair is clear.  Control
// conditions are split into the tile-local part (lcm, lcv: bits of the tile
// index, tested per element) and the outer part (ocm, ocv: tested once per tile).
struct Op {
    uint8_t kind;
    uint8_t lpair;   // tile-local bit that orders the pair
    uint8_t ny;      // Pauli: number of Y factors
    uint8_t fz;      // Pauli: parity of (flip & zy)
    uint8_t cbig;    // deferred rotation: |c| >= |s| (the factor c is deferred, else s)
    uint8_t orient;  // H / Y: the pass's index frame swaps the pair's logical roles
    uint8_t xpar;    // Pauli: parity the index frame adds to every element's sign
    uint8_t pad8;
    uint32_t lflip;  // tile-local flip mask
    uint32_t lcm, lcv;     // tile-local control condition
    uint32_t lzy;          // tile-local Y|Z mask (Pauli signs)
    uint32_t shift, tab;   // PLIST/W: shift and table offset (in complex entries)
    uint32_t gdefer;       // H / rotation whose scale factor the host keeps in the state's global scale
    uint64_t cmask, cval;  // global element condition (diagonal slow paths)
    uint64_t ocm, ocv;     // part of the condition on qubits outside the tile
    uint64_t zy;           // Pauli: global Y|Z mask; PLIST/W: extraction mask
    double c, s, sn;       // sn = -s
    double u, un;          // deferred rotation: u = s/c (cbig) or c/s, un = -u
    float fc, fs, fsn, fu, fun, fpad;  // the same in FP32 for the FP32 kernel
    df64 dc, ds, dsn, du, dun;         // the same as double-float pairs for the df64 kernel
};

struct Prog {
    int nops;
    int red;             // 0 none, 1 measurement split by rmask, 2 filter (g & rmask) == rval
    int defer;           // 1: uniform H / rotations defer their scale factor
    int ndense;          // OP_DENSE ops in the list
    uint64_t rmask, rval;
    uint32_t lrm, lrv;   // tile-local part of rmask / rval
    uint64_t orm, orv;   // part outside the tile
    uint32_t xm;         // index frame at the end of the pass: uncontrolled X gates on tile
                         // qubits move no data; physical element t holds logical t ^ xm
    int rswap;           // the frame flips the measured qubit: swap the two sums
    Op ops[kMaxOps];
    double tab[2 * kMaxTab];
};

struct PassArgs {
    void* re;
    void* im;
    uint64_t ofree;   // outer qubits enumerated by the tile index
    uint64_t ofix;    // value of the fixed outer qubits
    uint64_t ntiles;
    double* partials; // 2 per CTA
    double* result;   // 2 doubles
    unsigned int* ticket;
    unsigned int* err;  // error word (bulk staging only): set when a bounded wait gives up
    int K, L;
    int store;        // 0 for a reduction-only pass
    int stage;        // 1: tiles move by bulk asynchronous copies (runs of 2^L elements), 0: through registers
    uint8_t hb[kMaxHigh];  // global positions of the tile qubits >= L
    const void* dense;     // OP_DENSE data of this launch (op.tab selects a 32 KiB block)
    int dense_tc;          // 1: dense ops on the tensor cores (FP32, tiles >= 2^12), 0: CUDA cores
    uint32_t dense_off;    // byte offset of the dense work area in dynamic shared memory
    int df_in, df_out;     // double-float kernel: the state holds hi/lo FP32 pairs before / after the pass
    // mapped page-locked host copy of result (4 doubles, or null): the last CTA of a
    // reduction also writes (p0, p1) and the error word there, so the host reads them
    // after a stream synchronisation without a copy that could queue on the copy
    // engines behind other streams' bulk transfers
    double* result_host;
};

// ---- bulk asynchronous copies (the TMA engine's cp.async.bulk) and mbarriers
constexpr unsigned int kErrStageWait = 1u;   // a tile load did not complete in time
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0u;
}
// Waits for the phase with the given parity to complete, for at most kWaitLimitNs;
// false (and the error word set) when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned int* err,
                                                  unsigned int code) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > kWaitLimitNs) {
            if (err) atomicOr(err, code);
            return false;
        }
    }
    return true;
}
// global -> shared, completion counted in bytes on the mbarrier
__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(sdst)),
        "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// shared -> global, tracked by this thread's bulk groups
__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(ssrc)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// orders this thread's generic-proxy shared-memory accesses with later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <typename T> struct VecT;
template <> struct VecT<double> { typedef double2 type; static constexpr int W = 2; };
template <> struct VecT<float>  { typedef float4  type; static constexpr int W = 4; };
template <> struct VecT<df64>   { typedef double2 type; static constexpr int W = 2; };  // stored as doubles

template <typename T> constexpr bool kIsDf = std::is_same<T, df64>::value;

// a * b + c in the kernel's element type, with the precision spelled out: a
// float fused multiply-add stays on the FP32 pipe
template <typename T> __device__ __forceinline__ T tfma(T a, T b, T c) {
    if constexpr (kIsDf<T>) return df_fmadd(a, b, c);
    else if constexpr (sizeof(T) == 4) return __fmaf_rn(a, b, c);
    else return __fma_rn(a, b, c);
}

// a double as the kernel's element type (the df64 split uses integer operations)
template <typename T> __device__ __forceinline__ T tconv(double d) {
    if constexpr (kIsDf<T>) return df_from_double(d);
    else return (T)d;
}
template <typename T> __device__ __forceinline__ T tzero() {
    if constexpr (kIsDf<T>) return df64{0.0f, 0.0f};
    else return (T)0;
}

__device__ __forceinline__ uint32_t insert_zero(uint32_t p, uint32_t b) {
    const uint32_t lo = p & ((1u << b) - 1u);
    return ((p >> b) << (b + 1u)) | lo;
}

// p with a zero bit inserted at every set bit of m (ascending): enumerates the
// indices whose bits in m are zero, so a loop runs only over the elements a
// controlled or diagonal gate touches (every lane busy)
__device__ __forceinline__ uint32_t deposit_zeros(uint32_t p, uint32_t m) {
    while (m) {
        const uint32_t b = (uint32_t)(__ffs(m) - 1);
        p = insert_zero(p, b);
        m &= m - 1u;
    }
    return p;
}

__device__ __forceinline__ int parity64(uint64_t x) { return __popcll(x) & 1; }

// out = c*a + s*(i^k * b), the reference's rotate2 form (a*c -/+ x*s).  The
// data-dependent sign of i^k is a select between +s and -s (computed once per
// gate), which keeps it off the FP64 pipe.
template <typename T>
__device__ __forceinline__ void rot_k(T ar, T ai, T br, T bi, int k, T c, T sp, T sn, T& outr, T& outi) {
    const T xr = (k & 1) ? bi : br;
    const T xi = (k & 1) ? br : bi;
    const T fr = (k == 1 || k == 2) ? sn : sp;
    const T fi = (k >= 2) ? sn : sp;
    outr = ar * c + xr * fr;
    outi = ai * c + xi * fi;
}

// x with its sign flipped when f (an integer operation, off the floating-point pipes)
__device__ __forceinline__ double neg_if(double x, bool f) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)f << 63));
}
__device__ __forceinline__ float neg_if(float x, bool f) {
    return __uint_as_float(__float_as_uint(x) ^ ((unsigned)f << 31));
}
__device__ __forceinline__ df64 neg_if(df64 x, bool f) { return df_neg_if(x, f); }

// Deferred-scale rotation: with cbig, out = a + u*(i^k b) (u = s/c, the factor c
// deferred); otherwise out = u*a + i^k b (u = c/s, the factor s deferred).
// up = +u, un = -u.  One fused multiply-add per component either way.
template <typename T>
__device__ __forceinline__ void rot_deferred(T ar, T ai, T br, T bi, int k, T up, T un, bool cbig, T& outr,
                                             T& outi) {
    const T xr = (k & 1) ? bi : br;
    const T xi = (k & 1) ? br : bi;
    const bool nr = (k == 1 || k == 2), ni = (k >= 2);
    if (cbig) {
        outr = tfma<T>(xr, nr ? un : up, ar);
        outi = tfma<T>(xi, ni ? un : up, ai);
    } else {
        outr = tfma<T>(ar, up, neg_if(xr, nr));
        outi = tfma<T>(ai, up, neg_if(xi, ni));
    }
}

// part + |a|^2 (FP64 accumulation; FP32 amplitudes square in FP32)
__device__ __forceinline__ double add_sq(double part, double r, double i) { return __fma_rn(r, r, __fma_rn(i, i, part)); }
__device__ __forceinline__ double add_sq(double part, float r, float i) { return part + (double)fmaf(r, r, i * i); }
__device__ __forceinline__ double add_sq(double part, df64 r, df64 i) { return part + df_to_double(df_fmadd(r, r, i * i)); }

__device__ __forceinline__ void scale_vec(double2& v, double s) { v.x *= s; v.y *= s; }

// element e of the vector becomes element e ^ x (x < vector width)
__device__ __forceinline__ void permute_vec(double2& v, uint32_t x) {
    if (x & 1u) {
        const double t = v.x;
        v.x = v.y;
        v.y = t;
    }
}
__device__ __forceinline__ void permute_vec(float4& v, uint32_t x) {
    if (x & 1u) {
        float t = v.x; v.x = v.y; v.y = t;
        t = v.z; v.z = v.w; v.w = t;
    }
    if (x & 2u) {
        float t = v.x; v.x = v.z; v.z = t;
        t = v.y; v.y = v.w; v.w = t;
    }
}
__device__ __forceinline__ void scale_vec(float4& v, float s) { v.x *= s; v.y *= s; v.z *= s; v.w *= s; }

template <typename T>
__device__ __forceinline__ void block_reduce2(double& a, double& b, double (*sh)[33]) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sh[0][w] = a; sh[1][w] = b; }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (w == 0) {
        a = l < nw ? sh[0][l] : 0.0;
        b = l < nw ? sh[1][l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
    }
    __syncthreads();
}

}  // namespace sqk

#include "sq_dense.cuh"

namespace sqk {

// T = double (FP64 state), float (FP32 state), or df64 (FP64 state, arithmetic in
// double-float on the FP32 pipe; multi-tile passes only).  MAXT = 256 for
// multi-tile passes (three CTAs per SM), 1024 for single-tile passes.
//
// F: the optional parts compiled into this instantiation (PassFeat).  Each costs
// registers and instructions on every pass that carries it, used or not (the
// 28-qubit FP32 benchmark step ran 7 % slower with both in the one kernel), so
// the host picks the leanest instantiation that a pass needs:
//   PF_BULK   tiles staged by bulk asynchronous copies (multi-tile, not df64);
//   PF_DENSE  OP_DENSE blocks (on the CUDA cores through a scratch tile);
//   PF_TC     with PF_DENSE, FP32 blocks on the tensor cores.  A kernel that
//             contains tcgen05.alloc is given one resident CTA per SM by the
//             occupancy calculation, so only passes holding such blocks use it,
//             and its multi-tile form runs 512 threads (MAXT = 512) to keep twice
//             the warps on the SM.
template <typename T, int MAXT = 1024, int F = 0>
__global__ void __launch_bounds__(MAXT, MAXT == 256 ? 3 : 1) k_pass(const __grid_constant__ PassArgs a,
                                                                   const __grid_constant__ Prog p) {
    static_assert(!(F & PF_BULK) || (MAXT <= 512 && !kIsDf<T>), "bulk staging: multi-tile, not double-float");
    static_assert(!(F & PF_DENSE) || !kIsDf<T>, "double-float passes hold no dense blocks");
    static_assert(!(F & PF_TC) || ((F & PF_DENSE) && sizeof(T) == 4), "tensor-core blocks: FP32 dense passes");
    constexpr bool kBulk = (F & PF_BULK) != 0;
    constexpr bool kDense = (F & PF_DENSE) != 0;
    constexpr bool kTC = (F & PF_TC) != 0;
    typedef typename VecT<T>::type V;
    constexpr int W = VecT<T>::W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red_sh[2][33];
    __shared__ int last_flag;

    const int K = a.K, L = a.L;
    const uint32_t TS = 1u << K;
    const uint32_t lowmask = (1u << L) - 1u;
    // one tile buffer (re block then im block), or two when the next tile is
    // prefetched (staging mode 2); the run offsets follow the buffers
    const int nbuf = (kBulk && a.stage == 2) ? 2 : 1;
    T* tiles = reinterpret_cast<T*>(smem_raw);
    T* sre = tiles;
    T* sim = sre + TS;
    uint64_t* offs = reinterpret_cast<uint64_t*>(tiles + (size_t)nbuf * 2 * TS);
    const uint32_t nh = 1u << (K - L);
    for (uint32_t h = threadIdx.x; h < nh; h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < K - L; ++j)
            if ((h >> j) & 1u) o |= 1ull << a.hb[j];
        offs[h] = o;
    }
    // bulk staging: warp 0 issues one asynchronous copy per run of 2^L elements
    // (re and im) against an mbarrier, and writes tiles back the same way; the
    // host enables it only when a run is a multiple of 16 bytes
    // (only instantiations with PF_BULK; never single-tile passes)
    const bool bulk = kBulk && a.stage != 0;
    const uint32_t run_bytes = (1u << L) * (uint32_t)sizeof(T);
    __shared__ __align__(8) uint64_t stage_bar[2];
    uint32_t stage_phase = 0u;  // bit b: parity of the next completion of stage_bar[b]
    uint32_t stage_pend = 0u;   // bit b: a load into buffer b is in flight
    // dense ops: mbarriers, and on the tensor-core path a 64-column TMEM accumulator
    // held by warp 0 for the whole launch
    __shared__ __align__(16) DenseSmem dsm;
    const bool dense_tc = kTC && p.ndense > 0 && a.dense_tc != 0;
    uint32_t ph_b = 0u, ph_mma = 0u;
    int b_loaded = -1;
    unsigned char* dbuf = smem_raw + a.dense_off;
    if (threadIdx.x == 0) {
        if (bulk) {
            mbar_init(&stage_bar[0], 1u);
            mbar_init(&stage_bar[1], 1u);
        }
        if (dense_tc) {
            mbar_init(&dsm.bar_b, 1u);
            mbar_init(&dsm.bar_mma, 1u);
        }
        if (bulk || dense_tc) asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (dense_tc && threadIdx.x < 32) tmem_alloc(&dsm.tmem, kDenseTmemCols);
    if (dense_tc) tc_fence_before();
    __syncthreads();
    if (dense_tc) tc_fence_after();

    T* gre = reinterpret_cast<T*>(a.re);
    T* gim = reinterpret_cast<T*>(a.im);
    double acc0 = 0.0, acc1 = 0.0;

    // tile index -> global index of its element 0, and whether any op of the
    // pass touches it (uniform over the CTA)
    auto tile_base = [&](uint64_t tile) {
        uint64_t b = a.ofix, f = a.ofree, t = tile;
        while (f) {
            const uint64_t low = f & (~f + 1ull);
            if (t & 1ull) b |= low;
            t >>= 1;
            f ^= low;
        }
        return b;
    };
    auto tile_active = [&](uint64_t b) {
        // a frame permutes every tile; a pass that changes the storage format converts every tile
        bool any = p.red != 0 || p.xm != 0u || a.df_in != a.df_out;
        for (int k = 0; k < p.nops && !any; ++k) any = (b & p.ops[k].ocm) == p.ops[k].ocv;
        return any;
    };
    // warp 0 issues the bulk copies of one tile into buffer bi; the buffer's
    // previous bulk stores must have read it first
    auto issue_load = [&](uint64_t b, int bi) {
        if (threadIdx.x < 32) {
            bulk_wait_read_all();
            __syncwarp();
            T* dre = tiles + (size_t)bi * 2 * TS;
            T* dim = dre + TS;
            if (threadIdx.x == 0) mbar_arrive_expect_tx(&stage_bar[bi], 2u * TS * (uint32_t)sizeof(T));
            __syncwarp();
            for (uint32_t h = threadIdx.x; h < nh; h += 32) {
                const uint64_t g = b | offs[h];
                bulk_load(dre + (h << L), gre + g, run_bytes, &stage_bar[bi]);
                bulk_load(dim + (h << L), gim + g, run_bytes, &stage_bar[bi]);
            }
        }
        stage_pend |= 1u << bi;
    };

    uint64_t tile = blockIdx.x, base = 0;
    while (tile < a.ntiles && !tile_active(base = tile_base(tile))) tile += gridDim.x;
    int buf = 0;
    if (bulk && tile < a.ntiles) issue_load(base, 0);
    while (tile < a.ntiles) {
        uint64_t nxt = tile + gridDim.x, nbase = 0;
        while (nxt < a.ntiles && !tile_active(nbase = tile_base(nxt))) nxt += gridDim.x;
        sre = tiles + (size_t)buf * 2 * TS;
        sim = sre + TS;

        // ---- load the tile (16-byte vectors, runs of 2^L contiguous elements)
        if (bulk) {
            if (nbuf == 2 && nxt < a.ntiles) issue_load(nbase, buf ^ 1);  // prefetch the next tile
            const bool ok = mbar_wait_bounded(&stage_bar[buf], (stage_phase >> buf) & 1u, a.err, kErrStageWait);
            if (__syncthreads_or(!ok)) {
                // give every load in flight a second bounded wait, then leave
                for (int bi = 0; bi < 2; ++bi)
                    if ((stage_pend >> bi) & 1u) mbar_wait_bounded(&stage_bar[bi], (stage_phase >> bi) & 1u, nullptr, 0u);
                if (threadIdx.x < 32) {
                    bulk_wait_all();
                    if (dense_tc) tmem_dealloc(dsm.tmem, kDenseTmemCols);
                }
                return;
            }
            stage_phase ^= 1u << buf;
            stage_pend &= ~(1u << buf);
        } else if (kIsDf<T>) {  // doubles in HBM, double-float pairs in the tile
            const double* dre = reinterpret_cast<const double*>(a.re);
            const double* dim = reinterpret_cast<const double*>(a.im);
            for (uint32_t v = threadIdx.x; v < TS / 2; v += blockDim.x) {
                const uint32_t t = v * 2;
                const uint64_t g = base | offs[t >> L] | (t & lowmask);
                if (a.df_in) {  // already hi/lo pairs (an earlier pass of the same flush stored them)
                    *reinterpret_cast<float4*>(sre + t) = __ldcs(reinterpret_cast<const float4*>(dre + g));
                    *reinterpret_cast<float4*>(sim + t) = __ldcs(reinterpret_cast<const float4*>(dim + g));
                    continue;
                }
                const double2 r2 = __ldcs(reinterpret_cast<const double2*>(dre + g));
                const double2 i2 = __ldcs(reinterpret_cast<const double2*>(dim + g));
                const df64 r0 = df_from_double(r2.x), r1 = df_from_double(r2.y);
                const df64 i0 = df_from_double(i2.x), i1 = df_from_double(i2.y);
                *reinterpret_cast<float4*>(sre + t) = make_float4(r0.hi, r0.lo, r1.hi, r1.lo);
                *reinterpret_cast<float4*>(sim + t) = make_float4(i0.hi, i0.lo, i1.hi, i1.lo);
            }
        } else if ((1u << L) >= (uint32_t)W) {
            for (uint32_t v = threadIdx.x; v < TS / W; v += blockDim.x) {
                const uint32_t t = v * W;
                const uint64_t g = base | offs[t >> L] | (t & lowmask);
                *reinterpret_cast<V*>(sre + t) = __ldcs(reinterpret_cast<const V*>(gre + g));
                *reinterpret_cast<V*>(sim + t) = __ldcs(reinterpret_cast<const V*>(gim + g));
            }
        } else {  // states narrower than one vector
            for (uint32_t t = threadIdx.x; t < TS; t += blockDim.x) {
                const uint64_t g = base | offs[t >> L] | (t & lowmask);
                sre[t] = gre[g];
                sim[t] = gim[g];
            }
        }
        __syncthreads();

        // ---- gates.  sigma is a per-tile scale deferred by uniform H and Pauli
        // rotations (gates acting on every element of the tile): H stores
        // (a0+a1, a0-a1) and multiplies sigma by 1/sqrt(2); a rotation
        // c + i s P stores a + (s/c) iP a (or (c/s) a + iP a) and multiplies sigma
        // by c (or s).  Every gate is linear, so sigma commutes with the rest of
        // the pass and is applied once, before the reduction and the store.
        double sigma = 1.0;
        for (int k = 0; k < p.nops; ++k) {
            const Op& op = p.ops[k];
            if ((base & op.ocm) != op.ocv) continue;
            T c, s, sneg, up, un;
            if constexpr (kIsDf<T>) {
                c = op.dc; s = op.ds; sneg = op.dsn; up = op.du; un = op.dun;
            } else if constexpr (sizeof(T) == 8) {
                c = op.c; s = op.s; sneg = op.sn; up = op.u; un = op.un;
            } else {
                c = op.fc; s = op.fs; sneg = op.fsn; up = op.fu; un = op.fun;
            }
            const int kind = op.kind;
            const uint32_t lcm = op.lcm, lcv = op.lcv;
            if (kDense && kind == OP_DENSE) {
                bool ok = true;
                if constexpr (!kDense || kIsDf<T>) {
                    // not reached: the host runs passes with dense blocks in an instantiation with PF_DENSE
                } else if constexpr (kTC) {
                    if (dense_tc)
                        ok = dense_tc_apply(sre, TS, op, reinterpret_cast<const float*>(a.dense), dbuf, dsm, ph_b,
                                            ph_mma, b_loaded, a.err);
                    else
                        dense_cc<T>(sre, TS, op, reinterpret_cast<const double*>(a.dense) + (size_t)op.tab * 4096u,
                                    reinterpret_cast<T*>(dbuf), dsm);
                } else {
                    dense_cc<T>(sre, TS, op, reinterpret_cast<const double*>(a.dense) + (size_t)op.tab * 4096u,
                                reinterpret_cast<T*>(dbuf), dsm);
                }
                if (!ok) {  // a bounded wait gave up: nothing in flight is left behind
                    if (bulk && threadIdx.x < 32) bulk_wait_all();
                    if (dense_tc && threadIdx.x < 32) tmem_dealloc(dsm.tmem, kDenseTmemCols);
                    return;
                }
            } else if (kind <= OP_PAULI && !(kind == OP_PAULI && op.lflip == 0u) || kind == OP_W) {
                const uint32_t lp = op.lpair, lf = op.lflip;
                // pairs (t0, t0 ^ lf) with bit lp of t0 clear and its control bits
                // equal to lcv, enumerated directly (none if lp is a control bit
                // required to be set)
                const uint32_t sel = lcm | (1u << lp);
                const uint32_t npair = ((lcm & lcv) >> lp) & 1u ? 0u : TS >> __popc(sel);
                if (kind == OP_SWAPP) {
                    // include/suqa_cpu.hpp:223-253 (MCX), :268-319 (SWAP)
                    for (uint32_t u = threadIdx.x; u < npair; u += blockDim.x) {
                        const uint32_t t0 = deposit_zeros(u, sel) | lcv, t1 = t0 ^ lf;
                        const T a0r = sre[t0], a0i = sim[t0];
                        sre[t0] = sre[t1]; sim[t0] = sim[t1]; sre[t1] = a0r; sim[t1] = a0i;
                    }
                } else if (kind == OP_YP) {
                    // include/suqa_cpu.hpp:96-122: a1' = i a0, a0' = -i a1
                    const bool ori = op.orient != 0;  // logical roles swapped: Y negated
                    for (uint32_t u = threadIdx.x; u < npair; u += blockDim.x) {
                        const uint32_t t0 = deposit_zeros(u, sel) | lcv, t1 = t0 ^ lf;
                        const T a0r = sre[t0], a0i = sim[t0], a1r = sre[t1], a1i = sim[t1];
                        sre[t1] = neg_if(-a0i, ori); sim[t1] = neg_if(a0r, ori);
                        sre[t0] = neg_if(a1i, ori); sim[t0] = neg_if(-a1r, ori);
                    }
                } else if (kind == OP_HP) {
                    // include/suqa_cpu.hpp:150-206
                    if (lcm == 0u && (op.gdefer || p.defer)) {
                        const bool ori = op.orient != 0;
                        for (uint32_t pp = threadIdx.x; pp < TS / 2; pp += blockDim.x) {
                            const uint32_t t0 = insert_zero(pp, lp), t1 = t0 ^ lf;
                            const T a0r = sre[t0], a0i = sim[t0], a1r = sre[t1], a1i = sim[t1];
                            // logical (first, second) = (t0, t1), or (t1, t0) when oriented
                            const T sr = a0r + a1r, si = a0i + a1i;
                            const T dr = neg_if(a0r - a1r, ori), di = neg_if(a0i - a1i, ori);
                            sre[ori ? t1 : t0] = sr; sim[ori ? t1 : t0] = si;
                            sre[ori ? t0 : t1] = dr; sim[ori ? t0 : t1] = di;
                        }
                        if (!op.gdefer) sigma *= 0.7071067811865475;
                    } else {
                        const T h = tconv<T>(0.7071067811865475);
                        const bool ori = op.orient != 0;
                        for (uint32_t u = threadIdx.x; u < npair; u += blockDim.x) {
                            const uint32_t t0 = deposit_zeros(u, sel) | lcv, t1 = t0 ^ lf;
                            const T a0r = sre[t0], a0i = sim[t0], a1r = sre[t1], a1i = sim[t1];
                            const T sr = h * (a0r + a1r), si = h * (a0i + a1i);
                            const T dr = neg_if(h * (a0r - a1r), ori), di = neg_if(h * (a0i - a1i), ori);
                            sre[ori ? t1 : t0] = sr; sim[ori ? t1 : t0] = si;
                            sre[ori ? t0 : t1] = dr; sim[ori ? t0 : t1] = di;
                        }
                    }
                } else if (kind == OP_PAULI) {
                    // exp(i th P): a0' = c a0 + i s w(g1) a1, a1' = c a1 + i s w(g0) a0,
                    // w(g) = i^ny (-1)^parity(g & zy); the outer part of the parity is per tile
                    const int tpar = parity64(base & op.zy) ^ op.xpar;
                    const uint32_t lzy = op.lzy;
                    const int ny = op.ny, fz = op.fz;
                    if (lcm == 0u && (op.gdefer || p.defer)) {
                        const bool cbig = op.cbig != 0;
                        for (uint32_t pp = threadIdx.x; pp < TS / 2; pp += blockDim.x) {
                            const uint32_t t0 = insert_zero(pp, lp), t1 = t0 ^ lf;
                            const int pz0 = tpar ^ (__popc(t0 & lzy) & 1);
                            const int k1 = (1 + ny + 2 * pz0) & 3;
                            const int k0 = (1 + ny + 2 * (pz0 ^ fz)) & 3;
                            const T a0r = sre[t0], a0i = sim[t0], a1r = sre[t1], a1i = sim[t1];
                            T r0, i0, r1, i1;
                            rot_deferred<T>(a0r, a0i, a1r, a1i, k0, up, un, cbig, r0, i0);
                            rot_deferred<T>(a1r, a1i, a0r, a0i, k1, up, un, cbig, r1, i1);
                            sre[t0] = r0; sim[t0] = i0; sre[t1] = r1; sim[t1] = i1;
                        }
                        if (!op.gdefer) sigma *= cbig ? op.c : op.s;
                    } else {
                        for (uint32_t u = threadIdx.x; u < npair; u += blockDim.x) {
                            const uint32_t t0 = deposit_zeros(u, sel) | lcv, t1 = t0 ^ lf;
                            const int pz0 = tpar ^ (__popc(t0 & lzy) & 1);
                            const int k1 = (1 + ny + 2 * pz0) & 3;
                            const int k0 = (1 + ny + 2 * (pz0 ^ fz)) & 3;
                            const T a0r = sre[t0], a0i = sim[t0], a1r = sre[t1], a1i = sim[t1];
                            T r0, i0, r1, i1;
                            rot_k<T>(a0r, a0i, a1r, a1i, k0, c, s, sneg, r0, i0);
                            rot_k<T>(a1r, a1i, a0r, a0i, k1, c, s, sneg, r1, i1);
                            sre[t0] = r0; sim[t0] = i0; sre[t1] = r1; sim[t1] = i1;
                        }
                    }
                } else {  // OP_W: include/qms.cuh:245-309
                    for (uint32_t pp = threadIdx.x; pp < TS / 2; pp += blockDim.x) {
                        const uint32_t t0 = insert_zero(pp, lp), t1 = t0 ^ lf;
                        const uint64_t g0 = base | offs[t0 >> L] | (t0 & lowmask);
                        const uint32_t e = (uint32_t)((g0 & op.zy) >> op.shift);
                        const T f1 = tconv<T>(p.tab[2 * (op.tab + e)]), f2 = tconv<T>(p.tab[2 * (op.tab + e) + 1]);
                        const T a0r = sre[t0], a0i = sim[t0], a1r = sre[t1], a1i = sim[t1];
                        sre[t0] = f2 * a0r + f1 * a1r; sim[t0] = f2 * a0i + f1 * a1i;
                        sre[t1] = f1 * a0r - f2 * a1r; sim[t1] = f1 * a0i - f2 * a1i;
                    }
                }
            } else if (kind == OP_PHASE) {
                // include/suqa_kernels.cuh:175-190, :209-221: only the elements
                // whose bits in lcm equal lcv
                const uint32_t nsel = TS >> __popc(lcm);
                for (uint32_t u = threadIdx.x; u < nsel; u += blockDim.x) {
                    const uint32_t t = deposit_zeros(u, lcm) | lcv;
                    const T ar = sre[t], ai = sim[t];
                    sre[t] = ar * c - ai * s;
                    sim[t] = ai * c + ar * s;
                }
            } else if (kind == OP_PAULI) {  // all-Z string: diagonal c + i s (-1)^parity
                const int tpar = parity64(base & op.zy) ^ op.xpar;
                const uint32_t lzy = op.lzy;
                if (lcm == 0u && (op.gdefer || p.defer)) {
                    const bool cbig = op.cbig != 0;
                    for (uint32_t t = threadIdx.x; t < TS; t += blockDim.x) {
                        const T ar = sre[t], ai = sim[t];
                        T r, i;
                        rot_deferred<T>(ar, ai, ar, ai, (1 + 2 * (tpar ^ (__popc(t & lzy) & 1))) & 3, up, un, cbig, r, i);
                        sre[t] = r; sim[t] = i;
                    }
                    if (!op.gdefer) sigma *= cbig ? op.c : op.s;
                } else {
                    const uint32_t nsel = TS >> __popc(lcm);
                    for (uint32_t u = threadIdx.x; u < nsel; u += blockDim.x) {
                        const uint32_t t = deposit_zeros(u, lcm) | lcv;
                        const T ar = sre[t], ai = sim[t];
                        T r, i;
                        rot_k<T>(ar, ai, ar, ai, (1 + 2 * (tpar ^ (__popc(t & lzy) & 1))) & 3, c, s, sneg, r, i);
                        sre[t] = r; sim[t] = i;
                    }
                }
            } else {
                const bool unit = op.s == 1.0;
                for (uint32_t t = threadIdx.x; t < TS; t += blockDim.x) {
                    const uint64_t g = base | offs[t >> L] | (t & lowmask);
                    T ar = sre[t], ai = sim[t];
                    if (kind == OP_PLIST) {
                        // include/suqa_kernels.cuh:246-259 (guard: any gc bit set)
                        if ((g & op.cmask) == 0ull) continue;
                        const uint32_t e = (uint32_t)((g >> op.shift) & op.zy);
                        const T cx = tconv<T>(p.tab[2 * (op.tab + e)]), cy = tconv<T>(p.tab[2 * (op.tab + e) + 1]);
                        sre[t] = ar * cx - ai * cy;
                        sim[t] = ar * cy + ai * cx;
                    } else if (kind == OP_COLLAPSE) {
                        // src/suqa.cu:664-696: zero the discarded branch, rescale everything
                        // (a zero state gives 0 * inf = NaN everywhere, like the reference);
                        // a scale of exactly 1 (kept by the host's global scale) is skipped
                        const bool keep = (g & op.cmask) == op.cval;
                        if (unit) {
                            sre[t] = keep ? ar : tzero<T>();
                            sim[t] = keep ? ai : tzero<T>();
                        } else {
                            sre[t] = (keep ? ar : tzero<T>()) * s;
                            sim[t] = (keep ? ai : tzero<T>()) * s;
                        }
                    } else {  // OP_SCALE
                        sre[t] = ar * s;
                        sim[t] = ai * s;
                    }
                }
            }
            __syncthreads();
        }
        const T sg = tconv<T>(sigma);
        const double sg2 = sigma * sigma;

        // ---- reduction contribution and store.  Each thread sums the squared
        // magnitudes of its elements of this tile into an FP64 partial (an FP32
        // amplitude's |a|^2 is formed in FP32, the same operations in every
        // entry point, then added in FP64), then adds the partial, times the tile
        // scale sigma^2, to its accumulators; the split (red = 1) or filter
        // (red = 2) bit is enumerated directly when it lies in the tile, and
        // decided once per tile otherwise.
        if (p.red) {
            double part0 = 0.0, part1 = 0.0;
            if (p.red == 1 && p.lrm) {
                const uint32_t lb = (uint32_t)(__ffs(p.lrm) - 1);
                for (uint32_t pp = threadIdx.x; pp < TS / 2; pp += blockDim.x) {
                    const uint32_t t0 = insert_zero(pp, lb), t1 = t0 | (1u << lb);
                    part0 = add_sq(part0, sre[t0], sim[t0]);
                    part1 = add_sq(part1, sre[t1], sim[t1]);
                }
            } else if (p.red == 1) {
                for (uint32_t t = threadIdx.x; t < TS; t += blockDim.x) part0 = add_sq(part0, sre[t], sim[t]);
                if (base & p.rmask) {
                    part1 = part0;
                    part0 = 0.0;
                }
            } else if ((base & p.orm) == p.orv) {
                const uint32_t nsel = TS >> __popc(p.lrm);
                for (uint32_t u = threadIdx.x; u < nsel; u += blockDim.x) {
                    const uint32_t t = deposit_zeros(u, p.lrm) | p.lrv;
                    part0 = add_sq(part0, sre[t], sim[t]);
                }
            }
            acc0 += part0 * sg2;
            acc1 += part1 * sg2;
        }
        if (a.store) {
            const bool scaled = sigma != 1.0;
            const uint32_t xm = p.xm;
            if constexpr (kIsDf<T>) {
                double* dre = reinterpret_cast<double*>(a.re);
                double* dim = reinterpret_cast<double*>(a.im);
                for (uint32_t v = threadIdx.x; v < TS / 2; v += blockDim.x) {
                    const uint32_t t = v * 2;
                    const uint64_t g = base | offs[t >> L] | (t & lowmask);
                    // logical element t is the physical element t ^ xm
                    df64 r0 = sre[t ^ xm], r1 = sre[(t + 1) ^ xm], i0 = sim[t ^ xm], i1 = sim[(t + 1) ^ xm];
                    if (scaled) {
                        r0 = r0 * sg; r1 = r1 * sg; i0 = i0 * sg; i1 = i1 * sg;
                    }
                    if (a.df_out) {  // the next pass of this flush reads the pairs as they are
                        __stcs(reinterpret_cast<float4*>(dre + g), make_float4(r0.hi, r0.lo, r1.hi, r1.lo));
                        __stcs(reinterpret_cast<float4*>(dim + g), make_float4(i0.hi, i0.lo, i1.hi, i1.lo));
                    } else {
                        __stcs(reinterpret_cast<double2*>(dre + g), make_double2(df_to_double(r0), df_to_double(r1)));
                        __stcs(reinterpret_cast<double2*>(dim + g), make_double2(df_to_double(i0), df_to_double(i1)));
                    }
                }
            } else if (bulk && !scaled && (xm & lowmask) == 0u) {
                // the frame only permutes whole runs: logical run h is physical run h ^ xh
                fence_proxy_async_smem();
                __syncthreads();
                if (threadIdx.x < 32) {
                    const uint32_t xh = xm >> L;
                    for (uint32_t h = threadIdx.x; h < nh; h += 32) {
                        const uint64_t g = base | offs[h];
                        bulk_store(gre + g, sre + ((h ^ xh) << L), run_bytes);
                        bulk_store(gim + g, sim + ((h ^ xh) << L), run_bytes);
                    }
                    bulk_commit();
                }
            } else if ((1u << L) >= (uint32_t)W) {
                const uint32_t xv = xm & ~(uint32_t)(W - 1), xe = xm & (uint32_t)(W - 1);
                for (uint32_t v = threadIdx.x; v < TS / W; v += blockDim.x) {
                    const uint32_t t = v * W;
                    const uint64_t g = base | offs[t >> L] | (t & lowmask);
                    // logical element t is the physical element t ^ xm
                    V vr = *reinterpret_cast<const V*>(sre + (t ^ xv));
                    V vi = *reinterpret_cast<const V*>(sim + (t ^ xv));
                    if (xe) {
                        permute_vec(vr, xe);
                        permute_vec(vi, xe);
                    }
                    if (scaled) {
                        scale_vec(vr, sg);
                        scale_vec(vi, sg);
                    }
                    __stcs(reinterpret_cast<V*>(gre + g), vr);
                    __stcs(reinterpret_cast<V*>(gim + g), vi);
                }
            } else {
                for (uint32_t t = threadIdx.x; t < TS; t += blockDim.x) {
                    const uint64_t g = base | offs[t >> L] | (t & lowmask);
                    gre[g] = sre[t ^ xm] * sg;
                    gim[g] = sim[t ^ xm] * sg;
                }
            }
        }
        if (bulk) fence_proxy_async_smem();  // before later copies overwrite the buffer
        __syncthreads();
        if (bulk && nbuf == 1 && nxt < a.ntiles) issue_load(nbase, 0);
        tile = nxt;
        base = nbase;
        if (nbuf == 2) buf ^= 1;
    }
    if (bulk && threadIdx.x < 32) bulk_wait_all();  // stores complete before the CTA leaves
    if (dense_tc) {
        tc_fence_before();
        __syncthreads();
        if (threadIdx.x < 32) {
            tc_fence_after();
            tmem_dealloc(dsm.tmem, kDenseTmemCols);
        }
    }

    if (!p.red) return;
    if (p.rswap) {
        const double t = acc0;
        acc0 = acc1;
        acc1 = t;
    }
    // ---- deterministic two-level reduction: per-CTA partials, last CTA sums them
    block_reduce2<T>(acc0, acc1, red_sh);
    if (threadIdx.x == 0) {
        a.partials[2 * blockIdx.x] = acc0;
        a.partials[2 * blockIdx.x + 1] = acc1;
        __threadfence();
        const unsigned int tk = atomicAdd(a.ticket, 1u);
        last_flag = (tk == gridDim.x - 1u);
    }
    __syncthreads();
    if (!last_flag) return;
    __threadfence();
    double s0 = 0.0, s1 = 0.0;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        s0 += __ldcg(a.partials + 2 * b);
        s1 += __ldcg(a.partials + 2 * b + 1);
    }
    block_reduce2<T>(s0, s1, red_sh);
    if (threadIdx.x == 0) {
        a.result[0] = s0;
        a.result[1] = s1;
        if (a.result_host) {
            volatile double* h = a.result_host;
            h[0] = s0;
            h[1] = s1;
            h[3] = __ldcg(a.result + 3);  // the error word of this pass and earlier ones
        }
        *a.ticket = 0u;
    }
}

}  // namespace sqk
