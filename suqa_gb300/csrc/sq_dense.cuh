// Dense k-qubit blocks of the tile pass (OP_DENSE): consecutive gates on at most
// five tile qubits, fused on the host into one 32 x 32 complex matrix U, applied
// to every column of the tile (a column = the 32 amplitudes that differ only in
// the block's qubits) as a small complex GEMM.
//
// Tensor-core path (FP32 states, tiles of at least 2^12 amplitudes):
// D[c][n] = sum_k A[c][k] B[k][n] with k = (re/im, input index), n = (re/im,
// output index), A = the tile's columns, B = [[Re U, Im U], [-Im U, Re U]]^T, by
// tcgen05.mma kind::tf32 into a tensor-memory accumulator, M = 128 columns per
// chunk, N = 64, K = 64.  TF32 keeps 10 fraction bits, so each operand is split
// into a high part (rounded to TF32) and the remainder (rounded to TF32), and
// D = A_hi B_hi + A_hi B_lo + A_lo B_hi + A_lo B_lo: what is lost is the rounding
// of the remainders, about 2^-24 of each product.  B_hi and B_lo
// are prepared on the host in the operand layout; A is gathered from the tile
// per chunk.  Operand layout (no swizzle, K-major): per K-slice of 8 elements a
// 128 x 8 (A) or 64 x 8 (B) block of 8-row x 16-byte core matrices, the two
// halves of a core-matrix row pair 128 bytes apart (leading byte offset) and
// 8-row groups 256 bytes apart (stride byte offset).
//
// CUDA-core path (FP64 states, small tiles): y = U x per element, U in FP64
// from global memory, results through a shared-memory scratch copy.
#pragma once

namespace sqk {

constexpr int kDenseQubits = 5;
constexpr int kDenseDim = 1 << kDenseQubits;               // 32
constexpr uint32_t kDenseOperandBytes = 2u * 64u * 64u * 4u;  // B_hi + B_lo, 32 KiB
constexpr uint32_t kDenseABytes = 128u * 64u * 4u;          // one chunk of A, 32 KiB
constexpr uint32_t kDenseTmemCols = 128;  // the accumulator uses 64; the rest is margin
constexpr unsigned int kErrMmaWait = 2u;   // a tensor-core step did not complete in time

// instruction descriptor: D f32, A and B tf32, both K-major, N = 64, M = 128
constexpr uint32_t kIdescTf32 = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(kIdescTf32), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
// this warp's 32 lanes x 16 consecutive columns of 32-bit accumulators
__device__ __forceinline__ void tmem_ld_32x16(uint32_t taddr, float (&r)[16]) {
    uint32_t* u = reinterpret_cast<uint32_t*>(r);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]), "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
        : "r"(taddr)
        : "memory");
}
// the value rounded to TF32 (10 fraction bits, to nearest, ties away from zero):
// exactly representable, so the tensor core's own conversion leaves it unchanged
__device__ __forceinline__ float tf32_round(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// b-th set bit position of m, for b < popc(m)
__device__ __forceinline__ uint32_t nth_bit(uint32_t m, int b) {
    for (int i = 0; i < b; ++i) m &= m - 1u;
    return (uint32_t)(__ffs(m) - 1);
}
// bits of j placed at the set bits of m (ascending)
__device__ __forceinline__ uint32_t deposit_bits(uint32_t j, uint32_t m) {
    uint32_t r = 0u;
    for (int b = 0; m; ++b) {
        const uint32_t low = m & (~m + 1u);
        if ((j >> b) & 1u) r |= low;
        m ^= low;
    }
    return r;
}

struct DenseSmem {
    uint64_t bar_b;      // B operand loaded
    uint64_t bar_mma;    // MMA group finished
    uint32_t tmem;       // accumulator address
    uint32_t pad;
    uint32_t cdep[128];  // tile offset of chunk column m (block bits zero)
    uint32_t kdep[64];   // tile offset of operand index k = (re/im, j): re/im as +TS
};

}  // namespace sqk

namespace sqk {

// Bits of t at the set bits of m, packed (ascending).
__device__ __forceinline__ uint32_t extract_bits(uint32_t t, uint32_t m) {
    uint32_t r = 0u;
    for (int b = 0; m; ++b) {
        const uint32_t low = m & (~m + 1u);
        if (t & low) r |= 1u << b;
        m ^= low;
    }
    return r;
}

// One dense op on the tile by the tensor cores (FP32 tile of TS >= 4096
// amplitudes, re block then im block at tile; blockDim a multiple of 256).
// dbuf: A chunk (32 KiB) then B operand (32 KiB); gdense: this launch's operand
// blocks (32 KiB each, op.tab selects).  b_loaded remembers which operand block
// the B buffer holds across ops and tiles.  Returns false when a bounded wait
// gave up (the error word is set).
__device__ inline bool dense_tc_apply(float* tile, uint32_t TS, const Op& op, const float* gdense, unsigned char* dbuf,
                         DenseSmem& ds, uint32_t& ph_b, uint32_t& ph_mma, int& b_loaded, unsigned int* err) {
    const uint32_t bm = op.lflip;
    float* A = reinterpret_cast<float*>(dbuf);
    float* B = reinterpret_cast<float*>(dbuf + kDenseABytes);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    bool wait_b = false;
    if ((int)op.tab != b_loaded) {
        // the B buffer was last read by MMAs that completed (their commit was awaited)
        if (tid == 0) {
            mbar_arrive_expect_tx(&ds.bar_b, kDenseOperandBytes);
            bulk_load(B, gdense + (size_t)op.tab * (kDenseOperandBytes / 4u), kDenseOperandBytes, &ds.bar_b);
        }
        wait_b = true;
        b_loaded = (int)op.tab;
    }
    for (int k = tid; k < 64; k += blockDim.x) ds.kdep[k] = ((k >> 5) ? TS : 0u) + deposit_bits((uint32_t)k & 31u, bm);
    const uint32_t nchunk = (TS >> kDenseQubits) >> 7;
    const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
    for (uint32_t chunk = 0; chunk < nchunk; ++chunk) {
        for (int m = tid; m < 128; m += blockDim.x) ds.cdep[m] = deposit_zeros(chunk * 128u + (uint32_t)m, bm);
        __syncthreads();
        // gather A (128 columns x 64 operand indices) in the core-matrix layout: a warp
        // writes 8 rows x 16 bytes at a time
        const int r8 = lane >> 2, kq = lane & 3;
        // (the high part is stored already truncated to TF32, so the result does not
        // depend on how the tensor core converts FP32 inputs)
        for (int blk = warp; blk < 256; blk += nw) {
            const int sl = blk >> 5, g = (blk >> 1) & 15, kh = blk & 1;
            A[blk * 32 + lane] = tf32_round(tile[ds.cdep[g * 8 + r8] + ds.kdep[sl * 8 + kh * 4 + kq]]);
        }
        fence_proxy_async_smem();
        __syncthreads();
        bool ok = true;
        if (tid == 0) {
            if (wait_b) ok = mbar_wait_bounded(&ds.bar_b, ph_b, err, kErrMmaWait);
            tc_fence_after();
            if (ok) {
                for (int sl = 0; sl < 8; ++sl) {
                    const uint64_t ad = umma_desc(a0 + (uint32_t)sl * 4096u, 128u, 256u);
                    mma_tf32(ds.tmem, ad, umma_desc(b0 + (uint32_t)sl * 2048u, 128u, 256u), sl > 0 ? 1u : 0u);
                    mma_tf32(ds.tmem, ad, umma_desc(b0 + 16384u + (uint32_t)sl * 2048u, 128u, 256u), 1u);
                }
                mma_commit(&ds.bar_mma);
            }
        }
        if (wait_b) {
            ph_b ^= 1u;
            wait_b = false;
        }
        if (__syncthreads_or(!ok)) return false;
        ok = mbar_wait_bounded(&ds.bar_mma, ph_mma, err, kErrMmaWait);
        ph_mma ^= 1u;
        if (__syncthreads_or(!ok)) return false;
        // A_lo B_hi + A_lo B_lo with the remainders of the same elements, rounded to
        // TF32 (the tile is unchanged until the results are written back)
        for (int blk = warp; blk < 256; blk += nw) {
            const int sl = blk >> 5, g = (blk >> 1) & 15, kh = blk & 1;
            const float x = tile[ds.cdep[g * 8 + r8] + ds.kdep[sl * 8 + kh * 4 + kq]];
            A[blk * 32 + lane] = tf32_round(x - tf32_round(x));
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            for (int sl = 0; sl < 8; ++sl) {
                const uint64_t ad = umma_desc(a0 + (uint32_t)sl * 4096u, 128u, 256u);
                mma_tf32(ds.tmem, ad, umma_desc(b0 + (uint32_t)sl * 2048u, 128u, 256u), 1u);
                mma_tf32(ds.tmem, ad, umma_desc(b0 + 16384u + (uint32_t)sl * 2048u, 128u, 256u), 1u);
            }
            mma_commit(&ds.bar_mma);
        }
        ok = mbar_wait_bounded(&ds.bar_mma, ph_mma, err, kErrMmaWait);
        ph_mma ^= 1u;
        if (__syncthreads_or(!ok)) return false;
        tc_fence_after();
        // D (TMEM lane = column m, TMEM column = output index n): warp w reads lanes
        // 32 (w % 4) .. +31 and columns 32 (w / 4) .. +31 (re outputs, then im)
        if (warp < 8) {
            const uint32_t cb = ds.cdep[32 * (warp & 3) + lane];
            const bool write = (cb & op.lcm) == op.lcv;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                float r[16];
                const int k0 = 32 * (warp >> 2) + 16 * half;
                tmem_ld_32x16(ds.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)k0, r);
                if (write) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) tile[cb + ds.kdep[k0 + i]] = r[i];
                }
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    return true;
}

// One dense op by the CUDA cores: y = U x per column, U (32 x 32 complex FP64,
// [out][in], re/im interleaved) from global memory; outputs go through the
// scratch copy (2 TS elements) so every column reads its inputs unmodified.
template <typename T>
__device__ void dense_cc(T* tile, uint32_t TS, const Op& op, const double* U, T* scratch, DenseSmem& ds) {
    const uint32_t bm = op.lflip;
    for (int k = threadIdx.x; k < kDenseDim; k += blockDim.x) ds.kdep[k] = deposit_bits((uint32_t)k, bm);
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < TS; t += blockDim.x) {
        const uint32_t cb = t & ~bm;
        if ((cb & op.lcm) != op.lcv) {
            scratch[t] = tile[t];
            scratch[TS + t] = tile[TS + t];
            continue;
        }
        const uint32_t j = extract_bits(t, bm);
        const double* row = U + 2 * kDenseDim * j;
        double yr = 0.0, yi = 0.0;
        for (int i = 0; i < kDenseDim; ++i) {
            const uint32_t ti = cb | ds.kdep[i];
            const double xr = (double)tile[ti], xi = (double)tile[TS + ti];
            const double ur = row[2 * i], ui = row[2 * i + 1];
            yr = __fma_rn(ur, xr, __fma_rn(-ui, xi, yr));
            yi = __fma_rn(ur, xi, __fma_rn(ui, xr, yi));
        }
        scratch[t] = (T)yr;
        scratch[TS + t] = (T)yi;
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < 2 * TS; t += blockDim.x) tile[t] = scratch[t];
}

}  // namespace sqk
