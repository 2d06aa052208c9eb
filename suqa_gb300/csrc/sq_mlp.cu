// Warm-start network: a small MLP (in -> L hidden layers of H units with GELU ->
// out) trained and evaluated by hand-written kernels.  Weights and activations
// are stored in BF16, every product is accumulated in FP32, and the optimiser
// (Adam) keeps FP32 master weights.  The network is tiny (~35k parameters), so
// each kernel keeps a CTA's 16 rows of activations in shared memory, streams the
// BF16 weights from L2 and runs its products as warp-level MMAs (a 16-row block
// is exactly one MMA tile high).
//
// Layout: parameters are one flat FP32 array, layer by layer: W_l (out_l x in_l,
// row major) then b_l.  Forward for a row x: a_0 = x; z_l = W_l a_{l-1} + b_l;
// a_l = gelu(z_l) for hidden layers, y = z_L for the output layer, with
// gelu(z) = z * Phi(z) (erf form).  Rounding points (shared with the CPU oracle
// in oracle/mlp_oracle.py): W, a_l and the input are rounded to BF16; z_l and all
// sums are FP32.  Loss: mean over rows of sum over outputs of mask * (y - t)^2.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "sq.h"

namespace sqi {
void set_error(const char* msg);
}

namespace sqm {

constexpr int kMaxLayers = 6;
constexpr int kMaxWidth = 256;
constexpr int kRows = 16;  // batch rows per CTA

struct Geom {
    int nl;                 // number of weight layers (hidden layers + 1)
    int dims[kMaxLayers + 1];
    int woff[kMaxLayers];   // offset of W_l in the flat parameter array
    int boff[kMaxLayers];   // offset of b_l
    int nparams;
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    return cdf + z * pdf;
}
__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16(x)); }

// FP32 master -> BF16 working copy
__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) wb[i] = __float2bfloat16(w[i]);
}

// ---- warp-level tensor-core products (mma.sync) --------------------------------
// Fragment layouts (PTX ISA), g = lane / 4, t = lane % 4:
//   m16n8k16 .bf16: A a0 (g, 2t..2t+1), a1 (g+8, 2t..), a2 (g, 2t+8..), a3 (g+8, 2t+8..);
//                   B b0 (k = 2t..2t+1, n = g), b1 (k = 2t+8.., n = g);
//   m16n8k8 .tf32:  A a0 (g, t), a1 (g+8, t), a2 (g, t+4), a3 (g+8, t+4); B b0 (t, g), b1 (t+4, g);
//   D (both):       d0 (g, 2t), d1 (g, 2t+1), d2 (g+8, 2t), d3 (g+8, 2t+1).
// Each register of a BF16 fragment holds two elements, the lower index in the low half.
constexpr int kPitch = kMaxWidth + 8;  // shared row pitch: fragment loads of 8 rows spread over the banks

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // exact for BF16 values
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    const __nv_bfloat162 v = __halves2bfloat162(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// FP32 x = hi + lo with hi rounded to TF32; lo keeps the rest (the tensor cores
// read its top TF32 bits): two products give FP32 accuracy against an exact
// TF32 operand (BF16 weights and activations are exact in TF32)
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
    lo = __float_as_uint(x - __uint_as_float(hi));
}

// Forward for kRows rows per CTA; stores z_l (FP32) and a_l (BF16) of every layer
// for the backward pass.  act: [rows][sum of dims], z: [rows][sum of dims[1..]].
// Each layer is [16 rows x din] x W_l^T on the tensor cores (m16n8k16 BF16, FP32
// sums with the bias as the initial sum); warps take the 8-column output tiles.
__global__ void k_forward(Geom g, const __nv_bfloat16* __restrict__ wb, const float* __restrict__ x, int batch,
                          float* __restrict__ y, float* __restrict__ zbuf, __nv_bfloat16* __restrict__ abuf,
                          int ztot, int atot) {
    __shared__ float a_in[kRows][kPitch];
    __shared__ float a_out[kRows][kPitch];
    const int r0 = blockIdx.x * kRows;
    const int nr = min(kRows, batch - r0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int gq = lane >> 2, tq = lane & 3;
    // input, rounded to BF16; columns up to the next multiple of 16 zero
    const int kin = (g.dims[0] + 15) & ~15;
    for (int i = threadIdx.x; i < kRows * kin; i += blockDim.x) {
        const int r = i / kin, c = i % kin;
        const float v = (r < nr && c < g.dims[0]) ? bf(x[(size_t)(r0 + r) * g.dims[0] + c]) : 0.f;
        a_in[r][c] = v;
        if (r < nr && c < g.dims[0] && abuf) abuf[(size_t)(r0 + r) * atot + c] = __float2bfloat16(v);
    }
    __syncthreads();
    int zo = 0, ao = g.dims[0];
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int l = 0; l < g.nl; ++l) {
        const int din = g.dims[l], dout = g.dims[l + 1];
        const bool last = (l + 1 == g.nl);
        const int ksteps = (din + 15) >> 4, ntiles = (dout + 7) >> 3;
        const int kout = (dout + 15) & ~15;
        const __nv_bfloat16* W = wb + g.woff[l];
        for (int tile = warp; tile < ntiles; tile += nwarps) {
            const int c0 = tile * 8 + 2 * tq;  // this lane's output columns c0, c0 + 1
            const float bia0 = c0 < dout ? __bfloat162float(wb[g.boff[l] + c0]) : 0.f;
            const float bia1 = c0 + 1 < dout ? __bfloat162float(wb[g.boff[l] + c0 + 1]) : 0.f;
            float d[4] = {bia0, bia1, bia0, bia1};
            const int n = tile * 8 + gq;  // this lane's B column (output unit)
            const __nv_bfloat16* wrow = W + (size_t)n * din;
            auto wv = [&](int k) { return (n < dout && k < din) ? wrow[k] : zero; };
            for (int ks = 0; ks < ksteps; ++ks) {
                const int k0 = ks * 16 + 2 * tq;
                uint32_t a[4];
                a[0] = pack_bf16(a_in[gq][k0], a_in[gq][k0 + 1]);
                a[1] = pack_bf16(a_in[gq + 8][k0], a_in[gq + 8][k0 + 1]);
                a[2] = pack_bf16(a_in[gq][k0 + 8], a_in[gq][k0 + 9]);
                a[3] = pack_bf16(a_in[gq + 8][k0 + 8], a_in[gq + 8][k0 + 9]);
                mma_bf16(d, a, pack_bf16(wv(k0), wv(k0 + 1)), pack_bf16(wv(k0 + 8), wv(k0 + 9)));
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = gq + ((j & 2) ? 8 : 0), c = c0 + (j & 1);
                if (c >= dout) continue;
                const float z = d[j];
                const float a = last ? z : bf(gelu(z));
                a_out[r][c] = a;
                if (r >= nr) continue;
                if (zbuf) zbuf[(size_t)(r0 + r) * ztot + zo + c] = z;
                if (last) y[(size_t)(r0 + r) * dout + c] = z;
                else if (abuf) abuf[(size_t)(r0 + r) * atot + ao + c] = __float2bfloat16(a);
            }
        }
        // padding columns of the next layer's input are zero
        for (int i = threadIdx.x; i < kRows * (kout - dout); i += blockDim.x)
            a_out[i / (kout - dout)][dout + i % (kout - dout)] = 0.f;
        __syncthreads();
        for (int i = threadIdx.x; i < kRows * kout; i += blockDim.x) a_in[i / kout][i % kout] = a_out[i / kout][i % kout];
        __syncthreads();
        zo += dout;
        if (!last) ao += dout;
    }
}

// Backward for kRows rows per CTA: loss gradient, deltas layer by layer, weight
// and bias gradients accumulated into grad (FP32, atomics across CTAs).  Both
// products per layer on the tensor cores (m16n8k8 TF32; the FP32 deltas split
// hi + lo, the BF16 weights and activations exact in TF32):
//   dW[o][i] = sum_r d[r][o] a[r][i]   (M = outputs, N = inputs, K = the 16 rows)
//   d'[r][i] = sum_o d[r][o] W[o][i]   (M = rows, N = inputs, K = outputs)
__global__ void k_backward(Geom g, const __nv_bfloat16* __restrict__ wb, const float* __restrict__ y,
                           const float* __restrict__ t, const float* __restrict__ mask, int batch,
                           const float* __restrict__ zbuf, const __nv_bfloat16* __restrict__ abuf, int ztot, int atot,
                           float* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float d_cur[kRows][kPitch];
    __shared__ float d_prev[kRows][kPitch];
    const int r0 = blockIdx.x * kRows;
    const int nr = min(kRows, batch - r0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int gq = lane >> 2, tq = lane & 3;
    const int dl = g.dims[g.nl];
    const int kdl = (dl + 15) & ~15;
    // dL/dy = 2 * mask * (y - t) / batch; columns up to the next multiple of 16 zero
    float lsum = 0.f;
    for (int i = threadIdx.x; i < kRows * kdl; i += blockDim.x) {
        const int r = i / kdl, c = i % kdl;
        float d = 0.f;
        if (r < nr && c < dl) {
            const size_t k = (size_t)(r0 + r) * dl + c;
            const float m = mask ? mask[k] : 1.f;
            const float e = y[k] - t[k];
            d = 2.f * m * e / (float)batch;
            lsum += m * e * e;
        }
        d_cur[r][c] = d;
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, lsum / (float)batch);
    __syncthreads();
    // activation offsets of each layer's input
    int aoff[kMaxLayers + 1], zoff[kMaxLayers + 1];
    aoff[0] = 0;
    for (int l = 1; l < g.nl; ++l) aoff[l] = aoff[l - 1] + g.dims[l - 1];
    zoff[0] = 0;
    for (int l = 1; l <= g.nl; ++l) zoff[l] = zoff[l - 1] + g.dims[l];
    for (int l = g.nl - 1; l >= 0; --l) {
        const int din = g.dims[l], dout = g.dims[l + 1];
        const __nv_bfloat16* W = wb + g.woff[l];
        // weight gradients: 16-output x 8-input tiles, K = the CTA's 16 rows (two k-steps)
        {
            const int mt = (dout + 15) >> 4, nt = (din + 7) >> 3;
            for (int tile = warp; tile < mt * nt; tile += nwarps) {
                const int o0 = (tile / nt) * 16, i0 = (tile % nt) * 8;
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                const int ib = i0 + gq;  // this lane's B column (input unit)
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
                    const int ra = ks * 8 + tq;  // rows k = t and t + 4 of this k-step
                    uint32_t ahi[4], alo[4];
                    split_tf32(d_cur[ra][o0 + gq], ahi[0], alo[0]);
                    split_tf32(d_cur[ra][o0 + gq + 8], ahi[1], alo[1]);
                    split_tf32(d_cur[ra + 4][o0 + gq], ahi[2], alo[2]);
                    split_tf32(d_cur[ra + 4][o0 + gq + 8], ahi[3], alo[3]);
                    const float x0 = (ra < nr && ib < din)
                                         ? __bfloat162float(abuf[(size_t)(r0 + ra) * atot + aoff[l] + ib]) : 0.f;
                    const float x1 = (ra + 4 < nr && ib < din)
                                         ? __bfloat162float(abuf[(size_t)(r0 + ra + 4) * atot + aoff[l] + ib]) : 0.f;
                    const uint32_t b0 = __float_as_uint(x0), b1 = __float_as_uint(x1);
                    mma_tf32(d, ahi, b0, b1);
                    mma_tf32(d, alo, b0, b1);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int o = o0 + gq + ((j & 2) ? 8 : 0), i = i0 + 2 * tq + (j & 1);
                    if (o < dout && i < din) atomicAdd(grad + g.woff[l] + (size_t)o * din + i, d[j]);
                }
            }
        }
        for (int o = threadIdx.x; o < dout; o += blockDim.x) {
            float acc = 0.f;
            for (int r = 0; r < nr; ++r) acc += d_cur[r][o];
            atomicAdd(grad + g.boff[l] + o, acc);
        }
        if (l == 0) break;
        // delta of the previous layer: (d W) * gelu'(z_{l-1}); 16-row x 8-input tiles, K = outputs
        {
            const int ksteps = (dout + 7) >> 3, nt = (din + 7) >> 3;
            for (int tile = warp; tile < nt; tile += nwarps) {
                const int i0 = tile * 8, ib = i0 + gq;
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                for (int ks = 0; ks < ksteps; ++ks) {
                    const int k0 = ks * 8 + tq;  // outputs k = t and t + 4 of this k-step
                    uint32_t ahi[4], alo[4];
                    split_tf32(d_cur[gq][k0], ahi[0], alo[0]);
                    split_tf32(d_cur[gq + 8][k0], ahi[1], alo[1]);
                    split_tf32(d_cur[gq][k0 + 4], ahi[2], alo[2]);
                    split_tf32(d_cur[gq + 8][k0 + 4], ahi[3], alo[3]);
                    const float w0 = (k0 < dout && ib < din) ? __bfloat162float(W[(size_t)k0 * din + ib]) : 0.f;
                    const float w1 = (k0 + 4 < dout && ib < din) ? __bfloat162float(W[(size_t)(k0 + 4) * din + ib]) : 0.f;
                    const uint32_t b0 = __float_as_uint(w0), b1 = __float_as_uint(w1);
                    mma_tf32(d, ahi, b0, b1);
                    mma_tf32(d, alo, b0, b1);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int r = gq + ((j & 2) ? 8 : 0), i = i0 + 2 * tq + (j & 1);
                    if (i >= din) continue;
                    d_prev[r][i] = r < nr ? d[j] * gelu_grad(zbuf[(size_t)(r0 + r) * ztot + zoff[l - 1] + i]) : 0.f;
                }
            }
        }
        // the next layer's K: inputs up to the next multiple of 16, the padding zero
        const int kin = (din + 15) & ~15;
        for (int i = threadIdx.x; i < kRows * (kin - din); i += blockDim.x)
            d_prev[i / (kin - din)][din + i % (kin - din)] = 0.f;
        __syncthreads();
        for (int i = threadIdx.x; i < kRows * kin; i += blockDim.x) d_cur[i / kin][i % kin] = d_prev[i / kin][i % kin];
        __syncthreads();
    }
}

// Adam on the FP32 master weights (bias-corrected), then the gradient is cleared
__global__ void k_adam(float* __restrict__ w, float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gr = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        grad[i] = 0.f;
    }
}

}  // namespace sqm

struct sq_mlp {
    sqm::Geom g;
    float* w = nullptr;         // master weights
    __nv_bfloat16* wb = nullptr;
    float *grad = nullptr, *m = nullptr, *v = nullptr;
    float* loss = nullptr;
    int step = 0;
    int cap = 0;                // rows of the work buffers
    float *x = nullptr, *y = nullptr, *t = nullptr, *mask = nullptr, *z = nullptr;
    __nv_bfloat16* a = nullptr;
    int ztot = 0, atot = 0;
};

namespace {
int mfail(int code, const std::string& m) {
    sqi::set_error(m.c_str());
    return code;
}
#define SQM_CUDA(call)                                                                                \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return mfail(SQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int ensure_rows(sq_mlp* n, int rows) {
    if (rows <= n->cap) return SQ_OK;
    cudaFree(n->x); cudaFree(n->y); cudaFree(n->t); cudaFree(n->mask); cudaFree(n->z); cudaFree(n->a);
    const int din = n->g.dims[0], dout = n->g.dims[n->g.nl];
    SQM_CUDA(cudaMalloc(&n->x, sizeof(float) * rows * din));
    SQM_CUDA(cudaMalloc(&n->y, sizeof(float) * rows * dout));
    SQM_CUDA(cudaMalloc(&n->t, sizeof(float) * rows * dout));
    SQM_CUDA(cudaMalloc(&n->mask, sizeof(float) * rows * dout));
    SQM_CUDA(cudaMalloc(&n->z, sizeof(float) * (size_t)rows * n->ztot));
    SQM_CUDA(cudaMalloc(&n->a, sizeof(__nv_bfloat16) * (size_t)rows * n->atot));
    n->cap = rows;
    return SQ_OK;
}

int refresh_bf16(sq_mlp* n) {
    sqm::k_to_bf16<<<64, 256>>>(n->w, n->wb, n->g.nparams);
    SQM_CUDA(cudaGetLastError());
    return SQ_OK;
}

int run_forward(sq_mlp* n, const float* x_host, int batch, bool keep) {
    int rc = ensure_rows(n, batch);
    if (rc) return rc;
    SQM_CUDA(cudaMemcpy(n->x, x_host, sizeof(float) * batch * n->g.dims[0], cudaMemcpyHostToDevice));
    const int grid = (batch + sqm::kRows - 1) / sqm::kRows;
    sqm::k_forward<<<grid, 128>>>(n->g, n->wb, n->x, batch, n->y, keep ? n->z : nullptr, keep ? n->a : nullptr,
                                   n->ztot, n->atot);
    SQM_CUDA(cudaGetLastError());
    return SQ_OK;
}

int run_backward(sq_mlp* n, const float* t_host, const float* mask_host, int batch, float* loss_out) {
    const int dout = n->g.dims[n->g.nl];
    SQM_CUDA(cudaMemcpy(n->t, t_host, sizeof(float) * batch * dout, cudaMemcpyHostToDevice));
    if (mask_host) SQM_CUDA(cudaMemcpy(n->mask, mask_host, sizeof(float) * batch * dout, cudaMemcpyHostToDevice));
    SQM_CUDA(cudaMemset(n->loss, 0, sizeof(float)));
    const int grid = (batch + sqm::kRows - 1) / sqm::kRows;
    sqm::k_backward<<<grid, 256>>>(n->g, n->wb, n->y, n->t, mask_host ? n->mask : nullptr, batch, n->z, n->a, n->ztot,
                                    n->atot, n->grad, n->loss);
    SQM_CUDA(cudaGetLastError());
    if (loss_out) SQM_CUDA(cudaMemcpy(loss_out, n->loss, sizeof(float), cudaMemcpyDeviceToHost));
    return SQ_OK;
}
}  // namespace

extern "C" {

int sq_mlp_create(sq_mlp** out, uint32_t in, uint32_t hidden, uint32_t layers, uint32_t outdim, uint64_t seed) {
    if (!out) return mfail(SQ_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (in < 1 || outdim < 1 || hidden < 1 || layers < 1 || layers + 1 > (uint32_t)sqm::kMaxLayers ||
        in > (uint32_t)sqm::kMaxWidth || hidden > (uint32_t)sqm::kMaxWidth || outdim > (uint32_t)sqm::kMaxWidth)
        return mfail(SQ_ERR_ARG, "network dimensions out of range (widths <= 256, hidden layers <= 5)");
    sq_mlp* n = new sq_mlp();
    sqm::Geom& g = n->g;
    g.nl = (int)layers + 1;
    g.dims[0] = (int)in;
    for (uint32_t l = 1; l <= layers; ++l) g.dims[l] = (int)hidden;
    g.dims[g.nl] = (int)outdim;
    int off = 0;
    for (int l = 0; l < g.nl; ++l) {
        g.woff[l] = off;
        off += g.dims[l] * g.dims[l + 1];
        g.boff[l] = off;
        off += g.dims[l + 1];
    }
    g.nparams = off;
    n->ztot = 0;
    for (int l = 1; l <= g.nl; ++l) n->ztot += g.dims[l];
    n->atot = 0;
    for (int l = 0; l < g.nl; ++l) n->atot += g.dims[l];
    // He-style initialisation, deterministic in the seed
    std::vector<float> w(off, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < g.nl; ++l) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / (float)g.dims[l]));
        for (int i = 0; i < g.dims[l] * g.dims[l + 1]; ++i) w[g.woff[l] + i] = nd(rng);
    }
    if (cudaMalloc(&n->w, sizeof(float) * off) != cudaSuccess ||
        cudaMalloc(&n->wb, sizeof(__nv_bfloat16) * off) != cudaSuccess ||
        cudaMalloc(&n->grad, sizeof(float) * off) != cudaSuccess || cudaMalloc(&n->m, sizeof(float) * off) != cudaSuccess ||
        cudaMalloc(&n->v, sizeof(float) * off) != cudaSuccess || cudaMalloc(&n->loss, sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        sq_mlp_destroy(n);
        return mfail(SQ_ERR_NOMEM, "device allocation of the network failed");
    }
    cudaMemcpy(n->w, w.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
    cudaMemset(n->grad, 0, sizeof(float) * off);
    cudaMemset(n->m, 0, sizeof(float) * off);
    cudaMemset(n->v, 0, sizeof(float) * off);
    int rc = refresh_bf16(n);
    if (rc) {
        sq_mlp_destroy(n);
        return rc;
    }
    *out = n;
    return SQ_OK;
}

int sq_mlp_destroy(sq_mlp* n) {
    if (!n) return SQ_OK;
    cudaFree(n->w); cudaFree(n->wb); cudaFree(n->grad); cudaFree(n->m); cudaFree(n->v); cudaFree(n->loss);
    cudaFree(n->x); cudaFree(n->y); cudaFree(n->t); cudaFree(n->mask); cudaFree(n->z); cudaFree(n->a);
    delete n;
    return SQ_OK;
}

int sq_mlp_num_params(const sq_mlp* n, uint32_t* count) {
    if (!n || !count) return mfail(SQ_ERR_ARG, "null argument");
    *count = (uint32_t)n->g.nparams;
    return SQ_OK;
}

int sq_mlp_get_params(sq_mlp* n, float* flat) {
    if (!n || !flat) return mfail(SQ_ERR_ARG, "null argument");
    SQM_CUDA(cudaMemcpy(flat, n->w, sizeof(float) * n->g.nparams, cudaMemcpyDeviceToHost));
    return SQ_OK;
}

int sq_mlp_set_params(sq_mlp* n, const float* flat) {
    if (!n || !flat) return mfail(SQ_ERR_ARG, "null argument");
    SQM_CUDA(cudaMemcpy(n->w, flat, sizeof(float) * n->g.nparams, cudaMemcpyHostToDevice));
    n->step = 0;
    SQM_CUDA(cudaMemset(n->m, 0, sizeof(float) * n->g.nparams));
    SQM_CUDA(cudaMemset(n->v, 0, sizeof(float) * n->g.nparams));
    return refresh_bf16(n);
}

int sq_mlp_forward(sq_mlp* n, const float* x, uint32_t batch, float* y) {
    if (!n || !x || !y || batch == 0) return mfail(SQ_ERR_ARG, "null argument or empty batch");
    int rc = run_forward(n, x, (int)batch, false);
    if (rc) return rc;
    SQM_CUDA(cudaMemcpy(y, n->y, sizeof(float) * batch * n->g.dims[n->g.nl], cudaMemcpyDeviceToHost));
    return SQ_OK;
}

int sq_mlp_gradients(sq_mlp* n, const float* x, const float* t, const float* mask, uint32_t batch, float* grad,
                     float* loss) {
    if (!n || !x || !t || !grad || batch == 0) return mfail(SQ_ERR_ARG, "null argument or empty batch");
    SQM_CUDA(cudaMemset(n->grad, 0, sizeof(float) * n->g.nparams));
    int rc = run_forward(n, x, (int)batch, true);
    if (rc) return rc;
    rc = run_backward(n, t, mask, (int)batch, loss);
    if (rc) return rc;
    SQM_CUDA(cudaMemcpy(grad, n->grad, sizeof(float) * n->g.nparams, cudaMemcpyDeviceToHost));
    SQM_CUDA(cudaMemset(n->grad, 0, sizeof(float) * n->g.nparams));
    return SQ_OK;
}

int sq_mlp_train_step(sq_mlp* n, const float* x, const float* t, const float* mask, uint32_t batch, float lr,
                      float* loss) {
    if (!n || !x || !t || batch == 0) return mfail(SQ_ERR_ARG, "null argument or empty batch");
    int rc = run_forward(n, x, (int)batch, true);
    if (rc) return rc;
    rc = run_backward(n, t, mask, (int)batch, loss);
    if (rc) return rc;
    n->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
    sqm::k_adam<<<64, 256>>>(n->w, n->grad, n->m, n->v, n->g.nparams, lr, b1, b2, 1e-8f, c1, c2);
    SQM_CUDA(cudaGetLastError());
    return refresh_bf16(n);
}

}  // extern "C"
