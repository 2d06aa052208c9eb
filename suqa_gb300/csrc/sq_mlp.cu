// Warm-start network: a small MLP (in -> L hidden layers of H units with GELU ->
// out) trained and evaluated by hand-written kernels.  Weights and activations
// are stored in BF16, every product is accumulated in FP32, and the optimiser
// (Adam) keeps FP32 master weights.  The network is tiny (~35k parameters), so
// each kernel keeps a CTA's rows of activations in shared memory and streams
// the BF16 weights from L2; there is nothing GEMM-sized enough to feed tensor
// cores profitably.
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

// Forward for kRows rows per CTA; stores z_l (FP32) and a_l (BF16) of every layer
// for the backward pass.  act: [rows][sum of dims], z: [rows][sum of dims[1..]]
__global__ void k_forward(Geom g, const __nv_bfloat16* __restrict__ wb, const float* __restrict__ x, int batch,
                          float* __restrict__ y, float* __restrict__ zbuf, __nv_bfloat16* __restrict__ abuf,
                          int ztot, int atot) {
    __shared__ float a_in[kRows][kMaxWidth];
    __shared__ float a_out[kRows][kMaxWidth];
    const int r0 = blockIdx.x * kRows;
    const int nr = min(kRows, batch - r0);
    // input, rounded to BF16
    for (int i = threadIdx.x; i < kRows * g.dims[0]; i += blockDim.x) {
        const int r = i / g.dims[0], c = i % g.dims[0];
        const float v = r < nr ? bf(x[(size_t)(r0 + r) * g.dims[0] + c]) : 0.f;
        a_in[r][c] = v;
        if (r < nr && abuf) abuf[(size_t)(r0 + r) * atot + c] = __float2bfloat16(v);
    }
    __syncthreads();
    int zo = 0, ao = g.dims[0];
    for (int l = 0; l < g.nl; ++l) {
        const int din = g.dims[l], dout = g.dims[l + 1];
        const bool last = (l + 1 == g.nl);
        for (int o = threadIdx.x; o < dout; o += blockDim.x) {
            float acc[kRows];
            const float b = __bfloat162float(wb[g.boff[l] + o]);
#pragma unroll
            for (int r = 0; r < kRows; ++r) acc[r] = b;
            const __nv_bfloat16* wr = wb + g.woff[l] + (size_t)o * din;
            for (int i = 0; i < din; ++i) {
                const float w = __bfloat162float(wr[i]);
#pragma unroll
                for (int r = 0; r < kRows; ++r) acc[r] = fmaf(w, a_in[r][i], acc[r]);
            }
#pragma unroll
            for (int r = 0; r < kRows; ++r) {
                if (r >= nr) continue;
                const float z = acc[r];
                if (zbuf) zbuf[(size_t)(r0 + r) * ztot + zo + o] = z;
                const float a = last ? z : bf(gelu(z));
                a_out[r][o] = a;
                if (last) {
                    y[(size_t)(r0 + r) * dout + o] = z;
                } else if (abuf) {
                    abuf[(size_t)(r0 + r) * atot + ao + o] = __float2bfloat16(a);
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kRows * dout; i += blockDim.x) a_in[i / dout][i % dout] = a_out[i / dout][i % dout];
        __syncthreads();
        zo += dout;
        if (!last) ao += dout;
    }
}

// Backward for kRows rows per CTA: loss gradient, deltas layer by layer, weight
// and bias gradients accumulated into grad (FP32, atomics across CTAs).
__global__ void k_backward(Geom g, const __nv_bfloat16* __restrict__ wb, const float* __restrict__ y,
                           const float* __restrict__ t, const float* __restrict__ mask, int batch,
                           const float* __restrict__ zbuf, const __nv_bfloat16* __restrict__ abuf, int ztot, int atot,
                           float* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float d_cur[kRows][kMaxWidth];
    __shared__ float d_prev[kRows][kMaxWidth];
    const int r0 = blockIdx.x * kRows;
    const int nr = min(kRows, batch - r0);
    const int dl = g.dims[g.nl];
    // dL/dy = 2 * mask * (y - t) / batch
    float lsum = 0.f;
    for (int i = threadIdx.x; i < kRows * dl; i += blockDim.x) {
        const int r = i / dl, c = i % dl;
        float d = 0.f;
        if (r < nr) {
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
        // weight and bias gradients: dW[o][i] = sum_r d[r][o] * a_{l-1}[r][i]
        for (int idx = threadIdx.x; idx < dout * din; idx += blockDim.x) {
            const int o = idx / din, i = idx % din;
            float acc = 0.f;
            for (int r = 0; r < nr; ++r)
                acc = fmaf(d_cur[r][o], __bfloat162float(abuf[(size_t)(r0 + r) * atot + aoff[l] + i]), acc);
            atomicAdd(grad + g.woff[l] + idx, acc);
        }
        for (int o = threadIdx.x; o < dout; o += blockDim.x) {
            float acc = 0.f;
            for (int r = 0; r < nr; ++r) acc += d_cur[r][o];
            atomicAdd(grad + g.boff[l] + o, acc);
        }
        if (l == 0) break;
        // delta of the previous layer: (W^T d) * gelu'(z_{l-1})
        for (int idx = threadIdx.x; idx < kRows * din; idx += blockDim.x) {
            const int r = idx / din, i = idx % din;
            float acc = 0.f;
            if (r < nr) {
                for (int o = 0; o < dout; ++o)
                    acc = fmaf(__bfloat162float(wb[g.woff[l] + (size_t)o * din + i]), d_cur[r][o], acc);
                acc *= gelu_grad(zbuf[(size_t)(r0 + r) * ztot + zoff[l - 1] + i]);
            }
            d_prev[r][i] = acc;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < kRows * din; idx += blockDim.x) d_cur[idx / din][idx % din] = d_prev[idx / din][idx % din];
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
