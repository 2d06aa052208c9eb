// Batched real-time evolution of transverse-field Ising rings with basis
// probabilities recorded after every Trotter step: the reference's evo driver
// (src/evo.cu:51-98: re-initialise, evolve by exp(-iHt), prob_filter every
// basis pattern of the system register, write a row per time) for many rings at
// once, on the batch engine's register-resident Trotter evolution.
//
// A job is a ring of s spins (H = -J sum Z_i Z_{i+1} - h sum X_i), an initial
// product state (|0...0> or RY(ry_i) per spin), a step width dt and a number of
// steps K.  Row k (k = 0..K) holds the 2^s probabilities |a_x|^2 (FP64) after k
// first-order Trotter steps of width dt, each the ZZ bond phases
// exp(i J dt Z_i Z_{i+1}) then exp(i h dt X_i) on every spin.  The state is
// advanced step by step (the reference restarts from t = 0 for every row; the
// result is the same product of steps).
//
// One CTA per job, its state in shared memory; the CTA is one warp group of
// 2^(s-9) warps for rings longer than 9 spins (the top spin bits exchange
// between the warps), else one warp.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "sq.h"
#include "sq_batch_dev.cuh"

namespace sqi {
void set_error(const char* msg);
}

namespace sqe {
using namespace sqb;

struct EvoJob {
    int s, steps, warm, pad;
    double J, h, dt;
    double ry[20];
    unsigned long long out_off;  // first probability of the job's rows
};

// chunk geometry: m chunk bits (lane + register), G warps per group
__host__ __device__ inline void evo_geometry(int s, int* m, int* G) {
    if (s < 5) {
        *m = 0;
        *G = 1;
    } else if (s <= kChunkSpins) {
        *m = s;
        *G = 1;
    } else {
        *m = kChunkSpins;
        *G = 1 << (s - kChunkSpins);
    }
}

template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 1 : 3) k_evo(const EvoJob* __restrict__ jobs, const int* __restrict__ ids,
                                             double* __restrict__ probs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ Shared sh;
    __shared__ T tz[24], sz[24];
    __shared__ T xc, xs, tn;
    const EvoJob& J = jobs[ids[blockIdx.x]];
    const int s = J.s;
    Ctx<T, 0> cx;
    cx.n = s;
    cx.k = 0;
    cx.nl = s;
    cx.Nl = 1u << s;
    cx.rank = 0;
    cx.sh = &sh;
    cx.re = reinterpret_cast<T*>(smem_raw);
    cx.im = cx.re + (cx.Nl + cx.Nl / 32 + 1);
    cx.gre = cx.gim = nullptr;
    cx.stage = nullptr;
    cx.stage_elems = 0;
    int m, G;
    evo_geometry(s, &m, &G);
    const double hd = J.h * J.dt;
    const bool regs = m >= 5 && fabs(hd) < 0.78;  // |h dt| < pi/4: tan well conditioned
    // one Trotter step's tables (cos(h dt)^s folded into the ZZ phases on the register path)
    if (threadIdx.x <= (unsigned)s) {
        double shd, chd, sn, cs;
        sincos(hd, &shd, &chd);
        const double ch = regs ? pow(chd, (double)s) : 1.0;
        sincos(J.J * J.dt * (double)(s - 2 * (int)threadIdx.x), &sn, &cs);
        tz[threadIdx.x] = (T)(cs * ch);
        sz[threadIdx.x] = (T)(sn * ch);
        if (threadIdx.x == 0) {
            xc = (T)chd;
            xs = (T)shd;
            tn = (T)(shd / chd);
        }
    }
    cx.init();
    if (J.warm) {
        for (int i = 0; i < s; ++i) {
            double sn, cs;
            sincos(0.5 * J.ry[i], &sn, &cs);
            cx.ry(i, (T)cs, (T)sn);
        }
    }
    __syncthreads();
    double* out = probs + J.out_off;
    for (int k = 0; k <= J.steps; ++k) {
        if (k > 0) {
            if (!regs) {
                cx.trotter_step_smem(s, -1, tz, sz, xc, xs);
            } else {
                switch (m) {
                    case 5: cx.template evolve_regs<1, false>(s, -1, 1, 1, tz, sz, tn); break;
                    case 6: cx.template evolve_regs<2, false>(s, -1, 1, 1, tz, sz, tn); break;
                    case 7: cx.template evolve_regs<4, false>(s, -1, 1, 1, tz, sz, tn); break;
                    case 8: cx.template evolve_regs<8, false>(s, -1, 1, 1, tz, sz, tn); break;
                    default:
                        if (G > 1) cx.template evolve_regs<16, true>(s, -1, 1, G, tz, sz, tn);
                        else cx.template evolve_regs<16, false>(s, -1, 1, 1, tz, sz, tn);
                        break;
                }
            }
        }
        double* row = out + (size_t)k * cx.Nl;
        for (uint32_t i = threadIdx.x; i < cx.Nl; i += blockDim.x) {
            const double a = (double)cx.re[cx.at(i)], b = (double)cx.im[cx.at(i)];
            row[i] = a * a + b * b;
        }
        __syncthreads();
    }
}

}  // namespace sqe

namespace {
int efail(int code, const std::string& m) {
    sqi::set_error(m.c_str());
    return code;
}
}  // namespace

extern "C" int sq_tfim_evolve_batch(const sq_tfim_evolution* jobs, uint32_t njobs, int precision, double* probs,
                                    float* kernel_ms) {
    using namespace sqe;
    if (!jobs || njobs == 0 || !probs) return efail(SQ_ERR_ARG, "null or empty job list");
    if (precision != SQ_F64 && precision != SQ_F32) return efail(SQ_ERR_ARG, "unknown precision");
    const size_t esz = precision == SQ_F64 ? 8 : 4;
    std::vector<EvoJob> ej(njobs);
    size_t total = 0;
    for (uint32_t i = 0; i < njobs; ++i) {
        const sq_tfim_evolution& j = jobs[i];
        if (j.spins < 2 || j.spins > 12) return efail(SQ_ERR_ARG, "ring length out of range (2..12 spins)");
        if (!(j.dt > 0)) return efail(SQ_ERR_ARG, "step width must be positive");
        EvoJob& e = ej[i];
        e.s = (int)j.spins;
        e.steps = (int)j.steps;
        e.warm = j.warm_start ? 1 : 0;
        e.pad = 0;
        e.J = j.J;
        e.h = j.h;
        e.dt = j.dt;
        for (int k = 0; k < 20; ++k) e.ry[k] = j.ry[k];
        e.out_off = total;
        total += (size_t)(j.steps + 1) << j.spins;
    }
    // one launch per ring length (CTA size = the ring's warp group)
    std::vector<int> order(njobs);
    for (uint32_t i = 0; i < njobs; ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ej[a].s > ej[b].s; });
    EvoJob* d_jobs = nullptr;
    int* d_ids = nullptr;
    double* d_probs = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_jobs);
        cudaFree(d_ids);
        cudaFree(d_probs);
    };
    if (cudaMalloc(&d_jobs, sizeof(EvoJob) * njobs) != cudaSuccess ||
        cudaMalloc(&d_ids, sizeof(int) * njobs) != cudaSuccess ||
        cudaMalloc(&d_probs, sizeof(double) * total) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return efail(SQ_ERR_NOMEM, "device allocation for the evolution batch failed");
    }
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_jobs, ej.data(), sizeof(EvoJob) * njobs, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_ids, order.data(), sizeof(int) * njobs, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaEventRecord(e0, st);
    const void* kf = precision == SQ_F64 ? (const void*)&k_evo<double> : (const void*)&k_evo<float>;
    for (uint32_t a = 0; a < njobs && err == cudaSuccess;) {
        const int s = ej[order[a]].s;
        uint32_t b = a;
        while (b < njobs && ej[order[b]].s == s) ++b;
        int m, G;
        evo_geometry(s, &m, &G);
        const unsigned threads = 32u * (unsigned)G;
        const size_t smem = 2 * (((size_t)1 << s) + ((size_t)1 << s) / 32 + 1) * esz;
        err = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 1));
        if (err != cudaSuccess) break;
        const int* ids = d_ids + a;
        void* args[] = {(void*)&d_jobs, (void*)&ids, (void*)&d_probs};
        err = cudaLaunchKernel(kf, dim3(b - a), dim3(threads), args, smem, st);
        a = b;
    }
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(probs, d_probs, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    float ms = 0.f;
    if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    if (kernel_ms) *kernel_ms = ms;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cleanup();
    if (err != cudaSuccess) return efail(SQ_ERR_CUDA, std::string("evolution batch: ") + cudaGetErrorString(err));
    return SQ_OK;
}
