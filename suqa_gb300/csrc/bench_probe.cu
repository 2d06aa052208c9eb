// Benchmark support, not part of libsq's product ABI: built as its own library
// (libsq_probe.so) that only the benchmark and its test load.
//
// Device characterisation: the FP64 fused multiply-add rate of the CUDA cores
// (not the FP64 tensor path that DGEMM uses), the ceiling of the FP64 tile
// pass, whose gates are DADD/DMUL/DFMA streams.
#include <algorithm>
#include <string>

#include <cuda_runtime.h>

namespace {

std::string g_probe_err;

constexpr int kChains = 8;

__global__ void k_fp64_fma_rate(double* out, double a, double b, int iters) {
    double x[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) x[j] = threadIdx.x * 1e-9 + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) x[j] = fma(x[j], b, a);
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // one slot per thread of the grid
}

}  // namespace

extern "C" const char* sqb_last_error(void) { return g_probe_err.c_str(); }

// FP64 FMA instructions per second of the current device (independent chains on
// every SM), in G/s; returns 0, 1 (bad argument) or 2 (CUDA error).
extern "C" int sqb_fp64_fma_rate(double* gops, float* kernel_ms) {
    if (!gops) {
        g_probe_err = "null output";
        return 1;
    }
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = std::max(nsm, 1) * 4, threads = 256, iters = 4096;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(double) * blocks * threads);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {  // the first launch warms up
        e = cudaEventRecord(e0, 0);
        if (e == cudaSuccess) {
            k_fp64_fma_rate<<<blocks, threads>>>(out, 1e-12, 0.999999, iters);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) {
        g_probe_err = std::string("fp64 rate probe: ") + cudaGetErrorString(e);
        return 2;
    }
    *gops = (double)blocks * threads * iters * kChains / (ms * 1e-3) / 1e9;
    if (kernel_ms) *kernel_ms = ms;
    return 0;
}
