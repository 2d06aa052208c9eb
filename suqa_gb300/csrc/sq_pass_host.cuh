// Host-side entry points of the pass-kernel instantiations.  The kernel
// template (sq_pass.cuh) is instantiated in sq_pass_f64.cu, sq_pass_f32.cu,
// sq_pass_tc.cu and sq_pass_df.cu, compiled in parallel; the engine selects an
// instantiation by tag (KTag) and reaches it through these three functions.
#pragma once

#include <cuda_runtime.h>

#include "sq_pass.cuh"

namespace sqk {

template <typename T_, int MAXT_, int F_>
struct KTag {
    typedef T_ T;
    static constexpr int MAXT = MAXT_;
    static constexpr int F = F_;
};

// Opts the kernel into `smem` bytes of dynamic shared memory on `device` (above
// the default 48 KiB) and the whole L1 / shared array as shared memory.
// *fits = false when the tile does not fit.
template <typename T, int MAXT, int F>
cudaError_t pass_set_smem(int device, size_t smem, bool* fits);

// Resident CTAs per SM at this block and dynamic shared-memory size.
template <typename T, int MAXT, int F>
cudaError_t pass_occupancy(int block, size_t smem, int* ctas);

template <typename T, int MAXT, int F>
cudaError_t pass_launch(const PassArgs& a, const Prog& p, int grid, int block, size_t smem, cudaStream_t stream);

}  // namespace sqk

// Definitions and explicit instantiation, for the instantiation units only.
#ifdef SQK_PASS_DEFINE
#include <atomic>

namespace sqk {

template <typename T, int MAXT, int F>
cudaError_t pass_set_smem(int device, size_t smem, bool* fits) {
    // per device (the attribute belongs to the device's context); states may run in several host threads
    static std::atomic<int> configured[64];
    *fits = true;
    if ((int)smem <= 48 * 1024 || (device >= 0 && device < 64 && configured[device].load() >= (int)smem))
        return cudaSuccess;
    int optin = 0;
    cudaFuncAttributes fa;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_pass<T, MAXT, F>);
    if (e != cudaSuccess) return e;
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if ((int)smem > dyn) {
        *fits = false;
        return cudaSuccess;
    }
    e = cudaFuncSetAttribute(k_pass<T, MAXT, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    // tiles are staged explicitly, and several CTAs per SM hide each other's waits
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_pass<T, MAXT, F>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e == cudaSuccess && device >= 0 && device < 64) configured[device] = dyn;
    return e;
}

template <typename T, int MAXT, int F>
cudaError_t pass_occupancy(int block, size_t smem, int* ctas) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_pass<T, MAXT, F>, block, smem);
}

template <typename T, int MAXT, int F>
cudaError_t pass_launch(const PassArgs& a, const Prog& p, int grid, int block, size_t smem, cudaStream_t stream) {
    k_pass<T, MAXT, F><<<grid, block, smem, stream>>>(a, p);
    return cudaGetLastError();
}

}  // namespace sqk

#define SQK_PASS_INSTANTIATE(T, MAXT, F)                                                                     \
    template cudaError_t sqk::pass_set_smem<T, MAXT, F>(int, size_t, bool*);                                 \
    template cudaError_t sqk::pass_occupancy<T, MAXT, F>(int, size_t, int*);                                 \
    template cudaError_t sqk::pass_launch<T, MAXT, F>(const sqk::PassArgs&, const sqk::Prog&, int, int, size_t, \
                                                      cudaStream_t);
#endif
