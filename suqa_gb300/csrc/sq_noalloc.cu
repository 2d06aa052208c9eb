// Allocation-free variant of the measurement-probability reduction.
//
// sq_qubit_probs_noalloc() runs the same tile-pass kernel as the state API's
// reductions (sq_pass.cuh, reduction-only pass split by one qubit) on a state
// the caller owns, writing (p0, p1) to a caller-provided device buffer.  The
// per-CTA partial sums and the completion ticket that the state API keeps in
// buffers allocated by sq_state_create live here in one file-scope device
// array instead, so the call performs no device or host allocation at all.
//
// Who needs this: code that must not allocate device memory on the call path —
// a host application whose memory manager owns every device buffer and only
// lends out the caller's state, a plugin invoked from another language runtime
// that hands over raw device pointers, or a latency-critical loop where an
// allocation (and the implicit synchronisation it can cause) is not acceptable.
//
// Limits and sharing rules:
//  - the scratch array holds partial sums for at most kNoAllocMaxCtas CTAs
//    (2 doubles each, 64 KiB in total plus a 256-byte header); every GPU that
//    loads the library keeps this array resident until the process exits;
//  - a launch needing more CTAs than that is rejected with SQ_ERR_ARG;
//  - every call shares the one array, so calls whose kernels overlap on the
//    GPU (different streams without ordering between them) race and give wrong
//    results; calls ordered on one stream are safe;
//  - the first call on a device does a one-time set-up on that device (symbol
//    address lookup, zeroing of the ticket); make that first call before any
//    stream capture begins.
#include <cstring>
#include <mutex>

#include "sq.h"
#include "sq_pass.cuh"

namespace sqi {
void set_error(const char* msg);  // sq_engine.cu: text returned by sq_last_error()
}

namespace {

constexpr int kNoAllocMaxCtas = 4096;
constexpr int kHeaderDoubles = 32;  // 256 bytes: the ticket lives in the first word
constexpr size_t kScratchDoubles = kHeaderDoubles + 2 * (size_t)kNoAllocMaxCtas;

// The shared scratch: [0] ticket (as unsigned int), [32 ...] per-CTA partial pairs.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct DeviceScratch {
    double* ptr = nullptr;  // device address of g_noalloc_scratch on this device
    int nsm = 0;
    bool ready = false;
};

constexpr int kMaxDevices = 64;
DeviceScratch g_dev[kMaxDevices];
std::mutex g_mu;

int fail(int code, const char* msg) {
    sqi::set_error(msg);
    return code;
}

// One-time per-device set-up, run with that device current.
int setup_device(int dev, DeviceScratch** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceScratch& d = g_dev[dev];
    if (!d.ready) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail(SQ_ERR_CUDA, cudaGetErrorString(e));
        e = cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(SQ_ERR_CUDA, cudaGetErrorString(e));
        // the completion ticket must start at zero; the last CTA of every call
        // resets it, so this is needed once
        e = cudaMemset(p, 0, sizeof(double) * kHeaderDoubles);
        if (e != cudaSuccess) return fail(SQ_ERR_CUDA, cudaGetErrorString(e));
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return fail(SQ_ERR_CUDA, cudaGetErrorString(e));
        d.ptr = static_cast<double*>(p);
        d.ready = true;
    }
    *out = &d;
    return SQ_OK;
}

}  // namespace

extern "C" int sq_qubit_probs_noalloc(const void* re, const void* im, uint32_t n, int precision, uint32_t q,
                                      double* out_p01, void* stream) {
    if (!re || !im || !out_p01) return fail(SQ_ERR_ARG, "null pointer argument");
    if (n < 1 || n > 33) return fail(SQ_ERR_ARG, "qubit count must be in 1..33");
    if (q >= n) return fail(SQ_ERR_ARG, "qubit index out of range");
    if (precision != SQ_F64 && precision != SQ_F32) return fail(SQ_ERR_ARG, "unknown precision");
    // The reduction reads 16-byte vectors (two doubles or four floats) whenever a
    // tile holds at least one vector; raw pointers from another runtime (a view
    // with a storage offset, say) may not be aligned for that, and a misaligned
    // vector load would end the CUDA context.  Reject them here, before any launch.
    {
        const size_t esz = precision == SQ_F64 ? 8 : 4;
        const uint32_t kt = n < 10 ? n : 10;
        const size_t need = ((size_t)1 << kt) * esz >= 16 ? 16 : esz;
        if (((uintptr_t)re | (uintptr_t)im) % need != 0)
            return fail(SQ_ERR_ARG, need == 16 ? "re and im must be 16-byte aligned"
                                               : "re and im must be aligned to the element size");
        if ((uintptr_t)out_p01 % 8 != 0) return fail(SQ_ERR_ARG, "out_p01 must be 8-byte aligned");
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(SQ_ERR_NODEVICE, "no usable CUDA device");
    DeviceScratch* d = nullptr;
    int rc = setup_device(dev, &d);
    if (rc) return rc;

    // reduction-only pass over tiles of 2^K contiguous amplitudes (K <= 10 keeps
    // the staging buffer within the default 48 KiB of shared memory)
    const int K = (int)n < 10 ? (int)n : 10;
    const uint64_t all = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
    const uint64_t lowm = (1ull << K) - 1ull;
    sqk::PassArgs a;
    memset(&a, 0, sizeof(a));
    a.re = const_cast<void*>(re);
    a.im = const_cast<void*>(im);
    a.K = K;
    a.L = K;
    a.store = 0;
    a.ofix = 0;
    a.ofree = all & ~lowm;
    a.ntiles = 1ull << (n - (uint32_t)K);
    a.partials = d->ptr + kHeaderDoubles;
    a.result = out_p01;
    a.ticket = reinterpret_cast<unsigned int*>(d->ptr);
    const uint64_t want = (uint64_t)d->nsm * 8ull;
    const uint64_t grid = a.ntiles < want ? a.ntiles : want;
    if (grid > (uint64_t)kNoAllocMaxCtas)
        return fail(SQ_ERR_ARG, "launch needs more partial-sum slots than the static scratch holds (4096 CTAs)");

    static thread_local sqk::Prog p;
    p.nops = 0;
    p.red = 1;
    p.defer = 0;
    p.rmask = 1ull << q;
    p.rval = 0;
    // tiles are the low K qubits: the split qubit is tile-local or outer
    p.lrm = q < (uint32_t)K ? (1u << q) : 0u;
    p.lrv = 0u;
    p.orm = q < (uint32_t)K ? 0ull : (1ull << q);
    p.orv = 0ull;
    p.xm = 0u;
    p.rswap = 0;
    const int block = (K == (int)n) ? (K >= 10 ? 1024 : (K >= 8 ? 256 : 128)) : 256;
    const size_t esz = precision == SQ_F64 ? 8 : 4;
    const size_t smem = 2 * ((size_t)1 << K) * esz + 8;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (precision == SQ_F64)
        sqk::k_pass<double><<<(unsigned)grid, block, smem, s>>>(a, p);
    else
        sqk::k_pass<float><<<(unsigned)grid, block, smem, s>>>(a, p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SQ_ERR_CUDA, cudaGetErrorString(e));
    return SQ_OK;
}
