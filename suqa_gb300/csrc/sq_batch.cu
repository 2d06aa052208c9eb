// Host side of the batched QMS engine: resumable chain batches (sq_batch_*) and
// the one-shot sq_qms_tfim_batch.  Device code: sq_batch_dev.cuh.
//
// A batch sorts its chains into width classes (same qubit count n).  Each class
// gets a storage mode (one CTA with the state in shared memory; a cluster with
// the state spread over its CTAs' shared memory; a cluster working on the state
// in L2-resident global memory), a CTA size and a grid.  One launch per class
// advances every unfinished chain of the class by a quota of steps; a segment
// (the launches of all classes plus the work-counter reset) is captured once in
// a CUDA graph and replayed.  Optionally an autotuner times the candidate CTA
// sizes of each class on a sample of its chains (the same chains and seeds for
// every candidate, so every candidate does identical work) and keeps the
// fastest.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "sq.h"
#include "sq_batch_dev.cuh"

namespace sqi {
void set_error(const char* msg);
}

using namespace sqb;

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

const void* kernel_of(int precision, int mode) {
    if (precision == SQ_F64) {
        if (mode == 0) return kernel_for<double, 0>();
        if (mode == 1) return kernel_for<double, 1>();
        return kernel_for<double, 2>();
    }
    if (mode == 0) return kernel_for<float, 0>();
    if (mode == 1) return kernel_for<float, 1>();
    return kernel_for<float, 2>();
}

size_t padded(int q) { return ((size_t)1 << q) + ((size_t)1 << q) / 32 + 1; }

struct Class {
    int n, first, count;
    int smax;  // longest ring of the class
    int mode, kd, threads;
    unsigned grid;
    size_t smem;
    float probe_ms;
};

uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ULL) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ULL;
    }
    return h;
}

struct CkptHeader {
    char magic[8];
    uint32_t version, nchains, precision, pad;
    uint64_t state_elems, total_samples, chain_hash;
};

}  // namespace

struct sq_batch {
    int precision = SQ_F64;
    size_t esz = 8;
    int dev = 0, nsm = 1, optin = 0;
    cudaStream_t st = nullptr;
    sq_batch_opts opts{};
    uint32_t nchains = 0;
    std::vector<DevChain> dc;
    std::vector<int> order;
    std::vector<Class> classes;
    size_t total_samples = 0, state_elems = 0;
    uint64_t chain_hash = 0;
    DevChain* d_ch = nullptr;
    int* d_order = nullptr;
    unsigned int* d_next = nullptr;
    ChainRec* d_rec = nullptr;
    double* d_E = nullptr;
    double* d_A = nullptr;
    uint32_t* d_step = nullptr;
    void* d_states = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // one stream per width class: the classes run concurrently, so the tail of
    // one class (its last, longest chains) overlaps the others' work
    std::vector<cudaStream_t> cst;
    std::vector<cudaEvent_t> cev;
    cudaEvent_t fork = nullptr;

    ~sq_batch() {
        if (gexec) cudaGraphExecDestroy(gexec);
        for (cudaStream_t x : cst) cudaStreamDestroy(x);
        for (cudaEvent_t x : cev) cudaEventDestroy(x);
        if (fork) cudaEventDestroy(fork);
        cudaFree(d_ch); cudaFree(d_order); cudaFree(d_next); cudaFree(d_rec);
        cudaFree(d_E); cudaFree(d_A); cudaFree(d_step); cudaFree(d_states);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
    }

    // dynamic shared memory of class c at a CTA size: the state slice (modes 0,
    // 1) or the staging area of the warp-group exchange for rings longer than
    // 10 spins (mode 2)
    size_t smem_of(const Class& c, int threads) const {
        if (c.mode != 2) return 2 * padded(c.n - c.kd) * esz;
        return c.smax > kChunkSpins ? 2 * (size_t)threads * kStageR * esz : 0;
    }

    // grid (in CTAs) for class c at a CTA size, or 0 if it cannot launch
    int grid_for(const Class& c, int threads, unsigned* grid) const {
        const void* k = kernel_of(precision, c.mode);
        const size_t smem = smem_of(c, threads);
        *grid = 0;
        if (c.mode == 0) {
            int bps = 0;
            SQB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, threads, smem));
            if (bps <= 0) return SQ_OK;
            *grid = (unsigned)std::min<long long>((long long)bps * nsm, c.count);
            return SQ_OK;
        }
        const unsigned csize = 1u << c.kd;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(csize * 64u, 1, 1);
        cfg.blockDim = dim3((unsigned)threads, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = csize;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int ncl = 0;
        SQB_CUDA(cudaOccupancyMaxActiveClusters(&ncl, k, &cfg));
        if (ncl <= 0) return SQ_OK;
        long long live = std::min<long long>(ncl, c.count);
        if (c.mode == 2) {
            const uint64_t budget = opts.l2_budget_bytes ? opts.l2_budget_bytes : (64ull << 20);
            const uint64_t chain_bytes = ((uint64_t)2 << c.n) * esz;
            live = std::min<long long>(live, std::max<long long>(1, (long long)(budget / chain_bytes)));
        }
        *grid = (unsigned)(live * csize);
        return SQ_OK;
    }

    int launch_class(const Class& c, const KArgs& a, int threads, unsigned grid, cudaStream_t stream) {
        const void* k = kernel_of(precision, c.mode);
        KArgs karg = a;
        void* args[] = {(void*)&karg};
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid, 1, 1);
        cfg.blockDim = dim3((unsigned)threads, 1, 1);
        cfg.dynamicSmemBytes = smem_of(c, threads);
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        if (c.mode != 0) {
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = 1u << c.kd;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
        }
        SQB_CUDA(cudaLaunchKernelExC(&cfg, k, args));
        return SQ_OK;
    }

    KArgs args_for(size_t ci, uint32_t quota) const {
        const Class& c = classes[ci];
        KArgs a;
        a.chains = d_ch;
        a.order = d_order + c.first;
        a.count = c.count;
        a.next = d_next + ci;
        a.recs = d_rec;
        a.sE = d_E;
        a.sA = d_A;
        a.sStep = d_step;
        a.states = d_states;
        a.quota = quota;
        a.kdist = c.kd;
        a.stage_elems = c.mode == 2 ? (uint32_t)(smem_of(c, c.threads) / esz) : 0u;
        return a;
    }

    // one segment: reset the work counters, launch every class on its own
    // stream (widest first), join
    int enqueue_segment(uint32_t quota) {
        SQB_CUDA(cudaMemsetAsync(d_next, 0, sizeof(unsigned int) * classes.size(), st));
        SQB_CUDA(cudaEventRecord(fork, st));
        for (size_t ci = 0; ci < classes.size(); ++ci) {
            SQB_CUDA(cudaStreamWaitEvent(cst[ci], fork, 0));
            const int rc = launch_class(classes[ci], args_for(ci, quota), classes[ci].threads, classes[ci].grid, cst[ci]);
            if (rc != SQ_OK) return rc;
            SQB_CUDA(cudaEventRecord(cev[ci], cst[ci]));
        }
        for (size_t ci = 0; ci < classes.size(); ++ci) SQB_CUDA(cudaStreamWaitEvent(st, cev[ci], 0));
        return SQ_OK;
    }

    int build_graph(uint32_t quota) {
        if (gexec) {
            cudaGraphExecDestroy(gexec);
            gexec = nullptr;
        }
        cudaGraph_t g = nullptr;
        SQB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_segment(quota);
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc != SQ_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return fail(SQ_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        const cudaError_t ie = cudaGraphInstantiate(&gexec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            gexec = nullptr;
            return fail(SQ_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        }
        return SQ_OK;
    }

    // Time each candidate CTA size of class ci on one step of the same sample of
    // its chains (scratch copies: the batch's own chains are not advanced).
    int autotune_class(size_t ci) {
        Class& c = classes[ci];
        const int cands64[] = {128, 256};
        const int cands32[] = {128, 256, 512};
        const int* cands = precision == SQ_F64 ? cands64 : cands32;
        const int ncand = precision == SQ_F64 ? 2 : 3;
        unsigned cap = 0;
        for (int k = 0; k < ncand; ++k) {
            unsigned g = 0;
            const int rc = grid_for(c, cands[k], &g);
            if (rc != SQ_OK) return rc;
            const unsigned chains_live = c.mode == 0 ? g : (g >> c.kd);
            cap = std::max(cap, chains_live);
        }
        const int S = (int)std::min<unsigned>(cap, (unsigned)c.count);
        if (S <= 0) return fail(SQ_ERR_ARG, "chain class cannot be launched");
        const size_t per = ((size_t)2 << c.n);
        std::vector<DevChain> pc(S);
        for (int k = 0; k < S; ++k) {
            pc[k] = dc[order[c.first + k]];
            pc[k].state_off = (uint64_t)k * per;
            pc[k].out_offset = k;
            pc[k].steps = 1;
        }
        std::vector<int> po(S);
        for (int k = 0; k < S; ++k) po[k] = k;
        DevChain* d_pc = nullptr;
        int* d_po = nullptr;
        ChainRec* d_pr = nullptr;
        double *d_pE = nullptr, *d_pA = nullptr;
        uint32_t* d_pS = nullptr;
        void* d_ps = nullptr;
        unsigned int* d_pn = nullptr;
        auto done = [&]() {
            cudaFree(d_pc); cudaFree(d_po); cudaFree(d_pr); cudaFree(d_pE);
            cudaFree(d_pA); cudaFree(d_pS); cudaFree(d_ps); cudaFree(d_pn);
        };
        if (cudaMalloc(&d_pc, sizeof(DevChain) * S) != cudaSuccess || cudaMalloc(&d_po, sizeof(int) * S) != cudaSuccess ||
            cudaMalloc(&d_pr, sizeof(ChainRec) * S) != cudaSuccess || cudaMalloc(&d_pE, sizeof(double) * S) != cudaSuccess ||
            cudaMalloc(&d_pA, sizeof(double) * S) != cudaSuccess || cudaMalloc(&d_pS, sizeof(uint32_t) * S) != cudaSuccess ||
            cudaMalloc(&d_ps, per * esz * S) != cudaSuccess || cudaMalloc(&d_pn, sizeof(unsigned int)) != cudaSuccess) {
            cudaGetLastError();
            done();
            return fail(SQ_ERR_NOMEM, "autotuner scratch allocation failed");
        }
        cudaMemcpyAsync(d_pc, pc.data(), sizeof(DevChain) * S, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_po, po.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st);
        float best = -1.f;
        int best_t = c.threads;
        for (int k = 0; k < ncand; ++k) {
            unsigned g = 0;
            int rc = grid_for(c, cands[k], &g);
            if (rc != SQ_OK) { done(); return rc; }
            if (g == 0) continue;
            if (c.mode != 0) g = std::min<unsigned>(g, (unsigned)S << c.kd);
            else g = std::min<unsigned>(g, (unsigned)S);
            KArgs a;
            a.chains = d_pc;
            a.order = d_po;
            a.count = S;
            a.next = d_pn;
            a.recs = d_pr;
            a.sE = d_pE;
            a.sA = d_pA;
            a.sStep = d_pS;
            a.states = d_ps;
            a.quota = 1;
            a.kdist = c.kd;
            a.stage_elems = c.mode == 2 ? (uint32_t)(smem_of(c, cands[k]) / esz) : 0u;
            cudaMemsetAsync(d_pr, 0, sizeof(ChainRec) * S, st);
            cudaMemsetAsync(d_pn, 0, sizeof(unsigned int), st);
            cudaEventRecord(e0, st);
            rc = launch_class(c, a, cands[k], g, st);
            if (rc != SQ_OK) { done(); return rc; }
            cudaEventRecord(e1, st);
            std::vector<ChainRec> pr(S);
            cudaMemcpyAsync(pr.data(), d_pr, sizeof(ChainRec) * S, cudaMemcpyDeviceToHost, st);
            const cudaError_t se = cudaStreamSynchronize(st);
            if (se != cudaSuccess) {
                done();
                return fail(SQ_ERR_CUDA, std::string("autotune probe: ") + cudaGetErrorString(se));
            }
            float wall = 0.f;
            cudaEventElapsedTime(&wall, e0, e1);
            // Throughput measure: the summed per-chain SM time over the number of
            // chains resident at once (the time a perfectly balanced queue would
            // take), scaled to milliseconds by the probe's own wall clock so the
            // clock rate cancels.  The probe's wall time alone is set by its
            // single longest chain, which every candidate shares.
            double sum_cyc = 0.0, max_cyc = 1.0;
            for (const ChainRec& r : pr) {
                sum_cyc += (double)r.cycles;
                max_cyc = std::max(max_cyc, (double)r.cycles);
            }
            const unsigned live = c.mode == 0 ? g : (g >> c.kd);
            const float ms = (float)(sum_cyc / std::max(1u, live) / max_cyc * wall);
            if (best < 0.f || ms < best) {
                best = ms;
                best_t = cands[k];
            }
        }
        done();
        c.threads = best_t;
        unsigned g = 0;
        const int rc = grid_for(c, best_t, &g);
        if (rc != SQ_OK) return rc;
        if (g == 0) return fail(SQ_ERR_ARG, "chain class cannot be launched");
        c.grid = g;
        c.smem = smem_of(c, best_t);
        c.probe_ms = best;
        return SQ_OK;
    }
};

extern "C" int sq_batch_create(sq_batch** out, const sq_tfim_chain* chains, uint32_t nchains, int precision,
                               const sq_batch_opts* opts) {
    if (!out) return fail(SQ_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!chains || nchains == 0) return fail(SQ_ERR_ARG, "null or empty chain list");
    if (precision != SQ_F64 && precision != SQ_F32) return fail(SQ_ERR_ARG, "unknown precision");
    sq_batch_opts o{};
    if (opts) o = *opts;
    if (o.threads != 0 && o.threads != 128 && o.threads != 256 && o.threads != 512)
        return fail(SQ_ERR_ARG, "threads must be 0, 128, 256 or 512");
    if (precision == SQ_F64 && o.threads == 512) return fail(SQ_ERR_ARG, "FP64 batches run at most 256 threads per CTA");
    std::vector<DevChain> dcs(nchains);
    size_t total_samples = 0, state_elems = 0;
    for (uint32_t i = 0; i < nchains; ++i) {
        const sq_tfim_chain& c = chains[i];
        if (c.spins < 2 || c.spins > 20 || c.ene_qbits < 1 || c.ene_qbits > 7)
            return fail(SQ_ERR_ARG, "chain sizes out of range (spins 2..20, energy qubits 1..7)");
        if (c.spins + c.ene_qbits + 1 > 22) return fail(SQ_ERR_ARG, "chain wider than 22 qubits");
        if (c.reset_each == 0 || c.max_reverse == 0 || !(c.ene_max > c.ene_min) || !(c.dt > 0))
            return fail(SQ_ERR_ARG, "invalid chain parameters");
        DevChain& d = dcs[i];
        std::memset(&d, 0, sizeof(d));
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
        d.out_offset = (int)total_samples;
        d.state_off = state_elems;
        d.warm = c.warm_start ? 1 : 0;
        for (int k = 0; k < 20; ++k) d.ry[k] = c.ry[k];
        total_samples += c.steps;
        state_elems += (size_t)2 << d.n;
    }
    sq_batch* b = new sq_batch();
    b->precision = precision;
    b->esz = precision == SQ_F64 ? 8 : 4;
    b->opts = o;
    b->nchains = nchains;
    b->dc.swap(dcs);
    b->total_samples = total_samples;
    b->state_elems = state_elems;
    b->chain_hash = fnv1a(b->dc.data(), sizeof(DevChain) * nchains);
    int rc = SQ_OK;
    do {
        cudaError_t ce = cudaGetDevice(&b->dev);
        if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, b->dev);
        if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&b->optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev);
        if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
        if (ce == cudaSuccess) ce = cudaEventCreate(&b->e0);
        if (ce == cudaSuccess) ce = cudaEventCreate(&b->e1);
        cudaFuncAttributes fa;
        if (ce == cudaSuccess) ce = cudaFuncGetAttributes(&fa, kernel_of(precision, 1));
        if (ce != cudaSuccess) {
            rc = fail(SQ_ERR_CUDA, std::string("chain batch set-up: ") + cudaGetErrorString(ce));
            break;
        }
        // every kernel may use all the opt-in shared memory beside its static part;
        // clusters of 16 CTAs are allowed
        for (int md = 0; md < 3 && ce == cudaSuccess; ++md) {
            cudaFuncAttributes fm;
            ce = cudaFuncGetAttributes(&fm, kernel_of(precision, md));
            if (ce == cudaSuccess)
                ce = cudaFuncSetAttribute(kernel_of(precision, md), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          b->optin - (int)fm.sharedSizeBytes);
            if (ce == cudaSuccess && md != 0)
                ce = cudaFuncSetAttribute(kernel_of(precision, md), cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        }
        if (ce != cudaSuccess) {
            rc = fail(SQ_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(ce));
            break;
        }
        // widest chain whose state fits one CTA's shared memory
        const size_t static_smem = fa.sharedSizeBytes + 1024;
        int smem_q = 0;
        while (smem_q < 22 && 2 * padded(smem_q + 1) * b->esz + static_smem <= (size_t)b->optin) ++smem_q;
        if (o.cta_qubits) smem_q = std::min(smem_q, (int)o.cta_qubits);

        b->order.resize(nchains);
        for (uint32_t i = 0; i < nchains; ++i) b->order[i] = (int)i;
        std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return b->dc[x].n > b->dc[y].n; });
        std::vector<int> max_spins;
        for (uint32_t k = 0; k < nchains; ++k) {
            const DevChain& d = b->dc[b->order[k]];
            if (b->classes.empty() || b->classes.back().n != d.n) {
                b->classes.push_back({d.n, (int)k, 0, 0, 0, 0, 256, 0, 0, -1.f});
                max_spins.push_back(0);
            }
            b->classes.back().count++;
            max_spins.back() = std::max(max_spins.back(), d.s);
            b->classes.back().smax = max_spins.back();
        }
        const int def_threads = o.threads ? (int)o.threads : 256;
        for (size_t ci = 0; ci < b->classes.size(); ++ci) {
            Class& c = b->classes[ci];
            // the spins and at least one more qubit always stay local to a CTA
            const int kmax = std::min(4, c.n - max_spins[ci] - 1);
            const bool global = o.global_qubits && c.n >= (int)o.global_qubits;
            if (c.n <= smem_q && !global) {
                c.mode = 0;
                c.kd = 0;
            } else if (c.n - smem_q <= kmax && !global) {
                c.mode = 1;
                c.kd = c.n - smem_q;
            } else {
                c.mode = 2;
                c.kd = kmax;
            }
            if (c.kd < 0 || (c.mode == 1 && c.kd < 1)) {
                rc = fail(SQ_ERR_ARG, "a chain class cannot be laid out (too few qubits outside the spins)");
                break;
            }
            c.threads = def_threads;
            c.smem = b->smem_of(c, c.threads);
            if (ce != cudaSuccess) {
                rc = fail(SQ_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(ce));
                break;
            }
            rc = b->grid_for(c, c.threads, &c.grid);
            if (rc != SQ_OK) break;
            if (c.grid == 0) {
                rc = fail(SQ_ERR_ARG, "a chain class cannot be launched (shared memory or cluster size)");
                break;
            }
        }
        if (rc != SQ_OK) break;
        if (cudaMalloc(&b->d_ch, sizeof(DevChain) * nchains) != cudaSuccess ||
            cudaMalloc(&b->d_order, sizeof(int) * nchains) != cudaSuccess ||
            cudaMalloc(&b->d_next, sizeof(unsigned int) * b->classes.size()) != cudaSuccess ||
            cudaMalloc(&b->d_rec, sizeof(ChainRec) * nchains) != cudaSuccess ||
            cudaMalloc(&b->d_E, sizeof(double) * (b->total_samples + 1)) != cudaSuccess ||
            cudaMalloc(&b->d_A, sizeof(double) * (b->total_samples + 1)) != cudaSuccess ||
            cudaMalloc(&b->d_step, sizeof(uint32_t) * (b->total_samples + 1)) != cudaSuccess ||
            cudaMalloc(&b->d_states, b->state_elems * b->esz) != cudaSuccess) {
            cudaGetLastError();
            rc = fail(SQ_ERR_NOMEM, "device allocation for the chain batch failed");
            break;
        }
        ce = cudaMemcpyAsync(b->d_ch, b->dc.data(), sizeof(DevChain) * nchains, cudaMemcpyHostToDevice, b->st);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(b->d_order, b->order.data(), sizeof(int) * nchains, cudaMemcpyHostToDevice, b->st);
        if (ce == cudaSuccess) ce = cudaMemsetAsync(b->d_rec, 0, sizeof(ChainRec) * nchains, b->st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->st);
        if (ce != cudaSuccess) {
            rc = fail(SQ_ERR_CUDA, std::string("chain batch upload: ") + cudaGetErrorString(ce));
            break;
        }
        b->cst.resize(b->classes.size(), nullptr);
        b->cev.resize(b->classes.size(), nullptr);
        for (size_t ci = 0; ci < b->classes.size() && ce == cudaSuccess; ++ci) {
            ce = cudaStreamCreateWithFlags(&b->cst[ci], cudaStreamNonBlocking);
            if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->cev[ci], cudaEventDisableTiming);
        }
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
        if (ce != cudaSuccess) {
            rc = fail(SQ_ERR_CUDA, std::string("class streams: ") + cudaGetErrorString(ce));
            break;
        }
        if (o.autotune && o.threads == 0)
            for (size_t ci = 0; ci < b->classes.size() && rc == SQ_OK; ++ci) rc = b->autotune_class(ci);
        if (rc != SQ_OK) break;
        if (o.use_graph && o.segment_steps > 0) rc = b->build_graph(o.segment_steps);
    } while (false);
    if (rc != SQ_OK) {
        delete b;
        return rc;
    }
    *out = b;
    return SQ_OK;
}

extern "C" int sq_batch_destroy(sq_batch* b) {
    delete b;
    return SQ_OK;
}

extern "C" int sq_batch_run(sq_batch* b, uint32_t steps, float* kernel_ms) {
    if (!b) return fail(SQ_ERR_ARG, "null batch");
    if (kernel_ms) *kernel_ms = 0.f;
    if (steps == 0) return SQ_OK;
    const uint32_t seg = b->opts.segment_steps ? b->opts.segment_steps : steps;
    SQB_CUDA(cudaEventRecord(b->e0, b->st));
    uint32_t left = steps;
    while (left > 0) {
        const uint32_t q = std::min(left, seg);
        if (b->gexec && q == b->opts.segment_steps) {
            SQB_CUDA(cudaGraphLaunch(b->gexec, b->st));
        } else {
            const int rc = b->enqueue_segment(q);
            if (rc != SQ_OK) return rc;
        }
        left -= q;
    }
    SQB_CUDA(cudaEventRecord(b->e1, b->st));
    const cudaError_t se = cudaStreamSynchronize(b->st);
    if (se != cudaSuccess) return fail(SQ_ERR_CUDA, std::string("chain batch: ") + cudaGetErrorString(se));
    if (kernel_ms) SQB_CUDA(cudaEventElapsedTime(kernel_ms, b->e0, b->e1));
    return SQ_OK;
}

extern "C" int sq_batch_results(sq_batch* b, sq_chain_result* results, double* samples_E, double* samples_A,
                                uint32_t* samples_step) {
    if (!b) return fail(SQ_ERR_ARG, "null batch");
    if (results) {
        std::vector<ChainRec> rec(b->nchains);
        SQB_CUDA(cudaMemcpyAsync(rec.data(), b->d_rec, sizeof(ChainRec) * b->nchains, cudaMemcpyDeviceToHost, b->st));
        SQB_CUDA(cudaStreamSynchronize(b->st));
        for (uint32_t i = 0; i < b->nchains; ++i) {
            results[i].accepted = rec[i].accepted;
            results[i].failures = rec[i].failures;
            results[i].samples = rec[i].samples;
            results[i].phase_estimations = rec[i].nphi;
            results[i].cycles = rec[i].cycles;
            results[i].evolution_cycles = rec[i].evo_cycles;
        }
    }
    const size_t T = b->total_samples;
    if (samples_E) SQB_CUDA(cudaMemcpyAsync(samples_E, b->d_E, sizeof(double) * T, cudaMemcpyDeviceToHost, b->st));
    if (samples_A) SQB_CUDA(cudaMemcpyAsync(samples_A, b->d_A, sizeof(double) * T, cudaMemcpyDeviceToHost, b->st));
    if (samples_step) SQB_CUDA(cudaMemcpyAsync(samples_step, b->d_step, sizeof(uint32_t) * T, cudaMemcpyDeviceToHost, b->st));
    SQB_CUDA(cudaStreamSynchronize(b->st));
    return SQ_OK;
}

extern "C" int sq_batch_progress(sq_batch* b, uint32_t* steps_done) {
    if (!b || !steps_done) return fail(SQ_ERR_ARG, "null argument");
    std::vector<ChainRec> rec(b->nchains);
    SQB_CUDA(cudaMemcpyAsync(rec.data(), b->d_rec, sizeof(ChainRec) * b->nchains, cudaMemcpyDeviceToHost, b->st));
    SQB_CUDA(cudaStreamSynchronize(b->st));
    for (uint32_t i = 0; i < b->nchains; ++i) steps_done[i] = rec[i].step;
    return SQ_OK;
}

extern "C" int sq_batch_state(sq_batch* b, uint32_t chain, double* re, double* im) {
    if (!b || !re || !im) return fail(SQ_ERR_ARG, "null argument");
    if (chain >= b->nchains) return fail(SQ_ERR_ARG, "chain index out of range");
    ChainRec rec;
    SQB_CUDA(cudaMemcpyAsync(&rec, b->d_rec + chain, sizeof(ChainRec), cudaMemcpyDeviceToHost, b->st));
    SQB_CUDA(cudaStreamSynchronize(b->st));
    if (!rec.started) return fail(SQ_ERR_ARG, "chain has not run yet");
    const DevChain& d = b->dc[chain];
    const size_t N = (size_t)1 << d.n;
    std::vector<unsigned char> buf(2 * N * b->esz);
    SQB_CUDA(cudaMemcpyAsync(buf.data(), (unsigned char*)b->d_states + d.state_off * b->esz, buf.size(),
                             cudaMemcpyDeviceToHost, b->st));
    SQB_CUDA(cudaStreamSynchronize(b->st));
    if (b->precision == SQ_F64) {
        const double* p = (const double*)buf.data();
        std::copy(p, p + N, re);
        std::copy(p + N, p + 2 * N, im);
    } else {
        const float* p = (const float*)buf.data();
        for (size_t i = 0; i < N; ++i) {
            re[i] = p[i];
            im[i] = p[N + i];
        }
    }
    return SQ_OK;
}

extern "C" int sq_batch_checkpoint_size(const sq_batch* b, uint64_t* bytes) {
    if (!b || !bytes) return fail(SQ_ERR_ARG, "null argument");
    *bytes = sizeof(CkptHeader) + sizeof(ChainRec) * (uint64_t)b->nchains + b->state_elems * b->esz +
             b->total_samples * (2 * sizeof(double) + sizeof(uint32_t));
    return SQ_OK;
}

extern "C" int sq_batch_checkpoint(sq_batch* b, void* host, uint64_t bytes) {
    uint64_t need = 0;
    const int rc = sq_batch_checkpoint_size(b, &need);
    if (rc != SQ_OK) return rc;
    if (!host || bytes < need) return fail(SQ_ERR_ARG, "checkpoint buffer too small");
    unsigned char* p = (unsigned char*)host;
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, "SQBATCH1", 8);
    h.version = 1;
    h.nchains = b->nchains;
    h.precision = (uint32_t)b->precision;
    h.state_elems = b->state_elems;
    h.total_samples = b->total_samples;
    h.chain_hash = b->chain_hash;
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    const size_t T = b->total_samples;
    SQB_CUDA(cudaMemcpyAsync(p, b->d_rec, sizeof(ChainRec) * b->nchains, cudaMemcpyDeviceToHost, b->st));
    p += sizeof(ChainRec) * b->nchains;
    SQB_CUDA(cudaMemcpyAsync(p, b->d_states, b->state_elems * b->esz, cudaMemcpyDeviceToHost, b->st));
    p += b->state_elems * b->esz;
    SQB_CUDA(cudaMemcpyAsync(p, b->d_E, sizeof(double) * T, cudaMemcpyDeviceToHost, b->st));
    p += sizeof(double) * T;
    SQB_CUDA(cudaMemcpyAsync(p, b->d_A, sizeof(double) * T, cudaMemcpyDeviceToHost, b->st));
    p += sizeof(double) * T;
    SQB_CUDA(cudaMemcpyAsync(p, b->d_step, sizeof(uint32_t) * T, cudaMemcpyDeviceToHost, b->st));
    SQB_CUDA(cudaStreamSynchronize(b->st));
    return SQ_OK;
}

extern "C" int sq_batch_restore(sq_batch* b, const void* host, uint64_t bytes) {
    uint64_t need = 0;
    const int rc = sq_batch_checkpoint_size(b, &need);
    if (rc != SQ_OK) return rc;
    if (!host || bytes < need) return fail(SQ_ERR_ARG, "checkpoint too short");
    const unsigned char* p = (const unsigned char*)host;
    CkptHeader h;
    std::memcpy(&h, p, sizeof(h));
    if (std::memcmp(h.magic, "SQBATCH1", 8) != 0 || h.version != 1) return fail(SQ_ERR_ARG, "not a chain-batch checkpoint");
    if (h.nchains != b->nchains || h.precision != (uint32_t)b->precision || h.state_elems != b->state_elems ||
        h.total_samples != b->total_samples || h.chain_hash != b->chain_hash)
        return fail(SQ_ERR_ARG, "checkpoint was written by a batch with different chains or precision");
    p += sizeof(h);
    const size_t T = b->total_samples;
    SQB_CUDA(cudaMemcpyAsync(b->d_rec, p, sizeof(ChainRec) * b->nchains, cudaMemcpyHostToDevice, b->st));
    p += sizeof(ChainRec) * b->nchains;
    SQB_CUDA(cudaMemcpyAsync(b->d_states, p, b->state_elems * b->esz, cudaMemcpyHostToDevice, b->st));
    p += b->state_elems * b->esz;
    SQB_CUDA(cudaMemcpyAsync(b->d_E, p, sizeof(double) * T, cudaMemcpyHostToDevice, b->st));
    p += sizeof(double) * T;
    SQB_CUDA(cudaMemcpyAsync(b->d_A, p, sizeof(double) * T, cudaMemcpyHostToDevice, b->st));
    p += sizeof(double) * T;
    SQB_CUDA(cudaMemcpyAsync(b->d_step, p, sizeof(uint32_t) * T, cudaMemcpyHostToDevice, b->st));
    SQB_CUDA(cudaStreamSynchronize(b->st));
    return SQ_OK;
}

extern "C" int sq_batch_plan(const sq_batch* b, sq_batch_class* info, uint32_t max, uint32_t* nclasses) {
    if (!b || !nclasses) return fail(SQ_ERR_ARG, "null argument");
    *nclasses = (uint32_t)b->classes.size();
    for (uint32_t i = 0; info && i < max && i < b->classes.size(); ++i) {
        const Class& c = b->classes[i];
        info[i].n = (uint32_t)c.n;
        info[i].count = (uint32_t)c.count;
        info[i].mode = (uint32_t)c.mode;
        info[i].cluster = 1u << c.kd;
        info[i].threads = (uint32_t)c.threads;
        info[i].grid = c.grid;
        info[i].smem_bytes = (uint32_t)c.smem;
        info[i].probe_ms = c.probe_ms;
    }
    return SQ_OK;
}

extern "C" int sq_qms_tfim_batch(const sq_tfim_chain* chains, uint32_t nchains, int precision, sq_chain_result* results,
                                 double* samples_E, double* samples_A, uint32_t* samples_step, void* stream,
                                 float* kernel_ms) {
    if (!results) return fail(SQ_ERR_ARG, "null results");
    // the batch runs on its own stream: order it after the caller's work
    if (stream) SQB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    sq_batch* b = nullptr;
    int rc = sq_batch_create(&b, chains, nchains, precision, nullptr);
    if (rc != SQ_OK) return rc;
    uint32_t maxs = 0;
    for (uint32_t i = 0; i < nchains; ++i) maxs = std::max(maxs, chains[i].steps);
    rc = sq_batch_run(b, maxs, kernel_ms);
    if (rc == SQ_OK) rc = sq_batch_results(b, results, samples_E, samples_A, samples_step);
    sq_batch_destroy(b);
    return rc;
}
