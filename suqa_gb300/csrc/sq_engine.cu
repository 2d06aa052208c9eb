// libsq host side: state objects, the gate queue, the pass planner and the C ABI
// declared in include/sq.h.  Device work is the tile-pass kernel in sq_pass.cuh.
#include "sq.h"
#include "sq_pass.cuh"
#include "sq_pass_host.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define SQ_CUDA(call)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(SQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct HostOp {
    uint8_t kind = 0;
    uint8_t ny = 0;
    uint64_t flip = 0;              // global pair mask (0 for diagonal ops)
    uint64_t cmask = 0, cval = 0;   // element condition
    uint64_t skm = 0, skv = 0;      // condition under which the op can touch an element
    uint64_t zy = 0;
    uint32_t shift = 0;
    double c = 0.0, s = 0.0;
    std::vector<double> tab;        // complex pairs (PLIST: cos/sin, W: f1/f2)
    uint8_t gdefer = 0;             // its scale factor is kept in sq_state::gscale
    // OP_DENSE: 2^k x 2^k complex matrix (re, im interleaved, [out][in]) on the
    // qubits of flip, index bit b = the b-th lowest qubit of flip
    std::vector<double> dense;
};

using cplx = std::complex<double>;

inline int popc(uint64_t x) { return __builtin_popcountll(x); }

}  // namespace

// error text shared with the other translation units of libsq
namespace sqi {
void set_error(const char* msg) { g_err = msg; }
}  // namespace sqi

struct sq_state {
    uint32_t n = 0;
    int prec = SQ_F64;
    size_t esz = 8;
    uint64_t N = 0;
    void* data = nullptr;           // device: re block then im block
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<HostOp> pending;
    double* d_partials = nullptr;
    double* d_result = nullptr;
    unsigned int* d_ticket = nullptr;
    double* h_result = nullptr;     // pinned (and mapped, where the device can map host memory)
    double* h_result_dev = nullptr; // device address of h_result, or null: results come by copy
    int fusion = 1;
    // global scale: the state is gscale x the stored amplitudes.  Uncontrolled H
    // and Pauli rotations leave their common factor (1/sqrt 2, cos or sin of the
    // angle) here instead of multiplying every amplitude, and so do the
    // renormalisations of measurement and vnormalize; it is applied to memory
    // (one fused scale) before any read-out and when it drifts far from 1.
    double gscale = 1.0;
    int staging = 0;                // multi-tile passes: 0 registers, 1 bulk copies, 2 double-buffered bulk
    // dense blocks: automatic fusion threshold (0 = off), engine (0 tensor cores
    // where possible, 1 CUDA cores), and the per-launch operand ring
    // FP64 states: multi-tile passes of gates without tables or dense blocks run
    // their arithmetic in double-float on the FP32 pipe (sq_set_double_float)
    int dfloat = 0;
    int dense_fusion = 0;
    int dense_engine = 0;
    void* dense_dev = nullptr;      // kDenseSlots x kMaxDensePerPass x 32 KiB
    void* dense_host = nullptr;     // pinned mirror
    cudaEvent_t dense_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool dense_ev_used[4] = {false, false, false, false};
    uint32_t dense_slot = 0;
    int nsm = 1;
    int max_grid = 1;
    std::vector<std::pair<uint64_t, int>> occ_cache;  // (block << 32 | smem) -> resident CTAs per SM
    int kp = 0;                     // default tile size for this state
    sq_stats stats{};
    int device = 0;
    // kernel timing (sq_set_timing)
    int timing = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_open;
    std::vector<uint64_t> ev_bytes;
};

namespace {

constexpr int kSmallMaxF64 = 12;  // whole state in one CTA's shared memory
constexpr int kSmallMaxF32 = 13;
constexpr int kTileMaxF64 = 13;
constexpr int kTileMaxF32 = 14;

int small_max(const sq_state* s) { return s->prec == SQ_F64 ? kSmallMaxF64 : kSmallMaxF32; }
int tile_cap(const sq_state* s) { return s->prec == SQ_F64 ? kTileMaxF64 : kTileMaxF32; }

int default_tile(const sq_state* s) {
    if ((int)s->n <= small_max(s)) return (int)s->n;
    const int kmax = s->prec == SQ_F64 ? 12 : 13;
    int k = (int)s->n - 8;
    if (k < 8) k = 8;
    if (k > kmax) k = kmax;
    return k;
}

size_t tile_smem(const sq_state* s, int K, int L) {
    return (size_t)2 * ((size_t)1 << K) * s->esz + (size_t)8 * ((size_t)1 << (K - L));
}

// The pass kernel for element type T (FP64, FP32, or double-float arithmetic on
// an FP64 state), CTA size bound MAXT (multi-tile passes 256 threads, 512 with
// tensor-core blocks; single-tile passes up to 1024) and optional parts F
// (sq_pass.cuh, PassFeat), reached through the entry points of sq_pass_host.cuh.

// Opts the pass kernel into the shared memory a tile needs (above the default 48 KiB).
template <class Tag>
int configure_smem(sq_state* s, size_t smem) {
    bool fits = true;
    SQ_CUDA((sqk::pass_set_smem<typename Tag::T, Tag::MAXT, Tag::F>(s->device, smem, &fits)));
    if (!fits) return fail(SQ_ERR_UNSUPPORTED, "tile does not fit in shared memory");
    return SQ_OK;
}

// CTAs of the pass kernel resident per SM at this block and tile size (cached per
// state): a pass launches one full wave, every CTA looping over an equal share of
// the tiles, so no partial last wave leaves SMs idle.
template <class Tag>
int resident_ctas(sq_state* s, int block, size_t smem, int* out) {
    // kernels differ by element type and parts: FP64 and double-float passes of one state share the cache
    const uint64_t key = ((uint64_t)(std::is_same<typename Tag::T, sqk::df64>::value ? 1 : 0) << 63) |
                         ((uint64_t)Tag::F << 56) | ((uint64_t)block << 32) | (uint64_t)smem;
    for (const auto& kv : s->occ_cache)
        if (kv.first == key) {
            *out = kv.second;
            return SQ_OK;
        }
    int rc = configure_smem<Tag>(s, smem);
    if (rc) return rc;
    int occ = 0;
    SQ_CUDA((sqk::pass_occupancy<typename Tag::T, Tag::MAXT, Tag::F>(block, smem, &occ)));
    s->occ_cache.emplace_back(key, occ);
    *out = occ;
    return SQ_OK;
}

template <class Tag>
int launch_pass_t(sq_state* s, const sqk::PassArgs& a, const sqk::Prog& p, int grid, int block, size_t smem) {
    int rc = configure_smem<Tag>(s, smem);
    if (rc) return rc;
    SQ_CUDA((sqk::pass_launch<typename Tag::T, Tag::MAXT, Tag::F>(a, p, grid, block, smem, s->stream)));
    return SQ_OK;
}

// Calls fn(KTag<T, MAXT, F>{}) with the leanest instantiation a pass needs:
// double-float arithmetic, single tile (1024-thread bound), dense blocks (on the
// tensor cores: FP32 only), bulk staging (multi-tile passes without dense blocks).
template <class Fn>
int with_pass_kernel(const sq_state* s, bool use_df, bool single, bool dense, bool tc, bool bulk, Fn&& fn) {
    using sqk::KTag;
    using sqk::PF_BULK;
    using sqk::PF_DENSE;
    using sqk::PF_TC;
    if (use_df) return fn(KTag<sqk::df64, 256, 0>{});
    if (s->prec == SQ_F64) {
        if (single) return dense ? fn(KTag<double, 1024, PF_DENSE>{}) : fn(KTag<double, 1024, 0>{});
        if (dense) return fn(KTag<double, 256, PF_DENSE>{});
        return bulk ? fn(KTag<double, 256, PF_BULK>{}) : fn(KTag<double, 256, 0>{});
    }
    if (dense && tc)
        return single ? fn(KTag<float, 1024, PF_DENSE | PF_TC>{}) : fn(KTag<float, 512, PF_DENSE | PF_TC>{});
    if (single) return dense ? fn(KTag<float, 1024, PF_DENSE>{}) : fn(KTag<float, 1024, 0>{});
    if (dense) return fn(KTag<float, 256, PF_DENSE>{});
    return bulk ? fn(KTag<float, 256, PF_BULK>{}) : fn(KTag<float, 256, 0>{});
}

// ---- dense blocks ---------------------------------------------------------
constexpr int kDenseSlots = 4;
constexpr int kMaxDensePerPass = 8;
constexpr size_t kDenseBlockBytes = 32768;  // one dense op's data in a launch

uint64_t deposit64(uint64_t j, uint64_t m) {
    uint64_t r = 0;
    for (int b = 0; m; ++b) {
        const uint64_t low = m & (~m + 1ull);
        if ((j >> b) & 1ull) r |= low;
        m ^= low;
    }
    return r;
}
uint32_t extract64(uint64_t g, uint64_t m) {
    uint32_t r = 0;
    for (int b = 0; m; ++b) {
        const uint64_t low = m & (~m + 1ull);
        if (g & low) r |= 1u << b;
        m ^= low;
    }
    return r;
}

// Qubits an op reads or writes.
uint64_t op_support(const HostOp& h) { return h.flip | h.cmask | h.zy; }

// Ops whose stored action can be folded into a dense block.
bool op_fusable(const HostOp& h) {
    return (h.kind == sqk::OP_SWAPP || h.kind == sqk::OP_YP || h.kind == sqk::OP_HP || h.kind == sqk::OP_PAULI ||
            h.kind == sqk::OP_PHASE) &&
           h.tab.empty();
}

// Applies a queued op, in the form the pass kernel applies it (the factors of
// uncontrolled H and Pauli rotations stay in the global scale), to v, a vector
// over the qubits of bm (index bit b = the b-th lowest qubit of bm) holding
// every qubit the op touches.
void apply_stored(const HostOp& h, uint64_t bm, std::vector<cplx>& v) {
    const uint32_t D = (uint32_t)v.size();
    const cplx I(0.0, 1.0);
    auto ipow = [&](int k) -> cplx {
        switch (k & 3) {
            case 0: return cplx(1.0, 0.0);
            case 1: return I;
            case 2: return cplx(-1.0, 0.0);
            default: return -I;
        }
    };
    const bool deferred = h.cmask == 0ull && h.gdefer;
    const bool cbig = std::fabs(h.c) >= std::fabs(h.s);
    const double u = (h.kind == sqk::OP_PAULI && deferred) ? (cbig ? h.s / h.c : h.c / h.s) : 0.0;
    auto rot = [&](cplx a, cplx b, int k) -> cplx {
        const cplx ib = ipow(k) * b;
        if (deferred) return cbig ? a + u * ib : u * a + ib;
        return h.c * a + h.s * ib;
    };
    if (h.kind == sqk::OP_PHASE) {
        for (uint32_t j = 0; j < D; ++j)
            if ((deposit64(j, bm) & h.cmask) == h.cval) v[j] *= cplx(h.c, h.s);
        return;
    }
    if (h.kind == sqk::OP_PAULI && h.flip == 0ull) {  // all-Z string: diagonal
        for (uint32_t j = 0; j < D; ++j) {
            const uint64_t G = deposit64(j, bm);
            if (!deferred && (G & h.cmask) != h.cval) continue;
            v[j] = rot(v[j], v[j], (1 + 2 * (popc(G & h.zy) & 1)) & 3);
        }
        return;
    }
    const uint64_t low = h.flip & (~h.flip + 1ull);
    const int fz = popc(h.flip & h.zy) & 1;
    for (uint32_t j = 0; j < D; ++j) {
        const uint64_t G = deposit64(j, bm);
        if ((G & low) || (G & h.cmask) != h.cval) continue;
        const uint32_t j1 = extract64(G ^ h.flip, bm);
        const cplx a0 = v[j], a1 = v[j1];
        switch (h.kind) {
            case sqk::OP_SWAPP: v[j] = a1; v[j1] = a0; break;
            case sqk::OP_YP: v[j1] = I * a0; v[j] = -I * a1; break;
            case sqk::OP_HP:
                if (h.cmask == 0ull) {
                    v[j] = a0 + a1;
                    v[j1] = a0 - a1;
                } else {
                    v[j] = 0.7071067811865475 * (a0 + a1);
                    v[j1] = 0.7071067811865475 * (a0 - a1);
                }
                break;
            default: {  // OP_PAULI with X/Y factors
                const int pz0 = popc(G & h.zy) & 1;
                const int k1 = (1 + h.ny + 2 * pz0) & 3, k0 = (1 + h.ny + 2 * (pz0 ^ fz)) & 3;
                v[j] = rot(a0, a1, k0);
                v[j1] = rot(a1, a0, k1);
            }
        }
    }
}

// Replaces runs of at least min_weight fusable ops on at most five qubits by one
// dense op each (uncontrolled X gates weigh 0: the pass's index frame moves them
// for free).
std::vector<HostOp> fuse_dense(std::vector<HostOp>&& ops, int min_weight) {
    std::vector<HostOp> out;
    out.reserve(ops.size());
    size_t i = 0;
    auto weight = [](const HostOp& h) {
        return (h.kind == sqk::OP_SWAPP && h.cmask == 0ull && popc(h.flip) == 1) ? 0 : 1;
    };
    while (i < ops.size()) {
        if (!op_fusable(ops[i]) || popc(op_support(ops[i])) > sqk::kDenseQubits) {
            out.push_back(std::move(ops[i++]));
            continue;
        }
        uint64_t un = op_support(ops[i]);
        int w = weight(ops[i]);
        size_t j = i + 1;
        while (j < ops.size() && op_fusable(ops[j]) && popc(un | op_support(ops[j])) <= sqk::kDenseQubits) {
            un |= op_support(ops[j]);
            w += weight(ops[j]);
            ++j;
        }
        if (w >= min_weight && j - i >= 2) {
            const uint32_t D = 1u << popc(un);
            HostOp d;
            d.kind = sqk::OP_DENSE;
            d.flip = un;
            d.dense.assign(2 * (size_t)D * D, 0.0);
            std::vector<cplx> col(D);
            for (uint32_t c = 0; c < D; ++c) {
                std::fill(col.begin(), col.end(), cplx(0.0, 0.0));
                col[c] = 1.0;
                for (size_t k = i; k < j; ++k) apply_stored(ops[k], un, col);
                for (uint32_t r = 0; r < D; ++r) {
                    d.dense[2 * ((size_t)r * D + c)] = col[r].real();
                    d.dense[2 * ((size_t)r * D + c) + 1] = col[r].imag();
                }
            }
            out.push_back(std::move(d));
        } else {
            for (size_t k = i; k < j; ++k) out.push_back(std::move(ops[k]));
        }
        i = j;
    }
    return out;
}

// x rounded to TF32 (10 fraction bits, to nearest), as the kernel rounds its operand
float tf32_round_host(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b = (b + 0x1000u) & 0xFFFFE000u;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

// Writes one dense op's launch data into dst (kDenseBlockBytes): the op's matrix
// (on its k qubits, tile positions pos[0..k-1] ascending) extended by the identity
// to the five tile positions of bm5 (ascending), either as the tensor-core B
// operand (TF32 high and low parts, core-matrix layout) or as a 32 x 32 complex
// FP64 matrix for the CUDA-core path.
void write_dense_block(const HostOp& h, uint32_t opmask_local, uint32_t bm5, bool tc, unsigned char* dst) {
    const int k = popc(h.flip);
    const uint32_t Dk = 1u << k;
    // for each of the five block bits: which bit of the op's index it is, or -1
    int src[5];
    {
        int b = 0, ob = 0;
        for (uint32_t m = bm5; m; m &= m - 1u, ++b) {
            const uint32_t low = m & (~m + 1u);
            src[b] = (opmask_local & low) ? ob++ : -1;
        }
    }
    auto split = [&](uint32_t j5, uint32_t& jop, uint32_t& jx) {
        jop = 0;
        jx = 0;
        for (int b = 0; b < 5; ++b) {
            const uint32_t bit = (j5 >> b) & 1u;
            if (src[b] >= 0) jop |= bit << src[b];
            else jx |= bit << b;
        }
    };
    auto U5 = [&](uint32_t jo, uint32_t ji) -> cplx {
        uint32_t oo, ox, io, ix;
        split(jo, oo, ox);
        split(ji, io, ix);
        if (ox != ix) return cplx(0.0, 0.0);
        return cplx(h.dense[2 * ((size_t)oo * Dk + io)], h.dense[2 * ((size_t)oo * Dk + io) + 1]);
    };
    if (!tc) {
        double* out = reinterpret_cast<double*>(dst);
        for (uint32_t jo = 0; jo < 32; ++jo)
            for (uint32_t ji = 0; ji < 32; ++ji) {
                const cplx u = U5(jo, ji);
                out[2 * (jo * 32 + ji)] = u.real();
                out[2 * (jo * 32 + ji) + 1] = u.imag();
            }
        return;
    }
    float* hi = reinterpret_cast<float*>(dst);
    float* lo = hi + 4096;
    for (uint32_t n = 0; n < 64; ++n)
        for (uint32_t kk = 0; kk < 64; ++kk) {
            const cplx u = U5(n & 31u, kk & 31u);
            const int ro = (int)(n >> 5), ri = (int)(kk >> 5);
            // D[c][n] = sum_k A[c][k] B[k][n], A = (Re x, Im x), D = (Re y, Im y)
            const double val = (ro == 0) ? (ri == 0 ? u.real() : -u.imag()) : (ri == 0 ? u.imag() : u.real());
            const float fh = tf32_round_host((float)val);
            const size_t off = (size_t)(kk >> 3) * 512 + (n >> 3) * 64 + ((kk & 7) >> 2) * 32 + (n & 7) * 4 + (kk & 3);
            hi[off] = fh;
            lo[off] = tf32_round_host((float)(val - (double)fh));
        }
}

int ensure_dense_ring(sq_state* s) {
    if (s->dense_dev) return SQ_OK;
    const size_t bytes = (size_t)kDenseSlots * kMaxDensePerPass * kDenseBlockBytes;
    if (cudaMalloc(&s->dense_dev, bytes) != cudaSuccess || cudaMallocHost(&s->dense_host, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(SQ_ERR_NOMEM, "allocation of the dense-block buffers failed");
    }
    for (int i = 0; i < kDenseSlots; ++i) SQ_CUDA(cudaEventCreateWithFlags(&s->dense_ev[i], cudaEventDisableTiming));
    return SQ_OK;
}

// Whether a pass over ops[i0, i1) of an FP64 state runs the double-float kernel:
// the option is on, the pass is multi-tile (the tile size rule of run_pass) and
// holds no table ops (W, phase lists) or dense blocks.
bool pass_uses_df(const sq_state* s, const std::vector<HostOp>& ops, size_t i0, size_t i1) {
    if (s->prec != SQ_F64 || !s->dfloat) return false;
    const int n = (int)s->n;
    uint64_t need = 0;
    for (size_t i = i0; i < i1; ++i) {
        const uint8_t k = ops[i].kind;
        if (k == sqk::OP_DENSE || k == sqk::OP_W || k == sqk::OP_PLIST) return false;
        need |= ops[i].flip;
    }
    int K = s->kp;
    const int needbits = popc(need | 3ull);
    if (n > small_max(s) && needbits > K) K = needbits;
    if (s->staging == 2 && n > small_max(s)) K = std::max(needbits, 11);
    if (K > n) K = n;
    return K != n;
}

// Executes ops[i0, i1) as one pass, with an optional reduction at its end.
// df_in / df_out: the state holds double-float pairs before / after the pass
// (consecutive double-float passes of one flush, see flush()).
int run_pass(sq_state* s, const std::vector<HostOp>& ops, size_t i0, size_t i1, int red, uint64_t rmask,
             uint64_t rval, int df_in = 0, int df_out = 0) {
    const int n = (int)s->n;
    uint64_t need = 0;
    int ndense = 0;
    for (size_t i = i0; i < i1; ++i) {
        need |= ops[i].flip;
        if (ops[i].kind == sqk::OP_DENSE) ++ndense;
    }
    int K = s->kp;
    const int needbits = popc(need | 3ull);
    if ((int)s->n > small_max(s) && needbits > K) K = needbits;
    // dense blocks: FP32 tiles of 2^12 amplitudes (two CTAs per SM with the
    // tensor-core operands); FP64 (CUDA-core path, with a scratch copy of the
    // tile) at most 2^12
    if (ndense && (int)s->n > small_max(s)) K = std::max(needbits, 12);
    // double-buffered staging holds two tiles: 2^12 amplitudes (FP32) or 2^11 (FP64)
    // keep three CTAs per SM
    const bool dbuf = s->staging == 2 && !ndense && (int)s->n > small_max(s);
    if (dbuf) K = std::max(needbits, s->prec == SQ_F64 ? 11 : 12);
    if (K > n) K = n;
    if (K > tile_cap(s)) return fail(SQ_ERR_UNSUPPORTED, "gate touches too many qubits for one tile");
    if (ndense && s->prec == SQ_F64 && K > 12)
        return fail(SQ_ERR_UNSUPPORTED, "dense block in a pass whose tile exceeds 12 qubits (FP64)");
    if (ndense && K < sqk::kDenseQubits) return fail(SQ_ERR_UNSUPPORTED, "dense blocks need states of 5 qubits or more");
    const bool dense_tc = ndense && s->prec == SQ_F32 && K >= 12 && s->dense_engine == 0;
    // contiguous low block L, then the high tile qubits
    int L = K;
    while (L > 0 && L + popc(L >= 64 ? 0 : (need >> L)) > K) --L;
    uint64_t high = (L >= 64) ? 0 : (need & ~((1ull << L) - 1ull));
    for (int b = L; b < n && L + popc(high) < K; ++b)
        if (!((high >> b) & 1ull)) high |= 1ull << b;
    const uint64_t lowm = (L == 0) ? 0ull : ((1ull << L) - 1ull);
    const uint64_t tilemask = lowm | high;
    const uint64_t all = (n == 64) ? ~0ull : ((1ull << n) - 1ull);
    const uint64_t outer = all & ~tilemask;

    sqk::PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.re = s->data;
    a.im = (char*)s->data + s->N * s->esz;
    a.K = K;
    a.L = L;
    a.store = (i1 > i0) ? 1 : 0;
    a.partials = s->d_partials;
    a.result = s->d_result;
    a.result_host = s->h_result_dev;
    a.ticket = s->d_ticket;
    a.err = reinterpret_cast<unsigned int*>(s->d_result + 3);
    // bulk staging for multi-tile passes whose runs are whole 16-byte units of at
    // least 128 bytes (shorter runs cost more per copy than they save)
    {
        const uint64_t rb = ((uint64_t)1 << L) * s->esz;
        const bool ok = K < n && rb % 16 == 0 && rb >= 128;
        a.stage = !ok ? 0 : (dbuf ? 2 : (s->staging ? 1 : 0));
    }
    int nhb = 0;
    for (int b = L; b < n; ++b)
        if ((high >> b) & 1ull) a.hb[nhb++] = (uint8_t)b;
    // tile-local position of a global bit
    auto local_of = [&](int b) -> int {
        if (b < L) return b;
        for (int j = 0; j < nhb; ++j)
            if (a.hb[j] == b) return L + j;
        return -1;
    };

    // outer qubits every op of the pass requires at one value: the grid skips the rest
    // (not when the pass changes the storage format: every tile is converted)
    uint64_t fixm = 0, fixv = 0;
    if (!red && i1 > i0 && df_in == df_out) {
        fixm = outer;
        for (size_t i = i0; i < i1; ++i) fixm &= ops[i].skm;
        for (size_t i = i0 + 1; i < i1; ++i) fixm &= ~(ops[i].skv ^ ops[i0].skv);
        fixv = ops[i0].skv & fixm;
    }
    a.ofix = fixv;
    a.ofree = outer & ~fixm;
    a.ntiles = 1ull << popc(a.ofree);

    static thread_local sqk::Prog p;
    p.nops = 0;
    p.red = red;
    p.defer = 0;
    p.rmask = rmask;
    p.rval = rval;
    p.lrm = p.lrv = 0u;
    for (int b = 0; b < n; ++b) {
        const int lb = ((rmask >> b) & 1ull) ? local_of(b) : -1;
        if (lb < 0) continue;
        p.lrm |= 1u << lb;
        if ((rval >> b) & 1ull) p.lrv |= 1u << lb;
    }
    p.orm = rmask & outer;
    p.orv = rval & p.orm;
    // Index frame: an uncontrolled X on one tile qubit moves no data.  The pass
    // records it in xm (physical element t holds logical t ^ xm), later ops are
    // rewritten for the frame (control values, H / Y pair roles, Pauli sign
    // parity, collapse and reduction conditions) and the store writes every
    // element back to its logical position.  Passes with table ops (W, phase
    // lists: index-valued lookups) keep xm = 0.
    bool frame_ok = ndense == 0;  // dense blocks read the tile in logical order
    for (size_t i = i0; i < i1; ++i)
        if (ops[i].kind == sqk::OP_W || ops[i].kind == sqk::OP_PLIST) frame_ok = false;
    unsigned char* dslot = nullptr;
    int dslot_i = -1;
    int dcount = 0;
    if (ndense) {
        int rc = ensure_dense_ring(s);
        if (rc) return rc;
        dslot_i = (int)(s->dense_slot++ % kDenseSlots);
        if (s->dense_ev_used[dslot_i]) SQ_CUDA(cudaEventSynchronize(s->dense_ev[dslot_i]));  // its last launch is done
        dslot = static_cast<unsigned char*>(s->dense_host) + (size_t)dslot_i * kMaxDensePerPass * kDenseBlockBytes;
    }
    uint32_t xm = 0;       // tile-local frame
    uint64_t xg = 0;       // the same in global qubit positions
    uint32_t tabpos = 0;
    for (size_t i = i0; i < i1; ++i) {
        const HostOp& h = ops[i];
        if (frame_ok && h.kind == sqk::OP_SWAPP && h.cmask == 0ull && popc(h.flip) == 1) {
            const int lb = local_of(__builtin_ctzll(h.flip));
            if (lb < 0) return fail(SQ_ERR_UNSUPPORTED, "internal: gate qubit outside the pass tile");
            xm ^= 1u << lb;
            xg ^= h.flip;
            continue;
        }
        sqk::Op& o = p.ops[p.nops++];
        std::memset(&o, 0, sizeof(o));
        o.kind = h.kind;
        o.ny = h.ny;
        o.fz = (uint8_t)(popc(h.flip & h.zy) & 1);
        uint32_t lf = 0;
        for (int b = 0; b < n; ++b) {
            if (!((h.flip >> b) & 1ull)) continue;
            const int lb = local_of(b);
            if (lb < 0) return fail(SQ_ERR_UNSUPPORTED, "internal: gate qubit outside the pass tile");
            lf |= 1u << lb;
        }
        o.lflip = lf;
        o.lpair = (uint8_t)(lf ? __builtin_ctz(lf) : 0);
        uint32_t lcm = 0, lcv = 0, lzy = 0;
        for (int b = 0; b < n; ++b) {
            const int lb = local_of(b);
            if (lb < 0) continue;
            if ((h.cmask >> b) & 1ull) {
                lcm |= 1u << lb;
                if ((h.cval >> b) & 1ull) lcv |= 1u << lb;
            }
            if ((h.zy >> b) & 1ull) lzy |= 1u << lb;
        }
        o.lcm = lcm;
        // the pair's first physical element is the logical second one when the
        // frame flips the pair bit; a control bit inside the flip (SWAP) then flips too
        o.orient = (uint8_t)(lf ? ((xm >> o.lpair) & 1u) : 0u);
        o.lcv = lcv ^ (xm & lcm) ^ (o.orient ? (lf & lcm) : 0u);
        o.gdefer = h.gdefer;
        if ((h.kind == sqk::OP_HP || h.kind == sqk::OP_PAULI) && lcm == 0u && !h.gdefer) p.defer++;
        o.lzy = (h.kind == sqk::OP_PAULI) ? lzy : 0u;
        o.cmask = h.cmask;
        o.cval = h.cval ^ (xg & h.cmask);
        o.ocm = h.skm & outer;
        o.ocv = h.skv & o.ocm;
        // Pauli: the kernel takes the outer part of the sign parity per tile
        o.zy = (h.kind == sqk::OP_PAULI) ? (h.zy & outer) : h.zy;
        o.shift = h.shift;
        o.c = h.c;
        o.s = h.s;
        o.sn = -h.s;
        // deferred rotations store a + (s/c) iP a (|c| >= |s|) or (c/s) a + iP a
        o.cbig = std::fabs(h.c) >= std::fabs(h.s) ? 1 : 0;
        if (h.kind == sqk::OP_PAULI) o.u = o.cbig ? h.s / h.c : h.c / h.s;
        o.un = -o.u;
        o.fc = (float)o.c;
        o.fs = (float)o.s;
        o.fsn = (float)o.sn;
        o.fu = (float)o.u;
        o.fun = (float)o.un;
        o.dc = sqk::df_const_host(o.c);
        o.ds = sqk::df_const_host(o.s);
        o.dsn = sqk::df_const_host(o.sn);
        o.du = sqk::df_const_host(o.u);
        o.dun = sqk::df_const_host(o.un);
        o.xpar = (uint8_t)(h.kind == sqk::OP_PAULI ? (popc(xm & o.lzy) & 1) : 0);
        if (!h.tab.empty()) {
            o.tab = tabpos;
            std::memcpy(&p.tab[2 * tabpos], h.tab.data(), h.tab.size() * sizeof(double));
            tabpos += (uint32_t)(h.tab.size() / 2);
        }
        if (h.kind == sqk::OP_DENSE) {
            // extend the op's qubits to five tile bits with the lowest free ones
            uint32_t bm5 = lf;
            for (int b = 0; b < K && popc(bm5) < sqk::kDenseQubits; ++b)
                if (!((bm5 | lcm) >> b & 1u)) bm5 |= 1u << b;
            if (popc(bm5) != sqk::kDenseQubits) return fail(SQ_ERR_UNSUPPORTED, "no room for a dense block in the tile");
            o.lflip = bm5;
            o.tab = (uint32_t)dcount;
            write_dense_block(h, lf, bm5, dense_tc, dslot + (size_t)dcount * kDenseBlockBytes);
            ++dcount;
        }
    }

    p.xm = xm;
    p.ndense = dcount;
    p.rswap = (red == 1 && (xm & p.lrm)) ? 1 : 0;
    if (red == 2) p.lrv ^= xm & p.lrm;
    p.defer = p.defer >= 2 ? 1 : 0;  // deferring one factor costs as much as it saves
    const bool single = (K == n);
    // multi-tile passes with tensor-core dense blocks run one CTA per SM (a kernel
    // holding TMEM gets one), so they take 512 threads
    const int block = single ? (K >= 10 ? 1024 : (K >= 8 ? 256 : 128))
                             : ((ndense && s->prec == SQ_F32 && K >= 12 && s->dense_engine == 0) ? 512 : 256);
    // double-float arithmetic: FP64 multi-tile passes without tables or dense blocks
    const bool use_df = pass_uses_df(s, ops, i0, i1);
    if (use_df && single) return fail(SQ_ERR_UNSUPPORTED, "internal: double-float pass on a single tile");
    if ((df_in || df_out) && !use_df) return fail(SQ_ERR_UNSUPPORTED, "internal: double-float format on an FP64 pass");
    a.df_in = df_in;
    a.df_out = df_out;
    if (use_df) a.stage = 0;  // the tile is converted on its way in and out
    if (dcount) a.stage = 0;  // dense passes stage through registers (no bulk part in their kernels)
    size_t smem = tile_smem(s, K, L) + (a.stage == 2 ? (size_t)2 * ((size_t)1 << K) * s->esz : 0);
    if (dcount) {
        // the dense work area: tensor-core operands (A chunk + B), or the scratch tile
        a.dense_off = (uint32_t)((smem + 127) & ~(size_t)127);
        smem = a.dense_off + (dense_tc ? (size_t)2 * 32768 : (size_t)2 * ((size_t)1 << K) * s->esz);
        a.dense_tc = dense_tc ? 1 : 0;
        const size_t bytes = (size_t)dcount * kDenseBlockBytes;
        void* dev = static_cast<unsigned char*>(s->dense_dev) + (size_t)dslot_i * kMaxDensePerPass * kDenseBlockBytes;
        SQ_CUDA(cudaMemcpyAsync(dev, dslot, bytes, cudaMemcpyHostToDevice, s->stream));
        a.dense = dev;
    }
    int occ = 0;
    const bool bulk = a.stage != 0;
    {
        const int orc = with_pass_kernel(s, use_df, single, dcount > 0, dense_tc, bulk, [&](auto tag) {
            return resident_ctas<decltype(tag)>(s, block, smem, &occ);
        });
        if (orc) return orc;
    }
    const uint64_t wave = occ > 0 ? (uint64_t)s->nsm * (uint64_t)occ : (uint64_t)s->max_grid;
    int grid = (int)std::min<uint64_t>(a.ntiles, std::min<uint64_t>(wave, (uint64_t)s->max_grid));
    if (grid < 1) grid = 1;
    const uint64_t moved = a.ntiles * ((uint64_t)1 << K) * 2ull * s->esz * (a.store ? 2ull : 1ull);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (s->timing) {
        for (cudaEvent_t* e : {&e0, &e1}) {
            if (s->ev_pool.empty()) {
                SQ_CUDA(cudaEventCreate(e));
            } else {
                *e = s->ev_pool.back();
                s->ev_pool.pop_back();
            }
        }
        SQ_CUDA(cudaEventRecord(e0, s->stream));
    }
    const int rc = with_pass_kernel(s, use_df, single, dcount > 0, dense_tc, bulk, [&](auto tag) {
        return launch_pass_t<decltype(tag)>(s, a, p, grid, block, smem);
    });
    if (rc) return rc;
    if (dcount) {
        SQ_CUDA(cudaEventRecord(s->dense_ev[dslot_i], s->stream));
        s->dense_ev_used[dslot_i] = true;
    }
    if (s->timing) {
        SQ_CUDA(cudaEventRecord(e1, s->stream));
        s->ev_open.push_back({e0, e1});
        s->ev_bytes.push_back(moved);
    }
    // algorithmic flops: per amplitude the gate touches (tiles enumerated x 2^K x fraction)
    {
        const double amps = (double)a.ntiles * (double)((uint64_t)1 << K);
        double fl = 0.0;
        for (size_t i = i0; i < i1; ++i) {
            const HostOp& h = ops[i];
            const double frac = 1.0 / (double)(1ull << popc(h.cmask & ~h.flip));
            switch (h.kind) {
                case sqk::OP_HP: fl += 4.0 * amps * frac; break;
                case sqk::OP_PAULI: fl += 6.0 * amps * frac; break;
                case sqk::OP_PHASE: fl += 6.0 * amps * frac; break;
                case sqk::OP_PLIST: fl += 6.0 * amps; break;
                case sqk::OP_W: fl += 6.0 * amps; break;
                case sqk::OP_COLLAPSE: case sqk::OP_SCALE: fl += 2.0 * amps; break;
                case sqk::OP_DENSE: fl += 8.0 * sqk::kDenseDim * amps; break;  // 32 complex MACs per amplitude
                default: break;
            }
        }
        if (red) fl += 4.0 * amps;
        s->stats.flops += (uint64_t)fl;
    }
    s->stats.passes++;
    s->stats.launches++;
    s->stats.bytes_moved += moved;
    if (red) s->stats.reductions++;
    return SQ_OK;
}

// The kernels' error word (d_result[3], copied with a reduction's result into
// h_result[3]): a bounded wait inside a pass that gave up.
int device_error(sq_state* s) {
    unsigned int e = 0;
    const volatile double* h = s->h_result;
    const double w = h[3];
    std::memcpy(&e, &w, sizeof(e));
    if (e == 0u) return SQ_OK;
    return fail(SQ_ERR_CUDA, "a pass kernel gave up waiting for its tile copies (error word " + std::to_string(e) + ")");
}

// Applies every queued op; with red != 0 the last pass also reduces and the
// result is copied into s->h_result (synchronously).
int flush(sq_state* s, int red = 0, uint64_t rmask = 0, uint64_t rval = 0) {
    std::vector<HostOp> ops;
    ops.swap(s->pending);
    if (s->dense_fusion > 0 && s->prec == SQ_F32 && s->n >= (uint32_t)sqk::kDenseQubits && !ops.empty())
        ops = fuse_dense(std::move(ops), s->dense_fusion);
    size_t i = 0;
    const int kcap = ((int)s->n <= small_max(s)) ? (int)s->n : std::max(s->kp, std::min(tile_cap(s), (int)s->n));
    std::vector<std::pair<size_t, size_t>> ranges;
    while (i < ops.size()) {
        size_t j = i;
        uint64_t need = 0;
        uint32_t tab = 0;
        int nd = 0;
        while (j < ops.size()) {
            const HostOp& h = ops[j];
            if (h.kind == sqk::OP_DENSE && nd == kMaxDensePerPass) break;
            const uint64_t nn = need | h.flip;
            const int bits = popc(nn | 3ull);
            // passes with dense blocks keep to tiles of 2^12 amplitudes (two CTAs per SM
            // with the tensor-core operands)
            const int cap = (nd > 0 || h.kind == sqk::OP_DENSE) ? std::min(s->kp, 12) : s->kp;
            const bool fits_tile = ((int)s->n <= small_max(s)) ? true : (bits <= cap || (j == i && bits <= kcap));
            if (j > i && (!s->fusion || !fits_tile)) break;
            if (j == i && !fits_tile) return fail(SQ_ERR_UNSUPPORTED, "gate touches too many qubits for one tile");
            if ((int)(j - i) >= sqk::kMaxOps) break;
            if (tab + h.tab.size() / 2 > (size_t)sqk::kMaxTab) break;
            need = nn;
            tab += (uint32_t)(h.tab.size() / 2);
            if (h.kind == sqk::OP_DENSE) ++nd;
            ++j;
        }
        ranges.emplace_back(i, j);
        i = j;
    }
    // Consecutive double-float passes hand the state on as hi/lo FP32 pairs (the
    // same 8 bytes per component): only the first converts from doubles and only
    // the last converts back, so between flushes the state is always IEEE doubles.
    std::vector<char> df(ranges.size());
    for (size_t r = 0; r < ranges.size(); ++r) df[r] = pass_uses_df(s, ops, ranges[r].first, ranges[r].second);
    for (size_t r = 0; r < ranges.size(); ++r) {
        const bool last = (r + 1 == ranges.size());
        const int din = (r > 0 && df[r] && df[r - 1]) ? 1 : 0;
        const int dout = (!last && df[r] && df[r + 1]) ? 1 : 0;
        int rc = run_pass(s, ops, ranges[r].first, ranges[r].second, last ? red : 0, rmask, rval, din, dout);
        if (rc) return rc;
    }
    if (ops.empty() && red) {
        int rc = run_pass(s, ops, 0, 0, red, rmask, rval);
        if (rc) return rc;
    }
    if (red) {
        // the reduction's last CTA wrote the mapped copy; without a mapping, copy it
        if (!s->h_result_dev)
            SQ_CUDA(cudaMemcpyAsync(s->h_result, s->d_result, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        SQ_CUDA(cudaStreamSynchronize(s->stream));
        int rc = device_error(s);
        if (rc) return rc;
    }
    return SQ_OK;
}

int enqueue(sq_state* s, HostOp&& h) {
    s->pending.push_back(std::move(h));
    s->stats.gates++;
    if (s->pending.size() >= 4096) return flush(s);
    return SQ_OK;
}

// Applies the global scale to memory (as one scale op, fused into the next pass).
int materialize(sq_state* s) {
    if (s->gscale == 1.0) return SQ_OK;
    HostOp h;
    h.kind = sqk::OP_SCALE;
    h.s = s->gscale;
    s->gscale = 1.0;
    s->pending.push_back(std::move(h));
    if (s->pending.size() >= 4096) return flush(s);
    return SQ_OK;
}

// Multiplies the global scale by f; keeps the stored amplitudes in range (FP32
// has an 8-bit exponent) by materialising it when it leaves [2^-lim, 2^lim].
int scale_by(sq_state* s, double f) {
    s->gscale *= f;
    // stored amplitudes stay within the FP32 exponent range in FP32 and double-float modes
    const double lim = (s->prec == SQ_F64 && !s->dfloat) ? 300.0 : 40.0;
    const double e = std::fabs(std::log2(std::fabs(s->gscale)));
    if (e > lim) return materialize(s);
    return SQ_OK;
}

int check_q(const sq_state* s, uint32_t q) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (q >= s->n) return fail(SQ_ERR_ARG, "qubit index out of range");
    return SQ_OK;
}

int check_mask(const sq_state* s, uint64_t m) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (s->n < 64 && (m >> s->n)) return fail(SQ_ERR_ARG, "mask has bits beyond the register");
    return SQ_OK;
}

}  // namespace

extern "C" {

const char* sq_last_error(void) { return g_err.c_str(); }
const char* sq_version(void) { return "libsq 0.1 (sm_103a)"; }

int sq_state_create(sq_state** out, uint32_t n, int precision) {
    if (!out) return fail(SQ_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (n < 1 || n > 33) return fail(SQ_ERR_ARG, "qubit count must be in 1..33");
    if (precision != SQ_F64 && precision != SQ_F32) return fail(SQ_ERR_ARG, "unknown precision");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(SQ_ERR_NODEVICE, "no CUDA device");
    sq_state* s = new sq_state();
    s->n = n;
    s->prec = precision;
    s->esz = precision == SQ_F64 ? 8 : 4;
    s->N = 1ull << n;
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, s->device);
    s->max_grid = s->nsm * 8;
    s->kp = default_tile(s);
    size_t bytes = 2 * s->N * s->esz;
    if (cudaMalloc(&s->data, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return fail(SQ_ERR_NOMEM, "device allocation of the state failed");
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&s->d_partials, sizeof(double) * 2 * (size_t)s->max_grid) != cudaSuccess ||
        cudaMalloc(&s->d_result, sizeof(double) * 4) != cudaSuccess ||
        cudaMalloc(&s->d_ticket, sizeof(unsigned int)) != cudaSuccess ||
        cudaHostAlloc(reinterpret_cast<void**>(&s->h_result), sizeof(double) * 4, cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        sq_state_destroy(s);
        return fail(SQ_ERR_NOMEM, "allocation of work buffers failed");
    }
    {
        int can_map = 0;
        void* dptr = nullptr;
        if (cudaDeviceGetAttribute(&can_map, cudaDevAttrCanMapHostMemory, s->device) == cudaSuccess && can_map &&
            cudaHostGetDevicePointer(&dptr, s->h_result, 0) == cudaSuccess)
            s->h_result_dev = static_cast<double*>(dptr);
        cudaGetLastError();  // without a mapping the results come back by copy
    }
    s->own_stream = true;
    cudaMemsetAsync(s->d_ticket, 0, sizeof(unsigned int), s->stream);
    cudaMemsetAsync(s->d_result, 0, 4 * sizeof(double), s->stream);
    std::memset(s->h_result, 0, 4 * sizeof(double));
    int rc = sq_init_state(s);
    if (rc) {
        sq_state_destroy(s);
        return rc;
    }
    *out = s;
    return SQ_OK;
}

int sq_state_destroy(sq_state* s) {
    if (!s) return SQ_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto& pr : s->ev_open) {
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    for (auto e : s->ev_pool) cudaEventDestroy(e);
    if (s->data) cudaFree(s->data);
    if (s->d_partials) cudaFree(s->d_partials);
    if (s->d_result) cudaFree(s->d_result);
    if (s->d_ticket) cudaFree(s->d_ticket);
    if (s->h_result) cudaFreeHost(s->h_result);
    for (auto e : s->dense_ev)
        if (e) cudaEventDestroy(e);
    if (s->dense_dev) cudaFree(s->dense_dev);
    if (s->dense_host) cudaFreeHost(s->dense_host);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SQ_OK;
}

int sq_state_ptrs(sq_state* s, void** re, void** im) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = materialize(s);
    if (!rc) rc = flush(s);
    if (rc) return rc;
    if (re) *re = s->data;
    if (im) *im = (char*)s->data + s->N * s->esz;
    return SQ_OK;
}

int sq_state_nqubits(const sq_state* s, uint32_t* n, int* precision) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (n) *n = s->n;
    if (precision) *precision = s->prec;
    return SQ_OK;
}

int sq_set_stream(sq_state* s, void* stream) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = flush(s);
    if (rc) return rc;
    SQ_CUDA(cudaStreamSynchronize(s->stream));
    if (s->own_stream) cudaStreamDestroy(s->stream);
    if (stream) {
        s->stream = (cudaStream_t)stream;
        s->own_stream = false;
    } else {
        SQ_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    return SQ_OK;
}

int sq_flush(sq_state* s) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    return flush(s);
}

int sq_synchronize(sq_state* s) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = flush(s);
    if (rc) return rc;
    SQ_CUDA(cudaMemcpyAsync(&s->h_result[3], s->d_result + 3, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    SQ_CUDA(cudaStreamSynchronize(s->stream));
    return device_error(s);
}

int sq_set_fusion(sq_state* s, int enabled) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = flush(s);
    s->fusion = enabled ? 1 : 0;
    return rc;
}

int sq_set_staging(sq_state* s, int mode) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (mode < 0 || mode > 2)
        return fail(SQ_ERR_ARG, "staging mode must be 0 (registers), 1 (bulk copies) or 2 (bulk, double-buffered)");
    int rc = flush(s);
    s->staging = mode;
    return rc;
}

int sq_set_tile_qubits(sq_state* s, int k) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (k != 0 && (k < 6 || k > tile_cap(s))) return fail(SQ_ERR_ARG, "tile qubits out of range (0, or 6..tile cap)");
    int rc = flush(s);
    s->kp = k ? std::min(k, (int)s->n) : default_tile(s);
    if ((int)s->n <= small_max(s)) s->kp = (int)s->n;  // small states run as one tile
    return rc;
}

int sq_get_state(sq_state* s, double* re, double* im) {
    if (!s || !re || !im) return fail(SQ_ERR_ARG, "null argument");
    int rc = materialize(s);
    if (!rc) rc = flush(s);
    if (rc) return rc;
    if (s->prec == SQ_F64) {
        SQ_CUDA(cudaMemcpyAsync(re, s->data, s->N * 8, cudaMemcpyDeviceToHost, s->stream));
        SQ_CUDA(cudaMemcpyAsync(im, (char*)s->data + s->N * 8, s->N * 8, cudaMemcpyDeviceToHost, s->stream));
        SQ_CUDA(cudaStreamSynchronize(s->stream));
    } else {
        std::vector<float> tmp(2 * s->N);
        SQ_CUDA(cudaMemcpyAsync(tmp.data(), s->data, 2 * s->N * 4, cudaMemcpyDeviceToHost, s->stream));
        SQ_CUDA(cudaStreamSynchronize(s->stream));
        for (uint64_t i = 0; i < s->N; ++i) {
            re[i] = tmp[i];
            im[i] = tmp[s->N + i];
        }
    }
    return SQ_OK;
}

int sq_set_state(sq_state* s, const double* re, const double* im) {
    if (!s || !re || !im) return fail(SQ_ERR_ARG, "null argument");
    s->pending.clear();
    s->gscale = 1.0;
    if (s->prec == SQ_F64) {
        SQ_CUDA(cudaMemcpyAsync(s->data, re, s->N * 8, cudaMemcpyHostToDevice, s->stream));
        SQ_CUDA(cudaMemcpyAsync((char*)s->data + s->N * 8, im, s->N * 8, cudaMemcpyHostToDevice, s->stream));
        SQ_CUDA(cudaStreamSynchronize(s->stream));
    } else {
        std::vector<float> tmp(2 * s->N);
        for (uint64_t i = 0; i < s->N; ++i) {
            tmp[i] = (float)re[i];
            tmp[s->N + i] = (float)im[i];
        }
        SQ_CUDA(cudaMemcpyAsync(s->data, tmp.data(), 2 * s->N * 4, cudaMemcpyHostToDevice, s->stream));
        SQ_CUDA(cudaStreamSynchronize(s->stream));
    }
    return SQ_OK;
}

int sq_upload(sq_state* s, const void* re, const void* im) {
    if (!s || !re || !im) return fail(SQ_ERR_ARG, "null argument");
    s->pending.clear();
    s->gscale = 1.0;
    const size_t b = s->N * s->esz;
    SQ_CUDA(cudaMemcpyAsync(s->data, re, b, cudaMemcpyHostToDevice, s->stream));
    SQ_CUDA(cudaMemcpyAsync((char*)s->data + b, im, b, cudaMemcpyHostToDevice, s->stream));
    return SQ_OK;
}

int sq_download(sq_state* s, void* re, void* im) {
    if (!s || !re || !im) return fail(SQ_ERR_ARG, "null argument");
    int rc = materialize(s);
    if (!rc) rc = flush(s);
    if (rc) return rc;
    const size_t b = s->N * s->esz;
    SQ_CUDA(cudaMemcpyAsync(re, s->data, b, cudaMemcpyDeviceToHost, s->stream));
    SQ_CUDA(cudaMemcpyAsync(im, (char*)s->data + b, b, cudaMemcpyDeviceToHost, s->stream));
    SQ_CUDA(cudaStreamSynchronize(s->stream));
    return SQ_OK;
}

int sq_init_state(sq_state* s) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    s->pending.clear();
    s->gscale = 1.0;
    SQ_CUDA(cudaMemsetAsync(s->data, 0, 2 * s->N * s->esz, s->stream));
    if (s->prec == SQ_F64) {
        const double one = 1.0;
        SQ_CUDA(cudaMemcpyAsync(s->data, &one, 8, cudaMemcpyHostToDevice, s->stream));
    } else {
        const float one = 1.0f;
        SQ_CUDA(cudaMemcpyAsync(s->data, &one, 4, cudaMemcpyHostToDevice, s->stream));
    }
    SQ_CUDA(cudaStreamSynchronize(s->stream));
    return SQ_OK;
}

int sq_vnorm(sq_state* s, double* norm) {
    if (!s || !norm) return fail(SQ_ERR_ARG, "null argument");
    int rc = flush(s, 2, 0, 0);
    if (rc) return rc;
    *norm = std::sqrt(s->h_result[0]) * std::fabs(s->gscale);
    return SQ_OK;
}

int sq_vnormalize(sq_state* s) {
    double nrm = 0.0;
    int rc = sq_vnorm(s, &nrm);
    if (rc) return rc;
    s->stats.gates++;
    return scale_by(s, 1. / nrm);  // src/suqa.cu:105: multiply by 1./norm
}

// A global control mask may contain the gate's own qubits (the reference's QSA
// does this through aliased registers).  The reference loops then have definite
// semantics, reproduced here: X and Y act on the pair controlled by the other
// gc bits (include/suqa_cpu.hpp:69-122), H zeroes the amplitudes where every gc
// bit is set (its two output writes alias, :150-206).
static int pair_op(sq_state* s, uint8_t kind, uint32_t q, uint64_t gc) {
    int rc = check_q(s, q);
    if (rc || (rc = check_mask(s, gc))) return rc;
    const uint64_t b = 1ull << q;
    HostOp h;
    if ((gc & b) && kind == sqk::OP_HP) {
        h.kind = sqk::OP_PHASE;  // multiply by 0 + 0i
        h.cmask = gc;
        h.cval = gc;
        h.skm = gc;
        h.skv = gc;
        return enqueue(s, std::move(h));
    }
    const uint64_t g = gc & ~b;
    h.kind = kind;
    h.flip = b;
    h.cmask = g;
    h.cval = g;
    h.skm = g;
    h.skv = g;
    const bool defer = kind == sqk::OP_HP && g == 0;  // uncontrolled H: 1/sqrt(2) into the global scale
    h.gdefer = defer ? 1 : 0;
    rc = enqueue(s, std::move(h));
    if (rc || !defer) return rc;
    return scale_by(s, 0.7071067811865475);
}

int sq_apply_x(sq_state* s, uint32_t q, uint64_t gc) { return pair_op(s, sqk::OP_SWAPP, q, gc); }
int sq_apply_y(sq_state* s, uint32_t q, uint64_t gc) { return pair_op(s, sqk::OP_YP, q, gc); }
int sq_apply_h(sq_state* s, uint32_t q, uint64_t gc) { return pair_op(s, sqk::OP_HP, q, gc); }

static int phase_op(sq_state* s, uint64_t cmask, uint64_t cval, double c, double sn) {
    HostOp h;
    h.kind = sqk::OP_PHASE;
    h.cmask = cmask;
    h.cval = cval;
    h.skm = cmask;
    h.skv = cval;
    h.c = c;
    h.s = sn;
    return enqueue(s, std::move(h));
}

int sq_apply_u1(sq_state* s, uint32_t q, uint32_t q_mask, double phase, uint64_t gc) {
    int rc = check_q(s, q);
    if (rc || (rc = check_mask(s, gc))) return rc;
    const uint64_t b = 1ull << q;
    // src/suqa.cu:271-285: condition (i & (gc | 1<<q)) == gc | (q_mask << q)
    HostOp h;
    h.kind = sqk::OP_PHASE;
    h.cmask = gc | b;
    h.cval = gc | ((uint64_t)(q_mask & 1u) << q);
    h.skm = h.cmask;
    h.skv = h.cval;
    sincos(phase, &h.s, &h.c);
    return enqueue(s, std::move(h));
}

int sq_apply_mcx(sq_state* s, uint64_t control_mask, uint64_t mask_qs, uint32_t q_target) {
    int rc = check_q(s, q_target);
    if (rc || (rc = check_mask(s, control_mask)) || (rc = check_mask(s, mask_qs))) return rc;
    const uint64_t b = 1ull << q_target;
    if (mask_qs & ~control_mask) return fail(SQ_ERR_ARG, "mask_qs has bits outside control_mask");
    // the reference adds the target bit to both masks (include/suqa_cpu.hpp:237-238) and
    // tests the element with the target set; on the pair's lower element that is the
    // condition without the target bit
    HostOp h;
    h.kind = sqk::OP_SWAPP;
    h.flip = b;
    h.cmask = control_mask & ~b;
    h.cval = mask_qs & ~b;
    h.skm = h.cmask;
    h.skv = h.cval;
    return enqueue(s, std::move(h));
}

int sq_apply_mcu1(sq_state* s, uint64_t control_mask, uint64_t mask_qs, double phase) {
    int rc = check_mask(s, control_mask);
    if (rc || (rc = check_mask(s, mask_qs))) return rc;
    if (mask_qs & ~control_mask) return fail(SQ_ERR_ARG, "mask_qs has bits outside control_mask");
    HostOp h;
    h.kind = sqk::OP_PHASE;
    h.cmask = control_mask;
    h.cval = mask_qs;
    h.skm = control_mask;
    h.skv = mask_qs;
    sincos(phase, &h.s, &h.c);
    return enqueue(s, std::move(h));
}

int sq_apply_swap(sq_state* s, uint32_t q1, uint32_t q2, uint64_t gc) {
    int rc = check_q(s, q1);
    if (rc || (rc = check_q(s, q2)) || (rc = check_mask(s, gc))) return rc;
    if (q1 == q2) return fail(SQ_ERR_ARG, "swap of a qubit with itself");
    const uint64_t b1 = 1ull << q1, b2 = 1ull << q2;
    HostOp h;
    if (gc & (b1 | b2)) {
        // reference loop (include/suqa_cpu.hpp:299-311) with a swapped qubit inside gc:
        // it exchanges the other qubit where every gc bit is set; both inside: nothing
        const uint64_t freeb = (b1 | b2) & ~gc;
        if (!freeb) {
            s->stats.gates++;
            return SQ_OK;
        }
        h.kind = sqk::OP_SWAPP;
        h.flip = freeb;
        h.cmask = gc;
        h.cval = gc;
        h.skm = gc;
        h.skv = gc;
        return enqueue(s, std::move(h));
    }
    // pairs (i|b1, i|b2) for (i & (gc|b1|b2)) == gc: the pair's lower-bit element has
    // the higher bit set
    const uint64_t bhi = b1 > b2 ? b1 : b2;
    h.kind = sqk::OP_SWAPP;
    h.flip = b1 | b2;
    h.cmask = gc | bhi;
    h.cval = gc | bhi;
    h.skm = gc;
    h.skv = gc;
    return enqueue(s, std::move(h));
}

int sq_apply_phase_list(sq_state* s, uint32_t q0, uint32_t q_size, const double* phases, uint64_t gc) {
    if (!s || !phases) return fail(SQ_ERR_ARG, "null argument");
    // src/suqa.cu:420-422 validates q_size > 0 and the list length; the device table
    // holds 128 entries (include/suqa_kernels.cuh:242)
    if (q_size == 0 || q_size > 7) return fail(SQ_ERR_UNSUPPORTED, "invalid q_size for a phase list");
    if (q0 + q_size > s->n) return fail(SQ_ERR_ARG, "phase-list register out of range");
    int rc = check_mask(s, gc);
    if (rc) return rc;
    HostOp h;
    h.kind = sqk::OP_PLIST;
    h.cmask = gc;
    h.zy = (1ull << q_size) - 1ull;
    h.shift = q0;
    const uint32_t L = 1u << q_size;
    h.tab.resize(2 * L);
    for (uint32_t k = 0; k < L; ++k) sincos(phases[k], &h.tab[2 * k + 1], &h.tab[2 * k]);
    if (gc == 0) {  // the reference guard (i & gc) never holds: nothing to do
        s->stats.gates++;
        return SQ_OK;
    }
    return enqueue(s, std::move(h));
}

static bool ref_supported(uint32_t k, const uint32_t* ps) {
    if (k == 1 || k == 2) return true;
    if (k == 3) {
        uint32_t a[3] = {ps[0], ps[1], ps[2]};
        std::sort(a, a + 3);
        return a[2] == 3 && a[0] == a[1];
    }
    return false;
}

int sq_apply_pauli_rotation(sq_state* s, uint32_t k, const uint32_t* qubits, const uint32_t* paulis,
                            double phase, uint64_t gc, int flags) {
    if (!s || !qubits || !paulis) return fail(SQ_ERR_ARG, "null argument");
    if (k == 0 || k > 32) return fail(SQ_ERR_ARG, "Pauli string length must be in 1..32");
    int rc = check_mask(s, gc);
    if (rc) return rc;
    for (uint32_t t = 0; t < k; ++t)
        if (paulis[t] < 1 || paulis[t] > 3) return fail(SQ_ERR_ARG, "Pauli type must be 1 (X), 2 (Y) or 3 (Z)");
    const bool refmode = (flags & SQ_PAULI_REFERENCE) != 0;
    if (refmode && !ref_supported(k, paulis))
        return fail(SQ_ERR_UNSUPPORTED, "ERROR: unimplemented pauli TP rotation in the selected configuration");
    uint32_t pl[32];
    for (uint32_t t = 0; t < k; ++t) pl[t] = paulis[t];
    // reference XY kernel (include/suqa_cpu.hpp:408-411) applies exp(i t Y(x)X)
    if (refmode && k == 2 && ((pl[0] == 1 && pl[1] == 2) || (pl[0] == 2 && pl[1] == 1))) std::swap(pl[0], pl[1]);
    HostOp h;
    h.kind = sqk::OP_PAULI;
    uint64_t seen = 0;
    for (uint32_t t = 0; t < k; ++t) {
        if ((rc = check_q(s, qubits[t]))) return rc;
        const uint64_t b = 1ull << qubits[t];
        if (seen & b) return fail(SQ_ERR_ARG, "repeated qubit in a Pauli string");
        seen |= b;
        if (pl[t] == 1 || pl[t] == 2) h.flip |= b;
        if (pl[t] == 2 || pl[t] == 3) h.zy |= b;
        if (pl[t] == 2) h.ny++;
    }
    if (gc & seen) {
        if (!refmode) return fail(SQ_ERR_ARG, "global control mask overlaps the rotated qubits");
        // Reference loops with the global control on a rotated qubit
        // (include/suqa_cpu.hpp:338-527): their element pointers alias.  One qubit:
        // X applies e^{i phase} twice, Z applies e^{i phase} then e^{-i phase}, on the
        // elements with every gc bit set.  X(x)X with one qubit in gc applies
        // exp(i phase X) twice to the other qubit under gc; with both in gc it applies
        // e^{i phase} four times.  Other aliased patterns are not reproduced.
        double sn, cs;
        sincos(phase, &sn, &cs);
        if (k == 1 && pl[0] == 1) {
            if ((rc = phase_op(s, gc, gc, cs, sn))) return rc;
            return phase_op(s, gc, gc, cs, sn);
        }
        if (k == 1 && pl[0] == 3) {
            if ((rc = phase_op(s, gc, gc, cs, sn))) return rc;
            return phase_op(s, gc, gc, cs, -sn);
        }
        if (k == 2 && pl[0] == 1 && pl[1] == 1) {
            const uint64_t freeb = seen & ~gc;
            if (!freeb) {
                for (int r = 0; r < 4; ++r)
                    if ((rc = phase_op(s, gc, gc, cs, sn))) return rc;
                return SQ_OK;
            }
            for (int r = 0; r < 2; ++r) {
                HostOp x;
                x.kind = sqk::OP_PAULI;
                x.flip = freeb;
                x.cmask = gc;
                x.cval = gc;
                x.skm = gc;
                x.skv = gc;
                x.c = cs;
                x.s = sn;
                if ((rc = enqueue(s, std::move(x)))) return rc;
            }
            return SQ_OK;
        }
        return fail(SQ_ERR_UNSUPPORTED, "Pauli rotation with the global control on a rotated qubit "
                                        "(only X, Z and X(x)X reproduce the reference)");
    }
    // pair ops test the control on g0 (lowest flipped bit clear); diagonal ops on g
    h.cmask = gc;
    h.cval = gc;
    h.skm = gc;
    h.skv = gc;
    sincos(phase, &h.s, &h.c);
    // uncontrolled: the larger of cos and sin into the global scale, the kernel
    // stores a + (s/c) iP a (or (c/s) a + iP a); the same choice as the kernel's
    const bool defer = gc == 0;
    const double f = std::fabs(h.c) >= std::fabs(h.s) ? h.c : h.s;
    h.gdefer = defer ? 1 : 0;
    rc = enqueue(s, std::move(h));
    if (rc || !defer) return rc;
    return scale_by(s, f);
}

int sq_apply_unitary(sq_state* s, uint32_t k, const uint32_t* qubits, const double* u_re, const double* u_im,
                     uint64_t gc) {
    if (!s || !qubits || !u_re || !u_im) return fail(SQ_ERR_ARG, "null argument");
    if (k < 1 || k > (uint32_t)sqk::kDenseQubits) return fail(SQ_ERR_ARG, "dense blocks act on 1 to 5 qubits");
    if (s->n < (uint32_t)sqk::kDenseQubits) return fail(SQ_ERR_UNSUPPORTED, "dense blocks need states of 5 qubits or more");
    int rc = check_mask(s, gc);
    if (rc) return rc;
    uint64_t m = 0;
    for (uint32_t b = 0; b < k; ++b) {
        if ((rc = check_q(s, qubits[b]))) return rc;
        if (m >> qubits[b] & 1ull) return fail(SQ_ERR_ARG, "repeated qubit in a dense block");
        m |= 1ull << qubits[b];
    }
    if (gc & m) return fail(SQ_ERR_ARG, "global control mask overlaps the block's qubits");
    // caller's index bit b is qubits[b]; stored index bit b is the b-th lowest qubit
    uint32_t pos[5];
    for (uint32_t b = 0; b < k; ++b) pos[b] = (uint32_t)popc(m & ((1ull << qubits[b]) - 1ull));
    const uint32_t D = 1u << k;
    auto to_stored = [&](uint32_t j) {
        uint32_t r = 0;
        for (uint32_t b = 0; b < k; ++b)
            if ((j >> b) & 1u) r |= 1u << pos[b];
        return r;
    };
    HostOp h;
    h.kind = sqk::OP_DENSE;
    h.flip = m;
    h.cmask = gc;
    h.cval = gc;
    h.skm = gc;
    h.skv = gc;
    h.dense.assign(2 * (size_t)D * D, 0.0);
    for (uint32_t r = 0; r < D; ++r)
        for (uint32_t c = 0; c < D; ++c) {
            const size_t o = (size_t)to_stored(r) * D + to_stored(c);
            h.dense[2 * o] = u_re[(size_t)r * D + c];
            h.dense[2 * o + 1] = u_im[(size_t)r * D + c];
        }
    return enqueue(s, std::move(h));
}

int sq_set_double_float(sq_state* s, int enabled) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = flush(s);
    if (!rc && enabled && !s->dfloat && s->prec == SQ_F64 && std::fabs(std::log2(std::fabs(s->gscale))) > 40.0)
        rc = materialize(s);
    s->dfloat = (enabled && s->prec == SQ_F64) ? 1 : 0;
    return rc;
}

int sq_set_dense_fusion(sq_state* s, int min_gates) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (min_gates < 0) return fail(SQ_ERR_ARG, "min_gates must be >= 0");
    int rc = flush(s);
    s->dense_fusion = min_gates;
    return rc;
}

int sq_set_dense_engine(sq_state* s, int engine) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    if (engine != 0 && engine != 1) return fail(SQ_ERR_ARG, "dense engine must be 0 (tensor cores) or 1 (CUDA cores)");
    int rc = flush(s);
    s->dense_engine = engine;
    return rc;
}

int sq_apply_qms_w(sq_state* s, uint32_t q_acc, uint64_t mask_enew, uint32_t shift, uint32_t E_old,
                   double c_factor) {
    int rc = check_q(s, q_acc);
    if (rc || (rc = check_mask(s, mask_enew))) return rc;
    if (mask_enew & (1ull << q_acc)) return fail(SQ_ERR_ARG, "energy mask contains the acceptance qubit");
    const uint64_t levels = (mask_enew >> shift) + 1ull;
    if (levels > (uint64_t)sqk::kMaxTab) return fail(SQ_ERR_UNSUPPORTED, "energy register wider than 7 qubits");
    HostOp h;
    h.kind = sqk::OP_W;
    h.flip = 1ull << q_acc;
    h.zy = mask_enew;
    h.shift = shift;
    h.tab.resize(2 * levels);
    // include/qms.cuh:288-297: dE = Enew*c - E_old*c; f1 = exp(-dE/2), f2 = sqrt(1 - f1^2)
    for (uint64_t e = 0; e < levels; ++e) {
        const uint32_t Enew = (uint32_t)e;
        const double dE = (Enew * c_factor - E_old * c_factor);
        double fs1, fs2;
        if (dE > 0) {
            fs1 = std::exp(-dE / 2.0);
            fs2 = std::sqrt(1.0 - fs1 * fs1);
        } else {
            fs1 = 1.0;
            fs2 = 0.0;
        }
        h.tab[2 * e] = fs1;
        h.tab[2 * e + 1] = fs2;
    }
    return enqueue(s, std::move(h));
}

int sq_measure_qbit(sq_state* s, uint32_t q, double r, uint32_t* c) {
    int rc = check_q(s, q);
    if (rc) return rc;
    if (!c) return fail(SQ_ERR_ARG, "null output");
    const uint64_t b = 1ull << q;
    rc = flush(s, 1, b, 0);
    if (rc) return rc;
    const double g2 = s->gscale * s->gscale;
    const double p0 = s->h_result[0] * g2, p1 = s->h_result[1] * g2;
    // src/suqa.cu:690-695: c = r < prob1; keep branch c; multiply by 1./norm (kept
    // in the global scale; the pass only zeroes the other branch)
    const uint32_t cc = (uint32_t)(r < p1);
    const double keep = cc ? p1 : p0;
    HostOp h;
    h.kind = sqk::OP_COLLAPSE;
    h.cmask = b;
    h.cval = cc ? b : 0ull;
    h.s = 1.0;
    *c = cc;
    rc = enqueue(s, std::move(h));
    if (rc) return rc;
    return scale_by(s, 1. / std::sqrt(keep));
}

int sq_prob_filter(sq_state* s, uint64_t mask_qs, uint64_t mask, double* prob) {
    int rc = check_mask(s, mask_qs);
    if (rc) return rc;
    if (!prob) return fail(SQ_ERR_ARG, "null output");
    rc = flush(s, 2, mask_qs, mask);
    if (rc) return rc;
    *prob = s->h_result[0] * s->gscale * s->gscale;
    return SQ_OK;
}

int sq_get_stats(const sq_state* s, sq_stats* out) {
    if (!s || !out) return fail(SQ_ERR_ARG, "null argument");
    *out = s->stats;
    return SQ_OK;
}

int sq_set_timing(sq_state* s, int enabled) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = flush(s);
    s->timing = enabled ? 1 : 0;
    return rc;
}

int sq_kernel_time(sq_state* s, double* ms, uint64_t* launches, uint64_t* bytes) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    int rc = flush(s);
    if (rc) return rc;
    SQ_CUDA(cudaStreamSynchronize(s->stream));
    double tot = 0.0;
    uint64_t by = 0;
    for (size_t i = 0; i < s->ev_open.size(); ++i) {
        float t = 0.f;
        SQ_CUDA(cudaEventElapsedTime(&t, s->ev_open[i].first, s->ev_open[i].second));
        tot += t;
        by += s->ev_bytes[i];
        s->ev_pool.push_back(s->ev_open[i].first);
        s->ev_pool.push_back(s->ev_open[i].second);
    }
    if (ms) *ms = tot;
    if (launches) *launches = s->ev_open.size();
    if (bytes) *bytes = by;
    s->ev_open.clear();
    s->ev_bytes.clear();
    return SQ_OK;
}

int sq_reset_stats(sq_state* s) {
    if (!s) return fail(SQ_ERR_ARG, "null state");
    std::memset(&s->stats, 0, sizeof(s->stats));
    return SQ_OK;
}

}  // extern "C"
