// suqa:: API over libsq (the drop-in shim for the reference's src/suqa.cu).
// Mask construction mirrors the reference dispatcher (src/suqa.cu:45-757 there);
// the arithmetic runs in libsq's sm_103a kernels.
#include "suqa.cuh"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

ComplexVec suqa::state;
std::vector<double> suqa::rphase_m;
uint suqa::gc_mask = 0U;
uint suqa::nq = 0U;
#ifdef GPU
uint suqa::blocks = 1, suqa::threads = 128;
cudaStream_t suqa::stream1 = nullptr, suqa::stream2 = nullptr;
#endif

namespace {
sq_state* g_state = nullptr;
int g_precision = -1;

int default_precision() {
    if (g_precision >= 0) return g_precision;
    const char* e = std::getenv("SUQA_PRECISION");
    if (e && (std::strcmp(e, "f32") == 0 || std::strcmp(e, "fp32") == 0)) return SQ_F32;
    return SQ_F64;
}

void check(int rc) {
    if (rc == SQ_OK) return;
    throw std::runtime_error(std::string("suqa (libsq): ") + sq_last_error());
}

sq_state* st() {
    if (!g_state) throw std::runtime_error("suqa: state not allocated (call suqa::setup first)");
    return g_state;
}
}  // namespace

sq_state* suqa::engine() { return g_state; }
void suqa::set_precision(int p) { g_precision = p; }

void suqa::print_banner() {
    printf("\n   SUQA gate API on libsq (GB300, sm_103a)\n\n Simulator for Universal Quantum Algorithms\n\n");
}

GateCounterList suqa::gatecounters;

namespace {
// gate costs as the reference's GATECOUNT hooks (src/suqa.cu): a gate with
// `extra` controls of its own under the global mask costs mult x an
// (n + extra)-controlled Toffoli, n the mask's set bits when it last changed
void count_gate(uint extra, uint mult = 1U) {
    const GateRecord gr = GateCounter::n_ctrl_toffoli_gates(suqa::gatecounters.gc_mask_set_qbits + extra);
    suqa::gatecounters.increment_g1g2(mult * gr.ng1, mult * gr.ng2);
}
// a k-qubit Pauli rotation (src/suqa.cu, end of apply_pauli_TP_rotation): one n-
// and 2(k-1) (n+1)-controlled Toffolis, and with x > 0 non-Z factors two more
// n-controlled Toffolis and 2(x-1) CNOTs for the basis changes
void count_pauli(const std::vector<uint>& paulis) {
    const uint n = suqa::gatecounters.gc_mask_set_qbits;
    const uint k = (uint)paulis.size();
    const GateRecord g0 = GateCounter::n_ctrl_toffoli_gates(n), g1 = GateCounter::n_ctrl_toffoli_gates(n + 1);
    suqa::gatecounters.increment_g1g2(g0.ng1, g0.ng2);
    suqa::gatecounters.increment_g1g2(2 * (k - 1) * g1.ng1, 2 * (k - 1) * g1.ng2);
    uint x = 0;
    for (uint p : paulis)
        if (p != PAULI_Z) ++x;
    if (x > 0) {
        suqa::gatecounters.increment_g1g2(2 * g0.ng1, 2 * g0.ng2);
        suqa::gatecounters.increment_g1g2(0, 2 * (x - 1));
    }
}
}  // namespace

void suqa::activate_gc_mask(const bmReg& q_controls) {
    for (const auto& q : q_controls) suqa::gc_mask |= 1U << q;
    suqa::gatecounters.update_cmask_setbits(suqa::gc_mask);
}

void suqa::deactivate_gc_mask(const bmReg& q_controls) {
    for (const auto& q : q_controls) suqa::gc_mask &= ~(1U << q);
    suqa::gatecounters.update_cmask_setbits(suqa::gc_mask);
}

double suqa::vnorm() {
    double v = 0.0;
    check(sq_vnorm(st(), &v));
    return v;
}

void suqa::vnormalize() { check(sq_vnormalize(st())); }

void suqa::init_state() { check(sq_init_state(st())); }

void suqa::deallocate_state() {
    if (g_state) sq_state_destroy(g_state);
    g_state = nullptr;
    state.data = state.data_re = state.data_im = nullptr;
    state.vecsize = 0U;
}

void suqa::allocate_state(uint Dim) {
    deallocate_state();
    uint n = 0;
    while ((1U << n) < Dim) ++n;
    const int rc = sq_state_create(&g_state, n, default_precision());
    if (rc == SQ_ERR_NODEVICE) {
        // Without a usable GPU there is nothing to run on: say so and end with the
        // status code rather than an uncaught exception (the drivers allocate the
        // state before they open any output file).
        std::fprintf(stderr, "suqa (libsq): %s; the gate engine needs a GPU\n", sq_last_error());
        std::exit(SQ_ERR_NODEVICE);
    }
    check(rc);
    void *re = nullptr, *im = nullptr;
    check(sq_state_ptrs(g_state, &re, &im));
    state.vecsize = Dim;
    state.data = state.data_re = static_cast<double*>(re);
    state.data_im = static_cast<double*>(im);
}

// ---- single-qubit gates
void suqa::apply_x(uint q) {
    check(sq_apply_x(st(), q, suqa::gc_mask));
    count_gate(0);
}
void suqa::apply_x(const bmReg& qs) { for (const auto& q : qs) suqa::apply_x(q); }
void suqa::apply_y(uint q) {
    check(sq_apply_y(st(), q, suqa::gc_mask));
    count_gate(0);
}
void suqa::apply_y(const bmReg& qs) { for (const auto& q : qs) suqa::apply_y(q); }
void suqa::apply_z(uint q) { suqa::apply_u1(q, M_PI); }
void suqa::apply_z(const bmReg& qs) { for (const auto& q : qs) suqa::apply_u1(q, M_PI); }
void suqa::apply_h(uint q) {
    check(sq_apply_h(st(), q, suqa::gc_mask));
    count_gate(0);
}
void suqa::apply_h(const bmReg& qs) { for (const auto& q : qs) suqa::apply_h(q); }
void suqa::apply_t(uint q) { suqa::apply_u1(q, M_PI / 4.0); }
void suqa::apply_t(const bmReg& qs) { for (const auto& q : qs) suqa::apply_u1(q, M_PI / 4.0); }
void suqa::apply_tdg(uint q) { suqa::apply_u1(q, -M_PI / 4.0); }
void suqa::apply_tdg(const bmReg& qs) { for (const auto& q : qs) suqa::apply_u1(q, -M_PI / 4.0); }
void suqa::apply_s(uint q) { suqa::apply_u1(q, M_PI / 2.0); }
void suqa::apply_s(const bmReg& qs) { for (const auto& q : qs) suqa::apply_u1(q, M_PI / 2.0); }

void suqa::apply_u1(uint q, double phase) { suqa::apply_u1(q, 1U, phase); }
void suqa::apply_u1(uint q, uint q_mask, double phase) {
    check(sq_apply_u1(st(), q, q_mask, phase, suqa::gc_mask));
    count_gate(0);
}

// ---- multi-qubit gates: control masks as src/suqa.cu:289-393 builds them
void suqa::apply_cx(const uint& q_control, const uint& q_target, const uint& q_mask) {
    uint64_t mask_qs = suqa::gc_mask;
    const uint64_t mask = mask_qs | (1ull << q_control);
    if (q_mask) mask_qs |= 1ull << q_control;
    check(sq_apply_mcx(st(), mask, mask_qs, q_target));
    count_gate(1);
}

void suqa::apply_mcx(const bmReg& q_controls, const uint& q_target) {
    uint64_t mask = suqa::gc_mask;
    for (const auto& q : q_controls) mask |= 1ull << q;
    check(sq_apply_mcx(st(), mask, mask, q_target));
    count_gate((uint)q_controls.size());
}

void suqa::apply_mcx(const bmReg& q_controls, const bmReg& q_mask, const uint& q_target) {
    uint64_t mask = suqa::gc_mask, mask_qs = suqa::gc_mask;
    for (const auto& q : q_controls) mask |= 1ull << q;
    for (size_t k = 0; k < q_controls.size(); ++k)
        if (q_mask[k]) mask_qs |= 1ull << q_controls[k];
    check(sq_apply_mcx(st(), mask, mask_qs, q_target));
    count_gate((uint)q_controls.size());
}

void suqa::apply_cu1(uint q_control, uint q_target, double phase, uint q_mask) {
    uint64_t mask_qs = (1ull << q_target) | suqa::gc_mask;
    const uint64_t mask = mask_qs | (1ull << q_control);
    if (q_mask) mask_qs |= 1ull << q_control;
    check(sq_apply_mcu1(st(), mask, mask_qs, phase));
    count_gate(1);
}

void suqa::apply_mcu1(const bmReg& q_controls, const bmReg& q_mask, const uint& q_target, double phase) {
    uint64_t mask = (1ull << q_target) | suqa::gc_mask;
    for (const auto& q : q_controls) mask |= 1ull << q;
    uint64_t mask_qs = (1ull << q_target) | suqa::gc_mask;
    for (size_t k = 0; k < q_controls.size(); ++k)
        if (q_mask[k]) mask_qs |= 1ull << q_controls[k];
    check(sq_apply_mcu1(st(), mask, mask_qs, phase));
    count_gate((uint)q_controls.size());
}

void suqa::apply_mcu1(const bmReg& q_controls, const uint& q_target, double phase) {
    suqa::apply_mcu1(q_controls, std::vector<uint>(q_controls.size(), 1U), q_target, phase);
}

// a swap is three CNOTs (src/suqa.cu:409-415)
void suqa::apply_swap(const uint& q1, const uint& q2) {
    check(sq_apply_swap(st(), q1, q2, suqa::gc_mask));
    count_gate(1, 3U);
}

void suqa::apply_phase_list(uint q0, uint q_size, const std::vector<double>& phases) {
    if (!(q_size > 0U && (uint)phases.size() == (1U << q_size)))
        throw std::runtime_error("ERROR: in suqa::apply_phase_list(): invalid q_size or phases.size()");
    check(sq_apply_phase_list(st(), q0, q_size, phases.data(), suqa::gc_mask));
    // src/suqa.cu:442-453: 2^(q_size-2) (the reference's `1U<<(q_size+1)-3`, the
    // shift count taken modulo 32) times an n- plus an (n+1)-controlled Toffoli
    const uint fact = 1U << ((q_size + 1U - 3U) & 31U);
    const uint n = suqa::gatecounters.gc_mask_set_qbits;
    const GateRecord a = GateCounter::n_ctrl_toffoli_gates(n), b = GateCounter::n_ctrl_toffoli_gates(n + 1);
    suqa::gatecounters.increment_g1g2(fact * (a.ng1 + b.ng1), fact * (a.ng2 + b.ng2));
}

void suqa::apply_pauli_TP_rotation(const bmReg& q_apply, const std::vector<uint>& pauli_TPtype, double phase) {
    if (q_apply.size() != pauli_TPtype.size())
        throw std::runtime_error(
            "ERROR: in suqa::apply_pauli_TP_rotation(): mismatch between qubits number and pauli types specified");
    const int rc = sq_apply_pauli_rotation(st(), (uint32_t)q_apply.size(), q_apply.data(), pauli_TPtype.data(),
                                           phase, suqa::gc_mask, SQ_PAULI_REFERENCE);
    if (rc == SQ_ERR_UNSUPPORTED)
        throw std::runtime_error("ERROR: unimplemented pauli TP rotation in the selected configuration");
    check(rc);
    count_pauli(pauli_TPtype);
}

void suqa::apply_pauli_rotation(const bmReg& q_apply, const std::vector<uint>& paulis, double phase) {
    if (q_apply.size() != paulis.size())
        throw std::runtime_error("ERROR: in suqa::apply_pauli_rotation(): qubit and Pauli lists differ in length");
    check(sq_apply_pauli_rotation(st(), (uint32_t)q_apply.size(), q_apply.data(), paulis.data(), phase,
                                  suqa::gc_mask, SQ_PAULI_EXACT));
    count_pauli(paulis);
}

// ---- QFT (src/suqa.cu:611-661): H and controlled phases 2*pi/2^m
namespace {
void qft_crm(const uint& q_control, const uint& q_target, const int& m, const int& nqubits) {
    if (suqa::rphase_m.empty()) {
        // sized by the first call, as the reference's table
        suqa::rphase_m.resize(nqubits + 1);
        uint c = 1;
        for (int i = 0; i < nqubits + 1; ++i) {
            suqa::rphase_m[i] = (2.0 * M_PI / (double)c);
            c <<= 1;
        }
    }
    const int am = m > 0 ? m : -m;
    double rphase = am < (int)suqa::rphase_m.size() ? suqa::rphase_m[am] : (2.0 * M_PI / (double)(1U << am));
    if (m <= 0) rphase *= -1;
    suqa::apply_cu1(q_control, q_target, rphase);
}
}  // namespace

void suqa::apply_qft(const std::vector<uint>& qact) {
    const int qsize = (int)qact.size();
    for (int o = qsize - 1; o >= 0; o--) {
        suqa::apply_h(qact[o]);
        for (int i = o - 1; i >= 0; i--) qft_crm(qact[i], qact[o], +1 + (o - i), qsize);
    }
}

void suqa::apply_qft_inverse(const std::vector<uint>& qact) {
    const int qsize = (int)qact.size();
    for (int o = 0; o < qsize; o++) {
        for (int i = 0; i < o; i++) qft_crm(qact[i], qact[o], -1 - (o - i), qsize);
        suqa::apply_h(qact[o]);
    }
}

// ---- measurement (src/suqa.cu:673-757)
void suqa::measure_qbit(uint q, uint& c, double rdoub) {
    uint32_t cc = 0;
    check(sq_measure_qbit(st(), q, rdoub, &cc));
    c = cc;
}

void suqa::measure_qbits(const bmReg& qs, std::vector<uint>& cs, const std::vector<double>& rdoubs) {
    for (uint k = 0U; k < qs.size(); ++k) suqa::measure_qbit(qs[k], cs[k], rdoubs[k]);
}

void suqa::apply_reset(uint q, double rdoub) {
    uint c;
    suqa::measure_qbit(q, c, rdoub);
    if (c) suqa::apply_x(q);
}

void suqa::apply_reset(const bmReg& qs, std::vector<double> rdoubs) {
    for (uint i = 0; i < qs.size(); ++i) suqa::apply_reset(qs[i], rdoubs[i]);
}

void suqa::prob_filter(const bmReg& qs, const std::vector<uint>& q_mask, double& prob) {
    uint64_t mask_qs = 0U, mask = 0U;
    for (const auto& q : qs) mask_qs |= 1ull << q;
    for (uint k = 0U; k < q_mask.size(); ++k)
        if (q_mask[k]) mask |= (uint64_t)q_mask[k] << qs[k];
    check(sq_prob_filter(st(), mask_qs, mask, &prob));
}

void suqa::setup(uint num_qubits) {
    suqa::nq = num_qubits;
    printf("Running on gpu (libsq, sm_103a, %s amplitudes) in %s mode\n",
           default_precision() == SQ_F64 ? "FP64" : "FP32",
#ifdef NDEBUG
           "release"
#else
           "debug"
#endif
    );
    suqa::allocate_state(1U << suqa::nq);
}

void suqa::clear() {
    deallocate_state();
    suqa::gatecounters.print_counts();  // prints only when a driver registered counters
}

void suqa::debug_print_state() {
    if (!g_state) return;
    std::vector<double> re(state.size()), im(state.size());
    if (sq_get_state(g_state, re.data(), im.data()) != SQ_OK) return;
    double nrm = 0.0;
    sq_vnorm(g_state, &nrm);
    printf("vnorm = %.12lg\n", nrm);
    sparse_print(re.data(), im.data(), state.size());
}

// ---- io helpers (the reference's src/io.cpp counterparts)
int get_time(struct timeval* tp, struct timezone* tzp) {
    (void)tzp;
    namespace sc = std::chrono;
    auto d = sc::system_clock::now().time_since_epoch();
    auto s = sc::duration_cast<sc::seconds>(d);
    tp->tv_sec = s.count();
    tp->tv_usec = sc::duration_cast<sc::microseconds>(d - s).count();
    return 0;
}

bool file_exists(const char* fname) { return access(fname, F_OK) != -1; }

void sparse_print(double* v_re, double* v_im, size_t size) {
    size_t bits = 0;
    while (((size_t)1 << bits) < size) ++bits;
    for (size_t i = 0; i < size; ++i) {
        const double m2 = v_re[i] * v_re[i] + v_im[i] * v_im[i];
        if (m2 > 1e-10) {
            std::string idx = std::bitset<32>(i).to_string().substr(32 - bits);
            printf("|%s> (%5zu) -> (%.3e, %.3e ) : mod2= %.3e\n", idx.c_str(), i,
                   std::fabs(v_re[i]) > 1e-8 ? v_re[i] : 0.0, std::fabs(v_im[i]) > 1e-8 ? v_im[i] : 0.0, m2);
        }
    }
    std::cout << std::endl;
}
