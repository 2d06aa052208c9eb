// Quantum annealing by Szegedy walks on the suqa_gb300 engine: drop-in
// replacement of the reference's include/qsa.cuh (namespace qsa, same globals
// and functions, so the reference driver src/qsa.cu compiles unchanged).
//
// The walk operator W = lambda1 . U_x . U_y^-1 . lambda1 . U_y . U_x^-1 is built
// from energy phase estimations over the copied system, a Metropolis rotation of
// the acceptance qubit conditioned on the energy register, swaps of system and
// copy, and a reflection; phase estimation of W on the Szegedy register
// (apply_PE_szegedy) drives each annealing stage.  The gate sequence, the
// mask-stack semantics of the Szegedy controls and the order of random draws
// follow the reference exactly.  The reference's register layout is kept: the
// energy register starts at the same index as the triangle's copy register
// (bm_spin_tilde), so gates can act on qubits of the global control mask; libsq
// reproduces the reference semantics of those cases.
//
// Included by exactly one translation unit (the driver).
#pragma once
#include <cmath>
#include <vector>
#include "Rand.hpp"
#include "io.hpp"
#include "suqa.cuh"
#include "system.cuh"

void evolution_measure(const double& t, const int& n);
void evolution_szegedy(const double& t, const int& n);
void qsa_apply_C(const uint& Ci);
double measure_X(pcg& rgen);
void qsa_apply_C_inverse(const uint& Ci);
std::vector<double> get_C_weigthsums();

namespace qsa {

uint syst_qbits;
uint ene_qbits;
uint szegedy_qbits;
uint ene_levels;
uint nqubits;
uint Dim;
unsigned long long iseed = 0ULL;
double t_phase_estimation;
double t_PE_factor;
double t_PE_shift;
double t_phase_estimation_szegedy;
double t_PE_factor_szegedy;
double t_PE_shift_szegedy;
int n_phase_estimation;
double beta;
uint W_mask_E;

uint gc_mask_szegedy;

pcg rangen;

std::vector<double> E_measures;
std::vector<double> X_measures;

std::vector<double> rphase_m;
std::vector<double> rphase_m_szegedy;

inline void fill_phase_table(std::vector<double>& tab, const uint& n) {
    tab.resize(n);
    uint c = 1;
    for (uint i = 0; i < n; ++i) {
        tab[i] = (2.0 * M_PI / (double)c);
        c <<= 1;
    }
}
inline void fill_rphase(const uint& n) { fill_phase_table(rphase_m, n); }
inline void fill_rphase_szegedy(const uint& n) { fill_phase_table(rphase_m_szegedy, n); }

// The Szegedy control is the base of the global mask; inner controls add to it.
// (each change also refreshes the gate counters' control count, include/qsa.cuh:70-96)
inline void activate_gc_mask_szegedy(const bmReg& q_controls) {
    gc_mask_szegedy = 0U;
    for (const auto& q : q_controls) gc_mask_szegedy |= 1U << q;
    suqa::gc_mask = gc_mask_szegedy;
    suqa::gatecounters.update_cmask_setbits(suqa::gc_mask);
}
inline void deactivate_gc_mask_szegedy() {
    gc_mask_szegedy = 0U;
    suqa::gc_mask = 0U;
    suqa::gatecounters.update_cmask_setbits(suqa::gc_mask);
}
inline void activate_gc_mask_into_szegedy(const bmReg& q_controls) {
    for (const auto& q : q_controls) suqa::gc_mask |= 1U << q;
    suqa::gatecounters.update_cmask_setbits(suqa::gc_mask);
}
inline void deactivate_gc_mask_into_szegedy() {
    suqa::gc_mask = gc_mask_szegedy;
    suqa::gatecounters.update_cmask_setbits(suqa::gc_mask);
}

std::vector<uint> bm_states;
std::vector<uint> bm_enes;
std::vector<uint> bm_szegedy;
uint bm_acc;

inline void fill_bitmap() {
    bm_states.resize(syst_qbits);
    bm_enes.resize(ene_qbits);
    bm_szegedy.resize(szegedy_qbits);
    uint c = 0;
    for (uint i = 0; i < syst_qbits; ++i) bm_states[i] = c++;
    for (uint i = 0; i < ene_qbits; ++i) bm_enes[i] = c++;
    for (uint i = 0; i < szegedy_qbits; ++i) bm_szegedy[i] = c++;
    bm_acc = c;
    for (uint i = 0; i < ene_qbits; ++i) W_mask_E |= (1U << bm_enes[i]);
}

inline void check_register(const bmReg& qstate) {
    if (qstate.size() != syst_qbits) throw std::runtime_error("ERROR: controlled evolution has wrong number of state qbits");
}

inline void cevolution_measure(const double& t, const int& n, const uint& q_control, const bmReg& qstate) {
    check_register(qstate);
    suqa::activate_gc_mask({q_control});
    evolution_measure(t, n);
    suqa::deactivate_gc_mask({q_control});
}

inline void cevolution_szegedy_PE(const double& t, const int& n, const uint& q_control, const bmReg& qstate) {
    check_register(qstate);
    activate_gc_mask_into_szegedy({q_control});
    evolution_szegedy(t, n);
    deactivate_gc_mask_into_szegedy();
}

inline uint creg_to_uint(const std::vector<uint>& c_reg) {
    if (c_reg.size() < 1) throw std::runtime_error("ERROR: size of register zero.");
    uint ret = c_reg[0];
    for (uint j = 1U; j < c_reg.size(); ++j) ret += c_reg[j] << j;
    return ret;
}

inline std::vector<double> extract_rands(uint n) {
    std::vector<double> r(n);
    for (auto& x : r) x = rangen.doub();
    return r;
}

inline void reset_non_syst_qbits() {
    std::vector<double> r1 = extract_rands(ene_qbits);
    suqa::apply_reset(bm_enes, r1);
    std::vector<double> r2 = extract_rands(szegedy_qbits);
    suqa::apply_reset(bm_szegedy, r2);
    suqa::apply_reset(bm_acc, rangen.doub());
}

// QFTs over a phase table (controlled phases +-table[m])
inline void crm_from(const std::vector<double>& tab, const uint& qc, const uint& qt, const int& m) {
    double rphase = (m > 0) ? tab[m] : tab[-m];
    if (m <= 0) rphase *= -1;
    suqa::apply_cu1(qc, qt, rphase);
}
inline void qft_from(const std::vector<double>& tab, const std::vector<uint>& q) {
    const int k = (int)q.size();
    for (int o = k - 1; o >= 0; o--) {
        suqa::apply_h(q[o]);
        for (int i = o - 1; i >= 0; i--) crm_from(tab, q[i], q[o], +1 + (o - i));
    }
}
inline void qft_inverse_from(const std::vector<double>& tab, const std::vector<uint>& q) {
    const int k = (int)q.size();
    for (int o = 0; o < k; o++) {
        for (int i = 0; i < o; i++) crm_from(tab, q[i], q[o], -1 - (o - i));
        suqa::apply_h(q[o]);
    }
}
inline void qsa_crm(const uint& qc, const uint& qt, const int& m) { crm_from(rphase_m, qc, qt, m); }
inline void qsa_qft(const std::vector<uint>& q) { qft_from(rphase_m, q); }
inline void qsa_qft_inverse(const std::vector<uint>& q) { qft_inverse_from(rphase_m, q); }
inline void qsa_crm_szegedy(const uint& qc, const uint& qt, const int& m) { crm_from(rphase_m_szegedy, qc, qt, m); }
inline void qsa_qft_szegedy(const std::vector<uint>& q) { qft_from(rphase_m_szegedy, q); }
inline void qsa_qft_inverse_szegedy(const std::vector<uint>& q) { qft_inverse_from(rphase_m_szegedy, q); }

// energy phase estimation over the copy register (inside the Szegedy control)
inline void apply_phase_estimation(const std::vector<uint>& q_state, const std::vector<uint>& q_target, const double& t,
                                   const uint& n) {
    suqa::apply_h(q_target);
    for (int trg = (int)q_target.size() - 1; trg > -1; --trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        cevolution_szegedy_PE(-powr * t, powr * n, q_target[trg], q_state);
        suqa::apply_u1(q_target[trg], -powr * t * t_PE_shift);
    }
    qsa_qft_inverse(q_target);
}

inline void apply_phase_estimation_inverse(const std::vector<uint>& q_state, const std::vector<uint>& q_target,
                                           const double& t, const uint& n) {
    qsa_qft(q_target);
    for (uint trg = 0; trg < q_target.size(); ++trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        cevolution_szegedy_PE(powr * t, powr * n, q_target[trg], q_state);
        suqa::apply_u1(q_target[trg], powr * t * t_PE_shift);
    }
    suqa::apply_h(q_target);
}

// energy read-out phase estimation of the system on the Szegedy register
inline void apply_phase_estimation_measure(const std::vector<uint>& q_state, const std::vector<uint>& q_target,
                                           const double& t, const uint& n) {
    suqa::apply_h(q_target);
    for (int trg = (int)q_target.size() - 1; trg > -1; --trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        cevolution_measure(-powr * t, powr * n, q_target[trg], q_state);
        suqa::apply_u1(q_target[trg], -powr * t * t_PE_shift_szegedy);
    }
    qsa_qft_inverse_szegedy(q_target);
}

inline void apply_phase_estimation_measure_inverse(const std::vector<uint>& q_state, const std::vector<uint>& q_target,
                                                   const double& t, const uint& n) {
    qsa_qft_szegedy(q_target);
    for (uint trg = 0; trg < q_target.size(); ++trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        suqa::apply_u1(q_target[trg], powr * t * t_PE_shift_szegedy);
        cevolution_measure(powr * t, powr * n, q_target[trg], q_state);
    }
    suqa::apply_h(q_target);
}

inline uint draw_C() {
    const std::vector<double> w = get_C_weigthsums();
    const double x = rangen.doub();
    for (uint Ci = 0U; Ci < w.size(); ++Ci)
        if (x < w[Ci]) return Ci;
    return (uint)w.size();
}

// X on the energy qubits whose bit of x is 0 (selects the level x for a control)
inline void apply_ctrl_x(int x) {
    for (uint i = 0; i < ene_qbits; i++) {
        const int r = x % 2;
        if (r == 0) suqa::apply_x(bm_enes[i]);
        x = (x - r) / 2;
    }
}

inline double eigenvalue_trans(int x_2d) { return t_PE_shift + x_2d / (double)(t_PE_factor * ene_levels); }

// Metropolis rotation of the acceptance qubit for the energy level 2 (the level
// the reference hard-wires), RY by -+acos(exp(-beta E / 2))
inline void level_rotation(const double& beta_j, double sign) {
    const int level = 2;
    const double e = eigenvalue_trans(level);
    apply_ctrl_x(level);
    activate_gc_mask_into_szegedy(bm_enes);
    suqa::apply_pauli_TP_rotation({bm_acc}, {PAULI_Y}, sign * acos(exp(-0.5 * beta_j * e)));
    deactivate_gc_mask_into_szegedy();
    apply_ctrl_x(level);
}
inline void universal_rotation(const double& beta_j) { level_rotation(beta_j, -1.0); }
inline void universal_rotation_inverse(const double& beta_j) { level_rotation(beta_j, +1.0); }

// phase flip of the acceptance qubit's |0> on energy level 1
inline void universal_reflection() {
    apply_ctrl_x(1);
    activate_gc_mask_into_szegedy(bm_enes);
    suqa::apply_x(bm_acc);
    suqa::apply_u1(bm_acc, M_PI);
    suqa::apply_x(bm_acc);
    deactivate_gc_mask_into_szegedy();
    apply_ctrl_x(1);
}

inline void rotation(const double& beta_j) {
    suqa::apply_x(bm_enes[0]);
    activate_gc_mask_into_szegedy(bm_enes);
    suqa::apply_pauli_TP_rotation({bm_acc}, {PAULI_Y}, -acos(exp(-2 * beta_j)));
    deactivate_gc_mask_into_szegedy();
    suqa::apply_x(bm_enes[0]);
}

inline void rotation_inverse(const double& beta_j) {
    suqa::apply_x(bm_enes[0]);
    activate_gc_mask_into_szegedy(bm_enes);
    suqa::apply_pauli_TP_rotation({bm_acc}, {PAULI_Y}, acos(exp(-2 * beta_j)));
    deactivate_gc_mask_into_szegedy();
    suqa::apply_x(bm_enes[0]);
}

inline void apply_ux(const double& beta_j, const uint& Ci) {
    qsa_apply_C(Ci);
    apply_phase_estimation(bm_states, bm_enes, t_phase_estimation, n_phase_estimation);
    universal_rotation(beta_j);
    apply_phase_estimation_inverse(bm_states, bm_enes, t_phase_estimation, n_phase_estimation);
}

inline void apply_ux_inverse(const double& beta_j, const uint& Ci) {
    apply_phase_estimation(bm_states, bm_enes, t_phase_estimation, n_phase_estimation);
    universal_rotation_inverse(beta_j);
    apply_phase_estimation_inverse(bm_states, bm_enes, t_phase_estimation, n_phase_estimation);
    qsa_apply_C_inverse(Ci);
}

// swap system and copy, controlled on the acceptance qubit being 0
inline void swap_system_copy_on_reject() {
    suqa::apply_x(bm_acc);
    activate_gc_mask_into_szegedy({bm_acc});
    for (uint j = 0; j < bm_spin.size(); ++j) suqa::apply_swap(bm_spin[j], bm_spin_tilde[j]);
    deactivate_gc_mask_into_szegedy();
    suqa::apply_x(bm_acc);
}

inline void apply_uy(const double& beta_j, const uint& Ci) {
    apply_ux(beta_j, Ci);
    swap_system_copy_on_reject();
}

inline void apply_uy_inverse(const double& beta_j, const uint& Ci) {
    swap_system_copy_on_reject();
    apply_ux_inverse(beta_j, Ci);
}

inline void reflection() {
    suqa::apply_mcx(bm_enes, {1U, 0U}, bm_acc);
    suqa::apply_mcu1(bm_enes, {1U, 0U}, bm_acc, M_PI);
    suqa::apply_mcx(bm_enes, {1U, 0U}, bm_acc);
}

inline void apply_lambda1() {
    apply_phase_estimation(bm_states, bm_enes, t_phase_estimation, n_phase_estimation);
    universal_reflection();
    apply_phase_estimation_inverse(bm_states, bm_enes, t_phase_estimation, n_phase_estimation);
}

inline void apply_szegedy(const double& beta_j, const uint& Ci) {
    apply_lambda1();
    apply_ux(beta_j, Ci);
    apply_uy_inverse(beta_j, Ci);
    apply_lambda1();
    apply_uy(beta_j, Ci);
    apply_ux_inverse(beta_j, Ci);
}

inline void cevolution_szegedy(const uint& q_control, const bmReg& qstate, const int& powr, const double& beta_j,
                               const uint& Ci) {
    check_register(qstate);
    activate_gc_mask_szegedy({q_control});
    for (int mm = 0; mm < powr; ++mm) apply_szegedy(beta_j, Ci);
    deactivate_gc_mask_szegedy();
}

inline void apply_PE_szegedy(const std::vector<uint>& q_state, const std::vector<uint>& q_target, const double& beta_j,
                             const uint& Ci) {
    suqa::apply_h(q_target);
    for (int trg = (int)q_target.size() - 1; trg > -1; --trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        cevolution_szegedy(q_target[trg], q_state, (int)powr, beta_j, Ci);
    }
    qsa_qft_inverse_szegedy(q_target);
}

inline void setup() {
    fill_rphase(ene_qbits + 1);
    fill_rphase_szegedy(szegedy_qbits + 1);
    fill_bitmap();
}

inline void clear() {}

}  // namespace qsa
