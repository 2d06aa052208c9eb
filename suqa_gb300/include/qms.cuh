// Quantum Metropolis Sampling on the suqa_gb300 engine: drop-in replacement of
// the reference's include/qms.cuh (namespace qms, same globals and functions, so
// the reference driver src/qms.cu compiles unchanged against it).
//
// One Metropolis step (metro_step) follows the reference procedure exactly,
// including the order of every random draw, because the measured outcomes are
// part of the result:
//   reset the energy and acceptance registers (measure + flip);
//   phase estimation Phi; read E_old (classically) and flip the register back;
//   draw a move C; apply U = W . Phi . C; measure the acceptance qubit;
//   accepted: read E_new, Phi^-1, and on sampling steps record E and the system
//             observable, re-reset the register and re-project with Phi/Phi^-1;
//   rejected: U^-1, then up to max_reverse_attempts rounds of
//             {Phi, read E, Phi^-1; stop if E == E_old; U, measure acc, U^-1}.
// The W oracle (acceptance rotation by exp(-beta dE / 2)) is one libsq pass
// (sq_apply_qms_w) with its factors computed on the host.
//
// Like the reference, this header defines globals and is included by exactly
// one translation unit (the driver).
#pragma once
#include <vector>
#include "Rand.hpp"
#include "complex_defines.cuh"
#include "io.hpp"
#include "suqa.cuh"

// system plugin (see system.cuh)
void evolution(const double& t, const int& n);
double measure_X(pcg& rgen);
void apply_C(const uint& Ci);
void apply_C_inverse(const uint& Ci);
std::vector<double> get_C_weigthsums();

#ifdef GATECOUNT
// gate-cost records of a metro step, a sample, a measurement, a restoration
// (defined by the driver, as src/qms.cu:33-39)
extern GateCounter gctr_global;
extern GateCounter gctr_metrostep;
extern GateCounter gctr_sample;
extern GateCounter gctr_measure;
extern GateCounter gctr_reverse;
#endif

namespace qms {

uint syst_qbits;
uint syst_levels;
uint ene_qbits;
uint ene_levels;
uint nqubits;
uint Dim;
uint max_reverse_attempts;
uint metro_steps;
uint reset_each;
unsigned long long iseed = 0ULL;
double t_phase_estimation;
double t_PE_factor;
double t_PE_shift;
int n_phase_estimation;
uint gCi;
uint c_acc = 0;

bool record_reverse = false;
std::vector<uint> reverse_counters;

pcg rangen;

std::vector<double> X_measures;
std::vector<double> E_measures;

double c_factor;

// register layout: system qubits, energy register, acceptance qubit (the MSB)
std::vector<uint> bm_syst;
std::vector<uint> bm_enes_new;
uint bm_acc;

uint curr_E_old;      // last energy reading, as the register integer
double curr_E_old_d;  // ... and as an energy

uint W_mask;
uint W_mask_Enew;

inline void fill_bitmap() {
    bm_syst.resize(syst_qbits);
    bm_enes_new.resize(ene_qbits);
    uint c = 0;
    for (uint i = 0; i < syst_qbits; ++i) bm_syst[i] = c++;
    for (uint i = 0; i < ene_qbits; ++i) bm_enes_new[i] = c++;
    bm_acc = c;
}

inline void fill_W_utils(double beta, double t_PE_factor_) {
    c_factor = beta / (t_PE_factor_ * ene_levels);
    W_mask_Enew = 0U;
    for (uint i = 0; i < ene_qbits; ++i) W_mask_Enew |= (1U << bm_enes_new[i]);
    W_mask = (1U << bm_acc) | W_mask_Enew;
}

inline void cevolution(const double& t, const int& n, const uint& q_control, const bmReg& qsyst) {
    if (qsyst.size() != syst_qbits) throw std::runtime_error("ERROR: controlled evolution has wrong number of state qbits");
    suqa::activate_gc_mask({q_control});
    evolution(t, n);
    suqa::deactivate_gc_mask({q_control});
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
    std::vector<double> r = extract_rands(ene_qbits);
    suqa::apply_reset(bm_enes_new, r);
    suqa::apply_reset(bm_acc, rangen.doub());
}

// controlled powers of exp(-iHt) on the energy register, phase shift by E_min,
// then the inverse QFT
inline void apply_phase_estimation(const std::vector<uint>& q_syst, const std::vector<uint>& q_target, const double& t,
                                   const uint& n) {
    suqa::apply_h(q_target);
    for (int trg = (int)q_target.size() - 1; trg > -1; --trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        cevolution(-powr * t, powr * n, q_target[trg], q_syst);
        suqa::apply_u1(q_target[trg], -powr * t * t_PE_shift);
    }
    suqa::apply_qft_inverse(q_target);
}

inline void apply_phase_estimation_inverse(const std::vector<uint>& q_syst, const std::vector<uint>& q_target,
                                           const double& t, const uint& n) {
    suqa::apply_qft(q_target);
    for (uint trg = 0; trg < q_target.size(); ++trg) {
        const double powr = (double)(1U << (q_target.size() - 1 - trg));
        cevolution(powr * t, powr * n, q_target[trg], q_syst);
        suqa::apply_u1(q_target[trg], powr * t * t_PE_shift);
    }
    suqa::apply_h(q_target);
}

inline void apply_Phi() { apply_phase_estimation(bm_syst, bm_enes_new, t_phase_estimation, n_phase_estimation); }
inline void apply_Phi_inverse() {
    apply_phase_estimation_inverse(bm_syst, bm_enes_new, t_phase_estimation, n_phase_estimation);
}

inline uint draw_C() {
    const std::vector<double> w = get_C_weigthsums();
    const double x = rangen.doub();
    for (uint Ci = 0U; Ci < w.size(); ++Ci)
        if (x < w[Ci]) return Ci;
    return (uint)w.size();
}

inline void apply_W() {
    const int rc = sq_apply_qms_w(suqa::engine(), bm_acc, W_mask_Enew, bm_enes_new[0], curr_E_old, c_factor);
    if (rc != SQ_OK) throw std::runtime_error(std::string("qms::apply_W: ") + sq_last_error());
    // cost: one (2 e)-controlled Toffoli per pair of energy levels (include/qms.cuh:324-328)
    const GateRecord gr = GateCounter::n_ctrl_toffoli_gates(2 * ene_qbits);
    const uint npairs = (ene_levels * (ene_levels - 1)) / 2;
    suqa::gatecounters.increment_g1g2(npairs * gr.ng1, npairs * gr.ng2);
}

inline void apply_W_inverse() { apply_W(); }

inline void apply_U() {
    apply_C(gCi);
    apply_Phi();
    apply_W();
}

inline void apply_U_inverse() {
    apply_W_inverse();
    apply_Phi_inverse();
    apply_C_inverse(gCi);
}

inline double energy_of(uint e) { return t_PE_shift + e / (double)(t_PE_factor * ene_levels); }

// Records the system observable with the energy register reset around it, then
// re-projects the energy (the sampling branch of the reference step).
inline void sample_observable_and_reproject(std::vector<uint>& c_E) {
    X_measures.push_back(measure_X(rangen));
    for (uint ei = 0U; ei < ene_qbits; ++ei) suqa::apply_reset(bm_enes_new[ei], rangen.doub());
    apply_Phi();
    suqa::measure_qbits(bm_enes_new, c_E, extract_rands(ene_qbits));
    apply_Phi_inverse();
}

// return values: 1 accepted, 2 accepted and sampled, 3 rejected and restored,
// 4 rejected, restored and sampled, -1 restoration failed
inline int metro_step(bool take_measure) {
#ifdef GATECOUNT
    gctr_metrostep.new_record();
#endif
    reset_non_syst_qbits();
    apply_Phi();
    std::vector<uint> c_E_news(ene_qbits, 0), c_E_olds(ene_qbits, 0);
    suqa::measure_qbits(bm_enes_new, c_E_olds, extract_rands(ene_qbits));
    curr_E_old = creg_to_uint(c_E_olds);
    curr_E_old_d = energy_of(curr_E_old);
    for (uint ei = 0U; ei < ene_qbits; ++ei)
        if (c_E_olds[ei]) suqa::apply_x(bm_enes_new[ei]);

    gCi = draw_C();
    apply_U();
    suqa::measure_qbit(bm_acc, c_acc, rangen.doub());

    if (c_acc == 1U) {
        suqa::measure_qbits(bm_enes_new, c_E_news, extract_rands(ene_qbits));
        apply_Phi_inverse();
        if (!take_measure) return 1;
#ifdef GATECOUNT
        gctr_measure.new_record();
#endif
        E_measures.push_back(energy_of(creg_to_uint(c_E_news)));
        for (uint ei = 0U; ei < ene_qbits; ++ei)
            if (c_E_news[ei]) suqa::apply_x(bm_enes_new[ei]);
        sample_observable_and_reproject(c_E_news);
#ifdef GATECOUNT
        gctr_measure.deactivate();
        gctr_sample.new_record();
#endif
        return 2;
    }

    apply_U_inverse();
    int ret = 0;
    uint iters = 0;
#ifdef GATECOUNT
    gctr_reverse.new_record();
#endif
    while (iters < max_reverse_attempts) {
        apply_Phi();
        suqa::measure_qbits(bm_enes_new, c_E_news, extract_rands(ene_qbits));
        const uint Enew_meas = creg_to_uint(c_E_news);
        apply_Phi_inverse();
        if (curr_E_old == Enew_meas) {
            if (take_measure) {
                E_measures.push_back(curr_E_old_d);
                for (uint ei = 0U; ei < ene_qbits; ++ei) suqa::apply_reset(bm_enes_new[ei], rangen.doub());
                sample_observable_and_reproject(c_E_news);
                ret = 4;
            } else {
                ret = 3;
            }
            break;
        }
        uint c_acc_trash;
        apply_U();
        suqa::measure_qbit(bm_acc, c_acc_trash, rangen.doub());
        apply_U_inverse();
        iters++;
    }
#ifdef GATECOUNT
    gctr_reverse.deactivate();
#endif
    if (record_reverse) reverse_counters.push_back(iters);
    if (iters == max_reverse_attempts) return -1;
    return ret;
}

inline void setup(double beta) {
    fill_bitmap();
    fill_W_utils(beta, t_PE_factor);
}

inline void clear() {}

}  // namespace qms
