// The frustrated 3-spin triangle, H = X0X1 + X1X2 + X2X0, as a system plugin of
// the suqa_gb300 drop-in headers (same gate sequences as the reference's
// src/system.cu:6-151, so QMS/QSA runs reproduce the reference bit for bit in
// measured outcomes):
//  - init_state: |0>, X on spin 1, H on spin 1, CX(1 -> 0)
//  - evolution(t): exp(-iHt) as exp(-i t X_a X_b) for the pairs (1,2), (2,0), (0,1)
//  - moves C_i: Hadamard on spin i, weights 1/3 each
//  - observable: H^3, CX(0,1), CX(0,2), U1(2, pi/2), measure the spins, table
//    {2,0,2,0,-2,0,-2,0}
#include <cmath>
#include "Rand.hpp"
#include "system.cuh"

double g_beta;

void init_state() {
    suqa::init_state();
    suqa::apply_x(bm_spin[1]);
    suqa::apply_h(bm_spin[1]);
    suqa::apply_cx(bm_spin[1], bm_spin[0]);
}

static void xx_rotation(const bmReg& q, uint pos, double phase) {
    suqa::apply_pauli_TP_rotation({q[(pos + 1) % 3], q[(pos + 2) % 3]}, {PAULI_X, PAULI_X}, phase);
}

void evolution(const double& t, const int& n) {
    (void)n;
    for (uint k = 0; k < 3; ++k) xx_rotation(bm_spin, k, -t);
}

void qsa_init_state() {
    suqa::init_state();
    for (int k = 0; k < 3; ++k) suqa::apply_h(bm_spin[k]);
    for (int k = 0; k < 3; ++k) suqa::apply_cx(bm_spin[k], bm_spin_tilde[k]);
}

void evolution_szegedy(const double& t, const int& n) {
    (void)n;
    for (uint i = 0; i < 3; i++) {
        suqa::apply_pauli_TP_rotation({bm_spin_tilde[i % 3], bm_spin_tilde[(1 + i) % 3]}, {PAULI_X, PAULI_X}, -t);
        suqa::apply_pauli_TP_rotation({bm_spin[i % 3], bm_spin[(1 + i) % 3]}, {PAULI_X, PAULI_X}, t);
    }
}

void evolution_measure(const double& t, const int& n) {
    (void)n;
    for (uint i = 0; i < 3; i++)
        suqa::apply_pauli_TP_rotation({bm_spin[i % 3], bm_spin[(1 + i) % 3]}, {PAULI_X, PAULI_X}, -t);
}

void evolution_tracing(const double& t, const int& n) {
    (void)n;
    for (uint i = 0; i < 3; i++)
        suqa::apply_pauli_TP_rotation({bm_spin_tilde[i % 3], bm_spin_tilde[(1 + i) % 3]}, {PAULI_X, PAULI_X}, -t);
}

static const std::vector<double> k_observable = {2.0, 0.0, 2.0, 0.0, -2.0, 0.0, -2.0, 0.0};

static void measure_basis_change() {
    for (int k = 0; k < 3; ++k) suqa::apply_h(bm_spin[k]);
    suqa::apply_cx(bm_spin[0], bm_spin[1]);
    suqa::apply_cx(bm_spin[0], bm_spin[2]);
    suqa::apply_u1(bm_spin[2], M_PI * 0.5);
}

double measure_X(pcg& rgen) {
    std::vector<uint> bits(3);
    measure_basis_change();
    std::vector<double> r(3);
    for (auto& x : r) x = rgen.doub();
    suqa::measure_qbits(bm_spin, bits, r);
    measure_basis_change();  // the reference undoes the change by repeating it
    uint m = 0U;
    for (uint i = 0; i < 3; ++i) m |= (bits[i] << i);
    return k_observable[m];
}

static const std::vector<double> k_weights = {1. / 3, 2. / 3, 1.0};

void apply_C(const uint& Ci) {
    if (Ci > 2) throw std::runtime_error("ERROR: wrong move selection");
    suqa::apply_h(bm_spin[Ci]);
}

void apply_C_inverse(const uint& Ci) { apply_C(Ci); }

void qsa_apply_C(const uint& Ci) {
    if (Ci > 2) throw std::runtime_error("ERROR: wrong move selection");
    suqa::apply_h(bm_spin_tilde[Ci]);
}

void qsa_apply_C_inverse(const uint& Ci) {
    if (Ci > 2) throw std::runtime_error("ERROR: wrong move selection");
    suqa::apply_h(bm_spin_tilde[Ci]);
}

std::vector<double> get_C_weigthsums() { return k_weights; }
