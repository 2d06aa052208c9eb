// Transverse-field Ising ring, H = -J sum_i Z_i Z_{i+1} - h sum_i X_i (periodic),
// as a system plugin of the suqa_gb300 drop-in headers.  J and h come from the
// environment (TFIM_J, TFIM_H; default 1.0) because the qms command line has no
// slot for them.  evolution(t) = exp(-iHt) as ceil(|t|/dt) first-order Trotter
// steps (dt = 0.1): exp(i J d Z_i Z_{i+1}) on every bond, then exp(i h d X_i) on
// every spin.  Moves: Hadamard on spin i with probability 1/s.  Observable:
// magnetisation sum_i (1 - 2 b_i) read in the Z basis.  The batched device
// engine (sq_qms_tfim_batch) runs the same system.
#include <cmath>
#include <cstdlib>
#include "Rand.hpp"
#include "system.cuh"

static bmReg ring() {
    bmReg r(TFIM_SPINS);
    for (int i = 0; i < TFIM_SPINS; ++i) r[i] = (uint)i;
    return r;
}
const bmReg bm_spin = ring();

static double env_param(const char* name) {
    const char* v = std::getenv(name);
    return v ? std::strtod(v, nullptr) : 1.0;
}
static const double kJ = env_param("TFIM_J");
static const double kH = env_param("TFIM_H");
static const double kDt = 0.1;

void init_state() { suqa::init_state(); }

void evolution(const double& t, const int& n) {
    (void)n;
    int steps = (int)std::ceil(std::fabs(t) / kDt - 1e-9);
    if (steps < 1) steps = 1;
    const double d = t / (double)steps;
    for (int k = 0; k < steps; ++k) {
        for (int i = 0; i < TFIM_SPINS; ++i)
            suqa::apply_pauli_TP_rotation({bm_spin[i], bm_spin[(i + 1) % TFIM_SPINS]}, {PAULI_Z, PAULI_Z}, kJ * d);
        for (int i = 0; i < TFIM_SPINS; ++i) suqa::apply_pauli_TP_rotation({bm_spin[i]}, {PAULI_X}, kH * d);
    }
}

double measure_X(pcg& rgen) {
    std::vector<double> r(TFIM_SPINS);
    for (auto& x : r) x = rgen.doub();
    std::vector<uint> bits(TFIM_SPINS, 0U);
    suqa::measure_qbits(bm_spin, bits, r);
    double m = 0.0;
    for (int i = 0; i < TFIM_SPINS; ++i) m += bits[i] ? -1.0 : 1.0;
    return m;
}

void apply_C(const uint& Ci) {
    if (Ci >= (uint)TFIM_SPINS) throw std::runtime_error("ERROR: wrong move selection");
    suqa::apply_h(bm_spin[Ci]);
}

void apply_C_inverse(const uint& Ci) { apply_C(Ci); }

std::vector<double> get_C_weigthsums() {
    std::vector<double> w(TFIM_SPINS);
    for (int i = 0; i < TFIM_SPINS; ++i) w[i] = (i + 1 == TFIM_SPINS) ? 1.0 : (double)(i + 1) / (double)TFIM_SPINS;
    return w;
}
