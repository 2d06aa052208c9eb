// Transverse-field Ising ring, H = -J sum_i Z_i Z_{i+1} - h sum_i X_i (periodic),
// written against the reference's system-plugin API (src/system.cu:6-151 is the
// triangle instance of the same API).  Used to build the reference CPU qms driver
// for the batched-chain workload; J and h come from the environment (TFIM_J,
// TFIM_H; defaults 1.0 and 1.0) because the reference CLI has no slot for them.
//
// evolution(t) applies exp(-iHt) as ceil(|t|/dt) first-order Trotter steps of
// width dt = 0.1: each step is exp(i J d Z_i Z_{i+1}) for every bond, then
// exp(i h d X_i) for every spin, each through apply_pauli_TP_rotation (which
// applies exp(i phase P)).  Moves: Hadamard on spin i with probability 1/s.
// Observable ("A" column): magnetisation sum_i (1 - 2 b_i) read in the Z basis.
#include <cmath>
#include <cstdlib>
#include "system.cuh"
#include "Rand.hpp"

static bmReg make_spins() {
    bmReg r(TFIM_SPINS);
    for (int i = 0; i < TFIM_SPINS; ++i) r[i] = (uint)i;
    return r;
}
const bmReg bm_spin = make_spins();

static double env_or(const char* name, double dflt) {
    const char* v = std::getenv(name);
    return v ? std::strtod(v, nullptr) : dflt;
}

static const double tfim_J = env_or("TFIM_J", 1.0);
static const double tfim_h = env_or("TFIM_H", 1.0);
static const double tfim_dt = 0.1;

void init_state() {
    suqa::init_state();
}

void evolution(const double& t, const int& n) {
    (void)n;
    const double at = std::fabs(t);
    int steps = (int)std::ceil(at / tfim_dt - 1e-9);
    if (steps < 1) steps = 1;
    const double d = t / (double)steps;
    for (int k = 0; k < steps; ++k) {
        for (int i = 0; i < TFIM_SPINS; ++i) {
            const uint a = bm_spin[i], b = bm_spin[(i + 1) % TFIM_SPINS];
            suqa::apply_pauli_TP_rotation({a, b}, {PAULI_Z, PAULI_Z}, tfim_J * d);
        }
        for (int i = 0; i < TFIM_SPINS; ++i)
            suqa::apply_pauli_TP_rotation({bm_spin[i]}, {PAULI_X}, tfim_h * d);
    }
}

double measure_X(pcg& rgen) {
    std::vector<double> rd(TFIM_SPINS);
    for (auto& r : rd) r = rgen.doub();
    std::vector<uint> cs(TFIM_SPINS, 0U);
    suqa::measure_qbits(bm_spin, cs, rd);
    double m = 0.0;
    for (int i = 0; i < TFIM_SPINS; ++i) m += cs[i] ? -1.0 : 1.0;
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
