// System-plugin interface (the reference's include/system.cuh:17-40) for the
// frustrated 3-spin triangle, H = sum over pairs of X_i X_j: the compile-time
// register layout and the functions the QMS/QSA headers and drivers call.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>
#include "io.hpp"
#include "suqa.cuh"

const int syst_qbits = 3;  // number of system qubits
const bmReg bm_spin = {0, 1, 2};

void init_state();
void evolution(const double& t, const int& n);
void apply_C(const uint& Ci);
void apply_C_inverse(const uint& Ci);
std::vector<double> get_C_weigthsums();

// QSA specifics (the copy register aliases the energy register in the reference
// layout; kept for drop-in parity)
const bmReg bm_spin_tilde = {3, 4, 5};
void qsa_init_state();
void evolution_szegedy(const double& t, const int& n);
void evolution_measure(const double& t, const int& n);
void evolution_tracing(const double& t, const int& n);
void qsa_apply_C(const uint& Ci);
void qsa_apply_C_inverse(const uint& Ci);
