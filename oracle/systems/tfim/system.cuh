// Transverse-field Ising ring plugin header for the reference's system-plugin API
// (the reference's include/system.cuh:17-40 declares the same names for its
// 3-spin triangle).  Project-written; the spin count is fixed at compile time by
// -DTFIM_SPINS=s because the reference drivers read syst_qbits as a constant.
#pragma once
#include <vector>
#include <stdexcept>
#include "io.hpp"
#include "suqa.cuh"

#ifndef TFIM_SPINS
#define TFIM_SPINS 4
#endif

const int syst_qbits = TFIM_SPINS;
extern const bmReg bm_spin;

void init_state();
void evolution(const double& t, const int& n);
void apply_C(const uint& Ci);
void apply_C_inverse(const uint& Ci);
std::vector<double> get_C_weigthsums();
