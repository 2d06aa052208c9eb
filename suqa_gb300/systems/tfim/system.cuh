// System-plugin interface for a transverse-field Ising ring of TFIM_SPINS spins
// (the plugin API of the reference's include/system.cuh:17-40; the spin count is
// a compile-time constant there, so one driver is built per ring length).
#pragma once
#include <stdexcept>
#include <vector>
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
