// Drop-in replacement of the reference's include/suqa.cuh: the suqa:: gate API
// (include/suqa.cuh:94-176 there) with the same names, overloads, default
// arguments, globals and macros, implemented over the libsq C ABI
// (include/sq.h).  suqa::state's data pointers are device pointers owned by the
// engine; gates are queued and applied lazily by libsq, and every call that
// reads the state (measurements, prob_filter, vnorm) applies them first.
#pragma once
#include <algorithm>
#include <bitset>
#include <iostream>
#include <stdexcept>
#include <stdio.h>
#include <vector>
#include "io.hpp"
#include "complex_defines.cuh"
#include "gatecounters.hpp"
#include "sq.h"
#ifdef GPU
#include <cuda_runtime.h>
#endif

#define TWOSQINV 0.7071067811865475

typedef std::vector<uint> bmReg;
#define PAULI_ID 0
#define PAULI_X 1
#define PAULI_Y 2
#define PAULI_Z 3

#ifndef NDEBUG
#define DEBUG_READ_STATE() \
    { suqa::debug_print_state(); }
#else
#define DEBUG_READ_STATE()
#endif

namespace suqa {

extern ComplexVec state;
// gate-cost counters (reference include/gatecounters.hpp); drivers built with
// -DGATECOUNT register their counters here
extern GateCounterList gatecounters;

#ifdef GPU
#define NUM_THREADS 128
#define MAXBLOCKS 65535
extern uint blocks, threads;
extern cudaStream_t stream1, stream2;
#endif

// global control mask: every following gate is controlled on its set bits
extern uint gc_mask;
extern uint nq;

extern std::vector<double> rphase_m;  // for the QFT

void print_banner();

void activate_gc_mask(const bmReg& q_controls);
void deactivate_gc_mask(const bmReg& q_controls);

double vnorm();
void vnormalize();

void init_state();

void deallocate_state();
void allocate_state(uint Dim);

void apply_x(uint q);
void apply_x(const bmReg& qs);
void apply_y(uint q);
void apply_y(const bmReg& qs);
void apply_z(uint q);
void apply_z(const bmReg& qs);
void apply_h(uint q);
void apply_h(const bmReg& qs);
void apply_t(uint q);
void apply_t(const bmReg& qs);
void apply_tdg(uint q);
void apply_tdg(const bmReg& qs);
void apply_s(uint q);
void apply_s(const bmReg& qs);

void apply_u1(uint q, double phase);
void apply_u1(uint q, uint q_mask, double phase);

void apply_cx(const uint& q_control, const uint& q_target, const uint& q_mask = 1U);
void apply_mcx(const bmReg& q_controls, const uint& q_target);
void apply_mcx(const bmReg& q_controls, const bmReg& q_mask, const uint& q_target);

void apply_cu1(uint q_control, uint q_target, double phase, uint q_mask = 1U);
void apply_mcu1(const bmReg& q_controls, const uint& q_target, double phase);
void apply_mcu1(const bmReg& q_controls, const bmReg& q_mask, const uint& q_target, double phase);

void apply_swap(const uint& q1, const uint& q2);

void apply_phase_list(uint q0, uint q_size, const std::vector<double>& phases);

void apply_pauli_TP_rotation(const bmReg& q_apply, const std::vector<uint>& pauli_TPconst, double phase);

void apply_qft(const std::vector<uint>& qact);
void apply_qft_inverse(const std::vector<uint>& qact);

void measure_qbit(uint q, uint& c, double rdoub);
void measure_qbits(const bmReg& qs, std::vector<uint>& cs, const std::vector<double>& rdoubs);

void apply_reset(uint q, double rdoub);
void apply_reset(const bmReg& qs, std::vector<double> rdoubs);

void prob_filter(const bmReg& qs, const std::vector<uint>& q_mask, double& prob);

void setup(uint nq);
void clear();

// ---- extensions (no reference counterpart) ----
// The engine state behind suqa::state (for direct libsq calls).
sq_state* engine();
// Amplitude precision used by the next setup(): SQ_F64 (default) or SQ_F32.
// The SUQA_PRECISION environment variable ("f32"/"f64") sets the default.
void set_precision(int precision);
// exp(i phase P) for any Pauli string (the reference supports only a subset).
void apply_pauli_rotation(const bmReg& q_apply, const std::vector<uint>& paulis, double phase);
// Debug dump used by DEBUG_READ_STATE (copies the state to the host).
void debug_print_state();

};  // namespace suqa
