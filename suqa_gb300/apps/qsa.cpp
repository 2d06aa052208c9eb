// qsa: Szegedy-walk annealing ("quantum-quantum Metropolis") of the configured
// system on the GB300 engine.
//
// One sample = one annealing run plus a read-out.  A run resets the work
// registers, prepares the system's initial state, then walks through the
// stages beta_s = (s+1) beta / stages: per stage it draws a move, applies the
// walk-phase estimation at beta_s and reads the walk-phase register; a nonzero
// read-out means the state left the walk's stationary subspace and the run
// starts over (one restart).  A run that passes every stage is read out: the
// walk-phase estimation of the energy gives E, the system observable A.
//
// Output contract (shared with the reference CPU build): <out> gets a "# E A"
// header when it does not exist yet, then one "%.16lg\t%.16lg\t%d" row per
// sample (E, A, restarts so far over the whole run), written as soon as the
// sample is taken.  The random draws come in the reference's order: one move
// drawn and discarded at the start of every run, then per stage a move and the
// read-out draws.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "Rand.hpp"
#include "io.hpp"
#include "parser_qsa.hpp"
#include "qsa.cuh"
#include "suqa.cuh"
#include "system.cuh"

#ifdef GATECOUNT
// cost-table rows, in the order the table lists them
GateCounter gctr_global("global");
GateCounter gctr_annstep("ann. step");
GateCounter gctr_annealing("annealing");
GateCounter gctr_sample("sample");
GateCounter gctr_measure("measure");
#endif

namespace {

const char* kUsage =
    "usage: %s BETA SAMPLES ENE_QBITS WALK_QBITS OUTFILE [--seed S] [--annealing-sequences N (100)]\n"
    "          [--ene-min E0] [--ene-max E1] [--szegedy-min W0] [--szegedy-max W1] [--PE-steps N]\n"
    "  Anneals to inverse temperature BETA in N stages and reads out SAMPLES energies and observables.\n";

constexpr double kTwoPi = 6.283185307179586476925286766559;

struct Schedule {
    uint samples = 0, stages = 0;
    double walk_levels = 0.0;  // 2^WALK_QBITS
};

// Register sizes and the two phase-estimation scalings, into the qsa:: globals.
Schedule configure(const arg_list& a) {
    qsa::beta = a.beta;
    qsa::ene_qbits = (uint)a.ene_qbits;
    qsa::szegedy_qbits = (uint)a.szegedy_qbits;
    qsa::n_phase_estimation = a.pe_steps;
    if (a.seed > 0) qsa::rangen.set_seed(a.seed);  // otherwise the generator's own seed
    qsa::iseed = qsa::rangen.get_seed();

    qsa::syst_qbits = (uint)syst_qbits;
    qsa::nqubits = qsa::syst_qbits + qsa::ene_qbits + qsa::szegedy_qbits + 1;
    qsa::Dim = 1U << qsa::nqubits;
    qsa::ene_levels = 1U << qsa::ene_qbits;

    Schedule sch;
    sch.samples = (uint)a.sampling;
    sch.stages = (uint)a.annealing_sequences;
    sch.walk_levels = (double)(1U << qsa::szegedy_qbits);
    // each register's levels span its window [lo, hi] with spacing (hi-lo)/(levels-1)
    const double el = (double)qsa::ene_levels;
    qsa::t_PE_shift = a.ene_min;
    qsa::t_PE_factor = (el - 1.0) / (el * (a.ene_max - a.ene_min));
    qsa::t_phase_estimation = kTwoPi * qsa::t_PE_factor;
    const double wl = sch.walk_levels;
    qsa::t_PE_shift_szegedy = a.ene_min_szegedy;
    qsa::t_PE_factor_szegedy = (wl - 1.0) / (wl * (a.ene_max_szegedy - a.ene_min_szegedy));
    qsa::t_phase_estimation_szegedy = kTwoPi * qsa::t_PE_factor_szegedy;
    return sch;
}

// One pass through every annealing stage from a freshly prepared state;
// false when a stage's walk-phase read-out is nonzero.
bool anneal_once(const Schedule& sch, std::vector<uint>& readout) {
    (void)qsa::draw_C();  // drawn and unused, as in the reference's run loop
    qsa::reset_non_syst_qbits();
    qsa_init_state();
    const double dbeta = qsa::beta / (double)sch.stages;
    for (uint s = 0U; s < sch.stages; ++s) {
#ifdef GATECOUNT
        gctr_annstep.new_record();
#endif
        const uint move = qsa::draw_C();
        qsa::apply_PE_szegedy(qsa::bm_states, qsa::bm_szegedy, (double)(s + 1) * dbeta, move);
        suqa::measure_qbits(qsa::bm_szegedy, readout, qsa::extract_rands(qsa::szegedy_qbits));
#ifdef GATECOUNT
        gctr_annstep.deactivate();
#endif
        if (qsa::creg_to_uint(readout) != 0U) {
            std::printf("restart: stage %u read walk phase %u\n", s, qsa::creg_to_uint(readout));
            return false;
        }
    }
    return true;
}

// Energy from the walk-phase register after a completed anneal.
double read_energy(const Schedule& sch) {
    std::vector<uint> bits(qsa::szegedy_qbits, 0U);
    qsa::apply_phase_estimation_measure(qsa::bm_states, qsa::bm_szegedy, qsa::t_phase_estimation_szegedy,
                                        qsa::n_phase_estimation);
    suqa::measure_qbits(qsa::bm_szegedy, bits, qsa::extract_rands(qsa::szegedy_qbits));
    return qsa::t_PE_shift_szegedy + qsa::creg_to_uint(bits) / (double)(qsa::t_PE_factor_szegedy * sch.walk_levels);
}

void append_row(const std::string& path, double E, double A, int restarts) {
    FILE* f = std::fopen(path.c_str(), "a");
    if (!f) {
        std::fprintf(stderr, "qsa: cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fprintf(f, "%.16lg\t%.16lg\t%d\n", E, A, restarts);
    std::fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 6) {
        std::printf(kUsage, argv[0]);
        return 1;
    }
    arg_list args;
    try {
        parse_arguments(args, argc, argv);
    } catch (const char* e) {
        std::fprintf(stderr, "%s\n", e);
        return 1;
    }
    const Schedule sch = configure(args);
    suqa::print_banner();
    std::cout << "arguments:\n" << args << std::endl;
    const auto start = std::chrono::steady_clock::now();

    suqa::setup(qsa::nqubits);
    qsa::setup();
    if (!file_exists(args.outfile.c_str())) {
        FILE* f = std::fopen(args.outfile.c_str(), "w");
        if (!f) {
            std::fprintf(stderr, "qsa: cannot write %s\n", args.outfile.c_str());
            return 2;
        }
        std::fputs("# E A\n", f);
        std::fclose(f);
    }
#ifdef GATECOUNT
    for (GateCounter* c : {&gctr_global, &gctr_annstep, &gctr_annealing, &gctr_sample, &gctr_measure})
        suqa::gatecounters.add_counter(c);
    gctr_global.new_record();
#endif

    std::vector<uint> readout(qsa::szegedy_qbits, 0U);
    int restarts = 0;
    for (uint k = 0; k < sch.samples; ++k) {
#ifdef GATECOUNT
        gctr_sample.new_record();
        gctr_annealing.new_record();
#endif
        while (!anneal_once(sch, readout)) ++restarts;
#ifdef GATECOUNT
        gctr_annealing.deactivate();
        gctr_measure.new_record();
#endif
        const double E = read_energy(sch);
        const double A = measure_X(qsa::rangen);
        append_row(args.outfile, E, A, restarts);
        std::printf("sample %u of %u: E = %f\n", k + 1, sch.samples, E);
#ifdef GATECOUNT
        gctr_measure.deactivate();
#endif
    }
    std::printf("restarts: %d\n", restarts);

    qsa::clear();
    suqa::clear();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    std::printf("done in %.3f s\n", secs);
    return 0;
}
