// qsa driver on the suqa_gb300 engine: sampling loop with annealing restarts,
// final energy read-out and observable, output rows "%.16lg\t%.16lg\t%d" (E, A,
// restarts so far), as the reference's src/qsa.cu.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>
#include "Rand.hpp"
#include "io.hpp"
#include "parser_qsa.hpp"
#include "suqa.cuh"
#include "system.cuh"
#include "qsa.cuh"

#ifdef GATECOUNT
// gate-cost counters, placed as src/qsa.cu:33-39, 130-137, 160-264 places them
GateCounter gctr_global("global");
GateCounter gctr_annstep("ann. step");
GateCounter gctr_annealing("annealing");
GateCounter gctr_sample("sample");
GateCounter gctr_measure("measure");
#endif

static void save_measures(const std::string& path, int rej) {
    FILE* f = fopen(path.c_str(), "a");
    for (uint i = 0; i < qsa::E_measures.size(); ++i)
        fprintf(f, "%.16lg\t%.16lg\t%d\n", qsa::E_measures[i], qsa::X_measures[i], rej);
    fclose(f);
    qsa::E_measures.clear();
    qsa::X_measures.clear();
}

int main(int argc, char** argv) {
    if (argc < 6) {
        printf("usage: %s <beta> <sampling> <num ene qbits> <num szegedy qbits> <output file path>  "
               "[--seed <seed> (random)] [--annealing-sequences (100)]\n",
               argv[0]);
        return 1;
    }
    arg_list args;
    try {
        parse_arguments(args, argc, argv);
    } catch (const char* e) {
        fprintf(stderr, "%s\n", e);
        return 1;
    }
    qsa::beta = args.beta;
    qsa::ene_qbits = (uint)args.ene_qbits;
    qsa::szegedy_qbits = (uint)args.szegedy_qbits;
    const std::string out = args.outfile;
    qsa::n_phase_estimation = args.pe_steps;
    qsa::iseed = args.seed;
    const uint sampling = args.sampling;
    const uint annealing_sequences = args.annealing_sequences;
    if (qsa::iseed > 0) qsa::rangen.set_seed(qsa::iseed);
    qsa::iseed = qsa::rangen.get_seed();

    qsa::syst_qbits = (uint)syst_qbits;
    qsa::nqubits = qsa::syst_qbits + qsa::ene_qbits + qsa::szegedy_qbits + 1;
    qsa::Dim = (1U << qsa::nqubits);
    qsa::ene_levels = (1U << qsa::ene_qbits);
    const double szegedy_levels = (1U << qsa::szegedy_qbits);
    qsa::t_PE_shift = args.ene_min;
    qsa::t_PE_factor = (qsa::ene_levels - 1) / (double)(qsa::ene_levels * (args.ene_max - args.ene_min));
    qsa::t_phase_estimation = qsa::t_PE_factor * 8. * atan(1.0);
    qsa::t_PE_shift_szegedy = args.ene_min_szegedy;
    qsa::t_PE_factor_szegedy = (szegedy_levels - 1) / (double)((szegedy_levels) * (args.ene_max_szegedy - args.ene_min_szegedy));
    qsa::t_phase_estimation_szegedy = qsa::t_PE_factor_szegedy * 8. * atan(1.0);

    suqa::print_banner();
    std::cout << "arguments:\n" << args << std::endl;
    const auto t0 = std::chrono::high_resolution_clock::now();
    suqa::setup(qsa::nqubits);
    qsa::setup();

    if (!file_exists(out.c_str())) {
        FILE* f = fopen(out.c_str(), "w");
        fprintf(f, "# E A\n");
        fclose(f);
    }
#ifdef GATECOUNT
    for (GateCounter* c : {&gctr_global, &gctr_annstep, &gctr_annealing, &gctr_sample, &gctr_measure})
        suqa::gatecounters.add_counter(c);
    gctr_global.new_record();
#endif

    int rejection = 0, rejection1 = 0, itctr = 0;
    double mean = 0.0, sq = 0.0;
    const double beta_i = qsa::beta / ((double)annealing_sequences);
    for (uint sample = 0; sample < sampling;) {
#ifdef GATECOUNT
        gctr_sample.new_record();
        gctr_annealing.new_record();
#endif
        std::vector<uint> c_test(qsa::szegedy_qbits, 0), c_E(qsa::szegedy_qbits, 0);
        uint c_ac = 0U;
        bool done = false;
        while (!done) {
            bool restart = false;
            uint move = qsa::draw_C();
            qsa::reset_non_syst_qbits();
            qsa_init_state();
            for (uint s = 0U; s < annealing_sequences; s++) {
#ifdef GATECOUNT
                gctr_annstep.new_record();
#endif
                move = qsa::draw_C();
                qsa::apply_PE_szegedy(qsa::bm_states, qsa::bm_szegedy, (double)(s + 1) * beta_i, move);
                suqa::measure_qbits(qsa::bm_szegedy, c_test, qsa::extract_rands(qsa::szegedy_qbits));
#ifdef GATECOUNT
                gctr_annstep.deactivate();
#endif
                if (qsa::creg_to_uint(c_test) != 0U) {  // left the stationary subspace: restart
                    restart = true;
                    rejection1++;
                    printf("break after %d steps   eigenvalue:%d   \n", s, qsa::creg_to_uint(c_test));
                    break;
                }
            }
            if (!restart) done = true;
        }
#ifdef GATECOUNT
        gctr_annealing.deactivate();
#endif
        if (c_ac == 0U) {
#ifdef GATECOUNT
            gctr_measure.new_record();
#endif
            qsa::apply_phase_estimation_measure(qsa::bm_states, qsa::bm_szegedy, qsa::t_phase_estimation_szegedy,
                                                qsa::n_phase_estimation);
            suqa::measure_qbits(qsa::bm_szegedy, c_E, qsa::extract_rands(qsa::szegedy_qbits));
            const double E = qsa::t_PE_shift_szegedy +
                             qsa::creg_to_uint(c_E) / (double)(qsa::t_PE_factor_szegedy * szegedy_levels);
            printf("measured eigenvalue:%f\n", E);
            itctr++;
            mean += E;
            sq += E * E;
            if (itctr > 1)
                printf("mean=%f, std=%f; expected mean=%f\n", mean / itctr,
                       sqrt((sq - mean * mean / itctr) / ((itctr) * (itctr - 1))),
                       (6 - 6 * exp(4 * qsa::beta)) / (2 + 6 * exp(4 * qsa::beta)));
            qsa::E_measures.push_back(E);
            qsa::X_measures.push_back(measure_X(qsa::rangen));
            std::cout << "iteration: " << sample + 1 << "/" << sampling << std::endl;
            save_measures(out, rejection1);
#ifdef GATECOUNT
            gctr_measure.deactivate();
#endif
            ++sample;
        } else {
            rejection++;
        }
    }
    printf("n of rejection step cause by acceptance qubit= %d\n", rejection);
    printf("n of rejection step cause by energy qubits= %d\n", rejection1);
    qsa::clear();
    suqa::clear();
    const auto t1 = std::chrono::high_resolution_clock::now();
    std::cout << "All [DONE] in " << std::chrono::duration<double>(t1 - t0).count() << " seconds" << std::endl;
    return 0;
}
