// qms driver on the suqa_gb300 engine: command line, output file ("# E A" then
// "%.16lg %.16lg" rows appended about every 5% of the steps), re-initialisation
// after a failed restoration, acceptance report and the optional
// "<out>_revcounts" file follow the reference's src/qms.cu.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>
#include "Rand.hpp"
#include "io.hpp"
#include "parser_qms.hpp"
#include "suqa.cuh"
#include "system.cuh"
#include "qms.cuh"

#ifdef GATECOUNT
// gate-cost counters, registered as src/qms.cu:33-39, 97-106 does
GateCounter gctr_global("global");
GateCounter gctr_metrostep("metro step");
GateCounter gctr_sample("sample");
GateCounter gctr_measure("measure");
GateCounter gctr_reverse("reverse");
#endif

static void save_measures(const std::string& path) {
    FILE* f = fopen(path.c_str(), "a");
    for (uint i = 0; i < qms::E_measures.size(); ++i)
        fprintf(f, "%.16lg %.16lg\n", qms::E_measures[i], qms::X_measures[i]);
    fclose(f);
    qms::E_measures.clear();
    qms::X_measures.clear();
}

int main(int argc, char** argv) {
    if (argc < 6) {
        printf("usage: %s <beta> <metro steps> <reset each> <num ene qbits> <output file path> "
               "[--max-reverse <max reverse attempts> (100)] [--seed <seed> (random)] [--ene-min <min energy> (0.0)] "
               "[--ene-max <max energy> (1.0)] [--PE-steps <steps of PE evolution> (10)] "
               "[--thermalization <steps> (100)] [--record-reverse]\n",
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
    const double beta = args.beta;
    const int thermalization = args.thermalization;
    qms::metro_steps = (uint)args.metro_steps;
    qms::reset_each = (uint)args.reset_each;
    qms::ene_qbits = (uint)args.ene_qbits;
    const std::string out = args.outfile;
    qms::max_reverse_attempts = (uint)args.max_reverse_attempts;
    qms::n_phase_estimation = args.pe_steps;
    qms::record_reverse = args.record_reverse;
    qms::iseed = args.seed;
    if (qms::iseed > 0) qms::rangen.set_seed(qms::iseed);
    qms::iseed = qms::rangen.get_seed();

    qms::syst_qbits = (uint)syst_qbits;
    qms::nqubits = qms::syst_qbits + qms::ene_qbits + 1;
    std::cout << qms::nqubits << std::endl;
    qms::Dim = (1U << qms::nqubits);
    qms::ene_levels = (1U << qms::ene_qbits);
    qms::syst_levels = (1U << qms::syst_qbits);
    qms::t_PE_shift = args.ene_min;
    qms::t_PE_factor = (qms::ene_levels - 1) / (double)(qms::ene_levels * (args.ene_max - args.ene_min));
    qms::t_phase_estimation = qms::t_PE_factor * 8. * atan(1.0);  // 2 pi t_PE_factor

    suqa::print_banner();
    std::cout << "arguments:\n" << args << std::endl;
    const auto t0 = std::chrono::high_resolution_clock::now();

    suqa::setup(qms::nqubits);
    qms::setup(beta);
#ifdef GATECOUNT
    for (GateCounter* c : {&gctr_global, &gctr_metrostep, &gctr_sample, &gctr_measure, &gctr_reverse})
        suqa::gatecounters.add_counter(c);
    gctr_global.new_record();
    gctr_sample.new_record();
#endif
    init_state();

    const uint save_every = (qms::metro_steps + 19) / 20;
    uint accepted = 0U;
    if (!file_exists(out.c_str())) {
        FILE* f = fopen(out.c_str(), "w");
        fprintf(f, "# E A\n");
        fclose(f);
    }
    uint s0 = 0U;
    for (uint s = 0U; s < qms::metro_steps; ++s) {
        const bool take_measure = (s > s0 + (uint)thermalization && (s - s0) % qms::reset_each == 0U);
        const int ret = qms::metro_step(take_measure);
        if (ret < 0) {  // restoration failed: start again from the initial state
            init_state();
            s0 = s + 1;
        }
        if (ret == 1 || ret == 2) accepted++;
        if (s % save_every == 0) {
            std::cout << "iteration: " << s << "/" << qms::metro_steps << std::endl;
            save_measures(out);
        }
    }
    printf("\n\tacceptance: %3.2lg%%\n", (accepted / static_cast<double>(qms::metro_steps)) * 100.0);

    qms::clear();
    suqa::clear();
    if (qms::record_reverse) {
        FILE* f = fopen((out + "_revcounts").c_str(), "w");
        for (uint i = 0; i < qms::reverse_counters.size(); ++i)
            fprintf(f, "%d %d\n", i, static_cast<int>(qms::reverse_counters[i]));
        fclose(f);
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    std::cout << "All [DONE] in " << std::chrono::duration<double>(t1 - t0).count() << " seconds" << std::endl;
    return 0;
}
