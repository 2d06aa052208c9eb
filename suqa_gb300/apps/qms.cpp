// qms: quantum Metropolis sampling of the configured system on the GB300 engine.
//
// Output contract (shared with the reference CPU build, so that analysis
// scripts and the parity tests read both the same way):
//   * <out>: a "# E A" header when the file does not exist yet, then one
//     "%.16lg %.16lg" row per sample (energy, observable).  Samples are written
//     in chunks, at the steps s with s % ceil(steps / 20) == 0; samples taken
//     after the last such step are not written.
//   * stdout: an "acceptance: <percent>%" line ("%3.2lg" of the accepted share).
//   * <out>_revcounts with --record-reverse: "<attempt> <count>" per line.
//   * A failed restoration (metro_step < 0) restarts the chain from the initial
//     state, and the thermalisation window starts again after it.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "Rand.hpp"
#include "io.hpp"
#include "parser_qms.hpp"
#include "qms.cuh"
#include "suqa.cuh"
#include "system.cuh"

#ifdef GATECOUNT
// cost-table rows, in the order the table lists them
GateCounter gctr_global("global");
GateCounter gctr_metrostep("metro step");
GateCounter gctr_sample("sample");
GateCounter gctr_measure("measure");
GateCounter gctr_reverse("reverse");
#endif

namespace {

const char* kUsage =
    "usage: %s BETA STEPS RESET_EACH ENE_QBITS OUTFILE [--seed S] [--ene-min E0 (0.0)] [--ene-max E1 (1.0)]\n"
    "          [--max-reverse N (100)] [--PE-steps N (10)] [--thermalization N (100)] [--record-reverse]\n"
    "  Quantum Metropolis sampling at inverse temperature BETA for STEPS steps; a sample every\n"
    "  RESET_EACH steps after thermalisation; ENE_QBITS qubits of phase estimation on [E0, E1].\n";

constexpr double kTwoPi = 6.283185307179586476925286766559;

// Register sizes and phase-estimation scaling for the run, into the qms:: globals
// the algorithm header reads.
void configure(const arg_list& a) {
    qms::metro_steps = (uint)a.metro_steps;
    qms::reset_each = (uint)a.reset_each;
    qms::ene_qbits = (uint)a.ene_qbits;
    qms::max_reverse_attempts = (uint)a.max_reverse_attempts;
    qms::n_phase_estimation = a.pe_steps;
    qms::record_reverse = a.record_reverse;

    if (a.seed > 0) qms::rangen.set_seed(a.seed);  // otherwise the generator's own seed
    qms::iseed = qms::rangen.get_seed();

    qms::syst_qbits = (uint)syst_qbits;
    qms::nqubits = qms::syst_qbits + qms::ene_qbits + 1;  // + the acceptance qubit
    qms::Dim = 1U << qms::nqubits;
    qms::ene_levels = 1U << qms::ene_qbits;
    qms::syst_levels = 1U << qms::syst_qbits;

    // the register's 2^k levels span [E0, E1] with spacing (E1-E0)/(2^k-1)
    const double levels = (double)qms::ene_levels;
    qms::t_PE_shift = a.ene_min;
    qms::t_PE_factor = (levels - 1.0) / (levels * (a.ene_max - a.ene_min));
    qms::t_phase_estimation = kTwoPi * qms::t_PE_factor;
}

// The "# E A" sample file: samples collected by qms::metro_step are appended in
// chunks and removed from the in-memory lists.
class SampleLog {
public:
    explicit SampleLog(std::string path) : path_(std::move(path)) {
        if (!file_exists(path_.c_str())) write("w", "# E A\n");
    }
    void flush() {
        std::string rows;
        char buf[96];
        for (size_t i = 0; i < qms::E_measures.size(); ++i) {
            std::snprintf(buf, sizeof buf, "%.16lg %.16lg\n", qms::E_measures[i], qms::X_measures[i]);
            rows += buf;
        }
        write("a", rows);
        qms::E_measures.clear();
        qms::X_measures.clear();
    }

private:
    void write(const char* mode, const std::string& text) const {
        FILE* f = std::fopen(path_.c_str(), mode);
        if (!f) {
            std::fprintf(stderr, "qms: cannot write %s\n", path_.c_str());
            std::exit(2);
        }
        std::fputs(text.c_str(), f);
        std::fclose(f);
    }
    std::string path_;
};

// Runs the chain; returns the number of accepted moves.
uint run_chain(SampleLog& log, uint thermalization) {
    const uint steps = qms::metro_steps;
    const uint chunk = (steps + 19U) / 20U;  // about 5 % of the run per write
    uint accepted = 0U, since = 0U;          // `since`: first step after the last restart
    for (uint s = 0U; s < steps; ++s) {
        const uint age = s - since;
        const bool sample_now = s > since + thermalization && age % qms::reset_each == 0U;
        const int outcome = qms::metro_step(sample_now);
        if (outcome == 1 || outcome == 2) ++accepted;
        if (outcome < 0) {  // restoration failed: back to the initial state, thermalise again
            init_state();
            since = s + 1U;
        }
        if (s % chunk == 0U) {
            std::printf("step %u of %u\n", s, steps);
            log.flush();
        }
    }
    return accepted;
}

void write_reverse_counts(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return;
    for (size_t i = 0; i < qms::reverse_counters.size(); ++i)
        std::fprintf(f, "%d %d\n", (int)i, (int)qms::reverse_counters[i]);
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
    configure(args);
    suqa::print_banner();
    std::cout << "arguments:\n" << args << std::endl;
    const auto start = std::chrono::steady_clock::now();

    suqa::setup(qms::nqubits);
    qms::setup(args.beta);
#ifdef GATECOUNT
    for (GateCounter* c : {&gctr_global, &gctr_metrostep, &gctr_sample, &gctr_measure, &gctr_reverse})
        suqa::gatecounters.add_counter(c);
    gctr_global.new_record();
    gctr_sample.new_record();
#endif
    init_state();

    SampleLog log(args.outfile);
    const auto loop0 = std::chrono::steady_clock::now();
    const uint accepted = run_chain(log, (uint)args.thermalization);
    // the Metropolis loop alone (no process start, device set-up or initial state)
    std::printf("chain loop: %u steps in %.6f s\n", qms::metro_steps,
                std::chrono::duration<double>(std::chrono::steady_clock::now() - loop0).count());
    // the share first, then the percentage: the printed digits depend on the rounding order
    std::printf("\n\tacceptance: %3.2lg%%\n", (accepted / (double)qms::metro_steps) * 100.0);

    qms::clear();
    suqa::clear();
    if (qms::record_reverse) write_reverse_counts(args.outfile + "_revcounts");
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    std::printf("done in %.3f s\n", secs);
    return 0;
}
