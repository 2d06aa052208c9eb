// evo driver on the suqa_gb300 engine: for t = 0, dt, ..., total_steps*dt the
// system is re-initialised, evolved by exp(-iHt) and the 8 basis probabilities
// of the spins are appended as "%.12lg" x 9 rows (t, p000, p100, p010, p110,
// p001, p101, p011, p111), as the reference's src/evo.cu.
#include <cstdio>
#include <cstdlib>
#include <string>
#include "Rand.hpp"
#include "io.hpp"
#include "suqa.cuh"
#include "system.cuh"

int main(int argc, char** argv) {
    if (argc < 4) {
        printf("usage: %s <total_steps> <trotter_stepsize> <outfile>\n", argv[0]);
        return 1;
    }
    const int total_steps = atoi(argv[1]);
    const double dt = std::stod(argv[2]);
    const std::string out = argv[3];
    suqa::setup(syst_qbits);
    printf("arguments:\n total_steps = %d\n trotter_stepsize = %.16lg\n outfile = %s\n\n", total_steps, dt, out.c_str());
    init_state();
    const std::vector<std::vector<uint>> patterns = {{0U, 0U, 0U}, {1U, 0U, 0U}, {0U, 1U, 0U}, {1U, 1U, 0U},
                                                     {0U, 0U, 1U}, {1U, 0U, 1U}, {0U, 1U, 1U}, {1U, 1U, 1U}};
    for (uint ii = 0; ii <= (uint)total_steps; ++ii) {
        const double t = ii * dt;
        init_state();
        evolution(t, ii);
        double p[8];
        for (int k = 0; k < 8; ++k) suqa::prob_filter(bm_spin, patterns[k], p[k]);
        FILE* f = fopen(out.c_str(), "a");
        fprintf(f, "%.12lg %.12lg %.12lg %.12lg %.12lg %.12lg %.12lg %.12lg %.12lg\n", t, p[0], p[1], p[2], p[3], p[4],
                p[5], p[6], p[7]);
        fclose(f);
    }
    suqa::clear();
    return 0;
}
