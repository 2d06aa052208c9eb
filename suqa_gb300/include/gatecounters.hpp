// Gate-cost counters with the interface of the reference's
// include/gatecounters.hpp (GateRecord, GateCounter, GateCounterList), so
// drivers built with -DGATECOUNT register counters and get the same tables.
// The cost model is the reference's: a gate under n set control bits costs an
// n-controlled Toffoli, counted in one-qubit (ng1) and two-qubit (ng2) gates as
//   n = 0: 1 one-qubit gate;   n = 1: 1 CNOT;   n = 2: 9 one-qubit + 6 CNOT;
//   n >= 3: 2n-3 two-control Toffolis plus a CNOT.
// The engine always counts (into no counter unless a driver registers one), so
// the shim does not depend on how the driver was compiled.
#pragma once
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

typedef unsigned int uint;

struct GateRecord {
    uint ng1 = 0;  // one-qubit gates
    uint ng2 = 0;  // two-qubit gates
    GateRecord(uint g1 = 0, uint g2 = 0) : ng1(g1), ng2(g2) {}
};

class GateCounter {
public:
    std::string name;
    std::vector<GateRecord> grecords;
    bool active = false;

    explicit GateCounter(std::string n) : name(std::move(n)) {}

    void increment_g1g2(uint g1, uint g2) {
        if (!active) return;
        grecords.back().ng1 += g1;
        grecords.back().ng2 += g2;
    }
    void increment_g1g2(const GateRecord& gr) { increment_g1g2(gr.ng1, gr.ng2); }

    void new_record() {
        active = true;
        grecords.emplace_back();
    }
    void activate() { new_record(); }
    void deactivate() { active = false; }
    void clear() {
        active = false;
        grecords.clear();
    }

    static GateRecord n_ctrl_toffoli_gates(uint n) {
        if (n == 0) return GateRecord(1, 0);
        if (n == 1) return GateRecord(0, 1);
        if (n == 2) return GateRecord(9, 6);
        return GateRecord(9 * (2 * n - 3), 6 * (2 * n - 3) + 1);
    }

    // mean and standard error of ng1, ng2 over the records (records treated as
    // independent; the squares are formed in 32-bit unsigned arithmetic, as the
    // reference does)
    void get_info(double& mean1, double& err1, double& mean2, double& err2, size_t& iters) const {
        iters = grecords.size();
        double s1 = 0, s2 = 0, q1 = 0, q2 = 0;
        for (const GateRecord& r : grecords) {
            s1 += r.ng1;
            s2 += r.ng2;
            q1 += (uint)(r.ng1 * r.ng1);
            q2 += (uint)(r.ng2 * r.ng2);
        }
        mean1 = iters ? s1 / (double)iters : 0.0;
        mean2 = iters ? s2 / (double)iters : 0.0;
        err1 = err2 = 0.0;
        if (iters > 1) {
            err1 = std::sqrt(std::fabs(q1 / (double)iters - mean1 * mean1) / (iters - 1.0));
            err2 = std::sqrt(std::fabs(q2 / (double)iters - mean2 * mean2) / (iters - 1.0));
            if (err1 < 1e-10) err1 = 0.0;
            if (err2 < 1e-10) err2 = 0.0;
        }
    }
};

class GateCounterList {
public:
    uint gc_mask_set_qbits = 0;
    std::vector<GateCounter*> counters;

    void add_counter(GateCounter* c) { counters.push_back(c); }
    void increment_g1g2(uint g1, uint g2) {
        for (GateCounter* c : counters) c->increment_g1g2(g1, g2);
    }
    void increment_g1g2(const GateRecord& gr) { increment_g1g2(gr.ng1, gr.ng2); }
    // the number of control bits later gates see (taken when the mask changes)
    void update_cmask_setbits(uint cmask) {
        uint n = 0;
        for (; cmask; cmask &= cmask - 1u) ++n;
        gc_mask_set_qbits = n;
    }

    void print_counts() const {
        if (counters.empty()) return;
        printf("\n\nGate counts\n");
        printf("\n%-15s  %-9s  %-9s  %-9s  %-9s  %-9s  %-9s  %-9s\n", "counter name", "records", "tot_ng1", "<ng1>",
               "d<ng1>", "tot_ng2", "<ng2>", "<dng2>");
        for (const GateCounter* c : counters) {
            double m1, e1, m2, e2;
            size_t n;
            c->get_info(m1, e1, m2, e2, n);
            printf("%-15s  %-9zu  %-9u  %-9.3lg  %-9.3lg  %-9u  %-9.3lg  %-9.3lg\n", c->name.c_str(), n,
                   (uint)std::round(m1 * n), m1, e1, (uint)std::round(m2 * n), m2, e2);
        }
        printf("\n");
    }

    void print_counts_detailed() const {
        if (counters.empty()) return;
        printf("\n\nDetailed gate counts\n");
        for (const GateCounter* c : counters) {
            printf("\ngate counter '%s' (%zu records):\n", c->name.c_str(), c->grecords.size());
            uint k = 0;
            for (const GateRecord& r : c->grecords) printf("record %u: ng1=%u, ng2=%u\n", k++, r.ng1, r.ng2);
        }
        printf("\n");
    }
};
