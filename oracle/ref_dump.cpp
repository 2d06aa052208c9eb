// Golden dumper (test infrastructure, built only where the reference sources are
// present).  Replays a gate script through the reference suqa:: CPU engine
// (src/suqa.cu + include/suqa_cpu.hpp, dense release build) and writes every
// observable result at full precision (C99 hex floats) to the file in argv[1].
//
// Script grammar, one command per line (qubit lists are prefixed by their count):
//   setup n | init | vnorm | normalize | dump
//   setstate            (next line: 2^n re values then 2^n im values, hex floats)
//   gc_on k q..  | gc_off k q..
//   x q | y q | z q | h q | s q | t q | tdg q
//   u1 q phase | u1m q qmask phase
//   cx c t qmask | mcx k c.. t | mcxm k c.. m.. t
//   cu1 c t phase qmask | mcu1 k c.. t phase | mcu1m k c.. m.. t phase
//   swap a b | ptp k q.. p.. phase | qft k q.. | iqft k q..
//   measure q r | reset q r | prob k q.. m..
// Output lines: "M c" (measure), "P p" (prob), "N norm" (vnorm),
// "S n" followed by "re.." and "im.." lines (dump), "E msg" (reference threw).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sstream>
#include <iostream>
#include <stdexcept>
#include <vector>
#include "suqa.cuh"

static std::vector<uint> read_list(std::istringstream& is) {
    uint k = 0;
    is >> k;
    std::vector<uint> v(k);
    for (uint i = 0; i < k; ++i) is >> v[i];
    return v;
}

static double read_double(std::istringstream& is) {
    std::string tok;
    is >> tok;
    return std::strtod(tok.c_str(), nullptr);
}

static void dump_state(FILE* out) {
    const size_t N = suqa::state.size();
    fprintf(out, "S %zu\n", N);
    for (size_t i = 0; i < N; ++i) fprintf(out, "%a%c", suqa::state.data_re[i], i + 1 == N ? '\n' : ' ');
    for (size_t i = 0; i < N; ++i) fprintf(out, "%a%c", suqa::state.data_im[i], i + 1 == N ? '\n' : ' ');
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <out file> < script\n", argv[0]);
        return 2;
    }
    FILE* out = fopen(argv[1], "w");
    if (!out) return 2;
    bool have_state = false;
    std::string line;
    while (std::getline(std::cin, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        std::string cmd;
        is >> cmd;
        try {
            if (cmd == "setup") {
                uint n; is >> n;
                if (have_state) suqa::clear();
                suqa::gc_mask = 0U;
                suqa::setup(n);
                have_state = true;
            } else if (cmd == "init") {
                suqa::init_state();
            } else if (cmd == "setstate") {
                std::string vals;
                std::getline(std::cin, vals);
                std::istringstream vs(vals);
                const size_t N = suqa::state.size();
                for (size_t i = 0; i < 2 * N; ++i) {
                    std::string tok; vs >> tok;
                    suqa::state.data[i] = std::strtod(tok.c_str(), nullptr);
                }
            } else if (cmd == "vnorm") {
                fprintf(out, "N %a\n", suqa::vnorm());
            } else if (cmd == "normalize") {
                suqa::vnormalize();
            } else if (cmd == "dump") {
                dump_state(out);
            } else if (cmd == "gc_on") {
                suqa::activate_gc_mask(read_list(is));
            } else if (cmd == "gc_off") {
                suqa::deactivate_gc_mask(read_list(is));
            } else if (cmd == "x") { uint q; is >> q; suqa::apply_x(q);
            } else if (cmd == "y") { uint q; is >> q; suqa::apply_y(q);
            } else if (cmd == "z") { uint q; is >> q; suqa::apply_z(q);
            } else if (cmd == "h") { uint q; is >> q; suqa::apply_h(q);
            } else if (cmd == "s") { uint q; is >> q; suqa::apply_s(q);
            } else if (cmd == "t") { uint q; is >> q; suqa::apply_t(q);
            } else if (cmd == "tdg") { uint q; is >> q; suqa::apply_tdg(q);
            } else if (cmd == "u1") {
                uint q; is >> q; double ph = read_double(is);
                suqa::apply_u1(q, ph);
            } else if (cmd == "u1m") {
                uint q, m; is >> q >> m; double ph = read_double(is);
                suqa::apply_u1(q, m, ph);
            } else if (cmd == "cx") {
                uint c, t, m; is >> c >> t >> m;
                suqa::apply_cx(c, t, m);
            } else if (cmd == "mcx") {
                std::vector<uint> cs = read_list(is);
                uint t; is >> t;
                suqa::apply_mcx(cs, t);
            } else if (cmd == "mcxm") {
                std::vector<uint> cs = read_list(is);
                std::vector<uint> ms(cs.size());
                for (auto& m : ms) is >> m;
                uint t; is >> t;
                suqa::apply_mcx(cs, ms, t);
            } else if (cmd == "cu1") {
                uint c, t; is >> c >> t; double ph = read_double(is); uint m; is >> m;
                suqa::apply_cu1(c, t, ph, m);
            } else if (cmd == "mcu1") {
                std::vector<uint> cs = read_list(is);
                uint t; is >> t; double ph = read_double(is);
                suqa::apply_mcu1(cs, t, ph);
            } else if (cmd == "mcu1m") {
                std::vector<uint> cs = read_list(is);
                std::vector<uint> ms(cs.size());
                for (auto& m : ms) is >> m;
                uint t; is >> t; double ph = read_double(is);
                suqa::apply_mcu1(cs, ms, t, ph);
            } else if (cmd == "swap") {
                uint a, b; is >> a >> b;
                suqa::apply_swap(a, b);
            } else if (cmd == "ptp") {
                std::vector<uint> qs = read_list(is);
                std::vector<uint> ps(qs.size());
                for (auto& p : ps) is >> p;
                double ph = read_double(is);
                suqa::apply_pauli_TP_rotation(qs, ps, ph);
            } else if (cmd == "qft") {
                suqa::apply_qft(read_list(is));
            } else if (cmd == "iqft") {
                suqa::apply_qft_inverse(read_list(is));
            } else if (cmd == "measure") {
                uint q, c = 0; is >> q; double r = read_double(is);
                suqa::measure_qbit(q, c, r);
                fprintf(out, "M %u\n", c);
            } else if (cmd == "reset") {
                uint q; is >> q; double r = read_double(is);
                suqa::apply_reset(q, r);
            } else if (cmd == "prob") {
                std::vector<uint> qs = read_list(is);
                std::vector<uint> ms(qs.size());
                for (auto& m : ms) is >> m;
                double p = 0.0;
                suqa::prob_filter(qs, ms, p);
                fprintf(out, "P %a\n", p);
            } else {
                fprintf(stderr, "unknown command: %s\n", cmd.c_str());
                return 3;
            }
        } catch (const std::exception& e) {
            fprintf(out, "E %s\n", e.what());
        }
    }
    if (have_state) suqa::clear();
    fclose(out);
    return 0;
}
