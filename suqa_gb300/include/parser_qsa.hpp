// Command line of the qsa driver, as the reference's include/parser_qsa.hpp:
//   <beta> <sampling> <num ene qbits> <num szegedy qbits> <output file>
//   [--seed S (time)] [--ene-min E (-4)] [--ene-max E (8)] [--ene-min-szegedy E (-1)]
//   [--ene-max-szegedy E (3)] [--PE-steps N (1)] [--annealing-sequences N (100)]
#pragma once
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>

struct arg_list {
    double beta = 0.25;
    int ene_qbits = 0;
    int szegedy_qbits = 0;
    std::string outfile = "";
    unsigned long long int seed = 0;
    double ene_min = -4.0;
    double ene_max = 8.0;
    double ene_min_szegedy = -1.0;
    double ene_max_szegedy = 3.0;
    int pe_steps = 1;
    int annealing_sequences = 100;
    int sampling = 0;
};

inline std::ostream& operator<<(std::ostream& o, const arg_list& a) {
    o << "beta: " << a.beta << "\nnum E qbits: " << a.ene_qbits << "\nnum Szegedy qbits: " << a.szegedy_qbits
      << "\nseed: " << a.seed << "\nout datafile: " << a.outfile << "\nmin energy: " << a.ene_min
      << "\nmax energy: " << a.ene_max << "\nmin energy szegedy: " << a.ene_min_szegedy
      << "\nmax energy szegedy: " << a.ene_max_szegedy << "\nsteps of PE evolution: " << a.pe_steps
      << "\nannealing_sequences: " << a.annealing_sequences << "\nsampling: " << a.sampling << std::endl;
    return o;
}

inline void parse_arguments(arg_list& args, int argc, char** argv) {
    const int fixed = 5;
    args.beta = std::stod(argv[1], nullptr);
    args.sampling = std::atoi(argv[2]);
    args.ene_qbits = std::atoi(argv[3]);
    args.szegedy_qbits = std::atoi(argv[4]);
    args.outfile = argv[5];
    std::map<std::string, int> pos;
    for (int i = fixed + 1; i < argc; ++i) pos[argv[i]] = i;
    auto value = [&](const char* flag, const char* err) -> const char* {
        auto it = pos.find(flag);
        if (it == pos.end()) return nullptr;
        if (it->second + 1 >= argc) throw err;
        return argv[it->second + 1];
    };
    if (const char* v = value("--seed", "ERROR: set value after '--seed' flag")) args.seed = std::strtoull(v, nullptr, 10);
    if (const char* v = value("--ene-min", "ERROR: set value after '--ene-min' flag")) args.ene_min = std::stod(v);
    if (const char* v = value("--ene-max", "ERROR: set value after '--ene-max' flag")) args.ene_max = std::stod(v);
    if (const char* v = value("--ene-min-szegedy", "ERROR: set value after '--ene-min-szegedy' flag"))
        args.ene_min_szegedy = std::stod(v);
    if (const char* v = value("--ene-max-szegedy", "ERROR: set value after '--ene-max-szegedy' flag"))
        args.ene_max_szegedy = std::stod(v);
    if (const char* v = value("--PE-steps", "ERROR: set value after '--PE-steps' flag")) args.pe_steps = (int)std::stod(v);
    if (const char* v = value("--annealing-sequences", "ERROR: set value after '--annealing-sequences' flag"))
        args.annealing_sequences = (int)std::stod(v);
    if (args.beta <= 0.0) throw "ERROR: argument <beta> invalid";
    if (args.ene_qbits <= 0) throw "ERROR: argument <num ene qbits> non positive";
    if (args.szegedy_qbits <= 0) throw "ERROR: argument <num ene qbits> non positive";
    if (args.outfile == "") throw "ERROR: argument <output file path> empty";
    if (args.pe_steps <= 0) throw "ERROR: argument <steps of PE evolution> non positive";
    if (args.annealing_sequences <= 0) throw "ERROR: argument <annealing_sequences> non positive";
    if (args.sampling <= 0) throw "ERROR: argument <sampling> non positive";
}
