// Command line of the qms driver, as the reference's include/parser_qms.hpp:
//   <beta> <metro steps> <reset each> <num ene qbits> <output file>
//   [--max-reverse N (100)] [--seed S (time)] [--ene-min E (0)] [--ene-max E (1)]
//   [--PE-steps N (10)] [--thermalization N (100)] [--record-reverse]
// Errors are thrown as const char* like the reference.
#pragma once
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>

struct arg_list {
    double beta = 0.0;
    int metro_steps = 0;
    int reset_each = 0;
    int ene_qbits = 0;
    std::string outfile = "";
    int max_reverse_attempts = 100;
    unsigned long long int seed = 0;
    double ene_min = 0.0;
    double ene_max = 1.0;
    int pe_steps = 10;
    int thermalization = 100;
    bool record_reverse = false;
};

inline std::ostream& operator<<(std::ostream& o, const arg_list& a) {
    o << "beta: " << a.beta << "\nmetro steps: " << a.metro_steps << "\nreset each: " << a.reset_each
      << "\nnum E qbits " << a.ene_qbits << "\nmax reverse attempts: " << a.max_reverse_attempts
      << "\nseed: " << a.seed << "\nout datafile: " << a.outfile << "\nmin energy: " << a.ene_min
      << "\nmax energy: " << a.ene_max << "\nsteps of PE evolution: " << a.pe_steps
      << "\nthermalization: " << a.thermalization << "\nrecord reverse: " << a.record_reverse << std::endl;
    return o;
}

inline void parse_arguments(arg_list& args, int argc, char** argv) {
    const int fixed = 5;
    args.beta = std::stod(argv[1], nullptr);
    args.metro_steps = std::atoi(argv[2]);
    args.reset_each = std::atoi(argv[3]);
    args.ene_qbits = std::atoi(argv[4]);
    args.outfile = argv[5];
    std::map<std::string, int> pos;
    for (int i = fixed + 1; i < argc; ++i) pos[argv[i]] = i;
    auto value = [&](const char* flag, const char* err) -> const char* {
        auto it = pos.find(flag);
        if (it == pos.end()) return nullptr;
        if (it->second + 1 >= argc) throw err;
        return argv[it->second + 1];
    };
    if (pos.count("--record-reverse")) args.record_reverse = true;
    if (const char* v = value("--max-reverse", "ERROR: set value after '--max-reverse' flag"))
        args.max_reverse_attempts = std::atoi(v);
    if (const char* v = value("--seed", "ERROR: set value after '--seed' flag")) args.seed = std::strtoull(v, nullptr, 10);
    if (const char* v = value("--ene-min", "ERROR: set value after '--ene-min' flag")) args.ene_min = std::stod(v);
    if (const char* v = value("--ene-max", "ERROR: set value after '--ene-max' flag")) args.ene_max = std::stod(v);
    if (const char* v = value("--PE-steps", "ERROR: set value after '--PE-steps' flag")) args.pe_steps = (int)std::stod(v);
    if (const char* v = value("--thermalization", "ERROR: set value after '--thermalization' flag"))
        args.thermalization = (int)std::stod(v);
    if (args.beta <= 0.0) throw "ERROR: argument <beta> invalid";
    if (args.metro_steps <= 0) throw "ERROR: argument <metro steps> invalid";
    if (args.reset_each <= 0) throw "ERROR: argument <reset each> non positive";
    if (args.ene_qbits <= 0) throw "ERROR: argument <num ene qbits> non positive";
    if (args.outfile == "") throw "ERROR: argument <output file path> empty";
    if (args.max_reverse_attempts <= 0) throw "ERROR: argument <max reverse attempts> non positive";
    if (args.pe_steps <= 0) throw "ERROR: argument <steps of PE evolution> non positive";
}
