// Drop-in host programs for the reference's four evolution programs.
//
// Each program keeps the reference's parameter names (its compile-time
// constants, e.g. mpi_evolution.cpp:15-60), its input files (Data/ic.txt,
// Data/moore_ic.txt), its output files and their text format (default ostream
// precision), and its output cadence; the lattice work goes through the C ABI
// of liblattice_gpu.so.  Parameters come from `key = value` lines of a file
// given as `params=<file>` and from `key=value` arguments, the latter winning.
#pragma once

#include <map>
#include <string>

namespace axh {

// IcwEvolution is ic_w_evolution.cpp: evolution with its initial conditions
// made in-process (ic_func.cpp) and the total string length every step.
// InitialConditions is initialConditions.cpp (writes Data/ic.txt).
// SingleSemiAnalytic is singleSemiAnalytic.cpp (writes Data/SOR_Fields.txt,
// the straight-string profile the string IC families interpolate; host only).
enum class Program { MpiEvolution, Evolution, MooreMpiEvolution, MooreEvol, IcwEvolution, InitialConditions,
                     SingleSemiAnalytic };

// Parameter set: the reference defaults of `prog`, overridden by the file and
// the command line.  Unknown keys are an error.
class Params {
public:
    explicit Params(Program prog);
    void parse_args(int argc, char** argv);   // key=value ..., params=<file>
    void set(const std::string& key, const std::string& value);

    double num(const std::string& k) const;
    long long integer(const std::string& k) const;
    bool flag(const std::string& k) const;
    const std::string& str(const std::string& k) const;
    bool has(const std::string& k) const { return vals_.count(k) != 0; }

private:
    std::map<std::string, std::string> vals_;
};

// Runs the program; returns the process exit code.
int run_program(Program prog, int argc, char** argv);

}  // namespace axh
