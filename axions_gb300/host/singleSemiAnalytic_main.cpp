// Drop-in for the reference program singleSemiAnalytic.cpp: the radial profile
// of a straight string by successive over-relaxation, written to
// Data/SOR_Fields.txt.
#include "evolve.hpp"

int main(int argc, char** argv) { return axh::run_program(axh::Program::SingleSemiAnalytic, argc, argv); }
