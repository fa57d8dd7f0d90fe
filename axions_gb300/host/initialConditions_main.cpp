// Drop-in for the reference program initialConditions.cpp: same parameters and
// Data/ic.txt output for its "random" and "boost" families (the boosted
// string is built on the GPU from the straight-string table that
// singleSemiAnalytic writes); also converts field tables between the text and
// binary forms (ic_type = convert).
#include "evolve.hpp"

int main(int argc, char** argv) { return axh::run_program(axh::Program::InitialConditions, argc, argv); }
