// Drop-in for the reference program initialConditions.cpp: same parameters and
// Data/ic.txt output for its "random" family; also converts field tables
// between the text and binary forms (ic_type = convert).
#include "evolve.hpp"

int main(int argc, char** argv) { return axh::run_program(axh::Program::InitialConditions, argc, argv); }
