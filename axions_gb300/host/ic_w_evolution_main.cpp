// Drop-in for the reference program ic_w_evolution.cpp: same parameters (its
// constants and those of ic_func.cpp it uses) and output files; the lattice
// work, string detection and the string length run on the GPU.
#include "evolve.hpp"

int main(int argc, char** argv) { return axh::run_program(axh::Program::IcwEvolution, argc, argv); }
