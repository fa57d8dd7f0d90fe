// Drop-in for the reference program moore_mpi_evolution.cpp: same parameters, input and output
// files; the lattice work runs on the GPU through liblattice_gpu.so.
#include "evolve.hpp"

int main(int argc, char** argv) { return axh::run_program(axh::Program::MooreMpiEvolution, argc, argv); }
