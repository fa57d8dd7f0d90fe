// Force-included (g++ -include) into every reference build made by
// oracle/ref/build_ref.py.  TEST INFRASTRUCTURE ONLY.
//
// The reference writes all its text output through `ofstream` at the default
// 6 significant digits (e.g. evolution.cpp:1411-1420).  To compare doubles
// exactly, every ofstream the reference declares is replaced by one that
// starts at precision 17, which round-trips a double.  The standard headers
// are included first so the macro below touches only the reference's code.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

struct axr_ofstream : public std::ofstream {
    axr_ofstream() { this->precision(17); }
    explicit axr_ofstream(const char* p) : std::ofstream(p) { this->precision(17); }
    explicit axr_ofstream(const std::string& p) : std::ofstream(p) { this->precision(17); }
};

#define ofstream axr_ofstream
