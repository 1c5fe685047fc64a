// sum_shim.h - force-included when compiling the reference with OpenMP: its QIFT
// probability check names an undeclared `sum` in a reduction clause
// (cpp/state_vector.hpp:124-127), which does not compile without a declaration.
// TEST INFRASTRUCTURE ONLY.
#pragma once
static double sum;
