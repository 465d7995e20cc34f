// Test infrastructure only: exposes the reference's own cubic root finder
// (cyCodeBase/cyPolynomial.h:787, called from model/collision.cpp:254 with the default
// xError) through a C symbol, so the oracle's restatement can be checked against it.
// Compiled by oracle/Makefile from the reference tree; the output stays in oracle/_ref/.
#include "cyPolynomial.h"

extern "C" int ref_cubic_roots(const double* coef, double x0, double x1, double* roots) {
  return cy::CubicRoots(roots, coef, x0, x1);
}
