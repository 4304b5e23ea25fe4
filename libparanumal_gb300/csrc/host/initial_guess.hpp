// Initial-guess strategies of the linear solver (include/initialGuess.hpp:38-162,
// libs/linearSolver/initialGuess.cpp): before each solve FormInitialGuess(x, rhs) sets x
// from the history of earlier solves; after it Update(A, x) adds the new solution.
//   NONE     keep the caller's x                       ZERO  x = 0
//   CLASSIC  projection onto an A-image basis of earlier solutions (Fischer 1998),
//            restarted when full
//   QR       the same basis kept as a rolling QR factorisation (oldest column dropped
//            by Givens rotations when full)
//   EXTRAP   polynomial extrapolation in time of the last M solutions, coefficients by
//            minimum-norm (MINNORM) or column-pivoted QR (CPQR) solves
// History vectors live on the device (FP64, Nglobal each); the small dense algebra (inner
// product sums, Givens rotations, extrapolation coefficients) runs on the host, as in
// the reference.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "objects.hpp"

namespace lpg {

struct InitialGuess {
  virtual ~InitialGuess() = default;
  virtual int form(double* x, const double* rhs, cudaStream_t s) = 0;
  virtual int update(Elliptic* el, const double* x, cudaStream_t s) = 0;
  virtual int history() const { return 0; }   // current history dimension
};

// settings: INITIAL GUESS STRATEGY / HISTORY SPACE DIMENSION / EXTRAP DEGREE /
// EXTRAP COEFFS METHOD; nullptr + LPG_ERR_SETTINGS on bad values
std::unique_ptr<InitialGuess> make_initial_guess(const Settings& S, Platform* plat, int64_t N, int* status);

// Extrapolation weights c (M entries) of the last M equally spaced values evaluated one
// step ahead, exact for polynomials of degree m (Extrap::extrapCoeffs, initialGuess.cpp:440-468)
int extrap_coeffs(int m, int M, bool cpqr, std::vector<double>& c);

}  // namespace lpg
