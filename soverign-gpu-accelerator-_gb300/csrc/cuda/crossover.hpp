// Device crossover (basis purification); see crossover.cu.
#pragma once

#include <string>

namespace sankhya {
namespace dev {

// Largest m: the explicit basis inverse is m x m FP64 (8.6 GB at this size) and every
// basis change rewrites it.
constexpr int kCrossoverMaxRows = 32768;

// status[] values (simplex::BasisStatus order of the reference, src/simplex/basis.hpp:23-28)
constexpr int kBasic = 0, kAtLower = 1, kAtUpper = 2;

// return codes
constexpr int kCrossoverInvalidPivot = 1;
constexpr int kCrossoverRankDeficient = 2;
constexpr int kCrossoverTooLarge = 3;

// A: CSC (m x n); lb / ub: NULL = 0 / +inf; x_ipm: the interior point (n).
// basic (m): column of each basis row (>= n: an artificial column remained);
// status (n); x_out (n, optional): x after purification. message: the reference's
// error text for the failure codes.
int crossover(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, const double* lb,
              const double* ub, const double* x_ipm, int* basic, int* status, double* x_out, std::string* message);

}  // namespace dev
}  // namespace sankhya
