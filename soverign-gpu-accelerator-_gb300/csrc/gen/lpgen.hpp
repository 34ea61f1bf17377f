// Seeded synthetic LP families used for parity tests and benchmarks.
//   family 0: random sparse LP, m=500, n=1000, 1% density (seed 0xC0 + instance)
//   family 1: block-angular LP, 40 blocks of 500x1200 + 2000 linking rows,
//             m=22000, n=48000, 6 nnz per column (seed 0xC1 + instance)
//   family 2: 50-stage staircase transportation LP, m=200000, n=500000
//             (seed 0xC2 + instance)
//   family 3: member `instance` of the 512-LP uneven batch:
//             m ~ logUniform[200,5000], n = ceil(m*U[2,3]), density U[0.5%,2%]
//             (seed 0xC3*1e6 + instance)
// Families 0, 1, 3 are feasible and bounded by construction: b = A x0 with
// x0 ~ U[0.5,2] and c = A^T y0 + s0 with y0 ~ N(0,1), s0 ~ U[0.1,1].
// Family 2 has integer supplies / demands built from a strictly positive integer
// flow, so it is feasible with a strictly interior point; costs are >= 0, so it is
// bounded. Its supply and demand rows of each stage sum to the same vector, so
// each stage carries one linearly dependent row (the solver regularises it).
#pragma once

#include <cstdint>
#include <vector>

#include "sankhya/types.hpp"

namespace sankhya {
namespace gen {

struct GeneratedLP {
    Index m = 0, n = 0;
    std::vector<Index> col_ptrs;
    std::vector<Index> row_idx;
    std::vector<Float> vals;
    std::vector<Float> b, c;
};

// Portable 64-bit generator (xoshiro256** seeded through splitmix64).
class Rng {
public:
    explicit Rng(uint64_t seed);
    uint64_t next();
    double uniform();                       // [0, 1), 53-bit
    double uniform(double lo, double hi);   // [lo, hi)
    uint64_t below(uint64_t bound);         // uniform integer in [0, bound)
    double normal();                        // N(0,1) by Box-Muller
private:
    uint64_t s_[4];
    bool have_spare_ = false;
    double spare_ = 0.0;
};

GeneratedLP random_sparse_lp(Index m, Index n, double density, uint64_t seed);
GeneratedLP block_angular_lp(uint64_t seed, Index blocks = 40, Index block_rows = 500,
                             Index block_cols = 1200, Index link_rows = 2000,
                             Index nnz_per_block_col = 5);
// Family 2 is stages=50, supply=demand=1000, cap=2000, arcs=8000 (rows per stage
// supply + demand + cap, columns per stage arcs + cap).
GeneratedLP staircase_transport_lp(uint64_t seed, Index stages = 50, Index supply = 1000, Index demand = 1000,
                                   Index cap = 2000, Index arcs = 8000);
GeneratedLP family_lp(int family, int instance);

}  // namespace gen
}  // namespace sankhya
