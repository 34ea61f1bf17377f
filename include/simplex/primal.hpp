// Solver termination status shared with the reference's simplex module
// (src/simplex/primal.hpp:26-31). Only the status enum is provided: the CPU
// simplex itself is not part of this engine.
#pragma once

namespace sankhya {
namespace simplex {

enum class SimplexStatus { Optimal, Infeasible, Unbounded, IterationLimit };

}  // namespace simplex
}  // namespace sankhya
