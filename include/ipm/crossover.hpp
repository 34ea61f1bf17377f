// Crossover from an interior point to a basis (Megiddo purification) on the device.
// Replaces: ipm::generate_crossover_basis (src/ipm/crossover.cuh:30-33), which takes
// the reference's device upload of the model (gpu::DeviceModel); this one takes the
// host model and uploads what it needs. Same decisions, same results and the same
// exceptions: std::runtime_error("Crossover failed: Invalid pivot encountered") and
// std::runtime_error("Crossover failed: Matrix is rank deficient").
#pragma once

#include <vector>

#include "core/problem.hpp"
#include "simplex/basis.hpp"

namespace sankhya {
namespace ipm {

simplex::Basis generate_crossover_basis(const core::Model& model, const std::vector<Float>& x_ipm);

}  // namespace ipm
}  // namespace sankhya
