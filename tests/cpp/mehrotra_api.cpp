// A reference C++ caller of the device IPM, written against the reference's API:
// the calls and checks of the reference's tests/unit/test_mehrotra.cu:13-79
// (core::Model built with add_variable / add_constraint / finalize, then
// ipm::MehrotraSolver(model).solve() and the MehrotraResult fields status,
// iterations, primal_residual, dual_residual, duality_gap, objective_value, x, pi).
// It compiles against include/ipm/mehrotra.hpp unchanged and links
// libsankhya_gb300.so. Exit codes: 0 pass, 1 a check failed, 77 no CUDA device.
#include <cmath>
#include <cstdio>

#include <cuda_runtime.h>

#include "core/problem.hpp"
#include "ipm/mehrotra.hpp"

using namespace sankhya;
using sankhya::simplex::SimplexStatus;

static int failures = 0;
#define EXPECT(cond)                                                       \
    do {                                                                   \
        if (!(cond)) {                                                     \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #cond, __LINE__); \
            ++failures;                                                    \
        }                                                                  \
    } while (0)

int main() {
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
        std::printf("no CUDA device\n");
        return 77;
    }
    // min -3 x1 - 5 x2  s.t.  x1 + x2 + x3 = 4,  2 x1 + 3 x2 + x4 = 12,  x >= 0: optimum -20 at x2 = 4
    core::Model model;
    model.sense = OptimizationSense::Minimize;
    for (double cj : {-3.0, -5.0, 0.0, 0.0}) model.add_variable(cj);
    model.add_constraint({0, 1, 2}, {1.0, 1.0, 1.0}, 4.0);
    model.add_constraint({0, 1, 3}, {2.0, 3.0, 1.0}, 12.0);
    model.finalize();

    ipm::MehrotraSolver solver(model);
    ipm::MehrotraResult result;
    try {
        result = solver.solve();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "solve threw: %s\n", e.what());
        return 1;
    }
    EXPECT(result.status == SimplexStatus::Optimal);
    EXPECT(result.iterations > 0);
    EXPECT(result.primal_residual < 1e-6);
    EXPECT(result.dual_residual < 1e-6);
    EXPECT(result.duality_gap < 1e-6);
    EXPECT(std::fabs(result.objective_value + 20.0) <= 1e-4);
    EXPECT(result.x.size() == 4);
    EXPECT(result.pi.size() == 2);
    for (Float v : result.x) EXPECT(std::isfinite(v));
    for (Float v : result.pi) EXPECT(std::isfinite(v));
    std::printf("{\"status\": %d, \"iterations\": %d, \"objective\": %.15g, \"failures\": %d}\n",
                static_cast<int>(result.status), static_cast<int>(result.iterations), result.objective_value,
                failures);
    return failures ? 1 : 0;
}
