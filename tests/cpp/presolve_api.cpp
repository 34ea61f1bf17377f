// Source-compatibility check of the presolve C++ API: the same calls a reference
// user makes (core::Model::add_variable / add_constraint / finalize, then
// presolve::apply_ruiz_scaling(model, iterations)); prints the scaled model as
// JSON for tests/test_presolve.py.
#include <cstdio>

#include "core/problem.hpp"
#include "presolve/scaling.hpp"

using namespace sankhya;

static void dump(const char* name, const core::Model& m, bool last) {
    std::printf("\"%s\": {\"vals\": [", name);
    for (size_t k = 0; k < m.A.values.size(); ++k) std::printf("%s%.17g", k ? ", " : "", m.A.values[k]);
    std::printf("], \"rhs\": [");
    for (size_t k = 0; k < m.rhs.size(); ++k) std::printf("%s%.17g", k ? ", " : "", m.rhs[k]);
    std::printf("], \"obj\": [");
    for (size_t k = 0; k < m.obj.size(); ++k) std::printf("%s%.17g", k ? ", " : "", m.obj[k]);
    std::printf("], \"lb0\": %.17g, \"col_scale\": [%.17g, %.17g], \"row_scale\": [", m.lb[0], m.col_scale[0],
                m.col_scale[1]);
    for (size_t k = 0; k < m.row_scale.size(); ++k) std::printf("%s%.17g", k ? ", " : "", m.row_scale[k]);
    std::printf("]}%s\n", last ? "" : ",");
}

int main() {
    core::Model a;
    a.sense = OptimizationSense::Minimize;
    a.add_variable(1.0, 10.0, 20.0, VariableType::Continuous);
    a.add_variable(2.0, 0.0, math::kInfinity, VariableType::Continuous);
    a.add_constraint({0, 1}, {1e6, 1e-4}, 1e3);
    a.add_constraint({0, 1}, {1e-4, 1e6}, 1e3);
    a.finalize();
    presolve::apply_ruiz_scaling(a, 20);

    core::Model b;
    b.add_variable(1.0, 0.0, 1.0, VariableType::Binary);
    b.add_variable(2.0, 0.0, math::kInfinity, VariableType::Continuous);
    b.add_constraint({0, 1}, {100.0, 100.0}, 50.0);
    b.finalize();
    presolve::apply_ruiz_scaling(b);

    std::printf("{\n");
    dump("conditioning", a, false);
    dump("integer", b, true);
    std::printf("}\n");
    return 0;
}
