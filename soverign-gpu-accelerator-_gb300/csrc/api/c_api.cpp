// Public C API (include/sankhya/sankhya.h) over MehrotraSolver.
#include "sankhya/sankhya.h"

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "core/problem.hpp"
#include "ipm/mehrotra.hpp"
#include "parsers/mps_reader.hpp"

struct sankhya_env_s {
    sankhya::ipm::MehrotraOptions opts;
};

struct sankhya_model_s {
    sankhya::core::Model model;
    sankhya::ipm::MehrotraOptions opts;
    bool has_solution = false;
    double objval = 0.0;
    std::vector<double> x, pi;
};

extern "C" {

int sankhya_create_env(sankhya_env_t** env) {
    if (!env) return SANKHYA_ERROR_INVALID_ARGUMENT;
    try {
        *env = new sankhya_env_s();
        return SANKHYA_SUCCESS;
    } catch (...) {
        return SANKHYA_ERROR_INTERNAL;
    }
}

int sankhya_load_model(sankhya_env_t* env, const char* filename, sankhya_model_t** model) {
    if (!env || !filename || !model) return SANKHYA_ERROR_INVALID_ARGUMENT;
    try {
        auto* m = new sankhya_model_s();
        m->opts = env->opts;
        if (std::string(filename) == "fixture") {
            // min -x1 - x2  s.t.  x1 + s1 = 1, x2 + s2 = 1, all >= 0  (optimum -2)
            using sankhya::math::kInfinity;
            for (double c : {-1.0, -1.0, 0.0, 0.0}) m->model.add_variable(c, 0.0, kInfinity);
            m->model.add_constraint({0, 2}, {1.0, 1.0}, 1.0);
            m->model.add_constraint({1, 3}, {1.0, 1.0}, 1.0);
            m->model.finalize();
        } else {
            try {
                m->model = sankhya::parsers::read_mps(filename);
            } catch (...) {
                delete m;
                return SANKHYA_ERROR_LOAD_FAILED;
            }
        }
        *model = m;
        return SANKHYA_SUCCESS;
    } catch (...) {
        return SANKHYA_ERROR_INTERNAL;
    }
}

int sankhya_solve(sankhya_model_t* model) {
    if (!model) return SANKHYA_ERROR_INVALID_ARGUMENT;
    try {
        sankhya::ipm::MehrotraSolver solver(model->model, model->opts);
        auto r = solver.solve();
        if (r.status != sankhya::simplex::SimplexStatus::Optimal) {
            model->has_solution = false;
            return SANKHYA_ERROR_SOLVE_FAILED;
        }
        model->has_solution = true;
        model->objval = r.objective_value;
        model->x = std::move(r.x);
        model->pi = std::move(r.pi);
        return SANKHYA_SUCCESS;
    } catch (const std::invalid_argument&) {
        return SANKHYA_ERROR_INVALID_ARGUMENT;
    } catch (...) {
        return SANKHYA_ERROR_INTERNAL;
    }
}

int sankhya_get_objval(sankhya_model_t* model, double* objval) {
    if (!model || !objval) return SANKHYA_ERROR_INVALID_ARGUMENT;
    if (!model->has_solution) return SANKHYA_ERROR_NOT_AVAILABLE;
    *objval = model->objval;
    return SANKHYA_SUCCESS;
}

int sankhya_get_solution(sankhya_model_t* model, double* x, double* pi, int* n, int* m) {
    if (!model) return SANKHYA_ERROR_INVALID_ARGUMENT;
    if (!model->has_solution) return SANKHYA_ERROR_NOT_AVAILABLE;
    if (n) *n = static_cast<int>(model->x.size());
    if (m) *m = static_cast<int>(model->pi.size());
    if (x) std::memcpy(x, model->x.data(), sizeof(double) * model->x.size());
    if (pi) std::memcpy(pi, model->pi.data(), sizeof(double) * model->pi.size());
    return SANKHYA_SUCCESS;
}

void sankhya_free_model(sankhya_model_t* model) { delete model; }
void sankhya_free_env(sankhya_env_t* env) { delete env; }

}  // extern "C"
