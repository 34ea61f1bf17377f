// JSON-telemetry CLI: sankhya_cli <file.mps> | --family F [--instance I]
//                   [--fp64] [--reference-criteria] [--bounds] [--verbose]
// --bounds honours the model's variable bounds (the reference's IPM ignores them).
// Prints one JSON object on stdout with the reference CLI's keys in the same
// order (tests/benchmark/sankhya_benchmark_cli.cpp:84-97) followed by added keys;
// diagnostics go to stderr. The timer starts before the solver is constructed,
// as in the reference (:31), so solve_time_ms includes the setup.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "core/problem.hpp"
#include "ipm/mehrotra.hpp"
#include "parsers/mps_reader.hpp"
#include "sankhya/sk_ipm.h"

using namespace sankhya;

static std::string json_escape(const std::string& s) {
    std::string o;
    for (char ch : s) {
        if (ch == '"' || ch == '\\') { o += '\\'; o += ch; }
        else if (ch == '\n') o += "\\n";
        else o += ch;
    }
    return o;
}

int main(int argc, char** argv) {
    std::string path;
    int family = -1, instance = 0;
    ipm::MehrotraOptions opts;
    for (int a = 1; a < argc; ++a) {
        std::string t = argv[a];
        if (t == "--family" && a + 1 < argc) family = std::atoi(argv[++a]);
        else if (t == "--instance" && a + 1 < argc) instance = std::atoi(argv[++a]);
        else if (t == "--fp64") opts.precision = SK_PREC_FP64;
        else if (t == "--reference-criteria") opts.criteria = SK_CRIT_REFERENCE;
        else if (t == "--verbose") opts.verbose = 1;
        else if (t == "--bounds") opts.honor_bounds = true;
        else path = t;
    }
    if (path.empty() && family < 0) {
        std::fprintf(stderr, "Usage: sankhya_cli <mps_file> | --family F [--instance I] [--fp64] [--bounds]\n");
        return 1;
    }
    core::Model model;
    try {
        if (family >= 0) {
            sk_lp* lp = nullptr;
            if (sk_lp_generate(family, instance, &lp) != SK_OK) throw std::runtime_error(sk_last_error());
            int m, n, nz;
            const int *cp, *ri;
            const double *va, *b, *c;
            sk_lp_dims(lp, &m, &n, &nz);
            sk_lp_arrays(lp, &cp, &ri, &va, &b, &c);
            model = core::Model::from_csc(m, n, cp, ri, va, b, c);
            sk_lp_free(lp);
        } else {
            model = parsers::read_mps(path);
        }
    } catch (const std::exception& e) {
        std::printf("{\"error\": \"%s\"}\n", json_escape(e.what()).c_str());
        return 0;
    }
    auto t0 = std::chrono::high_resolution_clock::now();
    std::string status = "Failed";
    ipm::MehrotraResult r;
    std::string err;
    try {
        ipm::MehrotraSolver solver(model, opts);
        r = solver.solve();
        status = r.status == simplex::SimplexStatus::Optimal ? "Optimal" : "Failed";
    } catch (const std::exception& e) {
        err = e.what();
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
    const bool ok = status == "Optimal";
    std::printf("{\n");
    std::printf("  \"solver\": \"SANKHYA\",\n");
    std::printf("  \"status\": \"%s\",\n", status.c_str());
    std::printf("  \"execution_path\": \"GPU_ONLY\",\n");
    std::printf("  \"fallback_triggered\": \"NO\",\n");
    std::printf("  \"solve_time_ms\": %.6f,\n", ms);
    std::printf("  \"iterations\": %d,\n", r.iterations);
    std::printf("  \"objective\": %.15g,\n", ok ? r.objective_value : 0.0);
    std::printf("  \"primal_residual\": %.6g,\n", r.primal_residual);
    std::printf("  \"variables\": %zu,\n", model.obj.size());
    std::printf("  \"constraints\": %zu,\n", model.rhs.size());
    std::printf("  \"nnz\": %zu,\n", model.A.values.size());
    std::printf("  \"certificate_pass\": %s,\n",
                ok && r.info.rel_pinf <= 1e-8 && r.info.rel_dinf <= 1e-8 && r.info.rel_gap <= 1e-8 ? "true" : "false");
    std::printf("  \"precision_path\": \"%s\",\n",
                r.info.precision_path == 0 ? "fp64" : (r.info.precision_path == 1 ? "fp32" : "fp32+fp64"));
    std::printf("  \"learned_start\": %s,\n", r.info.learned_start ? "true" : "false");
    std::printf("  \"rel_gap\": %.6g,\n", r.info.rel_gap);
    std::printf("  \"rel_pinf\": %.6g,\n", r.info.rel_pinf);
    std::printf("  \"rel_dinf\": %.6g", r.info.rel_dinf);
    if (!err.empty()) std::printf(",\n  \"error\": \"%s\"", json_escape(err).c_str());
    std::printf("\n}\n");
    return 0;
}
