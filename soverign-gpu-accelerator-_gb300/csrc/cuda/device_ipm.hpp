// Device Mehrotra predictor-corrector IPM over a batch of independent LPs.
// Host code keeps only per-LP scalars (norms, step lengths, merit); every
// vector lives in device memory for the whole solve.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "cuda/dev_common.cuh"
#include "cuda/device_lp.hpp"
#include "cuda/kkt_engine.hpp"
#include "ipm/front_plan.hpp"
#include "sankhya/sk_ipm.h"

namespace sankhya {
namespace dev {

class Gnn;

struct LpResult {
    int status = SK_STATUS_ITERATION_LIMIT;
    int iterations = 0;
    double objective = 0.0;
    double primal_residual = 0.0, dual_residual = 0.0, duality_gap = 0.0;
    double rel_pinf = 0.0, rel_dinf = 0.0, rel_gap = 0.0;
    int switch_iteration = -1;
    int learned_start = 0;
    double start_merit = 0.0;      // max(rel pinf, rel dinf, rel gap) at the start point used
    double fallback_merit = 0.0;   // same for Mehrotra's start (learned-start runs only)
};

class DeviceIPM {
public:
    DeviceIPM(const std::vector<ipm::LpView>& lps, const std::vector<const double*>& b,
              const std::vector<const double*>& c, const sk_options& opt);
    ~DeviceIPM();

    void set_start(int lp, const double* x, const double* y, const double* s);
    // Network used by SK_START_LEARNED (not owned).
    void set_gnn(Gnn* g);
    // Keep each LP's iterate (scaled space) at the first iteration whose mu is
    // below `mu` (or the final iterate if mu never gets there); 0 disables.
    void set_capture(double mu);
    // Captured iterate as training targets: log x, log s (N) and y (M), device.
    bool capture_complete() const;
    const double* capture_logx() const;
    const double* capture_logs() const;
    const double* capture_y() const;
    void run();
    // Kernel-class breakdown at the current iterate (see sk_solver_profile).
    void profile(bool fp32, bool tensor, double* out18);
    void result(int lp, double* x, double* y, double* s, sk_info* info) const;
    int num_lps() const { return nlp_; }
    const ipm::FrontPlan& plan() const { return kkt_->plan(); }
    KktEngine& kkt() { return *kkt_; }
    const DeviceLP& device_lp() const { return lp_; }
    double setup_ms() const { return setup_ms_; }

private:
    struct Impl;
    std::unique_ptr<Impl> im_;
    std::unique_ptr<KktEngine> kkt_;
    DeviceLP lp_;
    int nlp_ = 0;
    double setup_ms_ = 0.0;
};

// Standalone SpMV y = alpha A x + beta y (CSR, FP64) used by the C ABI.
void spmv_csr(int rows, const int* rp, const int* ci, const double* v, const double* x, double alpha, double beta,
              double* y, cudaStream_t st);

}  // namespace dev
}  // namespace sankhya
