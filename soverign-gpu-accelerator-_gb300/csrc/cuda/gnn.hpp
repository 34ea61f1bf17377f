// Learned warm start: a bipartite row / column message-passing network over the
// (scaled) constraint matrix of a batch of LPs. 3 layers, hidden width 64,
// BF16 weights, FP32 accumulation, FP32 master weights for Adam.
//
//   column features f_c = (c_j, log(1 + nnz_j), ||A_.j||_2), row features
//   f_r = (b_i, log(1 + nnz_i), ||A_i.||_2), edge weight a_ij (all after Ruiz);
//   h_c = relu(E_c f_c + e_c), h_r = relu(E_r f_r + e_r);
//   per layer: m_r = deg_i^-1 sum_j a_ij h_c[j];  h_r = relu(W_rr h_r + W_rm m_r + b_r)
//              m_c = deg_j^-1 sum_i a_ij h_r[i];  h_c = relu(W_cc h_c + W_cm m_c + b_c)
//   outputs: (log x_j, log s_j) = H_c h_c + o_c,  y_i = H_r h_r + o_r.
// Targets are the solver's iterate captured when mu first drops below a threshold.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "cuda/dev_common.cuh"
#include "cuda/device_lp.hpp"

namespace sankhya {
namespace dev {

constexpr int kGnnHidden = 64;
constexpr int kGnnLayers = 3;

class Gnn {
public:
    explicit Gnn(unsigned long long seed);
    ~Gnn();
    int num_params() const { return static_cast<int>(nparams_); }
    void get_params(float* out) const;
    void set_params(const float* in);
    // Forward on the LP batch; writes log x, log s (n) and y (m) predictions into
    // out_logx, out_logs, out_y (device, scaled space). If targets are given,
    // returns the loss and keeps activations for backward().
    double forward(const DeviceLP& lp, cudaStream_t st, double* out_logx, double* out_logs, double* out_y,
                   const double* t_logx = nullptr, const double* t_logs = nullptr, const double* t_y = nullptr);
    // Gradient of the last forward's loss into grad_ (FP32); optional copy-out.
    void backward(const DeviceLP& lp, cudaStream_t st, float* grad_host = nullptr);
    void adam_step(cudaStream_t st, float lr);

private:
    void ensure(const DeviceLP& lp);
    size_t nparams_ = 0;
    float* master_ = nullptr;     // FP32 master weights
    uint16_t* wbf_ = nullptr;     // BF16 weights
    float* grad_ = nullptr;
    float* adam_m_ = nullptr;
    float* adam_v_ = nullptr;
    int adam_t_ = 0;
    // activations
    int capN_ = 0, capM_ = 0;
    float *fc_ = nullptr, *fr_ = nullptr;                 // features (N x 3, M x 3)
    float *hc_ = nullptr, *hr_ = nullptr;                 // (L+1) x N x H, (L+1) x M x H
    float *mc_ = nullptr, *mr_ = nullptr;                 // L x N x H, L x M x H
    float *oc_ = nullptr, *or_ = nullptr;                 // N x 2, M x 1
    float *dc_ = nullptr, *dr_ = nullptr, *dm_ = nullptr, *dt_ = nullptr;  // gradient work
    float *inv_deg_r_ = nullptr, *inv_deg_c_ = nullptr;
    double* loss_ = nullptr;
    const double *t_logx_ = nullptr, *t_logs_ = nullptr, *t_y_ = nullptr;
};

}  // namespace dev
}  // namespace sankhya
