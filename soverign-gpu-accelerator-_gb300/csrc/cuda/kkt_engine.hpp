// Device normal-equation engine: assembly of D (A Theta A^T) D + delta I into
// multifrontal fronts, level-scheduled tiled Cholesky (FP64 or FP32 fronts), and
// the multifrontal triangular solves. Replaces the reference's
// gpu::GPUKKTCholeskySolver (src/cuda/kkt.cu:177-870).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "cuda/dev_common.cuh"
#include "cuda/device_lp.hpp"
#include "ipm/front_plan.hpp"

namespace sankhya {
namespace dev {

struct PlanDev;

class KktEngine {
public:
    // The plan is copied into device memory; lp must stay alive.
    KktEngine(const ipm::FrontPlan& plan, const DeviceLP& lp, cudaStream_t stream);
    ~KktEngine();

    // Assembles and factors D (A diag(theta) A^T) D + delta I, D = 1/sqrt(max(|m_ii|, 1e-12)),
    // in FP64 (fp32 = false) or FP32 fronts. Returns true when every pivot was
    // positive (one host synchronisation).
    bool factor(const double* d_theta, double delta, bool fp32);
    // Device time of the factor() calls since reset_factor_time(), per front precision
    // (CUDA events around each factorisation graph).
    double factor_ms(bool fp32) const { return fact_ms_[fp32 ? 0 : 1]; }
    void reset_factor_time() { fact_ms_[0] = fact_ms_[1] = 0.0; }
    const std::vector<int>& mask32() const { return on32_h_; }   // per LP: 1 = fronts in that precision
    const std::vector<int>& mask64() const { return on64_h_; }
    // FP32 fronts: trailing updates on the tensor cores (tcgen05, TF32 x3; default) or
    // as exact FP32 SIMT arithmetic. Applies to the next factor() call.
    void set_tensor_update(bool on) { tensor_ = on; }
    // FP64 fronts: trailing updates as FP64-accurate products on the tensor cores
    // (BF16 digits, exact FP32 sums, integer epilogue; see k_update_oz) or on the
    // FP64 pipe (default). Applies to the next factor() call.
    void set_fp64_emulation(bool on) { emulate64_ = on; }
    bool fp64_emulation() const { return emulate64_; }
    // dst = D L^{-T} L^{-1} D src (batch row order), using the last factor. src
    // and dst may alias. Asynchronous on the engine stream.
    void apply_inverse(const double* d_src, double* d_dst);
    // dst = A diag(theta) A^T src (FP64, matrix-free).
    void apply_normal(const double* d_theta, const double* d_src, double* d_dst);
    // Which LPs of the batch are still being solved: factorisation and solves skip
    // the fronts of the others (their solve output rows are 0). All on initially.
    // apply_inverse then uses the last factor's precision for every LP.
    void set_active(const std::vector<char>& on);
    // Per-LP precision: LPs flagged in on32 use the FP32 fronts, those in on64 the
    // FP64 fronts (disjoint sets). factor(.., fp32) assembles and factors only the
    // fronts of its own set, leaving the other fronts of that precision as they
    // are, so an LP can be moved from on32 to on64 and factored alone. apply_inverse
    // applies the FP32 factor to the rows of on32 and the FP64 factor to the rows
    // of on64 (rows of neither get 0). Both sets must have been factored with the
    // current theta before apply_inverse.
    void set_masks(const std::vector<char>& on32, const std::vector<char>& on64);
    // LP of the front whose pivot failed in the last factor() (-1 if none).
    int failed_lp() const;
    // Every LP with a pivot that was not positive in the last factor() (ascending).
    const std::vector<int>& failed_lps() const { return failed_lps_; }
    // Restricts apply_inverse to the LPs flagged in `sub` (within the masks in force),
    // e.g. the LPs whose conjugate-gradient iteration has not converged yet; rows of
    // the other LPs then come out 0. unrestrict_solves() brings back the masks.
    void restrict_solves(const std::vector<char>& sub);
    void unrestrict_solves();

    // Diagnostics: one factorisation + one solve (of d_rhs) without graphs, with
    // CUDA events around every launch; fills out[17] as sk_solver_profile documents.
    void profile(const double* d_theta, double delta, bool fp32, const double* d_rhs, double* d_out,
                 double* out);   // out: 18 values (sk_solver_profile)

    bool last_fp32() const { return fp32_; }
    int failed_supernode() const { return failed_sn_; }
    const ipm::FrontPlan& plan() const { return plan_; }
    // Algorithmic bytes of one assembly (normal matrix into the fronts of element size `elem`).
    double assembly_bytes(size_t elem) const;
    double* diag_D() const { return D_.ptr; }
    // Copies the factored fronts to the host (FP64) for inspection.
    std::vector<double> fronts_host();
    // Diagonal of the last FP64 factor L (D (A Theta A^T) D + delta I = L L^T) in
    // elimination order (position k holds the pivot of batch row plan().perm[k]).
    std::vector<double> pivots_host();
    cudaStream_t stream() const { return st_; }
    // Non-zero when a triangular-solve task gave up waiting for a dependency
    // (synchronises). The solve result is then invalid.
    int solve_error();
    // Work vectors of length N available to callers between calls.
    double* scratch_n() const { return tn_.ptr; }

private:
    void run_factor_levels(bool fp32);
    void run_solve_levels();
    struct Prof;
    // The plan's tile steps restricted to the fronts of the LPs of one mask
    // (ipm::restrict_steps), rebuilt when the mask changes, so that a factorisation
    // of a few LPs of a large batch launches only their blocks (each launch of the
    // full plan has one block per tile of every front, and those of LPs that are
    // off still take an SM slot each).
    struct SubSteps {
        std::vector<int> mask;                  // the mask the lists were built for
        ipm::RestrictedSteps rs;
        Slot<int> d_items, d_prefix;
    };
    SubSteps sub_[2];                           // FP32 passes, FP64 passes
    std::vector<double> lp_work_;               // per LP: update blocks of one factorisation
    double total_work_ = 0.0;
    const SubSteps* pick_steps(bool fp32);
    template <class T> void launch_factor(T* F, T* Linv, Prof* prof = nullptr, const SubSteps* sub = nullptr);
    template <class T> void launch_solve(const T* F, const T* Linv, Prof* prof = nullptr);
    void ensure_fronts(bool fp32);
    void ensure_digits();
    PlanDev pd(bool fp32) const;
    void upload_mask(Slot<int>& dev, std::vector<int>& host, const std::vector<char>& on);
    template <class T> void solve_pass(const T* F, const T* Linv, const int* mask, bool keep, const double* d_src,
                                       double* d_dst, int graph);

    ipm::FrontPlan plan_;
    const DeviceLP& lp_;
    cudaStream_t st_;
    Arena arena_;
    Arena f32_arena_, f64_arena_;
    Slot<float> F32_, Linv32_;
    Slot<double> F64_, Linv64_;
    int64_t inv_size_ = 0;
    std::vector<int> fwd_task_off_, bwd_task_off_, gather_off_;
    int nflags_ = 0;
    // plan arrays
    Slot<int> sn_first_, sn_ncols_, sn_nrows_, sn_lda_, sn_parent_, rows_, ea_map_, ch_ptr_, ch_list_, perm_;
    Slot<int64_t> sn_F_off_, sn_f_off_, sn_rows_off_, ea_off_;
    Slot<int> step_items_, step_prefix_, round_items_, round_prefix_, level_sn_, blk_off_, flags_, counters_,
        solve_err_;
    Slot<int2> fwd_tasks_, bwd_tasks_;
    Slot<int> g_dst_, g_zp_, g_ptr_, g_src_;   // forward right-hand-side gather lists
    Slot<int> sn_lp_, on32_, on64_, q_lp_;    // LP of each front; per-precision LP masks; LP of each permuted row
    std::vector<int> on32_h_, on64_h_, sn_lp_h_;
    bool mixed_ = false;                        // set_masks in force (else one precision for all)
    bool restricted_ = false;                   // restrict_solves in force: full masks saved below
    std::vector<int> full32_h_, full64_h_;
    Slot<int> zc_sn_, zc_len_;                  // front-zeroing chunks: front, length and start offset
    Slot<int64_t> zc_off_;
    int64_t nzc_ = 0;
    Slot<int64_t> inv_off_;
    Slot<int64_t> slot_pos_, w_ptr_;
    Slot<int> slot_i_, slot_j_, w_col_;
    Slot<double> w_val_;
    // numeric work
    Slot<double> D_, Mdiag_, zp_, xp_, zsol_, fvec_, tn_, params_;
    Slot<int> err_;
    Slot<int> oz_cnt_;                          // per front: blocks of the first update tile done (fused potrf)
    bool fp32_ = false;
    int failed_sn_ = -1;
    std::vector<int> failed_lps_;
    Slot<int> lp_fail_;                         // per LP: a pivot failed in this factorisation
    const double* theta_bound_ = nullptr;
    bool tensor_ = true;
    bool emulate64_ = false;
    Arena dig_arena_;                           // digit planes and row exponents of the emulated FP64 update
    Slot<unsigned char> dig_, ldig_;            // panel-row digits; digits of each item's Linv rows
    Slot<int> dexp_, lexp_;
    int64_t max_step_items_ = 1;
    // FP64, FP32 SIMT update, FP32 tensor-core update, FP64 emulated on the tensor cores
    cudaGraphExec_t gfac_[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t fev_[2] = {nullptr, nullptr};
    double fact_ms_[2] = {0.0, 0.0};
    cudaGraphExec_t gsol_[2] = {nullptr, nullptr};
    const double* gfac_theta_[4] = {nullptr, nullptr, nullptr, nullptr};
};

}  // namespace dev
}  // namespace sankhya

namespace sankhya {
namespace dev {
// max |a_i| over n entries (synchronises; scratch64 holds 64 doubles).
double absmax_device(int n, const double* a, double* scratch64, cudaStream_t st);
void vec_diff(int n, const double* a, const double* b, double* out, cudaStream_t st);   // out = a - b
void vec_add(int n, const double* a, double* out, cudaStream_t st);                      // out += a
}  // namespace dev
}  // namespace sankhya
