// Learned warm start network: hand-written BF16-weight forward / backward
// kernels and Adam (see gnn.hpp for the model).
#include "cuda/gnn.hpp"

#include <cmath>
#include <cstring>

namespace sankhya {
namespace dev {

namespace {

constexpr int H = kGnnHidden;
constexpr int L = kGnnLayers;

// parameter layout (floats)
struct Layout {
    size_t Ec, ec, Er, er;
    size_t Wrr[L], Wrm[L], br[L], Wcc[L], Wcm[L], bc[L];
    size_t Hc, oc, Hr, orr;
    size_t total;
};

Layout make_layout() {
    Layout y{};
    size_t o = 0;
    y.Ec = o; o += H * 3; y.ec = o; o += H;
    y.Er = o; o += H * 3; y.er = o; o += H;
    for (int l = 0; l < L; ++l) {
        y.Wrr[l] = o; o += H * H; y.Wrm[l] = o; o += H * H; y.br[l] = o; o += H;
        y.Wcc[l] = o; o += H * H; y.Wcm[l] = o; o += H * H; y.bc[l] = o; o += H;
    }
    y.Hc = o; o += 2 * H; y.oc = o; o += 2;
    y.Hr = o; o += H; y.orr = o; o += 1;
    y.total = o;
    return y;
}

const Layout kLay = make_layout();

__device__ __forceinline__ float bf(uint16_t w) { return __uint_as_float(static_cast<uint32_t>(w) << 16); }

__host__ __device__ inline uint16_t to_bf16(float f) {   // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return static_cast<uint16_t>(u >> 16);   // inf / nan
    u += 0x7fffu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}

__global__ void k_to_bf16(int n, const float* __restrict__ w, uint16_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        uint32_t u = __float_as_uint(w[i]);
        if ((u & 0x7f800000u) != 0x7f800000u) u += 0x7fffu + ((u >> 16) & 1u);
        out[i] = static_cast<uint16_t>(u >> 16);
    }
}

// features and inverse degrees (rows from CSR, columns from CSC)
__global__ void k_features(int rows, const int* __restrict__ rp, const double* __restrict__ v,
                           const double* __restrict__ rhs, float* __restrict__ f, float* __restrict__ inv_deg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    double s2 = 0.0;
    for (int q = rp[i]; q < rp[i + 1]; ++q) s2 += v[q] * v[q];
    const int d = rp[i + 1] - rp[i];
    f[i * 3 + 0] = static_cast<float>(rhs[i]);
    f[i * 3 + 1] = logf(1.0f + static_cast<float>(d));
    f[i * 3 + 2] = static_cast<float>(sqrt(s2));
    inv_deg[i] = 1.0f / static_cast<float>(d > 0 ? d : 1);
}

// out[node][o] = relu(sum_k W[o][k] f[node][k] + b[o]), IN = 3
__global__ void k_embed(int nodes, const float* __restrict__ f, const uint16_t* __restrict__ W,
                        const uint16_t* __restrict__ b, float* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nodes * H) return;
    const int node = t / H, o = t % H;
    float acc = bf(b[o]);
    for (int k = 0; k < 3; ++k) acc += bf(W[o * 3 + k]) * f[node * 3 + k];
    out[t] = acc > 0.f ? acc : 0.f;
}

// out[node][o] = relu(W1[o] . x1[node] + W2[o] . x2[node] + b[o]); 256 threads, 32 nodes per block
__global__ void __launch_bounds__(256) k_layer(int nodes, const float* __restrict__ x1, const float* __restrict__ x2,
                                               const uint16_t* __restrict__ W1, const uint16_t* __restrict__ W2,
                                               const uint16_t* __restrict__ b, float* __restrict__ out) {
    __shared__ float Wt1[H * H], Wt2[H * H];   // [k][o]
    __shared__ float xs1[32][H + 1], xs2[32][H + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < H * H; idx += 256) {
        const int o = idx / H, k = idx % H;
        Wt1[k * H + o] = bf(W1[idx]);
        Wt2[k * H + o] = bf(W2[idx]);
    }
    const int n0 = blockIdx.x * 32;
    for (int idx = tid; idx < 32 * H; idx += 256) {
        const int nn = idx / H, k = idx % H;
        const int node = n0 + nn;
        xs1[nn][k] = node < nodes ? x1[static_cast<size_t>(node) * H + k] : 0.f;
        xs2[nn][k] = node < nodes ? x2[static_cast<size_t>(node) * H + k] : 0.f;
    }
    __syncthreads();
    const int o = tid & (H - 1), g = tid >> 6;
    const float bo = bf(b[o]);
    for (int nn = g; nn < 32; nn += 4) {
        const int node = n0 + nn;
        if (node >= nodes) break;
        float acc = bo;
        for (int k = 0; k < H; ++k) acc += Wt1[k * H + o] * xs1[nn][k] + Wt2[k * H + o] * xs2[nn][k];
        out[static_cast<size_t>(node) * H + o] = acc > 0.f ? acc : 0.f;
    }
}

// out[node][o] = W[o] . x[node] + b[o], o < OUT (warp per node)
__global__ void k_head(int nodes, int OUT, const float* __restrict__ x, const uint16_t* __restrict__ W,
                       const uint16_t* __restrict__ b, float* __restrict__ out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nodes) return;
    for (int o = 0; o < OUT; ++o) {
        float acc = 0.f;
        for (int k = lane; k < H; k += 32) acc += bf(W[o * H + k]) * x[static_cast<size_t>(warp) * H + k];
        for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
        if (lane == 0) out[warp * OUT + o] = acc + bf(b[o]);
    }
}

// out[r][:] = scale_out[r] * sum_q v[q] * in[ci[q]][:] * scale_in[ci[q]] (warp per row; scales optional)
__global__ void k_spmm(int rows, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                       const float* __restrict__ scale_out, const float* __restrict__ scale_in,
                       const float* __restrict__ in, float* __restrict__ out, int accumulate) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= rows) return;
    float a0 = 0.f, a1 = 0.f;
    for (int q = rp[warp]; q < rp[warp + 1]; ++q) {
        const int c = ci[q];
        const float w = static_cast<float>(v[q]) * (scale_in ? scale_in[c] : 1.f);
        a0 += w * in[static_cast<size_t>(c) * H + lane];
        a1 += w * in[static_cast<size_t>(c) * H + lane + 32];
    }
    const float so = scale_out ? scale_out[warp] : 1.f;
    float* o = out + static_cast<size_t>(warp) * H;
    if (accumulate) { o[lane] += so * a0; o[lane + 32] += so * a1; }
    else { o[lane] = so * a0; o[lane + 32] = so * a1; }
}

// loss: columns (log x, log s) vs targets, rows y vs target; writes d_out and adds the loss
__global__ void k_loss(int N, int M, const float* __restrict__ oc, const float* __restrict__ orr,
                       const double* __restrict__ tx, const double* __restrict__ ts, const double* __restrict__ ty,
                       float* __restrict__ doc, float* __restrict__ dor, double* loss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    const float wc = 1.0f / (2.0f * N), wr = 1.0f / M;
    if (t < N) {
        const float ex = oc[2 * t] - static_cast<float>(fmin(fmax(tx[t], -30.0), 30.0));
        const float es = oc[2 * t + 1] - static_cast<float>(fmin(fmax(ts[t], -30.0), 30.0));
        doc[2 * t] = 2.f * wc * ex;
        doc[2 * t + 1] = 2.f * wc * es;
        l += wc * (ex * ex + es * es);
    } else if (t < N + M) {
        const int i = t - N;
        const float ey = orr[i] - static_cast<float>(ty[i]);
        dor[i] = 2.f * wr * ey;
        l += wr * ey * ey;
    }
    l = warp_sum(l);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

// head backward: dx[node][k] = sum_o d[node][o] W[o][k]; dW, db accumulated
__global__ void k_head_bwd(int nodes, int OUT, const float* __restrict__ x, const float* __restrict__ d,
                           const uint16_t* __restrict__ W, float* __restrict__ dx, float* __restrict__ dW,
                           float* __restrict__ db) {
    __shared__ float sW[2 * H], sdb[2];
    const int tid = threadIdx.x;
    if (tid < 2 * H) sW[tid] = 0.f;
    if (tid < 2) sdb[tid] = 0.f;
    __syncthreads();
    const int warp = (blockIdx.x * blockDim.x + tid) >> 5, lane = tid & 31;
    if (warp < nodes) {
        for (int k = lane; k < H; k += 32) {
            float acc = 0.f;
            for (int o = 0; o < OUT; ++o) {
                const float dd = d[warp * OUT + o];
                acc += dd * bf(W[o * H + k]);
                atomicAdd(&sW[o * H + k], dd * x[static_cast<size_t>(warp) * H + k]);
            }
            dx[static_cast<size_t>(warp) * H + k] = acc;
        }
        if (lane < OUT) atomicAdd(&sdb[lane], d[warp * OUT + lane]);
    }
    __syncthreads();
    if (tid < OUT * H) atomicAdd(&dW[tid], sW[tid]);
    if (tid < OUT) atomicAdd(&db[tid], sdb[tid]);
}

// g = d * (y > 0) in place
__global__ void k_relu_mask(size_t n, const float* __restrict__ y, float* __restrict__ d) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && !(y[i] > 0.f)) d[i] = 0.f;
}

// dx[node][k] = sum_o g[node][o] W[o][k] (accumulate or overwrite); 32 nodes per block
__global__ void __launch_bounds__(256) k_lin_bwd_x(int nodes, const float* __restrict__ g,
                                                   const uint16_t* __restrict__ W, float* __restrict__ dx,
                                                   int accumulate) {
    __shared__ float sW[H * H];   // [o][k]
    __shared__ float gs[32][H + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < H * H; idx += 256) sW[idx] = bf(W[idx]);
    const int n0 = blockIdx.x * 32;
    for (int idx = tid; idx < 32 * H; idx += 256) {
        const int nn = idx / H, o = idx % H;
        const int node = n0 + nn;
        gs[nn][o] = node < nodes ? g[static_cast<size_t>(node) * H + o] : 0.f;
    }
    __syncthreads();
    const int k = tid & (H - 1), grp = tid >> 6;
    for (int nn = grp; nn < 32; nn += 4) {
        const int node = n0 + nn;
        if (node >= nodes) break;
        float acc = 0.f;
        for (int o = 0; o < H; ++o) acc += gs[nn][o] * sW[o * H + k];
        float* p = dx + static_cast<size_t>(node) * H + k;
        *p = accumulate ? *p + acc : acc;
    }
}

// dW[o][k] += sum_node g[node][o] x[node][k]; db[o] += sum_node g[node][o]; 256 nodes per block
template <int IN>
__global__ void __launch_bounds__(256) k_lin_bwd_w(int nodes, const float* __restrict__ g, const float* __restrict__ x,
                                                   float* __restrict__ dW, float* __restrict__ db) {
    constexpr int KG = IN >= 16 ? IN / 4 : IN;   // k per thread
    const int tid = threadIdx.x;
    const int o = tid & (H - 1), kg = tid >> 6;
    float acc[KG];
#pragma unroll
    for (int q = 0; q < KG; ++q) acc[q] = 0.f;
    float accb = 0.f;
    const int n0 = blockIdx.x * 256;
    const int n1 = min(nodes, n0 + 256);
    const bool active = IN >= 16 || kg == 0;
    for (int node = n0; node < n1; ++node) {
        const float gv = g[static_cast<size_t>(node) * H + o];
        if (gv == 0.f) continue;
        if (kg == 0) accb += gv;
        if (active)
#pragma unroll
            for (int q = 0; q < KG; ++q) acc[q] += gv * x[static_cast<size_t>(node) * IN + (IN >= 16 ? kg * KG : 0) + q];
    }
    if (active)
#pragma unroll
        for (int q = 0; q < KG; ++q) atomicAdd(&dW[o * IN + (IN >= 16 ? kg * KG : 0) + q], acc[q]);
    if (kg == 0) atomicAdd(&db[o], accb);
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = isfinite(g[i]) ? fminf(fmaxf(g[i], -10.f), 10.f) : 0.f;
    m[i] = 0.9f * m[i] + 0.1f * gi;
    v[i] = 0.999f * v[i] + 0.001f * gi * gi;
    w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + 1e-8f);
}

__global__ void k_out_f64(int n, int stride, int off, const float* __restrict__ in, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = static_cast<double>(in[static_cast<size_t>(i) * stride + off]);
}

inline int nb(int64_t n, int t = 256) { return static_cast<int>((n + t - 1) / t); }

}  // namespace

Gnn::Gnn(unsigned long long seed) {
    nparams_ = kLay.total;
    SK_CUDA(cudaMalloc(&master_, sizeof(float) * nparams_));
    SK_CUDA(cudaMalloc(&wbf_, sizeof(uint16_t) * nparams_));
    SK_CUDA(cudaMalloc(&grad_, sizeof(float) * nparams_));
    SK_CUDA(cudaMalloc(&adam_m_, sizeof(float) * nparams_));
    SK_CUDA(cudaMalloc(&adam_v_, sizeof(float) * nparams_));
    SK_CUDA(cudaMalloc(&loss_, sizeof(double)));
    SK_CUDA(cudaMemset(adam_m_, 0, sizeof(float) * nparams_));
    SK_CUDA(cudaMemset(adam_v_, 0, sizeof(float) * nparams_));
    // Glorot-uniform weights, zero biases (portable splitmix64 stream)
    std::vector<float> w(nparams_, 0.f);
    uint64_t st = seed ? seed : 0x5eedULL;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](size_t off, int fo, int fi) {
        const double lim = std::sqrt(6.0 / (fo + fi));
        for (int q = 0; q < fo * fi; ++q) w[off + q] = static_cast<float>((2.0 * next() - 1.0) * lim);
    };
    fill(kLay.Ec, H, 3);
    fill(kLay.Er, H, 3);
    for (int l = 0; l < L; ++l) {
        fill(kLay.Wrr[l], H, H); fill(kLay.Wrm[l], H, H); fill(kLay.Wcc[l], H, H); fill(kLay.Wcm[l], H, H);
    }
    fill(kLay.Hc, 2, H);
    fill(kLay.Hr, 1, H);
    for (size_t q = 0; q < H; ++q) { w[kLay.ec + q] = 0.01f; w[kLay.er + q] = 0.01f; }
    set_params(w.data());
}

Gnn::~Gnn() {
    for (void* p : {static_cast<void*>(master_), static_cast<void*>(wbf_), static_cast<void*>(grad_),
                    static_cast<void*>(adam_m_), static_cast<void*>(adam_v_), static_cast<void*>(loss_),
                    static_cast<void*>(fc_), static_cast<void*>(fr_), static_cast<void*>(hc_),
                    static_cast<void*>(hr_), static_cast<void*>(mc_), static_cast<void*>(mr_),
                    static_cast<void*>(oc_), static_cast<void*>(or_), static_cast<void*>(dc_),
                    static_cast<void*>(dr_), static_cast<void*>(dm_), static_cast<void*>(dt_),
                    static_cast<void*>(inv_deg_r_), static_cast<void*>(inv_deg_c_)})
        if (p) cudaFree(p);
}

void Gnn::get_params(float* out) const {
    SK_CUDA(cudaMemcpy(out, master_, sizeof(float) * nparams_, cudaMemcpyDeviceToHost));
}

void Gnn::set_params(const float* in) {
    SK_CUDA(cudaMemcpy(master_, in, sizeof(float) * nparams_, cudaMemcpyHostToDevice));
    k_to_bf16<<<nb(static_cast<int64_t>(nparams_)), 256>>>(static_cast<int>(nparams_), master_, wbf_);
    SK_CUDA(cudaGetLastError());
    SK_CUDA(cudaDeviceSynchronize());
}

void Gnn::ensure(const DeviceLP& lp) {
    if (lp.N <= capN_ && lp.M <= capM_) return;
    for (float** p : {&fc_, &fr_, &hc_, &hr_, &mc_, &mr_, &oc_, &or_, &dc_, &dr_, &dm_, &dt_, &inv_deg_r_, &inv_deg_c_})
        if (*p) { cudaFree(*p); *p = nullptr; }
    capN_ = lp.N;
    capM_ = lp.M;
    const size_t N = capN_, M = capM_, X = std::max(N, M);
    SK_CUDA(cudaMalloc(&fc_, sizeof(float) * N * 3));
    SK_CUDA(cudaMalloc(&fr_, sizeof(float) * M * 3));
    SK_CUDA(cudaMalloc(&hc_, sizeof(float) * (L + 1) * N * H));
    SK_CUDA(cudaMalloc(&hr_, sizeof(float) * (L + 1) * M * H));
    SK_CUDA(cudaMalloc(&mc_, sizeof(float) * L * N * H));
    SK_CUDA(cudaMalloc(&mr_, sizeof(float) * L * M * H));
    SK_CUDA(cudaMalloc(&oc_, sizeof(float) * N * 2));
    SK_CUDA(cudaMalloc(&or_, sizeof(float) * M));
    SK_CUDA(cudaMalloc(&dc_, sizeof(float) * 2 * N * H));
    SK_CUDA(cudaMalloc(&dr_, sizeof(float) * 2 * M * H));
    SK_CUDA(cudaMalloc(&dm_, sizeof(float) * X * H));
    SK_CUDA(cudaMalloc(&dt_, sizeof(float) * X * H));
    SK_CUDA(cudaMalloc(&inv_deg_r_, sizeof(float) * M));
    SK_CUDA(cudaMalloc(&inv_deg_c_, sizeof(float) * N));
}

double Gnn::forward(const DeviceLP& lp, cudaStream_t st, double* out_logx, double* out_logs, double* out_y,
                    const double* t_logx, const double* t_logs, const double* t_y) {
    ensure(lp);
    const int N = lp.N, M = lp.M;
    const size_t NH = static_cast<size_t>(N) * H, MH = static_cast<size_t>(M) * H;
    const uint16_t* w = wbf_;
    k_features<<<nb(N), 256, 0, st>>>(N, lp.t_rp, lp.t_v, lp.c, fc_, inv_deg_c_);
    k_features<<<nb(M), 256, 0, st>>>(M, lp.a_rp, lp.a_v, lp.b, fr_, inv_deg_r_);
    k_embed<<<nb(static_cast<int64_t>(N) * H), 256, 0, st>>>(N, fc_, w + kLay.Ec, w + kLay.ec, hc_);
    k_embed<<<nb(static_cast<int64_t>(M) * H), 256, 0, st>>>(M, fr_, w + kLay.Er, w + kLay.er, hr_);
    for (int l = 0; l < L; ++l) {
        float* hcl = hc_ + l * NH;
        float* hrl = hr_ + l * MH;
        k_spmm<<<nb(static_cast<int64_t>(M) * 32), 256, 0, st>>>(M, lp.a_rp, lp.a_ci, lp.a_v, inv_deg_r_, nullptr,
                                                                  hcl, mr_ + l * MH, 0);
        k_layer<<<nb(M, 32), 256, 0, st>>>(M, hrl, mr_ + l * MH, w + kLay.Wrr[l], w + kLay.Wrm[l], w + kLay.br[l],
                                            hrl + MH);
        k_spmm<<<nb(static_cast<int64_t>(N) * 32), 256, 0, st>>>(N, lp.t_rp, lp.t_ci, lp.t_v, inv_deg_c_, nullptr,
                                                                  hrl + MH, mc_ + l * NH, 0);
        k_layer<<<nb(N, 32), 256, 0, st>>>(N, hcl, mc_ + l * NH, w + kLay.Wcc[l], w + kLay.Wcm[l], w + kLay.bc[l],
                                            hcl + NH);
    }
    k_head<<<nb(static_cast<int64_t>(N) * 32), 256, 0, st>>>(N, 2, hc_ + L * NH, w + kLay.Hc, w + kLay.oc, oc_);
    k_head<<<nb(static_cast<int64_t>(M) * 32), 256, 0, st>>>(M, 1, hr_ + L * MH, w + kLay.Hr, w + kLay.orr, or_);
    if (out_logx) k_out_f64<<<nb(N), 256, 0, st>>>(N, 2, 0, oc_, out_logx);
    if (out_logs) k_out_f64<<<nb(N), 256, 0, st>>>(N, 2, 1, oc_, out_logs);
    if (out_y) k_out_f64<<<nb(M), 256, 0, st>>>(M, 1, 0, or_, out_y);
    SK_CUDA(cudaGetLastError());
    t_logx_ = t_logx;
    t_logs_ = t_logs;
    t_y_ = t_y;
    if (!t_logx) return 0.0;
    SK_CUDA(cudaMemsetAsync(loss_, 0, sizeof(double), st));
    // d_oc -> dm_ (N x 2), d_or -> dt_ (M)
    k_loss<<<nb(static_cast<int64_t>(N) + M), 256, 0, st>>>(N, M, oc_, or_, t_logx, t_logs, t_y, dm_, dt_, loss_);
    double h = 0.0;
    SK_CUDA(cudaMemcpyAsync(&h, loss_, sizeof(double), cudaMemcpyDeviceToHost, st));
    SK_CUDA(cudaStreamSynchronize(st));
    return h;
}

void Gnn::backward(const DeviceLP& lp, cudaStream_t st, float* grad_host) {
    const int N = lp.N, M = lp.M;
    const size_t NH = static_cast<size_t>(N) * H, MH = static_cast<size_t>(M) * H;
    const uint16_t* w = wbf_;
    float* gr = grad_;
    SK_CUDA(cudaMemsetAsync(gr, 0, sizeof(float) * nparams_, st));
    float* dhc = dc_;          // gradient w.r.t. hc[l] (current)
    float* dhc2 = dc_ + NH;    // next buffer
    float* dhr = dr_;
    float* dhr2 = dr_ + MH;
    // heads: dm_ holds d_oc (N x 2), dt_ holds d_or (M)
    k_head_bwd<<<nb(static_cast<int64_t>(N) * 32), 256, 0, st>>>(N, 2, hc_ + L * NH, dm_, w + kLay.Hc, dhc,
                                                                  gr + kLay.Hc, gr + kLay.oc);
    k_head_bwd<<<nb(static_cast<int64_t>(M) * 32), 256, 0, st>>>(M, 1, hr_ + L * MH, dt_, w + kLay.Hr, dhr,
                                                                  gr + kLay.Hr, gr + kLay.orr);
    for (int l = L - 1; l >= 0; --l) {
        float* hcl = hc_ + l * NH;
        float* hrl = hr_ + l * MH;
        // hc[l+1] = relu(Wcc hc[l] + Wcm mc[l] + bc)
        k_relu_mask<<<nb(static_cast<int64_t>(NH)), 256, 0, st>>>(NH, hcl + NH, dhc);
        k_lin_bwd_w<H><<<nb(N), 256, 0, st>>>(N, dhc, hcl, gr + kLay.Wcc[l], gr + kLay.bc[l]);
        k_lin_bwd_w<H><<<nb(N), 256, 0, st>>>(N, dhc, mc_ + l * NH, gr + kLay.Wcm[l], dt_);   // bias already taken
        k_lin_bwd_x<<<nb(N, 32), 256, 0, st>>>(N, dhc, w + kLay.Wcc[l], dhc2, 0);            // -> d hc[l]
        k_lin_bwd_x<<<nb(N, 32), 256, 0, st>>>(N, dhc, w + kLay.Wcm[l], dm_, 0);             // -> d mc[l]
        // mc[l] = diag(inv_deg_c) A^T hr[l+1]  =>  d hr[l+1] += A diag(inv_deg_c) d mc
        k_spmm<<<nb(static_cast<int64_t>(M) * 32), 256, 0, st>>>(M, lp.a_rp, lp.a_ci, lp.a_v, nullptr, inv_deg_c_,
                                                                  dm_, dhr, 1);
        // hr[l+1] = relu(Wrr hr[l] + Wrm mr[l] + br)
        k_relu_mask<<<nb(static_cast<int64_t>(MH)), 256, 0, st>>>(MH, hrl + MH, dhr);
        k_lin_bwd_w<H><<<nb(M), 256, 0, st>>>(M, dhr, hrl, gr + kLay.Wrr[l], gr + kLay.br[l]);
        k_lin_bwd_w<H><<<nb(M), 256, 0, st>>>(M, dhr, mr_ + l * MH, gr + kLay.Wrm[l], dt_);
        k_lin_bwd_x<<<nb(M, 32), 256, 0, st>>>(M, dhr, w + kLay.Wrr[l], dhr2, 0);            // -> d hr[l]
        k_lin_bwd_x<<<nb(M, 32), 256, 0, st>>>(M, dhr, w + kLay.Wrm[l], dm_, 0);             // -> d mr[l]
        // mr[l] = diag(inv_deg_r) A hc[l]  =>  d hc[l] += A^T diag(inv_deg_r) d mr
        k_spmm<<<nb(static_cast<int64_t>(N) * 32), 256, 0, st>>>(N, lp.t_rp, lp.t_ci, lp.t_v, nullptr, inv_deg_r_,
                                                                  dm_, dhc2, 1);
        std::swap(dhc, dhc2);
        std::swap(dhr, dhr2);
    }
    // embeddings
    k_relu_mask<<<nb(static_cast<int64_t>(NH)), 256, 0, st>>>(NH, hc_, dhc);
    k_lin_bwd_w<3><<<nb(N), 256, 0, st>>>(N, dhc, fc_, gr + kLay.Ec, gr + kLay.ec);
    k_relu_mask<<<nb(static_cast<int64_t>(MH)), 256, 0, st>>>(MH, hr_, dhr);
    k_lin_bwd_w<3><<<nb(M), 256, 0, st>>>(M, dhr, fr_, gr + kLay.Er, gr + kLay.er);
    SK_CUDA(cudaGetLastError());
    if (grad_host) {
        SK_CUDA(cudaMemcpyAsync(grad_host, gr, sizeof(float) * nparams_, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
    }
}

void Gnn::adam_step(cudaStream_t st, float lr) {
    ++adam_t_;
    const float c1 = 1.f - std::pow(0.9f, static_cast<float>(adam_t_));
    const float c2 = 1.f - std::pow(0.999f, static_cast<float>(adam_t_));
    k_adam<<<nb(static_cast<int64_t>(nparams_)), 256, 0, st>>>(static_cast<int>(nparams_), master_, grad_, adam_m_,
                                                                 adam_v_, lr, c1, c2);
    k_to_bf16<<<nb(static_cast<int64_t>(nparams_)), 256, 0, st>>>(static_cast<int>(nparams_), master_, wbf_);
    SK_CUDA(cudaGetLastError());
}

}  // namespace dev
}  // namespace sankhya
