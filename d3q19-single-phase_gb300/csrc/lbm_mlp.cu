// Learned LES closure, training side: the eddy-viscosity network
// (lbm_mlp.cuh) trained on the GPU with hand-written forward, backward and
// Adam kernels.  The reference has no counterpart.
//
// One CTA of 128 threads takes a tile of 128 samples and runs the forward
// pass, the loss and the backward pass in shared memory; weight gradients go
// to a global FP32 buffer with one atomic per weight and CTA, and k_adam
// applies Adam (Kingma & Ba 2015) to the FP32 master weights.  The five matrix
// products of a tile (X W1, H1 W2, H1^T dZ2, dZ2 W2^T, X^T dZ1) run on the
// tensor cores through mma.sync m16n8k16 with BF16 operands rounded from the
// FP32 values and FP32 accumulation; an FP32 FMA path of the same structure
// serves the gradient checks.  The products are 128x32x32 tiles, so a training
// step is bound by the latency of a tile's chain of stages (two waves of 512
// tiles at two CTAs per SM), not by the tensor-core rate; the gradient atomics
// take about 3% of it (measured against a copy without them).
//
// Loss: mean squared error of nu_t / nu against the targets.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lbm_internal.h"
#include "lbm_mlp.cuh"

namespace lbm {
int set_error(int code, const char* msg);   // lbm_capi.cu
}

struct lbm_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    float* d_param = nullptr;   // [kMlpParams]
    float* d_grad = nullptr;    // [kMlpParams]
    float* d_m = nullptr;       // Adam first moment
    float* d_v = nullptr;       // Adam second moment
    float* d_norm = nullptr;    // [kMlpNorm]: mean, 1/std
    float* d_X = nullptr;       // [n][kMlpIn]
    float* d_y = nullptr;       // [n]
    double* d_loss = nullptr;   // [loss_cap]
    int64_t n = 0, cap = 0, loss_cap = 0;
    int64_t t = 0;              // Adam steps taken
    uint64_t seed = 0;
};

namespace lbm {
namespace {

constexpr int kTile = 128;
// shared-memory layout of k_mlp_train (floats)
constexpr int kXs = 0;                      // [128][16] standardised inputs, zero-padded
constexpr int kW1s = kXs + kTile * 16;      // [16][32], rows >= 7 zero
constexpr int kW2s = kW1s + 16 * kMlpH;     // [32][32]
constexpr int kB1s = kW2s + kMlpH * kMlpH;
constexpr int kB2s = kB1s + kMlpH;
constexpr int kW3s = kB2s + kMlpH;
constexpr int kB3s = kW3s + kMlpH;          // 1 (+3 pad)
constexpr int kZ1 = kB3s + 4;               // [128][32]
constexpr int kH1 = kZ1 + kTile * kMlpH;
constexpr int kZ2 = kH1 + kTile * kMlpH;
constexpr int kH2 = kZ2 + kTile * kMlpH;
constexpr int kT = kH2 + kTile * kMlpH;     // [32][32] weight-gradient tile
constexpr int kDz3 = kT + kMlpH * kMlpH;    // [128]
constexpr int kSmemFloats = kDz3 + kTile;
constexpr size_t kTrainSmem = (size_t)kSmemFloats * sizeof(float);

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[m][n] = sum_k A(m,k) B(k,n) (+ bias[n]) for an M x N tile in shared
// memory, A(m,k) = A[m*am + k*ak], B(k,n) = B[k*bk + n*bn], C[m*ldc + n];
// M a multiple of 16, N of 8, K of 16.  C must not alias A or B.
template <bool TC>
__device__ void tile_gemm(const float* A, int am, int ak, const float* B, int bk, int bn, float* C, int ldc,
                          int M, int N, int K, const float* bias) {
    if constexpr (TC) {
        // mma.sync m16n8k16 fragments (PTX ISA): lane = 4*gid + tig;
        // A regs: (gid, 2tig..), (gid+8, 2tig..), (gid, 2tig+8..), (gid+8, 2tig+8..)
        // B regs: (k = 2tig.., n = gid), (k = 2tig+8.., n = gid)
        // C: (gid, 2tig..), (gid+8, 2tig..)
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
        const int gid = lane >> 2, tig = lane & 3;
        const int tn = N / 8, ntile = (M / 16) * tn;
        for (int t = warp; t < ntile; t += nwarp) {
            const int m0 = (t / tn) * 16, n0 = (t % tn) * 8;
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            const float* Ar0 = A + (m0 + gid) * am;
            const float* Ar1 = A + (m0 + gid + 8) * am;
            const float* Bc = B + (n0 + gid) * bn;
            for (int k0 = 0; k0 < K; k0 += 16) {
                const int k = k0 + 2 * tig;
                uint32_t a[4], b[2];
                a[0] = pack_bf16(Ar0[k * ak], Ar0[(k + 1) * ak]);
                a[1] = pack_bf16(Ar1[k * ak], Ar1[(k + 1) * ak]);
                a[2] = pack_bf16(Ar0[(k + 8) * ak], Ar0[(k + 9) * ak]);
                a[3] = pack_bf16(Ar1[(k + 8) * ak], Ar1[(k + 9) * ak]);
                b[0] = pack_bf16(Bc[k * bk], Bc[(k + 1) * bk]);
                b[1] = pack_bf16(Bc[(k + 8) * bk], Bc[(k + 9) * bk]);
                mma_bf16(c, a, b);
            }
            const int r0 = m0 + gid, cc = n0 + 2 * tig;
            const float b0 = bias ? bias[cc] : 0.f, b1 = bias ? bias[cc + 1] : 0.f;
            C[r0 * ldc + cc] = c[0] + b0;
            C[r0 * ldc + cc + 1] = c[1] + b1;
            C[(r0 + 8) * ldc + cc] = c[2] + b0;
            C[(r0 + 8) * ldc + cc + 1] = c[3] + b1;
        }
    } else {
        for (int e = threadIdx.x; e < M * N; e += blockDim.x) {
            const int m = e / N, n = e - m * N;
            float acc = bias ? bias[n] : 0.f;
            for (int k = 0; k < K; ++k) acc += A[m * am + k * ak] * B[k * bk + n * bn];
            C[m * ldc + n] = acc;
        }
    }
}

// sample index of row `row` of a random batch
__device__ __forceinline__ int64_t batch_index(uint64_t seed, int64_t step, int64_t row, int64_t n) {
    const uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)step * 0x9E3779B97F4A7C15ull + (uint64_t)row));
    return (int64_t)(h % (uint64_t)n);
}

// One tile of 128 samples: forward, loss, backward; gradients (of the mean
// loss: inv_count = 1 / samples) added to G, the loss sum to *loss.
// mode 0: rows blockIdx.x*128 + r of the data (masked beyond n);
// mode 1: `rows` random samples drawn with (seed, step).
template <bool TC>
__global__ void __launch_bounds__(kTile)
k_mlp_train(const float* __restrict__ P, const float* __restrict__ norm, const float* __restrict__ X,
            const float* __restrict__ y, int64_t n, int mode, int64_t rows, uint64_t seed, int64_t step,
            float inv_count, float* __restrict__ G, double* __restrict__ loss) {
    extern __shared__ float sm[];
    float* Xs = sm + kXs;
    float* W1s = sm + kW1s;
    float* W2s = sm + kW2s;
    float* b1s = sm + kB1s;
    float* b2s = sm + kB2s;
    float* w3s = sm + kW3s;
    float* Z1 = sm + kZ1;
    float* H1 = sm + kH1;
    float* Z2 = sm + kZ2;
    float* H2 = sm + kH2;
    float* T = sm + kT;
    float* dz3 = sm + kDz3;
    const int r = threadIdx.x;
    const int64_t row = (int64_t)blockIdx.x * kTile + r;
    bool valid;
    int64_t idx = 0;
    if (mode == 0) {
        valid = row < n;
        idx = row;
    } else {
        valid = row < rows;
        if (valid) idx = batch_index(seed, step, row, n);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k)
        Xs[r * 16 + k] = (valid && k < kMlpIn) ? (X[idx * kMlpIn + k] - norm[k]) * norm[kMlpIn + k] : 0.f;
    for (int e = r; e < 16 * kMlpH; e += kTile) W1s[e] = e < kMlpIn * kMlpH ? P[kOffW1 + e] : 0.f;
    for (int e = r; e < kMlpH * kMlpH; e += kTile) W2s[e] = P[kOffW2 + e];
    if (r < kMlpH) {
        b1s[r] = P[kOffB1 + r];
        b2s[r] = P[kOffB2 + r];
        w3s[r] = P[kOffW3 + r];
    }
    const float b3 = P[kOffB3];
    __syncthreads();
    // forward
    tile_gemm<TC>(Xs, 16, 1, W1s, kMlpH, 1, Z1, kMlpH, kTile, kMlpH, 16, b1s);
    __syncthreads();
    for (int e = r; e < kTile * kMlpH; e += kTile) H1[e] = mlp_silu(Z1[e]);
    __syncthreads();
    tile_gemm<TC>(H1, kMlpH, 1, W2s, kMlpH, 1, Z2, kMlpH, kTile, kMlpH, kMlpH, b2s);
    __syncthreads();
    for (int e = r; e < kTile * kMlpH; e += kTile) H2[e] = mlp_silu(Z2[e]);
    __syncthreads();
    float z3 = b3;
    for (int j = 0; j < kMlpH; ++j) z3 += H2[r * kMlpH + j] * w3s[j];
    const float diff = valid ? mlp_softplus(z3) - y[idx] : 0.f;
    dz3[r] = 2.f * diff * mlp_sigmoid(z3) * inv_count;
    double lsum = (double)diff * (double)diff;
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((r & 31) == 0) atomicAdd(loss, lsum);
    __syncthreads();
    // backward: output layer
    if (r < kMlpH) {
        float s = 0.f;
        for (int q = 0; q < kTile; ++q) s += dz3[q] * H2[q * kMlpH + r];
        atomicAdd(&G[kOffW3 + r], s);
    } else if (r == kMlpH) {
        float s = 0.f;
        for (int q = 0; q < kTile; ++q) s += dz3[q];
        atomicAdd(&G[kOffB3], s);
    }
    __syncthreads();
    // dZ2 (into H2)
    for (int e = r; e < kTile * kMlpH; e += kTile) H2[e] = dz3[e / kMlpH] * w3s[e % kMlpH] * mlp_silu_grad(Z2[e]);
    __syncthreads();
    if (r < kMlpH) {
        float s = 0.f;
        for (int q = 0; q < kTile; ++q) s += H2[q * kMlpH + r];
        atomicAdd(&G[kOffB2 + r], s);
    }
    // dW2 = H1^T dZ2
    tile_gemm<TC>(H1, 1, kMlpH, H2, kMlpH, 1, T, kMlpH, kMlpH, kMlpH, kTile, nullptr);
    __syncthreads();
    for (int e = r; e < kMlpH * kMlpH; e += kTile) atomicAdd(&G[kOffW2 + e], T[e]);
    // dH1 = dZ2 W2^T (into Z2)
    tile_gemm<TC>(H2, kMlpH, 1, W2s, 1, kMlpH, Z2, kMlpH, kTile, kMlpH, kMlpH, nullptr);
    __syncthreads();
    // dZ1 (in place)
    for (int e = r; e < kTile * kMlpH; e += kTile) Z2[e] *= mlp_silu_grad(Z1[e]);
    __syncthreads();
    if (r < kMlpH) {
        float s = 0.f;
        for (int q = 0; q < kTile; ++q) s += Z2[q * kMlpH + r];
        atomicAdd(&G[kOffB1 + r], s);
    }
    // dW1 = X^T dZ1 (rows >= 7 are padding)
    tile_gemm<TC>(Xs, 1, 16, Z2, kMlpH, 1, T, kMlpH, 16, kMlpH, kTile, nullptr);
    __syncthreads();
    for (int e = r; e < kMlpIn * kMlpH; e += kTile) atomicAdd(&G[kOffW1 + e], T[e]);
}

__global__ void k_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M, float* __restrict__ V,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float m = b1 * M[i] + (1.f - b1) * g;
    const float v = b2 * V[i] + (1.f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
    G[i] = 0.f;
}

__global__ void k_mlp_predict(const float* __restrict__ P, const float* __restrict__ norm,
                              const float* __restrict__ X, int64_t n, float* __restrict__ out) {
    __shared__ __align__(16) float Ps[kMlpParams];
    __shared__ float Ns[kMlpNorm];
    for (int e = threadIdx.x; e < kMlpParams; e += blockDim.x) Ps[e] = P[e];
    for (int e = threadIdx.x; e < kMlpNorm; e += blockDim.x) Ns[e] = norm[e];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) x[k] = X[i * kMlpIn + k];
    out[i] = mlp_infer_pairs(Ps, Ns, x);
}

// deterministic initial weights: uniform(-a, a) with a = sqrt(6 / (fan_in +
// fan_out)) (Glorot & Bengio 2010), zero biases
void init_params(uint64_t seed, std::vector<float>& p) {
    p.assign(kMlpParams, 0.f);
    uint64_t s = seed;
    auto uni = [&]() {
        s = splitmix64(s);
        return (double)(s >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    const double a1 = std::sqrt(6.0 / (kMlpIn + kMlpH)), a2 = std::sqrt(6.0 / (2 * kMlpH)),
                 a3 = std::sqrt(6.0 / (kMlpH + 1));
    for (int e = 0; e < kMlpIn * kMlpH; ++e) p[kOffW1 + e] = (float)(a1 * uni());
    for (int e = 0; e < kMlpH * kMlpH; ++e) p[kOffW2 + e] = (float)(a2 * uni());
    for (int e = 0; e < kMlpH; ++e) p[kOffW3 + e] = (float)(a3 * uni());
}

int cuda_err(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LBM_OK;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return set_error(LBM_ERR_CUDA, buf);
}
#define MCK(call) do { if (int rc_ = cuda_err((call), #call)) return rc_; } while (0)

int use_device(const lbm_mlp* m) { return cuda_err(cudaSetDevice(m->device), "cudaSetDevice"); }

int ensure_loss(lbm_mlp* m, int64_t k) {
    if (m->loss_cap >= k) return LBM_OK;
    cudaFree(m->d_loss);
    m->d_loss = nullptr;
    MCK(cudaMalloc(&m->d_loss, (size_t)k * sizeof(double)));
    m->loss_cap = k;
    return LBM_OK;
}

template <bool TC>
int launch_train(lbm_mlp* m, int mode, int64_t rows, int64_t step, float inv_count, double* loss) {
    MCK(cudaFuncSetAttribute(k_mlp_train<TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
    const int64_t nb = (rows + kTile - 1) / kTile;
    k_mlp_train<TC><<<(unsigned)nb, kTile, kTrainSmem, m->stream>>>(m->d_param, m->d_norm, m->d_X, m->d_y, m->n,
                                                                      mode, rows, m->seed, step, inv_count,
                                                                      m->d_grad, loss);
    return cuda_err(cudaGetLastError(), "k_mlp_train");
}

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_mlp_create(lbm_mlp** out, uint64_t seed, int32_t device) {
    if (!out) return set_error(LBM_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    lbm_mlp* m = new lbm_mlp();
    m->device = device;
    m->seed = seed;
    auto bail = [&](int rc) { lbm_mlp_destroy(m); return rc; };
    if (int rc = use_device(m)) return bail(rc);
    if (int rc = cuda_err(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate"))
        return bail(rc);
    float* blk = nullptr;
    if (int rc = cuda_err(cudaMalloc(&blk, (4 * (size_t)kMlpParams + kMlpNorm) * sizeof(float)), "cudaMalloc"))
        return bail(rc);
    m->d_param = blk;
    m->d_grad = blk + kMlpParams;
    m->d_m = blk + 2 * kMlpParams;
    m->d_v = blk + 3 * kMlpParams;
    m->d_norm = blk + 4 * kMlpParams;
    std::vector<float> p;
    init_params(seed, p);
    std::vector<float> norm(kMlpNorm, 0.f);
    for (int k = 0; k < kMlpIn; ++k) norm[kMlpIn + k] = 1.f;
    if (int rc = cuda_err(cudaMemcpy(m->d_param, p.data(), kMlpParams * 4, cudaMemcpyHostToDevice), "upload"))
        return bail(rc);
    if (int rc = cuda_err(cudaMemset(m->d_grad, 0, 3 * (size_t)kMlpParams * 4), "cudaMemset")) return bail(rc);
    if (int rc = cuda_err(cudaMemcpy(m->d_norm, norm.data(), kMlpNorm * 4, cudaMemcpyHostToDevice), "upload"))
        return bail(rc);
    *out = m;
    return LBM_OK;
}

int lbm_mlp_destroy(lbm_mlp* m) {
    if (!m) return LBM_OK;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->d_param);
    cudaFree(m->d_X);
    cudaFree(m->d_loss);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return LBM_OK;
}

int lbm_mlp_get(lbm_mlp* m, float* params, float* norm) {
    if (!m) return set_error(LBM_ERR_INVALID_ARG, "null network");
    if (int rc = use_device(m)) return rc;
    MCK(cudaStreamSynchronize(m->stream));
    if (params) MCK(cudaMemcpy(params, m->d_param, kMlpParams * 4, cudaMemcpyDeviceToHost));
    if (norm) MCK(cudaMemcpy(norm, m->d_norm, kMlpNorm * 4, cudaMemcpyDeviceToHost));
    return LBM_OK;
}

int lbm_mlp_set(lbm_mlp* m, const float* params, const float* norm) {
    if (!m) return set_error(LBM_ERR_INVALID_ARG, "null network");
    if (int rc = use_device(m)) return rc;
    MCK(cudaStreamSynchronize(m->stream));
    if (params) {
        MCK(cudaMemcpy(m->d_param, params, kMlpParams * 4, cudaMemcpyHostToDevice));
        MCK(cudaMemset(m->d_grad, 0, 3 * (size_t)kMlpParams * 4));   // gradient and Adam state restart
        m->t = 0;
    }
    if (norm) {
        for (int k = 0; k < kMlpIn; ++k)
            if (!(std::isfinite(norm[k]) && std::isfinite(norm[kMlpIn + k]) && norm[kMlpIn + k] > 0.f))
                return set_error(LBM_ERR_INVALID_ARG, "bad feature normalisation");
        MCK(cudaMemcpy(m->d_norm, norm, kMlpNorm * 4, cudaMemcpyHostToDevice));
    }
    return LBM_OK;
}

int lbm_mlp_set_data(lbm_mlp* m, const float* X, const float* y, int64_t n, int32_t set_norm) {
    if (!m || !X || !y || n <= 0) return set_error(LBM_ERR_INVALID_ARG, "null data or empty set");
    if (int rc = use_device(m)) return rc;
    MCK(cudaStreamSynchronize(m->stream));
    if (n > m->cap) {
        cudaFree(m->d_X);
        m->d_X = nullptr;
        MCK(cudaMalloc(&m->d_X, (size_t)n * (kMlpIn + 1) * sizeof(float)));
        m->cap = n;
    }
    m->d_y = m->d_X + (size_t)m->cap * kMlpIn;
    MCK(cudaMemcpy(m->d_X, X, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->d_y, y, (size_t)n * 4, cudaMemcpyHostToDevice));
    m->n = n;
    if (set_norm) {
        // per-feature mean and inverse standard deviation of the data (FP64 sums)
        float norm[kMlpNorm];
        for (int k = 0; k < kMlpIn; ++k) {
            double s = 0.0, s2 = 0.0;
            for (int64_t i = 0; i < n; ++i) {
                const double v = X[i * kMlpIn + k];
                s += v;
                s2 += v * v;
            }
            const double mean = s / (double)n;
            const double var = std::max(s2 / (double)n - mean * mean, 0.0);
            norm[k] = (float)mean;
            norm[kMlpIn + k] = (float)(1.0 / std::sqrt(var + 1e-12));
        }
        MCK(cudaMemcpy(m->d_norm, norm, sizeof(norm), cudaMemcpyHostToDevice));
    }
    return LBM_OK;
}

int lbm_mlp_train(lbm_mlp* m, int32_t steps, int32_t batch, float lr, int32_t flags, float* losses) {
    if (!m || steps < 0 || batch <= 0) return set_error(LBM_ERR_INVALID_ARG, "bad training arguments");
    if (m->n == 0) return set_error(LBM_ERR_STATE, "no training data (lbm_mlp_set_data)");
    if (int rc = use_device(m)) return rc;
    if (int rc = ensure_loss(m, std::max(steps, 1))) return rc;
    MCK(cudaMemsetAsync(m->d_loss, 0, (size_t)std::max(steps, 1) * sizeof(double), m->stream));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const bool fp32 = (flags & LBM_MLP_FP32) != 0;
    for (int s = 0; s < steps; ++s) {
        const int64_t step = m->t;
        int rc = fp32 ? launch_train<false>(m, 1, batch, step, 1.f / (float)batch, m->d_loss + s)
                      : launch_train<true>(m, 1, batch, step, 1.f / (float)batch, m->d_loss + s);
        if (rc) return rc;
        m->t += 1;
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)m->t)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)m->t)));
        k_adam<<<(kMlpParams + 255) / 256, 256, 0, m->stream>>>(m->d_param, m->d_grad, m->d_m, m->d_v, kMlpParams,
                                                               lr, b1, b2, eps, c1, c2);
        MCK(cudaGetLastError());
    }
    if (losses && steps > 0) {
        std::vector<double> h(steps);
        MCK(cudaMemcpyAsync(h.data(), m->d_loss, (size_t)steps * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
        MCK(cudaStreamSynchronize(m->stream));
        for (int s = 0; s < steps; ++s) losses[s] = (float)(h[s] / (double)batch);
    }
    MCK(cudaStreamSynchronize(m->stream));
    return LBM_OK;
}

int lbm_mlp_gradient(lbm_mlp* m, int32_t flags, double* loss, float* grad) {
    if (!m) return set_error(LBM_ERR_INVALID_ARG, "null network");
    if (m->n == 0) return set_error(LBM_ERR_STATE, "no data (lbm_mlp_set_data)");
    if (int rc = use_device(m)) return rc;
    if (int rc = ensure_loss(m, 1)) return rc;
    MCK(cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->stream));
    MCK(cudaMemsetAsync(m->d_grad, 0, kMlpParams * sizeof(float), m->stream));
    const float inv = 1.f / (float)m->n;
    const bool fp32 = (flags & LBM_MLP_FP32) != 0;
    int rc = fp32 ? launch_train<false>(m, 0, m->n, 0, inv, m->d_loss) : launch_train<true>(m, 0, m->n, 0, inv, m->d_loss);
    if (rc) return rc;
    double l = 0.0;
    MCK(cudaMemcpyAsync(&l, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    if (grad) MCK(cudaMemcpyAsync(grad, m->d_grad, kMlpParams * 4, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    MCK(cudaMemsetAsync(m->d_grad, 0, kMlpParams * sizeof(float), m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (loss) *loss = l / (double)m->n;
    return LBM_OK;
}

int lbm_mlp_predict(lbm_mlp* m, const float* X, int64_t n, float* out) {
    if (!m || !X || !out || n < 0) return set_error(LBM_ERR_INVALID_ARG, "null argument");
    if (n == 0) return LBM_OK;
    if (int rc = use_device(m)) return rc;
    float* d = nullptr;
    MCK(cudaMalloc(&d, (size_t)n * (kMlpIn + 1) * sizeof(float)));
    int rc = LBM_OK;
    do {
        if ((rc = cuda_err(cudaMemcpyAsync(d, X, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice, m->stream), "upload"))) break;
        k_mlp_predict<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(m->d_param, m->d_norm, d, n, d + (size_t)n * kMlpIn);
        if ((rc = cuda_err(cudaGetLastError(), "k_mlp_predict"))) break;
        if ((rc = cuda_err(cudaMemcpyAsync(out, d + (size_t)n * kMlpIn, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream), "download"))) break;
        rc = cuda_err(cudaStreamSynchronize(m->stream), "sync");
    } while (false);
    cudaFree(d);
    return rc;
}

}  // extern "C"
