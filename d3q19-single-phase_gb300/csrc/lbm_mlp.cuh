// The per-node eddy-viscosity network of the learned LES closure:
// 7 inputs -> 32 -> 32 -> 1, SiLU hidden layers, softplus output (nu_t / nu
// >= 0).  Shared by the training kernels (lbm_mlp.cu) and the LES collision
// that evaluates it per node with the weights in shared memory.
//
// Parameter vector (FP32, kMlpParams floats): W1[7][32] (row = input), b1[32],
// W2[32][32] (row = input), b2[32], w3[32], b3.  Inputs are standardised with
// a per-feature mean and inverse standard deviation (norm[0..6], norm[7..13])
// before the first layer.
#pragma once

#include <cmath>

namespace lbm {

constexpr int kMlpIn = 7;
constexpr int kMlpH = 32;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpIn * kMlpH;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpH;
constexpr int kMlpParams = kOffB3 + 1;          // 1345
constexpr int kMlpNorm = 2 * kMlpIn;

__host__ __device__ inline float mlp_sigmoid(float x) { return 1.f / (1.f + expf(-x)); }
__host__ __device__ inline float mlp_silu(float x) { return x * mlp_sigmoid(x); }
// d silu / dx = s (1 + x (1 - s)), s = sigmoid(x)
__host__ __device__ inline float mlp_silu_grad(float x) {
    const float s = mlp_sigmoid(x);
    return s * (1.f + x * (1.f - s));
}
__host__ __device__ inline float mlp_softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }

// Forward pass of one sample; x: raw features, P: parameters, norm: mean and
// inverse std.  Returns nu_t / nu.
__host__ __device__ inline float mlp_infer(const float* P, const float* norm, const float* x) {
    float xn[kMlpIn];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) xn[i] = (x[i] - norm[i]) * norm[kMlpIn + i];
    float h1[kMlpH];                                 // registers: every index is a constant
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
        float z = P[kOffB1 + j];
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i) z += xn[i] * P[kOffW1 + i * kMlpH + j];
        h1[j] = mlp_silu(z);
    }
    float z3 = P[kOffB3];
#pragma unroll 2
    for (int j = 0; j < kMlpH; ++j) {
        float z = P[kOffB2 + j];
#pragma unroll
        for (int i = 0; i < kMlpH; ++i) z += h1[i] * P[kOffW2 + i * kMlpH + j];
        z3 += mlp_silu(z) * P[kOffW3 + j];
    }
    return mlp_softplus(z3);
}

#ifdef __CUDACC__
// mlp_infer on the GPU with the hidden units taken two at a time: one packed
// FP32 fused multiply-add (fma.rn.f32x2, sm_100 and later) advances units j
// and j+1, each lane with the scalar version's operation and order, so the
// result is the same bit for bit with half the multiply-add instructions.
// P must be 8-byte aligned (weight pairs are read as float2).
__device__ __forceinline__ float mlp_infer_pairs(const float* P, const float* norm, const float* x) {
    float xn[kMlpIn];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) xn[i] = (x[i] - norm[i]) * norm[kMlpIn + i];
    float h1[kMlpH];
#pragma unroll
    for (int j = 0; j < kMlpH; j += 2) {
        float2 z = *reinterpret_cast<const float2*>(P + kOffB1 + j);
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i)
            z = __ffma2_rn(make_float2(xn[i], xn[i]), *reinterpret_cast<const float2*>(P + kOffW1 + i * kMlpH + j), z);
        h1[j] = mlp_silu(z.x);
        h1[j + 1] = mlp_silu(z.y);
    }
    float z3 = P[kOffB3];
#pragma unroll 1
    for (int j = 0; j < kMlpH; j += 2) {
        float2 z = *reinterpret_cast<const float2*>(P + kOffB2 + j);
#pragma unroll
        for (int i = 0; i < kMlpH; ++i)
            z = __ffma2_rn(make_float2(h1[i], h1[i]), *reinterpret_cast<const float2*>(P + kOffW2 + i * kMlpH + j), z);
        z3 += mlp_silu(z.x) * P[kOffW3 + j];
        z3 += mlp_silu(z.y) * P[kOffW3 + j + 1];
    }
    return mlp_softplus(z3);
}
#endif

}  // namespace lbm

namespace lbm {

// The 7 inputs of the closure from the resolved strain rate
// S = {xx, yy, zz, xy, yz, zx} (reference axes: x is the wall normal) and the
// distance to the nearest wall; invariant under rotations about the wall
// normal and reflections:
//   x0 = log(1 + |S| nu / u*^2)        strain magnitude in wall units, |S| = sqrt(2 S:S)
//   x1 = tr S / |S|                     dilatation ratio
//   x2 = sqrt(6) det(D) / (D:D)^(3/2)   strain state of the deviator D
//   x3 = D_xx / |D|                     normal strain along the wall normal
//   x4 = sqrt(D_xy^2 + D_xz^2) / |D|    shear between the normal and the wall plane
//   x5 = log(1 + d u* / nu)             wall distance in wall units
//   x6 = d / h                          wall distance in outer units
__host__ __device__ inline void closure_features(const float S[6], float dwall, float nu, float ustar, float h,
                                                 float x[kMlpIn]) {
    const float tr = S[0] + S[1] + S[2];
    const float off = S[3] * S[3] + S[4] * S[4] + S[5] * S[5];
    const float ss = S[0] * S[0] + S[1] * S[1] + S[2] * S[2] + 2.f * off;
    const float smag = sqrtf(2.f * ss);
    const float t3 = tr * (1.f / 3.f);
    const float d0 = S[0] - t3, d1 = S[1] - t3, d2 = S[2] - t3;
    const float i2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.f * off;
    const float det = d0 * (d1 * d2 - S[4] * S[4]) - S[3] * (S[3] * d2 - S[4] * S[5]) + S[5] * (S[3] * S[4] - d1 * S[5]);
    const float rn = sqrtf(i2) + 1e-30f;
    x[0] = log1pf(smag * nu / (ustar * ustar));
    x[1] = tr / (smag + 1e-30f);
    x[2] = 2.4494897f * det / (rn * rn * rn);
    x[3] = d0 / rn;
    x[4] = sqrtf(S[3] * S[3] + S[5] * S[5]) / rn;
    x[5] = log1pf(dwall * ustar / nu);
    x[6] = dwall / h;
}

}  // namespace lbm
