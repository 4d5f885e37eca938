// Two FP32 lanes in one value for the row kernels' collision.
//
// sm_100-class GPUs have packed FP32 instructions (add/mul/fma.rn.f32x2) that
// apply one operation to two FP32 values.  Each thread of the row kernels
// relaxes two adjacent nodes with identical arithmetic, so the collision of
// the pair is written once over F2 = (node x, node x+1) and issues half the
// floating-point instructions.  Products stay unrounded (P2) until an add or a
// subtract consumes them as one fused multiply-add, the contraction the
// compiler applies to scalar a*b+c; a product used on its own is rounded by
// a packed multiply.  Every operation is round-to-nearest, per lane, as the
// scalar instructions are.
#pragma once

#include <cuda_runtime.h>

namespace lbm {

struct F2 {
    float2 v;
    F2() = default;
    __host__ __device__ __forceinline__ F2(float s) : v(make_float2(s, s)) {}
    __host__ __device__ __forceinline__ F2(float a, float b) : v(make_float2(a, b)) {}
    __host__ __device__ __forceinline__ explicit F2(float2 x) : v(x) {}
    __device__ __forceinline__ F2& operator+=(const F2& o);
};

// x * y, not yet rounded
struct P2 {
    float2 a, b;
    __device__ __forceinline__ operator F2() const { return F2(__fmul2_rn(a, b)); }
};

__device__ __forceinline__ float2 neg2(float2 x) { return make_float2(-x.x, -x.y); }

__device__ __forceinline__ F2 operator+(F2 x, F2 y) { return F2(__fadd2_rn(x.v, y.v)); }
__device__ __forceinline__ F2 operator-(F2 x, F2 y) { return F2(__fadd2_rn(x.v, neg2(y.v))); }
__device__ __forceinline__ F2 operator-(F2 x) { return F2(neg2(x.v)); }
__device__ __forceinline__ F2& F2::operator+=(const F2& o) { v = __fadd2_rn(v, o.v); return *this; }

__device__ __forceinline__ P2 operator*(F2 x, F2 y) { return P2{x.v, y.v}; }
__device__ __forceinline__ P2 operator*(P2 p, F2 y) { return P2{__fmul2_rn(p.a, p.b), y.v}; }
__device__ __forceinline__ P2 operator*(F2 x, P2 p) { return P2{x.v, __fmul2_rn(p.a, p.b)}; }
__device__ __forceinline__ P2 operator-(P2 p) { return P2{neg2(p.a), p.b}; }

__device__ __forceinline__ F2 operator+(P2 p, F2 c) { return F2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ F2 operator+(F2 c, P2 p) { return F2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ F2 operator-(P2 p, F2 c) { return F2(__ffma2_rn(p.a, p.b, neg2(c.v))); }
__device__ __forceinline__ F2 operator-(F2 c, P2 p) { return F2(__ffma2_rn(neg2(p.a), p.b, c.v)); }
__device__ __forceinline__ F2 operator+(P2 p, P2 q) { return F2(__ffma2_rn(p.a, p.b, __fmul2_rn(q.a, q.b))); }
__device__ __forceinline__ F2 operator-(P2 p, P2 q) {
    return F2(__ffma2_rn(p.a, p.b, neg2(__fmul2_rn(q.a, q.b))));
}

}  // namespace lbm
