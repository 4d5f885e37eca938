// Fused collide + stream kernels: the AA in-place pattern.
//
// The reference streams in place with the sequential "swap" algorithm
// (Channel-Flow/collision.f90:222-264, ipstay/ipswap para.f90:209-210): each
// node stores its post-collision value f*_i into its own opposite slot
// (ipopp(i)) and then swaps the slots it shares with the already-visited
// neighbours.  That sweep is ordered and cannot run in parallel.  The GPU
// uses the AA pattern, which keeps one array and gives the same post-stream
// populations:
//   even step (state natural):  read slot i at x, collide, write f*_i to slot
//                               opp(i) at x -- exactly the reference's "stay"
//                               store, all accesses local;
//   odd step  (state swapped):  read f_i(x) from slot opp(i) at x - c_i, collide,
//                               write f*_i to slot i at x + c_i; after it the
//                               array is in natural orientation again.
// Every location is read and then written by one thread only, so no step needs
// a second array or a grid-wide barrier.  Half-way bounce-back at the walls
// (the imove<1 / imove>lx branches, collision.f90:229-230, 250-251) falls out of
// the same slots: a population that would come from beyond a wall is read from
// the node's own slot i, one that would leave through a wall is written to the
// node's own slot opp(i).  The periodic y/z exchange (collisionExchnge,
// collision.f90:281-372) becomes index wrap-around.
#include "lbm_internal.h"
#include "lbm_mlp.cuh"
#include "lbm_strain.cuh"

namespace lbm {

namespace {

constexpr int kBlockX = 256;

struct NodeIdx {
    uint32_t xs[3];     // X - 1, X, X + 1 (periodic)
    uint32_t yr[3];     // NX * (Y - 1, Y, Y + 1) (periodic)
    uint32_t zp[3];     // NXY * (Z - 1, Z, Z + 1) (only used inside the walls)
    __device__ __forceinline__ uint32_t at(int dx, int dy, int dz) const {
        return xs[dx + 1] + yr[dy + 1] + zp[dz + 1];
    }
};

__device__ __forceinline__ NodeIdx make_idx(const Geometry& g, int x, int y, int z) {
    NodeIdx I;
    I.xs[0] = (x == 0) ? g.NX - 1 : x - 1;
    I.xs[1] = x;
    I.xs[2] = (x == g.NX - 1) ? 0 : x + 1;
    const int ym = (y == 0) ? g.NY - 1 : y - 1;
    const int yp = (y == g.NY - 1) ? 0 : y + 1;
    I.yr[0] = (uint32_t)ym * g.NX;
    I.yr[1] = (uint32_t)y * g.NX;
    I.yr[2] = (uint32_t)yp * g.NX;
    I.zp[0] = (uint32_t)(z - 1) * g.NXY;
    I.zp[1] = (uint32_t)z * g.NXY;
    I.zp[2] = (uint32_t)(z + 1) * g.NXY;
    return I;
}

// WALL bit 0: this plane touches the lower wall (Z == 0, ref x = 1)
// WALL bit 1: this plane touches the upper wall (Z == NZ-1, ref x = nx)
template <int WALL>
__device__ __forceinline__ bool pull_bounces(int i) {
    return (DZg(i) == 1 && (WALL & 1)) || (DZg(i) == -1 && (WALL & 2));
}
template <int WALL>
__device__ __forceinline__ bool push_bounces(int i) {
    return (DZg(i) == 1 && (WALL & 2)) || (DZg(i) == -1 && (WALL & 1));
}

template <typename T, typename R, int WALL, bool FROZEN, bool YF = false>
__device__ __forceinline__ void odd_node(const PopPtrs<T>& P, const CollideConsts<R>& C,
                                         const NodeIdx& I, uint32_t n,
                                         R ufx, R ufy, R ufz, R& rho, R& jx, R& jy, R& jz)
{
    R f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (pull_bounces<WALL>(i)) f[i] = ld_pop(P.p[i] + n);
        else f[i] = ld_pop(P.p[OPPf(i)] + I.at(-DXg(i), -DYg(i), -DZg(i)));
    }
    collide<R, FROZEN, YF>(f, C, ufx, ufy, ufz, rho, jx, jy, jz);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (push_bounces<WALL>(i)) st_pop(P.p[OPPf(i)] + n, f[i]);
        else st_pop(P.p[i] + I.at(DXg(i), DYg(i), DZg(i)), f[i]);
    }
}

template <typename T, typename R, bool YF>
__global__ void __launch_bounds__(kBlockX)
k_step_even(PopPtrs<T> P, CollideConsts<R> C, Geometry g)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= g.NX) return;
    const uint32_t n = x + g.NX * (blockIdx.y + g.NY * blockIdx.z);
    R f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = ld_pop(P.p[i] + n);
    R rho, jx, jy, jz;
    collide<R, false, YF>(f, C, R(0), R(0), R(0), rho, jx, jy, jz);
#pragma unroll
    for (int i = 0; i < Q; ++i) st_pop(P.p[OPPf(i)] + n, f[i]);
}

template <typename T, typename R, bool YF>
__global__ void __launch_bounds__(kBlockX)
k_step_odd(PopPtrs<T> P, CollideConsts<R> C, Geometry g)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= g.NX) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const NodeIdx I = make_idx(g, x, y, z);
    const uint32_t n = I.at(0, 0, 0);
    R rho, jx, jy, jz;
    const int wall = (z == 0 ? 1 : 0) | (z == g.NZ - 1 ? 2 : 0);
    if (wall == 0)      odd_node<T, R, 0, false, YF>(P, C, I, n, R(0), R(0), R(0), rho, jx, jy, jz);
    else if (wall == 1) odd_node<T, R, 1, false, YF>(P, C, I, n, R(0), R(0), R(0), rho, jx, jy, jz);
    else if (wall == 2) odd_node<T, R, 2, false, YF>(P, C, I, n, R(0), R(0), R(0), rho, jx, jy, jz);
    else                odd_node<T, R, 3, false, YF>(P, C, I, n, R(0), R(0), R(0), rho, jx, jy, jz);
}

// ---------------------------------------------------------------------------
// Coarse-grid LES with the learned closure fused into the collision.  Per
// node: the strain rate from the non-equilibrium moments (Yu et al. 2006,
// with the shear rate of the node's previous collision, which produced that
// non-equilibrium part), the closure's seven features, the network with its
// weights in shared memory, and the shear moments relaxed at
// s9 = s13 = 1 / (3 (nu + nu_t) + 1/2).  Storage with S = 1 (FP32/FP64).
template <typename R, bool YF>
__device__ __forceinline__ void les_collide(R f[Q], const CollideConsts<R>& C, const DeviceState& s,
                                            const float* Ws, uint32_t n, int z) {
    R rho = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        rho += f[i];
        if (CXf(i)) jx += R(CXf(i)) * f[i];
        if (CYf(i)) jy += R(CYf(i)) * f[i];
        if (CZf(i)) jz += R(CZf(i)) * f[i];
    }
    jx += C.hFx; jy += C.hFy; jz += C.hFz;
    R S6[6];
    strain_from_moments<R>(f, rho, jx, jy, jz, C.ke * R(2394), (R)s.les_s9[n], S6);
    float Sf[6], x[kMlpIn];
#pragma unroll
    for (int k = 0; k < 6; ++k) Sf[k] = (float)S6[k];
    const float dwall = fminf((float)z + 0.5f, (float)s.g.NZ - (float)z - 0.5f);
    closure_features(Sf, dwall, (float)s.les_nu, s.les_ustar, s.les_h, x);
    float r = mlp_infer_pairs(Ws, Ws + kMlpParams, x);
    if (s.les_aplus > 0.f) {
        // van Driest damping (1 - exp(-y+/A+))^2 of the predicted nu_t
        const float e = 1.f - expf(-(dwall * s.les_ustar / (float)s.les_nu) / s.les_aplus);
        r *= e * e;
    }
    const R s9 = R(1) / (R(3) * (R)s.les_nu * (R(1) + (R)r) + R(0.5));
    s.les_s9[n] = (float)s9;
    CollideConsts<R> cl = C;
    cl.kp = s9 * R(1.0 / 36.0);
    cl.kw = s9 * R(1.0 / 12.0);
    cl.kxy = s9 * R(0.25);
    R a, b, c, d;
    collide<R, false, YF>(f, cl, R(0), R(0), R(0), a, b, c, d);
}

template <typename T, typename R, bool YF>
__global__ void __launch_bounds__(kBlockX) k_les_even(PopPtrs<T> P, CollideConsts<R> C, DeviceState s) {
    __shared__ __align__(16) float Ws[kMlpParams + kMlpNorm];
    for (int e = threadIdx.x; e < kMlpParams + kMlpNorm; e += blockDim.x) Ws[e] = s.les_w[e];
    __syncthreads();
    const Geometry& g = s.g;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= g.NX) return;
    const uint32_t n = x + g.NX * (blockIdx.y + g.NY * blockIdx.z);
    R f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = ld_pop(P.p[i] + n);
    les_collide<R, YF>(f, C, s, Ws, n, blockIdx.z);
#pragma unroll
    for (int i = 0; i < Q; ++i) st_pop(P.p[OPPf(i)] + n, f[i]);
}

template <typename T, typename R, int WALL, bool YF>
__device__ __forceinline__ void les_odd_node(const PopPtrs<T>& P, const CollideConsts<R>& C, const DeviceState& s,
                                             const float* Ws, const NodeIdx& I, uint32_t n, int z) {
    R f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (pull_bounces<WALL>(i)) f[i] = ld_pop(P.p[i] + n);
        else f[i] = ld_pop(P.p[OPPf(i)] + I.at(-DXg(i), -DYg(i), -DZg(i)));
    }
    les_collide<R, YF>(f, C, s, Ws, n, z);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (push_bounces<WALL>(i)) st_pop(P.p[OPPf(i)] + n, f[i]);
        else st_pop(P.p[i] + I.at(DXg(i), DYg(i), DZg(i)), f[i]);
    }
}

template <typename T, typename R, bool YF>
__global__ void __launch_bounds__(kBlockX) k_les_odd(PopPtrs<T> P, CollideConsts<R> C, DeviceState s) {
    __shared__ __align__(16) float Ws[kMlpParams + kMlpNorm];
    for (int e = threadIdx.x; e < kMlpParams + kMlpNorm; e += blockDim.x) Ws[e] = s.les_w[e];
    __syncthreads();
    const Geometry& g = s.g;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= g.NX) return;
    const int y = blockIdx.y, z = blockIdx.z;
    const NodeIdx I = make_idx(g, x, y, z);
    const uint32_t n = I.at(0, 0, 0);
    const int wall = (z == 0 ? 1 : 0) | (z == g.NZ - 1 ? 2 : 0);
    if (wall == 0)      les_odd_node<T, R, 0, YF>(P, C, s, Ws, I, n, z);
    else if (wall == 1) les_odd_node<T, R, 1, YF>(P, C, s, Ws, I, n, z);
    else if (wall == 2) les_odd_node<T, R, 2, YF>(P, C, s, Ws, I, n, z);
    else                les_odd_node<T, R, 3, YF>(P, C, s, Ws, I, n, z);
}

// Pre-relaxation step (main.f90:69-90): velocity frozen at uf (GPU layout,
// three planes of N doubles), rho = sum f.  rho holds the previous iteration's
// density on entry and this iteration's on exit; maxabs receives
// max |rho - rho_prev| as the bit pattern of a non-negative double.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

template <typename T, typename R>
__global__ void __launch_bounds__(kBlockX)
k_prerelax(PopPtrs<T> P, CollideConsts<R> C, Geometry g, int parity,
           const double* __restrict__ uf, size_t N, double* __restrict__ rho_arr,
           unsigned long long* maxabs)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 0.0;
    if (x < g.NX) {
        const int y = blockIdx.y, z = blockIdx.z;
        const NodeIdx I = make_idx(g, x, y, z);
        const uint32_t n = I.at(0, 0, 0);
        const R ufx = (R)uf[n], ufy = (R)uf[N + n], ufz = (R)uf[2 * N + n];
        R rho, jx, jy, jz;
        if (parity == 0) {
            R f[Q];
#pragma unroll
            for (int i = 0; i < Q; ++i) f[i] = ld_pop(P.p[i] + n);
            collide<R, true>(f, C, ufx, ufy, ufz, rho, jx, jy, jz);
#pragma unroll
            for (int i = 0; i < Q; ++i) st_pop(P.p[OPPf(i)] + n, f[i]);
        } else {
            const int wall = (z == 0 ? 1 : 0) | (z == g.NZ - 1 ? 2 : 0);
            if (wall == 0)      odd_node<T, R, 0, true>(P, C, I, n, ufx, ufy, ufz, rho, jx, jy, jz);
            else if (wall == 1) odd_node<T, R, 1, true>(P, C, I, n, ufx, ufy, ufz, rho, jx, jy, jz);
            else if (wall == 2) odd_node<T, R, 2, true>(P, C, I, n, ufx, ufy, ufz, rho, jx, jy, jz);
            else                odd_node<T, R, 3, true>(P, C, I, n, ufx, ufy, ufz, rho, jx, jy, jz);
        }
        const double r = (double)rho * (double)C.invS;
        local = fabs(r - rho_arr[n]);
        rho_arr[n] = r;
    }
    // warp max then one atomic per warp
    for (int o = 16; o > 0; o >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(maxabs, local);
}

template <typename T>
PopPtrs<T> pop_ptrs(const DeviceState& s) {
    PopPtrs<T> P;
    T* base = static_cast<T*>(s.f);
    for (int i = 0; i < Q; ++i) P.p[i] = base + (size_t)i * s.pstride;
    return P;
}

dim3 step_grid(const Geometry& g, int bx) {
    return dim3((g.NX + bx - 1) / bx, g.NY, g.NZ);
}
int block_x(const Geometry& g) {
    int bx = ((g.NX + 31) / 32) * 32;
    return bx > kBlockX ? kBlockX : bx;
}

template <int PREC>
cudaError_t step_impl(const DeviceState& s, int parity, cudaStream_t st) {
    using T = typename Prec<PREC>::T;
    using R = typename Prec<PREC>::R;
    const PopPtrs<T> P = pop_ptrs<T>(s);
    const int bx = block_x(s.g);
    const dim3 grid = step_grid(s.g, bx);
    const CollideConsts<R>* C;
    if constexpr (sizeof(R) == 8) C = &s.cd; else C = &s.cf;
    const bool yf = C->Fx == R(0) && C->Fz == R(0);
    if constexpr (PREC != LBM_PREC_FP16) {
        if (s.les_w) {
            if (yf) {
                if (parity == 0) k_les_even<T, R, true><<<grid, bx, 0, st>>>(P, *C, s);
                else             k_les_odd<T, R, true><<<grid, bx, 0, st>>>(P, *C, s);
            } else {
                if (parity == 0) k_les_even<T, R, false><<<grid, bx, 0, st>>>(P, *C, s);
                else             k_les_odd<T, R, false><<<grid, bx, 0, st>>>(P, *C, s);
            }
            return cudaGetLastError();
        }
    }
    if (yf) {
        if (parity == 0) k_step_even<T, R, true><<<grid, bx, 0, st>>>(P, *C, s.g);
        else             k_step_odd<T, R, true><<<grid, bx, 0, st>>>(P, *C, s.g);
    } else {
        if (parity == 0) k_step_even<T, R, false><<<grid, bx, 0, st>>>(P, *C, s.g);
        else             k_step_odd<T, R, false><<<grid, bx, 0, st>>>(P, *C, s.g);
    }
    return cudaGetLastError();
}

template <int PREC>
cudaError_t prerelax_impl(const DeviceState& s, int parity, const double* uf,
                          double* rho, unsigned long long* maxabs, cudaStream_t st) {
    using T = typename Prec<PREC>::T;
    using R = typename Prec<PREC>::R;
    const PopPtrs<T> P = pop_ptrs<T>(s);
    const int bx = block_x(s.g);
    const dim3 grid = step_grid(s.g, bx);
    const CollideConsts<R>* C;
    if constexpr (sizeof(R) == 8) C = &s.cd; else C = &s.cf;
    k_prerelax<T, R><<<grid, bx, 0, st>>>(P, *C, s.g, parity, uf, s.N, rho, maxabs);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step(const DeviceState& s, int parity, cudaStream_t st) {
    switch (s.prec) {
        case LBM_PREC_FP64: return step_impl<LBM_PREC_FP64>(s, parity, st);
        case LBM_PREC_FP32: return step_impl<LBM_PREC_FP32>(s, parity, st);
        case LBM_PREC_FP16: return step_impl<LBM_PREC_FP16>(s, parity, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_prerelax(const DeviceState& s, int parity, const double* uf,
                            double* rho, unsigned long long* maxabs, cudaStream_t st) {
    switch (s.prec) {
        case LBM_PREC_FP64: return prerelax_impl<LBM_PREC_FP64>(s, parity, uf, rho, maxabs, st);
        case LBM_PREC_FP32: return prerelax_impl<LBM_PREC_FP32>(s, parity, uf, rho, maxabs, st);
        case LBM_PREC_FP16: return prerelax_impl<LBM_PREC_FP16>(s, parity, uf, rho, maxabs, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lbm
