// Non-hot kernels: layout conversion between the reference's AoS FP64 array
// f(0:18,nx,ny,nz) and the device SoA storage, equilibrium initialisation,
// macroscopic fields and FP64 reductions for the diagnostics.
#include <algorithm>
#include <cmath>

#include "lbm_internal.h"
#include "lbm_strain.cuh"
#include "lbm_mlp.cuh"

namespace lbm {

// Channel initial velocity: Poiseuille profile along ref y (the steady laminar
// solution of saveload.f90:924-926 with ustar -> uc) plus uniform noise of
// +-amp*uc per component from the counter-based generator; the host copy
// channel_velocity_host gives identical bits.
__host__ __device__ inline void channel_velocity_node(int nx, int ny, int ix, int iy, int iz,
                                                      double uc, double amp, uint64_t seed,
                                                      double& u, double& v, double& w) {
    // ix, iy, iz are 0-based reference indices; the profile is the steady
    // laminar solution 4 uc ((nx/2)^2 - xx0^2) / nx^2, xx0 = |ix+1-0.5-nx/2|
    const double half = 0.5 * (double)nx;
    double xx0 = (double)ix + 0.5 - half;
    xx0 = xx0 < 0 ? -xx0 : xx0;
#ifdef __CUDA_ARCH__
    const double prof = __ddiv_rn(__dmul_rn(4.0 * uc, __dsub_rn(__dmul_rn(half, half), __dmul_rn(xx0, xx0))),
                                  __dmul_rn((double)nx, (double)nx));
#else
    const double prof = (4.0 * uc) * (half * half - xx0 * xx0) / ((double)nx * (double)nx);
#endif
    const uint64_t lin = (uint64_t)ix + (uint64_t)nx * ((uint64_t)iy + (uint64_t)ny * (uint64_t)iz);
    const double a = amp * uc;
#ifdef __CUDA_ARCH__
    u = __dmul_rn(a, uniform_pm1(seed, 3 * lin + 0));
    v = __dadd_rn(prof, __dmul_rn(a, uniform_pm1(seed, 3 * lin + 1)));
    w = __dmul_rn(a, uniform_pm1(seed, 3 * lin + 2));
#else
    u = a * uniform_pm1(seed, 3 * lin + 0);
    v = prof + a * uniform_pm1(seed, 3 * lin + 1);
    w = a * uniform_pm1(seed, 3 * lin + 2);
#endif
}

namespace {

template <typename T>
__device__ __forceinline__ T* pop_plane(const DeviceState& s, int i) {
    return static_cast<T*>(s.f) + (size_t)i * s.pstride;
}

// Natural (post-stream) populations of GPU node (x,y,z), true units, FP64.
// parity 0: slot i at n.  parity 1 (after an even AA step): f_i(x) sits in
// slot opp(i) at x - c_i, or in slot i at x when x - c_i is beyond a wall.
template <typename T>
__device__ void gather_natural(const DeviceState& s, int parity, int x, int y, int z,
                               double f[Q]) {
    const Geometry& g = s.g;
    const double invS = s.cd.invS;
    const uint32_t n = x + g.NX * (y + g.NY * (uint32_t)z);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        uint32_t m = n;
        int slot = i;
        if (parity) {
            const int zs = z - DZg(i);
            if (zs >= 0 && zs < g.NZ) {
                int xs = x - DXg(i); xs = xs < 0 ? xs + g.NX : (xs >= g.NX ? xs - g.NX : xs);
                int ys = y - DYg(i); ys = ys < 0 ? ys + g.NY : (ys >= g.NY ? ys - g.NY : ys);
                m = xs + g.NX * (ys + g.NY * (uint32_t)zs);
                slot = OPPf(i);
            }
        }
        f[i] = (double)ld_pop(pop_plane<T>(s, slot) + m) * invS;
    }
}

// Same, in the arithmetic type R of the diagnostics (FP32 for FP32/FP16
// storage, FP64 for FP64 storage).
template <typename T, typename R>
__device__ void gather_natural_r(const DeviceState& s, int parity, int x, int y, int z, R f[Q]) {
    const Geometry& g = s.g;
    const R invS = (R)s.cd.invS;
    const uint32_t n = x + g.NX * (y + g.NY * (uint32_t)z);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        uint32_t m = n;
        int slot = i;
        if (parity) {
            const int zs = z - DZg(i);
            if (zs >= 0 && zs < g.NZ) {
                int xs = x - DXg(i); xs = xs < 0 ? xs + g.NX : (xs >= g.NX ? xs - g.NX : xs);
                int ys = y - DYg(i); ys = ys < 0 ? ys + g.NY : (ys >= g.NY ? ys - g.NY : ys);
                m = xs + g.NX * (ys + g.NY * (uint32_t)zs);
                slot = OPPf(i);
            }
        }
        f[i] = (R)ld_pop(pop_plane<T>(s, slot) + m) * invS;
    }
}
template <typename T> struct DiagR { using type = float; };
template <> struct DiagR<double> { using type = double; };

template <typename T>
__device__ __forceinline__ void put(const DeviceState& s, int i, uint32_t n, double v_true) {
    const double S = s.cd.S;
    if constexpr (sizeof(T) == 8) pop_plane<T>(s, i)[n] = v_true * S;
    else st_pop(pop_plane<T>(s, i) + n, (float)(v_true * S));
}

// Thread mapping for reference-layout chunks: threadIdx.x/blockIdx.x -> ref y
// (GPU X, contiguous in the SoA planes), blockIdx.y -> ref x, blockIdx.z -> ref
// z inside the chunk.
struct RefNode { int ix, iy, iz; bool ok; };
__device__ __forceinline__ RefNode ref_node(const Geometry& g, int z0) {
    RefNode r;
    r.iy = blockIdx.x * blockDim.x + threadIdx.x;
    r.ix = blockIdx.y;
    r.iz = z0 + blockIdx.z;
    r.ok = r.iy < g.NX;
    return r;
}
// 0-based reference-layout linear node index (x fastest)
__device__ __forceinline__ size_t ref_lin(const Geometry& g, int ix, int iy, int iz) {
    return (size_t)ix + (size_t)g.NZ * ((size_t)iy + (size_t)g.NX * iz);
}
__device__ __forceinline__ uint32_t gpu_lin(const Geometry& g, int ix, int iy, int iz) {
    return (uint32_t)iy + g.NX * ((uint32_t)iz + g.NY * (uint32_t)ix);
}

template <typename T>
__global__ void k_aos_to_store(DeviceState s, const double* __restrict__ aos, int z0) {
    const RefNode r = ref_node(s.g, z0);
    if (!r.ok) return;
    const size_t src = 19 * ref_lin(s.g, r.ix, r.iy, r.iz - z0);
    const uint32_t n = gpu_lin(s.g, r.ix, r.iy, r.iz);
#pragma unroll
    for (int i = 0; i < Q; ++i) put<T>(s, i, n, aos[src + i]);
}

// Node flags of the particle checkpoint for ref z planes [z0, z0 + nzc), in
// reference layout: ibnodes = 1 solid / -1 fluid (saveload.f90:1359-1360),
// isnodes = 1-based id of the owning sphere / -1 (collision.f90:422).
__global__ void k_owner_to_ref(Geometry g, const int* __restrict__ owner, int32_t* __restrict__ ib,
                               int32_t* __restrict__ is, int z0) {
    RefNode r;
    r.iy = blockIdx.x * blockDim.x + threadIdx.x;
    r.ix = blockIdx.y;
    r.iz = z0 + blockIdx.z;
    if (r.iy >= g.NX) return;
    const int own = owner[gpu_lin(g, r.ix, r.iy, r.iz)];
    const size_t o = ref_lin(g, r.ix, r.iy, r.iz - z0);
    ib[o] = own >= 0 ? 1 : -1;
    is[o] = own >= 0 ? own + 1 : -1;
}

template <typename T>
__global__ void k_store_to_aos(DeviceState s, int parity, double* __restrict__ aos, int z0) {
    const RefNode r = ref_node(s.g, z0);
    if (!r.ok) return;
    double f[Q];
    gather_natural<T>(s, parity, r.iy, r.iz, r.ix, f);
    const size_t dst = 19 * ref_lin(s.g, r.ix, r.iy, r.iz - z0);
#pragma unroll
    for (int i = 0; i < Q; ++i) aos[dst + i] = f[i];
}

// initpop (initial.f90:19-46) at delta-rho = 0; explicit round-to-nearest
// operations (no FMA contraction) so that host code gets identical bits.
__device__ __forceinline__ void equilibrium_rn(double ux, double uy, double uz, double f[Q]) {
    const double usqr = __dmul_rn(1.5, __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)),
                                                 __dmul_rn(uz, uz)));
    f[0] = __dmul_rn(W0, __dsub_rn(0.0, usqr));
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const double G = __dadd_rn(__dadd_rn(__dmul_rn((double)CXf(i), ux), __dmul_rn((double)CYf(i), uy)),
                                   __dmul_rn((double)CZf(i), uz));
        const double t = __dsub_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(3.0, G)),
                                             __dmul_rn(__dmul_rn(4.5, G), G)), usqr);
        f[i] = __dmul_rn(weight(i), t);
    }
}

template <typename T>
__global__ void k_init_channel(DeviceState s, double uc, double amp, uint64_t seed) {
    const RefNode r = ref_node(s.g, 0);
    if (!r.ok) return;
    double u, v, w;
    channel_velocity_node(s.g.NZ, s.g.NX, r.ix, r.iy, r.iz, uc, amp, seed, u, v, w);
    double f[Q];
    equilibrium_rn(u, v, w, f);
    const uint32_t n = gpu_lin(s.g, r.ix, r.iy, r.iz);
#pragma unroll
    for (int i = 0; i < Q; ++i) put<T>(s, i, n, f[i]);
}

// Reference-layout fields <-> SoA nodes through shared-memory tiles.  The
// reference layout runs along x (wall-normal) fastest, the population planes
// along y (streamwise), so a kernel that walks either one strides through the
// other by nx*8 bytes per thread.  These kernels take a tile of 32 (x) x 32 (y)
// nodes at one z: the FP64 field side moves along x (coalesced 256-byte
// rows), the population side along y (coalesced plane rows), and the tile is
// turned around in shared memory.  FP64 storage computes in FP64 with the
// explicitly rounded operations of the oracle (same bits); FP32/FP16 storage
// computes in FP32, which is exact to well below its storage precision.
constexpr int kTile = 32, kTileRows = 8;

__device__ __forceinline__ void equilibrium_f(float ux, float uy, float uz, float f[Q]) {
    const float usqr = 1.5f * (ux * ux + uy * uy + uz * uz);
    f[0] = (float)W0 * (-usqr);
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const float G = (float)CXf(i) * ux + (float)CYf(i) * uy + (float)CZf(i) * uz;
        f[i] = (float)weight(i) * (3.f * G + 4.5f * G * G - usqr);
    }
}

template <typename T, typename R>
__global__ void __launch_bounds__(kTile * kTileRows)
k_initpop_t(DeviceState s, const double* __restrict__ ux, const double* __restrict__ uy,
            const double* __restrict__ uz, int z0) {
    __shared__ double U[3][kTile][kTile + 1];              // [y][x]
    const int nx = s.g.NZ, ny = s.g.NX;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int ix0 = blockIdx.y * kTile, iy0 = blockIdx.x * kTile, iz = z0 + blockIdx.z;
    const size_t base = (size_t)nx * ny * blockIdx.z;      // chunk-relative z plane
    for (int r = ty; r < kTile; r += kTileRows) {
        const int iy = iy0 + r, ix = ix0 + tx;
        if (iy < ny && ix < nx) {
            const size_t o = base + (size_t)ix + (size_t)nx * iy;
            U[0][r][tx] = ux[o];
            U[1][r][tx] = uy[o];
            U[2][r][tx] = uz[o];
        }
    }
    __syncthreads();
    for (int r = ty; r < kTile; r += kTileRows) {
        const int ix = ix0 + r, iy = iy0 + tx;
        if (ix >= nx || iy >= ny) continue;
        const uint32_t n = gpu_lin(s.g, ix, iy, iz);
        if constexpr (sizeof(R) == 8) {
            double f[Q];
            equilibrium_rn(U[0][tx][r], U[1][tx][r], U[2][tx][r], f);
#pragma unroll
            for (int i = 0; i < Q; ++i) put<T>(s, i, n, f[i]);
        } else {
            float f[Q];
            equilibrium_f((float)U[0][tx][r], (float)U[1][tx][r], (float)U[2][tx][r], f);
            const float S = s.cf.S;
#pragma unroll
            for (int i = 0; i < Q; ++i) st_pop(pop_plane<T>(s, i) + n, f[i] * S);
        }
    }
}

// Log-law initial velocity (initvel's turbulent branch, initial.f90:101-147)
// from tables the host computes with its libm (loglaw_tables_host): per
// wall plane m of the lower half the mean profile P[m] and the perturbation
// factors Ay[m], Ax[m]; per streamwise/spanwise column sin and cos of the
// perturbation's phase.  The device only multiplies and adds them in the
// reference's order, so it builds the same bits as the host restatement.
// Planes i = m + 1 and nx - m (1-based) share row m; with odd nx the middle
// plane keeps zero velocity, as initvel leaves it.
template <typename T>
__global__ void k_init_loglaw(DeviceState s, const double* __restrict__ tab, int nxh) {
    const RefNode r = ref_node(s.g, 0);
    if (!r.ok) return;
    const int nx = s.g.NZ;
    int m = -1;
    if (r.ix < nxh) m = r.ix;
    else if (nx - 1 - r.ix < nxh) m = nx - 1 - r.ix;
    double u = 0.0, v = 0.0;
    if (m >= 0) {
        const double* P = tab;
        const double* Ay = tab + nxh;
        const double* Ax = tab + 2 * (size_t)nxh;
        const double* Sn = tab + 3 * (size_t)nxh;
        const double* Cs = Sn + (size_t)s.g.NX * s.g.NY;
        const size_t col = (size_t)r.iy + (size_t)s.g.NX * r.iz;
        v = __dadd_rn(P[m], __dmul_rn(Ay[m], Sn[col]));
        u = __dadd_rn(0.0, __dmul_rn(Ax[m], Cs[col]));
    }
    double f[Q];
    equilibrium_rn(u, v, 0.0, f);
    const uint32_t n = gpu_lin(s.g, r.ix, r.iy, r.iz);
#pragma unroll
    for (int i = 0; i < Q; ++i) put<T>(s, i, n, f[i]);
}

// macrovar (collision.f90:394-418) for fluid nodes
template <typename R>
__device__ __forceinline__ void macro_of(const R f[Q], const R F[3], R& rho, R& ux, R& uy, R& uz) {
    R r = 0, a = 0, b = 0, c = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        r += f[i];
        if (CXf(i)) a += CXf(i) * f[i];
        if (CYf(i)) b += CYf(i) * f[i];
        if (CZf(i)) c += CZf(i) * f[i];
    }
    rho = r; ux = a + R(0.5) * F[0]; uy = b + R(0.5) * F[1]; uz = c + R(0.5) * F[2];
}

// macrovar through a shared-memory tile (see k_initpop_t): populations read
// along y, the four FP64 fields written along x.
template <typename T, typename R>
__global__ void __launch_bounds__(kTile * kTileRows)
k_macro_t(DeviceState s, int parity, double* rho, double* ux, double* uy, double* uz, int z0) {
    __shared__ double M[4][kTile][kTile + 1];              // [x][y]
    const int nx = s.g.NZ, ny = s.g.NX;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int ix0 = blockIdx.y * kTile, iy0 = blockIdx.x * kTile, iz = z0 + blockIdx.z;
    for (int r = ty; r < kTile; r += kTileRows) {
        const int ix = ix0 + r, iy = iy0 + tx;
        if (ix >= nx || iy >= ny) continue;
        double d, a, b, c;
        if constexpr (sizeof(R) == 8) {
            double f[Q];
            gather_natural<T>(s, parity, iy, iz, ix, f);
            const double F[3] = {(double)s.cd.Fx, (double)s.cd.Fy, (double)s.cd.Fz};
            macro_of<double>(f, F, d, a, b, c);
        } else {
            float f[Q];
            gather_natural_r<T, float>(s, parity, iy, iz, ix, f);
            const float F[3] = {s.cf.Fx, s.cf.Fy, s.cf.Fz};
            float fd, fa, fb, fc;
            macro_of<float>(f, F, fd, fa, fb, fc);
            d = fd; a = fa; b = fb; c = fc;
        }
        const int own = s.owner ? s.owner[gpu_lin(s.g, ix, iy, iz)] : -1;
        if (own >= 0) {
            // solid node: rigid-body velocity and rho = rhopart (collision.f90:420-458)
            const double* X = s.ppos + 3 * own;
            const double* U = s.pvel + 3 * own;
            const double* W = s.pomg + 3 * own;
            auto mi = [](double v, double L) { return v >= 0.5 * L ? v - L : (v < -0.5 * L ? v + L : v); };
            const double x0 = (ix + 0.5) - X[0];
            const double y0 = mi((iy + 0.5) - X[1], (double)s.g.NX);
            const double z0c = mi((iz + 0.5) - X[2], (double)s.g.NY);
            a = U[0] + (W[1] * z0c - W[2] * y0);
            b = U[1] + (W[2] * x0 - W[0] * z0c);
            c = U[2] + (W[0] * y0 - W[1] * x0);
            d = s.prho;
        }
        M[0][r][tx] = d;
        M[1][r][tx] = a;
        M[2][r][tx] = b;
        M[3][r][tx] = c;
    }
    __syncthreads();
    const size_t base = (size_t)nx * ny * blockIdx.z;
    for (int r = ty; r < kTile; r += kTileRows) {
        const int iy = iy0 + r, ix = ix0 + tx;
        if (iy >= ny || ix >= nx) continue;
        const size_t o = base + (size_t)ix + (size_t)nx * iy;
        if (rho) rho[o] = M[0][tx][r];
        if (ux) ux[o] = M[1][tx][r];
        if (uy) uy[o] = M[2][tx][r];
        if (uz) uz[o] = M[3][tx][r];
    }
}

// Strain rate from the non-equilibrium part of the populations, the two ways
// of sijstat01 (saveload.f90:2320-2432), FP64 per node, natural orientation,
// reference axes (x wall-normal):
//  method 1 (moment space, Yu et al. 2006, Appendix; saveload.f90:2322-2380):
//    the non-equilibrium parts of e, 3p_xx, p_ww, p_xy, p_yz, p_xz scaled by
//    the rates that relax them (s1, s9) give S_ij directly;
//  method 2 (population space, saveload.f90:2385-2432): S_ab =
//    (3 / 2 tau) sum_i c_ia c_ib (f_i - f_i^eq) with the incompressible
//    equilibrium of initial.f90:26-44.
// Outputs S_ij S_ij of both; solid nodes give 0 (the reference masks them).
// S_ij S_ij by both methods and the wall-normal/streamwise shear S_xy of both
// at fluid GPU node (x, y, z), FP64 (dissipation_calc, saveload.f90:4683-4778).
struct NodeStrain { double m1, m2, sxy1, sxy2; };
template <typename T>
__device__ NodeStrain node_strain(const DeviceState& s, int parity, int x, int y, int z) {
    double f[Q];
    gather_natural<T>(s, parity, x, y, z, f);
    const double F[3] = {(double)s.cd.Fx, (double)s.cd.Fy, (double)s.cd.Fz};
    double rho, ux, uy, uz;
    macro_of<double>(f, F, rho, ux, uy, uz);
    const double s1 = (double)s.cd.ke * 2394.0, s9 = (double)s.cd.kp * 36.0;
    NodeStrain r;
    double S6[6];
    strain_from_moments(f, rho, ux, uy, uz, s1, s9, S6);
    r.m1 = S6[0] * S6[0] + S6[1] * S6[1] + S6[2] * S6[2] + 2.0 * (S6[3] * S6[3] + S6[4] * S6[4] + S6[5] * S6[5]);
    r.sxy1 = S6[3];
    const double usq = 1.5 * (ux * ux + uy * uy + uz * uz);
    double a[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const double cu = CXf(i) * ux + CYf(i) * uy + CZf(i) * uz;
        const double fn = f[i] - weight(i) * (rho + 3.0 * cu + 4.5 * cu * cu - usq);
        a[0] += fn * (CXf(i) * CXf(i)); a[1] += fn * (CYf(i) * CYf(i)); a[2] += fn * (CZf(i) * CZf(i));
        a[3] += fn * (CXf(i) * CYf(i)); a[4] += fn * (CYf(i) * CZf(i)); a[5] += fn * (CZf(i) * CXf(i));
    }
    const double k = 1.5 * s9;                           // 1.5 / tau
    r.m2 = (a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + 2.0 * (a[3] * a[3] + a[4] * a[4] + a[5] * a[5])) * k * k;
    r.sxy2 = a[3] * k;
    return r;
}

template <typename T>
__global__ void k_strain(DeviceState s, int parity, double* __restrict__ m1, double* __restrict__ m2, int z0) {
    const RefNode r = ref_node(s.g, z0);
    if (!r.ok) return;
    const size_t o = ref_lin(s.g, r.ix, r.iy, r.iz - z0);
    const int own = s.owner ? s.owner[gpu_lin(s.g, r.ix, r.iy, r.iz)] : -1;
    if (own >= 0) {
        if (m1) m1[o] = 0.0;
        if (m2) m2[o] = 0.0;
        return;
    }
    const NodeStrain v = node_strain<T>(s, parity, r.iy, r.iz, r.ix);
    if (m1) m1[o] = v.m1;
    if (m2) m2[o] = v.m2;
}

// Training data of the closure, step 1: box filter of u and u_i u_j over
// factor^3 fine nodes into coarse cell (ixc, iyc, izc); out[9][nc] (u, v, w,
// uu, vv, ww, uv, vw, uw) in the coarse reference layout.
template <typename T>
__global__ void k_box_filter(DeviceState s, int parity, int factor, int nxc, int nyc, int nzc,
                             double* __restrict__ out) {
    const int ixc = blockIdx.x * blockDim.x + threadIdx.x;
    if (ixc >= nxc) return;
    const int iyc = blockIdx.y, izc = blockIdx.z;
    const double F[3] = {(double)s.cd.Fx, (double)s.cd.Fy, (double)s.cd.Fz};
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = 0; dz < factor; ++dz)
        for (int dy = 0; dy < factor; ++dy)
            for (int dx = 0; dx < factor; ++dx) {
                const int ix = ixc * factor + dx, iy = iyc * factor + dy, iz = izc * factor + dz;
                double f[Q];
                gather_natural<T>(s, parity, iy, iz, ix, f);
                double rho, u, v, w;
                macro_of<double>(f, F, rho, u, v, w);
                acc[0] += u; acc[1] += v; acc[2] += w;
                acc[3] += u * u; acc[4] += v * v; acc[5] += w * w;
                acc[6] += u * v; acc[7] += v * w; acc[8] += u * w;
            }
    const double inv = 1.0 / ((double)factor * factor * factor);
    const size_t nc = (size_t)nxc * nyc * nzc;
    const size_t o = (size_t)ixc + (size_t)nxc * ((size_t)iyc + (size_t)nyc * izc);
#pragma unroll
    for (int k = 0; k < 9; ++k) out[k * nc + o] = acc[k] * inv;
}

// Training data, step 2: on the coarse grid the strain of the filtered
// velocity (central differences; periodic in y and z, the no-slip image
// u = -u(first cell) across the walls), the closure features and the target
// nu_t* / nu_c = max(0, -tau^d : S / (2 S : S)) / nu_c with the subgrid stress
// tau = filtered(u u) - filtered(u) filtered(u) (least-squares eddy viscosity).
__global__ void k_closure_targets(const double* __restrict__ F9, int nxc, int nyc, int nzc, float nu_c,
                                  float ustar, float h_c, float* __restrict__ X, float* __restrict__ y) {
    const int ixc = blockIdx.x * blockDim.x + threadIdx.x;
    if (ixc >= nxc) return;
    const int iyc = blockIdx.y, izc = blockIdx.z;
    const size_t nc = (size_t)nxc * nyc * nzc;
    auto at = [&](int k, int ix, int iy, int iz) -> double {
        // velocity component k at a coarse cell, with the wall image in x
        double sgn = 1.0;
        if (ix < 0) { ix = 0; sgn = -1.0; }
        if (ix >= nxc) { ix = nxc - 1; sgn = -1.0; }
        iy = (iy + nyc) % nyc;
        iz = (iz + nzc) % nzc;
        return sgn * F9[k * nc + (size_t)ix + (size_t)nxc * ((size_t)iy + (size_t)nyc * iz)];
    };
    double G[3][3];                                   // G[a][b] = d u_a / d x_b
    for (int a = 0; a < 3; ++a) {
        G[a][0] = 0.5 * (at(a, ixc + 1, iyc, izc) - at(a, ixc - 1, iyc, izc));
        G[a][1] = 0.5 * (at(a, ixc, iyc + 1, izc) - at(a, ixc, iyc - 1, izc));
        G[a][2] = 0.5 * (at(a, ixc, iyc, izc + 1) - at(a, ixc, iyc, izc - 1));
    }
    const double S[6] = {G[0][0], G[1][1], G[2][2], 0.5 * (G[0][1] + G[1][0]), 0.5 * (G[1][2] + G[2][1]),
                         0.5 * (G[0][2] + G[2][0])};
    const size_t o = (size_t)ixc + (size_t)nxc * ((size_t)iyc + (size_t)nyc * izc);
    const double u = F9[o], v = F9[nc + o], w = F9[2 * nc + o];
    double tau[6] = {F9[3 * nc + o] - u * u, F9[4 * nc + o] - v * v, F9[5 * nc + o] - w * w,
                     F9[6 * nc + o] - u * v, F9[7 * nc + o] - v * w, F9[8 * nc + o] - u * w};
    const double t3 = (tau[0] + tau[1] + tau[2]) / 3.0;
    tau[0] -= t3; tau[1] -= t3; tau[2] -= t3;
    const double num = -(tau[0] * S[0] + tau[1] * S[1] + tau[2] * S[2] + 2.0 * (tau[3] * S[3] + tau[4] * S[4] + tau[5] * S[5]));
    const double den = 2.0 * (S[0] * S[0] + S[1] * S[1] + S[2] * S[2] + 2.0 * (S[3] * S[3] + S[4] * S[4] + S[5] * S[5]));
    const double nut = den > 0.0 ? fmax(num / den, 0.0) : 0.0;
    float Sf[6], x[kMlpIn];
    for (int k = 0; k < 6; ++k) Sf[k] = (float)S[k];
    const float dwall = fminf((float)ixc + 0.5f, (float)nxc - (float)ixc - 0.5f);
    closure_features(Sf, dwall, nu_c, ustar, h_c, x);
    for (int k = 0; k < kMlpIn; ++k) X[o * kMlpIn + k] = x[k];
    y[o] = (float)(nut / nu_c);
}

// Features of the closure from the populations of this lattice: the strain
// from the non-equilibrium moments (with the per-node shear rate of the last
// closure collision, or the molecular s9), as the fused LES collision computes
// them; X[n][7] with n in the reference layout (ix fastest).
template <typename T>
__global__ void k_les_features(DeviceState s, int parity, float ustar, float h, float* __restrict__ X, int z0) {
    const RefNode r = ref_node(s.g, z0);
    if (!r.ok) return;
    double f[Q];
    gather_natural<T>(s, parity, r.iy, r.iz, r.ix, f);
    const double F[3] = {(double)s.cd.Fx, (double)s.cd.Fy, (double)s.cd.Fz};
    double rho, ux, uy, uz;
    macro_of<double>(f, F, rho, ux, uy, uz);
    const uint32_t n = gpu_lin(s.g, r.ix, r.iy, r.iz);
    const double s9 = s.les_w ? (double)s.les_s9[n] : (double)s.cd.kp * 36.0;
    const double nu = (1.0 / ((double)s.cd.kp * 36.0) - 0.5) / 3.0;
    double S6[6];
    strain_from_moments(f, rho, ux, uy, uz, (double)s.cd.ke * 2394.0, s9, S6);
    float Sf[6], x[kMlpIn];
    for (int k = 0; k < 6; ++k) Sf[k] = (float)S6[k];
    const float dwall = fminf((float)r.ix + 0.5f, (float)s.g.NZ - (float)r.ix - 0.5f);
    closure_features(Sf, dwall, (float)nu, ustar, h, x);
    const size_t o = (size_t)r.ix + (size_t)s.g.NZ * ((size_t)r.iy + (size_t)s.g.NX * (size_t)r.iz);
    for (int k = 0; k < kMlpIn; ++k) X[o * kMlpIn + k] = x[k];
}

__global__ void k_ref_to_gpu_vec(Geometry g, size_t N, const double* __restrict__ ux,
                                 const double* __restrict__ uy, const double* __restrict__ uz,
                                 double* __restrict__ uf, int z0) {
    const RefNode r = ref_node(g, z0);
    if (!r.ok) return;
    const size_t src = ref_lin(g, r.ix, r.iy, r.iz - z0);
    const uint32_t n = gpu_lin(g, r.ix, r.iy, r.iz);
    uf[n] = ux[src]; uf[N + n] = uy[src]; uf[2 * N + n] = uz[src];
}

// Frozen velocity of the pre-relaxation from the populations themselves:
// sum_i c_i f_i of the natural populations (GPU layout, 3 planes of N).  For
// a state that initpop's equilibrium at delta-rho = 0 produced, this is the
// velocity it was built from (sum_i w_i c_i c_i = I/3, the other terms are
// odd in c), to rounding.
template <typename T>
__global__ void k_uf_from_f(DeviceState s, int parity, double* __restrict__ uf) {
    const RefNode r = ref_node(s.g, 0);
    if (!r.ok) return;
    double f[Q];
    gather_natural<T>(s, parity, r.iy, r.iz, r.ix, f);
    double a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        if (CXf(i)) a += CXf(i) * f[i];
        if (CYf(i)) b += CYf(i) * f[i];
        if (CZf(i)) c += CZf(i) * f[i];
    }
    const uint32_t n = gpu_lin(s.g, r.ix, r.iy, r.iz);
    uf[n] = a; uf[s.N + n] = b; uf[2 * s.N + n] = c;
}

constexpr int kRedThreads = 256;

// Plane sums for statistc2: block (b, Z) covers part of plane Z (ref x = Z+1).
// Per-node values in the diagnostics type R, sums in FP64.
// Plane sums of dissipation_calc (saveload.f90:4780-4814) over the fluid
// nodes of each wall-normal plane: {S_ij S_ij method 1, method 2, S_xy method
// 1, method 2, fluid nodes}; partial[NZ][nblk][LBM_DISSIPATION_COLS].
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_dissipation(DeviceState s, int parity, double* __restrict__ partial) {
    const Geometry& g = s.g;
    const int z = blockIdx.y;
    double acc[LBM_DISSIPATION_COLS] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const uint32_t plane = g.NXY;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < plane; t += gridDim.x * blockDim.x) {
        if (s.owner && s.owner[t + plane * (uint32_t)z] >= 0) continue;     // solid node
        const NodeStrain v = node_strain<T>(s, parity, (int)(t % g.NX), (int)(t / g.NX), z);
        acc[0] += v.m1; acc[1] += v.m2; acc[2] += v.sxy1; acc[3] += v.sxy2; acc[4] += 1.0;
    }
    __shared__ double sh[LBM_DISSIPATION_COLS][kRedThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < LBM_DISSIPATION_COLS; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < LBM_DISSIPATION_COLS) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) v += sh[threadIdx.x][w];
        partial[((size_t)z * gridDim.x + blockIdx.x) * LBM_DISSIPATION_COLS + threadIdx.x] = v;
    }
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
k_profiles(DeviceState s, int parity, double* __restrict__ partial) {
    using R = typename DiagR<T>::type;
    const Geometry& g = s.g;
    const int z = blockIdx.y;
    const R F[3] = {(R)s.cd.Fx, (R)s.cd.Fy, (R)s.cd.Fz};
    double acc[LBM_PROFILE_COLS];
#pragma unroll
    for (int k = 0; k < LBM_PROFILE_COLS; ++k) acc[k] = 0.0;
    const uint32_t plane = g.NXY;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < plane; t += gridDim.x * blockDim.x) {
        const int x = t % g.NX, y = t / g.NX;
        if (s.owner && s.owner[t + plane * (uint32_t)z] >= 0) continue;     // solid node
        R f[Q];
        gather_natural_r<T, R>(s, parity, x, y, z, f);
        R rho, ux, uy, uz;
        macro_of(f, F, rho, ux, uy, uz);
        const double dux = ux, duy = uy, duz = uz, drho = rho;
        acc[0] += dux; acc[1] += duy; acc[2] += duz;
        acc[3] += dux * duz; acc[4] += dux * duy; acc[5] += duy * duz;
        acc[6] += dux * dux; acc[7] += duy * duy; acc[8] += duz * duz;
        acc[9] += drho; acc[10] += drho * drho; acc[11] += 1.0;
    }
    __shared__ double sh[LBM_PROFILE_COLS][kRedThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < LBM_PROFILE_COLS; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < LBM_PROFILE_COLS) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) v += sh[threadIdx.x][w];
        partial[((size_t)z * gridDim.x + blockIdx.x) * LBM_PROFILE_COLS + threadIdx.x] = v;
    }
}

// Per-block extrema: {rho_max, rho_min, vmax, vmax_refidx, nonfinite}.
// Blocks walk whole streamwise rows (32-bit row arithmetic); per-node values in
// the diagnostics type R.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
k_extrema(DeviceState s, int parity, double* __restrict__ partial) {
    using R = typename DiagR<T>::type;
    const Geometry& g = s.g;
    const R F[3] = {(R)s.cd.Fx, (R)s.cd.Fy, (R)s.cd.Fz};
    R rmax = -INFINITY, rmin = INFINITY, vmax = -1;
    uint32_t vidx = 0xffffffffu;
    unsigned nonf = 0;
    const uint32_t rows = (uint32_t)g.NY * (uint32_t)g.NZ;
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const int y = (int)(r % (uint32_t)g.NY), z = (int)(r / (uint32_t)g.NY);
        for (int x = threadIdx.x; x < g.NX; x += blockDim.x) {
            if (s.owner && s.owner[x + g.NX * r] >= 0) continue;            // solid node
            R f[Q];
            gather_natural_r<T, R>(s, parity, x, y, z, f);
            bool finite = true;
#pragma unroll
            for (int i = 0; i < Q; ++i) finite &= isfinite(f[i]);
            if (!finite) { ++nonf; continue; }
            R rho, ux, uy, uz;
            macro_of(f, F, rho, ux, uy, uz);
            rmax = rho > rmax ? rho : rmax;
            rmin = rho < rmin ? rho : rmin;
            const R v = sqrt(ux * ux + uy * uy + uz * uz);
            const uint32_t ri = (uint32_t)z + (uint32_t)g.NZ * ((uint32_t)x + (uint32_t)g.NX * (uint32_t)y);
            if (v > vmax || (v == vmax && ri < vidx)) { vmax = v; vidx = ri; }
        }
    }
    __shared__ double sh[5][kRedThreads];
    sh[0][threadIdx.x] = rmax; sh[1][threadIdx.x] = rmin; sh[2][threadIdx.x] = vmax;
    sh[3][threadIdx.x] = vidx == 0xffffffffu ? 1e300 : (double)vidx; sh[4][threadIdx.x] = nonf;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const int o = threadIdx.x + h;
            sh[0][threadIdx.x] = fmax(sh[0][threadIdx.x], sh[0][o]);
            sh[1][threadIdx.x] = fmin(sh[1][threadIdx.x], sh[1][o]);
            const double va = sh[2][threadIdx.x], vb = sh[2][o];
            if (vb > va || (vb == va && sh[3][o] < sh[3][threadIdx.x])) {
                sh[2][threadIdx.x] = vb; sh[3][threadIdx.x] = sh[3][o];
            }
            sh[4][threadIdx.x] += sh[4][o];
        }
        __syncthreads();
    }
    if (threadIdx.x < 5) partial[(size_t)blockIdx.x * 5 + threadIdx.x] = sh[threadIdx.x][0];
}

// Subtract w_i*delta from every population.  The weights are symmetric
// (w_i = w_opp(i)) and every (population, node) value occupies exactly one
// slot in either AA orientation, so the slot's own weight is the right one.
template <typename T>
__global__ void k_add_rest(DeviceState s, double delta) {
    const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= s.N) return;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        T* p = pop_plane<T>(s, i) + n;
        const double v = (double)ld_pop(p) + weight(i) * delta * s.cd.S;
        if constexpr (sizeof(T) == 8) *p = v; else st_pop(p, (float)v);
    }
}

// Fluid mass and fluid node count (acc[0], acc[1]) for the mean-density
// removal of avedensity (collision.f90:487-513), with the array in natural
// orientation (every population in its own node's slot).  A thread takes
// 16 bytes of every plane (8 FP16, 4 FP32 or 2 FP64 nodes); sums per node in
// the storage's arithmetic type (FP32 for FP32/FP16: GB300's FP64 rate is
// 1/64 of FP32), FP64 per thread and per block, one atomic pair per block.
// Nodes beyond the last whole group are summed one by one.
template <typename T>
struct Vec16 {
    static constexpr int N = 16 / (int)sizeof(T);
    __device__ __forceinline__ static void load(const T* p, float (&v)[16 / sizeof(T)]) {
        const uint4 w = *reinterpret_cast<const uint4*>(p);
        if constexpr (sizeof(T) == 2) {
            const __half2* h = reinterpret_cast<const __half2*>(&w);
#pragma unroll
            for (int k = 0; k < 4; ++k) { const float2 f = __half22float2(h[k]); v[2 * k] = f.x; v[2 * k + 1] = f.y; }
        } else {
            const float* f = reinterpret_cast<const float*>(&w);
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = f[k];
        }
    }
    __device__ __forceinline__ static void store(T* p, const float (&v)[16 / sizeof(T)]) {
        uint4 w;
        if constexpr (sizeof(T) == 2) {
            __half2* h = reinterpret_cast<__half2*>(&w);
#pragma unroll
            for (int k = 0; k < 4; ++k) h[k] = __floats2half2_rn(v[2 * k], v[2 * k + 1]);
        } else {
            float* f = reinterpret_cast<float*>(&w);
#pragma unroll
            for (int k = 0; k < 4; ++k) f[k] = v[k];
        }
        *reinterpret_cast<uint4*>(p) = w;
    }
};

template <typename T>
__global__ void __launch_bounds__(256) k_fluid_mass(DeviceState s, double* __restrict__ acc) {
    using R = typename DiagR<T>::type;
    double m = 0.0, cnt = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (sizeof(T) < 8) {
        constexpr int V = Vec16<T>::N;
        const size_t groups = s.N / V;
        for (size_t gidx = t0; gidx < groups; gidx += stride) {
            const size_t n0 = gidx * V;
            float r[V];
#pragma unroll
            for (int v = 0; v < V; ++v) r[v] = 0.f;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                float x[V];
                Vec16<T>::load(pop_plane<T>(s, i) + n0, x);
#pragma unroll
                for (int v = 0; v < V; ++v) r[v] += x[v];
            }
            float part = 0.f, c = 0.f;
#pragma unroll
            for (int v = 0; v < V; ++v)
                if (!s.owner || s.owner[n0 + v] < 0) { part += r[v]; c += 1.f; }
            m += (double)part;
            cnt += (double)c;
        }
        for (size_t n = groups * V + t0; n < s.N; n += stride) {
            if (s.owner && s.owner[n] >= 0) continue;
            R r = 0;
#pragma unroll
            for (int i = 0; i < Q; ++i) r += (R)ld_pop(pop_plane<T>(s, i) + n);
            m += (double)r;
            cnt += 1.0;
        }
    } else {
        for (size_t n = t0; n < s.N; n += stride) {
            if (s.owner && s.owner[n] >= 0) continue;
            double r = 0.0;
#pragma unroll
            for (int i = 0; i < Q; ++i) r += ld_pop(pop_plane<T>(s, i) + n);
            m += r;
            cnt += 1.0;
        }
    }
    m *= s.cd.invS;
    for (int o = 16; o > 0; o >>= 1) {
        m += __shfl_xor_sync(0xffffffffu, m, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    __shared__ double sh[2][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh[0][w] = m; sh[1][w] = cnt; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += sh[0][k]; b += sh[1][k]; }
        atomicAdd(acc, a);
        atomicAdd(acc + 1, b);
    }
}

// Same sum with the array after an odd number of AA steps: each fluid node's
// populations are gathered from their parity-1 slots (every 100 steps only).
template <typename T>
__global__ void __launch_bounds__(256) k_fluid_mass_gather(DeviceState s, double* __restrict__ acc) {
    using R = typename DiagR<T>::type;
    const Geometry& g = s.g;
    double m = 0.0, cnt = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < s.N; n += stride) {
        if (s.owner && s.owner[n] >= 0) continue;
        const int x = (int)(n % g.NX), y = (int)((n / g.NX) % g.NY), z = (int)(n / g.NXY);
        R f[Q];
        gather_natural_r<T, R>(s, 1, x, y, z, f);
        R r = 0;
#pragma unroll
        for (int i = 0; i < Q; ++i) r += f[i];
        m += (double)r;
        cnt += 1.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        m += __shfl_xor_sync(0xffffffffu, m, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    __shared__ double sh[2][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh[0][w] = m; sh[1][w] = cnt; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += sh[0][k]; b += sh[1][k]; }
        atomicAdd(acc, a);
        atomicAdd(acc + 1, b);
    }
}

// Remove the mean density acc[0] / acc[1] (w_i * mean from every population),
// 16 bytes per plane and thread as above.  Every storage slot holds one
// population of one node in either parity, and slot opp(i) of the parity-1
// layout holds direction i with w_opp(i) = w_i, so the same pass serves both
// parities.
template <typename T>
__global__ void k_remove_mean(DeviceState s, const double* __restrict__ acc) {
    using R = typename DiagR<T>::type;
    const R dS = (R)((acc[1] > 0.0 ? -acc[0] / acc[1] : 0.0) * s.cd.S);   // scaled delta
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (sizeof(T) < 8) {
        constexpr int V = Vec16<T>::N;
        const size_t groups = s.N / V;
        if (t < groups) {
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                T* p = pop_plane<T>(s, i) + t * V;
                float x[V];
                Vec16<T>::load(p, x);
                const float d = (float)weight(i) * (float)dS;
#pragma unroll
                for (int v = 0; v < V; ++v) x[v] += d;
                Vec16<T>::store(p, x);
            }
        } else {
            const size_t n = groups * V + (t - groups);
            if (n >= s.N) return;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                T* p = pop_plane<T>(s, i) + n;
                st_pop(p, (float)((R)ld_pop(p) + (R)weight(i) * dS));
            }
        }
    } else {
        if (t >= s.N) return;
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            T* p = pop_plane<T>(s, i) + t;
            *p = ld_pop(p) + weight(i) * (double)dS;
        }
    }
}

dim3 ref_grid(const Geometry& g, int nzc, int bx) {
    return dim3((g.NX + bx - 1) / bx, g.NZ, nzc);
}
constexpr int kBx = 128;

}  // namespace

void channel_velocity_host(int nx, int ny, int nz, double uc, double amp, uint64_t seed,
                           double* ux, double* uy, double* uz) {
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const size_t o = (size_t)ix + (size_t)nx * ((size_t)iy + (size_t)ny * iz);
                channel_velocity_node(nx, ny, ix, iy, iz, uc, amp, seed, ux[o], uy[o], uz[o]);
            }
}

size_t loglaw_table_doubles(int nx, int ny, int nz) {
    return 3 * (size_t)(nx / 2) + 2 * (size_t)ny * (size_t)nz;
}

// Tables of initvel's turbulent branch (initial.f90:81-147) with its
// constants A9 (perturbation amplitude, 0 as shipped), alpha = beta9 = 1,
// cc = 60 and pi2 = 2*(4*atan(1)) (var_inc.f90:71-72).  Layout: P, Ay, Ax
// (nx/2 each), then sin and cos of alpha*y9 + beta9*z9 per column
// (iy + ny*iz).  Each expression keeps the reference's evaluation order.
void loglaw_tables_host(int nx, int ny, int nz, double ustar, double ystar, double a9, double* tab) {
    const int nxh = nx / 2;
    const double pi2 = 2.0 * (4.0 * std::atan(1.0));
    const double alpha = 1.0, beta9 = 1.0, cc = 60.0;
    const double ccc1 = -((double)ny / pi2 / alpha / ystar * a9 * ustar / cc / cc);
    double* P = tab;
    double* Ay = tab + nxh;
    double* Ax = tab + 2 * (size_t)nxh;
    double* Sn = tab + 3 * (size_t)nxh;
    double* Cs = Sn + (size_t)ny * nz;
    for (int m = 0; m < nxh; ++m) {
        const double yplus = ((double)(m + 1) - 0.5) / ystar;
        if (yplus < 10.8) {
            P[m] = yplus * ustar;
        } else {
            double u9 = std::log(yplus) / 0.41 + 5.0;
            P[m] = u9 * ustar;
        }
        const double ccc9 = std::exp(-yplus / cc);
        Ay[m] = ccc1 * yplus * ccc9;
        Ax[m] = a9 * ustar * (1.0 - ccc9 - yplus / cc * ccc9);
    }
    for (int k = 0; k < nz; ++k) {
        const double z9 = pi2 * ((double)(k + 1) - 0.5) / (double)nz;
        for (int j = 0; j < ny; ++j) {
            const double y9 = pi2 * ((double)(j + 1) - 0.5) / (double)ny;
            const double arg = alpha * y9 + beta9 * z9;
            Sn[(size_t)j + (size_t)ny * k] = std::sin(arg);
            Cs[(size_t)j + (size_t)ny * k] = std::cos(arg);
        }
    }
}

void loglaw_velocity_host(int nx, int ny, int nz, const double* tab, double* ux, double* uy, double* uz) {
    const int nxh = nx / 2;
    const double* P = tab;
    const double* Ay = tab + nxh;
    const double* Ax = tab + 2 * (size_t)nxh;
    const double* Sn = tab + 3 * (size_t)nxh;
    const double* Cs = Sn + (size_t)ny * nz;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const size_t o = (size_t)ix + (size_t)nx * ((size_t)iy + (size_t)ny * iz);
                int m = -1;
                if (ix < nxh) m = ix;
                else if (nx - 1 - ix < nxh) m = nx - 1 - ix;
                double u = 0.0, v = 0.0;
                if (m >= 0) {
                    const size_t col = (size_t)iy + (size_t)ny * iz;
                    v = P[m] + Ay[m] * Sn[col];
                    u = 0.0 + Ax[m] * Cs[col];
                }
                ux[o] = u;
                uy[o] = v;
                uz[o] = 0.0;
            }
}

#define LBM_DISPATCH(PREC_EXPR, CALL)                                   \
    switch (PREC_EXPR) {                                                \
        case LBM_PREC_FP64: { using T = double; CALL; } break;          \
        case LBM_PREC_FP32: { using T = float; CALL; } break;           \
        case LBM_PREC_FP16: { using T = __half; CALL; } break;          \
        default: return cudaErrorInvalidValue;                          \
    }                                                                   \
    return cudaGetLastError();

cudaError_t launch_aos_to_store(const DeviceState& s, const double* aos, int z0, int nzc,
                                cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_aos_to_store<T><<<ref_grid(s.g, nzc, kBx), kBx, 0, st>>>(s, aos, z0)))
}

cudaError_t launch_store_to_aos(const DeviceState& s, int parity, double* aos, int z0, int nzc,
                                cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_store_to_aos<T><<<ref_grid(s.g, nzc, kBx), kBx, 0, st>>>(s, parity, aos, z0)))
}

dim3 tile_grid(const Geometry& g, int nzc) {
    return dim3((unsigned)((g.NX + kTile - 1) / kTile), (unsigned)((g.NZ + kTile - 1) / kTile), (unsigned)nzc);
}

cudaError_t launch_initpop(const DeviceState& s, const double* ux, const double* uy,
                           const double* uz, int z0, int nzc, cudaStream_t st) {
    const dim3 blk(kTile, kTileRows);
    switch (s.prec) {
        case LBM_PREC_FP64: k_initpop_t<double, double><<<tile_grid(s.g, nzc), blk, 0, st>>>(s, ux, uy, uz, z0); break;
        case LBM_PREC_FP32: k_initpop_t<float, float><<<tile_grid(s.g, nzc), blk, 0, st>>>(s, ux, uy, uz, z0); break;
        case LBM_PREC_FP16: k_initpop_t<__half, float><<<tile_grid(s.g, nzc), blk, 0, st>>>(s, ux, uy, uz, z0); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_init_channel(const DeviceState& s, double uc, double amp, uint64_t seed,
                                cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_init_channel<T><<<ref_grid(s.g, s.g.NY, kBx), kBx, 0, st>>>(s, uc, amp, seed)))
}

cudaError_t launch_init_loglaw(const DeviceState& s, const double* tab, int nxh, cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_init_loglaw<T><<<ref_grid(s.g, s.g.NY, kBx), kBx, 0, st>>>(s, tab, nxh)))
}

cudaError_t launch_owner_to_ref(const DeviceState& s, const int* owner, int32_t* ib, int32_t* is, int z0, int nzc,
                               cudaStream_t st) {
    k_owner_to_ref<<<ref_grid(s.g, nzc, kBx), kBx, 0, st>>>(s.g, owner, ib, is, z0);
    return cudaGetLastError();
}

cudaError_t launch_macro(const DeviceState& s, int parity, double* rho, double* ux, double* uy,
                         double* uz, int z0, int nzc, cudaStream_t st) {
    const dim3 blk(kTile, kTileRows), grid = tile_grid(s.g, nzc);
    switch (s.prec) {
        case LBM_PREC_FP64: k_macro_t<double, double><<<grid, blk, 0, st>>>(s, parity, rho, ux, uy, uz, z0); break;
        case LBM_PREC_FP32: k_macro_t<float, float><<<grid, blk, 0, st>>>(s, parity, rho, ux, uy, uz, z0); break;
        case LBM_PREC_FP16: k_macro_t<__half, float><<<grid, blk, 0, st>>>(s, parity, rho, ux, uy, uz, z0); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_strain(const DeviceState& s, int parity, double* m1, double* m2, int z0, int nzc,
                          cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_strain<T><<<ref_grid(s.g, nzc, kBx), kBx, 0, st>>>(s, parity, m1, m2, z0)))
}

cudaError_t launch_box_filter(const DeviceState& s, int parity, int factor, int nxc, int nyc, int nzc,
                              double* out, cudaStream_t st) {
    const int bx = nxc < 128 ? nxc : 128;
    const dim3 grid((nxc + bx - 1) / bx, nyc, nzc);
    LBM_DISPATCH(s.prec, (k_box_filter<T><<<grid, bx, 0, st>>>(s, parity, factor, nxc, nyc, nzc, out)))
}

cudaError_t launch_closure_targets(const double* F9, int nxc, int nyc, int nzc, float nu_c, float ustar,
                                   float h_c, float* X, float* y, cudaStream_t st) {
    const int bx = nxc < 128 ? nxc : 128;
    const dim3 grid((nxc + bx - 1) / bx, nyc, nzc);
    k_closure_targets<<<grid, bx, 0, st>>>(F9, nxc, nyc, nzc, nu_c, ustar, h_c, X, y);
    return cudaGetLastError();
}

cudaError_t launch_les_features(const DeviceState& s, int parity, float ustar, float h, float* X,
                                cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_les_features<T><<<ref_grid(s.g, s.g.NY, kBx), kBx, 0, st>>>(s, parity, ustar, h, X, 0)))
}

cudaError_t launch_uf_from_f(const DeviceState& s, int parity, double* uf, cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_uf_from_f<T><<<ref_grid(s.g, s.g.NY, kBx), kBx, 0, st>>>(s, parity, uf)))
}

cudaError_t launch_ref_to_gpu_vec(const DeviceState& s, const double* ux, const double* uy,
                                  const double* uz, double* uf, int z0, int nzc, cudaStream_t st) {
    k_ref_to_gpu_vec<<<ref_grid(s.g, nzc, kBx), kBx, 0, st>>>(s.g, s.N, ux, uy, uz, uf, z0);
    return cudaGetLastError();
}

int profile_blocks(const DeviceState& s) {
    const uint32_t plane = s.g.NXY;
    int nb = (int)((plane + kRedThreads * 8 - 1) / (kRedThreads * 8));
    return nb < 1 ? 1 : (nb > 64 ? 64 : nb);
}

cudaError_t launch_dissipation(const DeviceState& s, int parity, double* partial, int nblk, cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_dissipation<T><<<dim3(nblk, s.g.NZ), kRedThreads, 0, st>>>(s, parity, partial)))
}

cudaError_t launch_profiles(const DeviceState& s, int parity, double* partial, int nblk,
                            cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_profiles<T><<<dim3(nblk, s.g.NZ), kRedThreads, 0, st>>>(s, parity, partial)))
}

cudaError_t launch_extrema(const DeviceState& s, int parity, double* partial,
                           cudaStream_t st) {
    LBM_DISPATCH(s.prec, (k_extrema<T><<<kExtremaBlocks, kRedThreads, 0, st>>>(s, parity, partial)))
}

cudaError_t launch_add_rest(const DeviceState& s, int parity, double delta, cudaStream_t st) {
    (void)parity;
    const unsigned nb = (unsigned)((s.N + 255) / 256);
    LBM_DISPATCH(s.prec, (k_add_rest<T><<<nb, 256, 0, st>>>(s, delta)))
}

cudaError_t launch_remove_mean_density(const DeviceState& s, int parity, double* acc, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(acc, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)std::max(1, 8 * s.sm_count);
    if (parity) {
        LBM_DISPATCH(s.prec, (k_fluid_mass_gather<T><<<grid, 256, 0, st>>>(s, acc)))
    }
    LBM_DISPATCH(s.prec, (k_fluid_mass<T><<<grid, 256, 0, st>>>(s, acc)))
}

cudaError_t launch_remove_mean_apply(const DeviceState& s, const double* acc, cudaStream_t st) {
    // one thread per 16-byte group plus the remainder nodes (FP16/FP32), one
    // per node (FP64)
    const size_t V = s.prec == LBM_PREC_FP64 ? 1 : (s.prec == LBM_PREC_FP32 ? 4 : 8);
    const size_t threads = V == 1 ? s.N : s.N / V + s.N % V;
    const unsigned nb = (unsigned)((threads + 255) / 256);
    LBM_DISPATCH(s.prec, (k_remove_mean<T><<<nb, 256, 0, st>>>(s, acc)))
}

}  // namespace lbm
