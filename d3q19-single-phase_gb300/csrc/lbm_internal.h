// Internal declarations shared by the CUDA translation units and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stddef.h>
#include <stdint.h>
#include <string>

#include "../../include/lbm_gb300.h"
#include "lbm_lattice.h"
#include "lbm_collide.cuh"

namespace lbm {

// Storage type of each precision and its arithmetic type.
template <int PREC> struct Prec;
template <> struct Prec<LBM_PREC_FP64> { using T = double; using R = double; };
template <> struct Prec<LBM_PREC_FP32> { using T = float;  using R = float; };
template <> struct Prec<LBM_PREC_FP16> { using T = __half; using R = float; };

__device__ __forceinline__ double ld_pop(const double* p) { return __ldg(p); }
__device__ __forceinline__ float  ld_pop(const float* p)  { return __ldg(p); }
__device__ __forceinline__ float  ld_pop(const __half* p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ void st_pop(double* p, double v) { *p = v; }
__device__ __forceinline__ void st_pop(float* p, float v)   { *p = v; }
__device__ __forceinline__ void st_pop(__half* p, float v)  { *p = __float2half_rn(v); }

// Bounds-checked build (-DLBM_BOUNDS_CHECK; the debug library of the build
// recipe): the index checks of the kernels record the site number of the
// first failing check in a device flag and skip the access, and the host
// reports it as an error after the call.  Nothing traps.  In the normal
// build every check is the constant true and compiles away.
#ifdef LBM_BOUNDS_CHECK
__device__ __forceinline__ bool bounds_ok(unsigned* flag, bool ok, unsigned site) {
    if (!ok && flag) atomicCAS(flag, 0u, site);
    return ok;
}
#define LBM_IN_BOUNDS(FLAG, COND, SITE) ::lbm::bounds_ok((FLAG), (COND), (SITE))
#else
#define LBM_IN_BOUNDS(FLAG, COND, SITE) true
#endif

// One base pointer per population plane, passed by value so that every
// address is a single IMAD.WIDE from the constant bank.
template <typename T>
struct PopPtrs { T* p[Q]; };

struct Geometry {
    int NX, NY, NZ;      // GPU axes (X = ref y, Y = ref z, Z = ref x)
    uint32_t NXY;        // NX*NY
};

// Moving spheres on the device (all FP64 state, 3 values per sphere).
// Per-sphere geometry in the forms the node kernels use, written once per
// update of the positions (no FP64 in the kernels that read it).
struct SphereGeom {
    int ci[3];          // floor of the centre, reference axes
    float h[3];         // 0.5 - (centre - ci): FP32 offset of node ci from the centre
    float delta;        // displacement of the last update, rounded up
    float U[3], W[3];   // velocity and angular velocity in FP32
    float pad[3];
};

struct DeviceParticles {
    int npart;
    int refill_cap;
    double R, rho_ratio, stf0, stf1, stf0_w, stf1_w, zeta;
    double *pos, *vel, *omg;          // centre, velocity, angular velocity
    double *force, *torque;           // hydrodynamic part of the last step
    double *fprev, *tprev;            // total force/torque of the previous step
    double *rep;                      // repulsion of the current step
    double *pos_prev;                 // centre before the last Newton-Euler update
    SphereGeom* geom;                 // [npart]
    int q_fp64;                       // FP64 link fractions for FP32/FP16 storage
    float Rf;                         // radius in FP32
    int* owner;                       // per node: sphere id, -1 fluid, -2 pending refill
    uint32_t* refill_node;
    int* refill_part;
    unsigned* counters;               // [0] refills, [1] links, [2] cell overflow, [3] refill overflow
    // cell list of the repulsion (ncell == 0: all-pairs search)
    int ncell, cell_nx, cell_ny, cell_nz;   // cells along reference x, y, z
    int* cell_count;                        // [ncell]
    int* cell_list;                         // [ncell][kCellCap] sphere ids
    // order in which the bounce-back kernel's CTAs take the spheres (sorted by
    // the Morton code of cells order_cs wide, so that neighbouring spheres,
    // which share cache lines of the population rows, run at the same time);
    // nullptr: index order.  order_key [npart], order_hist [order_nbins].
    int* order;
    int* order_key;
    int* order_hist;
    double order_cs;
    int order_nbins;
};
constexpr int kCellCap = 32;              // spheres per repulsion cell

// Everything a step needs; built once per context.
struct DeviceState {
    int prec;
    Geometry g;
    size_t N;            // nodes
    size_t pstride;      // elements between population planes
    void* f;             // 19 * pstride elements of the storage type
    CollideConsts<double> cd;
    CollideConsts<float> cf;
    unsigned* bounds;    // first failing bounds-check site (bounds-checked build)
    int sm_count;        // SMs of the device (persistent grids)
    int use_rows;        // 1: row-pipelined bulk-copy kernels for the step
    // spheres (owner == nullptr without spheres): fluid masks and the rigid
    // velocity of solid nodes for the diagnostics and macrovar
    const int* owner;
    const double *ppos, *pvel, *pomg;
    double prho;
    // learned LES closure (les_w == nullptr: off): network parameters and
    // feature normalisation (1345 + 14 floats), per-node shear rate of the
    // last collision, molecular viscosity and the wall units of the features
    const float* les_w;
    float* les_s9;
    double les_nu;
    float les_ustar, les_h;
    float les_aplus;     // van Driest damping constant A+ of nu_t (0: off)
};

// launchers (lbm_step.cu)
cudaError_t launch_step(const DeviceState& s, int parity, cudaStream_t st);
cudaError_t launch_prerelax(const DeviceState& s, int parity, const double* uf,
                            double* rho_prev_and_new, unsigned long long* maxabs,
                            cudaStream_t st);

// row-pipelined bulk-copy step (lbm_step_tma.cu), FP32/FP16 storage
bool rows_supported(const DeviceState& s);
cudaError_t prepare_step_rows();
cudaError_t launch_step_rows(const DeviceState& s, int parity, int* err, cudaStream_t st);

// field kernels (lbm_fields.cu)
// AoS FP64 chunk (reference layout, ref z planes [z0, z0+nzc)) <-> storage.
cudaError_t launch_aos_to_store(const DeviceState& s, const double* aos, int z0,
                                int nzc, cudaStream_t st);
cudaError_t launch_store_to_aos(const DeviceState& s, int parity, double* aos,
                                int z0, int nzc, cudaStream_t st);
// equilibrium from velocity arrays in reference layout (chunk of ref z planes)
cudaError_t launch_initpop(const DeviceState& s, const double* ux,
                           const double* uy, const double* uz, int z0, int nzc,
                           cudaStream_t st);
cudaError_t launch_init_channel(const DeviceState& s, double uc, double amp,
                                uint64_t seed, cudaStream_t st);
// particle checkpoint node flags (ibnodes, isnodes) for ref z planes
// [z0, z0+nzc), reference layout
cudaError_t launch_owner_to_ref(const DeviceState& s, const int* owner, int32_t* ib, int32_t* is, int z0, int nzc,
                               cudaStream_t st);
// macrovar for ref z planes [z0, z0+nzc) into reference-layout FP64 arrays
cudaError_t launch_macro(const DeviceState& s, int parity, double* rho,
                         double* ux, double* uy, double* uz, int z0, int nzc,
                         cudaStream_t st);
// velocity (nx*ny*nz*3 doubles, reference layout chunk) to GPU-layout frozen u
cudaError_t launch_strain(const DeviceState& s, int parity, double* m1, double* m2, int z0, int nzc,
                          cudaStream_t st);
cudaError_t launch_box_filter(const DeviceState& s, int parity, int factor, int nxc, int nyc, int nzc,
                              double* out, cudaStream_t st);
cudaError_t launch_closure_targets(const double* F9, int nxc, int nyc, int nzc, float nu_c, float ustar,
                                   float h_c, float* X, float* y, cudaStream_t st);
cudaError_t launch_les_features(const DeviceState& s, int parity, float ustar, float h, float* X,
                                cudaStream_t st);
// mean-density removal on the device, either parity: fluid mass into acc[2],
// then applied
cudaError_t launch_remove_mean_density(const DeviceState& s, int parity, double* acc, cudaStream_t st);
cudaError_t launch_remove_mean_apply(const DeviceState& s, const double* acc, cudaStream_t st);
// pre-relaxation's frozen velocity from the current natural populations
cudaError_t launch_uf_from_f(const DeviceState& s, int parity, double* uf, cudaStream_t st);
cudaError_t launch_ref_to_gpu_vec(const DeviceState& s, const double* ux,
                                  const double* uy, const double* uz,
                                  double* uf, int z0, int nzc, cudaStream_t st);
// plane sums (LBM_PROFILE_COLS per wall-normal plane) into partials
// [NZ][nblk][COLS]; nblk returned through the call.
cudaError_t launch_profiles(const DeviceState& s, int parity, double* partial,
                            int nblk, cudaStream_t st);
int profile_blocks(const DeviceState& s);
// dissipation_calc plane sums (LBM_DISSIPATION_COLS per wall-normal plane),
// same partial layout and block count as launch_profiles
cudaError_t launch_dissipation(const DeviceState& s, int parity, double* partial, int nblk, cudaStream_t st);
// per-block extrema for diag: partial[kExtremaBlocks][5] =
// {rho_max, rho_min, vmax, reference linear index of vmax, nonfinite count}
constexpr int kExtremaBlocks = 1024;
cudaError_t launch_extrema(const DeviceState& s, int parity, double* partial,
                           cudaStream_t st);
cudaError_t launch_add_rest(const DeviceState& s, int parity, double delta,
                            cudaStream_t st);

// splitmix64-based uniform in [-1, 1): identical on host and device
__host__ __device__ inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ inline double uniform_pm1(uint64_t seed, uint64_t key) {
    const uint64_t z = splitmix64(seed * 0xD1B54A32D192ED03ull + key);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

// moving spheres (lbm_particles.cu)
// dynamic shared memory of the bounce-back kernel for spheres of radius R
size_t particles_smem_bytes(double R);
cudaError_t particles_claim(const DeviceState& s, const DeviceParticles& P, cudaStream_t st);
// A second stream of the context with two events: the sphere pass forks the
// repulsion (which needs only the positions) onto it, concurrent with the
// bounce-back kernel, and joins it back before the Newton-Euler update.
// st == nullptr: everything runs on the main stream.
struct SideStream {
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
cudaError_t particles_after_step(const DeviceState& s, const DeviceParticles& P, int parity, int have_prev,
                                 cudaStream_t st, const SideStream& side);
// kernels that one particles_after_step launches
int particles_kernels_per_step(const DeviceParticles& P);
// re-sort the spheres into the bounce-back kernel's spatial order from their
// current positions (3 kernels); a no-op without an order buffer
cudaError_t particles_reorder(const DeviceParticles& P, cudaStream_t st);
constexpr int kReorderKernels = 3;
constexpr int kReorderEvery = 100;            // steps between re-sorts
cudaError_t particles_count_solid(const DeviceState& s, const DeviceParticles& P, unsigned long long* d_out,
                                  cudaStream_t st);

void channel_velocity_host(int nx, int ny, int nz, double uc, double amp,
                           uint64_t seed, double* ux, double* uy, double* uz);

// log-law initial velocity (initial.f90:101-147): host tables, the host
// field they give, and the device initial condition built from them
size_t loglaw_table_doubles(int nx, int ny, int nz);
void loglaw_tables_host(int nx, int ny, int nz, double ustar, double ystar, double a9, double* tab);
void loglaw_velocity_host(int nx, int ny, int nz, const double* tab, double* ux, double* uy, double* uz);
cudaError_t launch_init_loglaw(const DeviceState& s, const double* tab, int nxh, cudaStream_t st);

}  // namespace lbm
