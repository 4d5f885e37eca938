// lbm_profiles_noalloc: the statistc2 plane sums without any allocation.
//
// Some callers cannot allocate device memory when they want the flow
// statistics: a monitor that samples profiles while the solver owns a fixed
// memory budget, code that runs between the captures of a CUDA graph, or an
// embedding host whose allocator is not the CUDA runtime's.  lbm_profiles may
// cudaMalloc its reduction buffer on first use; this variant keeps the partial
// sums in a fixed array compiled into the library instead, and needs nothing
// from the caller but the context and the output array.
//
// Scratch: LBM_NOALLOC_MAX_PLANES wall-normal planes x (kBlocks + 1) x 12
// doubles (about 2 MB), resident on every GPU that loads the library until the
// process exits.  Every call overwrites all the entries it reads, so nothing
// needs clearing; calls that overlap on the GPU (two streams, two threads)
// share the array and race.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "lbm_internal.h"

namespace lbm {
// context internals, defined in lbm_capi.cu
const DeviceState* ctx_state(lbm_ctx* c, int* parity, cudaStream_t* stream, int* device);
int set_error(int code, const char* msg);
}  // namespace lbm

namespace {

constexpr int kBlocks = 4;                          // blocks per plane
constexpr int kMaxPlanes = LBM_NOALLOC_MAX_PLANES;
constexpr size_t kPartials = (size_t)kMaxPlanes * kBlocks * LBM_PROFILE_COLS;
constexpr size_t kTotals = (size_t)kMaxPlanes * LBM_PROFILE_COLS;

// [plane][block][col] partial sums, then [plane][col] totals
static __device__ __align__(256) double g_profile_scratch[kPartials + kTotals];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};
std::once_flag g_scratch_once[kMaxDevices];
cudaError_t g_scratch_err[kMaxDevices] = {};

__global__ void k_plane_totals(const double* __restrict__ partial, double* __restrict__ totals, int nplanes) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nplanes * LBM_PROFILE_COLS) return;
    const int z = t / LBM_PROFILE_COLS, col = t % LBM_PROFILE_COLS;
    double acc = 0.0;
    for (int b = 0; b < kBlocks; ++b) acc += partial[((size_t)z * kBlocks + b) * LBM_PROFILE_COLS + col];
    totals[t] = acc;
}

// Device address of the scratch array on `device` (which must be current).
// Resolved once per device; the first call on a device does it.
double* scratch_on(int device, cudaError_t* err) {
    std::call_once(g_scratch_once[device], [device] {
        void* p = nullptr;
        g_scratch_err[device] = cudaGetSymbolAddress(&p, g_profile_scratch);
        g_scratch_ptr[device] = g_scratch_err[device] == cudaSuccess ? static_cast<double*>(p) : nullptr;
    });
    *err = g_scratch_err[device];
    return g_scratch_ptr[device];
}

}  // namespace

extern "C" int lbm_profiles_noalloc(lbm_ctx* ctx, double* out) {
    using namespace lbm;
    if (!ctx || !out) return set_error(LBM_ERR_INVALID_ARG, "null argument");
    int parity = 0, device = 0;
    cudaStream_t st = nullptr;
    const DeviceState* s = ctx_state(ctx, &parity, &st, &device);
    const int nplanes = s->g.NZ;                 // reference nx
    if (nplanes > kMaxPlanes)
        return set_error(LBM_ERR_INVALID_ARG,
                         ("lbm_profiles_noalloc: nx = " + std::to_string(nplanes) +
                          " exceeds LBM_NOALLOC_MAX_PLANES = " + std::to_string(kMaxPlanes))
                             .c_str());
    if (device < 0 || device >= kMaxDevices) return set_error(LBM_ERR_INVALID_ARG, "device ordinal out of range");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return set_error(LBM_ERR_CUDA, cudaGetErrorString(e));
    double* scratch = scratch_on(device, &e);
    if (e != cudaSuccess || !scratch)
        return set_error(LBM_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
    double* partial = scratch;
    double* totals = scratch + kPartials;
    e = launch_profiles(*s, parity, partial, kBlocks, st);
    if (e == cudaSuccess) {
        const int n = nplanes * LBM_PROFILE_COLS;
        k_plane_totals<<<(n + 255) / 256, 256, 0, st>>>(partial, totals, nplanes);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, totals, (size_t)nplanes * LBM_PROFILE_COLS * sizeof(double),
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(LBM_ERR_CUDA, cudaGetErrorString(e));
    return LBM_OK;
}
