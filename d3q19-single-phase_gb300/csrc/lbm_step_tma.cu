// Row-pipelined AA step for FP32/FP16 storage: bulk-copy (TMA) staging of
// x-pencils in shared memory.
//
// Work item = one full streamwise row (all NX nodes at fixed Y, Z).  In the AA
// pattern every row read by an item is also written by that item and by no
// other (even step: plane i of row (Y,Z) -> plane opp(i) of the same row; odd
// step: plane opp(i) of row (Y,Z)-c_i -> plane i of row (Y,Z)+c_i, the same
// set), so items are independent and a whole row can be moved with one bulk
// copy per population.  Rows along X wrap onto themselves, which makes the
// periodic x-shift of the odd step a modular index inside shared memory.
//
// Each persistent CTA owns one SM and a ring of NSTAGE stage buffers of 19
// rows.  Thread 0 issues the 19 cp.async.bulk loads of an item into a stage
// with one mbarrier (expect_tx = 19 rows); all threads wait on it (bounded)
// and compute two adjacent nodes each.  Results go either
//   SOUT = true : into one of two shared-memory output buffers (x-shift and
//                 periodic wrap applied there) that thread 0 writes back with
//                 19 bulk stores at the start of the next item, or
//   SOUT = false: straight to HBM (aligned pairs as one 32/64-bit store,
//                 x-shifted populations element-wise) when shared memory is
//                 too small for output buffers (FP32 rows of 1024).
// NSTAGE-1 items are always in flight, so the bytes in flight per SM are set
// by shared memory, not by registers.
#include <algorithm>

#include "lbm_internal.h"

namespace lbm {

namespace {

constexpr uint32_t kSpinLimit = 1u << 22;    // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void bulk_store(void* dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// storage <-> arithmetic helpers for an aligned pair / a single element
__device__ __forceinline__ void ld_pair(const __half* p, float& a, float& b) {
    const float2 v = __half22float2(*reinterpret_cast<const __half2*>(p));
    a = v.x; b = v.y;
}
__device__ __forceinline__ void ld_pair(const float* p, float& a, float& b) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    a = v.x; b = v.y;
}
__device__ __forceinline__ float ld_one(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float ld_one(const float* p) { return *p; }
__device__ __forceinline__ void st_pair(__half* p, float a, float b) {
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
}
__device__ __forceinline__ void st_pair(float* p, float a, float b) {
    *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
__device__ __forceinline__ void st_one(__half* p, float a) { *p = __float2half_rn(a); }
__device__ __forceinline__ void st_one(float* p, float a) { *p = a; }

struct Item {
    int y, z;
    uint32_t row;                  // NX*(y + NY*z)
};
__device__ __forceinline__ Item item_of(const Geometry& g, uint32_t it) {
    Item I;
    I.y = it % g.NY;
    I.z = it / g.NY;
    I.row = (uint32_t)g.NX * it;
    return I;
}
__device__ __forceinline__ uint32_t row_at(const Geometry& g, int y, int z) {
    y = y < 0 ? y + g.NY : (y >= g.NY ? y - g.NY : y);
    return (uint32_t)g.NX * ((uint32_t)y + (uint32_t)g.NY * (uint32_t)z);
}
__device__ __forceinline__ int wall_of(const Geometry& g, int z) {
    return (z == 0 ? 1 : 0) | (z == g.NZ - 1 ? 2 : 0);
}
__device__ __forceinline__ bool pull_bb(int wall, int i) {
    return (DZg(i) == 1 && (wall & 1)) || (DZg(i) == -1 && (wall & 2));
}
__device__ __forceinline__ bool push_bb(int wall, int i) {
    return (DZg(i) == 1 && (wall & 2)) || (DZg(i) == -1 && (wall & 1));
}

// Source row of population i's staged input for an item.
template <typename T, bool ODD>
__device__ __forceinline__ const T* src_row(const PopPtrs<T>& P, const Geometry& g, const Item& I, int wall, int i) {
    if (!ODD || pull_bb(wall, i)) return P.p[i] + I.row;
    return P.p[OPPf(i)] + row_at(g, I.y - DYg(i), I.z - DZg(i));
}

// Destination row of population i's result for an item.
template <typename T, bool ODD>
__device__ __forceinline__ T* dst_row(const PopPtrs<T>& P, const Geometry& g, const Item& I, int wall, int i) {
    if (!ODD || push_bb(wall, i)) return P.p[OPPf(i)] + I.row;
    return P.p[i] + row_at(g, I.y + DYg(i), I.z + DZg(i));
}

template <typename T, bool ODD>
__device__ void store_item(const PopPtrs<T>& P, const Geometry& g, uint32_t it, uint32_t out_smem,
                           uint32_t row_bytes) {
    const Item I = item_of(g, it);
    const int wall = wall_of(g, I.z);
#pragma unroll
    for (int i = 0; i < Q; ++i)
        bulk_store(dst_row<T, ODD>(P, g, I, wall, i), out_smem + (uint32_t)i * row_bytes, row_bytes);
    bulk_commit();
}

template <typename T, bool ODD>
__device__ void issue_item(const PopPtrs<T>& P, const Geometry& g, uint32_t it, uint32_t stage_smem,
                           uint32_t bar, uint32_t row_bytes) {
    const Item I = item_of(g, it);
    const int wall = wall_of(g, I.z);
    mbar_expect_tx(bar, (uint32_t)Q * row_bytes);
#pragma unroll
    for (int i = 0; i < Q; ++i)
        bulk_load(stage_smem + (uint32_t)i * row_bytes, src_row<T, ODD>(P, g, I, wall, i), row_bytes, bar);
}

// Two adjacent nodes (x, x+1), x even, of one item.  out == nullptr: write
// straight to HBM; otherwise into the item's shared-memory output rows
// (population i's result row at out + i*NX, in destination x order).
template <typename T, bool ODD, int WALL, bool SOUT>
__device__ __forceinline__ void pair_update(const PopPtrs<T>& P, const CollideConsts<float>& C,
                                            const Geometry& g, const Item& I, const T* stage, T* out, int x) {
    const int NX = g.NX;
    const int xm1 = (x == 0) ? NX - 1 : x - 1;
    const int xp2 = (x + 2 == NX) ? 0 : x + 2;
    float fa[Q], fb[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const T* r = stage + i * NX;
        const int sh = (ODD && !pull_bb(WALL, i)) ? DXg(i) : 0;   // f_i(x) = row[x - sh]
        if (sh == 0) {
            ld_pair(r + x, fa[i], fb[i]);
        } else if (sh == 1) {
            fa[i] = ld_one(r + xm1); fb[i] = ld_one(r + x);
        } else {
            fa[i] = ld_one(r + x + 1); fb[i] = ld_one(r + xp2);
        }
    }
    float rho, jx, jy, jz;
    collide<float, false>(fa, C, 0.f, 0.f, 0.f, rho, jx, jy, jz);
    collide<float, false>(fb, C, 0.f, 0.f, 0.f, rho, jx, jy, jz);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const bool local = !ODD || push_bb(WALL, i);
        const int sh = local ? 0 : DXg(i);
        T* d;
        if (SOUT) d = out + i * NX;
        else d = local ? P.p[OPPf(i)] + I.row : P.p[i] + row_at(g, I.y + DYg(i), I.z + DZg(i));
        if (sh == 0) {
            st_pair(d + x, fa[i], fb[i]);
        } else if (sh == 1) {
            st_one(d + x + 1, fa[i]); st_one(d + xp2, fb[i]);
        } else {
            st_one(d + xm1, fa[i]); st_one(d + x, fb[i]);
        }
    }
}

template <typename T, bool ODD, bool SOUT>
__global__ void __launch_bounds__(512, 1)
k_step_rows(PopPtrs<T> P, CollideConsts<float> C, Geometry g, int nstage, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t row_bytes = (uint32_t)g.NX * sizeof(T);
    const uint32_t stage_bytes = (uint32_t)Q * row_bytes;
    const uint32_t bars = smem_addr(smem);                 // nstage mbarriers (8 B each)
    const uint32_t data = bars + 128;                       // stage buffers, 16-B aligned
    const uint32_t outs = data + (uint32_t)nstage * stage_bytes;   // 2 output buffers (SOUT)
    T* const stage_ptr0 = reinterpret_cast<T*>(smem + 128);
    T* const out_ptr0 = stage_ptr0 + (size_t)nstage * Q * g.NX;
    const uint32_t total = (uint32_t)g.NY * (uint32_t)g.NZ;
    const uint32_t G = gridDim.x;
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int s = 0; s < nstage; ++s) mbar_init(bars + 8 * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < nstage; ++s) {
            const uint32_t it = blockIdx.x + (uint32_t)s * G;
            if (it < total) issue_item<T, ODD>(P, g, it, data + s * stage_bytes, bars + 8 * s, row_bytes);
        }
    }
    const int npairs = g.NX >> 1;
    uint32_t k = 0;
    for (;; ++k) {
        const uint32_t it = blockIdx.x + k * G;
        if (it >= total) break;
        const int s = (int)(k % (uint32_t)nstage);
        const uint32_t phase = (k / (uint32_t)nstage) & 1u;
        const bool ok = mbar_wait(bars + 8 * s, phase);
        if (__syncthreads_or(!ok)) {
            // a bulk copy did not complete: flag it, drain what is in flight, leave
            if (tid == 0) {
                atomicExch(err, 1);
                // issued so far: items up to k+nstage-2 (k >= 1) or nstage-1 (k == 0)
                const uint32_t last = k == 0 ? (uint32_t)nstage - 1 : k + (uint32_t)nstage - 2;
                for (uint32_t j = k; j <= last; ++j) {
                    if (blockIdx.x + j * G >= total) break;
                    mbar_wait(bars + 8 * (j % nstage), (j / nstage) & 1u);
                }
                if (SOUT) bulk_wait_all();
            }
            return;
        }
        // every thread is past item k-1: its outputs can be written back and its
        // stage refilled
        if (tid == 0 && k >= 1) {
            if (SOUT) store_item<T, ODD>(P, g, it - G, outs + ((k - 1) & 1u) * stage_bytes, row_bytes);
            const uint32_t kk = k - 1 + (uint32_t)nstage;
            const uint32_t nit = blockIdx.x + kk * G;
            const int ps = (int)((k - 1) % (uint32_t)nstage);
            if (nit < total) issue_item<T, ODD>(P, g, nit, data + ps * stage_bytes, bars + 8 * ps, row_bytes);
        }
        const Item I = item_of(g, it);
        const int wall = wall_of(g, I.z);
        const T* stage = stage_ptr0 + (size_t)s * Q * g.NX;
        T* out = SOUT ? out_ptr0 + (size_t)(k & 1u) * Q * g.NX : nullptr;
        for (int p = tid; p < npairs; p += blockDim.x) {
            const int x = 2 * p;
            if (wall == 0)      pair_update<T, ODD, 0, SOUT>(P, C, g, I, stage, out, x);
            else if (wall == 1) pair_update<T, ODD, 1, SOUT>(P, C, g, I, stage, out, x);
            else if (wall == 2) pair_update<T, ODD, 2, SOUT>(P, C, g, I, stage, out, x);
            else                pair_update<T, ODD, 3, SOUT>(P, C, g, I, stage, out, x);
        }
        if (SOUT) {
            // generic-proxy writes to the output buffer must be visible to the
            // bulk store; the buffer written next (item k+1) was read by the
            // store of item k-1, which has to be finished before the barrier
            fence_proxy_async_smem();
            if (tid == 0) bulk_wait_read_all();
        }
    }
    if (SOUT) {
        __syncthreads();
        if (tid == 0 && k >= 1) {
            store_item<T, ODD>(P, g, blockIdx.x + (k - 1) * G, outs + ((k - 1) & 1u) * stage_bytes, row_bytes);
            bulk_wait_all();
        }
    }
}

template <typename T>
PopPtrs<T> pop_ptrs(const DeviceState& s) {
    PopPtrs<T> P;
    T* base = static_cast<T*>(s.f);
    for (int i = 0; i < Q; ++i) P.p[i] = base + (size_t)i * s.pstride;
    return P;
}

constexpr size_t kSmemBudget = 200 * 1024;

// Stage buffers (and output buffers when they fit) for a row of NX elements.
template <typename T>
void plan_for(const Geometry& g, int& nstage, bool& sout) {
    const size_t stage = (size_t)Q * g.NX * sizeof(T);
    const int with_out = (int)((kSmemBudget - 128) / stage) - 2;   // 2 output buffers
    if (with_out >= 3) {
        nstage = with_out > 4 ? 4 : with_out;
        sout = true;
        return;
    }
    const int ns = (int)((kSmemBudget - 128) / stage);
    nstage = ns > 4 ? 4 : ns;
    sout = false;
}

template <typename T>
cudaError_t rows_impl(const DeviceState& s, int parity, int* err, cudaStream_t st) {
    int ns;
    bool sout;
    plan_for<T>(s.g, ns, sout);
    const size_t stage = (size_t)Q * s.g.NX * sizeof(T);
    const size_t smem = 128 + (size_t)(ns + (sout ? 2 : 0)) * stage;
    const int threads = std::min(512, std::max(32, ((s.g.NX / 2 + 31) / 32) * 32));
    const PopPtrs<T> P = pop_ptrs<T>(s);
    const uint32_t total = (uint32_t)s.g.NY * (uint32_t)s.g.NZ;
    const unsigned grid = (unsigned)std::min<uint32_t>(total, (uint32_t)s.sm_count);
    if (sout) {
        if (parity == 0) k_step_rows<T, false, true><<<grid, threads, smem, st>>>(P, s.cf, s.g, ns, err);
        else             k_step_rows<T, true, true><<<grid, threads, smem, st>>>(P, s.cf, s.g, ns, err);
    } else {
        if (parity == 0) k_step_rows<T, false, false><<<grid, threads, smem, st>>>(P, s.cf, s.g, ns, err);
        else             k_step_rows<T, true, false><<<grid, threads, smem, st>>>(P, s.cf, s.g, ns, err);
    }
    return cudaGetLastError();
}

}  // namespace

bool rows_supported(const DeviceState& s) {
    if (s.prec == LBM_PREC_FP64) return false;
    const size_t es = s.prec == LBM_PREC_FP32 ? 4 : 2;
    if ((s.g.NX * es) % 16 != 0 || s.g.NX < 16) return false;          // 16-B bulk copies
    if ((s.pstride * es) % 16 != 0) return false;
    int ns;
    bool sout;
    if (s.prec == LBM_PREC_FP32) plan_for<float>(s.g, ns, sout);
    else plan_for<__half>(s.g, ns, sout);
    return ns >= 2 && s.sm_count > 0;
}

template <typename T>
cudaError_t set_smem_attr() {
    const int b = (int)kSmemBudget;
    cudaError_t e = cudaFuncSetAttribute(k_step_rows<T, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_rows<T, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_rows<T, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_rows<T, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return e;
}

cudaError_t prepare_step_rows() {
    cudaError_t e = set_smem_attr<float>();
    if (e == cudaSuccess) e = set_smem_attr<__half>();
    return e;
}

cudaError_t launch_step_rows(const DeviceState& s, int parity, int* err, cudaStream_t st) {
    if (s.prec == LBM_PREC_FP32) return rows_impl<float>(s, parity, err, st);
    if (s.prec == LBM_PREC_FP16) return rows_impl<__half>(s, parity, err, st);
    return cudaErrorInvalidValue;
}

}  // namespace lbm
