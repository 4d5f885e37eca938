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
// Each persistent CTA owns a ring of NSTAGE stage buffers of 19 rows, each
// with an mbarrier that completes when its 19 bulk copies have landed
// (expect_tx = 19 rows).  There is no CTA-wide barrier in the steady state:
// every warp computes its share of an item (two adjacent nodes per thread)
// and writes the results back into the stage in place -- in the AA pattern
// each node's outputs land exactly on stage positions that the same node
// read, so no other thread is disturbed -- then counts itself done on the
// stage's counter.  The last warp to finish a stage copies its 19 result
// rows back to HBM with bulk stores (lane i: the row slot i came from),
// waits until they have read the stage, and refills it with the item NSTAGE
// ahead.  Warps therefore drift freely up to NSTAGE-1 items apart, both
// directions of HBM traffic are whole-row bulk copies, and the bytes in
// flight are set by shared memory, not by registers.
//
// Every mbarrier wait is bounded.  A wait that gives up raises a CTA-wide
// abort flag and the global error flag (the host then reports the step as
// failed), and that lane waits no more: from then on no stage is refilled,
// so every other lane gives up at its next wait (bounded too), the loop
// runs out on whatever the stages hold, and before the CTA exits one thread
// waits (again bounded) for every stage's last issued load to land, so that
// no bulk copy still targets the CTA's shared memory when it exits.
#include <algorithm>

#include "lbm_f32x2.cuh"
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
// shared -> global bulk copy in this thread's bulk group
__device__ __forceinline__ void bulk_store(void* dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// this thread's bulk stores have finished reading shared memory
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// this thread's bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// generic-proxy shared-memory writes of this thread become visible to the
// async proxy (the bulk copies)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// storage <-> arithmetic helpers for an aligned pair / a single element
__device__ __forceinline__ F2 ld_pair(const __half* p) {
    return F2(__half22float2(*reinterpret_cast<const __half2*>(p)));
}
__device__ __forceinline__ F2 ld_pair(const float* p) { return F2(*reinterpret_cast<const float2*>(p)); }
__device__ __forceinline__ float ld_one(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float ld_one(const float* p) { return *p; }
__device__ __forceinline__ void st_pair(__half* p, F2 v) {
    *reinterpret_cast<__half2*>(p) = __float22half2_rn(v.v);
}
__device__ __forceinline__ void st_pair(float* p, F2 v) { *reinterpret_cast<float2*>(p) = v.v; }
__device__ __forceinline__ void st_one(__half* p, float a) { *p = __float2half_rn(a); }
__device__ __forceinline__ void st_one(float* p, float a) { *p = a; }

// Lattice lookups with a runtime population index (one lane per population
// when issuing bulk copies): values packed into 64-bit words at compile time.
constexpr uint64_t pack2(int (*f)(int)) {
    uint64_t w = 0;
    for (int i = 0; i < Q; ++i) w |= (uint64_t)(f(i) + 1) << (2 * i);
    return w;
}
constexpr int dy_c(int i) { return DYg(i); }
constexpr int dz_c(int i) { return DZg(i); }
constexpr uint64_t kDY = pack2(dy_c), kDZ = pack2(dz_c);
constexpr uint64_t pack_opp_lo() {
    uint64_t w = 0;
    for (int i = 0; i < 12; ++i) w |= (uint64_t)OPPf(i) << (5 * i);
    return w;
}
constexpr uint64_t pack_opp_hi() {
    uint64_t w = 0;
    for (int i = 12; i < Q; ++i) w |= (uint64_t)OPPf(i) << (5 * (i - 12));
    return w;
}
constexpr uint64_t kOPPlo = pack_opp_lo(), kOPPhi = pack_opp_hi();
__device__ __forceinline__ int dy_rt(int i) { return (int)((kDY >> (2 * i)) & 3u) - 1; }
__device__ __forceinline__ int dz_rt(int i) { return (int)((kDZ >> (2 * i)) & 3u) - 1; }
__device__ __forceinline__ int opp_rt(int i) {
    return i < 12 ? (int)((kOPPlo >> (5 * i)) & 31u) : (int)((kOPPhi >> (5 * (i - 12))) & 31u);
}

struct Item {
    int y, z;
    uint32_t row;                  // NX*(y + NY*z)
};
// item it: rows y .. y + K - 1 (y a multiple of K) at wall-normal z
template <int K>
__device__ __forceinline__ Item item_of(const Geometry& g, uint32_t it) {
    Item I;
    const uint32_t ny = (uint32_t)g.NY / K;
    I.y = K * (int)(it % ny);
    I.z = (int)(it / ny);
    I.row = (uint32_t)g.NX * ((uint32_t)I.y + (uint32_t)g.NY * (uint32_t)I.z);
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

// Source row of population i for an item (runtime i).  In the
// bounds-checked build a plane or row outside the lattice is reported at
// `site` and replaced by row 0 of plane 0 (the results are then invalid and
// the call fails).
template <typename T, bool ODD>
__device__ __forceinline__ const T* src_row(const PopPtrs<T>& P, const Geometry& g, const Item& I, int wall, int i,
                                            int r, unsigned* bflag, unsigned site) {
    const int dz = dz_rt(i);
    const bool bb = (dz == 1 && (wall & 1)) || (dz == -1 && (wall & 2));
#ifdef LBM_BOUNDS_CHECK
    int k = i;
    uint32_t row = I.row + (uint32_t)r * (uint32_t)g.NX;
    if (ODD && !bb) {
        k = opp_rt(i);
        row = row_at(g, I.y + r - dy_rt(i), I.z - dz);
    }
    if (!LBM_IN_BOUNDS(bflag, k >= 0 && k < Q && I.y + r < g.NY && row % (uint32_t)g.NX == 0 &&
                                  (size_t)row + g.NX <= (size_t)g.NXY * g.NZ, site))
        return P.p[0];
    return P.p[k] + row;
#else
    (void)bflag;
    (void)site;
    if (!ODD || bb) return P.p[i] + I.row + (uint32_t)r * (uint32_t)g.NX;
    return P.p[opp_rt(i)] + row_at(g, I.y + r - dy_rt(i), I.z - dz);
#endif
}
// Issued by one warp: lane i moves population i's row.  The mbarrier learns the
// byte count from lane 0 before any copy is issued.
// `issued` (a register of the issuing warp) records the loads this warp put
// into stage s for the drain on abort: bit s flips per load (the count's
// parity), bit 8 + s is set once one was issued.
// With K = 2 the slot holds the item's two rows of population i, one bulk
// copy when their source rows are adjacent in memory, two when the
// periodic y wrap separates them.
template <typename T, bool ODD, int K>
__device__ __forceinline__ void issue_item(const PopPtrs<T>& P, const Geometry& g, uint32_t it, uint32_t stage_smem,
                                           uint32_t bar, uint32_t row_bytes, int lane, int s, unsigned& issued,
                                           unsigned* bflag) {
    if (lane == 0) mbar_expect_tx(bar, (uint32_t)(Q * K) * row_bytes);
    __syncwarp();
    if (lane < Q) {
        const Item I = item_of<K>(g, it);
        const int wall = wall_of(g, I.z);
        const uint32_t dst = stage_smem + (uint32_t)(lane * K) * row_bytes;
        const T* s0 = src_row<T, ODD>(P, g, I, wall, lane, 0, bflag, 301);
        if constexpr (K == 1) {
            bulk_load(dst, s0, row_bytes, bar);
        } else {
            const T* s1 = src_row<T, ODD>(P, g, I, wall, lane, 1, bflag, 301);
            if (s1 == s0 + g.NX) {
                bulk_load(dst, s0, 2 * row_bytes, bar);
            } else {
                bulk_load(dst, s0, row_bytes, bar);
                bulk_load(dst + row_bytes, s1, row_bytes, bar);
            }
        }
    }
    issued = (issued ^ (1u << s)) | (1u << (8 + s));
}

// Two adjacent nodes (x, x+1), x even, of one item; the results go back into
// the stage buffer.  Output population i belongs in the row that stage slot
// opp(i) was loaded from (even step: plane opp(i) of this row; odd step:
// plane i of row (Y,Z)+c_i, the source row of slot opp(i); at a wall the
// bounced population stays in this row, which is again slot opp(i)), at the
// position x + c_ix (x at a wall and in the even step), from which the same
// node read slot opp(i).  Every thread therefore overwrites only stage
// positions that it has read itself, and the finished stage holds the item's
// results row for row, to be copied back to the addresses it was loaded from.
// F2 holds the pair's populations (node x, node x+1).  The FP16 odd step
// relaxes both nodes with packed FP32 instructions (C2): its x-shifted
// populations cost single-element shared-memory accesses, which leave it
// bound by instruction issue, and the packed collision halves the
// floating-point instructions (3.69 -> 3.39 ms per launch on the large
// channel).  The memory-bound kernels (FP16 even, FP32) keep the scalar
// collision per node (C), which measured 0.4% (FP16 even) and 1.7% (FP32)
// faster than the packed one.
template <typename T, bool ODD, int WALL, bool YF>
__device__ __forceinline__ void pair_update(const CollideConsts<float>& C, const CollideConsts<F2>& C2,
                                            const Geometry& g, T* stage, int ss, int x) {
    constexpr bool kPacked = ODD && sizeof(T) == 2;
    const int NX = g.NX;
    const int xm1 = (x == 0) ? NX - 1 : x - 1;
    const int xp2 = (x + 2 == NX) ? 0 : x + 2;
    F2 f[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const T* r = stage + i * ss;
        const int sh = (ODD && !pull_bb(WALL, i)) ? DXg(i) : 0;   // f_i(x) = row[x - sh]
        if (sh == 0) f[i] = ld_pair(r + x);
        else if (sh == 1) f[i] = F2(ld_one(r + xm1), ld_one(r + x));
        else f[i] = F2(ld_one(r + x + 1), ld_one(r + xp2));
    }
    if constexpr (kPacked) {
        F2 rho, jx, jy, jz;
        collide<F2, false, YF>(f, C2, F2(0.f), F2(0.f), F2(0.f), rho, jx, jy, jz);
    } else {
        float fa[Q], fb[Q], rho, jx, jy, jz;
#pragma unroll
        for (int i = 0; i < Q; ++i) { fa[i] = f[i].v.x; fb[i] = f[i].v.y; }
        collide<float, false, YF>(fa, C, 0.f, 0.f, 0.f, rho, jx, jy, jz);
        collide<float, false, YF>(fb, C, 0.f, 0.f, 0.f, rho, jx, jy, jz);
#pragma unroll
        for (int i = 0; i < Q; ++i) f[i] = F2(fa[i], fb[i]);
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const int sh = (ODD && !push_bb(WALL, i)) ? DXg(i) : 0;
        T* d = stage + OPPf(i) * ss;
        if (sh == 0) {
            st_pair(d + x, f[i]);
        } else if (sh == 1) {
            st_one(d + x + 1, f[i].v.x); st_one(d + xp2, f[i].v.y);
        } else {
            st_one(d + xm1, f[i].v.x); st_one(d + x, f[i].v.y);
        }
    }
}

// All pairs of an item handled by this thread; the wall case is fixed for
// the whole loop.
// pair p of the item: row p / (NX / 2) of its K rows, nodes 2 (p mod NX/2)
// and the next; slot i of the stage holds population i's K rows
template <typename T, bool ODD, int WALL, bool YF, int K>
__device__ __forceinline__ void item_pairs(const CollideConsts<float>& C, const CollideConsts<F2>& C2,
                                           const Geometry& g, T* stage, int tid, int nthreads, unsigned* bflag) {
    const int half = g.NX >> 1;
    const int npairs = K * half;
    for (int p = tid; p < npairs; p += nthreads) {
        const int rk = (K == 1 || p < half) ? 0 : 1;
        const int x = 2 * (p - rk * half);
        if (LBM_IN_BOUNDS(bflag, x + 1 < g.NX && (g.NX & 1) == 0, 303))
            pair_update<T, ODD, WALL, YF>(C, C2, g, stage + rk * g.NX, K * g.NX, x);
    }
}

// Issued by the last warp to finish an item: lane i copies result row i back
// to the row that slot i was loaded from, then waits until the copy has read
// the stage (the stage is refilled next).
template <typename T, bool ODD, int K>
__device__ __forceinline__ void store_item(const PopPtrs<T>& P, const Geometry& g, uint32_t it, uint32_t stage_smem,
                                           uint32_t row_bytes, int lane, unsigned* bflag) {
    if (lane < Q) {
        const Item I = item_of<K>(g, it);
        const int wall = wall_of(g, I.z);
        const uint32_t src = stage_smem + (uint32_t)(lane * K) * row_bytes;
        T* d0 = const_cast<T*>(src_row<T, ODD>(P, g, I, wall, lane, 0, bflag, 302));
        if constexpr (K == 1) {
            bulk_store(d0, src, row_bytes);
        } else {
            T* d1 = const_cast<T*>(src_row<T, ODD>(P, g, I, wall, lane, 1, bflag, 302));
            if (d1 == d0 + g.NX) {
                bulk_store(d0, src, 2 * row_bytes);
            } else {
                bulk_store(d0, src, row_bytes);
                bulk_store(d1, src + row_bytes, row_bytes);
            }
        }
        bulk_wait_read();
    }
    __syncwarp();
}

constexpr int kMaxStages = 5;

template <typename T, bool ODD, bool YF, int NT, int K>
__global__ void __launch_bounds__(NT, 512 / NT)
k_step_rows(PopPtrs<T> P, CollideConsts<float> C, CollideConsts<F2> C2, Geometry g, int nstage, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ unsigned int done_count[kMaxStages];
    __shared__ unsigned int issued_par, issued_any;
    __shared__ volatile int abort_flag;
    const uint32_t row_bytes = (uint32_t)g.NX * sizeof(T);
    const uint32_t stage_bytes = (uint32_t)(Q * K) * row_bytes;
    const uint32_t bars = smem_addr(smem);                 // nstage mbarriers (8 B each)
    const uint32_t data = bars + 128;                       // stage buffers, 16-B aligned
    T* const stage_ptr0 = reinterpret_cast<T*>(smem + 128);
    const uint32_t total = (uint32_t)g.NY / K * (uint32_t)g.NZ;
    const uint32_t G = gridDim.x;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const unsigned nwarps = NT / 32;
    unsigned* const bflag = reinterpret_cast<unsigned*>(err + 1);   // bounds-check site (checked build)
    (void)bflag;
    unsigned issued = 0;                                   // loads this warp issued, per stage

    if (tid == 0) {
        for (int s = 0; s < nstage; ++s) {
            mbar_init(bars + 8 * s, 1);
            done_count[s] = 0;
        }
        abort_flag = 0;
        issued_par = issued_any = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid < 32) {
        for (int s = 0; s < nstage; ++s) {
            const uint32_t it = blockIdx.x + (uint32_t)s * G;
            if (it < total)
                issue_item<T, ODD, K>(P, g, it, data + s * stage_bytes, bars + 8 * s, row_bytes, lane, s, issued,
                                   bflag);
        }
    }
    bool failed = false;
    for (uint32_t k = 0;; ++k) {
        const uint32_t it = blockIdx.x + k * G;
        if (it >= total) break;
        const int s = (int)(k % (uint32_t)nstage);
        // A lane whose wait gave up raises the abort flag and waits no more
        // (it computes on whatever the stages hold; the step is reported as
        // failed).  No stage is refilled after an abort, so every other lane
        // gives up at its next wait, bounded as well.  All lanes keep running
        // the same instructions, so the warp-wide shuffles stay complete.
        if (!failed && !mbar_wait(bars + 8 * s, (k / (uint32_t)nstage) & 1u)) {
            failed = true;
            abort_flag = 1;
        }
        const Item I = item_of<K>(g, it);
        const int wall = wall_of(g, I.z);
        T* stage = stage_ptr0 + (size_t)s * (Q * K) * g.NX;
        if (wall == 0)      item_pairs<T, ODD, 0, YF, K>(C, C2, g, stage, tid, NT, bflag);
        else if (wall == 1) item_pairs<T, ODD, 1, YF, K>(C, C2, g, stage, tid, NT, bflag);
        else if (wall == 2) item_pairs<T, ODD, 2, YF, K>(C, C2, g, stage, tid, NT, bflag);
        else                item_pairs<T, ODD, 3, YF, K>(C, C2, g, stage, tid, NT, bflag);
        // this warp has finished with stage s; the last warp copies the
        // results back and refills it
        fence_proxy_async();
        __syncwarp();
        unsigned last = 0;
        if (lane == 0) {
            __threadfence_block();
            last = atomicAdd(&done_count[s], 1u) == nwarps - 1;
            if (last) done_count[s] = 0;
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (last) {
            __threadfence_block();
            fence_proxy_async();
            // every warp has passed this stage's wait, so its load had landed:
            // storing it is safe even after an abort elsewhere; only the
            // refill is withheld then
            const int ab = abort_flag;
            store_item<T, ODD, K>(P, g, it, data + s * stage_bytes, row_bytes, lane, bflag);
            const uint32_t nit = blockIdx.x + (k + (uint32_t)nstage) * G;
            if (nit < total && !ab)
                issue_item<T, ODD, K>(P, g, nit, data + s * stage_bytes, bars + 8 * s, row_bytes, lane, s, issued,
                                   bflag);
        }
    }
    bulk_wait_all();
    if (lane == 0 && issued) {          // unconditionally: an abort may come later
        atomicXor(&issued_par, issued & 0xffu);
        atomicOr(&issued_any, issued >> 8);
    }
    __syncthreads();
    if (abort_flag && tid == 0) {
        // drain: with n loads issued into a stage in all, the latest completes
        // the phase with parity (n - 1) & 1; earlier phases have completed
        // before it (a stage is refilled only after every warp consumed it)
        for (int s = 0; s < nstage; ++s)
            if ((issued_any >> s) & 1u) (void)mbar_wait(bars + 8 * s, ((issued_par >> s) & 1u) ^ 1u);
        atomicExch(err, 1);
    }
}

template <typename T>
PopPtrs<T> pop_ptrs(const DeviceState& s) {
    PopPtrs<T> P;
    T* base = static_cast<T*>(s.f);
    for (int i = 0; i < Q; ++i) P.p[i] = base + (size_t)i * s.pstride;
    return P;
}

constexpr size_t kSmemPerSM = 224 * 1024;    // dynamic shared memory planned per SM

// Launch shape of the row kernels for a row of NX elements of T: two CTAs
// of 256 threads per SM whenever two stages per CTA fit, else one CTA of 512
// threads (rows of more than ~1.4 K FP16 or ~700 FP32 nodes).  Two CTAs keep
// twice the items in flight; with one CTA of 512 threads a row of up to 512
// pairs leaves threads idle in every item (the 512x256x256 channel ran at 32
// GLUPS in FP16 and 32 in FP32 that way, 54 and 42 with two CTAs).  Rows
// of up to 512 nodes with an even spanwise count are taken two per item
// (k = 2) when two CTAs with two such stages fit: an item of one short row
// gives a thread one pair, too little work between the item's waits.
struct RowPlan { int threads, ctas_per_sm, nstage, k; size_t smem; };

template <typename T>
RowPlan plan_rows(const Geometry& g) {
    const size_t stage1 = (size_t)Q * g.NX * sizeof(T);
    RowPlan r;
    r.k = (g.NX <= 512 && (g.NY & 1) == 0 && 2 * (128 + 2 * 2 * stage1) <= kSmemPerSM) ? 2 : 1;
    const size_t stage = (size_t)r.k * stage1;
    if (2 * (128 + 2 * stage) <= kSmemPerSM) {
        r.threads = 256;
        r.ctas_per_sm = 2;
    } else {
        r.threads = 512;
        r.ctas_per_sm = 1;
    }
    int ns = (int)((kSmemPerSM / r.ctas_per_sm - 128) / stage);
    r.nstage = ns > kMaxStages ? kMaxStages : ns;
    r.smem = 128 + (size_t)r.nstage * stage;
    return r;
}

// the FP32 collision constants, each duplicated into both lanes
CollideConsts<F2> pair_consts(const CollideConsts<float>& c) {
    CollideConsts<F2> r;
    r.S = c.S; r.invS = c.invS;
    r.Fx = c.Fx; r.Fy = c.Fy; r.Fz = c.Fz;
    r.hFx = c.hFx; r.hFy = c.hFy; r.hFz = c.hFz;
    r.ajx = c.ajx; r.ajy = c.ajy; r.ajz = c.ajz;
    r.fqx = c.fqx; r.fqy = c.fqy; r.fqz = c.fqz;
    r.thFx = c.thFx; r.thFy = c.thFy; r.thFz = c.thFz;
    r.ke = c.ke; r.keps = c.keps; r.kq = c.kq; r.kp = c.kp; r.kpi = c.kpi; r.kxy = c.kxy; r.km = c.km;
    r.kw = c.kw; r.kwi = c.kwi;
    r.oeps = c.oeps; r.oepsj = c.oepsj; r.oxx = c.oxx;
    return r;
}

template <typename T, bool YF, int NT, int K>
void launch_rows_nt(const DeviceState& s, const PopPtrs<T>& P, int parity, int* err, const RowPlan& r,
                    unsigned grid, cudaStream_t st) {
    const CollideConsts<F2> c2 = pair_consts(s.cf);
    if (parity == 0) k_step_rows<T, false, YF, NT, K><<<grid, NT, r.smem, st>>>(P, s.cf, c2, s.g, r.nstage, err);
    else             k_step_rows<T, true, YF, NT, K><<<grid, NT, r.smem, st>>>(P, s.cf, c2, s.g, r.nstage, err);
}

template <typename T>
cudaError_t rows_impl(const DeviceState& s, int parity, int* err, cudaStream_t st) {
    const RowPlan r = plan_rows<T>(s.g);
    const PopPtrs<T> P = pop_ptrs<T>(s);
    const uint32_t total = (uint32_t)s.g.NY / (uint32_t)r.k * (uint32_t)s.g.NZ;
    const unsigned grid = (unsigned)std::min<uint32_t>(total, (uint32_t)(s.sm_count * r.ctas_per_sm));
    const bool yf = s.cf.Fx == 0.0f && s.cf.Fz == 0.0f;
    if (r.threads == 256 && r.k == 2) {
        if (yf) launch_rows_nt<T, true, 256, 2>(s, P, parity, err, r, grid, st);
        else    launch_rows_nt<T, false, 256, 2>(s, P, parity, err, r, grid, st);
    } else if (r.threads == 256) {
        if (yf) launch_rows_nt<T, true, 256, 1>(s, P, parity, err, r, grid, st);
        else    launch_rows_nt<T, false, 256, 1>(s, P, parity, err, r, grid, st);
    } else {
        if (yf) launch_rows_nt<T, true, 512, 1>(s, P, parity, err, r, grid, st);
        else    launch_rows_nt<T, false, 512, 1>(s, P, parity, err, r, grid, st);
    }
    return cudaGetLastError();
}

template <typename T, bool YF, int NT, int K>
cudaError_t set_attr_nt() {
    const int b = (int)(kSmemPerSM / (512 / NT));
    cudaError_t e = cudaFuncSetAttribute(k_step_rows<T, false, YF, NT, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_rows<T, true, YF, NT, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return e;
}

template <typename T>
cudaError_t set_smem_attr() {
    cudaError_t e = set_attr_nt<T, false, 512, 1>();
    if (e == cudaSuccess) e = set_attr_nt<T, true, 512, 1>();
    if (e == cudaSuccess) e = set_attr_nt<T, false, 256, 1>();
    if (e == cudaSuccess) e = set_attr_nt<T, true, 256, 1>();
    if (e == cudaSuccess) e = set_attr_nt<T, false, 256, 2>();
    if (e == cudaSuccess) e = set_attr_nt<T, true, 256, 2>();
    return e;
}

}  // namespace

bool rows_supported(const DeviceState& s) {
    if (s.prec == LBM_PREC_FP64) return false;
    const size_t es = s.prec == LBM_PREC_FP32 ? 4 : 2;
    if ((s.g.NX * es) % 16 != 0 || s.g.NX < 16) return false;          // 16-B bulk copies
    if ((s.pstride * es) % 16 != 0) return false;
    const RowPlan r = s.prec == LBM_PREC_FP32 ? plan_rows<float>(s.g) : plan_rows<__half>(s.g);
    return r.nstage >= 2 && s.sm_count > 0;
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
