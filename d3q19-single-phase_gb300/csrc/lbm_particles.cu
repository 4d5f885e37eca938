// Moving spheres: geometry, interpolated bounce-back with momentum exchange,
// Newton-Euler and refilling, run after every fluid step.
//
// The reference declares the particle data (links, fill lists, particle state:
// var_inc.f90:120-150, para.f90:332-379; solid-node velocity in macrovar,
// collision.f90:420-458) but its particle library is not in the source tree.
// The algorithm here is this project's own (see the oracle's statement of the
// same steps):
//  1. the fluid step collides and streams every node, solid ones included;
//  2. k_ibb, one CTA per sphere: every link (fluid x_f, direction c_i into the
//     sphere) gets the population coming back from the wall by interpolated
//     bounce-back (Bouzidi, Firdaouss & Lallemand 2001: quadratic for q < 1/2,
//     linear for q >= 1/2) with the moving-wall term, read and written
//     through the AA orientation of the
//     step just taken; the momentum exchanged (Galilean-invariant form, Wen et
//     al. 2014) is reduced per sphere with warp shuffles into FP64 force and
//     torque;
//  3. k_bin + k_repulsion_cells (a cell list; k_repulsion, all pairs, for
//     small domains): soft-sphere repulsion summed in sphere-index order, on
//     the context's second stream while k_ibb runs (it needs only the
//     positions); k_newton, one thread per sphere, after both: the FP64
//     Newton-Euler update
//     (average of this step's and the previous step's force and torque);
//  4. k_shell<release>, then k_shell<claim>: node ownership follows the new
//     positions along the thin shell swept by each surface; nodes that leave
//     a sphere are queued;
//  5. k_refill: queued nodes get the equilibrium at the wall velocity plus the
//     non-equilibrium part of the fluid neighbour closest to the outward
//     normal.
// Geometry decisions (inside tests, q, the refill direction) use explicit
// round-to-nearest FP64 operations so that they agree bit for bit with the
// CPU oracle.
#include <algorithm>
#include <cmath>

#include "lbm_internal.h"

namespace lbm {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInvSqrt2 = 0.70710678118654752440;
constexpr int kPThreads = 256;

// Lattice lookups with a runtime direction index, packed into 64-bit words at
// compile time (a constexpr table indexed at run time would live in local
// memory).
constexpr uint64_t pack_c(int which) {
    uint64_t w = 0;
    for (int i = 0; i < Q; ++i) {
        const int v = which == 0 ? CXf(i) : (which == 1 ? CYf(i) : CZf(i));
        w |= (uint64_t)(v + 1) << (2 * i);
    }
    return w;
}
constexpr uint64_t kCX = pack_c(0), kCY = pack_c(1), kCZ = pack_c(2);
constexpr uint64_t pack_opp(int lo) {
    uint64_t w = 0;
    for (int i = lo; i < lo + 12 && i < Q; ++i) w |= (uint64_t)OPPf(i) << (5 * (i - lo));
    return w;
}
constexpr uint64_t kOPP0 = pack_opp(0), kOPP1 = pack_opp(12);
__device__ __forceinline__ int cx_rt(int i) { return (int)((kCX >> (2 * i)) & 3u) - 1; }
__device__ __forceinline__ int cy_rt(int i) { return (int)((kCY >> (2 * i)) & 3u) - 1; }
__device__ __forceinline__ int cz_rt(int i) { return (int)((kCZ >> (2 * i)) & 3u) - 1; }
__device__ __forceinline__ int opp_rt(int i) {
    return i < 12 ? (int)((kOPP0 >> (5 * i)) & 31u) : (int)((kOPP1 >> (5 * (i - 12))) & 31u);
}
__device__ __forceinline__ double w_rt(int i) { return i == 0 ? W0 : (i <= 6 ? W1 : W2); }

__device__ __forceinline__ double dmin_image(double d, double L) {
    if (d >= 0.5 * L) d = __dsub_rn(d, L);
    else if (d < -0.5 * L) d = __dadd_rn(d, L);
    return d;
}

// offset from the centre of sphere p to the node with reference indices
// (ix, iy, iz) (0-based)
__device__ __forceinline__ void offset(const DeviceParticles& P, const Geometry& g, int p, int ix, int iy, int iz,
                                       double d[3]) {
    d[0] = __dsub_rn((double)ix + 0.5, P.pos[3 * p + 0]);
    d[1] = dmin_image(__dsub_rn((double)iy + 0.5, P.pos[3 * p + 1]), (double)g.NX);
    d[2] = dmin_image(__dsub_rn((double)iz + 0.5, P.pos[3 * p + 2]), (double)g.NY);
}
__device__ __forceinline__ double norm2_rn(const double d[3]) {
    return __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
}
__device__ __forceinline__ bool inside(const double d[3], double R) { return norm2_rn(d) <= __dmul_rn(R, R); }

// periodic wrap of an index within one period of [0, n) (all callers stay
// within [-n, 2n): box edges and stencils reach at most R + 3 nodes out)
__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

struct Range { int lo, n; };

// Node range of a bounding box along one axis from the geometry record:
// nodes whose centres lie within ext of the sphere centre, plus any node
// within FP32 rounding of that (callers pass a margin in ext).
__device__ __forceinline__ Range box_g(int ci, float h, float ext, int n, bool periodic) {
    int a = ci + (int)floorf(-h - ext);
    int b = ci + (int)ceilf(ext - h);
    if (!periodic) {
        if (a < 0) a = 0;
        if (b > n - 1) b = n - 1;
    }
    Range r;
    r.lo = a;
    r.n = b >= a ? b - a + 1 : 0;
    return r;
}

// GPU node index of reference indices (ix wall-normal, iy streamwise, iz spanwise)
__device__ __forceinline__ uint32_t gnode(const Geometry& g, int ix, int iy, int iz) {
    return (uint32_t)iy + (uint32_t)g.NX * ((uint32_t)iz + (uint32_t)g.NY * (uint32_t)ix);
}

template <typename T>
__device__ __forceinline__ T* plane(const DeviceState& s, int k) {
    return static_cast<T*>(s.f) + (size_t)k * s.pstride;
}

// Storage location of the natural post-stream population k at reference node
// (ix,iy,iz): parity 0 -> slot k there; parity 1 (after an even AA step) ->
// slot opp(k) at the node - c_k, or slot k there when that is beyond a wall.
struct Slot { int k; uint32_t n; };
__device__ __forceinline__ Slot natural_slot(const Geometry& g, int parity, int k, int ix, int iy, int iz) {
    Slot s;
    s.k = k;
    s.n = gnode(g, ix, iy, iz);
    if (parity) {
        const int sx = ix - cx_rt(k);
        if (sx >= 0 && sx < g.NZ) {
            s.k = opp_rt(k);
            s.n = gnode(g, sx, wrapi(iy - cy_rt(k), g.NX), wrapi(iz - cz_rt(k), g.NY));
        }
    }
    return s;
}
// Same in the link arithmetic type RT (no FP64 conversions for FP32/FP16).
template <typename T, typename RT>
__device__ __forceinline__ RT read_nat_r(const DeviceState& s, int parity, int k, int ix, int iy, int iz) {
    const Slot sl = natural_slot(s.g, parity, k, ix, iy, iz);
    if constexpr (sizeof(RT) == 8) return (double)ld_pop(plane<T>(s, sl.k) + sl.n) * s.cd.invS;
    else return (float)ld_pop(plane<T>(s, sl.k) + sl.n) * s.cf.invS;
}
template <typename T, typename RT>
__device__ __forceinline__ void write_nat_r(const DeviceState& s, int parity, int k, int ix, int iy, int iz, RT v) {
    const Slot sl = natural_slot(s.g, parity, k, ix, iy, iz);
    T* p = plane<T>(s, sl.k) + sl.n;
    if constexpr (sizeof(T) == 8) *p = (double)v * s.cd.S;
    else if constexpr (sizeof(RT) == 8) st_pop(p, (float)(v * s.cd.S));
    else st_pop(p, v * s.cf.S);
}

// population at a storage address, in the link arithmetic type RT
template <typename T, typename RT>
__device__ __forceinline__ RT pop_r(const DeviceState& s, const T* a) {
    if constexpr (sizeof(RT) == 8) return (double)ld_pop(a) * s.cd.invS;
    else return (float)ld_pop(a) * s.cf.invS;
}
template <typename T, typename RT>
__device__ __forceinline__ void put_r(const DeviceState& s, T* a, RT v) {
    if constexpr (sizeof(T) == 8) *a = (double)v * s.cd.S;
    else if constexpr (sizeof(RT) == 8) st_pop(a, (float)(v * s.cd.S));
    else st_pop(a, v * s.cf.S);
}

template <typename T>
__device__ __forceinline__ double read_nat(const DeviceState& s, int parity, int k, int ix, int iy, int iz) {
    const Slot sl = natural_slot(s.g, parity, k, ix, iy, iz);
    return (double)ld_pop(plane<T>(s, sl.k) + sl.n) * s.cd.invS;
}
template <typename T>
__device__ __forceinline__ void write_nat(const DeviceState& s, int parity, int k, int ix, int iy, int iz, double v) {
    const Slot sl = natural_slot(s.g, parity, k, ix, iy, iz);
    T* p = plane<T>(s, sl.k) + sl.n;
    if constexpr (sizeof(T) == 8) *p = v * s.cd.S;
    else st_pop(p, (float)(v * s.cd.S));
}

// ---------------------------------------------------------------------------
// Ownership update along the thin shell swept by a sphere surface.  A node
// owned by sphere p lies inside p's previous position, so within R + delta of
// the new centre (delta: displacement of this step), and a node at less than
// R - delta from the new centre was inside the previous sphere and is owned
// already.  One warp per sphere; lane j takes (spanwise, wall-normal) rows of
// the bounding box, intersects each row with that shell in FP32 (with a
// margin far above the FP32 error) and decides the few nodes found by their
// FP32 squared distance, or by the exact FP64 test of the oracle where that
// lies within in_band() of R^2.  `full` claims every node inside (placement).
// Claims take the highest sphere index (atomicMax), the oracle's outcome of
// claiming in index order where spheres overlap; nodes that a sphere released
// inside another one are claimed by k_reclaim.
constexpr int kShellWarps = 4;
constexpr float kShellEps = 0.01f;

// FP32 squared distance error bound: node offsets are an exact integer plus
// the FP32 fraction of the geometry record (error <= 2^-24 |d| + 2^-25 per
// axis for |d| < 64), so |r2_f32 - r2| < 6e-7 r2 + 1e-5; the band is wider.
__device__ __forceinline__ float in_band(float R2) { return 1e-5f * R2 + 1e-3f; }

template <bool CLAIM>
__global__ void __launch_bounds__(32 * kShellWarps) k_shell(DeviceParticles P, Geometry g, int* owner, int full,
                                                            unsigned* bflag) {
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * kShellWarps + (threadIdx.x >> 5);
    if (p >= P.npart) return;                       // whole warps leave together
    const SphereGeom G = P.geom[p];
    const float delta = full ? 0.f : G.delta;
    const float Rf = P.Rf, R2 = Rf * Rf, band = in_band(R2);
    float r_in, r_out;
    if (CLAIM) {
        r_in = full ? -1.f : Rf - delta - kShellEps;
        r_out = Rf + kShellEps;
    } else {
        r_in = Rf - kShellEps;
        r_out = Rf + delta + kShellEps;
    }
    const float ext = r_out + 1.f;
    const Range rx = box_g(G.ci[0], G.h[0], ext, g.NZ, false);
    const Range ry = box_g(G.ci[1], G.h[1], ext, g.NX, true);
    const Range rz = box_g(G.ci[2], G.h[2], ext, g.NY, true);
    const float yl0 = (float)(ry.lo - G.ci[1]) + G.h[1];    // offset of row node a = 0
    const float ro2 = r_out * r_out, ri2 = r_in > 0.f ? r_in * r_in : -1.f;
    const int nrows = rz.n * rx.n;
    if (nrows <= 0) return;
    // rows b + rz.n * c, lane-strided without a division per row
    int b = lane % rz.n, c = lane / rz.n;
    const int sb = 32 % rz.n, sc = 32 / rz.n;
    for (int r = lane; r < nrows; r += 32) {
        const float oz = (float)(rz.lo + b - G.ci[2]) + G.h[2], ox = (float)(rx.lo + c - G.ci[0]) + G.h[0];
        const float rho2 = oz * oz + ox * ox;
        if (rho2 <= ro2) {
            const float hi = sqrtf(ro2 - rho2);
            const float lo = rho2 < ri2 ? sqrtf(ri2 - rho2) : -1.f;
            const int ix = rx.lo + c, iz = wrapi(rz.lo + b, g.NY);
            // row nodes with |y| in [lo, hi]: one segment, or two around the hole
            int s0[2], s1[2];
            if (lo < 0.f) {
                s0[0] = (int)ceilf(-hi - yl0); s1[0] = (int)floorf(hi - yl0);
                s0[1] = 0; s1[1] = -1;
            } else {
                s0[0] = (int)ceilf(-hi - yl0); s1[0] = (int)floorf(-lo - yl0);
                s0[1] = (int)ceilf(lo - yl0); s1[1] = (int)floorf(hi - yl0);
            }
            for (int k = 0; k < 2; ++k) {
                const int a0 = max(s0[k], 0), a1 = min(s1[k], ry.n - 1);
                for (int a = a0; a <= a1; ++a) {
                    const float oy = (float)(ry.lo + a - G.ci[1]) + G.h[1];
                    const float r2 = rho2 + oy * oy;
                    const int iy = wrapi(ry.lo + a, g.NX);
                    bool in;
                    if (r2 < R2 - band) in = true;
                    else if (r2 > R2 + band) in = false;
                    else {
                        double d[3];
                        offset(P, g, p, ix, iy, iz, d);
                        in = inside(d, P.R);
                    }
                    const uint32_t n = gnode(g, ix, iy, iz);
                    if (!LBM_IN_BOUNDS(bflag, ix >= 0 && ix < g.NZ && n < g.NXY * (uint32_t)g.NZ, 201)) continue;
                    if (CLAIM) {
                        if (in) atomicMax(owner + n, p);        // the highest index among overlapping spheres
                    } else if (!in && owner[n] == p) {
                        owner[n] = -2;
                        const unsigned q = atomicAdd(&P.counters[0], 1u);
                        if (q < (unsigned)P.refill_cap) {
                            P.refill_node[q] = n;
                            P.refill_part[q] = p;
                        } else {
                            atomicOr(&P.counters[3], 1u);      // refill list overflow
                        }
                    }
                }
            }
        }
        b += sb;
        c += sc;
        if (b >= rz.n) { b -= rz.n; ++c; }
    }
}

// Interpolated bounce-back on every link of sphere blockIdx.x, after a step
// that left the populations in orientation `parity`.  RT: link arithmetic and
// q (FP64 for FP64 storage; FP32 for FP32/FP16 storage, where an FP64 q per
// link would cost more than the fluid step at GB300's FP64 rate), node
// offsets always from FP64 positions, force and torque sums of FP64 accuracy
// per thread and FP64 per sphere.
// qc = |d|^2 - R^2 of the node, computed once per node in FP64
template <typename RT>
__device__ __forceinline__ RT link_q(const double d[3], int cx, int cy, int cz, double qc) {
    if constexpr (sizeof(RT) == 8) {
        const double qa = (double)(cx * cx + cy * cy + cz * cz);
        const double qb = __dadd_rn(__dadd_rn(d[0] * cx, d[1] * cy), d[2] * cz);
        double disc = __dsub_rn(__dmul_rn(qb, qb), __dmul_rn(qa, qc));
        if (disc < 0.0) disc = 0.0;
        double q = __ddiv_rn(__dsub_rn(-qb, __dsqrt_rn(disc)), qa);
        return q < 1e-6 ? 1e-6 : (q > 1.0 ? 1.0 : q);
    } else {
        const float x = (float)d[0], y = (float)d[1], z = (float)d[2];
        const float qa = (float)(cx * cx + cy * cy + cz * cz);
        const float qb = x * cx + y * cy + z * cz;
        float disc = qb * qb - qa * (float)qc;
        disc = disc < 0.f ? 0.f : disc;
        float q = (-qb - sqrtf(disc)) / qa;
        return q < 1e-6f ? 1e-6f : (q > 1.f ? 1.f : q);
    }
}

// ---------------------------------------------------------------------------
// Interpolated bounce-back.
//
// One CTA per sphere.  The owner values of the sphere's bounding box plus a
// two-node stencil margin are staged once in shared memory as two bit masks
// per streamwise row (bit a: node owned by this sphere; node fluid), together
// with per-axis tables of the FP32 offset from the sphere centre and of the
// node index.  The links of direction c_i in row (b, c) are then one word
// operation: fluid(b, c) & owned(b + c_iz, c + c_ix) shifted by c_iy.  The
// rows within R + 1.5 of the centre are listed, and the work is cut into
// units (direction, 32 listed rows) dealt to the warps; lane j takes listed
// row j of the unit, and the set bits of the lanes are streamed through a
// 256-entry queue per warp, so that every lane of a warp processes links --
// two at a time, both links' loads in flight before either is finished.
//
// With the AA orientation the six accesses of a link touch the four nodes
// x_f + c_i (solid), x_f, x_f - c_i, x_f - 2c_i in the planes i and opp(i):
// orientation 1 swaps the two planes and moves the slot-i accesses by -c_i
// and the slot-opp(i) accesses by +c_i.
//
// RT: link arithmetic and q (FP64 with correctly rounded operations for FP64
// storage, bit-consistent with the oracle; FP32 with hardware reciprocals for
// FP32/FP16 storage, where an FP64 q per link would cost more than the fluid
// step at GB300's FP64 rate).  Force and torque: per-thread sums in FP64
// (FP64 storage) or in compensated FP32 (ForceAcc), per-sphere sums of the
// threads' partials in FP64.

// bit a of the result = bit a + cy of x
template <typename W>
__device__ __forceinline__ W shift_a(W x, int cy) {
    return cy > 0 ? (x >> 1) : (cy < 0 ? (x << 1) : x);
}
__device__ __forceinline__ int lowest_bit(uint32_t m) { return __ffs((int)m) - 1; }
__device__ __forceinline__ int lowest_bit(unsigned long long m) { return __ffsll((long long)m) - 1; }

// per-direction constants (a shared-memory table built once per CTA)
struct IbbDir {
    float fcx, fcy, fcz, mw6;     // c_i as floats, -6 w_i
    float qa, inv_qa;             // |c_i|^2 and its inverse
    int packed;                   // (cx+1) | (cy+1) << 2 | (cz+1) << 4 | opp(i) << 8
    int pad;
};

// staged box of one sphere, in shared memory
template <typename W>
struct IbbBox {
    int S;                        // row stride: row (b, c) at b + S * c
    const W* own;                 // bit a: owned by this sphere
    const W* fluid;               // bit a: fluid
    const int* rowIdx;            // node-index term of row (b, c)
    const float *tA, *tB, *tC;    // FP32 offset from the centre per staged index
    const int* wA;                // wrapped streamwise node per staged a
    const int* wZ;                // wrapped spanwise node per staged b (FP64 path)
    const IbbDir* dir;            // [Q]
    int xlo;                      // wall-normal node of staged c = 0
    float R2f;                    // R^2 in FP32
};

// A link between its gathers and its finish: its packed coordinates (with
// the partner flags), q, the populations read and the address of the
// returning population.  The finish recomputes the rest of the geometry from
// (a, b, c, i) and q, so a lane can keep several links in flight.
template <typename T, typename RT>
struct IbbLink {
    uint32_t v;                   // a | b << 8 | c << 16 | i << 24 | ok1 << 29 | ok2 << 30
    RT q, A, X, Y;
    T* w;                         // storage of the returning population
};
constexpr uint32_t kOk1 = 1u << 29, kOk2 = 1u << 30;

// Offset from the sphere's centre to the fluid node of staged coordinates
// (a, b, c): FP64 from the position for FP64 storage, the staged FP32 table
// otherwise.
template <typename RT, typename W>
__device__ __forceinline__ void ibb_offset(const DeviceParticles& P, const Geometry& g, int p, const IbbBox<W>& B,
                                           int a, int b, int c, RT d[3]) {
    if constexpr (sizeof(RT) == 8) {
        offset(P, g, p, B.xlo + c, B.wA[a], B.wZ[b], d);
    } else {
        d[0] = B.tC[c]; d[1] = B.tA[a]; d[2] = B.tB[b];
    }
}

// Gathers of one link: entry (a, b, c, i) = staged coordinates of the fluid
// node and the direction.  X and Y are the interpolation partners: (B, C) at
// x_f, x_f - c_i in direction i for q < 1/2 (quadratic), D at x_f - c_i in
// direction opp(i) otherwise (linear: ok2 is cleared for q >= 1/2, Y is not
// read).
template <typename T, typename RT, typename W, bool Q64>
__device__ __forceinline__ IbbLink<T, RT> ibb_gather(const DeviceState& s, const DeviceParticles& P, int p,
                                                     int parity, const IbbBox<W>& B, uint32_t v) {
    IbbLink<T, RT> L;
    const int a = v & 255, b = (v >> 8) & 255, c = (v >> 16) & 255, i = (int)(v >> 24);
    const IbbDir D = B.dir[i];
    const int cx = (D.packed & 3) - 1, cy = ((D.packed >> 2) & 3) - 1, cz = ((D.packed >> 4) & 3) - 1;
    const int ib = D.packed >> 8;
    const int dr = cz + B.S * cx;                      // row offset of c_i
    const int r0 = b + B.S * c;
    L.v = v;
    L.q = RT(1); L.A = L.X = L.Y = RT(0);
    L.w = nullptr;
    // the staged box holds every node the link touches: rows r0 - 2dr ..
    // r0 + dr and streamwise positions a - 2cy .. a + cy
    if (!LBM_IN_BOUNDS(s.bounds, i >= 1 && i < Q && a >= 2 && a + 2 < B.S && b >= 2 && b + 2 < B.S && c >= 2 &&
                                     c + 2 < B.S, 221))
        return L;
    bool ok1 = (B.fluid[r0 - dr] >> (a - cy)) & 1;
    bool ok2 = ok1 && ((B.fluid[r0 - 2 * dr] >> (a - 2 * cy)) & 1);
    const uint32_t gx = (uint32_t)(B.wA[a] + B.rowIdx[r0]);
    const uint32_t gs = (uint32_t)(B.wA[a + cy] + B.rowIdx[r0 + dr]);
    uint32_t ga = 0, gb = 0;
    if (ok1) ga = (uint32_t)(B.wA[a - cy] + B.rowIdx[r0 - dr]);
    if (ok2) gb = (uint32_t)(B.wA[a - 2 * cy] + B.rowIdx[r0 - 2 * dr]);
    if (!LBM_IN_BOUNDS(s.bounds, gx < s.N && gs < s.N && ga < s.N && gb < s.N, 222))
        return L;
    const T* Pi = plane<T>(s, i);
    const T* Pib = plane<T>(s, ib);
    if constexpr (sizeof(RT) == 8) {
        double dd[3];
        ibb_offset<RT, W>(P, s.g, p, B, a, b, c, dd);
        L.q = link_q<double>(dd, cx, cy, cz, __dsub_rn(norm2_rn(dd), __dmul_rn(P.R, P.R)));
    } else if constexpr (Q64) {
        double dd[3];
        offset(P, s.g, p, B.xlo + c, B.wA[a], B.wZ[b], dd);
        L.q = (float)link_q<double>(dd, cx, cy, cz, __dsub_rn(norm2_rn(dd), __dmul_rn(P.R, P.R)));
    } else {
        const float d0 = B.tC[c], d1 = B.tA[a], d2 = B.tB[b];
        const float qc = d0 * d0 + d1 * d1 + d2 * d2 - B.R2f;
        const float qb = d0 * D.fcx + d1 * D.fcy + d2 * D.fcz;
        const float disc = qb * qb - qc * D.qa;
        const float sq = disc > 0.f ? disc * rsqrtf(disc) : 0.f;
        float q = (-qb - sq) * D.inv_qa;
        L.q = q < 1e-6f ? 1e-6f : (q > 1.f ? 1.f : q);
    }
    const bool near = L.q < RT(0.5);
    // q >= 1/2 takes the linear form: Bouzidi's quadratic q >= 1/2 form
    // extrapolates (coefficient -(2q-1)/(2q+1) on the second partner) and at
    // tau ~ 0.507 with MRTtype 1's s16 = 1.98 it drives a growing mode in
    // narrow gaps between spheres
    if (!near) ok2 = false;
    const T* pX = near ? (parity ? Pib + ga : Pi + gx) : (parity ? Pi + gx : Pib + ga);
    const T* pY = near ? (parity ? Pib + gb : Pi + ga) : (parity ? Pi + ga : Pib + gb);
    L.w = const_cast<T*>(parity ? Pi + gs : Pib + gx);
    L.A = pop_r<T, RT>(s, parity ? Pib + gx : Pi + gs);
    L.X = ok1 ? pop_r<T, RT>(s, pX) : RT(0);
    L.Y = ok2 ? pop_r<T, RT>(s, pY) : RT(0);
    L.v = v | (ok1 ? kOk1 : 0u) | (ok2 ? kOk2 : 0u);
    return L;
}

// Per-lane sums of a sphere's force and torque.  FP64 storage sums in FP64.
// FP32/FP16 storage computes each link's momentum in FP32 and sums it with
// an error-free transformation (Knuth's TwoSum: s + c carries the exact sum
// of s and x), so a lane's sum of n terms is accurate to 2u|S| + O(n^2 u^2)
// sum|x| (u = 2^-24), i.e. to about FP64 accuracy for the ~20 links a lane
// takes; the lanes' partial sums s + c are then reduced in FP64.
template <typename RT>
struct ForceAcc {
    double s[6];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < 6; ++k) s[k] = 0.0;
    }
    __device__ __forceinline__ void add(int k, double x) { s[k] += x; }
    __device__ __forceinline__ double total(int k) const { return s[k]; }
};
template <>
struct ForceAcc<float> {
    float s[6], c[6];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < 6; ++k) s[k] = c[k] = 0.f;
    }
    __device__ __forceinline__ void add(int k, float x) {
        const float t = __fadd_rn(s[k], x);
        const float z = __fsub_rn(t, s[k]);
        c[k] = __fadd_rn(c[k], __fadd_rn(__fsub_rn(s[k], __fsub_rn(t, z)), __fsub_rn(x, z)));
        s[k] = t;
    }
    __device__ __forceinline__ double total(int k) const { return (double)s[k] + (double)c[k]; }
};

// Interpolation, the returning population and the exchanged momentum and its
// moment (added to acc).  The wall point x_f + q c_i, its velocity and the
// moving-wall term come from the link's coordinates and q.
template <typename T, typename RT, typename W>
__device__ __forceinline__ void ibb_finish(const DeviceState& s, const DeviceParticles& P, int p,
                                           const IbbBox<W>& B, const IbbLink<T, RT>& L, const RT (&UW)[6],
                                           ForceAcc<RT>& acc) {
#ifdef LBM_BOUNDS_CHECK
    if (L.w == nullptr) return;                        // a skipped (out-of-bounds) link
#endif
    const int a = L.v & 255, b = (L.v >> 8) & 255, c = (L.v >> 16) & 255, i = (int)((L.v >> 24) & 31u);
    const bool ok1 = (L.v & kOk1) != 0, ok2 = (L.v & kOk2) != 0;
    const IbbDir D = B.dir[i];
    RT fcx, fcy, fcz, mw6;
    if constexpr (sizeof(RT) == 8) {
        fcx = (D.packed & 3) - 1; fcy = ((D.packed >> 2) & 3) - 1; fcz = ((D.packed >> 4) & 3) - 1;
        mw6 = -6.0 * (i <= 6 ? W1 : W2);
    } else {
        fcx = D.fcx; fcy = D.fcy; fcz = D.fcz;
        mw6 = D.mw6;
    }
    RT d[3];
    ibb_offset<RT, W>(P, s.g, p, B, a, b, c, d);
    const RT q = L.q, A = L.A;
    const RT x0 = d[0] + q * fcx, x1 = d[1] + q * fcy, x2 = d[2] + q * fcz;
    const RT uw0 = UW[0] + (UW[4] * x2 - UW[5] * x1);
    const RT uw1 = UW[1] + (UW[5] * x0 - UW[3] * x2);
    const RT uw2 = UW[2] + (UW[3] * x1 - UW[4] * x0);
    const RT mw = mw6 * ((fcx * uw0 + fcy * uw1) + fcz * uw2);
    RT fn;
    if (q < RT(0.5)) {
        if (ok2) fn = q * (RT(1) + RT(2) * q) * A + (RT(1) - RT(4) * q * q) * L.X + q * (RT(2) * q - RT(1)) * L.Y + mw;
        else if (ok1) fn = RT(2) * q * A + (RT(1) - RT(2) * q) * L.X + mw;
        else fn = A + mw;
    } else {
        if (ok1) {
            if constexpr (sizeof(RT) == 8) {
                fn = (A + mw) / (RT(2) * q) + (RT(2) * q - RT(1)) / (RT(2) * q) * L.X;
            } else {
                const float h = __fdividef(1.f, 2.f * q);
                fn = (A + mw) * h + (2.f * q - 1.f) * h * L.X;
            }
        } else {
            fn = A + mw;
        }
    }
    put_r<T, RT>(s, L.w, fn);
    // Galilean-invariant momentum exchange
    const RT sA = A + fn, dA = fn - A;
    const RT p0 = fcx * sA + uw0 * dA, p1 = fcy * sA + uw1 * dA, p2 = fcz * sA + uw2 * dA;
    acc.add(0, p0); acc.add(1, p1); acc.add(2, p2);
    acc.add(3, x1 * p2 - x2 * p1);
    acc.add(4, x2 * p0 - x0 * p2);
    acc.add(5, x0 * p1 - x1 * p0);
}

// NL links per lane: all gathers in flight before the first finish
template <typename T, typename RT, typename W, bool Q64, int NL>
__device__ __forceinline__ void ibb_links(const DeviceState& s, const DeviceParticles& P, int p, int parity,
                                          const IbbBox<W>& B, const uint32_t (&v)[NL], const RT (&UW)[6],
                                          ForceAcc<RT>& acc) {
    IbbLink<T, RT> L[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) L[k] = ibb_gather<T, RT, W, Q64>(s, P, p, parity, B, v[k]);
#pragma unroll
    for (int k = 0; k < NL; ++k) ibb_finish<T, RT, W>(s, P, p, B, L[k], UW, acc);
}

constexpr int kIbbQueue = 256;        // link queue entries per warp (a power of 2)
constexpr int kIbbLinks = 2;         // links per lane in flight (kIbbQueue >= 64 kIbbLinks)
constexpr int kIbbStageRows = 16;     // owner rows in flight per warp while staging

// shared-memory plan of k_ibb for spheres of radius R with row words of
// wbits bits; bytes == 0 when the staged rows do not fit one word.  The
// staging buffers (kIbbStageRows owner rows of wbits ints per warp) share
// their space with the link queues, which are used only afterwards.
struct IbbPlan { int S, own_off, fluid_off, row_off, tab_off, dir_off, list_off, queue_off, bytes; };
__host__ __device__ inline IbbPlan ibb_plan(double R, int wbits) {
    IbbPlan pl;
    pl.S = (int)floor(2.0 * (R + 1.5)) + 3 + 4;         // staged nodes per axis, at most
    const int SS = pl.S * pl.S, wb = wbits / 8;
    pl.own_off = 0;
    pl.fluid_off = pl.own_off + SS * wb;
    pl.row_off = pl.fluid_off + SS * wb;
    pl.tab_off = pl.row_off + SS * 4;
    pl.dir_off = pl.tab_off + 5 * pl.S * 4;
    pl.dir_off = (pl.dir_off + 15) & ~15;
    pl.list_off = pl.dir_off + Q * (int)sizeof(IbbDir);
    pl.queue_off = (pl.list_off + SS * 2 + 15) & ~15;
    const int queue_bytes = (kPThreads / 32) * kIbbQueue * 4;
    const int stage_bytes = (kPThreads / 32) * kIbbStageRows * wbits * 4;
    pl.bytes = pl.S <= wbits ? pl.queue_off + (queue_bytes > stage_bytes ? queue_bytes : stage_bytes) : 0;
    return pl;
}

// 4-byte asynchronous copy global -> shared (completes at cp_async_wait_all
// of the issuing thread)
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

template <typename T, typename RT, typename W, bool Q64>
__global__ void __launch_bounds__(kPThreads, sizeof(RT) == 8 ? 2 : 4)
    k_ibb(DeviceState s, DeviceParticles P, int parity, IbbPlan pl) {
    extern __shared__ __align__(16) unsigned char ibb_smem[];
    __shared__ int nact;
    const Geometry& g = s.g;
    const int p = P.order ? P.order[blockIdx.x] : (int)blockIdx.x;
    const SphereGeom G = P.geom[p];
    const float ext = P.Rf + 1.5f;
    const Range rx = box_g(G.ci[0], G.h[0], ext, g.NZ, false);
    const Range ry = box_g(G.ci[1], G.h[1], ext, g.NX, true);
    const Range rz = box_g(G.ci[2], G.h[2], ext, g.NY, true);
    const int SA = ry.n + 4, SB = rz.n + 4, SC = rx.n + 4, S = pl.S;
    const int ya = ry.lo - 2, zb = rz.lo - 2, xc = rx.lo - 2;   // node of staged index 0
    W* own = reinterpret_cast<W*>(ibb_smem + pl.own_off);
    W* fluid = reinterpret_cast<W*>(ibb_smem + pl.fluid_off);
    int* rowIdx = reinterpret_cast<int*>(ibb_smem + pl.row_off);
    float* tA = reinterpret_cast<float*>(ibb_smem + pl.tab_off);
    float* tB = tA + S;
    float* tC = tB + S;
    int* wA = reinterpret_cast<int*>(tC + S);
    int* wZ = wA + S;
    IbbDir* dir = reinterpret_cast<IbbDir*>(ibb_smem + pl.dir_off);
    uint16_t* rowlist = reinterpret_cast<uint16_t*>(ibb_smem + pl.list_off);
    uint32_t* queue = reinterpret_cast<uint32_t*>(ibb_smem + pl.queue_off);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int NXY = g.NX * g.NY;
    if (threadIdx.x == 0) nact = 0;
    for (int t = threadIdx.x; t < SA; t += blockDim.x) {
        tA[t] = (float)(ya + t - G.ci[1]) + G.h[1];
        wA[t] = wrapi(ya + t, g.NX);
    }
    for (int t = threadIdx.x; t < SB; t += blockDim.x) {
        tB[t] = (float)(zb + t - G.ci[2]) + G.h[2];
        wZ[t] = wrapi(zb + t, g.NY);
    }
    for (int t = threadIdx.x; t < SC; t += blockDim.x) tC[t] = (float)(xc + t - G.ci[0]) + G.h[0];
    for (int t = threadIdx.x; t < SB * SC; t += blockDim.x) {
        const int b = t % SB, c = t / SB;
        rowIdx[b + S * c] = wrapi(zb + b, g.NY) * g.NX + (xc + c) * NXY;
    }
    if (threadIdx.x < Q) {
        const int i = threadIdx.x;
        IbbDir d;
        const int cx = cx_rt(i), cy = cy_rt(i), cz = cz_rt(i);
        d.fcx = (float)cx; d.fcy = (float)cy; d.fcz = (float)cz;
        d.mw6 = (float)(-6.0 * w_rt(i));
        d.qa = (float)(cx * cx + cy * cy + cz * cz);
        d.inv_qa = d.qa == 1.f ? 1.f : 0.5f;
        d.packed = (cx + 1) | ((cy + 1) << 2) | ((cz + 1) << 4) | (opp_rt(i) << 8);
        d.pad = 0;
        dir[i] = d;
    }
    __syncthreads();                                     // the staging reads wZ, tB, tC
    // staging: a warp takes kIbbStageRows consecutive rows at a time; lane j
    // copies nodes a = j (and j + 32) of each into the warp's buffer with
    // asynchronous copies (all rows in flight at once, no registers held),
    // then the rows become the two masks by ballots over the lane's own
    // copies.  Rows beyond R + 4.5 of the centre are not read (masks 0): the
    // links start on rows within R + 1.5 and read the masks at most two rows
    // further in each of b and c (2 sqrt 2 < 3).
    {
        const int* __restrict__ owner = P.owner;
        const int nrows = SB * SC;
        const int a0 = wrapi(ya + lane, g.NX);
        const int a1 = sizeof(W) == 8 ? wrapi(ya + lane + 32, g.NX) : 0;
        constexpr int WI = 8 * (int)sizeof(W);           // ints per buffered row
        int* const buf = reinterpret_cast<int*>(ibb_smem + pl.queue_off) + wid * kIbbStageRows * WI;
        const float lim = (ext + 3.f) * (ext + 3.f);
        for (int r0 = wid * kIbbStageRows; r0 < nrows; r0 += nw * kIbbStageRows) {
            const int nr = min(kIbbStageRows, nrows - r0);
            const int b0 = r0 % SB, c0 = r0 / SB;
            unsigned read = 0;                           // bit u: row r0 + u was copied
            for (int u = 0, b = b0, c = c0; u < nr; ++u) {
                const int ix = xc + c;
                if (ix >= 0 && ix < g.NZ && tB[b] * tB[b] + tC[c] * tC[c] <= lim) {
                    read |= 1u << u;
                    const int* row = owner + ((size_t)g.NX * (uint32_t)wZ[b] + (size_t)NXY * (uint32_t)ix);
                    if (lane < SA) cp_async4(buf + u * WI + lane, row + a0);
                    if (sizeof(W) == 8 && lane + 32 < SA) cp_async4(buf + u * WI + 32 + lane, row + a1);
                }
                if (++b == SB) { b = 0; ++c; }
            }
            cp_async_wait_all();
            for (int u = 0, b = b0, c = c0; u < nr; ++u) {
                const bool rv = (read >> u) & 1u;
                const int o0 = (rv && lane < SA) ? buf[u * WI + lane] : -3;
                W pw = (W)__ballot_sync(0xffffffffu, o0 == p), fw = (W)__ballot_sync(0xffffffffu, o0 == -1);
                if constexpr (sizeof(W) == 8) {
                    const int o1 = (rv && lane + 32 < SA) ? buf[u * WI + 32 + lane] : -3;
                    pw |= (W)__ballot_sync(0xffffffffu, o1 == p) << 32;
                    fw |= (W)__ballot_sync(0xffffffffu, o1 == -1) << 32;
                }
                if (lane == 0 && LBM_IN_BOUNDS(s.bounds, b < S && c < S, 223)) {
                    own[b + S * c] = pw;
                    fluid[b + S * c] = fw;
                }
                if (++b == SB) { b = 0; ++c; }
            }
            __syncwarp();                                // the buffer is refilled next
        }
    }
    __syncthreads();
    // rows that can hold links: (b, c) within R + 1.5 of the centre
    {
        const float lim = ext * ext + 0.01f;
        const int nr = rz.n * rx.n;
        for (int t0 = wid * 32; t0 < nr; t0 += 32 * nw) {
            const int t = t0 + lane;
            bool keep = false;
            int b = 0, c = 0;
            if (t < nr) {
                b = 2 + t % rz.n; c = 2 + t / rz.n;
                keep = tB[b] * tB[b] + tC[c] * tC[c] <= lim;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            int base = 0;
            if (lane == 0 && bal) base = atomicAdd(&nact, __popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (keep) rowlist[base + __popc(bal & ((1u << lane) - 1u))] = (uint16_t)(b | (c << 8));
        }
    }
    IbbBox<W> Bx;
    Bx.S = S; Bx.own = own; Bx.fluid = fluid; Bx.rowIdx = rowIdx;
    Bx.tA = tA; Bx.tB = tB; Bx.tC = tC; Bx.wA = wA; Bx.wZ = wZ; Bx.dir = dir;
    Bx.xlo = xc;
    Bx.R2f = P.Rf * P.Rf;
    RT UW[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if constexpr (sizeof(RT) == 8) {
            UW[k] = P.vel[3 * p + k];
            UW[3 + k] = P.omg[3 * p + k];
        } else {
            UW[k] = G.U[k];
            UW[3 + k] = G.W[k];
        }
    }
    ForceAcc<RT> acc;
    acc.zero();
    const unsigned lt = (1u << lane) - 1u;
    uint32_t* q = queue + wid * kIbbQueue;
    int head = 0, tail = 0;
    __syncthreads();
    // units (direction i, chunk of 32 rows); lane j on row 32 k + j
    {
        const W amask = (((W)1 << ry.n) - 1) << 2;      // candidate nodes a in [2, 2 + ry.n)
        const int na = nact;
        const int nch = (na + 31) >> 5;
        const int nunits = (Q - 1) * nch;
        for (int u = wid; u < nunits; u += nw) {
            const int i = 1 + u / nch, k = u - (i - 1) * nch;
            const int rr = (k << 5) + lane;
            W m = 0;
            int b = 0, c = 0;
            if (rr < na) {
                const int rc = rowlist[rr];
                b = rc & 255; c = rc >> 8;
                const int pk = dir[i].packed;
                const int cx = (pk & 3) - 1, cy = ((pk >> 2) & 3) - 1, cz = ((pk >> 4) & 3) - 1;
                m = fluid[b + S * c] & shift_a(own[(b + cz) + S * (c + cx)], cy) & amask;
            }
            // append the set bits of all lanes (a prefix over the lanes)
            const int n = __popc(m);
            int incl = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int tot = __shfl_sync(0xffffffffu, incl, 31);
            if (tot == 0) continue;
            if (tail - head + tot <= kIbbQueue) {
                int pos = tail + incl - n;
                const uint32_t hi = ((uint32_t)b << 8) | ((uint32_t)c << 16) | ((uint32_t)i << 24);
                while (m) {
                    q[(pos++) & (kIbbQueue - 1)] = (uint32_t)lowest_bit(m) | hi;
                    m &= m - 1;
                }
                tail += tot;
            } else {
                // more links than the queue has room for: one bit per lane at a time
                while (__any_sync(0xffffffffu, m != 0)) {
                    const bool has = m != 0;
                    int a = 0;
                    if (has) { a = lowest_bit(m); m &= m - 1; }
                    const unsigned bal = __ballot_sync(0xffffffffu, has);
                    if (has) q[(tail + __popc(bal & lt)) & (kIbbQueue - 1)] = (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16) | ((uint32_t)i << 24);
                    tail += __popc(bal);
                    if (tail - head >= 32) {
                        __syncwarp();
                        const uint32_t v[1] = {q[(head + lane) & (kIbbQueue - 1)]};
                        head += 32;
                        __syncwarp();
                        ibb_links<T, RT, W, Q64, 1>(s, P, p, parity, Bx, v, UW, acc);
                    }
                }
            }
            while (tail - head >= 32 * kIbbLinks) {
                __syncwarp();
                uint32_t v[kIbbLinks];
#pragma unroll
                for (int k = 0; k < kIbbLinks; ++k) v[k] = q[(head + 32 * k + lane) & (kIbbQueue - 1)];
                head += 32 * kIbbLinks;
                __syncwarp();
                ibb_links<T, RT, W, Q64, kIbbLinks>(s, P, p, parity, Bx, v, UW, acc);
            }
        }
        __syncwarp();
        while (tail - head >= 32) {
            const uint32_t v[1] = {q[(head + lane) & (kIbbQueue - 1)]};
            head += 32;
            ibb_links<T, RT, W, Q64, 1>(s, P, p, parity, Bx, v, UW, acc);
        }
        if (lane < tail - head) {
            const uint32_t v[1] = {q[(head + lane) & (kIbbQueue - 1)]};
            ibb_links<T, RT, W, Q64, 1>(s, P, p, parity, Bx, v, UW, acc);
        }
    }
    // per-sphere FP64 reduction: warp shuffles, then across warps
    __shared__ double sh[6][kPThreads / 32];
    __shared__ int shn[kPThreads / 32];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double v = acc.total(k);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][wid] = v;
    }
    if (lane == 0) shn[wid] = tail;
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int ww = 0; ww < nw; ++ww) v += sh[threadIdx.x][ww];
        if (threadIdx.x < 3) P.force[3 * p + threadIdx.x] = v;
        else P.torque[3 * p + threadIdx.x - 3] = v;
    }
    if (threadIdx.x == 0) {
        unsigned nl = 0;
        for (int ww = 0; ww < nw; ++ww) nl += (unsigned)shn[ww];
        atomicAdd(&P.counters[1], nl);
    }
}

template <typename T, typename RT, typename W, bool Q64>
cudaError_t launch_ibb_q(const DeviceState& s, const DeviceParticles& P, int parity, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k_ibb<T, RT, W, Q64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_ibb<T, RT, W, Q64><<<P.npart, kPThreads, smem, st>>>(s, P, parity, ibb_plan(P.R, 8 * (int)sizeof(W)));
    return cudaGetLastError();
}
template <typename T, typename RT, typename W>
cudaError_t launch_ibb(const DeviceState& s, const DeviceParticles& P, int parity, size_t smem, cudaStream_t st) {
    // FP64 storage computes q in FP64 anyway
    if (sizeof(RT) == 4 && P.q_fp64) return launch_ibb_q<T, RT, W, true>(s, P, parity, smem, st);
    return launch_ibb_q<T, RT, W, false>(s, P, parity, smem, st);
}

size_t ibb_smem_bytes(double R) {
    const IbbPlan p32 = ibb_plan(R, 32);
    return (size_t)(p32.bytes ? p32.bytes : ibb_plan(R, 64).bytes);
}

__device__ __forceinline__ double repulse(double h, double zeta, double k0, double k1) {
    if (h >= zeta) return 0.0;
    const double a = __ddiv_rn(__dsub_rn(zeta, h), zeta);
    double f = __dmul_rn(__dmul_rn(k0, a), a);
    if (h < 0.0) f = __dadd_rn(f, __ddiv_rn(__dmul_rn(k1, -h), zeta));
    return f;
}

// Soft-sphere repulsion gathered per sphere in index order (old positions).
// Pairs are screened in FP32 (positions staged in shared memory) with a
// margin; only pairs within reach get the exact FP64 evaluation.
constexpr int kRepTile = 128;
__global__ void __launch_bounds__(kRepTile) k_repulsion(DeviceParticles P, Geometry g) {
    __shared__ float3 tile[kRepTile];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = s < P.npart;
    const double R = P.R;
    const double L1 = (double)g.NX, L2 = (double)g.NY;
    const float fL1 = (float)L1, fL2 = (float)L2;
    const float reach = (float)(2.0 * R + P.zeta) + 0.01f;
    const float reach2 = reach * reach;
    double rep[3] = {0.0, 0.0, 0.0};
    const double xs0 = act ? P.pos[3 * s] : 0.0, xs1 = act ? P.pos[3 * s + 1] : 0.0, xs2 = act ? P.pos[3 * s + 2] : 0.0;
    const float fx0 = (float)xs0, fx1 = (float)xs1, fx2 = (float)xs2;
    for (int base = 0; base < P.npart; base += kRepTile) {
        const int j = base + threadIdx.x;
        if (j < P.npart) tile[threadIdx.x] = make_float3((float)P.pos[3 * j], (float)P.pos[3 * j + 1], (float)P.pos[3 * j + 2]);
        __syncthreads();
        const int nt = min(kRepTile, P.npart - base);
        if (act) {
            for (int k = 0; k < nt; ++k) {
                const int t = base + k;
                if (t == s) continue;
                float e0 = tile[k].x - fx0, e1 = tile[k].y - fx1, e2 = tile[k].z - fx2;
                e1 = e1 >= 0.5f * fL1 ? e1 - fL1 : (e1 < -0.5f * fL1 ? e1 + fL1 : e1);
                e2 = e2 >= 0.5f * fL2 ? e2 - fL2 : (e2 < -0.5f * fL2 ? e2 + fL2 : e2);
                if (e0 * e0 + e1 * e1 + e2 * e2 > reach2) continue;
                const double d0 = __dsub_rn(P.pos[3 * t], xs0);
                const double d1 = dmin_image(__dsub_rn(P.pos[3 * t + 1], xs1), L1);
                const double d2 = dmin_image(__dsub_rn(P.pos[3 * t + 2], xs2), L2);
                const double dd[3] = {d0, d1, d2};
                const double dist = __dsqrt_rn(norm2_rn(dd));
                const double fm = repulse(__dsub_rn(dist, 2.0 * R), P.zeta, P.stf0, P.stf1);
                if (fm != 0.0 && dist > 0.0) {
                    rep[0] = __dsub_rn(rep[0], __ddiv_rn(__dmul_rn(fm, d0), dist));
                    rep[1] = __dsub_rn(rep[1], __ddiv_rn(__dmul_rn(fm, d1), dist));
                    rep[2] = __dsub_rn(rep[2], __ddiv_rn(__dmul_rn(fm, d2), dist));
                }
            }
        }
        __syncthreads();
    }
    if (!act) return;
    const double hl = __dsub_rn(xs0, R), hu = __dsub_rn(__dsub_rn((double)g.NZ, xs0), R);
    rep[0] = __dadd_rn(rep[0], repulse(hl, P.zeta, P.stf0_w, P.stf1_w));
    rep[0] = __dsub_rn(rep[0], repulse(hu, P.zeta, P.stf0_w, P.stf1_w));
    P.rep[3 * s] = rep[0]; P.rep[3 * s + 1] = rep[1]; P.rep[3 * s + 2] = rep[2];
}

// Cell of a sphere centre in the repulsion cell list (cells of equal width
// along each axis, at least one reach wide).
__device__ __forceinline__ int cell_of(const DeviceParticles& P, const Geometry& g, int s, int& cx, int& cy, int& cz) {
    cx = min(P.cell_nx - 1, max(0, (int)(P.pos[3 * s] * P.cell_nx / g.NZ)));
    cy = min(P.cell_ny - 1, max(0, (int)(P.pos[3 * s + 1] * P.cell_ny / g.NX)));
    cz = min(P.cell_nz - 1, max(0, (int)(P.pos[3 * s + 2] * P.cell_nz / g.NY)));
    return cx + P.cell_nx * (cy + P.cell_ny * cz);
}

__global__ void k_bin(DeviceParticles P, Geometry g) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.npart) return;
    int cx, cy, cz;
    const int cell = cell_of(P, g, s, cx, cy, cz);
    const int k = atomicAdd(&P.cell_count[cell], 1);
    if (k < kCellCap) P.cell_list[(size_t)cell * kCellCap + k] = s;
    else atomicExch(&P.counters[2], 1u);
}

// exact FP64 pair term of spheres s and t (old positions), as the oracle
__device__ __forceinline__ void pair_repulsion(const DeviceParticles& P, double L1, double L2, int s, int t,
                                               double rep[3]) {
    const double d0 = __dsub_rn(P.pos[3 * t], P.pos[3 * s]);
    const double d1 = dmin_image(__dsub_rn(P.pos[3 * t + 1], P.pos[3 * s + 1]), L1);
    const double d2 = dmin_image(__dsub_rn(P.pos[3 * t + 2], P.pos[3 * s + 2]), L2);
    const double dd[3] = {d0, d1, d2};
    const double dist = __dsqrt_rn(norm2_rn(dd));
    const double fm = repulse(__dsub_rn(dist, 2.0 * P.R), P.zeta, P.stf0, P.stf1);
    if (fm != 0.0 && dist > 0.0) {
        rep[0] = __dsub_rn(rep[0], __ddiv_rn(__dmul_rn(fm, d0), dist));
        rep[1] = __dsub_rn(rep[1], __ddiv_rn(__dmul_rn(fm, d1), dist));
        rep[2] = __dsub_rn(rep[2], __ddiv_rn(__dmul_rn(fm, d2), dist));
    }
}

// Repulsion from the cell list: one warp per sphere, lane k < 27 on one
// neighbour cell.  Partners within reach (FP32 screen with a margin) are
// collected, sorted by sphere id and summed in that order with the exact
// FP64 pair term, so that the result is the oracle's index-ordered sum.  A
// bin that overflowed at this step sends every sphere to the all-pairs scan.
constexpr int kRepWarps = 8;
constexpr int kRepMaxPartners = 64;
__global__ void __launch_bounds__(32 * kRepWarps) k_repulsion_cells(DeviceParticles P, Geometry g) {
    __shared__ int partners[kRepWarps][kRepMaxPartners];
    __shared__ int npart_w[kRepWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = blockIdx.x * kRepWarps + w;
    if (s >= P.npart) return;                       // whole warps leave together
    const double R = P.R;
    const double L1 = (double)g.NX, L2 = (double)g.NY;
    const float fL1 = (float)L1, fL2 = (float)L2;
    const float reach = (float)(2.0 * R + P.zeta) + 0.01f;
    const float reach2 = reach * reach;
    const float fx0 = (float)P.pos[3 * s], fx1 = (float)P.pos[3 * s + 1], fx2 = (float)P.pos[3 * s + 2];
    if (lane == 0) npart_w[w] = 0;
    __syncwarp();
    const bool all_pairs = *(volatile unsigned*)&P.counters[2] != 0;
    auto consider = [&](int t) {
        if (t == s) return;
        float e0 = (float)P.pos[3 * t] - fx0, e1 = (float)P.pos[3 * t + 1] - fx1, e2 = (float)P.pos[3 * t + 2] - fx2;
        e1 = e1 >= 0.5f * fL1 ? e1 - fL1 : (e1 < -0.5f * fL1 ? e1 + fL1 : e1);
        e2 = e2 >= 0.5f * fL2 ? e2 - fL2 : (e2 < -0.5f * fL2 ? e2 + fL2 : e2);
        if (e0 * e0 + e1 * e1 + e2 * e2 > reach2) return;
        const int k = atomicAdd(&npart_w[w], 1);
        if (k < kRepMaxPartners) partners[w][k] = t;
    };
    if (all_pairs) {
        for (int t = lane; t < P.npart; t += 32) consider(t);
    } else if (lane < 27) {
        int cx, cy, cz;
        cell_of(P, g, s, cx, cy, cz);
        const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
        const int nx = cx + ox;
        if (nx >= 0 && nx < P.cell_nx) {
            const int ny = (cy + oy + P.cell_ny) % P.cell_ny, nz = (cz + oz + P.cell_nz) % P.cell_nz;
            const int cell = nx + P.cell_nx * (ny + P.cell_ny * nz);
            const int n = min(P.cell_count[cell], kCellCap);
            for (int k = 0; k < n; ++k) consider(P.cell_list[(size_t)cell * kCellCap + k]);
        }
    }
    __syncwarp();
    if (lane != 0) return;
    const int n = npart_w[w];
    double rep[3] = {0.0, 0.0, 0.0};
    if (n <= kRepMaxPartners) {
        int* list = partners[w];
        for (int i = 1; i < n; ++i) {                // insertion sort by sphere id
            const int v = list[i];
            int j = i - 1;
            while (j >= 0 && list[j] > v) { list[j + 1] = list[j]; --j; }
            list[j + 1] = v;
        }
        for (int i = 0; i < n; ++i) pair_repulsion(P, L1, L2, s, list[i], rep);
    } else {
        for (int t = 0; t < P.npart; ++t)            // a crowd beyond the list: plain index order
            if (t != s) pair_repulsion(P, L1, L2, s, t, rep);
    }
    const double xs0 = P.pos[3 * s];
    const double hl = __dsub_rn(xs0, R), hu = __dsub_rn(__dsub_rn((double)g.NZ, xs0), R);
    rep[0] = __dadd_rn(rep[0], repulse(hl, P.zeta, P.stf0_w, P.stf1_w));
    rep[0] = __dsub_rn(rep[0], repulse(hu, P.zeta, P.stf0_w, P.stf1_w));
    P.rep[3 * s] = rep[0]; P.rep[3 * s + 1] = rep[1]; P.rep[3 * s + 2] = rep[2];
}

// Nodes released at this step that lie inside another sphere (overlapping
// spheres) are claimed by the highest-index sphere containing them, as the
// oracle's claim of every inside node does.  The candidates come from the
// cell list binned before the update (a centre moves less than two nodes per
// step, within one cell), or from all spheres when there is no cell list or a
// bin overflowed.
__global__ void k_reclaim(DeviceParticles P, Geometry g, int* owner) {
    const unsigned cnt = min(P.counters[0], (unsigned)P.refill_cap);
    const bool all = P.ncell == 0 || *(volatile unsigned*)&P.counters[2] != 0;
    const float R2 = P.Rf * P.Rf, band = in_band(R2), reach2 = (P.Rf + 0.1f) * (P.Rf + 0.1f);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const uint32_t n = P.refill_node[k];
        const int iy = (int)(n % (uint32_t)g.NX);
        const int iz = (int)((n / (uint32_t)g.NX) % (uint32_t)g.NY);
        const int ix = (int)(n / g.NXY);
        int best = -1;
        auto test = [&](int t) {
            if (t <= best) return;
            const SphereGeom G = P.geom[t];
            int dy = iy - G.ci[1], dz = iz - G.ci[2];             // periodic image first, in integers
            dy = dy > g.NX / 2 ? dy - g.NX : (dy < -(g.NX / 2) ? dy + g.NX : dy);
            dz = dz > g.NY / 2 ? dz - g.NY : (dz < -(g.NY / 2) ? dz + g.NY : dz);
            const float ox = (float)(ix - G.ci[0]) + G.h[0];
            const float oy = (float)dy + G.h[1];
            const float oz = (float)dz + G.h[2];
            const float r2 = ox * ox + oy * oy + oz * oz;
            if (r2 > reach2) return;
            bool in;
            if (r2 < R2 - band) in = true;
            else if (r2 > R2 + band) in = false;
            else {
                double d[3];
                offset(P, g, t, ix, iy, iz, d);
                in = inside(d, P.R);
            }
            if (in) best = t;
        };
        if (all) {
            for (int t = 0; t < P.npart; ++t) test(t);
        } else {
            const int cx = min(P.cell_nx - 1, (int)((ix + 0.5) * P.cell_nx / g.NZ));
            const int cy = min(P.cell_ny - 1, (int)((iy + 0.5) * P.cell_ny / g.NX));
            const int cz = min(P.cell_nz - 1, (int)((iz + 0.5) * P.cell_nz / g.NY));
            for (int k3 = 0; k3 < 27; ++k3) {
                const int nx = cx + k3 % 3 - 1;
                if (nx < 0 || nx >= P.cell_nx) continue;
                const int ny = (cy + (k3 / 3) % 3 - 1 + P.cell_ny) % P.cell_ny;
                const int nz = (cz + k3 / 9 - 1 + P.cell_nz) % P.cell_nz;
                const int cell = nx + P.cell_nx * (ny + P.cell_ny * nz);
                const int m = min(P.cell_count[cell], kCellCap);
                for (int j = 0; j < m; ++j) test(P.cell_list[(size_t)cell * kCellCap + j]);
            }
        }
        if (best >= 0) atomicMax(owner + n, best);
    }
}

// Geometry record of sphere s from its FP64 state; delta: displacement of
// the update just made.
__device__ __forceinline__ void write_geom(const DeviceParticles& P, int s, double delta) {
    SphereGeom G;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double c = P.pos[3 * s + a];
        G.ci[a] = (int)floor(c);
        G.h[a] = 0.5f - (float)(c - (double)G.ci[a]);
        G.U[a] = (float)P.vel[3 * s + a];
        G.W[a] = (float)P.omg[3 * s + a];
        G.pad[a] = 0.f;
    }
    G.delta = __double2float_ru(delta);
    P.geom[s] = G;
}

__global__ void k_geom(DeviceParticles P) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < P.npart) write_geom(P, s, 0.0);
}

// Newton-Euler update (FP64), driven by the average of this step's and the
// previous step's total force and torque: stable for a coupling stiffness
// zeta/m < 2, twice the range of second-order Adams-Bashforth, which light
// small spheres exceed (radius 4, density ratio 2 at tau ~ 0.504 blew up
// within 250 steps).  The body force that drives the fluid also acts on the
// sphere volume.
__global__ void k_newton(DeviceParticles P, Geometry g, double bfx, double bfy, double bfz, int have_prev) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.npart) return;
    const double R = P.R;
    const double L1 = (double)g.NX, L2 = (double)g.NY;
    const double vol = __dmul_rn(__dmul_rn(__dmul_rn(4.0 / 3.0 * kPi, R), R), R);
    const double m = __dmul_rn(P.rho_ratio, vol);
    const double I = __dmul_rn(__dmul_rn(__dmul_rn(0.4, m), R), R);
    const double bf[3] = {bfx, bfy, bfz};
    for (int a = 0; a < 3; ++a) {
        const double Ft = __dadd_rn(__dadd_rn(P.force[3 * s + a], P.rep[3 * s + a]), __dmul_rn(bf[a], vol));
        const double Tt = P.torque[3 * s + a];
        const double fp = have_prev ? P.fprev[3 * s + a] : Ft;
        const double tp = have_prev ? P.tprev[3 * s + a] : Tt;
        const double u0 = P.vel[3 * s + a];
        const double u1 = __dadd_rn(u0, __ddiv_rn(__dmul_rn(0.5, __dadd_rn(Ft, fp)), m));
        P.vel[3 * s + a] = u1;
        P.omg[3 * s + a] = __dadd_rn(P.omg[3 * s + a], __ddiv_rn(__dmul_rn(0.5, __dadd_rn(Tt, tp)), I));
        P.pos_prev[3 * s + a] = P.pos[3 * s + a];
        P.pos[3 * s + a] = __dadd_rn(P.pos[3 * s + a], __dmul_rn(0.5, __dadd_rn(u0, u1)));
        P.fprev[3 * s + a] = Ft;
        P.tprev[3 * s + a] = Tt;
    }
    // a non-finite or runaway state (more than one lattice unit per step)
    // stops the sphere where it was and is reported by the host
    bool bad = false;
    for (int a = 0; a < 3; ++a)
        bad |= !(fabs(P.vel[3 * s + a]) <= 1.0) || !(fabs(P.pos[3 * s + a] - P.pos_prev[3 * s + a]) <= 1.0);
    if (bad) {
        for (int a = 0; a < 3; ++a) P.pos[3 * s + a] = P.pos_prev[3 * s + a];
        atomicOr(&P.counters[3], 2u);
    }
    double disp2 = 0.0;
    for (int a = 0; a < 3; ++a) {
        const double d = P.pos[3 * s + a] - P.pos_prev[3 * s + a];
        disp2 += d * d;
    }
    double y = P.pos[3 * s + 1], z = P.pos[3 * s + 2];
    if (y >= L1) y = __dsub_rn(y, L1);
    else if (y < 0.0) y = __dadd_rn(y, L1);
    if (z >= L2) z = __dsub_rn(z, L2);
    else if (z < 0.0) z = __dadd_rn(z, L2);
    P.pos[3 * s + 1] = y;
    P.pos[3 * s + 2] = z;
    write_geom(P, s, sqrt(disp2));
}

__device__ __forceinline__ void feq_dev(double rho, double ux, double uy, double uz, double* fe) {
    const double usqr = __dmul_rn(1.5, __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz)));
    fe[0] = __dmul_rn(W0, __dsub_rn(rho, usqr));
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const double G = __dadd_rn(__dadd_rn(CXf(i) * ux, CYf(i) * uy), CZf(i) * uz);
        fe[i] = __dmul_rn(weight(i), __dsub_rn(__dadd_rn(__dadd_rn(rho, __dmul_rn(3.0, G)), __dmul_rn(__dmul_rn(4.5, G), G)), usqr));
    }
}

template <typename T>
__device__ __forceinline__ void refill_node(const DeviceState& s, const DeviceParticles& P, int parity, unsigned k) {
    const Geometry& g = s.g;
    const uint32_t n = P.refill_node[k];
    const int* owner = P.owner;
    if (!LBM_IN_BOUNDS(s.bounds, n < g.NXY * (uint32_t)g.NZ && P.refill_part[k] >= 0 &&
                                     P.refill_part[k] < P.npart, 211)) return;
    if (owner[n] != -2) return;
    const int p = P.refill_part[k];
    const int iy = (int)(n % (uint32_t)g.NX);
    const int iz = (int)((n / (uint32_t)g.NX) % (uint32_t)g.NY);
    const int ix = (int)(n / g.NXY);
    double d[3];
    offset(P, g, p, ix, iy, iz, d);
    int best = -1, bx = 0, by = 0, bz = 0;
    double bs = -1e300;
    for (int i = 1; i < Q; ++i) {
        const int cx = cx_rt(i), cy = cy_rt(i), cz = cz_rt(i);
        const int sx = ix + cx;
        if (sx < 0 || sx >= g.NZ) continue;
        const int sy = wrapi(iy + cy, g.NX), sz = wrapi(iz + cz, g.NY);
        if (owner[gnode(g, sx, sy, sz)] != -1) continue;
        double sc = __dadd_rn(__dadd_rn(d[0] * cx, d[1] * cy), d[2] * cz);
        if (i >= 7) sc = __dmul_rn(sc, kInvSqrt2);
        if (sc > bs) { bs = sc; best = i; bx = sx; by = sy; bz = sz; }
    }
    const double* U = P.vel + 3 * p;
    const double* W = P.omg + 3 * p;
    const double uw0 = __dadd_rn(U[0], __dsub_rn(__dmul_rn(W[1], d[2]), __dmul_rn(W[2], d[1])));
    const double uw1 = __dadd_rn(U[1], __dsub_rn(__dmul_rn(W[2], d[0]), __dmul_rn(W[0], d[2])));
    const double uw2 = __dadd_rn(U[2], __dsub_rn(__dmul_rn(W[0], d[1]), __dmul_rn(W[1], d[0])));
    double fe[Q];
    if (best < 0) {
        feq_dev(0.0, uw0, uw1, uw2, fe);
#pragma unroll
        for (int i = 0; i < Q; ++i) write_nat<T>(s, parity, i, ix, iy, iz, fe[i]);
        return;
    }
    double gq[Q];
    double r = 0.0, a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        gq[i] = read_nat<T>(s, parity, i, bx, by, bz);
        r = __dadd_rn(r, gq[i]);
        a = __dadd_rn(a, CXf(i) * gq[i]);
        b = __dadd_rn(b, CYf(i) * gq[i]);
        c = __dadd_rn(c, CZf(i) * gq[i]);
    }
    a = __dadd_rn(a, s.cd.Fx / 2.0);
    b = __dadd_rn(b, s.cd.Fy / 2.0);
    c = __dadd_rn(c, s.cd.Fz / 2.0);
    double fn[Q];
    feq_dev(r, a, b, c, fn);
    feq_dev(r, uw0, uw1, uw2, fe);
#pragma unroll
    for (int i = 0; i < Q; ++i) write_nat<T>(s, parity, i, ix, iy, iz, __dadd_rn(fe[i], __dsub_rn(gq[i], fn[i])));
}

// Refilling of nodes queued by k_shell<release> that are still fluid (-2).
template <typename T>
__global__ void k_refill(DeviceState s, DeviceParticles P, int parity) {
    const unsigned cnt = min(P.counters[0], (unsigned)P.refill_cap);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x)
        refill_node<T>(s, P, parity, k);
}

__global__ void k_refill_done(DeviceParticles P) {
    const unsigned cnt = min(P.counters[0], (unsigned)P.refill_cap);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const uint32_t n = P.refill_node[k];
        if (P.owner[n] == -2) P.owner[n] = -1;
    }
}

// ---------------------------------------------------------------------------
// Spatial order of the spheres for the bounce-back kernel.  A 128-byte line of
// an FP16 population row spans 64 streamwise nodes, wider than a sphere, so
// neighbouring spheres share many of the lines their links gather; taking the
// spheres in index order (random positions) fetches those lines once per
// sphere, taking neighbours together lets them hit in L2 (on the
// 1024x512x512 channel with 16384 spheres: 12.4 -> 8.7 GB of DRAM reads per
// step).  The order is a counting sort by the Morton code of cells order_cs
// wide (the ties in any order); each CTA still computes exactly its own
// sphere, so the order changes no result.

// 7 bits -> every third bit
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x7fu;
    v = (v | (v << 8)) & 0x0000f00fu;
    v = (v | (v << 4)) & 0x000c30c3u;
    v = (v | (v << 2)) & 0x00249249u;
    return v;
}

__global__ void k_order_hist(DeviceParticles P) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.npart) return;
    const double inv = 1.0 / P.order_cs;
    const uint32_t a = (uint32_t)fmax(0.0, floor(P.pos[3 * s] * inv));        // wall-normal
    const uint32_t b = (uint32_t)fmax(0.0, floor(P.pos[3 * s + 1] * inv));    // streamwise
    const uint32_t c = (uint32_t)fmax(0.0, floor(P.pos[3 * s + 2] * inv));    // spanwise
    uint32_t key = spread3(b) | (spread3(c) << 1) | (spread3(a) << 2);
    if (key >= (uint32_t)P.order_nbins) key = (uint32_t)P.order_nbins - 1;   // guards rounding at the far edges
    P.order_key[s] = (int)key;
    atomicAdd(&P.order_hist[key], 1);
}

// exclusive prefix sum of order_hist in place, one CTA
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_order_scan(DeviceParticles P) {
    __shared__ int part[kScanThreads];
    const int n = P.order_nbins;
    const int chunk = (n + kScanThreads - 1) / kScanThreads;
    const int lo = threadIdx.x * chunk, hi = min(n, lo + chunk);
    int sum = 0;
    for (int i = lo; i < hi; ++i) sum += P.order_hist[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {          // inclusive scan of the chunk sums
        const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - sum;
    for (int i = lo; i < hi; ++i) {
        const int c = P.order_hist[i];
        P.order_hist[i] = run;
        run += c;
    }
}

__global__ void k_order_scatter(DeviceParticles P) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.npart) return;
    P.order[atomicAdd(&P.order_hist[P.order_key[s]], 1)] = s;
}

__global__ void k_count_solid(const int* owner, size_t N, unsigned long long* out) {
    unsigned long long c = 0;
    for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x)
        c += owner[n] >= 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, c);
}

}  // namespace

size_t particles_smem_bytes(double R) { return ibb_smem_bytes(R); }

cudaError_t particles_claim(const DeviceState& s, const DeviceParticles& P, cudaStream_t st) {
    if (P.npart == 0) return cudaSuccess;
    k_geom<<<(P.npart + 127) / 128, 128, 0, st>>>(P);
    k_shell<true><<<(P.npart + kShellWarps - 1) / kShellWarps, 32 * kShellWarps, 0, st>>>(P, s.g, P.owner, 1, s.bounds);
    return cudaGetLastError();
}

// Everything that follows a fluid step when spheres are present.
cudaError_t particles_after_step(const DeviceState& s, const DeviceParticles& P, int parity, int have_prev,
                                 cudaStream_t st, const SideStream& side) {
    if (P.npart == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(P.counters, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    // the repulsion reads only the positions and writes only P.rep, the cell
    // list and counters[2], none of which the bounce-back kernel touches: it
    // runs on the side stream while k_ibb runs
    cudaStream_t rs = st;
    if (side.st) {
        if ((e = cudaEventRecord(side.fork, st)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(side.st, side.fork, 0)) != cudaSuccess) return e;
        rs = side.st;
    }
    if (P.ncell > 0) {
        e = cudaMemsetAsync(P.cell_count, 0, (size_t)P.ncell * sizeof(int), rs);
        if (e == cudaSuccess) e = cudaMemsetAsync(P.counters + 2, 0, sizeof(unsigned), rs);
        if (e != cudaSuccess) return e;
        k_bin<<<(P.npart + 255) / 256, 256, 0, rs>>>(P, s.g);
        k_repulsion_cells<<<(P.npart + kRepWarps - 1) / kRepWarps, 32 * kRepWarps, 0, rs>>>(P, s.g);
    } else {
        k_repulsion<<<(P.npart + kRepTile - 1) / kRepTile, kRepTile, 0, rs>>>(P, s.g);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (side.st && (e = cudaEventRecord(side.join, side.st)) != cudaSuccess) return e;
    const size_t smem = ibb_smem_bytes(P.R);
    const bool w32 = ibb_plan(P.R, 32).bytes != 0;
    switch (s.prec) {
        case LBM_PREC_FP64:
            e = w32 ? launch_ibb<double, double, uint32_t>(s, P, parity, smem, st)
                    : launch_ibb<double, double, unsigned long long>(s, P, parity, smem, st);
            break;
        case LBM_PREC_FP32:
            e = w32 ? launch_ibb<float, float, uint32_t>(s, P, parity, smem, st)
                    : launch_ibb<float, float, unsigned long long>(s, P, parity, smem, st);
            break;
        default:
            e = w32 ? launch_ibb<__half, float, uint32_t>(s, P, parity, smem, st)
                    : launch_ibb<__half, float, unsigned long long>(s, P, parity, smem, st);
            break;
    }
    if (e != cudaSuccess) return e;
    if (side.st && (e = cudaStreamWaitEvent(st, side.join, 0)) != cudaSuccess) return e;
    k_newton<<<(P.npart + 127) / 128, 128, 0, st>>>(P, s.g, s.cd.Fx, s.cd.Fy, s.cd.Fz, have_prev);
    k_shell<false><<<(P.npart + kShellWarps - 1) / kShellWarps, 32 * kShellWarps, 0, st>>>(P, s.g, P.owner, 0, s.bounds);
    k_shell<true><<<(P.npart + kShellWarps - 1) / kShellWarps, 32 * kShellWarps, 0, st>>>(P, s.g, P.owner, 0, s.bounds);
    k_reclaim<<<std::max(1, 2 * s.sm_count), 256, 0, st>>>(P, s.g, P.owner);
    // refills: a few per sphere and step; a grid of 4 CTAs per SM strides the list
    const unsigned nb = (unsigned)std::min<long long>((P.refill_cap + 255) / 256, 4LL * std::max(s.sm_count, 1));
    switch (s.prec) {
        case LBM_PREC_FP64: k_refill<double><<<nb, 256, 0, st>>>(s, P, parity); break;
        case LBM_PREC_FP32: k_refill<float><<<nb, 256, 0, st>>>(s, P, parity); break;
        default: k_refill<__half><<<nb, 256, 0, st>>>(s, P, parity); break;
    }
    k_refill_done<<<nb, 256, 0, st>>>(P);
    return cudaGetLastError();
}

// k_ibb, repulsion (k_bin + k_repulsion_cells, or k_repulsion), k_newton,
// two k_shell, k_reclaim, k_refill, k_refill_done
cudaError_t particles_reorder(const DeviceParticles& P, cudaStream_t st) {
    if (P.npart == 0 || !P.order) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(P.order_hist, 0, (size_t)P.order_nbins * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const unsigned nb = (unsigned)((P.npart + 255) / 256);
    k_order_hist<<<nb, 256, 0, st>>>(P);
    k_order_scan<<<1, kScanThreads, 0, st>>>(P);
    k_order_scatter<<<nb, 256, 0, st>>>(P);
    return cudaGetLastError();
}

int particles_kernels_per_step(const DeviceParticles& P) {
    if (P.npart == 0) return 0;
    return P.ncell > 0 ? 9 : 8;
}

cudaError_t particles_count_solid(const DeviceState& s, const DeviceParticles& P, unsigned long long* d_out,
                                  cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_count_solid<<<1024, 256, 0, st>>>(P.owner, s.N, d_out);
    return cudaGetLastError();
}

}  // namespace lbm
