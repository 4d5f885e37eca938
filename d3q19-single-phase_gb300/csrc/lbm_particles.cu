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
//     sphere) gets the population coming back from the wall by quadratic
//     interpolated bounce-back (Bouzidi, Firdaouss & Lallemand 2001) with the
//     moving-wall term, read and written through the AA orientation of the
//     step just taken; the momentum exchanged (Galilean-invariant form, Wen et
//     al. 2014) is reduced per sphere with warp shuffles into FP64 force and
//     torque;
//  3. k_newton, one thread per sphere: soft-sphere repulsion and the FP64
//     Newton-Euler update (second-order Adams-Bashforth);
//  4. k_release / k_claim: node ownership follows the new positions; nodes
//     that leave a sphere are queued;
//  5. k_refill: queued nodes get the equilibrium at the wall velocity plus the
//     non-equilibrium part of the fluid neighbour closest to the outward
//     normal.
// Geometry decisions (inside tests, q, the refill direction) use explicit
// round-to-nearest FP64 operations so that they agree bit for bit with the
// CPU oracle.
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

// Walk a bounding box with a stride of blockDim.x nodes without integer
// division per node; callers put the streamwise (contiguous) axis first so
// that the lanes of a warp touch neighbouring addresses.
struct BoxWalk {
    int a, b, c, na, nb, nc;
    int sa, sb, sc;                       // the stride in mixed radix (na, nb)
    __device__ __forceinline__ BoxWalk(int t, int step, int na_, int nb_, int nc_) : na(na_), nb(nb_), nc(nc_) {
        if (na <= 0 || nb <= 0) { a = b = 0; c = nc; sa = sb = sc = 0; return; }
        a = t % na;
        const int r = t / na;
        b = r % nb;
        c = r / nb;
        sa = step % na;
        const int rs = step / na;
        sb = rs % nb;
        sc = rs / nb;
    }
    __device__ __forceinline__ bool valid() const { return c < nc; }
    __device__ __forceinline__ void advance() {
        a += sa;
        int carry = 0;
        if (a >= na) { a -= na; carry = 1; }
        b += sb + carry;
        carry = 0;
        if (b >= nb) { b -= nb; carry = 1; }
        c += sc + carry;
    }
};

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

// Inside test screened in FP32 (node and centre coordinates rounded to FP32,
// error well below the band); only nodes within the band around the surface
// get the exact FP64 test, which is the one the oracle uses.
struct Centre { double x, y, z; float fx, fy, fz; };
__device__ __forceinline__ Centre centre_of(const DeviceParticles& P, int p) {
    Centre c;
    c.x = P.pos[3 * p]; c.y = P.pos[3 * p + 1]; c.z = P.pos[3 * p + 2];
    c.fx = (float)c.x; c.fy = (float)c.y; c.fz = (float)c.z;
    return c;
}
__device__ __forceinline__ float fmin_image(float d, float L) {
    return d >= 0.5f * L ? d - L : (d < -0.5f * L ? d + L : d);
}
__device__ __forceinline__ float dist2_fast(const Centre& c, const Geometry& g, int ix, int iy, int iz) {
    const float x = ((float)ix + 0.5f) - c.fx;
    const float y = fmin_image(((float)iy + 0.5f) - c.fy, (float)g.NX);
    const float z = fmin_image(((float)iz + 0.5f) - c.fz, (float)g.NY);
    return x * x + y * y + z * z;
}
// 1 inside, 0 outside, -1 undecided (needs the exact FP64 test)
__device__ __forceinline__ int inside_screen(float r2, double R) {
    const float R2 = (float)(R * R);
    const float band = 1e-3f * R2 + 0.05f;
    return r2 < R2 - band ? 1 : (r2 > R2 + band ? 0 : -1);
}

// periodic wrap of an index within one period of [0, n) (all callers stay
// within [-n, 2n): box edges and stencils reach at most R + 3 nodes out)
__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// node-index range of a bounding box along one axis (same rule as the oracle)
struct Range { int lo, n; };
__device__ __forceinline__ Range box(double c, double ext, int n, bool periodic) {
    int a = (int)floor(__dsub_rn(__dsub_rn(c, ext), 0.5));
    int b = (int)ceil(__dsub_rn(__dadd_rn(c, ext), 0.5));
    if (periodic) {
        if (b - a + 1 >= n) { a = 0; b = n - 1; }
    } else {
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
__global__ void __launch_bounds__(kPThreads) k_claim(DeviceParticles P, Geometry g, int* owner) {
    const int p = blockIdx.x;
    const Range rx = box(P.pos[3 * p], P.R, g.NZ, false);
    const Range ry = box(P.pos[3 * p + 1], P.R, g.NX, true);
    const Range rz = box(P.pos[3 * p + 2], P.R, g.NY, true);
    const Centre c = centre_of(P, p);
    for (BoxWalk w(threadIdx.x, blockDim.x, ry.n, rz.n, rx.n); w.valid(); w.advance()) {
        const int iy = wrapi(ry.lo + w.a, g.NX), iz = wrapi(rz.lo + w.b, g.NY), ix = rx.lo + w.c;
        int in = inside_screen(dist2_fast(c, g, ix, iy, iz), P.R);
        if (in < 0) {
            double d[3];
            offset(P, g, p, ix, iy, iz, d);
            in = inside(d, P.R);
        }
        if (in) owner[gnode(g, ix, iy, iz)] = p;
    }
}

__global__ void __launch_bounds__(kPThreads) k_release(DeviceParticles P, Geometry g, int* owner) {
    const int p = blockIdx.x;
    const Centre c = centre_of(P, p);
    const double ext = P.R + 1.5;
    const Range rx = box(P.pos[3 * p], ext, g.NZ, false);
    const Range ry = box(P.pos[3 * p + 1], ext, g.NX, true);
    const Range rz = box(P.pos[3 * p + 2], ext, g.NY, true);
    for (BoxWalk w(threadIdx.x, blockDim.x, ry.n, rz.n, rx.n); w.valid(); w.advance()) {
        const int iy = wrapi(ry.lo + w.a, g.NX), iz = wrapi(rz.lo + w.b, g.NY), ix = rx.lo + w.c;
        const uint32_t n = gnode(g, ix, iy, iz);
        if (owner[n] != p) continue;
        int in = inside_screen(dist2_fast(c, g, ix, iy, iz), P.R);
        if (in < 0) {
            double d[3];
            offset(P, g, p, ix, iy, iz, d);
            in = inside(d, P.R);
        }
        if (in) continue;
        owner[n] = -2;
        const unsigned k = atomicAdd(&P.counters[0], 1u);
        if (k < (unsigned)P.refill_cap) {
            P.refill_node[k] = n;
            P.refill_part[k] = p;
        } else {
            atomicExch(&P.counters[3], 1u);      // refill list overflow
        }
    }
}

// Interpolated bounce-back on every link of sphere blockIdx.x, after a step
// that left the populations in orientation `parity`.  RT: link arithmetic and
// q (FP64 for FP64 storage; FP32 for FP32/FP16 storage, where an FP64 q per
// link would cost more than the fluid step at GB300's FP64 rate), node
// offsets always from FP64 positions, sums in FP64 per node and per sphere.
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
// two-node stencil margin are staged once in shared memory as one byte per
// node (0 fluid, 1 this sphere, 2 another sphere, a node being refilled or
// beyond a wall), together with per-axis tables of the FP32 offset from the
// sphere centre and of the node index.  Phase 1 walks the candidate nodes
// (one per thread, streamwise fastest), finds their links from the staged
// bytes and appends them, with warp-aggregated counts, to 18 per-direction
// buckets.  Phase 2 cuts the buckets into chunks of 32 links of one direction
// and deals the chunks to the warps, so that every lane of a warp works on the
// same direction at neighbouring streamwise nodes.  A link that finds its
// bucket full is processed at once by the thread that found it.
//
// With the AA orientation the six accesses of a link touch the four nodes
// x_f + c_i (solid), x_f, x_f - c_i, x_f - 2c_i in the planes i and opp(i):
// orientation 1 swaps the two planes and moves the slot-i accesses by -c_i
// and the slot-opp(i) accesses by +c_i.
//
// RT: link arithmetic and q (FP64 with correctly rounded operations for FP64
// storage, bit-consistent with the oracle; FP32 with hardware reciprocals for
// FP32/FP16 storage, where an FP64 q per link would cost more than the fluid
// step at GB300's FP64 rate).  Force and torque are summed in FP64 per thread
// and per sphere.

// staged box of one sphere, in shared memory
struct IbbBox {
    int SA, SAB;                  // strides of the staged byte box
    int A0;                       // staged streamwise index of candidate a = 0
    const uint8_t* flag;          // [SC][SB][SA]
    const float *tA, *tB, *tC;    // FP32 offset from the centre per staged index
    const int *wA, *wB, *wC;      // node-index terms per staged index
    const int* wZ;                // wrapped spanwise index per staged b (FP64 path)
    int xlo;                      // wall-normal node of staged c = 0
    float R2f;                    // R^2 in FP32
};

// per-direction constants (warp-uniform in phase 2)
template <typename T, typename RT>
struct IbbDir {
    int i, cx, cy, cz, off;
    RT fcx, fcy, fcz, mw6, qa, inv_qa;
    const T* Pi;
    const T* Pib;
};
template <typename T, typename RT>
__device__ __forceinline__ IbbDir<T, RT> ibb_dir(const DeviceState& s, const IbbBox& B, int i) {
    IbbDir<T, RT> d;
    d.i = i;
    d.cx = cx_rt(i); d.cy = cy_rt(i); d.cz = cz_rt(i);
    d.off = d.cy + B.SA * d.cz + B.SAB * d.cx;
    d.fcx = (RT)d.cx; d.fcy = (RT)d.cy; d.fcz = (RT)d.cz;
    d.mw6 = (RT)(-6.0 * w_rt(i));
    d.qa = (RT)(d.cx * d.cx + d.cy * d.cy + d.cz * d.cz);
    d.inv_qa = d.qa == RT(1) ? RT(1) : RT(0.5);
    d.Pi = plane<T>(s, i);
    d.Pib = plane<T>(s, opp_rt(i));
    return d;
}

struct IbbSphereVel { double U[3], W[3]; };

// One link: staged coordinates (a, b, c) of the fluid node, direction d.i.
// Adds the exchanged momentum and its moment to acc[6].
template <typename T, typename RT>
__device__ __forceinline__ void ibb_link(const DeviceState& s, const DeviceParticles& P, int p, int parity,
                                         const IbbBox& B, const IbbDir<T, RT>& d, int a, int b, int c,
                                         const RT (&UW)[6], RT (&acc)[6]) {
    const int base = a + B.SA * b + B.SAB * c;
    const bool ok1 = B.flag[base - d.off] == 0;
    const bool ok2 = ok1 && B.flag[base - 2 * d.off] == 0;
    const uint32_t gx = (uint32_t)(B.wA[a] + B.wB[b] + B.wC[c]);
    const uint32_t gs = (uint32_t)(B.wA[a + d.cy] + B.wB[b + d.cz] + B.wC[c + d.cx]);
    uint32_t ga = 0, gb = 0;
    if (ok1) ga = (uint32_t)(B.wA[a - d.cy] + B.wB[b - d.cz] + B.wC[c - d.cx]);
    if (ok2) gb = (uint32_t)(B.wA[a - 2 * d.cy] + B.wB[b - 2 * d.cz] + B.wC[c - 2 * d.cx]);
    RT q, d0, d1, d2;
    if constexpr (sizeof(RT) == 8) {
        double dd[3];
        offset(P, s.g, p, B.xlo + c, B.wA[a], B.wZ[b], dd);
        q = link_q<double>(dd, d.cx, d.cy, d.cz, __dsub_rn(norm2_rn(dd), __dmul_rn(P.R, P.R)));
        d0 = dd[0]; d1 = dd[1]; d2 = dd[2];
    } else {
        d0 = B.tC[c]; d1 = B.tA[a]; d2 = B.tB[b];
        const float qc = d0 * d0 + d1 * d1 + d2 * d2 - B.R2f;
        const float qb = d0 * d.fcx + d1 * d.fcy + d2 * d.fcz;
        const float disc = qb * qb - qc * d.qa;
        const float sq = disc > 0.f ? disc * rsqrtf(disc) : 0.f;
        q = (-qb - sq) * d.inv_qa;
        q = q < 1e-6f ? 1e-6f : (q > 1.f ? 1.f : q);
    }
    const RT r0 = d0 + q * d.fcx, r1 = d1 + q * d.fcy, r2 = d2 + q * d.fcz;
    const RT uw0 = UW[0] + (UW[4] * r2 - UW[5] * r1);
    const RT uw1 = UW[1] + (UW[5] * r0 - UW[3] * r2);
    const RT uw2 = UW[2] + (UW[3] * r1 - UW[4] * r0);
    const RT mw = d.mw6 * ((d.fcx * uw0 + d.fcy * uw1) + d.fcz * uw2);
    const RT A = pop_r<T, RT>(s, parity ? d.Pib + gx : d.Pi + gs);
    RT fn;
    if (q < RT(0.5)) {
        if (ok2) {
            const RT Bv = pop_r<T, RT>(s, parity ? d.Pib + ga : d.Pi + gx);
            const RT Cv = pop_r<T, RT>(s, parity ? d.Pib + gb : d.Pi + ga);
            fn = q * (RT(1) + RT(2) * q) * A + (RT(1) - RT(4) * q * q) * Bv + q * (RT(2) * q - RT(1)) * Cv + mw;
        } else if (ok1) {
            const RT Bv = pop_r<T, RT>(s, parity ? d.Pib + ga : d.Pi + gx);
            fn = RT(2) * q * A + (RT(1) - RT(2) * q) * Bv + mw;
        } else {
            fn = A + mw;
        }
    } else {
        if (ok2) {
            const RT D = pop_r<T, RT>(s, parity ? d.Pi + gx : d.Pib + ga);
            const RT E = pop_r<T, RT>(s, parity ? d.Pi + ga : d.Pib + gb);
            if constexpr (sizeof(RT) == 8) {
                const RT k = RT(1) / (q * (RT(2) * q + RT(1)));
                fn = k * A + (RT(2) * q - RT(1)) / q * D - (RT(2) * q - RT(1)) / (RT(2) * q + RT(1)) * E + k * mw;
            } else {
                const float t = 2.f * q + 1.f, k = __fdividef(1.f, q * t), m = 2.f * q - 1.f;
                fn = k * (A + mw) + m * (t * k) * D - m * (q * k) * E;
            }
        } else if (ok1) {
            const RT D = pop_r<T, RT>(s, parity ? d.Pi + gx : d.Pib + ga);
            if constexpr (sizeof(RT) == 8) {
                fn = (A + mw) / (RT(2) * q) + (RT(2) * q - RT(1)) / (RT(2) * q) * D;
            } else {
                const float h = __fdividef(1.f, 2.f * q);
                fn = (A + mw) * h + (2.f * q - 1.f) * h * D;
            }
        } else {
            fn = A + mw;
        }
    }
    put_r<T, RT>(s, const_cast<T*>(parity ? d.Pi + gs : d.Pib + gx), fn);
    // Galilean-invariant momentum exchange
    const RT sA = A + fn, dA = fn - A;
    const RT p0 = d.fcx * sA + uw0 * dA, p1 = d.fcy * sA + uw1 * dA, p2 = d.fcz * sA + uw2 * dA;
    acc[0] += p0; acc[1] += p1; acc[2] += p2;
    acc[3] += r1 * p2 - r2 * p1;
    acc[4] += r2 * p0 - r0 * p2;
    acc[5] += r0 * p1 - r1 * p0;
}

// a link that found its bucket full (rare: the buckets hold the links of a
// whole sphere surface), processed by the thread that found it
template <typename T, typename RT>
__device__ __forceinline__ void ibb_link_cold(const DeviceState& s, const DeviceParticles& P, int p, int parity,
                                           const IbbBox& B, int i, int a, int b, int c, const RT (&UW)[6],
                                           RT (&acc)[6]) {
    const IbbDir<T, RT> d = ibb_dir<T, RT>(s, B, i);
    ibb_link<T, RT>(s, P, p, parity, B, d, a, b, c, UW, acc);
}

// shared-memory plan of k_ibb (bytes from the start of dynamic shared memory)
struct IbbPlan { int bcap, nmax, SAmax, SBmax, flag_off, tab_off, bytes; };
__host__ __device__ inline IbbPlan ibb_plan(double R) {
    IbbPlan pl;
    // links per direction: lattice lines crossing a sphere, <= pi R^2 sqrt(2)
    // on average; a margin, rounded to whole warps
    pl.bcap = ((int)(1.25 * 1.41421356 * 3.14159265 * R * R) + 64 + 31) & ~31;
    pl.nmax = (int)floor(2.0 * (R + 1.5)) + 3;        // candidate nodes per axis
    pl.SAmax = pl.nmax + 10;                            // + margin and 4-node alignment
    pl.SBmax = pl.nmax + 4;
    pl.flag_off = (Q - 1) * pl.bcap * 4;
    pl.tab_off = pl.flag_off + ((pl.SAmax * pl.SBmax * pl.SBmax + 15) & ~15);
    pl.bytes = pl.tab_off + (2 * pl.SAmax + 5 * pl.SBmax) * 4;
    return pl;
}

template <typename T, typename RT>
__global__ void __launch_bounds__(kPThreads, sizeof(RT) == 8 ? 2 : 4)
    k_ibb(DeviceState s, DeviceParticles P, int parity, int vec4) {
    extern __shared__ __align__(16) unsigned char ibb_smem[];
    __shared__ int cnt[Q - 1];
    __shared__ int cpre[Q];
    const Geometry& g = s.g;
    const int p = blockIdx.x;
    const double R = P.R;
    IbbPlan pl = ibb_plan(R);
    if (P.link_bucket > 0 && P.link_bucket < pl.bcap) pl.bcap = P.link_bucket;
    uint32_t* bucket = reinterpret_cast<uint32_t*>(ibb_smem);       // [Q-1][bcap] packed (a,b,c)
    uint8_t* flag = ibb_smem + pl.flag_off;
    float* tA = reinterpret_cast<float*>(ibb_smem + pl.tab_off);
    float* tB = tA + pl.SAmax;
    float* tC = tB + pl.SBmax;
    int* wA = reinterpret_cast<int*>(tC + pl.SBmax);
    int* wB = wA + pl.SAmax;
    int* wC = wB + pl.SBmax;
    int* wZ = wC + pl.SBmax;
    const double ext = R + 1.5;
    const Range rx = box(P.pos[3 * p], ext, g.NZ, false);
    const Range ry = box(P.pos[3 * p + 1], ext, g.NX, true);
    const Range rz = box(P.pos[3 * p + 2], ext, g.NY, true);
    // staged streamwise range starts on a multiple of 4 nodes (16-byte owner loads)
    const int ga0 = (ry.lo - 2) & ~3;
    const int SA = (ry.lo + ry.n + 2 - ga0 + 3) & ~3, SB = rz.n + 4, SC = rx.n + 4, SAB = SA * SB;
    const int A0 = ry.lo - ga0;
    const Centre cen = centre_of(P, p);
    const int cix = (int)floor(cen.x), ciy = (int)floor(cen.y), ciz = (int)floor(cen.z);
    if (threadIdx.x < Q - 1) cnt[threadIdx.x] = 0;
    for (int t = threadIdx.x; t < SA; t += blockDim.x) {
        tA[t] = (float)(ga0 + t - ciy) + (0.5f - (float)(cen.y - ciy));
        wA[t] = wrapi(ga0 + t, g.NX);
    }
    for (int t = threadIdx.x; t < SB; t += blockDim.x) {
        tB[t] = (float)(rz.lo - 2 + t - ciz) + (0.5f - (float)(cen.z - ciz));
        wZ[t] = wrapi(rz.lo - 2 + t, g.NY);
        wB[t] = wZ[t] * g.NX;
    }
    for (int t = threadIdx.x; t < SC; t += blockDim.x) {
        tC[t] = (float)(rx.lo - 2 + t - cix) + (0.5f - (float)(cen.x - cix));
        wC[t] = (rx.lo - 2 + t) * (g.NX * g.NY);
    }
    const int* __restrict__ owner = P.owner;
    if (vec4) {
        // four owner values per 16-byte load (NX is a multiple of 4)
        const int qA = SA >> 2;
        BoxWalk w(threadIdx.x, blockDim.x, qA, SB, SC);
        const int tot = qA * SB * SC;
        for (int done = 0; done < tot; done += 2 * (int)blockDim.x) {
            int4 o[2];
            int li[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                li[u] = -1;
                o[u] = make_int4(-3, -3, -3, -3);
                if (w.valid()) {
                    li[u] = 4 * w.a + SA * w.b + SAB * w.c;
                    const int ix = rx.lo - 2 + w.c;
                    if (ix >= 0 && ix < g.NZ)
                        o[u] = __ldg(reinterpret_cast<const int4*>(
                            owner + gnode(g, ix, wrapi(ga0 + 4 * w.a, g.NX), wrapi(rz.lo - 2 + w.b, g.NY))));
                    w.advance();
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (li[u] < 0) continue;
                const int v[4] = {o[u].x, o[u].y, o[u].z, o[u].w};
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) word |= (uint32_t)(v[k] == -1 ? 0 : (v[k] == p ? 1 : 2)) << (8 * k);
                *reinterpret_cast<uint32_t*>(flag + li[u]) = word;
            }
        }
    } else {
        BoxWalk w(threadIdx.x, blockDim.x, SA, SB, SC);
        for (; w.valid(); w.advance()) {
            const int ix = rx.lo - 2 + w.c;
            int o = -3;
            if (ix >= 0 && ix < g.NZ) o = __ldg(owner + gnode(g, ix, wrapi(ga0 + w.a, g.NX), wrapi(rz.lo - 2 + w.b, g.NY)));
            flag[w.a + SA * w.b + SAB * w.c] = o == -1 ? 0 : (o == p ? 1 : 2);
        }
    }
    IbbBox Bx;
    Bx.SA = SA; Bx.SAB = SAB; Bx.A0 = A0; Bx.flag = flag;
    Bx.tA = tA; Bx.tB = tB; Bx.tC = tC; Bx.wA = wA; Bx.wB = wB; Bx.wC = wC; Bx.wZ = wZ;
    Bx.xlo = rx.lo - 2;
    Bx.R2f = (float)(R * R);
    RT UW[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) { UW[k] = (RT)P.vel[3 * p + k]; UW[3 + k] = (RT)P.omg[3 * p + k]; }
    const float shell2 = (float)((R + 1.5) * (R + 1.5));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    RT acc[6] = {0, 0, 0, 0, 0, 0};
    __syncthreads();
    // phase 1: links of the candidate nodes, from the staged bytes
    {
        const int total = rx.n * ry.n * rz.n;
        const int rounds = (total + blockDim.x - 1) / blockDim.x;
        BoxWalk w(threadIdx.x, blockDim.x, ry.n, rz.n, rx.n);
        for (int round = 0; round < rounds; ++round) {
            unsigned mask = 0;
            int a = 0, b = 0, c = 0;
            if (w.valid()) {
                a = w.a + A0; b = w.b + 2; c = w.c + 2;
                const int base = a + SA * b + SAB * c;
                if (flag[base] == 0 && tA[a] * tA[a] + tB[b] * tB[b] + tC[c] * tC[c] <= shell2) {
#pragma unroll
                    for (int i = 1; i < Q; ++i)
                        if (flag[base + CYf(i) + SA * CZf(i) + SAB * CXf(i)] == 1) mask |= 1u << i;
                }
                w.advance();
            }
            const uint32_t packed = (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16);
            if (!__any_sync(0xffffffffu, mask)) continue;
#pragma unroll
            for (int i = 1; i < Q; ++i) {
                const bool has = (mask >> i) & 1u;
                const unsigned bal = __ballot_sync(0xffffffffu, has);
                if (!bal) continue;
                int b0 = 0;
                if (lane == 0) b0 = atomicAdd(&cnt[i - 1], __popc(bal));
                b0 = __shfl_sync(0xffffffffu, b0, 0);
                if (has) {
                    const int pos = b0 + __popc(bal & lt);
                    if (pos < pl.bcap) bucket[(i - 1) * pl.bcap + pos] = packed;
                    else ibb_link_cold<T, RT>(s, P, p, parity, Bx, i, a, b, c, UW, acc);
                }
            }
        }
    }
    __syncthreads();
    // chunks of 32 links per direction, prefix over the directions
    if (wid == 0) {
        const int n = lane < Q - 1 ? min(cnt[lane], pl.bcap) : 0;
        int v = (n + 31) >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane < Q - 1) cpre[lane + 1] = v;
        if (lane == 0) cpre[0] = 0;
    }
    __syncthreads();
    // phase 2: chunks dealt to the warps
    {
        const int nch = cpre[Q - 1];
        int k = 0;
        for (int ch = wid; ch < nch; ch += nw) {
            while (ch >= cpre[k + 1]) ++k;
            const int e = ((ch - cpre[k]) << 5) + lane;
            if (e >= min(cnt[k], pl.bcap)) continue;
            const IbbDir<T, RT> d = ibb_dir<T, RT>(s, Bx, k + 1);
            const uint32_t v = bucket[k * pl.bcap + e];
            ibb_link<T, RT>(s, P, p, parity, Bx, d, v & 255, (v >> 8) & 255, (v >> 16) & 255, UW, acc);
        }
    }
    // per-sphere FP64 reduction: warp shuffles, then across warps
    __shared__ double sh[6][kPThreads / 32];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double v = (double)acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int ww = 0; ww < nw; ++ww) v += sh[threadIdx.x][ww];
        if (threadIdx.x < 3) P.force[3 * p + threadIdx.x] = v;
        else P.torque[3 * p + threadIdx.x - 3] = v;
    }
    if (threadIdx.x == 0) {
        unsigned nl = 0;
        for (int i = 0; i < Q - 1; ++i) nl += (unsigned)cnt[i];
        atomicAdd(&P.counters[1], nl);
    }
}

size_t ibb_smem_bytes(double R) { return (size_t)ibb_plan(R).bytes; }

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

// Newton-Euler update (second-order Adams-Bashforth, FP64); the body force
// that drives the fluid also acts on the sphere volume.
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
        const double u1 = __dadd_rn(u0, __ddiv_rn(__dsub_rn(__dmul_rn(1.5, Ft), __dmul_rn(0.5, fp)), m));
        P.vel[3 * s + a] = u1;
        P.omg[3 * s + a] = __dadd_rn(P.omg[3 * s + a], __ddiv_rn(__dsub_rn(__dmul_rn(1.5, Tt), __dmul_rn(0.5, tp)), I));
        P.pos[3 * s + a] = __dadd_rn(P.pos[3 * s + a], __dmul_rn(0.5, __dadd_rn(u0, u1)));
        P.fprev[3 * s + a] = Ft;
        P.tprev[3 * s + a] = Tt;
    }
    double y = P.pos[3 * s + 1], z = P.pos[3 * s + 2];
    if (y >= L1) y = __dsub_rn(y, L1);
    else if (y < 0.0) y = __dadd_rn(y, L1);
    if (z >= L2) z = __dsub_rn(z, L2);
    else if (z < 0.0) z = __dadd_rn(z, L2);
    P.pos[3 * s + 1] = y;
    P.pos[3 * s + 2] = z;
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

// Refilling of nodes queued by k_release that are still fluid (-2).
template <typename T>
__global__ void k_refill(DeviceState s, DeviceParticles P, int parity) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned cnt = min(P.counters[0], (unsigned)P.refill_cap);
    if (k >= cnt) return;
    const Geometry& g = s.g;
    const uint32_t n = P.refill_node[k];
    const int* owner = P.owner;
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

__global__ void k_refill_done(DeviceParticles P) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned cnt = min(P.counters[0], (unsigned)P.refill_cap);
    if (k >= cnt) return;
    const uint32_t n = P.refill_node[k];
    if (P.owner[n] == -2) P.owner[n] = -1;
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
    k_claim<<<P.npart, kPThreads, 0, st>>>(P, s.g, P.owner);
    return cudaGetLastError();
}

// Everything that follows a fluid step when spheres are present.
cudaError_t particles_after_step(const DeviceState& s, const DeviceParticles& P, int parity, int have_prev,
                                 cudaStream_t st) {
    if (P.npart == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(P.counters, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    const size_t smem = ibb_smem_bytes(P.R);
    // 16-byte owner loads need rows that start on 4-node boundaries
    const int vec4 = (s.g.NX % 4 == 0 && ((uintptr_t)P.owner & 15) == 0) ? 1 : 0;
    switch (s.prec) {
        case LBM_PREC_FP64:
            e = cudaFuncSetAttribute(k_ibb<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_ibb<double, double><<<P.npart, kPThreads, smem, st>>>(s, P, parity, vec4);
            break;
        case LBM_PREC_FP32:
            e = cudaFuncSetAttribute(k_ibb<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_ibb<float, float><<<P.npart, kPThreads, smem, st>>>(s, P, parity, vec4);
            break;
        default:
            e = cudaFuncSetAttribute(k_ibb<__half, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_ibb<__half, float><<<P.npart, kPThreads, smem, st>>>(s, P, parity, vec4);
            break;
    }
    if (e != cudaSuccess) return e;
    k_repulsion<<<(P.npart + kRepTile - 1) / kRepTile, kRepTile, 0, st>>>(P, s.g);
    k_newton<<<(P.npart + 127) / 128, 128, 0, st>>>(P, s.g, s.cd.Fx, s.cd.Fy, s.cd.Fz, have_prev);
    k_release<<<P.npart, kPThreads, 0, st>>>(P, s.g, P.owner);
    k_claim<<<P.npart, kPThreads, 0, st>>>(P, s.g, P.owner);
    const unsigned nb = (unsigned)((P.refill_cap + 255) / 256);
    switch (s.prec) {
        case LBM_PREC_FP64: k_refill<double><<<nb, 256, 0, st>>>(s, P, parity); break;
        case LBM_PREC_FP32: k_refill<float><<<nb, 256, 0, st>>>(s, P, parity); break;
        default: k_refill<__half><<<nb, 256, 0, st>>>(s, P, parity); break;
    }
    k_refill_done<<<nb, 256, 0, st>>>(P);
    return cudaGetLastError();
}

cudaError_t particles_count_solid(const DeviceState& s, const DeviceParticles& P, unsigned long long* d_out,
                                  cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_count_solid<<<1024, 256, 0, st>>>(P.owner, s.N, d_out);
    return cudaGetLastError();
}

}  // namespace lbm
