/*
 * FP64 CPU oracle for the D3Q19 channel-flow time step -- TEST
 * INFRASTRUCTURE ONLY (see lbm_oracle.h for who may use it and for its parity
 * status).  Each function restates the mathematics of the reference routine
 * it names; none of the reference's source text is reproduced.
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -fPIC -shared (see
 * oracle/Makefile).  Floating-point contraction is off so that results do not
 * depend on the host CPU's FMA support.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { Q = 19 };

/* d'Humieres (2002) lattice, para.f90:176-214 */
static const int CX[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CY[Q] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CZ[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int OPP[Q] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
/* the reference's split of directions for the swap sweep (para.f90:209-210):
 * "stay" directions point to neighbours not yet visited in z-y-x order,
 * "swap" directions to neighbours already visited */
static const int STAY[10] = {0, 1, 3, 5, 7, 8, 11, 12, 15, 16};
static const int SWAP[9] = {2, 4, 6, 9, 10, 13, 14, 17, 18};

static double weight(int i) { return i == 0 ? 1.0 / 3.0 : (i <= 6 ? 1.0 / 18.0 : 1.0 / 36.0); }

/* Moment matrix, row k as a polynomial in the lattice velocity c (d'Humieres
 * et al. 2002, Phil. Trans. R. Soc. A 360:437, eq. A1): the basis the
 * reference's evlm1..15 and back-transform coefficients val1..val9 encode
 * (collision.f90:103-220, para.f90:143-170).  Order:
 * rho, e, eps, jx, qx, jy, qy, jz, qz, 3pxx, 3pixx, pww, piww, pxy, pyz, pxz,
 * mx, my, mz. */
static int moment_entry(int k, int i) {
    const int x = CX[i], y = CY[i], z = CZ[i];
    const int c2 = x * x + y * y + z * z;
    switch (k) {
        case 0: return 1;
        case 1: return 19 * c2 - 30;
        case 2: return (21 * c2 * c2 - 53 * c2 + 24) / 2;
        case 3: return x;
        case 4: return (5 * c2 - 9) * x;
        case 5: return y;
        case 6: return (5 * c2 - 9) * y;
        case 7: return z;
        case 8: return (5 * c2 - 9) * z;
        case 9: return 3 * x * x - c2;
        case 10: return (3 * c2 - 5) * (3 * x * x - c2);
        case 11: return y * y - z * z;
        case 12: return (3 * c2 - 5) * (y * y - z * z);
        case 13: return x * y;
        case 14: return y * z;
        case 15: return x * z;
        case 16: return x * (y * y - z * z);
        case 17: return y * (z * z - x * x);
        case 18: return z * (x * x - y * y);
    }
    return 0;
}

static int g_M[Q][Q];
static double g_d[Q];
static int g_init = 0;

static void init_tables(void) {
    if (g_init) return;
    for (int k = 0; k < Q; ++k) {
        long s = 0;
        for (int i = 0; i < Q; ++i) {
            g_M[k][i] = moment_entry(k, i);
            s += (long)g_M[k][i] * g_M[k][i];
        }
        g_d[k] = (double)s;
    }
    g_init = 1;
}

void orc_moment_row(int k, int* row, double* norm2) {
    init_tables();
    for (int i = 0; i < Q; ++i) row[i] = g_M[k][i];
    *norm2 = g_d[k];
}

/* Guo-type forcing term of collision.f90:64-82 */
static void force_term(const orc_params* p, double ux, double uy, double uz, double* Fbar) {
    const double fx = p->force[0], fy = p->force[1], fz = p->force[2];
    const double G3 = ux * fx + uy * fy + uz * fz;
    Fbar[0] = -G3;
    for (int i = 1; i < Q; ++i) {
        const double G1 = CX[i] * fx + CY[i] * fy + CZ[i] * fz;
        const double G2 = CX[i] * ux + CY[i] * uy + CZ[i] * uz;
        Fbar[i] = weight(i) * (3.0 * G1 + 9.0 * G1 * G2 - 3.0 * G3);
    }
}

void orc_force_moments(const orc_params* p, double ux, double uy, double uz, double* mf) {
    init_tables();
    double Fbar[Q];
    force_term(p, ux, uy, uz, Fbar);
    for (int k = 0; k < Q; ++k) {
        double s = 0.0;
        for (int i = 0; i < Q; ++i) s += g_M[k][i] * Fbar[i];
        mf[k] = s;
    }
}

/* collision_MRT for one node (collision.f90:56-230): rho and u are the
 * macrovar values the reference reads from its arrays. */
void orc_collide_node(const orc_params* p, const double* f, double rho, double ux, double uy,
                      double uz, double* fpost) {
    init_tables();
    double Fbar[Q], f9[Q], m[Q], meq[Q], s[Q];
    force_term(p, ux, uy, uz, Fbar);
    for (int i = 0; i < Q; ++i) f9[i] = f[i] + 0.5 * Fbar[i];   /* :84 */

    for (int k = 0; k < Q; ++k) {
        double a = 0.0;
        for (int i = 0; i < Q; ++i) a += g_M[k][i] * f9[i];
        m[k] = a;
    }
    /* equilibria (collision.f90:86-101) in delta-rho and j */
    const double usq = ux * ux + uy * uy + uz * uz;
    meq[1] = -11.0 * rho + 19.0 * usq;
    meq[2] = p->omegepsl * rho + p->omegepslj * usq;
    meq[4] = -2.0 / 3.0 * ux;
    meq[6] = -2.0 / 3.0 * uy;
    meq[8] = -2.0 / 3.0 * uz;
    meq[9] = 2.0 * ux * ux - uy * uy - uz * uz;
    meq[10] = p->omegxx * meq[9];
    meq[11] = uy * uy - uz * uz;
    meq[12] = p->omegxx * meq[11];
    meq[13] = ux * uy;
    meq[14] = uy * uz;
    meq[15] = ux * uz;
    meq[16] = meq[17] = meq[18] = 0.0;
    /* rates (collision.f90:140-154) */
    s[1] = p->s1; s[2] = p->s2;
    s[4] = s[6] = s[8] = p->s4;
    s[9] = s[11] = p->s9;
    s[10] = s[12] = p->s10;
    s[13] = s[14] = s[15] = p->s13;
    s[16] = s[17] = s[18] = p->s16;
    double ms[Q];
    for (int k = 0; k < Q; ++k) ms[k] = m[k] - s[k] * (m[k] - meq[k]);
    /* conserved moments come from the macroscopic arrays (tl1, tl6, tl8, tl10) */
    ms[0] = rho; ms[3] = ux; ms[5] = uy; ms[7] = uz;
    /* back-transform f = M^T diag(1/d) m* (collision.f90:157-220), then the
     * second half of the forcing (:230) */
    for (int i = 0; i < Q; ++i) {
        double a = 0.0;
        for (int k = 0; k < Q; ++k) a += g_M[k][i] * (ms[k] / g_d[k]);
        fpost[i] = a + 0.5 * Fbar[i];
    }
}

#define NODE(ix, iy, iz) ((size_t)(ix) + (size_t)nx * ((size_t)(iy) + (size_t)ny * (size_t)(iz)))
#define F(ip, n) f[(size_t)(ip) + (size_t)Q * (n)]

/* macrovar, collision.f90:391-418 */
void orc_macrovar(const orc_params* p, const double* f, int nx, int ny, int nz, double* rho,
                  double* ux, double* uy, double* uz) {
    const size_t N = (size_t)nx * ny * nz;
    for (size_t n = 0; n < N; ++n) {
        const double* g = f + (size_t)Q * n;
        double r = 0.0, a = 0.0, b = 0.0, c = 0.0;
        for (int i = 0; i < Q; ++i) {
            r += g[i];
            a += CX[i] * g[i];
            b += CY[i] * g[i];
            c += CZ[i] * g[i];
        }
        if (rho) rho[n] = r;
        if (ux) ux[n] = a + p->force[0] / 2.0;
        if (uy) uy[n] = b + p->force[1] / 2.0;
        if (uz) uz[n] = c + p->force[2] / 2.0;
    }
}

/* rhoupdat, collision.f90:469-480 */
void orc_rhoupdat(const double* f, int nx, int ny, int nz, double* rho) {
    const size_t N = (size_t)nx * ny * nz;
    for (size_t n = 0; n < N; ++n) {
        double r = f[(size_t)Q * n];
        for (int i = 1; i < Q; ++i) r += f[(size_t)Q * n + i];
        rho[n] = r;
    }
}

/* initpop, initial.f90:26-44 (rho = 0) */
void orc_initpop(int nx, int ny, int nz, const double* ux, const double* uy, const double* uz,
                 double* f) {
    const size_t N = (size_t)nx * ny * nz;
    for (size_t n = 0; n < N; ++n) {
        const double u = ux[n], v = uy[n], w = uz[n];
        const double usqr = 1.5 * ((u * u + v * v) + w * w);
        f[(size_t)Q * n] = weight(0) * (0.0 - usqr);
        for (int i = 1; i < Q; ++i) {
            const double G = (CX[i] * u + CY[i] * v) + CZ[i] * w;
            f[(size_t)Q * n + i] = weight(i) * (((0.0 + 3.0 * G) + (4.5 * G) * G) - usqr);
        }
    }
}

/*
 * collision_MRT + collisionExchnge for a single rank that is its own y and z
 * neighbour (collision.f90:50-372).  The sweep visits nodes in z-y-x order.
 * Each post-collision population either bounces back at an x wall, crosses a
 * y or z face into a send buffer, or is placed with the stay/swap rule.
 * Buffers are filled with NaN first: any slot the exchange reads without the
 * sweep having written it would poison the result.
 */
typedef struct {
    int nx, ny, nz;
    double* yp;   /* leaving through +y: [pop][x][z+1], z in -1..nz */
    double* ym;   /* leaving through -y */
    double* zp;   /* leaving through +z: [pop][x][y], y in 0..ny-1 */
    double* zm;
} faces;

#define YB(b, ip, x, zk) (b)[((size_t)(ip) * fc->nx + (size_t)(x)) * (size_t)(fc->nz + 2) + (size_t)((zk) + 1)]
#define ZB(b, ip, x, yk) (b)[((size_t)(ip) * fc->nx + (size_t)(x)) * (size_t)fc->ny + (size_t)(yk)]

static void deliver(double* f, const faces* fc, int ip, int ix, int iy, int iz, double v, int swap) {
    const int nx = fc->nx, ny = fc->ny, nz = fc->nz;
    const int xm = ix + CX[ip], ym = iy + CY[ip], zm = iz + CZ[ip];
    const size_t here = NODE(ix, iy, iz);
    if (xm < 0 || xm >= nx) {                /* half-way bounce-back */
        F(OPP[ip], here) = v;
    } else if (ym < 0) {
        YB(fc->ym, ip, xm, zm) = v;
    } else if (ym >= ny) {
        YB(fc->yp, ip, xm, zm) = v;
    } else if (zm < 0) {
        ZB(fc->zm, ip, xm, ym) = v;
    } else if (zm >= nz) {
        ZB(fc->zp, ip, xm, ym) = v;
    } else if (!swap) {
        F(OPP[ip], here) = v;
    } else {
        const size_t nb = NODE(xm, ym, zm);
        F(OPP[ip], here) = F(ip, nb);
        F(ip, nb) = v;
    }
}

static void exchange(double* f, const faces* fc) {
    const int nx = fc->nx, ny = fc->ny, nz = fc->nz;
    /* y phase: what left through +y arrives at y = 0; through -y at y = ny-1.
     * Diagonals with an x component skip the x edge that bounced back. */
    static const int up[5] = {3, 7, 8, 15, 17}, dn[5] = {4, 9, 10, 16, 18};
    for (int k = 0; k < 5; ++k) {
        for (int iz = 0; iz < nz; ++iz)
            for (int ix = 0; ix < nx; ++ix) {
                const int ipu = up[k], ipd = dn[k];
                if (!(CX[ipu] == 1 && ix == 0) && !(CX[ipu] == -1 && ix == nx - 1))
                    F(ipu, NODE(ix, 0, iz)) = YB(fc->yp, ipu, ix, iz);
                if (!(CX[ipd] == 1 && ix == 0) && !(CX[ipd] == -1 && ix == nx - 1))
                    F(ipd, NODE(ix, ny - 1, iz)) = YB(fc->ym, ipd, ix, iz);
            }
    }
    /* corners: populations that left through a y face and a z face are
     * forwarded into the z send buffers at their wrapped y position */
    for (int ix = 0; ix < nx; ++ix) {
        ZB(fc->zm, 17, ix, 0) = YB(fc->yp, 17, ix, -1);
        ZB(fc->zm, 18, ix, ny - 1) = YB(fc->ym, 18, ix, -1);
        ZB(fc->zp, 15, ix, 0) = YB(fc->yp, 15, ix, nz);
        ZB(fc->zp, 16, ix, ny - 1) = YB(fc->ym, 16, ix, nz);
    }
    /* z phase */
    static const int zu[5] = {5, 11, 12, 15, 16}, zd[5] = {6, 13, 14, 17, 18};
    for (int k = 0; k < 5; ++k)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const int ipu = zu[k], ipd = zd[k];
                if (!(CX[ipu] == 1 && ix == 0) && !(CX[ipu] == -1 && ix == nx - 1))
                    F(ipu, NODE(ix, iy, 0)) = ZB(fc->zp, ipu, ix, iy);
                if (!(CX[ipd] == 1 && ix == 0) && !(CX[ipd] == -1 && ix == nx - 1))
                    F(ipd, NODE(ix, iy, nz - 1)) = ZB(fc->zm, ipd, ix, iy);
            }
}

int orc_step_swap(const orc_params* p, double* f, int nx, int ny, int nz, const double* rho,
                  const double* ux, const double* uy, const double* uz) {
    faces fcs;
    faces* fc = &fcs;
    fc->nx = nx; fc->ny = ny; fc->nz = nz;
    const size_t ny_sz = (size_t)Q * nx * (nz + 2), nz_sz = (size_t)Q * nx * ny;
    double* buf = (double*)malloc((2 * ny_sz + 2 * nz_sz) * sizeof(double));
    if (!buf) return -1;
    for (size_t i = 0; i < 2 * ny_sz + 2 * nz_sz; ++i) buf[i] = NAN;
    fc->yp = buf; fc->ym = buf + ny_sz; fc->zp = buf + 2 * ny_sz; fc->zm = buf + 2 * ny_sz + nz_sz;

    double fin[Q], fpost[Q];
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const size_t n = NODE(ix, iy, iz);
                memcpy(fin, f + (size_t)Q * n, sizeof(fin));
                orc_collide_node(p, fin, rho[n], ux[n], uy[n], uz[n], fpost);
                for (int k = 0; k < 10; ++k) deliver(f, fc, STAY[k], ix, iy, iz, fpost[STAY[k]], 0);
                for (int k = 0; k < 9; ++k) deliver(f, fc, SWAP[k], ix, iy, iz, fpost[SWAP[k]], 1);
            }
    exchange(f, fc);
    free(buf);
    return 0;
}

static inline int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

static void push_node(const orc_params* p, const double* fin, double* fout, int nx, int ny, int nz,
                      int ix, int iy, int iz, double rho, double ux, double uy, double uz) {
    double fpost[Q];
    const size_t n = NODE(ix, iy, iz);
    orc_collide_node(p, fin + (size_t)Q * n, rho, ux, uy, uz, fpost);
    for (int i = 0; i < Q; ++i) {
        const int xm = ix + CX[i];
        if (xm < 0 || xm >= nx) {
            fout[(size_t)OPP[i] + (size_t)Q * n] = fpost[i];
        } else {
            const size_t m = NODE(xm, wrap(iy + CY[i], ny), wrap(iz + CZ[i], nz));
            fout[(size_t)i + (size_t)Q * m] = fpost[i];
        }
    }
}

void orc_step_push(const orc_params* p, const double* fin, double* fout, int nx, int ny, int nz,
                   const double* rho, const double* ux, const double* uy, const double* uz) {
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const size_t n = NODE(ix, iy, iz);
                push_node(p, fin, fout, nx, ny, nz, ix, iy, iz, rho[n], ux[n], uy[n], uz[n]);
            }
}

int orc_run(const orc_params* p, double* f, int nx, int ny, int nz, int nsteps, int mode,
            double* rho_out, double* ux_out, double* uy_out, double* uz_out) {
    const size_t N = (size_t)nx * ny * nz;
    double* m = (double*)malloc(4 * N * sizeof(double));
    double* g = mode == 1 ? (double*)malloc((size_t)Q * N * sizeof(double)) : NULL;
    if (!m || (mode == 1 && !g)) { free(m); free(g); return -1; }
    double *rho = m, *ux = m + N, *uy = m + 2 * N, *uz = m + 3 * N;
    orc_macrovar(p, f, nx, ny, nz, rho, ux, uy, uz);          /* main.f90:136 */
    for (int s = 0; s < nsteps; ++s) {
        if (mode == 0) {
            if (orc_step_swap(p, f, nx, ny, nz, rho, ux, uy, uz)) { free(m); return -1; }
        } else {
            orc_step_push(p, f, g, nx, ny, nz, rho, ux, uy, uz);
            memcpy(f, g, (size_t)Q * N * sizeof(double));
        }
        orc_macrovar(p, f, nx, ny, nz, rho, ux, uy, uz);      /* main.f90:161 */
    }
    if (rho_out) memcpy(rho_out, rho, N * sizeof(double));
    if (ux_out) memcpy(ux_out, ux, N * sizeof(double));
    if (uy_out) memcpy(uy_out, uy, N * sizeof(double));
    if (uz_out) memcpy(uz_out, uz, N * sizeof(double));
    free(m);
    free(g);
    return 0;
}

/* main.f90:69-90: the density relaxes with the velocity frozen */
int orc_prerelax(const orc_params* p, double* f, int nx, int ny, int nz, const double* ux,
                 const double* uy, const double* uz, double eps, int maxit, int* iters,
                 double* err) {
    const size_t N = (size_t)nx * ny * nz;
    double* rho = (double*)calloc(N, sizeof(double));    /* initpop: rho = 0 */
    double* rhop = (double*)malloc(N * sizeof(double));
    if (!rho || !rhop) { free(rho); free(rhop); return -1; }
    int istep = 0;
    double e = 0.0;
    for (;;) {
        memcpy(rhop, rho, N * sizeof(double));
        orc_rhoupdat(f, nx, ny, nz, rho);
        if (orc_step_swap(p, f, nx, ny, nz, rho, ux, uy, uz)) { free(rho); free(rhop); return -1; }
        e = 0.0;
        for (size_t n = 0; n < N; ++n) {
            const double d = fabs(rho[n] - rhop[n]);
            if (d > e) e = d;
        }
        if (e <= eps || istep > maxit) break;
        ++istep;
    }
    if (iters) *iters = istep;
    if (err) *err = e;
    free(rho);
    free(rhop);
    return e <= eps ? 0 : 1;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* CPU baseline: the same per-node arithmetic, macrovar fused into the sweep,
 * two lattices, z planes distributed over OpenMP threads */
int orc_run_omp(const orc_params* p, double* f, int nx, int ny, int nz, int nsteps, int nthreads) {
    const size_t N = (size_t)nx * ny * nz;
    double* g = (double*)malloc((size_t)Q * N * sizeof(double));
    if (!g) return -1;
    double* a = f;
    double* b = g;
    init_tables();
    for (int s = 0; s < nsteps; ++s) {
#pragma omp parallel for schedule(static) num_threads(nthreads) collapse(2)
        for (int iz = 0; iz < nz; ++iz)
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix) {
                    const double* h = a + (size_t)Q * NODE(ix, iy, iz);
                    double r = 0.0, u = 0.0, v = 0.0, w = 0.0;
                    for (int i = 0; i < Q; ++i) {
                        r += h[i]; u += CX[i] * h[i]; v += CY[i] * h[i]; w += CZ[i] * h[i];
                    }
                    push_node(p, a, b, nx, ny, nz, ix, iy, iz, r, u + p->force[0] / 2.0,
                              v + p->force[1] / 2.0, w + p->force[2] / 2.0);
                }
        double* t = a; a = b; b = t;
    }
    if (a != f) memcpy(f, a, (size_t)Q * N * sizeof(double));
    free(g);
    return 0;
}

/* statistc2 plane sums (saveload.f90:1392-1423), all nodes fluid */
void orc_profiles(const double* rho, const double* ux, const double* uy, const double* uz, int nx,
                  int ny, int nz, double* out) {
    memset(out, 0, sizeof(double) * 12 * (size_t)nx);
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const size_t n = NODE(ix, iy, iz);
                double* o = out + 12 * (size_t)ix;
                const double u = ux[n], v = uy[n], w = uz[n], r = rho[n];
                o[0] += u; o[1] += v; o[2] += w;
                o[3] += u * w; o[4] += u * v; o[5] += v * w;
                o[6] += u * u; o[7] += v * v; o[8] += w * w;
                o[9] += r; o[10] += r * r; o[11] += 1.0;
            }
}

/* counter-based generator shared with the device initial condition */
static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double upm1(uint64_t seed, uint64_t key) {
    const uint64_t z = mix64(seed * 0xD1B54A32D192ED03ull + key);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

void orc_channel_velocity(int nx, int ny, int nz, double uc, double amp, uint64_t seed, double* ux,
                          double* uy, double* uz) {
    const double half = 0.5 * (double)nx;
    const double a = amp * uc;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const size_t n = NODE(ix, iy, iz);
                double xx0 = (double)ix + 0.5 - half;
                if (xx0 < 0) xx0 = -xx0;
                const double prof = (4.0 * uc) * (half * half - xx0 * xx0) / ((double)nx * (double)nx);
                const uint64_t lin = (uint64_t)n;
                ux[n] = a * upm1(seed, 3 * lin + 0);
                uy[n] = prof + a * upm1(seed, 3 * lin + 1);
                uz[n] = a * upm1(seed, 3 * lin + 2);
            }
}
