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
    init_tables();
#pragma omp parallel for schedule(static)
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

/* initvel, turbulent branch (initial.f90:75-147, one rank: kk = k, jj = j):
 * law-of-the-wall mean profile mirrored about the centre, then the
 * perturbation loop with the reference's constants (A9 = a9, alpha = beta9 =
 * 1, cc = 60).  1-based plane loops as written; each expression keeps the
 * reference's evaluation order. */
void orc_loglaw_velocity(int nx, int ny, int nz, double ustar, double ystar, double a9, double* ux,
                         double* uy, double* uz) {
    const size_t N = (size_t)nx * ny * nz;
    const int nxh = nx / 2;
    const double pi2 = 2.0 * (4.0 * atan(1.0));
    const double A9 = a9, alpha = 1.0, beta9 = 1.0, cc = 60.0;
    const double ccc1 = -((double)ny / pi2 / alpha / ystar * A9 * ustar / cc / cc);
    for (size_t n = 0; n < N; ++n) ux[n] = uy[n] = uz[n] = 0.0;
    for (int i = 1; i <= nxh; ++i) {
        const double yplus = ((double)i - 0.5) / ystar;
        double v;
        if (yplus < 10.8) {
            v = yplus * ustar;
        } else {
            double u9 = log(yplus) / 0.41 + 5.0;
            v = u9 * ustar;
        }
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j) {
                uy[NODE(i - 1, j, k)] = v;
                uy[NODE(nx - i, j, k)] = v;
            }
    }
    for (int k = 1; k <= nz; ++k) {
        const double z9 = pi2 * ((double)k - 0.5) / (double)nz;
        for (int j = 1; j <= ny; ++j) {
            const double y9 = pi2 * ((double)j - 0.5) / (double)ny;
            for (int i = 1; i <= nxh; ++i) {
                const double yplus = ((double)i - 0.5) / ystar;
                const double ccc9 = exp(-yplus / cc);
                double u9 = ccc1 * yplus * ccc9 * sin(alpha * y9 + beta9 * z9);
                uy[NODE(i - 1, j - 1, k - 1)] = uy[NODE(i - 1, j - 1, k - 1)] + u9;
                uy[NODE(nx - i, j - 1, k - 1)] = uy[NODE(nx - i, j - 1, k - 1)] + u9;
                const double ccc10 = A9 * ustar * (1.0 - ccc9 - yplus / cc * ccc9);
                u9 = ccc10 * cos(alpha * y9 + beta9 * z9);
                ux[NODE(i - 1, j - 1, k - 1)] = ux[NODE(i - 1, j - 1, k - 1)] + u9;
                ux[NODE(nx - i, j - 1, k - 1)] = ux[NODE(nx - i, j - 1, k - 1)] + u9;
            }
        }
    }
}

/* =========================================================================
 * Moving spheres.  The reference declares links, fill lists and particle
 * state (var_inc.f90:120-150, para.f90:332-379, solid-node velocity in
 * macrovar collision.f90:420-458) but ships no algorithm; the
 * algorithm below is the project's own design, restated on the CPU as the
 * checker of the GPU kernels:
 *   - geometry: node (ix,iy,iz) (0-based) sits at (ix+1/2, iy+1/2, iz+1/2);
 *     it is solid for sphere p when |r - X_p|^2 <= R^2 (minimal image in the
 *     periodic y and z);
 *   - link (x_f, i): fluid x_f with x_f + c_i inside sphere p; q in (0,1] is
 *     the fraction of c_i from x_f to the surface;
 *   - interpolated bounce-back after streaming (Bouzidi, Firdaouss &
 *     Lallemand 2001): quadratic for q < 1/2, linear for q >= 1/2, with the
 *     moving-wall term -6 w_i c_i.u_w (Lallemand & Luo 2003); falling back to
 *     linear, then to simple bounce-back, when the stencil leaves the fluid
 *     or the domain;
 *   - momentum exchange in the Galilean-invariant form of Wen et al. (2014),
 *     on the stored deviations (the rest-state term 2 w_i rho0 c_i, a pure
 *     geometry sum over the surface, is left out);
 *   - soft-sphere repulsion between spheres and from the walls within zeta,
 *     magnitude stf0 ((zeta-h)/zeta)^2 + stf1 (-h)/zeta for overlap, with the
 *     reference's constants (para.f90:357-360);
 *   - Newton-Euler in FP64, driven by the average of the total force (and
 *     torque) of this step and the previous one: stable for a coupling
 *     stiffness zeta/m < 2, twice the range of second-order Adams-Bashforth,
 *     which light small spheres (radius 4, density ratio 2 at tau ~ 0.504)
 *     exceed; the average also damps the step-to-step oscillation of the
 *     momentum-exchange force.  The body force that drives the fluid also
 *     acts on the sphere volume;
 *   - refilling of uncovered nodes: equilibrium at the local wall velocity
 *     plus the non-equilibrium part of the fluid neighbour closest to the
 *     outward normal (equilibrium + non-equilibrium extrapolation).
 * ========================================================================= */

static double min_image(double d, double L) {
    if (d >= 0.5 * L) d -= L;
    else if (d < -0.5 * L) d += L;
    return d;
}

/* Seeded sphere placement (the reference seeds its particle placement with
 * iseedp, para.f90:362, but ships the placement code in the absent particle
 * library).  Candidate k's attempt a draws three uniforms from the counter
 * generator with consecutive keys; x lies in [R + wall_gap, nx - R - wall_gap],
 * y and z anywhere in the periodic spans; a candidate is accepted when its
 * minimal-image distance to every placed sphere is at least 2R + gap.  The
 * overlap test here is a plain scan over all placed spheres; it accepts and
 * rejects exactly the candidates that a cell-list search would.  Returns 0, or
 * -1 when a sphere cannot be placed in 100000 attempts. */
int orc_particles_place(int nx, int ny, int nz, int npart, double radius, double gap, double wall_gap,
                        uint64_t seed, double* pos) {
    const double lo = radius + wall_gap, hi = (double)nx - radius - wall_gap;
    if (!(hi > lo)) return -1;
    const double dmin = 2.0 * radius + gap;
    uint64_t key = 0;
    for (int k = 0; k < npart; ++k) {
        int placed = 0;
        for (int attempt = 0; attempt < 100000 && !placed; ++attempt) {
            const double x = lo + (hi - lo) * 0.5 * (upm1(seed, key++) + 1.0);
            const double y = ny * 0.5 * (upm1(seed, key++) + 1.0);
            const double z = nz * 0.5 * (upm1(seed, key++) + 1.0);
            int ok = 1;
            for (int j = 0; j < k && ok; ++j) {
                const double d0 = pos[3 * j] - x;
                const double d1 = min_image(pos[3 * j + 1] - y, (double)ny);
                const double d2 = min_image(pos[3 * j + 2] - z, (double)nz);
                if (d0 * d0 + d1 * d1 + d2 * d2 < dmin * dmin) ok = 0;
            }
            if (!ok) continue;
            pos[3 * k] = x;
            pos[3 * k + 1] = y;
            pos[3 * k + 2] = z;
            placed = 1;
        }
        if (!placed) return -1;
    }
    return 0;
}

/* offset from sphere center to node (ix,iy,iz) and the inside test */
static void node_offset(const orc_particles* P, int p, int ix, int iy, int iz, int ny, int nz, double d[3]) {
    d[0] = ((double)ix + 0.5) - P->pos[3 * p + 0];
    d[1] = min_image(((double)iy + 0.5) - P->pos[3 * p + 1], (double)ny);
    d[2] = min_image(((double)iz + 0.5) - P->pos[3 * p + 2], (double)nz);
}
static int inside_d(const double d[3], double R) {
    return (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2] <= R * R;
}

/* bounding-box range along one axis: [lo, hi] of node indices, periodic or not;
 * a periodic range that would cover the whole axis is returned as [0, n-1] */
static void box_range(double c, double ext, int n, int periodic, int* lo, int* hi) {
    int a = (int)floor(c - ext - 0.5), b = (int)ceil(c + ext - 0.5);
    if (periodic) {
        if (b - a + 1 >= n) { a = 0; b = n - 1; }
    } else {
        if (a < 0) a = 0;
        if (b > n - 1) b = n - 1;
    }
    *lo = a; *hi = b;
}
static int wrapi(int a, int n) { a %= n; return a < 0 ? a + n : a; }

void orc_mark_solid(const orc_particles* P, int nx, int ny, int nz, int* owner) {
    const size_t N = (size_t)nx * ny * nz;
    for (size_t n = 0; n < N; ++n) owner[n] = -1;
    for (int p = 0; p < P->npart; ++p) {
        int x0, x1, y0, y1, z0, z1;
        box_range(P->pos[3 * p], P->radius, nx, 0, &x0, &x1);
        box_range(P->pos[3 * p + 1], P->radius, ny, 1, &y0, &y1);
        box_range(P->pos[3 * p + 2], P->radius, nz, 1, &z0, &z1);
        for (int zz = z0; zz <= z1; ++zz)
            for (int yy = y0; yy <= y1; ++yy)
                for (int ix = x0; ix <= x1; ++ix) {
                    const int iy = wrapi(yy, ny), iz = wrapi(zz, nz);
                    double d[3];
                    node_offset(P, p, ix, iy, iz, ny, nz, d);
                    if (inside_d(d, P->radius)) owner[NODE(ix, iy, iz)] = p;
                }
    }
}

/* incompressible deviation equilibrium (initial.f90:26-44 at density rho) */
static void feq_dev(double rho, double ux, double uy, double uz, double* fe) {
    const double usqr = 1.5 * ((ux * ux + uy * uy) + uz * uz);
    fe[0] = weight(0) * (rho - usqr);
    for (int i = 1; i < Q; ++i) {
        const double G = (CX[i] * ux + CY[i] * uy) + CZ[i] * uz;
        fe[i] = weight(i) * (((rho + 3.0 * G) + (4.5 * G) * G) - usqr);
    }
}

static double link_q(const double d[3], int i, double R) {
    const double a = (double)(CX[i] * CX[i] + CY[i] * CY[i] + CZ[i] * CZ[i]);
    const double b = (d[0] * CX[i] + d[1] * CY[i]) + d[2] * CZ[i];
    const double c = ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) - R * R;
    double disc = b * b - a * c;
    if (disc < 0.0) disc = 0.0;
    double q = (-b - sqrt(disc)) / a;
    if (q < 1e-6) q = 1e-6;
    if (q > 1.0) q = 1.0;
    return q;
}

/* Interpolated bounce-back for every link of every sphere on natural
 * post-stream populations F; accumulates force and torque. */
static int ibb_pass(const orc_params* p, orc_particles* P, double* F, int nx, int ny, int nz, const int* owner) {
    int nl = 0;
    const double R = P->radius;
    for (int s = 0; s < P->npart; ++s) {
        double fx = 0, fy = 0, fz = 0, tx = 0, ty = 0, tz = 0;
        const double* U = P->vel + 3 * s;
        const double* W = P->omg + 3 * s;
        int x0, x1, y0, y1, z0, z1;
        box_range(P->pos[3 * s], R + 1.5, nx, 0, &x0, &x1);
        box_range(P->pos[3 * s + 1], R + 1.5, ny, 1, &y0, &y1);
        box_range(P->pos[3 * s + 2], R + 1.5, nz, 1, &z0, &z1);
        for (int zz = z0; zz <= z1; ++zz)
            for (int yy = y0; yy <= y1; ++yy)
                for (int ix = x0; ix <= x1; ++ix) {
                    const int iy = wrapi(yy, ny), iz = wrapi(zz, nz);
                    const size_t xf = NODE(ix, iy, iz);
                    if (owner[xf] != -1) continue;
                    double d[3];
                    node_offset(P, s, ix, iy, iz, ny, nz, d);
                    for (int i = 1; i < Q; ++i) {
                        const int sx = ix + CX[i];
                        if (sx < 0 || sx >= nx) continue;
                        const size_t ys = NODE(sx, wrapi(iy + CY[i], ny), wrapi(iz + CZ[i], nz));
                        if (owner[ys] != s) continue;
                        ++nl;
                        const double q = link_q(d, i, R);
                        const double r0 = d[0] + q * CX[i], r1 = d[1] + q * CY[i], r2 = d[2] + q * CZ[i];
                        const double uw0 = U[0] + (W[1] * r2 - W[2] * r1);
                        const double uw1 = U[1] + (W[2] * r0 - W[0] * r2);
                        const double uw2 = U[2] + (W[0] * r1 - W[1] * r0);
                        const double cu = (CX[i] * uw0 + CY[i] * uw1) + CZ[i] * uw2;
                        const double mw = -6.0 * weight(i) * cu;
                        const int ib = OPP[i];
                        /* stencil nodes x_f - c_i, x_f - 2 c_i */
                        const int ax = ix - CX[i], bx = ix - 2 * CX[i];
                        int ok1 = 0, ok2 = 0;
                        size_t n1 = 0, n2 = 0;
                        if (ax >= 0 && ax < nx) {
                            n1 = NODE(ax, wrapi(iy - CY[i], ny), wrapi(iz - CZ[i], nz));
                            ok1 = owner[n1] == -1;
                        }
                        if (ok1 && bx >= 0 && bx < nx) {
                            n2 = NODE(bx, wrapi(iy - 2 * CY[i], ny), wrapi(iz - 2 * CZ[i], nz));
                            ok2 = owner[n2] == -1;
                        }
                        const double A = F[(size_t)i + Q * ys];
                        double fn;
                        if (q < 0.5) {
                            if (ok2) {
                                const double B = F[(size_t)i + Q * xf], C = F[(size_t)i + Q * n1];
                                fn = q * (1.0 + 2.0 * q) * A + (1.0 - 4.0 * q * q) * B + q * (2.0 * q - 1.0) * C + mw;
                            } else if (ok1) {
                                const double B = F[(size_t)i + Q * xf];
                                fn = 2.0 * q * A + (1.0 - 2.0 * q) * B + mw;
                            } else {
                                fn = A + mw;
                            }
                        } else {
                            /* linear for q >= 1/2 (the quadratic form's extrapolating third
                             * coefficient destabilises narrow gaps at s16 = 1.98) */
                            if (ok1) {
                                const double D = F[(size_t)ib + Q * n1];
                                fn = (A + mw) / (2.0 * q) + (2.0 * q - 1.0) / (2.0 * q) * D;
                            } else {
                                fn = A + mw;
                            }
                        }
                        F[(size_t)ib + Q * xf] = fn;
                        /* Galilean-invariant momentum exchange */
                        const double sA = A + fn, dA = fn - A;
                        const double p0 = CX[i] * sA + uw0 * dA, p1 = CY[i] * sA + uw1 * dA, p2 = CZ[i] * sA + uw2 * dA;
                        fx += p0; fy += p1; fz += p2;
                        tx += r1 * p2 - r2 * p1;
                        ty += r2 * p0 - r0 * p2;
                        tz += r0 * p1 - r1 * p0;
                    }
                }
        P->force[3 * s] = fx; P->force[3 * s + 1] = fy; P->force[3 * s + 2] = fz;
        P->torque[3 * s] = tx; P->torque[3 * s + 1] = ty; P->torque[3 * s + 2] = tz;
    }
    (void)p;
    return nl;
}

static double repulse(double h, double zeta, double k0, double k1) {
    if (h >= zeta) return 0.0;
    const double a = (zeta - h) / zeta;
    double f = k0 * a * a;
    if (h < 0.0) f += k1 * (-h) / zeta;
    return f;
}

/* soft-sphere repulsion, gathered per sphere in index order */
static void repulsion(const orc_particles* P, int nx, int ny, int nz, int s, double out[3]) {
    const double R = P->radius;
    out[0] = out[1] = out[2] = 0.0;
    for (int t = 0; t < P->npart; ++t) {
        if (t == s) continue;
        const double d0 = P->pos[3 * t] - P->pos[3 * s];
        const double d1 = min_image(P->pos[3 * t + 1] - P->pos[3 * s + 1], (double)ny);
        const double d2 = min_image(P->pos[3 * t + 2] - P->pos[3 * s + 2], (double)nz);
        const double dist = sqrt((d0 * d0 + d1 * d1) + d2 * d2);
        const double fm = repulse(dist - 2.0 * R, P->zeta, P->stf0, P->stf1);
        if (fm != 0.0 && dist > 0.0) {
            out[0] -= fm * d0 / dist; out[1] -= fm * d1 / dist; out[2] -= fm * d2 / dist;
        }
    }
    const double hl = P->pos[3 * s] - R, hu = (double)nx - P->pos[3 * s] - R;
    out[0] += repulse(hl, P->zeta, P->stf0_w, P->stf1_w);
    out[0] -= repulse(hu, P->zeta, P->stf0_w, P->stf1_w);
}

static void newton_euler(const orc_params* p, orc_particles* P, int nx, int ny, int nz) {
    const double R = P->radius;
    const double vol = 4.0 / 3.0 * 3.14159265358979323846 * R * R * R;
    const double m = P->rho_ratio * vol, I = 0.4 * m * R * R;
    double* rep = (double*)malloc(sizeof(double) * 3 * (size_t)P->npart);
    for (int s = 0; s < P->npart; ++s) repulsion(P, nx, ny, nz, s, rep + 3 * s);
    for (int s = 0; s < P->npart; ++s) {
        double Ft[3], Tt[3];
        for (int a = 0; a < 3; ++a) {
            Ft[a] = P->force[3 * s + a] + rep[3 * s + a] + p->force[a] * vol;
            Tt[a] = P->torque[3 * s + a];
        }
        if (!P->have_prev)
            for (int a = 0; a < 3; ++a) { P->force_prev[3 * s + a] = Ft[a]; P->torque_prev[3 * s + a] = Tt[a]; }
        for (int a = 0; a < 3; ++a) {
            const double u0 = P->vel[3 * s + a];
            const double u1 = u0 + 0.5 * (Ft[a] + P->force_prev[3 * s + a]) / m;
            P->vel[3 * s + a] = u1;
            P->omg[3 * s + a] += 0.5 * (Tt[a] + P->torque_prev[3 * s + a]) / I;
            P->pos[3 * s + a] += 0.5 * (u0 + u1);
            P->force_prev[3 * s + a] = Ft[a];
            P->torque_prev[3 * s + a] = Tt[a];
        }
        const double L1 = (double)ny, L2 = (double)nz;
        if (P->pos[3 * s + 1] >= L1) P->pos[3 * s + 1] -= L1;
        else if (P->pos[3 * s + 1] < 0.0) P->pos[3 * s + 1] += L1;
        if (P->pos[3 * s + 2] >= L2) P->pos[3 * s + 2] -= L2;
        else if (P->pos[3 * s + 2] < 0.0) P->pos[3 * s + 2] += L2;
    }
    P->have_prev = 1;
    free(rep);
}

static const double INV_SQRT2 = 0.70710678118654752440;

/* geometry update to the new positions and refilling of uncovered nodes */
static int regeometry(const orc_params* p, orc_particles* P, double* F, int nx, int ny, int nz, int* owner) {
    const double R = P->radius;
    size_t cap = 1024, cnt = 0;
    size_t* list = (size_t*)malloc(cap * sizeof(size_t));
    int* lpart = (int*)malloc(cap * sizeof(int));
    /* release: nodes that leave their sphere become pending (-2) */
    for (int s = 0; s < P->npart; ++s) {
        int x0, x1, y0, y1, z0, z1;
        box_range(P->pos[3 * s], R + 1.5, nx, 0, &x0, &x1);
        box_range(P->pos[3 * s + 1], R + 1.5, ny, 1, &y0, &y1);
        box_range(P->pos[3 * s + 2], R + 1.5, nz, 1, &z0, &z1);
        for (int zz = z0; zz <= z1; ++zz)
            for (int yy = y0; yy <= y1; ++yy)
                for (int ix = x0; ix <= x1; ++ix) {
                    const int iy = wrapi(yy, ny), iz = wrapi(zz, nz);
                    const size_t n = NODE(ix, iy, iz);
                    if (owner[n] != s) continue;
                    double d[3];
                    node_offset(P, s, ix, iy, iz, ny, nz, d);
                    if (inside_d(d, R)) continue;
                    owner[n] = -2;
                    if (cnt == cap) {
                        cap *= 2;
                        list = (size_t*)realloc(list, cap * sizeof(size_t));
                        lpart = (int*)realloc(lpart, cap * sizeof(int));
                    }
                    list[cnt] = n; lpart[cnt] = s; ++cnt;
                }
    }
    /* claim: nodes inside the new spheres */
    for (int s = 0; s < P->npart; ++s) {
        int x0, x1, y0, y1, z0, z1;
        box_range(P->pos[3 * s], R, nx, 0, &x0, &x1);
        box_range(P->pos[3 * s + 1], R, ny, 1, &y0, &y1);
        box_range(P->pos[3 * s + 2], R, nz, 1, &z0, &z1);
        for (int zz = z0; zz <= z1; ++zz)
            for (int yy = y0; yy <= y1; ++yy)
                for (int ix = x0; ix <= x1; ++ix) {
                    const int iy = wrapi(yy, ny), iz = wrapi(zz, nz);
                    double d[3];
                    node_offset(P, s, ix, iy, iz, ny, nz, d);
                    if (inside_d(d, R)) owner[NODE(ix, iy, iz)] = s;
                }
    }
    /* refill pending nodes from the fluid neighbour closest to the normal */
    int nref = 0;
    for (size_t k = 0; k < cnt; ++k) {
        const size_t n = list[k];
        if (owner[n] != -2) continue;
        const int s = lpart[k];
        const int ix = (int)(n % (size_t)nx), iy = (int)((n / (size_t)nx) % (size_t)ny), iz = (int)(n / ((size_t)nx * ny));
        double d[3];
        node_offset(P, s, ix, iy, iz, ny, nz, d);
        int best = -1;
        double bs = -1e300;
        size_t bn = 0;
        for (int i = 1; i < Q; ++i) {
            const int sx = ix + CX[i];
            if (sx < 0 || sx >= nx) continue;
            const size_t y = NODE(sx, wrapi(iy + CY[i], ny), wrapi(iz + CZ[i], nz));
            if (owner[y] != -1) continue;
            double sc = (d[0] * CX[i] + d[1] * CY[i]) + d[2] * CZ[i];
            if (i >= 7) sc = sc * INV_SQRT2;
            if (sc > bs) { bs = sc; best = i; bn = y; }
        }
        const double* U = P->vel + 3 * s;
        const double* W = P->omg + 3 * s;
        const double uw0 = U[0] + (W[1] * d[2] - W[2] * d[1]);
        const double uw1 = U[1] + (W[2] * d[0] - W[0] * d[2]);
        const double uw2 = U[2] + (W[0] * d[1] - W[1] * d[0]);
        double fe[Q];
        if (best < 0) {
            feq_dev(0.0, uw0, uw1, uw2, fe);
            for (int i = 0; i < Q; ++i) F[(size_t)i + Q * n] = fe[i];
        } else {
            const double* g = F + Q * bn;
            double r = 0.0, a = 0.0, b = 0.0, c = 0.0;
            for (int i = 0; i < Q; ++i) { r += g[i]; a += CX[i] * g[i]; b += CY[i] * g[i]; c += CZ[i] * g[i]; }
            a += p->force[0] / 2.0; b += p->force[1] / 2.0; c += p->force[2] / 2.0;
            double fn[Q];
            feq_dev(r, a, b, c, fn);
            feq_dev(r, uw0, uw1, uw2, fe);
            for (int i = 0; i < Q; ++i) F[(size_t)i + Q * n] = fe[i] + (g[i] - fn[i]);
        }
        ++nref;
    }
    /* refilled nodes join the fluid only now, so no refill reads another's */
    for (size_t k = 0; k < cnt; ++k)
        if (owner[list[k]] == -2) owner[list[k]] = -1;
    free(list);
    free(lpart);
    return nref;
}

int orc_particle_step(const orc_params* p, orc_particles* P, double* f, int nx, int ny, int nz, int* owner,
                      int* nlinks, int* nrefill) {
    const size_t N = (size_t)nx * ny * nz;
    double* m = (double*)malloc(4 * N * sizeof(double));
    double* g = (double*)malloc((size_t)Q * N * sizeof(double));
    if (!m || !g) { free(m); free(g); return -1; }
    orc_macrovar(p, f, nx, ny, nz, m, m + N, m + 2 * N, m + 3 * N);
    orc_step_push(p, f, g, nx, ny, nz, m, m + N, m + 2 * N, m + 3 * N);
    const int nl = ibb_pass(p, P, g, nx, ny, nz, owner);
    newton_euler(p, P, nx, ny, nz);
    const int nr = regeometry(p, P, g, nx, ny, nz, owner);
    memcpy(f, g, (size_t)Q * N * sizeof(double));
    free(m);
    free(g);
    if (nlinks) *nlinks = nl;
    if (nrefill) *nrefill = nr;
    return 0;
}
