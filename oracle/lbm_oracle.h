/*
 * FP64 CPU oracle for the D3Q19 channel-flow time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path: it
 * may be loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg, never by the product library or its Python package.
 *
 * Parity status: the reference (Fortran 90 + MPI) cannot be compiled in this
 * environment (no Fortran compiler, no MPI) and ships no test vectors, so the
 * oracle is pinned by the reference's only known answer -- the analytic
 * Poiseuille start-up series written by outputuy (saveload.f90:920-936) -- and
 * by self-consistency: the sequential swap sweep with the reference's
 * exchange rules and an independent two-lattice push must agree bit for bit.
 * There are no executed-reference vectors ("parity unpinned" against the
 * Fortran binary itself).
 *
 * Arrays use the reference layout: f(0:18,nx,ny,nz) column-major, macroscopic
 * fields (nx,ny,nz); x wall-normal, y streamwise, z spanwise.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H
#include <stdint.h>

typedef struct orc_params {
    double s1, s2, s4, s9, s10, s13, s16;   /* para.f90:106-141 */
    double omegepsl, omegepslj, omegxx;
    double force[3];                        /* FORCING, collision.f90:522-524 */
} orc_params;

/* one node of collision_MRT: pre-collision f, macroscopic rho/u -> f* */
void orc_collide_node(const orc_params* p, const double* f, double rho, double ux,
                      double uy, double uz, double* fpost);
/* M Fbar evaluated numerically (19 moments) for the closed-form check */
void orc_force_moments(const orc_params* p, double ux, double uy, double uz, double* mf);
/* moment matrix row k (19 integers) and its squared norm */
void orc_moment_row(int k, int* row, double* norm2);

void orc_macrovar(const orc_params* p, const double* f, int nx, int ny, int nz,
                  double* rho, double* ux, double* uy, double* uz);
void orc_initpop(int nx, int ny, int nz, const double* ux, const double* uy,
                 const double* uz, double* f);
void orc_rhoupdat(const double* f, int nx, int ny, int nz, double* rho);

/* collision_MRT + collisionExchnge on one rank with periodic y/z neighbours
 * (the rank is its own neighbour in both directions), in place */
int orc_step_swap(const orc_params* p, double* f, int nx, int ny, int nz,
                  const double* rho, const double* ux, const double* uy,
                  const double* uz);
/* same physics as a two-lattice push, fin -> fout */
void orc_step_push(const orc_params* p, const double* fin, double* fout, int nx,
                   int ny, int nz, const double* rho, const double* ux,
                   const double* uy, const double* uz);

/* main.f90:136-161: macrovar, then nsteps x (collision + exchange + macrovar).
 * mode 0: swap sweep, mode 1: two-lattice push.  Macro arrays (may be NULL)
 * receive the final macrovar. */
int orc_run(const orc_params* p, double* f, int nx, int ny, int nz, int nsteps,
            int mode, double* rho, double* ux, double* uy, double* uz);

/* main.f90:69-90 with rhoupdat; returns 0, or 1 if not converged */
int orc_prerelax(const orc_params* p, double* f, int nx, int ny, int nz,
                 const double* ux, const double* uy, const double* uz, double eps,
                 int maxit, int* iters, double* err);

/* CPU baseline: fused macro+collide+push over nsteps with OpenMP threads */
int orc_run_omp(const orc_params* p, double* f, int nx, int ny, int nz, int nsteps,
                int nthreads);
int orc_max_threads(void);

/* plane sums of statistc2 (12 columns per wall-normal plane) */
void orc_profiles(const double* rho, const double* ux, const double* uy,
                  const double* uz, int nx, int ny, int nz, double* out);

/* channel initial velocity: Poiseuille + counter-based noise (same bits as
 * the device initial condition) */
void orc_channel_velocity(int nx, int ny, int nz, double uc, double amp,
                          uint64_t seed, double* ux, double* uy, double* uz);

/* initvel's turbulent branch (initial.f90:101-147): law-of-the-wall profile
 * plus the perturbation with amplitude a9 (A9, 0 as shipped) */
void orc_loglaw_velocity(int nx, int ny, int nz, double ustar, double ystar, double a9,
                         double* ux, double* uy, double* uz);

/* seeded non-overlapping sphere centres (reference axes, 3*npart): the same
 * counter-generator draws and acceptance rule as the library's placement;
 * returns 0, or -1 if the spheres do not fit */
int orc_particles_place(int nx, int ny, int nz, int npart, double radius, double gap,
                        double wall_gap, uint64_t seed, double* pos);

/* ---- moving spheres (the reference declares the data but ships no
 * algorithm; this is the project's own design, restated here as
 * the checker of the GPU kernels) ---------------------------------------- */
typedef struct orc_particles {
    int npart;
    double radius, rho_ratio;
    double stf0, stf1, stf0_w, stf1_w, zeta;
    double *pos, *vel, *omg;          /* 3*npart each, reference axes        */
    double *force, *torque;           /* hydrodynamic, last step (3*npart)   */
    double *force_prev, *torque_prev; /* total of the previous step         */
    int have_prev;
} orc_particles;

/* owner[n] = particle id of the node, -1 for fluid (reference layout) */
void orc_mark_solid(const orc_particles* P, int nx, int ny, int nz, int* owner);
/* one full particle-laden step on natural-orientation populations:
 * push step -> interpolated bounce-back + momentum exchange -> repulsion ->
 * Newton-Euler -> geometry update -> refilling */
int orc_particle_step(const orc_params* p, orc_particles* P, double* f, int nx, int ny, int nz,
                      int* owner, int* nlinks, int* nrefill);

#endif
