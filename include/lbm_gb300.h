/*
 * lbm_gb300.h - C ABI of the GB300 (sm_103a) D3Q19 channel-flow time step.
 *
 * The reference (UDel-CFD/D3Q19-Single-Phase, Fortran 90 + MPI) exposes its
 * hot path as argument-less subroutines working on module globals
 * (Channel-Flow/var_inc.f90:84-150).  This header replaces them with explicit
 * calls on an opaque context that owns all device state:
 *
 *   reference subroutine                         replaced by
 *   ------------------------------------------   -------------------------------
 *   para (rates, lattice, para.f90:106-214)      lbm_params_init / lbm_create
 *   FORCING (collision.f90:515-527)              lbm_params.force[3]
 *   initpop (initial.f90:19-46)                  lbm_initpop
 *   initvel + initpop for the channel configs    lbm_init_channel (device IC)
 *   initvel turbulent branch + initpop           lbm_init_loglaw (device IC)
 *     (initial.f90:75-147, ivel = .true.)
 *   collision_MRT + collisionExchnge + macrovar  lbm_step
 *     (collision.f90:24-273, 281-372, 378-463;
 *      call order main.f90:157-161)
 *   rhoupdat + pre-relaxation loop               lbm_prerelax
 *     (collision.f90:469-480, main.f90:69-90)
 *   macrovar results rho, ux, uy, uz             lbm_macrovar
 *   f(0:18,lx,ly,lz) in memory                   lbm_upload_f / lbm_download_f
 *   avedensity (collision.f90:487-513)           lbm_avedensity
 *   diag / statistc / statistc2 sums             lbm_diag / lbm_profiles
 *     (saveload.f90:1202-1676)
 *   saveinitflow / savecntdflow /                lbm_save_flow / lbm_load_flow
 *   loadinitflow / loadcntdflow
 *     (saveload.f90:102-231, 296-332)
 *
 * Conventions
 *  - Every call returns 0 (LBM_OK) or a negative LBM_ERR_* code; nothing
 *    exits or throws across the ABI.  lbm_strerror() gives a message and
 *    lbm_last_error() the detail of the most recent failure on this thread.
 *  - Host arrays use the reference layout and axes: f(0:18,nx,ny,nz) in
 *    Fortran (column-major) order, i.e. flat index
 *    ip + 19*((ix-1) + nx*((iy-1) + ny*(iz-1))); macroscopic arrays are
 *    (nx,ny,nz).  x is wall-normal (half-way bounce-back walls at x=1/2 and
 *    x=nx+1/2), y is streamwise and z spanwise, both periodic.  Population
 *    order is d'Humieres et al. (2002) as in para.f90:176-214.
 *  - Populations are deviations from the rest state (f_i - w_i rho0), the
 *    reference's own stored variable (initial.f90:26-44).  All host arrays are
 *    double precision, the reference's -r8 REAL.
 *  - Host pointers are borrowed only for the duration of a call.  Calls are
 *    synchronous at the ABI edge unless named *_async.  One host thread per
 *    context; one GPU and one CUDA stream per context (lbm_stream): every
 *    call's work is ordered on it.  With spheres, the sphere pass forks the
 *    repulsion onto a second stream of the context and joins it back on the
 *    context's stream before the Newton-Euler update.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    LBM_OK = 0,
    LBM_ERR_INVALID_ARG = -1,   /* bad pointer, size or parameter            */
    LBM_ERR_CUDA = -2,          /* a CUDA runtime call failed                */
    LBM_ERR_OOM = -3,           /* device or pinned host allocation failed   */
    LBM_ERR_STATE = -4,         /* call not valid in the context's state     */
    LBM_ERR_NOT_CONVERGED = -5, /* pre-relaxation hit its iteration limit    */
    LBM_ERR_IO = -6,            /* checkpoint file missing/short/corrupt     */
    LBM_ERR_NONFINITE = -7,     /* NaN/Inf detected in the populations       */
    LBM_ERR_UNSUPPORTED = -8    /* feature not available in this build/GPU   */
};

/* ---- storage precision of the populations -------------------------------- */
enum {
    LBM_PREC_FP64 = 0,  /* FP64 storage, FP64 arithmetic (parity path)           */
    LBM_PREC_FP32 = 1,  /* FP32 storage, FP32 arithmetic                         */
    LBM_PREC_FP16 = 2   /* FP16 storage of scale*(f_i - w_i), FP32 arithmetic    */
};

/* MRT rate sets of para.f90:110-141 */
enum { LBM_MRT_STABLE = 1, LBM_MRT_LBGK = 2, LBM_MRT_LOWDISS = 3 };

/*
 * Run parameters.  Mirrors the scalar globals that para.f90 computes and
 * collision_MRT reads (var_inc.f90:85-93).  Fill it with lbm_params_init()
 * and override fields, or copy them from an existing para.f90 run.
 */
typedef struct lbm_params {
    int32_t nx, ny, nz;       /* lattice size, reference axes (var_inc.f90:51) */
    int32_t precision;        /* LBM_PREC_*                                    */
    double  s1, s2, s4, s9, s10, s13, s16;  /* MRT relaxation rates            */
    double  omegepsl, omegepslj, omegxx;    /* equilibrium coefficients        */
    double  force[3];         /* uniform body force (force_realx/y/z)          */
    double  fp16_scale;       /* fixed FP16 storage scale (0 -> 32768)         */
    int32_t device;           /* CUDA device ordinal                           */
    int32_t flags;            /* LBM_FLAG_* bits                               */
} lbm_params;

/* lbm_params.flags: use the one-node-per-thread step kernels even where the
 * row-pipelined bulk-copy kernels apply (FP32/FP16 storage, 16-byte rows). */
#define LBM_FLAG_SIMPLE_STEP 1

/* Global diagnostics over fluid nodes (diag, saveload.f90:1507-1676, plus the
 * mass and momentum sums of avedensity, collision.f90:487-513).  Velocities
 * are the macrovar ones (momentum including F/2), reference axes. */
typedef struct lbm_stats {
    int64_t nfluid;           /* fluid node count                              */
    double  rho_sum;          /* sum of delta-rho (mass drift monitor)         */
    double  mom_sum[3];       /* sum of ux, uy, uz                             */
    double  usq_sum[3];       /* sum of ux^2, uy^2, uz^2                       */
    double  rho_max, rho_min; /* extreme delta-rho                             */
    double  vmax;             /* max |u|                                       */
    int32_t vmax_at[3];       /* 1-based (ix,iy,iz) of vmax                    */
    int32_t nonfinite;        /* number of nodes with a NaN/Inf population     */
} lbm_stats;

/* Number of columns lbm_profiles writes per wall-normal plane; the order is
 * sum over the plane of: ux, uy, uz, ux*uz, ux*uy, uy*uz, ux^2, uy^2, uz^2,
 * rho, rho^2, fluid count (the sums of statistc2, saveload.f90:1392-1423). */
#define LBM_PROFILE_COLS 12
#define LBM_DISSIPATION_COLS 5

typedef struct lbm_ctx lbm_ctx;

const char* lbm_strerror(int code);
const char* lbm_last_error(void);
int lbm_version(void);

/* Fill p with the para.f90 values for the given lattice, MRT type
 * (para.f90:106-141: s9 = s13 = 1/(3 visc + 0.5)) and streamwise body force
 * (applied along reference y, FORCING collision.f90:522-524). */
int lbm_params_init(lbm_params* p, int32_t nx, int32_t ny, int32_t nz,
                    int32_t mrt_type, double visc, double force_y,
                    int32_t precision);

/* Allocate device state for p (populations in HBM, SoA, in-place).  Replaces
 * allocarray (para.f90:418-447) for the fluid arrays. */
int lbm_create(const lbm_params* p, lbm_ctx** out);
int lbm_destroy(lbm_ctx* ctx);

/* Device bytes held by the context. */
int lbm_device_bytes(const lbm_ctx* ctx, size_t* bytes);

/* Populations in the reference layout f(0:18,nx,ny,nz), natural
 * (post-streaming) orientation, FP64.  Upload resets the step parity. */
int lbm_upload_f(lbm_ctx* ctx, const double* f);
int lbm_download_f(lbm_ctx* ctx, double* f);

/* initpop (initial.f90:19-46): f = equilibrium at delta-rho = 0 for the given
 * velocity arrays (nx,ny,nz). */
int lbm_initpop(lbm_ctx* ctx, const double* ux, const double* uy,
                const double* uz);

/* Device-side initial condition for the channel configurations: laminar
 * Poiseuille profile along y with centreline velocity uc (the analytic
 * steady solution of saveload.f90:926) plus uniform random perturbations of
 * +-amp*uc in all three components drawn from a counter-based generator
 * (splitmix64 of seed and node index), then initpop.  Host code can
 * reproduce the same field exactly; see lbm_channel_velocity. */
int lbm_init_channel(lbm_ctx* ctx, double uc, double amp, uint64_t seed);

/* Host-side copy of the velocity field lbm_init_channel builds (arrays of
 * nx*ny*nz doubles, reference layout). Needs no context or GPU. */
int lbm_channel_velocity(int32_t nx, int32_t ny, int32_t nz, double uc,
                         double amp, uint64_t seed, double* ux, double* uy,
                         double* uz);

/* initvel's turbulent branch + initpop on the device (initial.f90:101-147,
 * the ivel = .true. start of para.f90:59-72, and initial.f90:19-46): the
 * law-of-the-wall streamwise profile u_y = y+ u* for y+ < 10.8, else
 * u*(ln(y+)/0.41 + 5), y+ = (i - 1/2)/ystar for the wall-normal planes
 * i = 1..nx/2, mirrored onto planes nx+1-i (with odd nx the middle plane
 * stays at rest), plus initvel's perturbation with amplitude a9 (the
 * reference's A9, 0.0 as shipped, which makes it vanish):
 *   u_y += A9'(y+) sin(y9 + z9),  u_x += A9 u* (1 - e - y+ e/60) cos(y9 + z9),
 *   e = exp(-y+/60), A9'(y+) = -ny/(2 pi) /ystar * A9 u* / 60^2 * y+ e,
 *   y9 = 2 pi (j - 1/2)/ny, z9 = 2 pi (k - 1/2)/nz;
 * then f = equilibrium at delta-rho = 0.  ystar = visc/ustar (para.f90:66).
 * The transcendental factors are evaluated on the host (one per wall plane
 * and per column); lbm_loglaw_velocity returns the identical field. */
int lbm_init_loglaw(lbm_ctx* ctx, double ustar, double ystar, double a9);

/* Host-side copy of the velocity field lbm_init_loglaw builds (arrays of
 * nx*ny*nz doubles, reference layout); the velocity arrays the
 * pre-relaxation (lbm_prerelax) needs.  Needs no context or GPU. */
int lbm_loglaw_velocity(int32_t nx, int32_t ny, int32_t nz, double ustar,
                        double ystar, double a9, double* ux, double* uy,
                        double* uz);

/* nsteps x (collision_MRT + periodic exchange + macrovar); synchronous. */
int lbm_step(lbm_ctx* ctx, int32_t nsteps);
/* Same, enqueued on the context's stream without waiting. */
int lbm_step_async(lbm_ctx* ctx, int32_t nsteps);
int lbm_synchronize(lbm_ctx* ctx);
/* Per-step CUDA-event timing inside lbm_step: with timing enabled (capacity =
 * steps to record), every step records events around its fluid kernel and
 * around the particle kernels that follow it.  lbm_timing_get returns the
 * summed milliseconds of the recorded steps (fluid kernels of even and odd
 * steps separately) and the number recorded; it synchronizes the stream. */
int lbm_timing_enable(lbm_ctx* ctx, int32_t capacity);
int lbm_timing_get(lbm_ctx* ctx, double* fluid_even_ms, double* fluid_odd_ms,
                   double* particle_ms, int64_t* steps_even, int64_t* steps_odd);
/* Kernels launched by lbm_step / lbm_step_async on this context since it was
 * created: one step kernel per step, plus the sphere pass (8 or 9 kernels)
 * and, every 100 steps with spheres, the two kernels of the mean-density
 * removal and the three that re-sort the spheres into the bounce-back
 * kernel's spatial order.  No counterpart in the reference (instrumentation
 * of the step). */
int lbm_step_launches(const lbm_ctx* ctx, int64_t* nlaunch);
/* The context's cudaStream_t, for event timing by the caller. */
int lbm_stream(lbm_ctx* ctx, void** stream);
/* Steps taken since the last upload / init. */
int lbm_step_count(const lbm_ctx* ctx, int64_t* nsteps);
/* Set the step counter, e.g. to istep0 after loadcntdflow, so that the
 * every-100-steps work of the main loop (main.f90:163) keeps the absolute
 * step numbering of the run being continued. */
int lbm_set_step_count(lbm_ctx* ctx, int64_t nsteps);

/* Density pre-relaxation of main.f90:69-90 with the velocity frozen at
 * (ux,uy,uz) (arrays (nx,ny,nz)): repeat {rho = sum f (rhoupdat);
 * collision with the frozen velocity} until max|rho - rho_prev| <= eps or the
 * iteration counter exceeds maxit.  iters/err receive the final counter and
 * residual.  Returns LBM_ERR_NOT_CONVERGED only if maxit was exceeded.
 * ux = uy = uz = NULL freezes the velocity of the current populations
 * instead (sum_i c_i f_i, which is the initial velocity itself right after
 * lbm_initpop, lbm_init_channel or lbm_init_loglaw), so a device initial
 * condition needs no host velocity arrays. */
int lbm_prerelax(lbm_ctx* ctx, const double* ux, const double* uy,
                 const double* uz, double eps, int32_t maxit, int32_t* iters,
                 double* err);

/* macrovar (collision.f90:378-418): rho = sum f, u = sum c f + F/2, written to
 * host arrays (nx,ny,nz); any pointer may be NULL to skip it. */
int lbm_macrovar(lbm_ctx* ctx, double* rho, double* ux, double* uy,
                 double* uz);

/* Global fluid-node diagnostics (diag) computed on the device in FP64. */
int lbm_diag(lbm_ctx* ctx, lbm_stats* st);

/* S_ij S_ij of the strain rate from the non-equilibrium populations, per
 * node, both methods of sijstat01 (saveload.f90:2320-2432): m1 from the
 * non-equilibrium moments (Yu et al. 2006), m2 from f - f^eq in population
 * space.  Host arrays of nx*ny*nz doubles in the reference layout (either may
 * be NULL); solid nodes give 0. */
int lbm_strain(lbm_ctx* ctx, double* sij2_m1, double* sij2_m2);

/* Plane sums of dissipation_calc (saveload.f90:4644-4882) over the fluid
 * nodes of each wall-normal plane: out[LBM_DISSIPATION_COLS*nx] with column c
 * of plane ix at out[c + LBM_DISSIPATION_COLS*(ix-1)]: S_ij S_ij from the
 * non-equilibrium moments (method 1), from f - f^eq (method 2), S_xy of both
 * methods (x wall-normal, y streamwise), each with the reference's formula
 * and sign: -1.5 neqm13 (= +du_y/dx / 2 in a shear flow u_y(x)) and
 * (1.5/tau) sum f_neq c_x c_y (= -du_y/dx / 2), and the fluid node count.  Divided
 * by the count they are the columns 3-6 of dissipation.dat; epsilon =
 * 2 nu <S_ij S_ij>.  FP64 per node. */
int lbm_dissipation(lbm_ctx* ctx, double* out);
/* Plane sums for statistc/statistc2: out[LBM_PROFILE_COLS*nx], column-major
 * (column c of plane ix at out[c + LBM_PROFILE_COLS*(ix-1)]). FP64. */
int lbm_profiles(lbm_ctx* ctx, double* out);

/* The plane sums of lbm_profiles, computed without allocating anything.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc when they want the statistics -- a monitor sampling profiles
 * while the solver owns a fixed memory budget, code running between the
 * captures of a CUDA graph, or a host whose allocator is not the CUDA
 * runtime's.  (lbm_profiles may allocate its reduction buffer on first use.)
 * The partial sums live in a device array compiled into the library, sized
 * for at most LBM_NOALLOC_MAX_PLANES wall-normal planes (about 2 MB, held on
 * every GPU that loads the library until the process exits); a context with
 * nx above that is rejected with LBM_ERR_INVALID_ARG.  The first call on a
 * device looks up that array's device address, so make the first call before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU race with each other.  Each call overwrites every entry it reads, so
 * results never depend on a previous call.  On success no host memory is
 * allocated either.  out: LBM_PROFILE_COLS*nx doubles, as lbm_profiles. */
#define LBM_NOALLOC_MAX_PLANES 4096
int lbm_profiles_noalloc(lbm_ctx* ctx, double* out);

/* avedensity (collision.f90:487-513): subtract the fluid-mean delta-rho from
 * every node; here applied to the rest population so that rho = sum f moves
 * by the mean.  mean (may be NULL) receives the value removed. */
int lbm_avedensity(lbm_ctx* ctx, double* mean);

/* Checkpoints in the reference's Fortran unformatted sequential format (4-byte
 * record markers, gfortran sub-records above 2 GiB):
 *   kind 0: finit.NNN   = {istat}{f}             (saveinitflow, :102-124)
 *   kind 1: endrunflow  = {istep,istat,imovie}{f} (savecntdflow, :196-231)
 * f is FP64, natural orientation, reference layout.  ints[] carries the
 * integer header (1 or 3 values). */
int lbm_save_flow(lbm_ctx* ctx, const char* path, int32_t kind,
                  const int32_t* ints);
int lbm_load_flow(lbm_ctx* ctx, const char* path, int32_t kind,
                  int32_t* ints);

/* ---- moving spheres ------------------------------------------------------
 * The reference declares particle state, links and fill lists
 * (var_inc.f90:120-150, para.f90:332-379, macrovar's solid branch
 * collision.f90:420-458) but ships no particle algorithm.  With spheres set,
 * every lbm_step also does: interpolated bounce-back (Bouzidi, quadratic for
 * q < 1/2 and linear for q >= 1/2, moving wall) and Galilean-invariant
 * momentum exchange on every boundary
 * link, soft-sphere repulsion (sphere-sphere and sphere-wall), the FP64
 * Newton-Euler update (driven by the average of this step's and the previous
 * step's force and torque), the geometry update and
 * the refilling of uncovered nodes.  Positions are in reference axes with node
 * (ix,iy,iz) (1-based) at (ix-1/2, iy-1/2, iz-1/2), as in macrovar. */
typedef struct lbm_particle_params {
    int32_t npart;            /* number of spheres (npart, var_inc.f90:66)     */
    int32_t flags;            /* LBM_PFLAG_* bits                              */
    double  radius;           /* rad (var_inc.f90:67)                          */
    double  rho_ratio;        /* rhopart / rho0                                */
    double  stf0, stf1;       /* sphere-sphere repulsion (para.f90:357-358)    */
    double  stf0_w, stf1_w;   /* sphere-wall repulsion (para.f90:359-360)      */
    double  zeta;             /* repulsion range, lattice units                */
} lbm_particle_params;

/* lbm_particle_params.flags: compute the boundary-link fractions q in FP64
 * for FP32/FP16 storage too (default: FP32 from the FP64 centre split into an
 * exact integer part and an FP32 fraction, |dq| < 1e-5; FP64 q costs about
 * 20 FP64 operations per link at GB300's 1/64 FP64 rate). */
#define LBM_PFLAG_Q_FP64 1

/* Defaults of para.f90:339-379 for npart spheres of the given radius. */
int lbm_particle_params_init(lbm_particle_params* pp, int32_t npart, double radius,
                             double rho_ratio);
/* Seeded random placement (counter-based generator): centres uniform in the
 * domain, at least `gap` lattice units between sphere surfaces (periodic in
 * y and z) and `wall_gap` between a surface and a wall.  pos: 3*npart. */
int lbm_particles_place(int32_t nx, int32_t ny, int32_t nz, int32_t npart,
                        double radius, double gap, double wall_gap,
                        uint64_t seed, double* pos);
/* Attach spheres to a context (allocates the node ownership array and the
 * particle state on the device) and mark the solid nodes.  vel/omg may be
 * NULL (zero). */
int lbm_particles_set(lbm_ctx* ctx, const lbm_particle_params* pp,
                      const double* pos, const double* vel, const double* omg);
/* Particle state after the last step; any pointer may be NULL.  force and
 * torque are the hydrodynamic (momentum-exchange) parts of the last step. */
int lbm_particles_get(lbm_ctx* ctx, double* pos, double* vel, double* omg,
                      double* force, double* torque);
/* Force history: total force and torque (hydrodynamic + repulsion + body
 * force) of the previous step, forcepp/torqpp of savecntdpart01
 * (saveload.f90:523-560), which the Newton-Euler update averages with the
 * current step's.  set: continue a run exactly (without it the first update
 * after lbm_particles_set uses the current force alone). */
int lbm_particles_get_history(lbm_ctx* ctx, double* fprev, double* tprev);
int lbm_particles_set_history(lbm_ctx* ctx, const double* fprev, const double* tprev);
/* Particle checkpoint in the reference's endrunpart2D format for one
 * process (savecntdpart / loadcntdpart, saveload.f90:604-693), Fortran
 * unformatted sequential records, FP64 reals and 4-byte integers:
 *   {nps, ipglb(msize)} {ibnodes(lx,ly,lz), isnodes(lx,ly,lz)}
 *   {yp(3,msize), thetap(3,msize)} {forcepp(3,msize), torqpp(3,msize)}
 *   {dwdt(3,msize), domgdt(3,msize)} {ypglb(3,npart), wp(3,npart), omgp(3,npart)}
 * with msize = 10 npart (para.f90:369, one process), ibnodes 1 solid / -1
 * fluid, isnodes the 1-based owning sphere / -1, forcepp/torqpp the
 * force history (total force and torque of the last step),
 * dwdt/domgdt that force / mass and torque / moment of inertia, thetap zero
 * (orientation is not integrated).  lbm_load_part attaches the spheres (as
 * lbm_particles_set with pp, whose npart must equal the file's nps) from
 * ypglb/wp/omgp, restores the history, and rebuilds the node flags from the
 * centres. */
int lbm_save_part(lbm_ctx* ctx, const char* path);
int lbm_load_part(lbm_ctx* ctx, const char* path, const lbm_particle_params* pp);
/* Solid node count, boundary links and refilled nodes of the last step. */
int lbm_particle_counts(lbm_ctx* ctx, int64_t* nsolid, int64_t* nlinks,
                        int64_t* nrefill);

/* ---- Learned LES closure (no reference counterpart) --------------------
 * A per-node network maps 7 features of the resolved strain (from the
 * non-equilibrium moments) and the wall distance to nu_t / nu >= 0:
 * 7 -> 32 -> 32 -> 1, SiLU hidden layers, softplus output.  Parameters (FP32):
 * W1[7][32] (row = input), b1[32], W2[32][32], b2[32], w3[32], b3; inputs are
 * standardised with norm[0..6] (mean) and norm[7..13] (1 / std).  Training
 * runs on the GPU: forward, backward (BF16 tensor-core GEMMs with FP32
 * accumulation, or FP32 with LBM_MLP_FP32) and Adam on the FP32 master
 * weights; loss = mean squared error of nu_t / nu. */
#define LBM_MLP_IN 7
#define LBM_MLP_HIDDEN 32
#define LBM_MLP_PARAMS 1345
#define LBM_MLP_NORM 14
#define LBM_MLP_FP32 1          /* flags: FP32 FMA products instead of BF16 tensor cores */
typedef struct lbm_mlp lbm_mlp;
/* Glorot-uniform weights from the seed, zero biases, identity normalisation. */
int lbm_mlp_create(lbm_mlp** m, uint64_t seed, int32_t device);
int lbm_mlp_destroy(lbm_mlp* m);
/* params: LBM_MLP_PARAMS floats, norm: LBM_MLP_NORM floats (either may be
 * NULL).  Setting the parameters restarts the Adam state. */
int lbm_mlp_get(lbm_mlp* m, float* params, float* norm);
int lbm_mlp_set(lbm_mlp* m, const float* params, const float* norm);
/* Training set: X[n][7] raw features, y[n] targets nu_t / nu (host FP32);
 * set_norm != 0 takes the normalisation from the mean and std of X. */
int lbm_mlp_set_data(lbm_mlp* m, const float* X, const float* y, int64_t n, int32_t set_norm);
/* `steps` Adam steps (beta 0.9/0.999, eps 1e-8) on random batches of `batch`
 * samples; losses (may be NULL) receives each step's batch loss. */
int lbm_mlp_train(lbm_mlp* m, int32_t steps, int32_t batch, float lr, int32_t flags, float* losses);
/* Loss and gradient of the mean loss over the whole training set. */
int lbm_mlp_gradient(lbm_mlp* m, int32_t flags, double* loss, float* grad);
/* nu_t / nu for X[n][7] (FP32 forward pass, the one the LES collision runs). */
int lbm_mlp_predict(lbm_mlp* m, const float* X, int64_t n, float* out);

/* Coarse-grid LES: the closure fused into the collision.  Per node the strain
 * rate from the non-equilibrium moments (Yu et al. 2006, with the shear rate
 * of the node's previous collision), the 7 features (strain invariants with
 * the wall normal, wall distance in wall units u* / nu and in units of h),
 * the network (weights in shared memory) and s9 = s13 = 1 / (3 (nu + nu_t) +
 * 1/2).  params == NULL turns it off.  FP32/FP64 storage, particle-free
 * channels; steps use the one-node-per-thread kernels while it is on. */
int lbm_les_set(lbm_ctx* ctx, const float* params, const float* norm, double ustar, double h);
/* Near-wall damping of the closure's eddy viscosity (no counterpart in the
 * reference, whose LES has no closure): nu_t is multiplied by
 * (1 - exp(-y+/A+))^2, y+ = d u* / nu with d the cell centre's wall distance
 * (van Driest 1956; A+ = 26 is the classical constant).  aplus = 0 (the
 * default) turns it off. */
int lbm_les_wall_damping(lbm_ctx* ctx, double aplus);
/* nu_t / nu of the last collision per node (host, nx*ny*nz doubles, reference
 * layout). */
int lbm_les_nut(lbm_ctx* ctx, double* nut);
/* The closure's 7 features per node from this lattice's populations, as the
 * fused collision computes them (strain from the non-equilibrium moments with
 * the node's last closure rate, or the molecular s9 when the closure is off).
 * X[n][7] FP32 host, nodes in the reference layout. */
int lbm_les_features(lbm_ctx* ctx, double ustar, double h, float* X);
/* Training data of the closure from a fine (DNS) lattice of this context: box
 * filter by `factor` (dividing nx, ny, nz) of u and u_i u_j; on the coarse
 * grid the strain of the filtered velocity (central differences, no-slip
 * image across the walls), the closure features in the coarse grid's units
 * (nu_c = nu / factor, u* the same, h_c = h / factor: acoustic scaling) and the
 * target nu_t* / nu_c = max(0, -tau^d : S / (2 S : S)) / nu_c, tau the subgrid
 * stress.  Coarse cells in the reference layout: X[nc][7], y[nc] (FP32),
 * ubar[3][nc] (FP64, filtered velocity); any may be NULL. */
int lbm_les_training_data(lbm_ctx* ctx, int32_t factor, double ustar, double h, float* X, float* y,
                          double* ubar);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
