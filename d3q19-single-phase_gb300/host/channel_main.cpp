// channel_gb300: the reference's driver (Channel-Flow/main.f90) on the C ABI.
//
// Same call order as main.f90:
//   para (para.f90)              -> parameters from key=value arguments
//   allocarray                   -> lbm_create
//   new run: initvel + FORCING + initpop (+ pre-relaxation) + saveinitflow
//            (main.f90:52-107)   -> lbm_init_channel or lbm_init_loglaw /
//                                   lbm_prerelax / lbm_save_flow
//   restart: loadcntdflow        -> lbm_load_flow (main.f90:118-121)
//   ipart: initpartpos + beads   -> lbm_particles_place / lbm_particles_set
//          (para.f90:339-379); the mean-density removal every 100 steps
//          (main.f90:163-167) runs inside lbm_step
//   time loop (main.f90:142-208) -> lbm_step, diag every ndiag steps
//                                   (saveload.f90:1507-1676), statistc2 every
//                                   nstat steps (saveload.f90:1348-1502), wall
//                                   clock limit
//   savecntdflow                 -> lbm_save_flow (kind 1)
//   savecntdpart / loadcntdpart  -> lbm_save_part / lbm_load_part
//                                   (endrunpart2D.<istep>.000, saveload.f90:604-693)
//
// Usage: channel_gb300 [key=value ...], keys (defaults = configuration c0):
//   nx ny nz          lattice, reference axes (wall-normal, streamwise, spanwise)
//   visc ustar h      viscosity, friction velocity, half height (force = ustar^2/h)
//   mrt               MRT rate set 1/2/3 (para.f90:110-141)
//   s16               rate of the third-order odd moments, overriding the set
//   precision         fp64 | fp32 | fp16
//   steps ndiag nstat main-loop length and output cadence
//   ivel              initial velocity: poiseuille (the benchmark channels: laminar
//                     profile + seeded noise), loglaw (initvel's turbulent start,
//                     initial.f90:101-147) or rest (ivel = .false.)
//   uc amp seed       initial Poiseuille centreline, noise amplitude, seed
//   a9                amplitude A9 of initvel's perturbation (loglaw; 0 as shipped)
//   prerelax          1: run the density pre-relaxation of main.f90:69-90
//   out               output directory for diag.dat / profiles2.dat / checkpoints
//   restart           checkpoint to continue from (endrunflow format)
//   save              1: write endrunflow2D16x8.<istep>.000 at the end
//   time_limit        wall-clock bound in seconds (para.f90:50-55)
//   ndiss             every ndiss steps append dissipation.dat (dissipation_calc,
//                     saveload.f90:4644-4882); 0 = off, as the reference's main loop
//   npart rad rhopart spheres: count, radius, density ratio (0 spheres: ipart off)
//   iseedp gap wgap   seeded placement: seed, surface gaps sphere-sphere and sphere-wall
//   qfp64             1: boundary-link fractions in FP64 for FP32/FP16 storage
//   restart_part      endrunpart2D file to continue the spheres from
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "lbm_gb300.h"

namespace {

std::map<std::string, std::string> g_args;

// makedir (para.f90:311-317): the output directory and its parents exist
// before the run writes into them
bool make_dirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i <= path.size(); ++i) {
        if ((i == path.size() || path[i] == '/') && !cur.empty() && cur != "." && cur != "/") {
            if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
        }
        if (i < path.size()) cur += path[i];
    }
    return true;
}

double argd(const char* k, double d) {
    auto it = g_args.find(k);
    return it == g_args.end() ? d : std::atof(it->second.c_str());
}
long argi(const char* k, long d) {
    auto it = g_args.find(k);
    return it == g_args.end() ? d : std::atol(it->second.c_str());
}
std::string args(const char* k, const char* d) {
    auto it = g_args.find(k);
    return it == g_args.end() ? std::string(d) : it->second;
}

int check(int rc, const char* what) {
    if (rc != LBM_OK) {
        std::fprintf(stderr, "%s failed: %s (%s)\n", what, lbm_strerror(rc), lbm_last_error());
        std::exit(2);
    }
    return rc;
}

// statistc2 normalisation and its 15 columns (saveload.f90:1442-1496)
void write_profiles(const std::string& path, const std::vector<double>& prof, int nx, long istep,
                    double ustar, double ystar, long nyz) {
    FILE* fp = std::fopen(path.c_str(), "a");
    if (!fp) return;
    std::fprintf(fp, " %ld\n", istep);
    const int lxh = nx / 2;
    for (int i = 1; i <= nx; ++i) {
        const double* r = &prof[(size_t)LBM_PROFILE_COLS * (i - 1)];
        const double n = r[11];
        const double vx = r[0] / n / ustar, vy = r[1] / n / ustar, vz = r[2] / n / ustar;
        const double sxx = r[6] / n / (ustar * ustar) - vx * vx;
        const double syy = r[7] / n / (ustar * ustar) - vy * vy;
        const double szz = r[8] / n / (ustar * ustar) - vz * vz;
        const double sxz = r[3] / n / (ustar * ustar) - vx * vz;
        const double sxy = r[4] / n / (ustar * ustar) - vx * vy;
        const double syz = r[5] / n / (ustar * ustar) - vy * vz;
        const double pr = r[9] / n / (ustar * ustar);
        const double prsq = r[10] / n / std::pow(ustar, 4) - pr * pr;
        const double volf = n / (double)nyz;
        double yplus = (i - 0.5) / ystar;
        if (i > lxh) yplus = (nx - i + 0.5) / ystar;
        std::fprintf(fp, "  %15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E\n",
                     i - 0.5, yplus, vx, vy, vz, sxx, syy, szz, sxz, sxy, syz, pr, prsq, volf, 1.0 - volf);
    }
    std::fclose(fp);
}

// dissipation_calc output (saveload.f90:4846-4872): plane means of S_ij S_ij
// and S_xy by both methods
void write_dissipation(const std::string& path, const std::vector<double>& d, int nx, long istep, double ystar) {
    FILE* fp = std::fopen(path.c_str(), "a");
    if (!fp) return;
    std::fprintf(fp, " %ld\n", istep);
    const int lxh = nx / 2;
    for (int i = 1; i <= nx; ++i) {
        const double* r = &d[(size_t)LBM_DISSIPATION_COLS * (i - 1)];
        const double n = r[4];
        double yplus = (i - 0.5) / ystar;
        if (i > lxh) yplus = (nx - i + 0.5) / ystar;
        std::fprintf(fp, "  %16.6E%16.6E%16.6E%16.6E%16.6E%16.6E\n", i - 0.5, yplus, r[0] / n, r[1] / n, r[2] / n,
                     r[3] / n);
    }
    std::fclose(fp);
}

}  // namespace

int main(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) {
            std::fprintf(stderr, "argument %s is not key=value\n", argv[i]);
            return 1;
        }
        g_args[std::string(argv[i], eq - argv[i])] = eq + 1;
    }
    const int nx = (int)argi("nx", 64), ny = (int)argi("ny", 128), nz = (int)argi("nz", 64);
    const double visc = argd("visc", 0.0012), ustar = argd("ustar", 0.0035), h = argd("h", 32.0);
    const double force = ustar * ustar / h;
    const int mrt = (int)argi("mrt", 1);
    const std::string precs = args("precision", "fp64");
    const int prec = precs == "fp16" ? LBM_PREC_FP16 : (precs == "fp32" ? LBM_PREC_FP32 : LBM_PREC_FP64);
    const long nsteps = argi("steps", 100), ndiag = argi("ndiag", 250), nstat = argi("nstat", 1000);
    const std::string out = args("out", ".");
    if (!make_dirs(out)) {
        std::fprintf(stderr, "cannot create the output directory %s\n", out.c_str());
        return 1;
    }
    const double time_bond = argd("time_limit", (720.0 - 10.0) * 60.0);

    lbm_params p;
    check(lbm_params_init(&p, nx, ny, nz, mrt, visc, force, prec), "lbm_params_init");
    if (g_args.count("s16")) p.s16 = argd("s16", p.s16);
    lbm_ctx* ctx = nullptr;
    check(lbm_create(&p, &ctx), "lbm_create");

    long istep0 = 0;
    int32_t hdr[3] = {0, 0, 0};
    if (g_args.count("restart")) {
        check(lbm_load_flow(ctx, args("restart", "").c_str(), 1, hdr), "loadcntdflow");
        istep0 = hdr[0];
        check(lbm_set_step_count(ctx, istep0), "istep0");
        std::printf("Loading flow... istep0=%ld\n", istep0);
    } else {
        const double uc = argd("uc", 0.05), amp = argd("amp", 0.05);
        const uint64_t seed = (uint64_t)argi("seed", 20240611);
        const std::string ivel = args("ivel", "poiseuille");
        const double a9 = argd("a9", 0.0);
        const size_t n = (size_t)nx * ny * nz;
        std::vector<double> u, v, w;
        if (ivel == "loglaw") {
            // initvel with ivel = .true. (turbulent start, initial.f90:101-147)
            check(lbm_init_loglaw(ctx, ustar, visc / ustar, a9), "initvel+initpop");
        } else if (ivel == "rest") {
            // initvel with ivel = .false. (stationary start, initial.f90:97-100)
            u.assign(n, 0.0); v.assign(n, 0.0); w.assign(n, 0.0);
            check(lbm_initpop(ctx, u.data(), v.data(), w.data()), "initpop");
        } else if (ivel == "poiseuille") {
            check(lbm_init_channel(ctx, uc, amp, seed), "initvel+initpop");
        } else {
            std::fprintf(stderr, "ivel must be poiseuille, loglaw or rest\n");
            return 1;
        }
        if (argi("prerelax", 0)) {
            // the velocity stays frozen at the initial condition's, which the
            // library reads back from the populations (no host sweep)
            int32_t it = 0;
            double err = 0;
            const int rc = lbm_prerelax(ctx, nullptr, nullptr, nullptr, 1e-5, 15000, &it, &err);
            if (rc != LBM_OK && rc != LBM_ERR_NOT_CONVERGED) check(rc, "prerelax");
            std::printf(" final relaxation => %d %.6E\n", it, err);
            int32_t istat = 0;
            check(lbm_save_flow(ctx, (out + "/finit.000").c_str(), 0, &istat), "saveinitflow");
        }
    }
    // spheres (ipart): placement or restart, then the solid masks
    const int npart = (int)argi("npart", 0);
    if (npart > 0) {
        const double rad = argd("rad", 8.0), rhopart = argd("rhopart", 2.0);
        lbm_particle_params pp;
        check(lbm_particle_params_init(&pp, npart, rad, rhopart), "particle parameters");
        if (argi("qfp64", 0)) pp.flags |= LBM_PFLAG_Q_FP64;
        if (g_args.count("restart_part")) {
            check(lbm_load_part(ctx, args("restart_part", "").c_str(), &pp), "loadcntdpart");
        } else {
            std::vector<double> pos(3 * (size_t)npart);
            check(lbm_particles_place(nx, ny, nz, npart, rad, argd("gap", 2.0), argd("wgap", 1.0),
                                      (uint64_t)argi("iseedp", 12345), pos.data()),
                  "initpartpos");
            check(lbm_particles_set(ctx, &pp, pos.data(), nullptr, nullptr), "beads");
        }
        int64_t nsolid = 0, nlinks = 0, nrefill = 0;
        check(lbm_particle_counts(ctx, &nsolid, &nlinks, &nrefill), "particle counts");
        std::printf(" spheres: %d of radius %.3f, %lld solid nodes\n", npart, rad, (long long)nsolid);
    }
    std::printf("Loading successful\n");

    const double ystar = visc / ustar;
    std::vector<double> prof((size_t)LBM_PROFILE_COLS * nx), diss((size_t)LBM_DISSIPATION_COLS * nx);
    const long ndiss = argi("ndiss", 0);
    const auto t0 = std::chrono::steady_clock::now();
    long istep = istep0;
    for (istep = istep0 + 1; istep <= istep0 + nsteps; ++istep) {
        check(lbm_step(ctx, 1), "collision_MRT");
        if (istep % ndiag == 0) {
            lbm_stats st;
            const int rc = lbm_diag(ctx, &st);
            const double nf = (double)st.nfluid;
            const double um = st.mom_sum[0] / nf, vm = st.mom_sum[1] / nf, wm = st.mom_sum[2] / nf;
            const double ur = std::sqrt(std::fmax(st.usq_sum[0] / nf - um * um, 0.0));
            const double vr = std::sqrt(std::fmax(st.usq_sum[1] / nf - vm * vm, 0.0));
            const double wr = std::sqrt(std::fmax(st.usq_sum[2] / nf - wm * wm, 0.0));
            FILE* fp = std::fopen((out + "/diag.dat").c_str(), "a");
            if (fp) {
                std::fprintf(fp, "  %16.6E%16.6E%6d%6d%6d%16.6E%16.6E%16.6E%16.6E%16.6E%16.6E%16.6E%16.6E%16.6E\n",
                             (double)istep, st.vmax, st.vmax_at[0], st.vmax_at[1], st.vmax_at[2], um / ustar,
                             vm / ustar, wm / ustar, ur / ustar, vr / ustar, wr / ustar,
                             1.0 - nf / ((double)nx * ny * nz), st.rho_max, st.rho_min);
                std::fclose(fp);
            }
            std::printf(" istep=%ld vmax=%.6E rho=[%.6E, %.6E] mass=%.6E\n", istep, st.vmax, st.rho_min,
                        st.rho_max, st.rho_sum);
            if (rc == LBM_ERR_NONFINITE) {
                std::fprintf(stderr, "non-finite populations at step %ld\n", istep);
                lbm_destroy(ctx);
                return 3;
            }
        }
        if (istep % nstat == 0) {
            check(lbm_profiles(ctx, prof.data()), "statistc2");
            write_profiles(out + "/profiles2.dat", prof, nx, istep, ustar, ystar, (long)ny * nz);
        }
        if (ndiss > 0 && istep % ndiss == 0) {
            check(lbm_dissipation(ctx, diss.data()), "dissipation_calc");
            write_dissipation(out + "/dissipation.dat", diss, nx, istep, ystar);
        }
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > time_bond) break;
    }
    const long done = (istep > istep0 + nsteps ? nsteps : istep - istep0);
    const double time_max = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (argi("save", 0)) {
        char name[64];
        std::snprintf(name, sizeof(name), "/endrunflow2D16x8.%07ld.000", istep0 + done);
        int32_t h3[3] = {(int32_t)(istep0 + done), 0, 0};
        check(lbm_save_flow(ctx, (out + name).c_str(), 1, h3), "savecntdflow");
        if (npart > 0) {
            std::snprintf(name, sizeof(name), "/endrunpart2D.%07ld.000", istep0 + done);
            check(lbm_save_part(ctx, (out + name).c_str()), "savecntdpart");
        }
    }
    std::printf(" time_max = %.6f  steps = %ld  GLUPS = %.4f\n", time_max, done,
                (double)nx * ny * nz * done / time_max / 1e9);
    lbm_destroy(ctx);
    return 0;
}
