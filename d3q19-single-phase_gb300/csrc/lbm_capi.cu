// extern "C" boundary of liblbm_gb300.so: context management, host<->device
// layout conversion, the step loop, pre-relaxation, diagnostics and
// checkpoint files.  See include/lbm_gb300.h for the contract.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lbm_internal.h"

using namespace lbm;

struct lbm_ctx {
    lbm_params p{};
    DeviceState s{};
    cudaStream_t stream = nullptr;
    int parity = 0;            // 0: natural orientation, 1: after an even AA step
    int64_t nsteps = 0;
    int64_t nlaunch = 0;          // kernels launched by lbm_step / lbm_step_async
    double* d_stage = nullptr; // FP64 staging for layout conversion
    double* d_mass = nullptr;  // fluid mass and node count (mean-density removal)
    float* d_les = nullptr;    // closure network parameters + normalisation
    float* d_s9 = nullptr;     // per-node shear rate of the closure
    int use_rows_saved = 0;    // the step kernel choice without the closure
    size_t stage_elems = 0;
    double* d_red = nullptr;   // reduction partials
    size_t red_elems = 0;
    double* d_uf = nullptr;    // frozen velocity for pre-relaxation (GPU layout)
    double* d_rho = nullptr;   // pre-relaxation density
    unsigned long long* d_max = nullptr;
    int* d_err = nullptr;      // set by a kernel whose bounded wait gave up
    DeviceParticles P{};       // spheres (npart == 0: none)
    lbm_particle_params pp{};
    lbm::SideStream side;      // the sphere pass's second stream (created with the spheres)
    int have_prev = 0;         // previous-step force and torque available
    int order_age = 0;         // steps since the spheres' spatial order was sorted
    unsigned long long* d_count = nullptr;
    // per-step timing (lbm_timing_enable): 3 events per recorded step
    std::vector<cudaEvent_t> tev;
    std::vector<int> tpar;
    int tcap = 0, tn = 0;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(LBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);        \
    } while (0)

// Reference-layout element counts
size_t nodes(const lbm_params& p) { return (size_t)p.nx * p.ny * p.nz; }
size_t plane_nodes(const lbm_params& p) { return (size_t)p.nx * p.ny; }   // one ref z plane

template <typename R>
CollideConsts<R> make_consts(const lbm_params& p, double S) {
    CollideConsts<R> c;
    c.S = (R)S; c.invS = (R)(1.0 / S);
    c.Fx = (R)p.force[0]; c.Fy = (R)p.force[1]; c.Fz = (R)p.force[2];
    c.hFx = (R)(0.5 * S * p.force[0]); c.hFy = (R)(0.5 * S * p.force[1]); c.hFz = (R)(0.5 * S * p.force[2]);
    c.ajx = (R)(S * p.force[0] / 10.0); c.ajy = (R)(S * p.force[1] / 10.0); c.ajz = (R)(S * p.force[2] / 10.0);
    c.fqx = (R)(-(2.0 / 3.0) * S * p.force[0] / 40.0);
    c.fqy = (R)(-(2.0 / 3.0) * S * p.force[1] / 40.0);
    c.fqz = (R)(-(2.0 / 3.0) * S * p.force[2] / 40.0);
    c.thFx = (R)(S * p.force[0] / 3.0); c.thFy = (R)(S * p.force[1] / 3.0); c.thFz = (R)(S * p.force[2] / 3.0);
    c.ke = (R)(p.s1 / 2394.0);
    c.keps = (R)(p.s2 / 252.0);
    c.kq = (R)(p.s4 / 40.0);
    c.kp = (R)(p.s9 / 36.0);
    c.kpi = (R)(p.s10 / 72.0);
    c.kxy = (R)(p.s13 / 4.0);
    c.km = (R)(p.s16 / 8.0);
    c.kw = (R)(p.s9 / 12.0);
    c.kwi = (R)(p.s10 / 24.0);
    c.oeps = (R)p.omegepsl; c.oepsj = (R)p.omegepslj; c.oxx = (R)p.omegxx;
    return c;
}

size_t elem_size(int prec) {
    return prec == LBM_PREC_FP64 ? 8 : (prec == LBM_PREC_FP32 ? 4 : 2);
}

int check_ctx(const lbm_ctx* c) {
    if (!c) return fail(LBM_ERR_INVALID_ARG, "null context");
    return LBM_OK;
}

int set_device(const lbm_ctx* c) {
    CK(cudaSetDevice(c->p.device));
    return LBM_OK;
}

// planes of the reference z axis that fit in the staging buffer for k arrays
int chunk_planes(const lbm_ctx* c, size_t per_node_doubles) {
    const size_t per_plane = plane_nodes(c->p) * per_node_doubles;
    size_t k = c->stage_elems / per_plane;
    if (k < 1) k = 1;
    if (k > (size_t)c->p.nz) k = c->p.nz;
    return (int)k;
}

int ensure_stage(lbm_ctx* c, size_t elems) {
    if (c->stage_elems >= elems) return LBM_OK;
    if (c->d_stage) cudaFree(c->d_stage);
    c->d_stage = nullptr;
    c->stage_elems = 0;
    CK(cudaMalloc(&c->d_stage, elems * sizeof(double)));
    c->stage_elems = elems;
    return LBM_OK;
}

int ensure_red(lbm_ctx* c, size_t elems) {
    if (c->red_elems >= elems) return LBM_OK;
    if (c->d_red) cudaFree(c->d_red);
    c->d_red = nullptr;
    c->red_elems = 0;
    CK(cudaMalloc(&c->d_red, elems * sizeof(double)));
    c->red_elems = elems;
    return LBM_OK;
}

int sync(lbm_ctx* c) {
    CK(cudaStreamSynchronize(c->stream));
    if (c->d_err) {
        int flag[2] = {0, 0};
        CK(cudaMemcpy(flag, c->d_err, sizeof(flag), cudaMemcpyDeviceToHost));
        if (flag[0] || flag[1]) {
            cudaMemset(c->d_err, 0, sizeof(flag));
            if (flag[1])
                return fail(LBM_ERR_STATE, "bounds check failed at site " + std::to_string(flag[1]) +
                                               "; the access was skipped and the results are invalid");
            return fail(LBM_ERR_CUDA, "a step kernel's bulk-copy wait timed out; populations are invalid");
        }
    }
    if (c->P.npart > 0) {
        unsigned flag = 0;
        CK(cudaMemcpy(&flag, c->P.counters + 3, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (flag) {
            cudaMemset(c->P.counters + 3, 0, sizeof(unsigned));
            if (flag & 2u) return fail(LBM_ERR_STATE, "non-finite or runaway sphere motion (velocity above 1 per step)");
            return fail(LBM_ERR_STATE, "refill list overflow: spheres moved too far in one step");
        }
    }
    return LBM_OK;
}

// ---- Fortran unformatted sequential records (gfortran convention) -------
constexpr int64_t kMaxSub = 2147483639;  // bytes of data per sub-record

bool write_marker(FILE* fp, int32_t v) { return fwrite(&v, 4, 1, fp) == 1; }

struct RecordWriter {
    // Writes one logical record of `total` bytes in sub-records; data arrives
    // in pieces through put().
    FILE* fp;
    int64_t total, done = 0, sub_left = 0, sub_len = 0;
    bool first = true, ok = true;
    RecordWriter(FILE* f, int64_t t) : fp(f), total(t) {
        if (total == 0) { ok = write_marker(fp, 0) && write_marker(fp, 0); }
    }
    void open_sub() {
        sub_len = std::min<int64_t>(kMaxSub, total - done);
        const bool more = done + sub_len < total;
        ok = ok && write_marker(fp, (int32_t)(more ? -sub_len : sub_len));
        sub_left = sub_len;
    }
    void close_sub() {
        ok = ok && write_marker(fp, (int32_t)(first ? sub_len : -sub_len));
        first = false;
    }
    void put(const void* data, int64_t n) {
        const char* b = static_cast<const char*>(data);
        while (n > 0 && ok) {
            if (sub_left == 0) open_sub();
            const int64_t k = std::min(n, sub_left);
            ok = ok && fwrite(b, 1, (size_t)k, fp) == (size_t)k;
            b += k; n -= k; sub_left -= k; done += k;
            if (sub_left == 0) close_sub();
        }
    }
};

struct RecordReader {
    FILE* fp;
    int64_t sub_left = 0, total = 0;
    bool more = true, ok = true, first = true;
    explicit RecordReader(FILE* f) : fp(f) { next_sub(); }
    void next_sub() {
        int32_t m;
        if (fread(&m, 4, 1, fp) != 1) { ok = false; return; }
        more = m < 0;
        sub_left = m < 0 ? -(int64_t)m : m;
        total += sub_left;
    }
    void end_sub() {
        int32_t m;
        if (fread(&m, 4, 1, fp) != 1) { ok = false; return; }
        const int64_t len = m < 0 ? -(int64_t)m : m;
        (void)len;
        first = false;
    }
    // read exactly n bytes of user data, crossing sub-records
    bool get(void* data, int64_t n) {
        char* b = static_cast<char*>(data);
        while (n > 0 && ok) {
            if (sub_left == 0) {
                if (!more) { ok = false; break; }
                end_sub();
                next_sub();
                continue;
            }
            const int64_t k = std::min(n, sub_left);
            if (fread(b, 1, (size_t)k, fp) != (size_t)k) { ok = false; break; }
            b += k; n -= k; sub_left -= k;
        }
        return ok;
    }
    // skip the rest of the record and its trailing marker; true if the record
    // held exactly the data consumed
    bool finish() {
        if (!ok) return false;
        const bool exact = sub_left == 0 && !more;
        while (ok && (sub_left > 0 || more)) {
            if (sub_left > 0) {
                if (fseek(fp, (long)sub_left, SEEK_CUR) != 0) ok = false;
                sub_left = 0;
            } else { end_sub(); next_sub(); }
        }
        if (ok) end_sub();
        return ok && exact;
    }
};

}  // namespace

namespace lbm {
// Context internals for entry points defined in other translation units.
const DeviceState* ctx_state(lbm_ctx* c, int* parity, cudaStream_t* stream, int* device) {
    *parity = c->parity;
    *stream = c->stream;
    *device = c->p.device;
    return &c->s;
}
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace lbm

extern "C" {

const char* lbm_strerror(int code) {
    switch (code) {
        case LBM_OK: return "success";
        case LBM_ERR_INVALID_ARG: return "invalid argument";
        case LBM_ERR_CUDA: return "CUDA runtime error";
        case LBM_ERR_OOM: return "out of memory";
        case LBM_ERR_STATE: return "invalid state for this call";
        case LBM_ERR_NOT_CONVERGED: return "pre-relaxation did not converge";
        case LBM_ERR_IO: return "checkpoint file error";
        case LBM_ERR_NONFINITE: return "non-finite populations";
        case LBM_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown error";
}

const char* lbm_last_error(void) { return g_last_error.c_str(); }

int lbm_version(void) { return 100; }

int lbm_params_init(lbm_params* p, int32_t nx, int32_t ny, int32_t nz, int32_t mrt_type,
                    double visc, double force_y, int32_t precision) {
    if (!p) return fail(LBM_ERR_INVALID_ARG, "null params");
    if (nx < 1 || ny < 1 || nz < 1) return fail(LBM_ERR_INVALID_ARG, "lattice size must be positive");
    if (!(visc > 0.0)) return fail(LBM_ERR_INVALID_ARG, "viscosity must be positive");
    std::memset(p, 0, sizeof(*p));
    p->nx = nx; p->ny = ny; p->nz = nz;
    p->precision = precision;
    // para.f90:106-141
    const double tau = 3.0 * visc + 0.5;
    p->s9 = 1.0 / tau;
    p->s13 = p->s9;
    switch (mrt_type) {
        case LBM_MRT_STABLE:
            p->s1 = 1.5; p->s2 = 1.4; p->s4 = 1.2; p->s10 = 1.4; p->s16 = 1.98;
            p->omegepsl = 0.0; p->omegepslj = -475.0 / 63.0; p->omegxx = 0.0;
            break;
        case LBM_MRT_LBGK:
            p->s1 = p->s9; p->s2 = p->s9; p->s4 = p->s9; p->s10 = p->s9; p->s16 = p->s9;
            p->omegepsl = 3.0; p->omegepslj = -11.0 / 2.0; p->omegxx = -1.0 / 2.0;
            break;
        case LBM_MRT_LOWDISS:
            p->s1 = 1.8; p->s2 = p->s1; p->s4 = p->s9; p->s10 = p->s1; p->s16 = p->s1;
            p->omegepsl = 3.0; p->omegepslj = -11.0 / 2.0; p->omegxx = -1.0 / 2.0;
            break;
        default:
            return fail(LBM_ERR_INVALID_ARG, "MRT type must be 1, 2 or 3");
    }
    p->force[0] = 0.0; p->force[1] = force_y; p->force[2] = 0.0;   // FORCING, collision.f90:522-524
    p->fp16_scale = 32768.0;
    p->device = 0;
    if (precision < LBM_PREC_FP64 || precision > LBM_PREC_FP16)
        return fail(LBM_ERR_INVALID_ARG, "precision must be LBM_PREC_FP64/FP32/FP16");
    return LBM_OK;
}

int lbm_create(const lbm_params* p, lbm_ctx** out) {
    if (!p || !out) return fail(LBM_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return fail(LBM_ERR_INVALID_ARG, "lattice size must be positive");
    if (p->nz > 65535 || p->nx > 65535) return fail(LBM_ERR_INVALID_ARG, "nx and nz are limited to 65535");
    if (nodes(*p) >= (size_t)1 << 32) return fail(LBM_ERR_INVALID_ARG, "more than 2^32-1 nodes");
    if (p->precision < LBM_PREC_FP64 || p->precision > LBM_PREC_FP16)
        return fail(LBM_ERR_INVALID_ARG, "bad precision");
    const double S = p->precision == LBM_PREC_FP16 ? (p->fp16_scale > 0 ? p->fp16_scale : 32768.0) : 1.0;
    if (!std::isfinite(S)) return fail(LBM_ERR_INVALID_ARG, "bad fp16 scale");
    for (double v : {p->s1, p->s2, p->s4, p->s9, p->s10, p->s13, p->s16, p->omegepsl, p->omegepslj,
                     p->omegxx, p->force[0], p->force[1], p->force[2]})
        if (!std::isfinite(v)) return fail(LBM_ERR_INVALID_ARG, "non-finite parameter");

    lbm_ctx* c = new (std::nothrow) lbm_ctx();
    if (!c) return fail(LBM_ERR_OOM, "host allocation failed");
    c->p = *p;
    if (c->p.precision == LBM_PREC_FP16) c->p.fp16_scale = S;
    cudaError_t e = cudaSetDevice(p->device);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaSetDevice"); }
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }

    DeviceState& s = c->s;
    s.prec = p->precision;
    s.g.NX = p->ny; s.g.NY = p->nz; s.g.NZ = p->nx;
    s.g.NXY = (uint32_t)p->ny * (uint32_t)p->nz;
    s.N = nodes(*p);
    // planes start on 256-byte boundaries
    const size_t es = elem_size(s.prec);
    const size_t align = 256 / es;
    s.pstride = (s.N + align - 1) / align * align;
    e = cudaMalloc(&s.f, (size_t)Q * s.pstride * es);
    if (e != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,
                    std::string("population allocation: ") + cudaGetErrorString(e));
    }
    s.cd = make_consts<double>(c->p, S);
    s.cf = make_consts<float>(c->p, S);
    cudaDeviceGetAttribute(&s.sm_count, cudaDevAttrMultiProcessorCount, p->device);
    s.use_rows = !(p->flags & LBM_FLAG_SIMPLE_STEP) && rows_supported(s);
    if (s.use_rows && prepare_step_rows() != cudaSuccess) s.use_rows = 0;
    c->use_rows_saved = s.use_rows;
    // error flags: [0] a bounded wait gave up, [1] the first failing
    // bounds-check site (bounds-checked build only)
    e = cudaMalloc(&c->d_err, 2 * sizeof(int));
    if (e != cudaSuccess) { lbm_destroy(c); return cuda_fail(e, "cudaMalloc(error flag)"); }
    cudaMemsetAsync(c->d_err, 0, 2 * sizeof(int), c->stream);
    c->s.bounds = reinterpret_cast<unsigned*>(c->d_err + 1);
    // staging: up to 256 MB, at least one reference z plane of AoS populations
    const size_t want = std::max<size_t>(plane_nodes(*p) * Q, (size_t)32 << 20);
    const size_t stage = std::min<size_t>(want, std::max<size_t>(plane_nodes(*p) * Q, s.N * Q));
    int rc = ensure_stage(c, stage);
    if (rc != LBM_OK) { lbm_destroy(c); return rc; }
    cudaMemsetAsync(s.f, 0, (size_t)Q * s.pstride * es, c->stream);
    rc = sync(c);
    if (rc != LBM_OK) { lbm_destroy(c); return rc; }
    *out = c;
    return LBM_OK;
}

int lbm_destroy(lbm_ctx* c) {
    if (!c) return LBM_OK;
    cudaSetDevice(c->p.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->s.f);
    cudaFree(c->d_stage);
    cudaFree(c->d_red);
    cudaFree(c->d_uf);
    cudaFree(c->d_rho);
    cudaFree(c->d_max);
    cudaFree(c->d_err);
    cudaFree(c->d_count);
    for (cudaEvent_t e : c->tev) cudaEventDestroy(e);
    cudaFree(c->P.pos);
    cudaFree(c->P.owner);
    cudaFree(c->P.refill_node);
    cudaFree(c->P.refill_part);
    cudaFree(c->P.counters);
    cudaFree(c->P.cell_count);
    cudaFree(c->P.geom);
    cudaFree(c->P.order);
    cudaFree(c->d_les);
    cudaFree(c->d_s9);
    cudaFree(c->d_mass);
    if (c->side.st) {
        cudaStreamSynchronize(c->side.st);
        cudaStreamDestroy(c->side.st);
    }
    if (c->side.fork) cudaEventDestroy(c->side.fork);
    if (c->side.join) cudaEventDestroy(c->side.join);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return LBM_OK;
}

int lbm_device_bytes(const lbm_ctx* c, size_t* bytes) {
    if (check_ctx(c) || !bytes) return fail(LBM_ERR_INVALID_ARG, "null argument");
    *bytes = (size_t)Q * c->s.pstride * elem_size(c->s.prec) + c->stage_elems * 8 + c->red_elems * 8 +
             (c->d_uf ? 3 * c->s.N * 8 : 0) + (c->d_rho ? c->s.N * 8 : 0);
    return LBM_OK;
}

int lbm_upload_f(lbm_ctx* c, const double* f) {
    if (check_ctx(c) || !f) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (int rc = set_device(c)) return rc;
    const int k = chunk_planes(c, Q);
    const size_t per_plane = plane_nodes(c->p) * Q;
    for (int z0 = 0; z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        CK(cudaMemcpyAsync(c->d_stage, f + (size_t)z0 * per_plane, (size_t)nzc * per_plane * 8,
                           cudaMemcpyHostToDevice, c->stream));
        CK(launch_aos_to_store(c->s, c->d_stage, z0, nzc, c->stream));
    }
    c->parity = 0;
    c->nsteps = 0;
    return sync(c);
}

int lbm_download_f(lbm_ctx* c, double* f) {
    if (check_ctx(c) || !f) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (int rc = set_device(c)) return rc;
    const int k = chunk_planes(c, Q);
    const size_t per_plane = plane_nodes(c->p) * Q;
    for (int z0 = 0; z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        CK(launch_store_to_aos(c->s, c->parity, c->d_stage, z0, nzc, c->stream));
        CK(cudaMemcpyAsync(f + (size_t)z0 * per_plane, c->d_stage, (size_t)nzc * per_plane * 8,
                           cudaMemcpyDeviceToHost, c->stream));
    }
    return sync(c);
}

int lbm_initpop(lbm_ctx* c, const double* ux, const double* uy, const double* uz) {
    if (check_ctx(c) || !ux || !uy || !uz) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (int rc = set_device(c)) return rc;
    const int k = chunk_planes(c, 3);
    const size_t pp = plane_nodes(c->p);
    for (int z0 = 0; z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        const size_t n = (size_t)nzc * pp;
        double* du = c->d_stage;
        double* dv = du + n;
        double* dw = dv + n;
        CK(cudaMemcpyAsync(du, ux + (size_t)z0 * pp, n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dv, uy + (size_t)z0 * pp, n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dw, uz + (size_t)z0 * pp, n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(launch_initpop(c->s, du, dv, dw, z0, nzc, c->stream));
    }
    c->parity = 0;
    c->nsteps = 0;
    return sync(c);
}

int lbm_init_channel(lbm_ctx* c, double uc, double amp, uint64_t seed) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (!std::isfinite(uc) || !std::isfinite(amp)) return fail(LBM_ERR_INVALID_ARG, "non-finite argument");
    if (int rc = set_device(c)) return rc;
    CK(launch_init_channel(c->s, uc, amp, seed, c->stream));
    c->parity = 0;
    c->nsteps = 0;
    return sync(c);
}

int lbm_channel_velocity(int32_t nx, int32_t ny, int32_t nz, double uc, double amp, uint64_t seed,
                         double* ux, double* uy, double* uz) {
    if (nx < 1 || ny < 1 || nz < 1 || !ux || !uy || !uz) return fail(LBM_ERR_INVALID_ARG, "bad argument");
    channel_velocity_host(nx, ny, nz, uc, amp, seed, ux, uy, uz);
    return LBM_OK;
}

int lbm_init_loglaw(lbm_ctx* c, double ustar, double ystar, double a9) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (!(ustar > 0.0) || !(ystar > 0.0) || !std::isfinite(ustar) || !std::isfinite(ystar) || !std::isfinite(a9))
        return fail(LBM_ERR_INVALID_ARG, "ustar and ystar must be positive and finite, a9 finite");
    if (int rc = set_device(c)) return rc;
    const int nx = c->p.nx, ny = c->p.ny, nz = c->p.nz;
    const size_t nt = loglaw_table_doubles(nx, ny, nz);
    std::vector<double> tab(nt);
    loglaw_tables_host(nx, ny, nz, ustar, ystar, a9, tab.data());
    if (int rc = ensure_stage(c, nt)) return rc;
    CK(cudaMemcpyAsync(c->d_stage, tab.data(), nt * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(launch_init_loglaw(c->s, c->d_stage, nx / 2, c->stream));
    c->parity = 0;
    c->nsteps = 0;
    return sync(c);
}

int lbm_loglaw_velocity(int32_t nx, int32_t ny, int32_t nz, double ustar, double ystar, double a9, double* ux,
                        double* uy, double* uz) {
    if (nx < 1 || ny < 1 || nz < 1 || !ux || !uy || !uz) return fail(LBM_ERR_INVALID_ARG, "bad argument");
    if (!(ustar > 0.0) || !(ystar > 0.0) || !std::isfinite(ustar) || !std::isfinite(ystar) || !std::isfinite(a9))
        return fail(LBM_ERR_INVALID_ARG, "ustar and ystar must be positive and finite, a9 finite");
    std::vector<double> tab(loglaw_table_doubles(nx, ny, nz));
    loglaw_tables_host(nx, ny, nz, ustar, ystar, a9, tab.data());
    loglaw_velocity_host(nx, ny, nz, tab.data(), ux, uy, uz);
    return LBM_OK;
}

int lbm_step_async(lbm_ctx* c, int32_t nsteps) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (nsteps < 0) return fail(LBM_ERR_INVALID_ARG, "negative step count");
    for (int32_t k = 0; k < nsteps; ++k) {
        const bool timed = c->tn < c->tcap;
        if (timed) CK(cudaEventRecord(c->tev[3 * c->tn], c->stream));
        if (c->s.use_rows) CK(launch_step_rows(c->s, c->parity, c->d_err, c->stream));
        else CK(launch_step(c->s, c->parity, c->stream));
        ++c->nlaunch;
        if (timed) CK(cudaEventRecord(c->tev[3 * c->tn + 1], c->stream));
        const int was = c->parity;
        c->parity ^= 1;
        ++c->nsteps;
        if (c->P.npart > 0) {
            if (++c->order_age >= kReorderEvery) {       // keep the spatial order current
                CK(particles_reorder(c->P, c->stream));
                c->nlaunch += kReorderKernels;
                c->order_age = 0;
            }
            CK(particles_after_step(c->s, c->P, c->parity, c->have_prev, c->stream, c->side));
            c->nlaunch += particles_kernels_per_step(c->P);
            c->have_prev = 1;
            // main.f90:163-167: with particles, every 100 steps the mean
            // density is removed to correct the mass the interpolated
            // bounce-back loses (avedensity)
            if (c->nsteps % 100 == 0) {
                CK(launch_remove_mean_density(c->s, c->parity, c->d_mass, c->stream));
                CK(launch_remove_mean_apply(c->s, c->d_mass, c->stream));
                c->nlaunch += 2;
            }
        }
        if (timed) {
            CK(cudaEventRecord(c->tev[3 * c->tn + 2], c->stream));
            c->tpar[c->tn] = was;
            ++c->tn;
        }
    }
    return LBM_OK;
}

int lbm_step(lbm_ctx* c, int32_t nsteps) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (int rc = set_device(c)) return rc;
    if (int rc = lbm_step_async(c, nsteps)) return rc;
    return sync(c);
}

int lbm_synchronize(lbm_ctx* c) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    return sync(c);
}

int lbm_stream(lbm_ctx* c, void** stream) {
    if (check_ctx(c) || !stream) return fail(LBM_ERR_INVALID_ARG, "null argument");
    *stream = (void*)c->stream;
    return LBM_OK;
}

int lbm_step_count(const lbm_ctx* c, int64_t* n) {
    if (check_ctx(c) || !n) return fail(LBM_ERR_INVALID_ARG, "null argument");
    *n = c->nsteps;
    return LBM_OK;
}

int lbm_set_step_count(lbm_ctx* c, int64_t n) {
    if (check_ctx(c) || n < 0) return fail(LBM_ERR_INVALID_ARG, "bad step count");
    c->nsteps = n;
    return LBM_OK;
}

int lbm_prerelax(lbm_ctx* c, const double* ux, const double* uy, const double* uz, double eps,
                 int32_t maxit, int32_t* iters, double* err) {
    const bool from_f = !ux && !uy && !uz;      // frozen velocity from the current populations
    if (check_ctx(c) || (!from_f && (!ux || !uy || !uz))) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (!(eps >= 0.0) || maxit < 0) return fail(LBM_ERR_INVALID_ARG, "bad eps or maxit");
    if (int rc = set_device(c)) return rc;
    const size_t N = c->s.N;
    if (!c->d_uf) CK(cudaMalloc(&c->d_uf, 3 * N * sizeof(double)));
    if (!c->d_rho) CK(cudaMalloc(&c->d_rho, N * sizeof(double)));
    if (!c->d_max) CK(cudaMalloc(&c->d_max, sizeof(unsigned long long)));
    const int k = chunk_planes(c, 3);
    const size_t pp = plane_nodes(c->p);
    if (from_f) CK(launch_uf_from_f(c->s, c->parity, c->d_uf, c->stream));
    for (int z0 = 0; !from_f && z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        const size_t n = (size_t)nzc * pp;
        double* du = c->d_stage;
        CK(cudaMemcpyAsync(du, ux + (size_t)z0 * pp, n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(du + n, uy + (size_t)z0 * pp, n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(du + 2 * n, uz + (size_t)z0 * pp, n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(launch_ref_to_gpu_vec(c->s, du, du + n, du + 2 * n, c->d_uf, z0, nzc, c->stream));
    }
    // initpop leaves rho = 0 (initial.f90:32); main.f90:71 copies it to rhop
    CK(cudaMemsetAsync(c->d_rho, 0, N * sizeof(double), c->stream));
    int32_t istep = 0;
    double rhoerr = 0.0;
    for (;;) {
        CK(cudaMemsetAsync(c->d_max, 0, sizeof(unsigned long long), c->stream));
        CK(launch_prerelax(c->s, c->parity, c->d_uf, c->d_rho, c->d_max, c->stream));
        c->parity ^= 1;
        unsigned long long bits = 0;
        CK(cudaMemcpyAsync(&bits, c->d_max, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
        if (int rc = sync(c)) return rc;
        std::memcpy(&rhoerr, &bits, sizeof(double));
        if (!(rhoerr == rhoerr)) return fail(LBM_ERR_NONFINITE, "NaN density during pre-relaxation");
        if (rhoerr <= eps || istep > maxit) break;   // main.f90:85
        ++istep;
    }
    if (iters) *iters = istep;
    if (err) *err = rhoerr;
    c->nsteps = 0;
    if (rhoerr > eps) return fail(LBM_ERR_NOT_CONVERGED, "pre-relaxation exceeded maxit");
    return LBM_OK;
}

int lbm_macrovar(lbm_ctx* c, double* rho, double* ux, double* uy, double* uz) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (int rc = set_device(c)) return rc;
    const int k = chunk_planes(c, 4);
    const size_t pp = plane_nodes(c->p);
    double* outs[4] = {rho, ux, uy, uz};
    for (int z0 = 0; z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        const size_t n = (size_t)nzc * pp;
        double* d[4];
        for (int a = 0; a < 4; ++a) d[a] = outs[a] ? c->d_stage + a * n : nullptr;
        CK(launch_macro(c->s, c->parity, d[0], d[1], d[2], d[3], z0, nzc, c->stream));
        for (int a = 0; a < 4; ++a)
            if (outs[a])
                CK(cudaMemcpyAsync(outs[a] + (size_t)z0 * pp, d[a], n * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    return sync(c);
}

int lbm_strain(lbm_ctx* c, double* m1, double* m2) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (!m1 && !m2) return LBM_OK;
    if (int rc = set_device(c)) return rc;
    const int k = chunk_planes(c, 2);
    const size_t pp = plane_nodes(c->p);
    for (int z0 = 0; z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        const size_t n = (size_t)nzc * pp;
        double* d1 = m1 ? c->d_stage : nullptr;
        double* d2 = m2 ? c->d_stage + n : nullptr;
        CK(launch_strain(c->s, c->parity, d1, d2, z0, nzc, c->stream));
        if (m1) CK(cudaMemcpyAsync(m1 + (size_t)z0 * pp, d1, n * 8, cudaMemcpyDeviceToHost, c->stream));
        if (m2) CK(cudaMemcpyAsync(m2 + (size_t)z0 * pp, d2, n * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    return sync(c);
}

int lbm_les_wall_damping(lbm_ctx* c, double aplus) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (!(aplus >= 0.0) || !std::isfinite(aplus)) return fail(LBM_ERR_INVALID_ARG, "A+ must be finite and >= 0");
    c->s.les_aplus = (float)aplus;
    return LBM_OK;
}

int lbm_les_set(lbm_ctx* c, const float* params, const float* norm, double ustar, double h) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (int rc = set_device(c)) return rc;
    if (!params) {
        c->s.les_w = nullptr;
        c->s.use_rows = c->use_rows_saved;
        return LBM_OK;
    }
    if (!norm || !(ustar > 0.0) || !(h > 0.0)) return fail(LBM_ERR_INVALID_ARG, "closure needs norm, ustar > 0, h > 0");
    if (c->p.precision == LBM_PREC_FP16) return fail(LBM_ERR_INVALID_ARG, "the LES closure runs with FP32 or FP64 storage");
    if (c->P.npart > 0) return fail(LBM_ERR_STATE, "the LES closure is for particle-free channels");
    if (!c->d_les) {
        CK(cudaMalloc(&c->d_les, (LBM_MLP_PARAMS + LBM_MLP_NORM) * sizeof(float)));
        CK(cudaMalloc(&c->d_s9, c->s.N * sizeof(float)));
    }
    CK(cudaMemcpyAsync(c->d_les, params, LBM_MLP_PARAMS * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_les + LBM_MLP_PARAMS, norm, LBM_MLP_NORM * sizeof(float), cudaMemcpyHostToDevice,
                       c->stream));
    {
        // the first collision's features use the molecular rate
        std::vector<float> s9(c->s.N, (float)c->p.s9);
        CK(cudaMemcpyAsync(c->d_s9, s9.data(), c->s.N * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->s.les_w = c->d_les;
    c->s.les_s9 = c->d_s9;
    c->s.les_nu = (1.0 / c->p.s9 - 0.5) / 3.0;
    c->s.les_ustar = (float)ustar;
    c->s.les_h = (float)h;
    c->s.use_rows = 0;
    return sync(c);
}

int lbm_les_training_data(lbm_ctx* c, int32_t factor, double ustar, double h, float* X, float* y, double* ubar) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (factor < 1 || c->p.nx % factor || c->p.ny % factor || c->p.nz % factor || !(ustar > 0.0) || !(h > 0.0))
        return fail(LBM_ERR_INVALID_ARG, "factor must divide nx, ny, nz; ustar and h positive");
    if (c->P.npart > 0) return fail(LBM_ERR_STATE, "training data come from a particle-free channel");
    if (int rc = set_device(c)) return rc;
    const int nxc = c->p.nx / factor, nyc = c->p.ny / factor, nzc = c->p.nz / factor;
    const size_t nc = (size_t)nxc * nyc * nzc;
    double* d9 = nullptr;
    float* dxy = nullptr;
    CK(cudaMalloc(&d9, 9 * nc * sizeof(double)));
    int rc = LBM_OK;
    do {
        if (cudaMalloc(&dxy, (LBM_MLP_IN + 1) * nc * sizeof(float)) != cudaSuccess) { rc = fail(LBM_ERR_CUDA, "cudaMalloc"); break; }
        const double nu_f = (1.0 / c->p.s9 - 0.5) / 3.0;
        cudaError_t e = launch_box_filter(c->s, c->parity, factor, nxc, nyc, nzc, d9, c->stream);
        if (e == cudaSuccess)
            e = launch_closure_targets(d9, nxc, nyc, nzc, (float)(nu_f / factor), (float)ustar, (float)(h / factor),
                                       dxy, dxy + LBM_MLP_IN * nc, c->stream);
        if (e == cudaSuccess && X) e = cudaMemcpyAsync(X, dxy, LBM_MLP_IN * nc * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && y) e = cudaMemcpyAsync(y, dxy + LBM_MLP_IN * nc, nc * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && ubar) e = cudaMemcpyAsync(ubar, d9, 3 * nc * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { rc = fail(LBM_ERR_CUDA, std::string("closure training data: ") + cudaGetErrorString(e)); break; }
    } while (false);
    cudaFree(d9);
    cudaFree(dxy);
    if (rc) return rc;
    return sync(c);
}

int lbm_les_features(lbm_ctx* c, double ustar, double h, float* X) {
    if (check_ctx(c) || !X || !(ustar > 0.0) || !(h > 0.0)) return fail(LBM_ERR_INVALID_ARG, "bad argument");
    if (int rc = set_device(c)) return rc;
    float* d = nullptr;
    CK(cudaMalloc(&d, c->s.N * LBM_MLP_IN * sizeof(float)));
    cudaError_t e = launch_les_features(c->s, c->parity, (float)ustar, (float)h, d, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(X, d, c->s.N * LBM_MLP_IN * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("closure features: ") + cudaGetErrorString(e));
    return sync(c);
}

int lbm_les_nut(lbm_ctx* c, double* nut) {
    if (check_ctx(c) || !nut) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (!c->s.les_w) return fail(LBM_ERR_STATE, "the LES closure is off (lbm_les_set)");
    if (int rc = set_device(c)) return rc;
    std::vector<float> s9(c->s.N);
    CK(cudaMemcpyAsync(s9.data(), c->d_s9, c->s.N * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (int rc = sync(c)) return rc;
    const double nu = c->s.les_nu;
    const Geometry& g = c->s.g;
    for (int Z = 0; Z < g.NZ; ++Z)
        for (int Y = 0; Y < g.NY; ++Y)
            for (int X = 0; X < g.NX; ++X) {
                const double s = s9[(size_t)X + (size_t)g.NX * ((size_t)Y + (size_t)g.NY * Z)];
                // GPU (X, Y, Z) = reference (y, z, x)
                nut[(size_t)Z + (size_t)c->p.nx * ((size_t)X + (size_t)c->p.ny * Y)] = ((1.0 / s - 0.5) / 3.0) / nu - 1.0;
            }
    return LBM_OK;
}

int lbm_profiles(lbm_ctx* c, double* out) {
    if (check_ctx(c) || !out) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (int rc = set_device(c)) return rc;
    const int nb = profile_blocks(c->s);
    const size_t need = (size_t)c->s.g.NZ * nb * LBM_PROFILE_COLS;
    if (int rc = ensure_red(c, need)) return rc;
    CK(launch_profiles(c->s, c->parity, c->d_red, nb, c->stream));
    std::vector<double> h(need);
    CK(cudaMemcpyAsync(h.data(), c->d_red, need * 8, cudaMemcpyDeviceToHost, c->stream));
    if (int rc = sync(c)) return rc;
    for (int z = 0; z < c->s.g.NZ; ++z)
        for (int k = 0; k < LBM_PROFILE_COLS; ++k) {
            double acc = 0.0;
            for (int b = 0; b < nb; ++b) acc += h[((size_t)z * nb + b) * LBM_PROFILE_COLS + k];
            out[k + (size_t)LBM_PROFILE_COLS * z] = acc;
        }
    return LBM_OK;
}

int lbm_dissipation(lbm_ctx* c, double* out) {
    if (check_ctx(c) || !out) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (int rc = set_device(c)) return rc;
    const int nb = profile_blocks(c->s);
    const size_t need = (size_t)c->s.g.NZ * nb * LBM_DISSIPATION_COLS;
    if (int rc = ensure_red(c, need)) return rc;
    CK(launch_dissipation(c->s, c->parity, c->d_red, nb, c->stream));
    std::vector<double> h(need);
    CK(cudaMemcpyAsync(h.data(), c->d_red, need * 8, cudaMemcpyDeviceToHost, c->stream));
    if (int rc = sync(c)) return rc;
    for (int z = 0; z < c->s.g.NZ; ++z)
        for (int k = 0; k < LBM_DISSIPATION_COLS; ++k) {
            double acc = 0.0;
            for (int b = 0; b < nb; ++b) acc += h[((size_t)z * nb + b) * LBM_DISSIPATION_COLS + k];
            out[k + (size_t)LBM_DISSIPATION_COLS * z] = acc;
        }
    return LBM_OK;
}

int lbm_diag(lbm_ctx* c, lbm_stats* st) {
    if (check_ctx(c) || !st) return fail(LBM_ERR_INVALID_ARG, "null argument");
    std::vector<double> prof((size_t)LBM_PROFILE_COLS * c->p.nx);
    if (int rc = lbm_profiles(c, prof.data())) return rc;
    std::memset(st, 0, sizeof(*st));
    double n = 0.0;
    for (int ix = 0; ix < c->p.nx; ++ix) {
        const double* r = &prof[(size_t)LBM_PROFILE_COLS * ix];
        st->mom_sum[0] += r[0]; st->mom_sum[1] += r[1]; st->mom_sum[2] += r[2];
        st->usq_sum[0] += r[6]; st->usq_sum[1] += r[7]; st->usq_sum[2] += r[8];
        st->rho_sum += r[9];
        n += r[11];
    }
    const size_t need = (size_t)kExtremaBlocks * 5;
    if (int rc = ensure_red(c, need)) return rc;
    CK(launch_extrema(c->s, c->parity, c->d_red, c->stream));
    std::vector<double> h(need);
    CK(cudaMemcpyAsync(h.data(), c->d_red, need * 8, cudaMemcpyDeviceToHost, c->stream));
    if (int rc = sync(c)) return rc;
    double rmax = -INFINITY, rmin = INFINITY, vmax = -1.0, vidx = 1e300, nonf = 0.0;
    for (int b = 0; b < kExtremaBlocks; ++b) {
        const double* r = &h[(size_t)b * 5];
        rmax = std::max(rmax, r[0]);
        rmin = std::min(rmin, r[1]);
        if (r[2] > vmax || (r[2] == vmax && r[3] < vidx)) { vmax = r[2]; vidx = r[3]; }
        nonf += r[4];
    }
    st->nfluid = (int64_t)(n + 0.5);
    st->rho_max = rmax;
    st->rho_min = rmin;
    st->vmax = vmax;
    const int64_t li = (int64_t)vidx;
    st->vmax_at[0] = (int32_t)(li % c->p.nx) + 1;
    st->vmax_at[1] = (int32_t)((li / c->p.nx) % c->p.ny) + 1;
    st->vmax_at[2] = (int32_t)(li / ((int64_t)c->p.nx * c->p.ny)) + 1;
    st->nonfinite = (int32_t)nonf;
    return st->nonfinite ? fail(LBM_ERR_NONFINITE, "non-finite populations present") : LBM_OK;
}

int lbm_avedensity(lbm_ctx* c, double* mean) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    std::vector<double> prof((size_t)LBM_PROFILE_COLS * c->p.nx);
    if (int rc = lbm_profiles(c, prof.data())) return rc;
    double s = 0.0, n = 0.0;
    for (int ix = 0; ix < c->p.nx; ++ix) {
        s += prof[(size_t)LBM_PROFILE_COLS * ix + 9];
        n += prof[(size_t)LBM_PROFILE_COLS * ix + 11];
    }
    const double m = n > 0 ? s / n : 0.0;
    if (mean) *mean = m;
    CK(launch_add_rest(c->s, c->parity, -m, c->stream));
    return sync(c);
}

int lbm_save_flow(lbm_ctx* c, const char* path, int32_t kind, const int32_t* ints) {
    if (check_ctx(c) || !path || !ints) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (kind != 0 && kind != 1) return fail(LBM_ERR_INVALID_ARG, "kind must be 0 or 1");
    if (int rc = set_device(c)) return rc;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(LBM_ERR_IO, std::string("cannot open ") + path);
    const int nints = kind == 0 ? 1 : 3;
    {
        RecordWriter w(fp, 4 * nints);
        w.put(ints, 4 * nints);
        if (!w.ok) { std::fclose(fp); return fail(LBM_ERR_IO, "write failed"); }
    }
    const size_t per_plane = plane_nodes(c->p) * Q;
    RecordWriter w(fp, (int64_t)(nodes(c->p) * Q * 8));
    const int k = chunk_planes(c, Q);
    std::vector<double> h((size_t)k * per_plane);
    for (int z0 = 0; z0 < c->p.nz && w.ok; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        cudaError_t e = launch_store_to_aos(c->s, c->parity, c->d_stage, z0, nzc, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h.data(), c->d_stage, (size_t)nzc * per_plane * 8, cudaMemcpyDeviceToHost,
                                c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { std::fclose(fp); return cuda_fail(e, "checkpoint download"); }
        w.put(h.data(), (int64_t)nzc * per_plane * 8);
    }
    const bool ok = w.ok && w.done == w.total;
    if (std::fclose(fp) != 0 || !ok) return fail(LBM_ERR_IO, "write failed");
    return LBM_OK;
}

int lbm_load_flow(lbm_ctx* c, const char* path, int32_t kind, int32_t* ints) {
    if (check_ctx(c) || !path) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (kind != 0 && kind != 1) return fail(LBM_ERR_INVALID_ARG, "kind must be 0 or 1");
    if (int rc = set_device(c)) return rc;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(LBM_ERR_IO, std::string("cannot open ") + path);
    const int nints = kind == 0 ? 1 : 3;
    int32_t hdr[3] = {0, 0, 0};
    {
        RecordReader r(fp);
        if (!r.ok || !r.get(hdr, 4 * nints) || !r.finish()) {
            std::fclose(fp);
            return fail(LBM_ERR_IO, "bad header record (expected " + std::to_string(nints) + " integers)");
        }
    }
    RecordReader r(fp);
    const size_t per_plane = plane_nodes(c->p) * Q;
    const int k = chunk_planes(c, Q);
    std::vector<double> h((size_t)k * per_plane);
    for (int z0 = 0; z0 < c->p.nz; z0 += k) {
        const int nzc = std::min(k, c->p.nz - z0);
        if (!r.get(h.data(), (int64_t)nzc * per_plane * 8)) {
            std::fclose(fp);
            return fail(LBM_ERR_IO, "population record too short for this lattice");
        }
        cudaError_t e = cudaMemcpyAsync(c->d_stage, h.data(), (size_t)nzc * per_plane * 8,
                                        cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = launch_aos_to_store(c->s, c->d_stage, z0, nzc, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { std::fclose(fp); return cuda_fail(e, "checkpoint upload"); }
    }
    const bool exact = r.finish();
    std::fclose(fp);
    if (!exact) return fail(LBM_ERR_IO, "population record size does not match this lattice");
    if (ints) for (int i = 0; i < nints; ++i) ints[i] = hdr[i];
    c->parity = 0;
    c->nsteps = 0;
    return LBM_OK;
}

int lbm_particle_params_init(lbm_particle_params* pp, int32_t npart, double radius, double rho_ratio) {
    if (!pp) return fail(LBM_ERR_INVALID_ARG, "null params");
    if (npart < 0 || !(radius > 0.0) || !(rho_ratio > 0.0)) return fail(LBM_ERR_INVALID_ARG, "bad sphere parameters");
    std::memset(pp, 0, sizeof(*pp));
    pp->npart = npart;
    pp->radius = radius;
    pp->rho_ratio = rho_ratio;
    // Feng & Michaelides stiffness constants of para.f90:357-360
    pp->stf0 = 0.025; pp->stf1 = 0.002; pp->stf0_w = 0.025; pp->stf1_w = 0.002;
    pp->zeta = 1.0;
    return LBM_OK;
}

int lbm_particles_place(int32_t nx, int32_t ny, int32_t nz, int32_t npart, double radius, double gap,
                        double wall_gap, uint64_t seed, double* pos) {
    if (nx < 1 || ny < 1 || nz < 1 || npart < 0 || !(radius > 0.0) || !pos || gap < 0 || wall_gap < 0)
        return fail(LBM_ERR_INVALID_ARG, "bad placement arguments");
    const double lo = radius + wall_gap, hi = (double)nx - radius - wall_gap;
    if (!(hi > lo)) return fail(LBM_ERR_INVALID_ARG, "channel too narrow for the spheres");
    const double dmin = 2.0 * radius + gap;
    // cell grid for the overlap test: cells at least dmin wide
    const int cy = std::max(1, (int)(ny / dmin)), cz = std::max(1, (int)(nz / dmin)), cx = std::max(1, (int)(nx / dmin));
    std::vector<std::vector<int>> cells((size_t)cx * cy * cz);
    auto cell_of = [&](double x, double y, double z, int& a, int& b, int& c2) {
        a = std::min(cx - 1, (int)(x / nx * cx));
        b = std::min(cy - 1, (int)(y / ny * cy));
        c2 = std::min(cz - 1, (int)(z / nz * cz));
    };
    auto mi = [](double d, double L) { return d >= 0.5 * L ? d - L : (d < -0.5 * L ? d + L : d); };
    uint64_t key = 0;
    for (int32_t k = 0; k < npart; ++k) {
        bool placed = false;
        for (int attempt = 0; attempt < 100000 && !placed; ++attempt) {
            const double x = lo + (hi - lo) * 0.5 * (uniform_pm1(seed, key++) + 1.0);
            const double y = ny * 0.5 * (uniform_pm1(seed, key++) + 1.0);
            const double z = nz * 0.5 * (uniform_pm1(seed, key++) + 1.0);
            int a, b, c2;
            cell_of(x, y, z, a, b, c2);
            bool ok = true;
            for (int da = -1; da <= 1 && ok; ++da) {
                const int aa = a + da;
                if (aa < 0 || aa >= cx) continue;
                for (int db = -1; db <= 1 && ok; ++db) {
                    if (cy < 3 && db != 0 && (cy == 1 || db == 1)) continue;
                    const int bb = ((b + db) % cy + cy) % cy;
                    for (int dc = -1; dc <= 1 && ok; ++dc) {
                        if (cz < 3 && dc != 0 && (cz == 1 || dc == 1)) continue;
                        const int cc = ((c2 + dc) % cz + cz) % cz;
                        for (int j : cells[((size_t)aa * cy + bb) * cz + cc]) {
                            const double d0 = pos[3 * j] - x, d1 = mi(pos[3 * j + 1] - y, ny), d2 = mi(pos[3 * j + 2] - z, nz);
                            if (d0 * d0 + d1 * d1 + d2 * d2 < dmin * dmin) { ok = false; break; }
                        }
                    }
                }
            }
            if (!ok) continue;
            pos[3 * k] = x; pos[3 * k + 1] = y; pos[3 * k + 2] = z;
            cells[((size_t)a * cy + b) * cz + c2].push_back(k);
            placed = true;
        }
        if (!placed) return fail(LBM_ERR_INVALID_ARG, "could not place all spheres (volume fraction too high)");
    }
    return LBM_OK;
}

int lbm_particles_set(lbm_ctx* c, const lbm_particle_params* pp, const double* pos, const double* vel,
                      const double* omg) {
    if (check_ctx(c) || !pp || (pp->npart > 0 && !pos)) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (pp->npart < 0 || !(pp->radius > 0.0) || !(pp->rho_ratio > 0.0) || !(pp->zeta > 0.0))
        return fail(LBM_ERR_INVALID_ARG, "bad sphere parameters");
    // the bounce-back kernel stages a sphere's bounding box in shared memory,
    // and the periodic spans must hold a sphere with its stencil reach
    const size_t smem = lbm::particles_smem_bytes(pp->radius);
    if (smem == 0 || smem > 227u * 1024u)
        return fail(LBM_ERR_INVALID_ARG, "sphere radius too large (at most 27 lattice units)");
    if (pp->npart > 0 && ((double)c->p.ny < 2.0 * pp->radius + 8.0 || (double)c->p.nz < 2.0 * pp->radius + 8.0))
        return fail(LBM_ERR_INVALID_ARG, "periodic span smaller than 2*radius + 8");
    for (int32_t k = 0; k < pp->npart; ++k) {
        const double x = pos[3 * k];
        if (!(x - pp->radius > 0.0) || !(x + pp->radius < (double)c->p.nx))
            return fail(LBM_ERR_INVALID_ARG, "sphere " + std::to_string(k) + " crosses a wall");
        if (!std::isfinite(pos[3 * k + 1]) || !std::isfinite(pos[3 * k + 2]))
            return fail(LBM_ERR_INVALID_ARG, "non-finite sphere position");
    }
    if (int rc = set_device(c)) return rc;
    const int n = pp->npart;
    DeviceParticles& P = c->P;
    // Detach the old spheres before their arrays are freed: a failure below
    // then leaves a particle-free context, never one whose step or field
    // kernels read freed or null sphere arrays.
    P.npart = 0;
    c->s.owner = nullptr;
    c->s.ppos = c->s.pvel = c->s.pomg = nullptr;
    if (P.pos) { cudaFree(P.pos); P.pos = nullptr; }
    if (P.geom) { cudaFree(P.geom); P.geom = nullptr; }
    if (P.order) { cudaFree(P.order); P.order = nullptr; }
    if (!P.owner) CK(cudaMalloc(&P.owner, c->s.N * sizeof(int)));
    if (!P.counters) CK(cudaMalloc(&P.counters, 4 * sizeof(unsigned)));
    if (!c->d_count) CK(cudaMalloc(&c->d_count, sizeof(unsigned long long)));
    if (!c->d_mass) CK(cudaMalloc(&c->d_mass, 2 * sizeof(double)));
    if (!c->side.st) {
        // the sphere pass's second stream; set only once all three exist
        if (!c->side.fork) CK(cudaEventCreateWithFlags(&c->side.fork, cudaEventDisableTiming));
        if (!c->side.join) CK(cudaEventCreateWithFlags(&c->side.join, cudaEventDisableTiming));
        cudaStream_t st = nullptr;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        c->side.st = st;
    }
    const int cap = std::max(4096, 64 * n);
    if (P.refill_cap < cap) {
        cudaFree(P.refill_node);
        cudaFree(P.refill_part);
        P.refill_node = nullptr;
        P.refill_part = nullptr;
        CK(cudaMalloc(&P.refill_node, (size_t)cap * sizeof(uint32_t)));
        CK(cudaMalloc(&P.refill_part, (size_t)cap * sizeof(int)));
        P.refill_cap = cap;
    }
    const size_t m = 3 * (size_t)std::max(n, 1);
    CK(cudaMalloc(&P.pos, 9 * m * sizeof(double)));
    P.vel = P.pos + m; P.omg = P.vel + m; P.force = P.omg + m; P.torque = P.force + m;
    P.fprev = P.torque + m; P.tprev = P.fprev + m; P.rep = P.tprev + m; P.pos_prev = P.rep + m;
    CK(cudaMemsetAsync(P.pos, 0, 9 * m * sizeof(double), c->stream));
    CK(cudaMalloc(&P.geom, (size_t)std::max(n, 1) * sizeof(SphereGeom)));
    if (n > 0) {
        CK(cudaMemcpyAsync(P.pos, pos, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(P.pos_prev, pos, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        if (vel) CK(cudaMemcpyAsync(P.vel, vel, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        if (omg) CK(cudaMemcpyAsync(P.omg, omg, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaMemsetAsync(P.counters, 0, 4 * sizeof(unsigned), c->stream));
    CK(cudaMemsetAsync(P.owner, 0xff, c->s.N * sizeof(int), c->stream));   // -1: fluid
    {
        // repulsion cells at least one reach (2R + zeta) wide; three or more
        // cells per periodic span, else the all-pairs search
        const double reach = 2.0 * pp->radius + pp->zeta + 0.05;
        const int ny = (int)std::floor((double)c->p.ny / reach), nz = (int)std::floor((double)c->p.nz / reach);
        const int nx = std::max(1, (int)std::floor((double)c->p.nx / reach));
        const long long ncell = (long long)nx * ny * nz;
        cudaFree(P.cell_count);
        P.cell_count = nullptr;
        P.cell_list = nullptr;
        P.ncell = 0;
        if (n > 1 && ny >= 3 && nz >= 3 && ncell <= (1LL << 24)) {
            CK(cudaMalloc(&P.cell_count, (size_t)ncell * (1 + kCellCap) * sizeof(int)));
            P.cell_list = P.cell_count + ncell;
            P.ncell = (int)ncell;
            P.cell_nx = nx; P.cell_ny = ny; P.cell_nz = nz;
        }
    }
    P.npart = n;
    P.R = pp->radius; P.rho_ratio = pp->rho_ratio;
    P.Rf = (float)pp->radius;
    P.q_fp64 = (pp->flags & LBM_PFLAG_Q_FP64) ? 1 : 0;
    P.stf0 = pp->stf0; P.stf1 = pp->stf1; P.stf0_w = pp->stf0_w; P.stf1_w = pp->stf1_w; P.zeta = pp->zeta;
    c->pp = *pp;
    c->have_prev = 0;
    if (n > 0) {
        // the bounce-back kernel's spatial order: Morton cells 2R wide, at
        // most 2^7 per axis (coarser cells on larger domains)
        double cs = 2.0 * pp->radius;
        int bits = 0;
        for (;;) {
            const int mx = (int)std::ceil(std::max({(double)c->p.nx, (double)c->p.ny, (double)c->p.nz}) / cs);
            bits = 0;
            while ((1 << bits) < mx) ++bits;
            if (bits <= 7) break;
            cs *= 2.0;
        }
        P.order_cs = cs;
        P.order_nbins = 1 << (3 * bits);
        CK(cudaMalloc(&P.order, (2 * (size_t)n + (size_t)P.order_nbins) * sizeof(int)));
        P.order_key = P.order + n;
        P.order_hist = P.order_key + n;
    }
    CK(particles_claim(c->s, P, c->stream));
    CK(particles_reorder(P, c->stream));
    c->order_age = 0;
    c->s.owner = P.owner;
    c->s.ppos = P.pos; c->s.pvel = P.vel; c->s.pomg = P.omg;
    c->s.prho = pp->rho_ratio;
    return sync(c);
}

int lbm_particles_get(lbm_ctx* c, double* pos, double* vel, double* omg, double* force, double* torque) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (c->P.npart == 0) return fail(LBM_ERR_STATE, "no spheres set");
    if (int rc = set_device(c)) return rc;
    const size_t b = 3 * (size_t)c->P.npart * sizeof(double);
    const double* src[5] = {c->P.pos, c->P.vel, c->P.omg, c->P.force, c->P.torque};
    double* dst[5] = {pos, vel, omg, force, torque};
    for (int k = 0; k < 5; ++k)
        if (dst[k]) CK(cudaMemcpyAsync(dst[k], src[k], b, cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int lbm_particles_get_history(lbm_ctx* c, double* fprev, double* tprev) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (c->P.npart == 0) return fail(LBM_ERR_STATE, "no spheres set");
    if (int rc = set_device(c)) return rc;
    const size_t b = 3 * (size_t)c->P.npart * sizeof(double);
    if (fprev) CK(cudaMemcpyAsync(fprev, c->P.fprev, b, cudaMemcpyDeviceToHost, c->stream));
    if (tprev) CK(cudaMemcpyAsync(tprev, c->P.tprev, b, cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int lbm_particles_set_history(lbm_ctx* c, const double* fprev, const double* tprev) {
    if (check_ctx(c) || !fprev || !tprev) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (c->P.npart == 0) return fail(LBM_ERR_STATE, "no spheres set");
    const size_t m = 3 * (size_t)c->P.npart;
    for (size_t k = 0; k < m; ++k)
        if (!std::isfinite(fprev[k]) || !std::isfinite(tprev[k])) return fail(LBM_ERR_INVALID_ARG, "non-finite history");
    if (int rc = set_device(c)) return rc;
    CK(cudaMemcpyAsync(c->P.fprev, fprev, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->P.tprev, tprev, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (int rc = sync(c)) return rc;
    c->have_prev = 1;
    return LBM_OK;
}

// savecntdpart / loadcntdpart (saveload.f90:604-693) for one process.
int lbm_save_part(lbm_ctx* c, const char* path) {
    if (check_ctx(c) || !path) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (c->P.npart == 0) return fail(LBM_ERR_STATE, "no spheres set");
    if (int rc = set_device(c)) return rc;
    const int np = c->P.npart;
    const size_t msize = 10 * (size_t)np;                  // para.f90:369 with nproc = 1
    const size_t m3 = 3 * (size_t)np;
    std::vector<double> st(5 * m3);                         // pos, vel, omg, fprev, tprev
    const double* src[5] = {c->P.pos, c->P.vel, c->P.omg, c->P.fprev, c->P.tprev};
    for (int k = 0; k < 5; ++k)
        CK(cudaMemcpyAsync(st.data() + k * m3, src[k], m3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (int rc = sync(c)) return rc;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(LBM_ERR_IO, std::string("cannot open ") + path);
    bool ok = true;
    auto record = [&](std::initializer_list<std::pair<const void*, int64_t>> parts) {
        int64_t total = 0;
        for (auto& q : parts) total += q.second;
        RecordWriter w(fp, total);
        for (auto& q : parts) w.put(q.first, q.second);
        ok = ok && w.ok && w.done == w.total;
    };
    // {nps, ipglb(msize)}
    std::vector<int32_t> ipglb(msize, 0);
    for (int k = 0; k < np; ++k) ipglb[k] = k + 1;
    const int32_t nps = np;
    record({{&nps, 4}, {ipglb.data(), (int64_t)(4 * msize)}});
    // {ibnodes(lx,ly,lz), isnodes(lx,ly,lz)}: converted plane chunks
    if (ok) {
        const size_t pp = plane_nodes(c->p);
        const int kz = chunk_planes(c, 1);
        RecordWriter w(fp, (int64_t)(8 * nodes(c->p)));
        std::vector<int32_t> h(2 * (size_t)kz * pp);
        for (int pass = 0; pass < 2 && w.ok; ++pass) {
            for (int z0 = 0; z0 < c->p.nz && w.ok; z0 += kz) {
                const int nzc = std::min(kz, c->p.nz - z0);
                int32_t* ib = reinterpret_cast<int32_t*>(c->d_stage);
                int32_t* is = ib + (size_t)nzc * pp;
                cudaError_t e = launch_owner_to_ref(c->s, c->P.owner, ib, is, z0, nzc, c->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(h.data(), pass == 0 ? ib : is, (size_t)nzc * pp * 4, cudaMemcpyDeviceToHost,
                                        c->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
                if (e != cudaSuccess) { std::fclose(fp); return cuda_fail(e, "node flags download"); }
                w.put(h.data(), (int64_t)nzc * pp * 4);
            }
        }
        ok = w.ok && w.done == w.total;
    }
    // {yp, thetap}, {forcepp, torqpp}, {dwdt, domgdt}: local arrays of msize
    // particles (here the first npart); thetap is not integrated (zero);
    // dwdt, domgdt = total force / mass and torque / moment of inertia of the
    // last step
    std::vector<double> a(3 * msize, 0.0), b(3 * msize, 0.0);
    auto fill = [&](std::vector<double>& v, const double* x, double scale) {
        std::fill(v.begin(), v.end(), 0.0);
        for (size_t k = 0; k < m3; ++k) v[k] = x[k] * scale;
    };
    const double R = c->P.R;
    const double mass = c->P.rho_ratio * (4.0 / 3.0 * 3.14159265358979323846 * R * R * R);
    const double inertia = 0.4 * mass * R * R;
    const int64_t lb = (int64_t)(8 * 3 * msize);
    fill(a, st.data(), 1.0);
    std::fill(b.begin(), b.end(), 0.0);
    if (ok) record({{a.data(), lb}, {b.data(), lb}});
    fill(a, st.data() + 3 * m3, 1.0);
    fill(b, st.data() + 4 * m3, 1.0);
    if (ok) record({{a.data(), lb}, {b.data(), lb}});
    fill(a, st.data() + 3 * m3, 1.0 / mass);
    fill(b, st.data() + 4 * m3, 1.0 / inertia);
    if (ok) record({{a.data(), lb}, {b.data(), lb}});
    // {ypglb, wp, omgp} (process 0)
    const int64_t gb = (int64_t)(8 * m3);
    if (ok) record({{st.data(), gb}, {st.data() + m3, gb}, {st.data() + 2 * m3, gb}});
    if (std::fclose(fp) != 0 || !ok) return fail(LBM_ERR_IO, "write failed");
    return LBM_OK;
}

int lbm_load_part(lbm_ctx* c, const char* path, const lbm_particle_params* pp) {
    if (check_ctx(c) || !path || !pp) return fail(LBM_ERR_INVALID_ARG, "null argument");
    if (pp->npart <= 0) return fail(LBM_ERR_INVALID_ARG, "npart must be positive");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(LBM_ERR_IO, std::string("cannot open ") + path);
    const int np = pp->npart;
    const size_t m3 = 3 * (size_t)np;
    auto bad = [&](const std::string& why) { std::fclose(fp); return fail(LBM_ERR_IO, why); };
    // {nps, ipglb(msize)}: msize from the record length
    std::vector<int32_t> ipglb;
    size_t msize = 0;
    {
        RecordReader r(fp);
        int32_t nps = 0;
        if (!r.ok || r.more || r.total < 4 || (r.total - 4) % 4 != 0 || !r.get(&nps, 4))
            return bad("bad {nps, ipglb} record");
        msize = (size_t)(r.total - 4) / 4;
        if (nps != np || msize < (size_t)np) return bad("file holds " + std::to_string(nps) + " spheres, expected " +
                                                        std::to_string(np));
        ipglb.resize(msize);
        if (!r.get(ipglb.data(), (int64_t)(4 * msize)) || !r.finish()) return bad("bad {nps, ipglb} record");
        std::vector<char> seen(np, 0);
        for (int k = 0; k < np; ++k) {
            const int id = ipglb[k];
            if (id < 1 || id > np || seen[id - 1]) return bad("ipglb is not a permutation of 1..npart");
            seen[id - 1] = 1;
        }
    }
    // {ibnodes, isnodes} and {yp, thetap}: rebuilt from the centres / unused
    for (int k = 0; k < 2; ++k) {
        RecordReader r(fp);
        if (r.ok) r.finish();                                   // skip: finish() is false for a partial read
        if (!r.ok) return bad("truncated particle checkpoint");
    }
    // {forcepp, torqpp} in local order -> global order
    std::vector<double> fl(3 * msize), tl(3 * msize), fprev(m3), tprev(m3);
    {
        RecordReader r(fp);
        if (!r.ok || !r.get(fl.data(), (int64_t)(8 * 3 * msize)) || !r.get(tl.data(), (int64_t)(8 * 3 * msize)) ||
            !r.finish())
            return bad("bad {forcepp, torqpp} record");
        for (int k = 0; k < np; ++k)
            for (int a = 0; a < 3; ++a) {
                fprev[3 * (ipglb[k] - 1) + a] = fl[3 * k + a];
                tprev[3 * (ipglb[k] - 1) + a] = tl[3 * k + a];
            }
    }
    {
        RecordReader r(fp);                                     // {dwdt, domgdt}
        if (r.ok) r.finish();
        if (!r.ok) return bad("truncated particle checkpoint");
    }
    std::vector<double> g(3 * m3);                              // ypglb, wp, omgp
    {
        RecordReader r(fp);
        if (!r.ok || !r.get(g.data(), (int64_t)(8 * 3 * m3)) || !r.finish())
            return bad("bad {ypglb, wp, omgp} record");
    }
    std::fclose(fp);
    if (int rc = lbm_particles_set(c, pp, g.data(), g.data() + m3, g.data() + 2 * m3)) return rc;
    return lbm_particles_set_history(c, fprev.data(), tprev.data());
}

int lbm_particle_counts(lbm_ctx* c, int64_t* nsolid, int64_t* nlinks, int64_t* nrefill) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (c->P.npart == 0) {
        if (nsolid) *nsolid = 0;
        if (nlinks) *nlinks = 0;
        if (nrefill) *nrefill = 0;
        return LBM_OK;
    }
    if (int rc = set_device(c)) return rc;
    unsigned cnt[4];
    CK(cudaMemcpyAsync(cnt, c->P.counters, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
    unsigned long long ns = 0;
    CK(particles_count_solid(c->s, c->P, c->d_count, c->stream));
    CK(cudaMemcpyAsync(&ns, c->d_count, sizeof(ns), cudaMemcpyDeviceToHost, c->stream));
    if (int rc = sync(c)) return rc;
    if (nsolid) *nsolid = (int64_t)ns;
    if (nlinks) *nlinks = cnt[1];
    if (nrefill) *nrefill = cnt[0];
    return LBM_OK;
}

int lbm_timing_enable(lbm_ctx* c, int32_t capacity) {
    if (check_ctx(c) || capacity < 0) return fail(LBM_ERR_INVALID_ARG, "bad argument");
    if (int rc = set_device(c)) return rc;
    CK(cudaStreamSynchronize(c->stream));
    for (cudaEvent_t e : c->tev) cudaEventDestroy(e);
    c->tev.assign(3 * (size_t)capacity, nullptr);
    for (auto& e : c->tev) CK(cudaEventCreate(&e));
    c->tpar.assign(capacity, 0);
    c->tcap = capacity;
    c->tn = 0;
    return LBM_OK;
}

int lbm_step_launches(const lbm_ctx* c, int64_t* n) {
    if (!c || !n) return fail(LBM_ERR_INVALID_ARG, "null argument");
    *n = c->nlaunch;
    return LBM_OK;
}

int lbm_timing_get(lbm_ctx* c, double* fe, double* fo, double* pm, int64_t* ne, int64_t* no) {
    if (check_ctx(c)) return LBM_ERR_INVALID_ARG;
    if (int rc = sync(c)) return rc;
    double se = 0, so = 0, sp = 0;
    int64_t ce = 0, co = 0;
    for (int k = 0; k < c->tn; ++k) {
        float a = 0, b = 0;
        CK(cudaEventElapsedTime(&a, c->tev[3 * k], c->tev[3 * k + 1]));
        CK(cudaEventElapsedTime(&b, c->tev[3 * k + 1], c->tev[3 * k + 2]));
        if (c->tpar[k] == 0) { se += a; ++ce; } else { so += a; ++co; }
        sp += b;
    }
    if (fe) *fe = se;
    if (fo) *fo = so;
    if (pm) *pm = sp;
    if (ne) *ne = ce;
    if (no) *no = co;
    return LBM_OK;
}

}  // extern "C"
