// gd_api.cu -- host side of the C ABI declared in include/gd2d.h.
//
// Replaces the host part of the reference's main() (kernel.cu:3810-4470): allocation,
// host<->device transfer, the ping-pong step loop with funk_time, and error checks.  The
// reference checks every launch with cudaGetLastError + cudaDeviceSynchronize and calls
// exit(-1) (kernel.cu:4044-4084); here every entry point returns a status, never exits,
// and never synchronises unless it says so.
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <utility>

#include "../../include/gd2d.h"
#include "gd_internal.cuh"
#include "gd_ctx.h"
#include "gd_kernels.h"

using gd::CPlanes;
using gd::Params;
using gd::Planes;
using gd::Scalars;

namespace {
std::atomic<int> g_last_cuda_error{0};
// device / pinned-host allocations and releases made through the helpers below
std::atomic<long long> g_allocs{0}, g_frees{0};

gd_status cuda_fail(cudaError_t e) {
    g_last_cuda_error.store((int)e);
    return GD_ERR_CUDA;
}
}  // namespace

#define GD_CUDA(call)                                 \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_);  \
    } while (0)


namespace {

bool finite_pos(double v) { return std::isfinite(v) && v > 0.0; }

gd_status validate(const gd_config* c) {
    if (!c) return GD_ERR_INVALID_ARG;
    if (c->N < 3 || c->M < 3 || c->N > (1 << 28) || c->M > (1 << 28)) return GD_ERR_INVALID_ARG;
    if ((long long)c->N * c->M > (1LL << 40)) return GD_ERR_INVALID_ARG;
    if (!finite_pos(c->dx) || !finite_pos(c->dy)) return GD_ERR_INVALID_ARG;
    if (!std::isfinite(c->x0) || !std::isfinite(c->y0)) return GD_ERR_INVALID_ARG;
    if (!(std::isfinite(c->gamma) && c->gamma > 1.0)) return GD_ERR_INVALID_ARG;
    if (!finite_pos(c->krit)) return GD_ERR_INVALID_ARG;
    if (c->physics != GD_EULER && c->physics != GD_MHD) return GD_ERR_INVALID_ARG;
    if (c->geometry != GD_CARTESIAN && c->geometry != GD_AXISYM) return GD_ERR_INVALID_ARG;
    if (c->order != 1 && c->order != 2) return GD_ERR_INVALID_ARG;
    if (c->mode != GD_MODE_FAST && c->mode != GD_MODE_PARITY) return GD_ERR_INVALID_ARG;
    if (c->physics == GD_EULER && c->method != GD_METHOD_HLLC && c->method != GD_METHOD_HLL)
        return GD_ERR_INVALID_ARG;
    if (c->physics == GD_MHD && c->method != GD_METHOD_HLLC_MHD && c->method != GD_METHOD_HLLD)
        return GD_ERR_INVALID_ARG;
    for (int s = 0; s < 4; ++s)
        if (c->bc[s] < GD_BC_PERIODIC || c->bc[s] > GD_BC_AMBIENT_KEEPB) return GD_ERR_INVALID_ARG;
    if ((c->bc[0] == GD_BC_PERIODIC) != (c->bc[1] == GD_BC_PERIODIC)) return GD_ERR_INVALID_ARG;
    if ((c->bc[2] == GD_BC_PERIODIC) != (c->bc[3] == GD_BC_PERIODIC)) return GD_ERR_INVALID_ARG;
    // the axisymmetric sources divide by the radius y of every cell centre
    if (c->geometry == GD_AXISYM && !(c->y0 > 0.0)) return GD_ERR_INVALID_ARG;
    if (!(std::isfinite(c->frozen_radius) && c->frozen_radius >= 0.0)) return GD_ERR_INVALID_ARG;
    if (c->scheme < GD_SCHEME_TVD || c->scheme > GD_SCHEME_HANCOCK) return GD_ERR_INVALID_ARG;
    if (c->scheme != GD_SCHEME_TVD) {
        if (!finite_pos(c->x_max) || !finite_pos(c->y_max)) return GD_ERR_INVALID_ARG;
        // Kernel_GKR is written for one setting: axisymmetric MHD, HLLD faces (its metod 3,
        // kernel.cu:3123-3233) and its own ghost cells on the four sides (kernel.cu:2701-2960)
        const int want[4] = {GD_BC_MIRROR_X, GD_BC_OUTFLOW, GD_BC_AXIS, GD_BC_AMBIENT_KEEPB};
        if (c->physics != GD_MHD || c->geometry != GD_AXISYM || c->method != GD_METHOD_HLLD)
            return GD_ERR_UNSUPPORTED;
        for (int s = 0; s < 4; ++s)
            if (c->bc[s] != want[s]) return GD_ERR_UNSUPPORTED;
    }
    return GD_OK;
}

Params make_params(const gd_config& c) {
    Params P{};
    P.N = c.N;
    P.M = c.M;
    P.physics = c.physics;
    P.geometry = c.geometry;
    P.order = c.order;
    P.method = c.method;
    for (int s = 0; s < 4; ++s) P.bc[s] = c.bc[s];
    P.dx = c.dx;
    P.dy = c.dy;
    P.x0 = c.x0;
    P.y0 = c.y0;
    P.gamma = c.gamma;
    P.krit = c.krit;
    P.frozen_radius = c.frozen_radius;
    P.frozen = c.frozen_radius > 0.0 ? 1 : 0;
    P.scheme = c.scheme;
    P.x_max = c.x_max;
    P.y_max = c.y_max;
    P.gm1 = c.gamma - 1.0;
    P.inv_dx = 1.0 / c.dx;
    P.inv_dy = 1.0 / c.dy;
    P.inv_gm1 = 1.0 / (c.gamma - 1.0);
    P.hgm1 = 0.5 * (c.gamma - 1.0);
    P.g_gm1 = c.gamma / (c.gamma - 1.0);
    P.ambient_p = 1.0 / c.gamma;
    // rad passed to the flux: dy on x-faces in the Euler kernels (kernel.cu:1811, 3562),
    // dx on x-faces in the MHD kernels (kernel.cu:2560)
    if (c.physics == GD_EULER) {
        P.krad_x = c.krit * c.dy;
        P.krad_y = c.krit * c.dx;
    } else {
        P.krad_x = c.krit * c.dx;
        P.krad_y = c.krit * c.dy;
    }
    return P;
}

cudaError_t launch_step(gd_ctx* ctx, const Params& P, const CPlanes& in, const Planes& out,
                        const double* T_do, unsigned long long* T_bits, Scalars* rot,
                        Scalars* ctr, int dt_only, cudaStream_t st) {
    ctx->launches += ctx->step_launches;
    if (P.scheme != GD_SCHEME_TVD)
        return ctx->cfg.mode == GD_MODE_PARITY
                   ? gd::launch_hancock_parity(P, in, out, T_do, T_bits, rot, ctr, dt_only, st)
                   : gd::launch_hancock_fast(P, in, out, T_do, T_bits, rot, ctr, dt_only, st,
                                             ctx->side);
    if (ctx->cfg.mode == GD_MODE_PARITY)
        return gd::launch_parity(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
    if (P.physics == GD_EULER)
        return gd::launch_euler_fast(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
    return gd::launch_mhd_fast(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
}

}  // namespace

namespace gd {
gd_status cuda_error(cudaError_t e) { return cuda_fail(e); }

cudaError_t dev_alloc_bytes(void** p, size_t bytes) {
    g_allocs.fetch_add(1);
    return cudaMalloc(p, bytes);
}
cudaError_t host_alloc_bytes(void** p, size_t bytes) {
    g_allocs.fetch_add(1);
    return cudaMallocHost(p, bytes);
}
cudaError_t dev_free(void* p) {
    if (p == nullptr) return cudaSuccess;
    g_frees.fetch_add(1);
    return cudaFree(p);
}
cudaError_t host_free(void* p) {
    if (p == nullptr) return cudaSuccess;
    g_frees.fetch_add(1);
    return cudaFreeHost(p);
}
// Configuration checks and launch parameters for entry points that have no context.
gd_status validate_config(const gd_config* c) { return validate(c); }
Params params_from_config(const gd_config& c) { return make_params(c); }
}  // namespace gd

extern "C" {

int gd_abi_version(void) { return GD_ABI_VERSION; }

int gd_last_cuda_error(void) { return g_last_cuda_error.load(); }

gd_status gd_alloc_counts(long long* allocs, long long* frees) {
    if (!allocs || !frees) return GD_ERR_INVALID_ARG;
    *allocs = g_allocs.load();
    *frees = g_frees.load();
    return GD_OK;
}

const char* gd_status_string(gd_status s) {
    switch (s) {
        case GD_OK: return "ok";
        case GD_ERR_INVALID_ARG: return "invalid argument";
        case GD_ERR_CUDA: return "CUDA error";
        case GD_ERR_NONPHYSICAL: return "non-finite state";
        case GD_ERR_TIMEOUT: return "device wait timed out";
        case GD_ERR_UNSUPPORTED: return "unsupported combination";
    }
    return "unknown status";
}

gd_status gd_create(const gd_config* cfg, gd_ctx** out) {
    if (!out) return GD_ERR_INVALID_ARG;
    *out = nullptr;
    gd_status v = validate(cfg);
    if (v != GD_OK) return v;
    gd_ctx* ctx = new (std::nothrow) gd_ctx();
    if (!ctx) return GD_ERR_INVALID_ARG;
    ctx->cfg = *cfg;
    ctx->P = make_params(*cfg);
    ctx->nf = cfg->physics == GD_MHD ? 7 : 4;
    ctx->K = (long long)cfg->N * cfg->M;
    cudaError_t e = cudaGetDevice(&ctx->device);
    const size_t plane_bytes = sizeof(double) * (size_t)ctx->K * ctx->nf;
    if (e == cudaSuccess) e = gd::dev_alloc(&ctx->state[0], plane_bytes);
    if (e == cudaSuccess) e = gd::dev_alloc(&ctx->state[1], plane_bytes);
    if (e == cudaSuccess) e = gd::dev_alloc(&ctx->sc, sizeof(Scalars));
    if (e == cudaSuccess) e = cudaMemset(ctx->sc, 0, sizeof(Scalars));
    if (e == cudaSuccess) {
        Scalars h{};
        h.T_do = 1e-8;  // main(): *host_T_do = 0.00000001 (kernel.cu:3861)
        double reset = gd::kTReset;
        std::memcpy(&h.T_bits, &reset, sizeof(double));
        e = cudaMemcpy(ctx->sc, &h, sizeof(Scalars), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && cfg->mode == GD_MODE_FAST) {
        if (cfg->scheme != GD_SCHEME_TVD) {
            e = gd::prepare_hancock_fast();
            ctx->step_launches = 2;  // edge band and interior tiles
            if (e == cudaSuccess) {
                ctx->side = new (std::nothrow) gd::HancockStreams{nullptr, nullptr, nullptr};
                if (!ctx->side) e = cudaErrorMemoryAllocation;
            }
            if (e == cudaSuccess)
                e = cudaStreamCreateWithFlags(&ctx->side->stream, cudaStreamNonBlocking);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&ctx->side->fork, cudaEventDisableTiming);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&ctx->side->join, cudaEventDisableTiming);
        } else {
            e = cfg->physics == GD_EULER ? gd::prepare_euler_fast() : gd::prepare_mhd_fast();
        }
    }
    if (e == cudaSuccess) e = cudaMemset(ctx->state[0], 0, plane_bytes);
    if (e == cudaSuccess) e = cudaMemset(ctx->state[1], 0, plane_bytes);
    if (e != cudaSuccess) {
        gd_destroy(ctx);
        return cuda_fail(e);
    }
    *out = ctx;
    return GD_OK;
}

gd_status gd_destroy(gd_ctx* ctx) {
    if (!ctx) return GD_ERR_INVALID_ARG;
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    gd::dev_free(ctx->state[0]);
    gd::dev_free(ctx->state[1]);
    gd::dev_free(ctx->sc);
    gd::dev_free(ctx->aos);
    gd::adj_free(ctx);
    gd::io_free(ctx);
    gd::pipe_free(ctx);
    if (ctx->side) {
        if (ctx->side->join) cudaEventDestroy(ctx->side->join);
        if (ctx->side->fork) cudaEventDestroy(ctx->side->fork);
        if (ctx->side->stream) cudaStreamDestroy(ctx->side->stream);
        delete ctx->side;
    }
    delete ctx;
    return GD_OK;
}

gd_status gd_get_config(const gd_ctx* ctx, gd_config* out) {
    if (!ctx || !out) return GD_ERR_INVALID_ARG;
    *out = ctx->cfg;
    return GD_OK;
}

gd_status gd_step_ref(gd_ctx* ctx, const double* s, const double* u, const double* b,
                      double* s2, double* u2, double* b2, double* T, const double* T_do, int i,
                      int method, gd_stream stream) {
    (void)i;
    if (!ctx || !s || !u || !s2 || !u2 || !T || !T_do) return GD_ERR_INVALID_ARG;
    if (ctx->nf == 7 && (!b || !b2)) return GD_ERR_INVALID_ARG;
    Params P = ctx->P;
    if (method != GD_METHOD_CONFIG) {
        if (ctx->cfg.physics == GD_EULER && method != GD_METHOD_HLLC && method != GD_METHOD_HLL)
            return GD_ERR_INVALID_ARG;
        if (ctx->cfg.physics == GD_MHD && method != GD_METHOD_HLLC_MHD && method != GD_METHOD_HLLD)
            return GD_ERR_INVALID_ARG;
        if (ctx->cfg.scheme != GD_SCHEME_TVD && method != GD_METHOD_HLLD)
            return GD_ERR_UNSUPPORTED;
        P.method = method;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the step reads and writes the reference layout itself: one launch, no staging
    CPlanes in{};
    in.s = s;
    in.u = u;
    in.b = ctx->nf == 7 ? b : nullptr;
    Planes out{};
    out.s = s2;
    out.u = u2;
    out.b = ctx->nf == 7 ? b2 : nullptr;
    GD_CUDA(launch_step(ctx, P, in, out, T_do, (unsigned long long*)T, nullptr, ctx->sc, 0, st));
    return GD_OK;
}

gd_status gd_funk_time(gd_ctx* ctx, double* T, double* T_do, double* TT, int* i,
                       gd_stream stream) {
    if (!ctx || !T || !T_do || !TT || !i) return GD_ERR_INVALID_ARG;
    GD_CUDA(gd::launch_funk_time(T, T_do, TT, i, (cudaStream_t)stream));
    ctx->launches += 1;
    return GD_OK;
}

gd_status gd_import(gd_ctx* ctx, const double* s, const double* u, const double* b, int is_host,
                    gd_stream stream) {
    if (!ctx || !s || !u || (ctx->nf == 7 && !b)) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const double *ds = s, *du = u, *db = b;
    if (is_host) {
        if (!ctx->aos) GD_CUDA(gd::dev_alloc(&ctx->aos, sizeof(double) * 7 * (size_t)ctx->K));
        double* hs = ctx->aos;
        double* hu = hs + 2 * ctx->K;
        double* hb = hu + 2 * ctx->K;
        GD_CUDA(cudaMemcpyAsync(hs, s, sizeof(double) * 2 * ctx->K, cudaMemcpyHostToDevice, st));
        GD_CUDA(cudaMemcpyAsync(hu, u, sizeof(double) * 2 * ctx->K, cudaMemcpyHostToDevice, st));
        if (ctx->nf == 7)
            GD_CUDA(cudaMemcpyAsync(hb, b, sizeof(double) * 3 * ctx->K, cudaMemcpyHostToDevice, st));
        ds = hs;
        du = hu;
        db = hb;
    }
    GD_CUDA(gd::launch_aos_to_soa(ds, du, db, ctx->planes(ctx->cur), ctx->K, ctx->nf, st));
    ctx->launches += 1;
    return GD_OK;
}

gd_status gd_export(gd_ctx* ctx, double* s, double* u, double* b, int is_host, gd_stream stream) {
    if (!ctx || !s || !u || (ctx->nf == 7 && !b)) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    double *ds = s, *du = u, *db = b;
    if (is_host) {
        if (!ctx->aos) GD_CUDA(gd::dev_alloc(&ctx->aos, sizeof(double) * 7 * (size_t)ctx->K));
        ds = ctx->aos;
        du = ds + 2 * ctx->K;
        db = du + 2 * ctx->K;
    }
    GD_CUDA(gd::launch_soa_to_aos(gd_ctx::cplanes(ctx->planes(ctx->cur)), ds, du, db, ctx->K,
                                  ctx->nf, st));
    ctx->launches += 1;
    if (is_host) {
        GD_CUDA(cudaMemcpyAsync(s, ds, sizeof(double) * 2 * ctx->K, cudaMemcpyDeviceToHost, st));
        GD_CUDA(cudaMemcpyAsync(u, du, sizeof(double) * 2 * ctx->K, cudaMemcpyDeviceToHost, st));
        if (ctx->nf == 7)
            GD_CUDA(cudaMemcpyAsync(b, db, sizeof(double) * 3 * ctx->K, cudaMemcpyDeviceToHost, st));
        GD_CUDA(cudaStreamSynchronize(st));
    }
    return GD_OK;
}

gd_status gd_set_time(gd_ctx* ctx, double T_do, double TT, gd_stream stream) {
    if (!ctx || !(std::isfinite(T_do) && T_do >= 0.0) || !std::isfinite(TT))
        return GD_ERR_INVALID_ARG;
    GD_CUDA(gd::launch_set_time(ctx->sc, T_do, TT, (cudaStream_t)stream));
    ctx->launches += 1;
    return GD_OK;
}

gd_status gd_init_dt(gd_ctx* ctx, gd_stream stream) {
    if (!ctx) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    GD_CUDA(gd::launch_reset_T(ctx->sc, st));
    ctx->launches += 1;
    const Planes cur = ctx->planes(ctx->cur);
    GD_CUDA(launch_step(ctx, ctx->P, gd_ctx::cplanes(cur), ctx->planes(1 - ctx->cur),
                        &ctx->sc->T_do, &ctx->sc->T_bits, nullptr, nullptr, 1, st));
    GD_CUDA(gd::launch_dt_commit(ctx->sc, st));
    ctx->launches += 1;
    return GD_OK;
}

static gd_status advance_plain(gd_ctx* ctx, int nsteps, cudaStream_t st) {
    for (int s = 0; s < nsteps; ++s) {
        const Planes in = ctx->planes(ctx->cur), out = ctx->planes(1 - ctx->cur);
        if (ctx->dt_policy == GD_DT_CURRENT) {
            // the CFL dt of this step's own input state (T was reset by the last rotation)
            GD_CUDA(launch_step(ctx, ctx->P, gd_ctx::cplanes(in), out, &ctx->sc->T_do,
                                &ctx->sc->T_bits, nullptr, nullptr, 1, st));
            GD_CUDA(gd::launch_dt_commit(ctx->sc, st));
            ctx->launches += 1;
        }
        GD_CUDA(launch_step(ctx, ctx->P, gd_ctx::cplanes(in), out, &ctx->sc->T_do,
                            &ctx->sc->T_bits, ctx->sc, ctx->sc, 0, st));
        ctx->cur ^= 1;
    }
    return GD_OK;
}

static long long launches_per_step(const gd_ctx* ctx) {
    return ctx->dt_policy == GD_DT_CURRENT ? 2LL * ctx->step_launches + 1 : ctx->step_launches;
}

gd_status gd_advance(gd_ctx* ctx, int nsteps, int use_graph, gd_stream stream) {
    if (!ctx || nsteps < 0) return GD_ERR_INVALID_ARG;
    if (nsteps == 0) return GD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (!use_graph) return advance_plain(ctx, nsteps, st);
    const auto key = std::make_pair(nsteps, ctx->cur);
    auto it = ctx->graphs.find(key);
    if (it == ctx->graphs.end()) {
        cudaStream_t cap = st;
        bool own = false;
        if (cap == nullptr) {  // the legacy default stream cannot be captured
            GD_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            own = true;
        }
        const int cur0 = ctx->cur;
        const long long l0 = ctx->launches;
        cudaGraph_t g = nullptr;
        GD_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        gd_status s = advance_plain(ctx, nsteps, cap);
        cudaError_t ce = cudaStreamEndCapture(cap, &g);
        ctx->cur = cur0;  // capture did not execute anything
        ctx->launches = l0;
        if (own) cudaStreamDestroy(cap);
        if (s != GD_OK) {
            if (g) cudaGraphDestroy(g);
            return s;
        }
        if (ce != cudaSuccess) return cuda_fail(ce);
        cudaGraphExec_t ge = nullptr;
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ce);
        it = ctx->graphs.emplace(key, ge).first;
    }
    GD_CUDA(cudaGraphLaunch(it->second, st));
    ctx->launches += (long long)nsteps * launches_per_step(ctx);
    if (nsteps & 1) ctx->cur ^= 1;
    return GD_OK;
}

gd_status gd_set_dt_policy(gd_ctx* ctx, int policy) {
    if (!ctx || (policy != GD_DT_LAGGED && policy != GD_DT_CURRENT)) return GD_ERR_INVALID_ARG;
    if (policy != ctx->dt_policy) {
        for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
        ctx->graphs.clear();
        ctx->dt_policy = policy;
    }
    return GD_OK;
}

gd_status gd_advance_to(gd_ctx* ctx, double t_end, long long max_steps, int use_graph,
                        long long* steps_taken, gd_stream stream) {
    if (steps_taken) *steps_taken = 0;
    if (!ctx || !(std::isfinite(t_end) && t_end > 0.0) || max_steps < 0)
        return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    struct TimeView {
        double T_do, t_state;
    };
    auto read_time = [&](TimeView* tv) -> gd_status {
        Scalars h{};
        GD_CUDA(cudaMemcpyAsync(&h, ctx->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        GD_CUDA(cudaStreamSynchronize(st));
        tv->T_do = h.T_do;
        tv->t_state = h.t_state;
        return GD_OK;
    };
    TimeView tv{};
    gd_status s = read_time(&tv);
    if (s != GD_OK) return s;
    if (!(t_end > tv.t_state)) return GD_ERR_INVALID_ARG;
    GD_CUDA(gd::launch_set_end(ctx->sc, t_end, st));
    ctx->launches += 1;
    long long taken = 0;
    // close enough: the last, limited step lands on t_end up to the rounding of the sum
    const double tol = 1e-14 * t_end;
    while (taken < max_steps) {
        s = read_time(&tv);
        if (s != GD_OK) break;
        const double left = t_end - tv.t_state;
        if (left <= tol || !(tv.T_do > 0.0)) break;
        // about half of the steps the current dt needs: the dt may grow, and a step after
        // t_end is reached would be a zero-dt step
        const double need = left / tv.T_do;
        long long chunk = need > 4.0 ? (long long)(0.5 * need) : 1;
        if (chunk > max_steps - taken) chunk = max_steps - taken;
        if (chunk > (1 << 20)) chunk = 1 << 20;
        s = gd_advance(ctx, (int)chunk, use_graph, stream);
        if (s != GD_OK) break;
        taken += chunk;
    }
    const cudaError_t e = gd::launch_set_end(ctx->sc, 0.0, st);
    ctx->launches += 1;
    if (steps_taken) *steps_taken = taken;
    if (s != GD_OK) return s;
    if (e != cudaSuccess) return cuda_fail(e);
    return GD_OK;
}

gd_status gd_get_stats(gd_ctx* ctx, gd_stats* out, gd_stream stream) {
    if (!ctx || !out) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    Scalars h{};
    GD_CUDA(cudaMemcpyAsync(&h, ctx->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    GD_CUDA(cudaStreamSynchronize(st));
    double T;
    std::memcpy(&T, &h.T_bits, sizeof(double));
    out->t = h.TT;
    out->dt = h.T_do;
    out->dt_next = T;
    out->steps = h.step;
    out->rho_floor_hits = (long long)h.rho_floor;
    out->p_floor_hits = (long long)h.p_floor;
    out->nonfinite = (long long)h.nonfinite;
    out->t_state = h.t_state;
    const bool floors = ctx->floor_limit > 0 &&
                        out->rho_floor_hits + out->p_floor_hits > ctx->floor_limit;
    return (h.nonfinite || floors) ? GD_ERR_NONPHYSICAL : GD_OK;
}

gd_status gd_set_floor_limit(gd_ctx* ctx, long long max_floor_hits) {
    if (!ctx || max_floor_hits < 0) return GD_ERR_INVALID_ARG;
    ctx->floor_limit = max_floor_hits;
    return GD_OK;
}

gd_status gd_field_ptr(gd_ctx* ctx, int f, const double** out) {
    if (!ctx || !out || f < 0 || f >= ctx->nf) return GD_ERR_INVALID_ARG;
    *out = ctx->state[ctx->cur] + (size_t)f * ctx->K;
    return GD_OK;
}

long long gd_launch_count(const gd_ctx* ctx) { return ctx ? ctx->launches : 0; }

gd_status gd_probe_fp64_peak(double* flops_out) {
    if (!flops_out) return GD_ERR_INVALID_ARG;
    GD_CUDA(gd::probe_fp64_peak(flops_out));
    return GD_OK;
}

gd_status gd_check_int_mul(long long pairs, unsigned long long seed, long long* counts_out) {
    if (!counts_out || pairs <= 0 || pairs > (1LL << 34)) return GD_ERR_INVALID_ARG;
    GD_CUDA(gd::check_imul(pairs, seed, counts_out));
    return GD_OK;
}

gd_status gd_check_fast_roots(long long count, unsigned long long seed, long long* out) {
    if (!out || count <= 0 || count > (1LL << 34)) return GD_ERR_INVALID_ARG;
    GD_CUDA(gd::check_roots(count, seed, out));
    return GD_OK;
}

gd_status gd_probe_faces(int physics, int method, double gamma, int axis, long long n,
                         const double* L, const double* R, double* flux, double* speed,
                         gd_stream stream) {
    if (physics != GD_EULER && physics != GD_MHD) return GD_ERR_INVALID_ARG;
    if (physics == GD_EULER && method != GD_METHOD_HLL && method != GD_METHOD_HLLC)
        return GD_ERR_INVALID_ARG;
    if (physics == GD_MHD && method != GD_METHOD_HLLC_MHD && method != GD_METHOD_HLLD)
        return GD_ERR_INVALID_ARG;
    if (!(std::isfinite(gamma) && gamma > 1.0)) return GD_ERR_INVALID_ARG;
    if ((axis != 0 && axis != 1) || n < 0 || n > (1LL << 36)) return GD_ERR_INVALID_ARG;
    if (n > 0 && (!L || !R || !flux || !speed)) return GD_ERR_INVALID_ARG;
    Params P{};
    P.physics = physics;
    P.method = method;
    P.gamma = gamma;
    P.gm1 = gamma - 1.0;
    P.inv_gm1 = 1.0 / (gamma - 1.0);
    P.hgm1 = 0.5 * (gamma - 1.0);
    P.g_gm1 = gamma / (gamma - 1.0);
    const cudaStream_t st = (cudaStream_t)stream;
    GD_CUDA(physics == GD_EULER ? gd::launch_euler_face_probe(P, n, axis, L, R, flux, speed, st)
                                : gd::launch_mhd_face_probe(P, n, axis, L, R, flux, speed, st));
    return GD_OK;
}

}  // extern "C"
