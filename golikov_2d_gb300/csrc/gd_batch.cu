// gd_batch.cu -- many independent grids of uneven sizes (C ABI, include/gd2d.h).
//
// All grids' states live in one pool per ping-pong buffer (SoA planes of each grid back to
// back).  The persistent schedule advances every grid by one step in a single launch of
// euler_batch_kernel, whose CTAs stride over the flattened (grid, tile) list; each grid keeps
// its own dt minimum, dt rotation and time (last-tile ticket per grid), so grids never wait
// for one another inside a step.  A captured CUDA graph replays n such launches.  The looped
// schedule (one plain launch per grid per step) is the baseline it replaces.
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include "../../include/gd2d.h"
#include "gd_internal.cuh"
#include "gd_kernels.h"

using gd::BatchGrid;
using gd::CPlanes;
using gd::Params;
using gd::Planes;
using gd::Scalars;

namespace {
gd_status cuda_status(cudaError_t e) { return e == cudaSuccess ? GD_OK : gd::cuda_error(e); }
}  // namespace

#define GD_TRY(call)                                        \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_status(e_);      \
    } while (0)

struct gd_batch {
    int ngrids = 0;
    int order = 2;
    int nf = 4;
    std::vector<gd_config> cfgs;
    std::vector<Params> params;
    std::vector<long long> K;
    std::vector<size_t> offset;  // start of each grid's planes in a pool, in doubles
    size_t pool_doubles = 0;
    long long total_cells = 0;
    long long max_K = 0;
    double* pool[2] = {nullptr, nullptr};
    Scalars* sc = nullptr;          // ngrids
    Scalars* sc_tune = nullptr;     // ngrids, used by the autotuner
    double* aos = nullptr;          // staging for host import / export (7 * max_K)
    BatchGrid* d_grids[gd::kEulerVariants] = {};
    int2* d_items[gd::kEulerVariants] = {};
    int nitems[gd::kEulerVariants] = {};
    int ctas[gd::kEulerVariants] = {};
    double tuned_ms[gd::kEulerVariants] = {};
    int variant = 0;
    int cur = 0;
    long long launches = 0;
    std::map<std::tuple<int, int, int, int>, cudaGraphExec_t> graphs;

    Planes planes(int g, int which) const {
        Planes p{};
        for (int f = 0; f < nf; ++f) p.f[f] = pool[which] + offset[g] + (size_t)f * K[g];
        return p;
    }
};

namespace {

CPlanes as_const(const Planes& p) {
    CPlanes c{};
    for (int f = 0; f < gd::kMaxFields; ++f) c.f[f] = p.f[f];
    return c;
}

gd_status step_persistent(gd_batch* b, int variant, int dt_only, Scalars* sc_override,
                          cudaStream_t st) {
    GD_TRY(gd::launch_euler_batch(variant, b->order, b->d_grids[variant], b->d_items[variant],
                                  b->nitems[variant], b->cur, dt_only, sc_override,
                                  b->ctas[variant], st));
    b->launches += 1;
    return GD_OK;
}

// One plain launch per grid; with `sync` the host waits for each launch before the next, as
// the reference's main loop does after each of its launches (kernel.cu:4113-4137).
gd_status step_looped(gd_batch* b, bool sync, cudaStream_t st) {
    for (int g = 0; g < b->ngrids; ++g) {
        Scalars* sc = b->sc + g;
        GD_TRY(gd::launch_euler_fast_v(b->variant, b->params[g], as_const(b->planes(g, b->cur)),
                                       b->planes(g, b->cur ^ 1), &sc->T_do, &sc->T_bits, sc, sc,
                                       0, st));
        b->launches += 1;
        if (sync) GD_TRY(cudaStreamSynchronize(st));
    }
    return GD_OK;
}

gd_status advance_plain(gd_batch* b, int nsteps, int schedule, cudaStream_t st) {
    for (int s = 0; s < nsteps; ++s) {
        gd_status r = schedule == GD_BATCH_PERSISTENT
                          ? step_persistent(b, b->variant, 0, nullptr, st)
                          : step_looped(b, schedule == GD_BATCH_LOOPED_SYNC, st);
        if (r != GD_OK) return r;
        b->cur ^= 1;
    }
    return GD_OK;
}

}  // namespace

extern "C" {

gd_status gd_batch_create(const gd_config* cfgs, int ngrids, gd_batch** out) {
    if (!out || !cfgs || ngrids <= 0) return GD_ERR_INVALID_ARG;
    *out = nullptr;
    for (int g = 0; g < ngrids; ++g) {
        const gd_status v = gd::validate_config(&cfgs[g]);
        if (v != GD_OK) return v;
        if (cfgs[g].physics != GD_EULER || cfgs[g].mode != GD_MODE_FAST) return GD_ERR_UNSUPPORTED;
        if (cfgs[g].order != cfgs[0].order) return GD_ERR_INVALID_ARG;
    }
    gd_batch* b = new (std::nothrow) gd_batch();
    if (!b) return GD_ERR_INVALID_ARG;
    b->ngrids = ngrids;
    b->order = cfgs[0].order;
    b->cfgs.assign(cfgs, cfgs + ngrids);
    size_t off = 0;
    for (int g = 0; g < ngrids; ++g) {
        b->params.push_back(gd::params_from_config(cfgs[g]));
        const long long K = (long long)cfgs[g].N * cfgs[g].M;
        b->K.push_back(K);
        b->offset.push_back(off);
        off += (size_t)b->nf * K;
        b->total_cells += K;
        b->max_K = K > b->max_K ? K : b->max_K;
    }
    b->pool_doubles = off;
    cudaError_t e = gd::prepare_euler_fast();
    if (e == cudaSuccess) e = gd::dev_alloc(&b->pool[0], sizeof(double) * off);
    if (e == cudaSuccess) e = gd::dev_alloc(&b->pool[1], sizeof(double) * off);
    if (e == cudaSuccess) e = cudaMemset(b->pool[0], 0, sizeof(double) * off);
    if (e == cudaSuccess) e = cudaMemset(b->pool[1], 0, sizeof(double) * off);
    if (e == cudaSuccess) e = gd::dev_alloc(&b->sc, sizeof(Scalars) * ngrids);
    if (e == cudaSuccess) e = gd::dev_alloc(&b->sc_tune, sizeof(Scalars) * ngrids);
    if (e == cudaSuccess) {
        std::vector<Scalars> h(ngrids);
        const double reset = gd::kTReset;
        for (auto& s : h) {
            std::memset(&s, 0, sizeof(Scalars));
            s.T_do = 1e-8;
            std::memcpy(&s.T_bits, &reset, sizeof(double));
        }
        e = cudaMemcpy(b->sc, h.data(), sizeof(Scalars) * ngrids, cudaMemcpyHostToDevice);
    }
    int dev = 0, sms = 1;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int v = 0; v < gd::kEulerVariants && e == cudaSuccess; ++v) {
        int tx, ty;
        gd::euler_tile_shape(v, &tx, &ty);
        std::vector<BatchGrid> hg(ngrids);
        std::vector<int2> items;
        for (int g = 0; g < ngrids; ++g) {
            BatchGrid& d = hg[g];
            std::memset(&d, 0, sizeof(BatchGrid));
            d.P = b->params[g];
            d.state[0] = b->pool[0] + b->offset[g];
            d.state[1] = b->pool[1] + b->offset[g];
            d.K = b->K[g];
            d.sc = b->sc + g;
            d.tiles_x = (cfgs[g].N + tx - 1) / tx;
            d.ntiles = d.tiles_x * ((cfgs[g].M + ty - 1) / ty);
            for (int t = 0; t < d.ntiles; ++t) items.push_back(make_int2(g, t));
        }
        b->nitems[v] = (int)items.size();
        const int per_sm = gd::euler_batch_blocks_per_sm(b->order, v);
        const int full = per_sm * sms;
        b->ctas[v] = b->nitems[v] < full ? b->nitems[v] : full;
        e = gd::dev_alloc(&b->d_grids[v], sizeof(BatchGrid) * ngrids);
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_grids[v], hg.data(), sizeof(BatchGrid) * ngrids,
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = gd::dev_alloc(&b->d_items[v], sizeof(int2) * items.size());
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_items[v], items.data(), sizeof(int2) * items.size(),
                           cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        gd_batch_destroy(b);
        return gd::cuda_error(e);
    }
    *out = b;
    return GD_OK;
}

gd_status gd_batch_destroy(gd_batch* b) {
    if (!b) return GD_ERR_INVALID_ARG;
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    for (int v = 0; v < gd::kEulerVariants; ++v) {
        gd::dev_free(b->d_grids[v]);
        gd::dev_free(b->d_items[v]);
    }
    gd::dev_free(b->pool[0]);
    gd::dev_free(b->pool[1]);
    gd::dev_free(b->sc);
    gd::dev_free(b->sc_tune);
    gd::dev_free(b->aos);
    delete b;
    return GD_OK;
}

gd_status gd_batch_import(gd_batch* b, int grid, const double* s, const double* u,
                          const double* bfield, int is_host, gd_stream stream) {
    (void)bfield;
    if (!b || grid < 0 || grid >= b->ngrids || !s || !u) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const long long K = b->K[grid];
    const double *ds = s, *du = u;
    if (is_host) {
        if (!b->aos) GD_TRY(gd::dev_alloc(&b->aos, sizeof(double) * 7 * (size_t)b->max_K));
        GD_TRY(cudaMemcpyAsync(b->aos, s, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, st));
        GD_TRY(cudaMemcpyAsync(b->aos + 2 * K, u, sizeof(double) * 2 * K, cudaMemcpyHostToDevice,
                               st));
        ds = b->aos;
        du = b->aos + 2 * K;
    }
    GD_TRY(gd::launch_aos_to_soa(ds, du, nullptr, b->planes(grid, b->cur), K, b->nf, st));
    b->launches += 1;
    return GD_OK;
}

gd_status gd_batch_export(gd_batch* b, int grid, double* s, double* u, double* bfield,
                          int is_host, gd_stream stream) {
    (void)bfield;
    if (!b || grid < 0 || grid >= b->ngrids || !s || !u) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const long long K = b->K[grid];
    double *ds = s, *du = u;
    if (is_host) {
        if (!b->aos) GD_TRY(gd::dev_alloc(&b->aos, sizeof(double) * 7 * (size_t)b->max_K));
        ds = b->aos;
        du = b->aos + 2 * K;
    }
    GD_TRY(gd::launch_soa_to_aos(as_const(b->planes(grid, b->cur)), ds, du, nullptr, K, b->nf,
                                 st));
    b->launches += 1;
    if (is_host) {
        GD_TRY(cudaMemcpyAsync(s, ds, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost, st));
        GD_TRY(cudaMemcpyAsync(u, du, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost, st));
        GD_TRY(cudaStreamSynchronize(st));
    }
    return GD_OK;
}

gd_status gd_batch_set_time(gd_batch* b, double T_do, double TT, gd_stream stream) {
    if (!b || !(std::isfinite(T_do) && T_do >= 0.0) || !std::isfinite(TT)) return GD_ERR_INVALID_ARG;
    GD_TRY(gd::launch_batch_set_time(b->d_grids[0], b->ngrids, T_do, TT, (cudaStream_t)stream));
    b->launches += 1;
    return GD_OK;
}

gd_status gd_batch_init_dt(gd_batch* b, gd_stream stream) {
    if (!b) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    GD_TRY(gd::launch_batch_reset_T(b->d_grids[0], b->ngrids, st));
    const gd_status r = step_persistent(b, b->variant, 1, nullptr, st);
    if (r != GD_OK) return r;
    GD_TRY(gd::launch_batch_dt_commit(b->d_grids[0], b->ngrids, st));
    b->launches += 2;
    return GD_OK;
}

gd_status gd_batch_advance(gd_batch* b, int nsteps, int schedule, int use_graph,
                           gd_stream stream) {
    if (!b || nsteps < 0 ||
        (schedule != GD_BATCH_PERSISTENT && schedule != GD_BATCH_LOOPED &&
         schedule != GD_BATCH_LOOPED_SYNC))
        return GD_ERR_INVALID_ARG;
    if (schedule == GD_BATCH_LOOPED_SYNC && use_graph) return GD_ERR_INVALID_ARG;
    if (nsteps == 0) return GD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (!use_graph) return advance_plain(b, nsteps, schedule, st);
    const auto key = std::make_tuple(nsteps, b->cur, schedule, b->variant);
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
        cudaStream_t cap = st;
        bool own = false;
        if (cap == nullptr) {
            GD_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            own = true;
        }
        const int cur0 = b->cur;
        const long long l0 = b->launches;
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        gd_status s = ce == cudaSuccess ? advance_plain(b, nsteps, schedule, cap)
                                        : gd::cuda_error(ce);
        if (ce == cudaSuccess) ce = cudaStreamEndCapture(cap, &g);
        b->cur = cur0;
        b->launches = l0;
        if (own) cudaStreamDestroy(cap);
        if (s != GD_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return s != GD_OK ? s : gd::cuda_error(ce);
        }
        cudaGraphExec_t ge = nullptr;
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return gd::cuda_error(ce);
        it = b->graphs.emplace(key, ge).first;
    }
    GD_TRY(cudaGraphLaunch(it->second, st));
    b->launches += (long long)nsteps * (schedule == GD_BATCH_PERSISTENT ? 1 : b->ngrids);
    if (nsteps & 1) b->cur ^= 1;
    return GD_OK;
}

gd_status gd_batch_autotune(gd_batch* b, int reps, gd_stream stream) {
    if (!b || reps <= 0) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    GD_TRY(cudaEventCreate(&e0));
    GD_TRY(cudaEventCreate(&e1));
    int best = b->variant;
    float best_ms = 0.f;
    for (int v = 0; v < gd::kEulerVariants; ++v) {
        // Time `reps` steps writing only the spare buffer and scratch scalars: the state,
        // dt and time of the batch are unchanged.
        GD_TRY(cudaMemcpyAsync(b->sc_tune, b->sc, sizeof(Scalars) * b->ngrids,
                               cudaMemcpyDeviceToDevice, st));
        gd_status r = step_persistent(b, v, 0, b->sc_tune, st);  // warm-up
        if (r != GD_OK) return r;
        GD_TRY(cudaEventRecord(e0, st));
        for (int k = 0; k < reps; ++k) {
            r = step_persistent(b, v, 0, b->sc_tune, st);
            if (r != GD_OK) return r;
        }
        GD_TRY(cudaEventRecord(e1, st));
        GD_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        GD_TRY(cudaEventElapsedTime(&ms, e0, e1));
        ms /= reps;
        b->tuned_ms[v] = ms;
        if (v == 0 || ms < best_ms) {
            best_ms = ms;
            best = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->variant = best;
    return GD_OK;
}

gd_status gd_batch_get_stats(gd_batch* b, int grid, gd_stats* out, gd_stream stream) {
    if (!b || !out || grid < 0 || grid >= b->ngrids) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    Scalars h{};
    GD_TRY(cudaMemcpyAsync(&h, b->sc + grid, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    GD_TRY(cudaStreamSynchronize(st));
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
    return h.nonfinite ? GD_ERR_NONPHYSICAL : GD_OK;
}

gd_status gd_batch_get_info(const gd_batch* b, gd_batch_info* out) {
    if (!b || !out) return GD_ERR_INVALID_ARG;
    out->ngrids = b->ngrids;
    out->total_cells = b->total_cells;
    gd::euler_tile_shape(b->variant, &out->tile_x, &out->tile_y);
    out->ctas = b->ctas[b->variant];
    out->tiles = b->nitems[b->variant];
    for (int v = 0; v < 4; ++v) out->tuned_ms[v] = v < gd::kEulerVariants ? b->tuned_ms[v] : 0.0;
    return GD_OK;
}

long long gd_batch_launch_count(const gd_batch* b) { return b ? b->launches : 0; }

}  // extern "C"
