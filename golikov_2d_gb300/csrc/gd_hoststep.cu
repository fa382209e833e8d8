// gd_hoststep.cu -- gd_step_host: one step of the resident loop whose state comes from host
// memory and whose result goes back to host memory, with the transfers overlapped with the
// step.
//
// The reference moves its state between host and device with blocking cudaMemcpy calls
// around its loop (kernel.cu:4005-4010, 4093-4095, 4163-4165).  gd_import + gd_advance(1) +
// gd_export does the same in three sequential phases.  Here the grid is cut into bands of
// whole tile rows.  Band k's rows go up, in the reference's AoS layout, to a device staging
// buffer on one copy stream; on the caller's stream band k is stepped as soon as its
// neighbours' rows (the stencil's halo) are there, the step reading the staging buffer
// itself and writing its output both to the context's planes (the resident state) and to
// an AoS staging buffer, from which it goes down on a second copy stream while later bands
// are stepped: no conversion pass.  The two copy directions and the SMs work at once, so a step costs
// about the step itself plus one band of each copy.  The whole banded step is captured into
// a CUDA graph per (host buffers, plane set) and replayed, so its few hundred copies and
// launches reach the GPU in one submission.  The step is the same kernel with the
// same arithmetic, launched once per band (Params::tile_row0 / tile_rows); the bands' blocks
// share one dt rotation ticket, so dt, time and counters are those of gd_advance(1).
#include <cstring>
#include <new>

#include "../../include/gd2d.h"
#include "gd_ctx.h"
#include "gd_internal.cuh"
#include "gd_kernels.h"

using gd::CPlanes;
using gd::Params;
using gd::Planes;

namespace {

#define HS_TRY(call)                                   \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return e_;              \
    } while (0)

bool device_visible_host(const void* p) {
    if (p == nullptr) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory: clear the error, not visible
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

cudaError_t pipe_create(gd_ctx* ctx) {
    gd::HostPipe* p = new (std::nothrow) gd::HostPipe();
    if (!p) return cudaErrorMemoryAllocation;
    ctx->pipe = p;
    // The copy streams' conversion kernels and the Hancock edge launch are short and gate
    // the next band's step or the downloads: at the highest priority their blocks are
    // dispatched ahead of the queued blocks of the band steps (at equal priority the edge
    // launch waited behind all of them and every download with it).
    int prio_low = 0, prio_high = 0;
    HS_TRY(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    HS_TRY(cudaStreamCreateWithPriority(&p->up, cudaStreamNonBlocking, prio_high));
    HS_TRY(cudaStreamCreateWithPriority(&p->down, cudaStreamNonBlocking, prio_high));
    HS_TRY(cudaStreamCreateWithPriority(&p->edge, cudaStreamNonBlocking, prio_high));
    for (cudaStream_t& c : p->comp) HS_TRY(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
    HS_TRY(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&p->start, &p->down_done, &p->comp_done, &p->edge_done, &p->up_done})
        HS_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (int k = 0; k < gd::kMaxBands; ++k) {
        HS_TRY(cudaEventCreateWithFlags(&p->ev_up[k], cudaEventDisableTiming));
        HS_TRY(cudaEventCreateWithFlags(&p->ev_out[k], cudaEventDisableTiming));
    }
    HS_TRY(gd::dev_alloc(&p->aos_in, sizeof(double) * 7 * (size_t)ctx->K));
    HS_TRY(gd::dev_alloc(&p->aos_out, sizeof(double) * 7 * (size_t)ctx->K));
    return cudaSuccess;
}

// all or nothing: a partly created pipeline is released, so a later call starts afresh
cudaError_t pipe_init(gd_ctx* ctx) {
    if (ctx->pipe) return cudaSuccess;
    const cudaError_t e = pipe_create(ctx);
    if (e != cudaSuccess) gd::pipe_free(ctx);
    return e;
}

// AoS views of rows [r0, r1): s (2 per cell), u (2), b (3), at base + {0, 2K, 4K}
struct Rows {
    long long c0, n;  // first cell, cells
};

cudaError_t copy_rows(double* dst_s, double* dst_u, double* dst_b, const double* src_s,
                      const double* src_u, const double* src_b, Rows r, int nf, cudaMemcpyKind k,
                      cudaStream_t st) {
    HS_TRY(cudaMemcpyAsync(dst_s + 2 * r.c0, src_s + 2 * r.c0, sizeof(double) * 2 * r.n, k, st));
    HS_TRY(cudaMemcpyAsync(dst_u + 2 * r.c0, src_u + 2 * r.c0, sizeof(double) * 2 * r.n, k, st));
    if (nf == 7)
        HS_TRY(cudaMemcpyAsync(dst_b + 3 * r.c0, src_b + 3 * r.c0, sizeof(double) * 3 * r.n, k,
                               st));
    return cudaSuccess;
}


// The banded step.  Returns a CUDA error or cudaSuccess; the caller synchronises.
cudaError_t banded_step(gd_ctx* ctx, const double* s, const double* u, const double* b,
                        double* s2, double* u2, double* b2, int TX, int TY, cudaStream_t st) {
    gd::HostPipe* p = ctx->pipe;
    const int N = ctx->cfg.N, M = ctx->cfg.M, nf = ctx->nf;
    const long long K = ctx->K;
    // The fast Hancock step's interior tiles start at row 2 and its edge cells (two rows or
    // columns from every edge) are a launch of their own; a band there is the rows between
    // two interior tile-row boundaries, edge cells included.
    const bool hk = ctx->cfg.mode == GD_MODE_FAST && ctx->cfg.scheme != GD_SCHEME_TVD;
    const int T = hk ? (M - 4 + TY - 1) / TY : (M + TY - 1) / TY;  // tile (block) rows
    const int nx = hk ? (N - 4 + TX - 1) / TX : (N + TX - 1) / TX;  // tiles per tile row
    // Smaller bands shorten the pipeline's fill (two bands up before the first step) and
    // drain (one band down after the last).  The bands are stepped on kCompStreams streams
    // in turn, so a band of half a wave of the kernels' resident blocks (two per SM) keeps
    // about one and a half waves in flight; 2 to kMaxBands bands of >= 2 block rows.
    int sms = 0;
    HS_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const long long per_band_min = sms > 0 ? sms : 1;
    int B = (int)(((long long)nx * T) / per_band_min);
    if (B > gd::kMaxBands) B = gd::kMaxBands;
    if (B > T / 2) B = T / 2;
    if (B < 2) B = 2;
    // halo rows of the stencil: two for minmod TVD and for the Hancock step (whatever its
    // `order`), one at first order
    const int H = (ctx->cfg.order == 2 || ctx->cfg.scheme != GD_SCHEME_TVD) ? 2 : 1;
    const bool wrap = ctx->cfg.bc[2] == GD_BC_PERIODIC;
    auto band_tiles = [&](int k, int* t0, int* t1) {
        *t0 = (int)((long long)k * T / B);
        *t1 = (int)((long long)(k + 1) * T / B);
    };
    // first row of band k (band B: M)
    auto row_bound = [&](int k) -> int {
        if (k <= 0) return 0;
        if (k >= B) return M;
        const int t = (int)((long long)k * T / B);
        return hk ? 2 + t * TY : t * TY;
    };
    auto band_rows = [&](int k) {
        const int r0 = row_bound(k), r1 = row_bound(k + 1);
        return Rows{(long long)r0 * N, (long long)(r1 - r0) * N};
    };
    // the last band's upload leaves out the seam rows a periodic y-edge has sent first
    auto band_rows_up = [&](int k) {
        Rows r = band_rows(k);
        if (wrap && k == B - 1) r.n -= (long long)H * N;
        return r;
    };
    double* ai = p->aos_in;
    double* ao = p->aos_out;
    HS_TRY(cudaEventRecord(p->start, st));
    HS_TRY(cudaStreamWaitEvent(p->up, p->start, 0));
    HS_TRY(cudaStreamWaitEvent(p->down, p->start, 0));
    // up stream: host rows to the AoS staging; the seam rows first, then the bands in order
    const Rows wrap_rows{(long long)(M - H) * N, (long long)H * N};
    if (wrap)
        HS_TRY(copy_rows(ai, ai + 2 * K, ai + 4 * K, s, u, b, wrap_rows, nf,
                         cudaMemcpyHostToDevice, p->up));
    int n_up = 0;  // bands whose upload is enqueued
    auto enqueue_up = [&](int upto) -> cudaError_t {
        for (; n_up <= upto && n_up < B; ++n_up) {
            const Rows r = band_rows_up(n_up);
            HS_TRY(copy_rows(ai, ai + 2 * K, ai + 4 * K, s, u, b, r, nf,
                             cudaMemcpyHostToDevice, p->up));
            HS_TRY(cudaEventRecord(p->ev_up[n_up], p->up));
        }
        return cudaSuccess;
    };
    // down stream: band k's result from the AoS staging to the host while later bands are
    // stepped
    auto enqueue_down = [&](int k) -> cudaError_t {
        HS_TRY(cudaStreamWaitEvent(p->down, p->ev_out[k], 0));
        if (hk) HS_TRY(cudaStreamWaitEvent(p->down, p->edge_done, 0));
        return copy_rows(s2, u2, b2, ao, ao + 2 * K, ao + 4 * K, band_rows(k), nf,
                         cudaMemcpyDeviceToHost, p->down);
    };
    // The host enqueues in the order the GPU needs the work: two bands up, then per band the
    // next upload, the step and the download, so the first step is queued after two bands'
    // uploads rather than after all of them (each band is a dozen API calls).
    HS_TRY(enqueue_up(1));
    // the step on band k once bands k and k + 1 are up (band k - 1, and the seam rows, came
    // before), bands taken in turn by the caller's stream and kCompStreams - 1 more:
    // the bands write disjoint rows and share one rotation ticket, so later bands' blocks
    // may start while the last wave of this one drains
    Params P = ctx->P;
    unsigned int nblocks = (unsigned int)(nx * T);
    if (hk) {
        // the edge cells in one launch over the whole grid (a band's few edge cells would
        // sit on a few SMs for as long as all of them take), the tiles band by band
        nblocks = gd::hancock_fast_blocks(P, 0, M, 1);
        for (int k = 0; k < B; ++k)
            nblocks += gd::hancock_fast_blocks(P, row_bound(k), row_bound(k + 1), 2);
    }
    P.tile_nblocks = nblocks;
    // in: the AoS staging of the upload; out: the next resident plane set and the AoS
    // staging of the download
    CPlanes in{};
    in.s = ai;
    in.u = ai + 2 * K;
    in.b = nf == 7 ? ai + 4 * K : nullptr;
    Planes out = ctx->planes(1 - ctx->cur);
    out.s = ao;
    out.u = ao + 2 * K;
    out.b = nf == 7 ? ao + 4 * K : nullptr;
    for (int k = 0; k < B; ++k) {
        HS_TRY(enqueue_up(k + 2));
        const int si = k % gd::kCompStreams;
        const cudaStream_t cs = si == 0 ? st : p->comp[si - 1];
        HS_TRY(cudaStreamWaitEvent(cs, p->ev_up[k + 1 < B ? k + 1 : k], 0));
        int t0, t1;
        band_tiles(k, &t0, &t1);
        P.tile_row0 = t0;
        P.tile_rows = t1 - t0;
        ctx->launches += 1;
        unsigned long long* Tb = &ctx->sc->T_bits;
        if (hk)
            HS_TRY(gd::launch_hancock_fast_rows(P, in, out, &ctx->sc->T_do, Tb, ctx->sc, ctx->sc,
                                                row_bound(k), row_bound(k + 1), nblocks, 2, cs));
        else if (ctx->cfg.mode == GD_MODE_PARITY)
            HS_TRY(P.scheme != GD_SCHEME_TVD
                       ? gd::launch_hancock_parity(P, in, out, &ctx->sc->T_do, Tb, ctx->sc,
                                                   ctx->sc, 0, cs)
                       : gd::launch_parity(P, in, out, &ctx->sc->T_do, Tb, ctx->sc, ctx->sc, 0,
                                           cs));
        else if (P.physics == GD_EULER)
            HS_TRY(gd::launch_euler_fast(P, in, out, &ctx->sc->T_do, Tb, ctx->sc, ctx->sc, 0,
                                         cs));
        else
            HS_TRY(gd::launch_mhd_fast(P, in, out, &ctx->sc->T_do, Tb, ctx->sc, ctx->sc, 0, cs));
        HS_TRY(cudaEventRecord(p->ev_out[k], cs));
        if (!hk) HS_TRY(enqueue_down(k));
    }
    if (hk) {
        // every upload is enqueued: the edge launch (it reads all of them), then the
        // downloads, each of which waits for it
        HS_TRY(cudaStreamWaitEvent(p->edge, p->ev_up[B - 1], 0));
        HS_TRY(gd::launch_hancock_fast_rows(P, in, out, &ctx->sc->T_do, &ctx->sc->T_bits,
                                            ctx->sc, ctx->sc, 0, M, nblocks, 1, p->edge));
        HS_TRY(cudaEventRecord(p->edge_done, p->edge));
        for (int k = 0; k < B; ++k) HS_TRY(enqueue_down(k));
    }
    // the caller's stream joins every stream the step used (a capture must end with all
    // of them joined; a stream no band used never joined it)
    for (int c = 1; c < B && c < gd::kCompStreams; ++c) {
        HS_TRY(cudaEventRecord(p->comp_done, p->comp[c - 1]));
        HS_TRY(cudaStreamWaitEvent(st, p->comp_done, 0));
    }
    if (hk) HS_TRY(cudaStreamWaitEvent(st, p->edge_done, 0));
    HS_TRY(cudaEventRecord(p->up_done, p->up));
    HS_TRY(cudaStreamWaitEvent(st, p->up_done, 0));
    HS_TRY(cudaEventRecord(p->down_done, p->down));
    HS_TRY(cudaStreamWaitEvent(st, p->down_done, 0));
    return cudaSuccess;
}

// The graph of the banded step for these host buffers and the current plane set: a cached
// one, or a new capture of banded_step (replacing the oldest).  Capturing executes nothing.
cudaError_t step_graph(gd_ctx* ctx, const double* s, const double* u, const double* b,
                       double* s2, double* u2, double* b2, int TX, int TY, gd::StepGraph** out) {
    gd::HostPipe* p = ctx->pipe;
    const void* buf[6] = {s, u, b, s2, u2, b2};
    for (gd::StepGraph& g : p->graphs) {
        if (!g.exec || g.cur != ctx->cur) continue;
        bool same = true;
        for (int i = 0; i < 6; ++i) same = same && g.buf[i] == buf[i];
        if (same) {
            *out = &g;
            return cudaSuccess;
        }
    }
    gd::StepGraph& g = p->graphs[p->next_graph];
    p->next_graph = (p->next_graph + 1) % gd::kStepGraphs;
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = gd::StepGraph{};
    const long long l0 = ctx->launches;
    HS_TRY(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = banded_step(ctx, s, u, b, s2, u2, b2, TX, TY, p->cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(p->cap, &graph);
    const long long n = ctx->launches - l0;
    ctx->launches = l0;  // counted when a replay runs
    if (e == cudaSuccess) e = ee;
    // the kernel nodes keep the priorities of the streams they were captured on
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&g.exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        g.exec = nullptr;
        return e;
    }
    for (int i = 0; i < 6; ++i) g.buf[i] = buf[i];
    g.cur = ctx->cur;
    g.launches = n;
    *out = &g;
    return cudaSuccess;
}

}  // namespace

namespace gd {
void pipe_free(gd_ctx* ctx) {
    HostPipe* p = ctx->pipe;
    if (!p) return;
    for (StepGraph& g : p->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    gd::dev_free(p->aos_in);
    gd::dev_free(p->aos_out);
    for (cudaEvent_t e : {p->start, p->down_done, p->comp_done, p->edge_done, p->up_done})
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < kMaxBands; ++k) {
        if (p->ev_up[k]) cudaEventDestroy(p->ev_up[k]);
        if (p->ev_out[k]) cudaEventDestroy(p->ev_out[k]);
    }
    if (p->up) cudaStreamDestroy(p->up);
    if (p->down) cudaStreamDestroy(p->down);
    for (cudaStream_t c : p->comp)
        if (c) cudaStreamDestroy(c);
    if (p->edge) cudaStreamDestroy(p->edge);
    if (p->cap) cudaStreamDestroy(p->cap);
    delete p;
    ctx->pipe = nullptr;
}
}  // namespace gd

extern "C" gd_status gd_step_host(gd_ctx* ctx, const double* s, const double* u, const double* b,
                                  double* s2, double* u2, double* b2, gd_stream stream) {
    if (!ctx || !s || !u || !s2 || !u2) return GD_ERR_INVALID_ARG;
    if (ctx->nf == 7 && (!b || !b2)) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const gd_config& c = ctx->cfg;
    int TX = 32, TY = 0;  // the block shape of the launch the bands are cut for
    if (c.mode == GD_MODE_PARITY)
        TY = gd::kParityBlockRows;
    else if (c.scheme != GD_SCHEME_TVD)
        TY = gd::hancock_tile_height();
    else if (c.physics == GD_EULER)
        gd::euler_tile_shape(0, &TX, &TY);
    else
        TY = gd::mhd_tile_height();
    // the banded pipeline: the reference's dt protocol, grids of at least four tile (block)
    // rows, host buffers the device can read and write (pinned)
    const int rows = (c.mode == GD_MODE_FAST && c.scheme != GD_SCHEME_TVD) ? c.M - 4 : c.M;
    const bool banded = ctx->dt_policy == GD_DT_LAGGED && rows > 0 && (rows + TY - 1) / TY >= 4 &&
                        device_visible_host(s) && device_visible_host(u) &&
                        device_visible_host(b) && device_visible_host(s2) &&
                        device_visible_host(u2) && device_visible_host(b2);
    if (!banded) {
        gd_status r = gd_import(ctx, s, u, b, 1, stream);
        if (r == GD_OK) r = gd_advance(ctx, 1, 0, stream);
        if (r == GD_OK) r = gd_export(ctx, s2, u2, b2, 1, stream);
        return r;
    }
    cudaError_t e = pipe_init(ctx);
    gd::StepGraph* g = nullptr;
    if (e == cudaSuccess) e = step_graph(ctx, s, u, b, s2, u2, b2, TX, TY, &g);
    if (e == cudaSuccess) e = cudaGraphLaunch(g->exec, st);
    if (e == cudaSuccess) ctx->launches += g->launches;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return gd::cuda_error(e);
    ctx->cur ^= 1;
    return GD_OK;
}
