// gd_adj_api.cu -- C ABI of the differentiation entry points (include/gd2d.h):
// gd_adj_forward, gd_adj_backward, gd_tangent, gd_adj_replay.
//
// Checkpointing: the forward run stores the state every `ckpt_every` steps and the dt of
// every step.  The backward sweep walks the segments from last to first; each segment is
// recomputed once from its checkpoint (storing each step's input state and the flux
// differences / Powell term the update used), then stepped back in reverse.  The last
// segment is recorded that way during the forward run itself, so it is not recomputed.
// Memory is O(nsteps / every + every) states instead of O(nsteps).
#include <cstring>
#include <new>

#include "../../include/gd2d.h"
#include "gd_ctx.h"
#include "gd_kernels.h"

namespace gd {

void adj_free(gd_ctx* ctx) {
    AdjStore* a = ctx->adj;
    if (!a) return;
    gd::dev_free(a->dts);
    gd::dev_free(a->ckpt);
    gd::dev_free(a->seg);
    gd::dev_free(a->aux);
    gd::dev_free(a->lam);
    gd::dev_free(a->scratch);
    gd::dev_free(a->tbits);
    gd::dev_free(a->seg2);
    gd::dev_free(a->aux2);
    for (cudaEvent_t e : {a->ev_start, a->ev_rec[0], a->ev_rec[1], a->ev_rev[0], a->ev_rev[1]})
        if (e) cudaEventDestroy(e);
    if (a->side) cudaStreamDestroy(a->side);
    delete a;
    ctx->adj = nullptr;
}

}  // namespace gd

namespace {

#define GD_TRY(call)                                          \
    do {                                                      \
        const cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return gd::cuda_error(e_);     \
    } while (0)

bool adj_supported(const gd_ctx* ctx) {
    const gd_config& c = ctx->cfg;
    for (int s = 0; s < 4; ++s)
        if (c.bc[s] != GD_BC_PERIODIC) return false;
    const bool flux = (c.physics == GD_MHD && c.method == GD_METHOD_HLLD) ||
                      (c.physics == GD_EULER && c.method == GD_METHOD_HLLC);
    return c.scheme == GD_SCHEME_TVD && flux && c.order == 2 && c.geometry == GD_CARTESIAN &&
           c.mode == GD_MODE_FAST && c.frozen_radius == 0.0;
}

// planes of update terms stored per recorded step: MHD d[0..6] and the Powell term, Euler
// d[0..3]
int aux_planes(const gd_ctx* ctx) { return ctx->nf == 7 ? 8 : 4; }

// the fast step writing its update terms to `aux` (null: not stored)
cudaError_t step_aux(const gd_ctx* ctx, const Params& P, const CPlanes& in, const Planes& out,
                     const double* T_do, unsigned long long* T_bits, Scalars* rot, Scalars* ctr,
                     double* aux, cudaStream_t st) {
    return ctx->nf == 7 ? gd::launch_mhd_fast_aux(P, in, out, T_do, T_bits, rot, ctr, aux, st)
                        : gd::launch_euler_fast_aux(P, in, out, T_do, T_bits, rot, ctr, aux, st);
}

cudaError_t reverse_step(const gd_ctx* ctx, const Params& P, const CPlanes& U, const double* aux,
                         const CPlanes& lam_out, const Planes& lam_in, double* scratch,
                         const double* T_do, cudaStream_t st) {
    return ctx->nf == 7
               ? gd::launch_adjoint_step(P, U, aux, lam_out, lam_in, scratch, T_do, st)
               : gd::launch_adjoint_step_euler(P, U, aux, lam_out, lam_in, scratch, T_do, st);
}

// (Re)allocates the recording store for nsteps steps with a checkpoint every `every`
// steps; called only when the recording's shape changes, so a gradient loop allocates once.
gd_status alloc_store(gd_ctx* ctx, int nsteps, int every, size_t state) {
    const long long K = ctx->K;
    gd::adj_free(ctx);
    gd::AdjStore* a = new (std::nothrow) gd::AdjStore();
    if (!a) return GD_ERR_INVALID_ARG;
    ctx->adj = a;
    a->nsteps = nsteps;
    a->every = every;
    a->nckpt = (nsteps + every - 1) / every;
    GD_TRY(gd::dev_alloc(&a->dts, sizeof(double) * nsteps));
    GD_TRY(gd::dev_alloc(&a->ckpt, state * a->nckpt));
    GD_TRY(gd::dev_alloc(&a->seg, state * (every + 1)));
    const int naux = aux_planes(ctx);
    GD_TRY(gd::dev_alloc(&a->aux, sizeof(double) * naux * (size_t)K * every));
    GD_TRY(gd::dev_alloc(&a->lam, 2 * state));
    const int nscr = ctx->nf == 7 ? gd::adjoint_scratch_planes()
                                  : gd::adjoint_euler_scratch_planes();
    GD_TRY(gd::dev_alloc(&a->scratch, sizeof(double) * (size_t)nscr * (size_t)K));
    GD_TRY(gd::dev_alloc(&a->tbits, sizeof(double)));
    GD_TRY(gd::dev_alloc(&a->seg2, state * (every + 1)));
    GD_TRY(gd::dev_alloc(&a->aux2, sizeof(double) * naux * (size_t)K * every));
    GD_TRY(cudaStreamCreateWithFlags(&a->side, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&a->ev_start, &a->ev_rec[0], &a->ev_rec[1], &a->ev_rev[0],
                           &a->ev_rev[1]})
        GD_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    GD_TRY(gd::prepare_adjoint());
    return GD_OK;
}

Planes planes_at(double* base, int nf, long long K) {
    Planes p{};
    for (int f = 0; f < nf; ++f) p.f[f] = base + (size_t)f * K;
    return p;
}

CPlanes cplanes_at(const double* base, int nf, long long K) {
    CPlanes p{};
    for (int f = 0; f < nf; ++f) p.f[f] = base + (size_t)f * K;
    return p;
}

}  // namespace

extern "C" {

gd_status gd_adj_forward(gd_ctx* ctx, int nsteps, int ckpt_every, gd_stream stream) {
    if (!ctx || nsteps < 1 || ckpt_every < 1) return GD_ERR_INVALID_ARG;
    if (!adj_supported(ctx)) return GD_ERR_UNSUPPORTED;
    // the recording steps and the recomputed segments use the dt rotated by the previous
    // step (GD_DT_LAGGED); under GD_DT_CURRENT the steps taken would not be the recorded map
    if (ctx->dt_policy != GD_DT_LAGGED) return GD_ERR_UNSUPPORTED;
    const long long K = ctx->K;
    const int nf = ctx->nf;
    const int every = ckpt_every < nsteps ? ckpt_every : nsteps;
    const size_t state = sizeof(double) * (size_t)nf * K;
    gd::AdjStore* a = ctx->adj;
    if (!a || a->nsteps != nsteps || a->every != every) {
        const gd_status r = alloc_store(ctx, nsteps, every, state);
        if (r != GD_OK) {
            gd::adj_free(ctx);  // all or nothing: the next call allocates afresh
            return r;
        }
        a = ctx->adj;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // The last two segments are stepped out of the two segment buffers with the update terms
    // stored (the last in seg/aux, the one before in seg2/aux2: the buffers the backward sweep
    // alternates between), so the sweep starts reversing at once and recomputes two segments
    // fewer.
    const int k_last = (a->nckpt - 1) * every;
    const int k_prev = a->nckpt >= 2 ? k_last - every : k_last;
    a->seg_holds = -1;
    a->seg2_holds = -1;
    for (int s = 0; s < nsteps; ++s) {
        if (s % every == 0)
            GD_TRY(cudaMemcpyAsync(a->ckpt + (size_t)(s / every) * nf * K, ctx->state[ctx->cur],
                                   state, cudaMemcpyDeviceToDevice, st));
        GD_TRY(cudaMemcpyAsync(a->dts + s, &ctx->sc->T_do, sizeof(double),
                               cudaMemcpyDeviceToDevice, st));
        if (s < k_prev) {
            const gd_status r = gd_advance(ctx, 1, 0, stream);
            if (r != GD_OK) return r;
            continue;
        }
        // the same step as gd_advance (dt rotation and counters included), reading its input
        // from buffer[j] and writing its output to buffer[j + 1]
        const bool last = s >= k_last;
        double* seg = last ? a->seg : a->seg2;
        double* aux = last ? a->aux : a->aux2;
        const int j = s - (last ? k_last : k_prev);
        if (j == 0)
            GD_TRY(cudaMemcpyAsync(seg, ctx->state[ctx->cur], state, cudaMemcpyDeviceToDevice,
                                   st));
        GD_TRY(step_aux(ctx, ctx->P, cplanes_at(seg + (size_t)j * nf * K, nf, K),
                        planes_at(seg + (size_t)(j + 1) * nf * K, nf, K), &ctx->sc->T_do,
                        &ctx->sc->T_bits, ctx->sc, ctx->sc,
                        aux + (size_t)j * aux_planes(ctx) * K, st));
        ctx->launches += 1;
        // the segment's last output is the context's state for what follows
        if (j + 1 == (last ? nsteps - k_last : every))
            GD_TRY(cudaMemcpyAsync(ctx->state[ctx->cur], seg + (size_t)(j + 1) * nf * K, state,
                                   cudaMemcpyDeviceToDevice, st));
    }
    a->seg_holds = a->nckpt - 1;
    if (a->nckpt >= 2) a->seg2_holds = a->nckpt - 2;
    return GD_OK;
}

gd_status gd_adj_backward(gd_ctx* ctx, const double* gs, const double* gu, const double* gb,
                          double* os, double* ou, double* ob, gd_stream stream) {
    if (!ctx || !ctx->adj || !gs || !gu || !os || !ou) return GD_ERR_INVALID_ARG;
    if (ctx->nf == 7 && (!gb || !ob)) return GD_ERR_INVALID_ARG;
    gd::AdjStore* a = ctx->adj;
    const long long K = ctx->K;
    const int nf = ctx->nf;
    const Params& P = ctx->P;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t state = sizeof(double) * (size_t)nf * K;
    double* lam[2] = {a->lam, a->lam + (size_t)nf * K};
    double* segb[2] = {a->seg, a->seg2};
    double* auxb[2] = {a->aux, a->aux2};
    int c = 0;
    GD_TRY(gd::launch_aos_to_soa(gs, gu, gb, planes_at(lam[0], nf, K), K, nf, st));
    auto seg_range = [&](int sg, int* k0, int* len) {
        *k0 = sg * a->every;
        const int k1 = *k0 + a->every < a->nsteps ? *k0 + a->every : a->nsteps;
        *len = k1 - *k0;
    };
    // the input states and update terms of every step of segment sg, into buffer b
    auto recompute = [&](int sg, int b, cudaStream_t s) -> gd_status {
        int k0, len;
        seg_range(sg, &k0, &len);
        GD_TRY(cudaMemcpyAsync(segb[b], a->ckpt + (size_t)sg * nf * K, state,
                               cudaMemcpyDeviceToDevice, s));
        for (int j = 0; j < len; ++j) {
            GD_TRY(step_aux(ctx, P, cplanes_at(segb[b] + (size_t)j * nf * K, nf, K),
                            planes_at(segb[b] + (size_t)(j + 1) * nf * K, nf, K),
                            a->dts + k0 + j, (unsigned long long*)a->tbits, nullptr, nullptr,
                            auxb[b] + (size_t)j * aux_planes(ctx) * K, s));
            ctx->launches += 1;
        }
        return GD_OK;
    };
    // Segments last to first.  While segment sg is reversed out of buffer b on `st`, segment
    // sg - 1 is recomputed into buffer b ^ 1 on the side stream, after the reversal that last
    // read that buffer; the reversal of sg - 1 waits for its recomputation.  Same launches and
    // inputs as one stream, so the result is the same bit for bit.
    int holds[2] = {a->seg_holds, a->seg2_holds};
    const int last = a->nckpt - 1;
    int b = holds[1] == last ? 1 : 0;
    if (holds[b] != last) {
        const gd_status r = recompute(last, b, st);
        if (r != GD_OK) return r;
        holds[b] = last;
    }
    GD_TRY(cudaEventRecord(a->ev_start, st));
    GD_TRY(cudaStreamWaitEvent(a->side, a->ev_start, 0));
    bool other_busy = false;  // buffer b ^ 1 has a recorded reversal to wait for
    for (int sg = last; sg >= 0; --sg) {
        bool wait_rec = false;
        if (sg > 0 && holds[b ^ 1] != sg - 1) {
            if (other_busy) GD_TRY(cudaStreamWaitEvent(a->side, a->ev_rev[b ^ 1], 0));
            const gd_status r = recompute(sg - 1, b ^ 1, a->side);
            if (r != GD_OK) return r;
            GD_TRY(cudaEventRecord(a->ev_rec[b ^ 1], a->side));
            holds[b ^ 1] = sg - 1;
            wait_rec = true;
        }
        int k0, len;
        seg_range(sg, &k0, &len);
        for (int j = len - 1; j >= 0; --j) {
            GD_TRY(reverse_step(ctx, P, cplanes_at(segb[b] + (size_t)j * nf * K, nf, K),
                                auxb[b] + (size_t)j * aux_planes(ctx) * K,
                                cplanes_at(lam[c], nf, K), planes_at(lam[c ^ 1], nf, K),
                                a->scratch, a->dts + k0 + j, st));
            ctx->launches += 3;
            c ^= 1;
        }
        if (sg > 0) {
            GD_TRY(cudaEventRecord(a->ev_rev[b], st));
            if (wait_rec) GD_TRY(cudaStreamWaitEvent(st, a->ev_rec[b ^ 1], 0));
            other_busy = true;
            b ^= 1;
        }
    }
    // the reversal only reads the buffers: they still hold what they were filled with
    a->seg_holds = holds[0];
    a->seg2_holds = holds[1];
    GD_TRY(gd::launch_soa_to_aos(cplanes_at(lam[c], nf, K), os, ou, ob, K, nf, st));
    return GD_OK;
}

gd_status gd_tangent(gd_ctx* ctx, const double* vs, const double* vu, const double* vb,
                     double* os, double* ou, double* ob, gd_stream stream) {
    if (!ctx || !ctx->adj || !vs || !vu || !os || !ou) return GD_ERR_INVALID_ARG;
    if (ctx->nf == 7 && (!vb || !ob)) return GD_ERR_INVALID_ARG;
    gd::AdjStore* a = ctx->adj;
    const long long K = ctx->K;
    const int nf = ctx->nf;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t state = sizeof(double) * (size_t)nf * K;
    double* t[2] = {a->lam, a->lam + (size_t)nf * K};
    double* u[2] = {a->seg, a->seg + (size_t)nf * K};
    a->seg_holds = -1;  // seg is the work space of this sweep
    GD_TRY(gd::launch_aos_to_soa(vs, vu, vb, planes_at(t[0], nf, K), K, nf, st));
    GD_TRY(cudaMemcpyAsync(u[0], a->ckpt, state, cudaMemcpyDeviceToDevice, st));
    int c = 0;
    for (int k = 0; k < a->nsteps; ++k) {
        const CPlanes ui = cplanes_at(u[c], nf, K), ti = cplanes_at(t[c], nf, K);
        const Planes uo = planes_at(u[c ^ 1], nf, K), to = planes_at(t[c ^ 1], nf, K);
        GD_TRY(nf == 7 ? gd::launch_mhd_tangent(ctx->P, ui, ti, uo, to, a->dts + k, st)
                       : gd::launch_euler_tangent(ctx->P, ui, ti, uo, to, a->dts + k, st));
        ctx->launches += 1;
        c ^= 1;
    }
    GD_TRY(gd::launch_soa_to_aos(cplanes_at(t[c], nf, K), os, ou, ob, K, nf, st));
    return GD_OK;
}

gd_status gd_adj_replay(gd_ctx* ctx, const double* s, const double* u, const double* b,
                        double* os, double* ou, double* ob, gd_stream stream) {
    if (!ctx || !ctx->adj || !s || !u || !os || !ou) return GD_ERR_INVALID_ARG;
    if (ctx->nf == 7 && (!b || !ob)) return GD_ERR_INVALID_ARG;
    gd::AdjStore* a = ctx->adj;
    const long long K = ctx->K;
    const int nf = ctx->nf;
    cudaStream_t st = (cudaStream_t)stream;
    double* w[2] = {a->seg, a->seg + (size_t)nf * K};
    a->seg_holds = -1;  // seg is the work space of this sweep
    GD_TRY(gd::launch_aos_to_soa(s, u, b, planes_at(w[0], nf, K), K, nf, st));
    int c = 0;
    for (int k = 0; k < a->nsteps; ++k) {
        GD_TRY(step_aux(ctx, ctx->P, cplanes_at(w[c], nf, K), planes_at(w[c ^ 1], nf, K),
                        a->dts + k, (unsigned long long*)a->tbits, nullptr, nullptr, nullptr,
                        st));
        ctx->launches += 1;
        c ^= 1;
    }
    GD_TRY(gd::launch_soa_to_aos(cplanes_at(w[c], nf, K), os, ou, ob, K, nf, st));
    return GD_OK;
}

gd_status gd_adj_switches(gd_ctx* ctx, const double* sp, const double* up, const double* bp,
                          const double* sm, const double* um, const double* bm, double* osp,
                          double* oup, double* obp, double* osm, double* oum, double* obm,
                          long long* counts, gd_stream stream) {
    if (!ctx || !ctx->adj || !counts) return GD_ERR_INVALID_ARG;
    if (ctx->nf != 7) return GD_ERR_UNSUPPORTED;  // the switch codes are those of HLLD
    for (const void* p : {(const void*)sp, (const void*)up, (const void*)bp, (const void*)sm,
                          (const void*)um, (const void*)bm, (const void*)osp, (const void*)oup,
                          (const void*)obp, (const void*)osm, (const void*)oum, (const void*)obm})
        if (!p) return GD_ERR_INVALID_ARG;
    gd::AdjStore* a = ctx->adj;
    const long long K = ctx->K;
    const int nf = ctx->nf;
    const int nk = gd::switch_kinds();
    cudaStream_t st = (cudaStream_t)stream;
    // work space: both runs' two states in the two segment buffers (each holds at least two
    // states), their update terms in the two aux buffers, marks and counters in scratch
    double* wp[2] = {a->seg, a->seg + (size_t)nf * K};
    double* wm[2] = {a->seg2, a->seg2 + (size_t)nf * K};
    a->seg_holds = -1;
    a->seg2_holds = -1;
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(a->scratch);
    unsigned char* step_mark = reinterpret_cast<unsigned char*>(a->scratch + 8);
    unsigned char* ever_mark = step_mark + K;
    GD_TRY(cudaMemsetAsync(a->scratch, 0, 64 + 2 * (size_t)K, st));
    GD_TRY(gd::launch_aos_to_soa(sp, up, bp, planes_at(wp[0], nf, K), K, nf, st));
    GD_TRY(gd::launch_aos_to_soa(sm, um, bm, planes_at(wm[0], nf, K), K, nf, st));
    ctx->launches += 2;
    int c = 0;
    for (int k = 0; k < a->nsteps; ++k) {
        const CPlanes ip = cplanes_at(wp[c], nf, K), im = cplanes_at(wm[c], nf, K);
        GD_TRY(gd::launch_switch_faces(ctx->P, ip, im, ctr, step_mark, st));
        GD_TRY(step_aux(ctx, ctx->P, ip, planes_at(wp[c ^ 1], nf, K), a->dts + k,
                        (unsigned long long*)a->tbits, nullptr, nullptr, a->aux, st));
        GD_TRY(step_aux(ctx, ctx->P, im, planes_at(wm[c ^ 1], nf, K), a->dts + k,
                        (unsigned long long*)a->tbits, nullptr, nullptr, a->aux2, st));
        GD_TRY(gd::launch_switch_cells(ctx->P, ip, a->aux, im, a->aux2, ctr, step_mark,
                                       ever_mark, st));
        ctx->launches += 4;
        c ^= 1;
    }
    GD_TRY(gd::launch_switch_total(K, ever_mark, ctr, st));
    GD_TRY(gd::launch_soa_to_aos(cplanes_at(wp[c], nf, K), osp, oup, obp, K, nf, st));
    GD_TRY(gd::launch_soa_to_aos(cplanes_at(wm[c], nf, K), osm, oum, obm, K, nf, st));
    ctx->launches += 3;
    unsigned long long h[16] = {};
    GD_TRY(cudaMemcpyAsync(h, ctr, sizeof(unsigned long long) * nk, cudaMemcpyDeviceToHost, st));
    GD_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < nk; ++i) counts[i] = (long long)h[i];
    return GD_OK;
}

}  // extern "C"
