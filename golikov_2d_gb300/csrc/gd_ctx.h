// gd_ctx.h -- the context behind the C ABI's gd_ctx handle (internal).
#pragma once

#include <map>
#include <utility>

#include "../../include/gd2d.h"
#include "gd_internal.cuh"

namespace gd {

// Record of a differentiated forward run (gd_adj_forward): dt sequence, checkpoints and
// work buffers of the reverse and tangent sweeps.
// gd_step_host: the two copy streams, the events of the band pipeline and the AoS staging
// of the input and of the output (7 K doubles each: s 2K, u 2K, b 3K), which the step reads
// and writes directly.
// The banded step is captured once per (host buffers, current plane set) into a CUDA graph
// and replayed: a graph launch puts all of a step's copies and launches on the GPU at once,
// where enqueuing them one API call at a time (a dozen per band) paces a short step.
// At most 32 bands: every band's upload and download is a copy of its own, and at 64 bands
// the per-copy cost outweighed the shorter fill and drain (KH 4096^2 host to host: 4.42 ms
// per step at 64 bands, 4.26 at 32, 4.50 at 16).
constexpr int kMaxBands = 32;
constexpr int kCompStreams = 3;  // the caller's stream and two more
constexpr int kStepGraphs = 4;   // cached step graphs (two per ping-pong pair of host buffers)
struct StepGraph {
    const void* buf[6] = {};  // s, u, b, s2, u2, b2
    int cur = -1;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;  // kernel launches one replay makes
};
struct HostPipe {
    cudaStream_t up = nullptr, down = nullptr, edge = nullptr;
    cudaStream_t comp[kCompStreams - 1] = {};
    cudaStream_t cap = nullptr;  // the origin stream of the captures
    cudaEvent_t start = nullptr, down_done = nullptr, comp_done = nullptr, edge_done = nullptr;
    cudaEvent_t up_done = nullptr;
    cudaEvent_t ev_up[kMaxBands] = {}, ev_out[kMaxBands] = {};
    double* aos_in = nullptr;
    double* aos_out = nullptr;
    StepGraph graphs[kStepGraphs];
    int next_graph = 0;  // slot the next capture replaces
};

struct AdjStore {
    int nsteps = 0, every = 0, nckpt = 0;
    double* dts = nullptr;       // nsteps
    double* ckpt = nullptr;      // nckpt * nf * K: state at steps 0, every, 2 every, ...
    double* seg = nullptr;       // (every + 1) * nf * K: states of one segment
    double* aux = nullptr;       // every * 8 * K: flux differences and Powell term per step
    double* lam = nullptr;       // 2 * nf * K
    double* scratch = nullptr;   // adjoint_scratch_planes() * K
    double* tbits = nullptr;     // dt accumulator the recompute pass writes (unused value)
    int seg_holds = -1;          // segment whose input states and update terms seg/aux hold
    // second segment buffer: the backward sweep recomputes segment k-1 into one buffer on
    // `side` while it reverses segment k out of the other
    double* seg2 = nullptr;      // as seg
    double* aux2 = nullptr;      // as aux
    int seg2_holds = -1;         // segment seg2/aux2 hold
    cudaStream_t side = nullptr;
    cudaEvent_t ev_start = nullptr, ev_rec[2] = {nullptr, nullptr}, ev_rev[2] = {nullptr, nullptr};
};

// Work buffers of the state I/O entry points (gd_io.cu), grown on demand.
struct IoScratch {
    char* dev = nullptr;   // device: line slots, lengths, offsets, scan partials, output
    size_t dev_cap = 0;
    char* host = nullptr;  // pinned staging for file reads and writes
    size_t host_cap = 0;
};

}  // namespace gd

using gd::CPlanes;
using gd::Params;
using gd::Planes;
using gd::Scalars;

struct gd_ctx {
    gd_config cfg;
    Params P;
    int nf = 4;
    long long K = 0;
    int device = 0;
    double* state[2] = {nullptr, nullptr};  // nf planes of K doubles each
    int cur = 0;
    Scalars* sc = nullptr;                  // device scalars of the resident state
    double* aos = nullptr;                  // 7 * K: AoS staging for host import/export
    long long launches = 0;
    int step_launches = 1;                  // kernel launches of one step (fast Hancock: 2)
    int dt_policy = GD_DT_LAGGED;           // gd_set_dt_policy
    long long floor_limit = 0;              // gd_set_floor_limit (0: none)
    gd::HancockStreams* side = nullptr;     // fast Hancock: stream + events of the band launch
    gd::HostPipe* pipe = nullptr;           // gd_step_host: copy streams, events, AoS staging
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (nsteps, cur) -> graph
    gd::AdjStore* adj = nullptr;            // differentiation record (gd_adj_forward)
    gd::IoScratch* io = nullptr;            // state I/O work buffers (gd_io.cu)

    Planes planes(int which) const {
        Planes p{};
        for (int f = 0; f < gd::kMaxFields; ++f)
            p.f[f] = f < nf ? state[which] + (size_t)f * K : nullptr;
        return p;
    }
    static CPlanes cplanes(const Planes& p) {
        CPlanes c{};
        for (int f = 0; f < gd::kMaxFields; ++f) c.f[f] = p.f[f];
        return c;
    }
};

namespace gd {
void adj_free(gd_ctx* ctx);
void io_free(gd_ctx* ctx);
void pipe_free(gd_ctx* ctx);
}  // namespace gd
