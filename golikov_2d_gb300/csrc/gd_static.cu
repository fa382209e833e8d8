// gd_static.cu -- one step in the reference layout without any device allocation.
//
// gd_step_ref needs scratch memory beyond its inputs and outputs: SoA staging planes for the
// converted state and a small block of counters.  A context allocates those with cudaMalloc.
// Some callers cannot let a library allocate: a host program that owns every byte of device
// memory through its own pool (a coupled multi-physics driver, an in-situ analysis
// framework), or one on a latency-critical path, because cudaMalloc allocates outside the
// owner's budget and cudaFree synchronises the whole device.  gd_step_ref_static serves them:
// its scratch is the file-scope device array below, of a fixed size stated in gd2d.h
// (GD_STATIC_MAX_CELLS cells), present on every GPU that loads this library until the
// process exits.
//
// Host code must not pass `g_static_scratch` itself to a kernel: in host code that name is
// only a stand-in for the device variable.  Its device address is obtained once per device
// with cudaGetSymbolAddress, with that device current, and that address is what the
// kernels receive.
#include <mutex>

#include "../../include/gd2d.h"
#include "gd_internal.cuh"
#include "gd_kernels.h"

namespace {

constexpr size_t kHeaderBytes = 256;  // counters (gd::Scalars), padded
constexpr size_t kPlaneBytes = sizeof(double) * (size_t)GD_STATIC_MAX_CELLS;
constexpr size_t kScratchBytes = kHeaderBytes + 2 * gd::kMaxFields * kPlaneBytes;
static_assert(sizeof(gd::Scalars) <= kHeaderBytes, "counter block does not fit its slot");
static_assert(kScratchBytes == GD_STATIC_SCRATCH_BYTES, "gd2d.h states a different size");

// Layout: [counters | 7 input planes | 7 output planes], each plane N*M doubles at most
// GD_STATIC_MAX_CELLS.  Shared by every call on a device; contents persist between calls.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Per-device set-up, done by the first call on that device with the device current:
// the device address of the scratch array and the fast kernels' shared-memory attributes.
gd_status scratch_for_device(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return gd::cuda_error(e);
        if (p == nullptr) return GD_ERR_CUDA;
        e = gd::prepare_euler_fast();
        if (e == cudaSuccess) e = gd::prepare_mhd_fast();
        if (e == cudaSuccess) e = gd::prepare_hancock_fast();
        if (e != cudaSuccess) return gd::cuda_error(e);
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GD_OK;
}

}  // namespace

extern "C" gd_status gd_step_ref_static(const gd_config* cfg, const double* s, const double* u,
                                        const double* b, double* s2, double* u2, double* b2,
                                        double* T, const double* T_do, int method,
                                        gd_stream stream) {
    const gd_status v = gd::validate_config(cfg);
    if (v != GD_OK) return v;
    if (!s || !u || !s2 || !u2 || !T || !T_do) return GD_ERR_INVALID_ARG;
    const int nf = cfg->physics == GD_MHD ? 7 : 4;
    if (nf == 7 && (!b || !b2)) return GD_ERR_INVALID_ARG;
    const long long K = (long long)cfg->N * cfg->M;
    if (K > GD_STATIC_MAX_CELLS) return GD_ERR_INVALID_ARG;  // beyond the fixed scratch
    gd::Params P = gd::params_from_config(*cfg);
    if (method != GD_METHOD_CONFIG) {
        if (cfg->physics == GD_EULER && method != GD_METHOD_HLLC && method != GD_METHOD_HLL)
            return GD_ERR_INVALID_ARG;
        if (cfg->physics == GD_MHD && method != GD_METHOD_HLLC_MHD && method != GD_METHOD_HLLD)
            return GD_ERR_INVALID_ARG;
        if (cfg->scheme != GD_SCHEME_TVD && method != GD_METHOD_HLLD) return GD_ERR_UNSUPPORTED;
        P.method = method;
    }
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return gd::cuda_error(ce);
    if (dev < 0 || dev >= kMaxDevices) return GD_ERR_UNSUPPORTED;
    void* base = nullptr;
    const gd_status st = scratch_for_device(dev, &base);
    if (st != GD_OK) return st;

    cudaStream_t cs = (cudaStream_t)stream;
    gd::Scalars* ctr = static_cast<gd::Scalars*>(base);
    double* planes = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kHeaderBytes);
    gd::Planes in{}, out{};
    gd::CPlanes cin{}, cout{};
    for (int f = 0; f < nf; ++f) {
        in.f[f] = planes + (size_t)f * K;
        out.f[f] = planes + (size_t)(nf + f) * K;
        cin.f[f] = in.f[f];
        cout.f[f] = out.f[f];
    }
    // the floor / non-finite counters start from zero at every call
    ce = cudaMemsetAsync(ctr, 0, sizeof(gd::Scalars), cs);
    if (ce == cudaSuccess) ce = gd::launch_aos_to_soa(s, u, b, in, K, nf, cs);
    if (ce != cudaSuccess) return gd::cuda_error(ce);
    cudaError_t e;
    unsigned long long* Tb = (unsigned long long*)T;
    if (cfg->scheme != GD_SCHEME_TVD)
        e = cfg->mode == GD_MODE_PARITY
                ? gd::launch_hancock_parity(P, cin, out, T_do, Tb, nullptr, ctr, 0, cs)
                : gd::launch_hancock_fast(P, cin, out, T_do, Tb, nullptr, ctr, 0, cs);
    else if (cfg->mode == GD_MODE_PARITY)
        e = gd::launch_parity(P, cin, out, T_do, (unsigned long long*)T, nullptr, ctr, 0, cs);
    else if (cfg->physics == GD_EULER)
        e = gd::launch_euler_fast(P, cin, out, T_do, (unsigned long long*)T, nullptr, ctr, 0, cs);
    else
        e = gd::launch_mhd_fast(P, cin, out, T_do, (unsigned long long*)T, nullptr, ctr, 0, cs);
    if (e == cudaSuccess) e = gd::launch_soa_to_aos(cout, s2, u2, b2, K, nf, cs);
    if (e != cudaSuccess) return gd::cuda_error(e);
    return GD_OK;
}
