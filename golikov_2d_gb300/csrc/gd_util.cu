// gd_util.cu -- layout conversion, the funk_time rotation, scalar setup, the FP64
// throughput probe and the check of the integer-pipe multiplication.
#include "gd_internal.cuh"
#include "gd_kernels.h"

namespace gd {
namespace {

// Reference AoS (kernel.cu:3814-3825) -> SoA planes.  s, u: double2[K]; b: double3[K].
__global__ void aos_to_soa_kernel(const double2* __restrict__ s, const double2* __restrict__ u,
                                  const double* __restrict__ b, Planes out, long long K, int nf) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
         k += (long long)gridDim.x * blockDim.x) {
        const double2 sv = s[k], uv = u[k];
        out.f[0][k] = sv.x;
        out.f[1][k] = sv.y;
        out.f[2][k] = uv.x;
        out.f[3][k] = uv.y;
        if (nf > 4) {
            out.f[4][k] = b[3 * k];
            out.f[5][k] = b[3 * k + 1];
            out.f[6][k] = b[3 * k + 2];
        }
    }
}

__global__ void soa_to_aos_kernel(CPlanes in, double2* __restrict__ s, double2* __restrict__ u,
                                  double* __restrict__ b, long long K, int nf) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
         k += (long long)gridDim.x * blockDim.x) {
        s[k] = make_double2(in.f[0][k], in.f[1][k]);
        u[k] = make_double2(in.f[2][k], in.f[3][k]);
        if (nf > 4) {
            b[3 * k] = in.f[4][k];
            b[3 * k + 1] = in.f[5][k];
            b[3 * k + 2] = in.f[6][k];
        }
    }
}

// kernel.cu:1722-1733 without the progress print.
__global__ void funk_time_kernel(double* T, double* T_do, double* TT, int* i) {
    *T_do = *T;
    *TT = *TT + *T_do;
    *T = kTReset;
    *i = *i + 1;
}

__device__ __forceinline__ void set_time_kernel_body(Scalars* sc, double T_do, double TT) {
    sc->T_do = T_do;
    sc->TT = TT;
    sc->t_state = TT;
    sc->T_bits = (unsigned long long)__double_as_longlong(kTReset);
    sc->done = 0;
}

__global__ void set_time_kernel(Scalars* sc, double T_do, double TT) {
    set_time_kernel_body(sc, T_do, TT);
}

// End of a dt-only pass: T_do <- T (limited by t_end when set), T <- 1e7 (TT and the step
// counter unchanged).
__global__ void dt_commit_kernel(Scalars* sc) {
    sc->T_cfl = __longlong_as_double((long long)sc->T_bits);
    sc->T_do = clamp_to_end(sc, sc->T_cfl);
    sc->T_bits = (unsigned long long)__double_as_longlong(kTReset);
    sc->done = 0;
}

// Sets t_end and limits the pending T_do to it; t_end = 0 clears it and gives back the CFL dt
// the limit replaced (TT follows, so that it still includes the pending dt).
__global__ void set_end_kernel(Scalars* sc, double t_end) {
    if (t_end > 0.0) {
        sc->T_cfl = sc->T_do;
        sc->t_end = t_end;
        const double T = clamp_to_end(sc, sc->T_cfl);
        sc->TT = sc->TT + (T - sc->T_do);
        sc->T_do = T;
    } else {
        if (sc->t_end > 0.0) {
            sc->TT = sc->TT + (sc->T_cfl - sc->T_do);
            sc->T_do = sc->T_cfl;
        }
        sc->t_end = 0.0;
    }
}

__global__ void reset_T_kernel(Scalars* sc) {
    sc->T_bits = (unsigned long long)__double_as_longlong(kTReset);
    sc->done = 0;
}

// Per-grid versions for a batch: one thread per grid.
__global__ void batch_set_time_kernel(BatchGrid* grids, int ngrids, double T_do, double TT) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ngrids) set_time_kernel_body(grids[g].sc, T_do, TT);
}
__global__ void batch_reset_T_kernel(BatchGrid* grids, int ngrids) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngrids) return;
    Scalars* sc = grids[g].sc;
    sc->T_bits = (unsigned long long)__double_as_longlong(kTReset);
    sc->done = 0;
}
__global__ void batch_dt_commit_kernel(BatchGrid* grids, int ngrids) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngrids) return;
    Scalars* sc = grids[g].sc;
    sc->T_do = __longlong_as_double((long long)sc->T_bits);
    sc->T_bits = (unsigned long long)__double_as_longlong(kTReset);
    sc->done = 0;
}

// 8 independent DFMA chains per thread, ITER iterations each.
template <int ITER>
__global__ void fp64_fma_kernel(double* sink, double a, double b) {
    double x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = threadIdx.x * 1e-9 + j;
#pragma unroll 4
    for (int it = 0; it < ITER; ++it) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == 1.2345) sink[threadIdx.x] = s;  // keeps the chains alive
}

int grid_for(long long K) {
    long long g = (K + 255) / 256;
    return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t launch_aos_to_soa(const double* s, const double* u, const double* b, Planes out,
                              long long K, int nf, cudaStream_t st) {
    aos_to_soa_kernel<<<grid_for(K), 256, 0, st>>>((const double2*)s, (const double2*)u, b, out,
                                                    K, nf);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(CPlanes in, double* s, double* u, double* b, long long K, int nf,
                              cudaStream_t st) {
    soa_to_aos_kernel<<<grid_for(K), 256, 0, st>>>(in, (double2*)s, (double2*)u, b, K, nf);
    return cudaGetLastError();
}

cudaError_t launch_funk_time(double* T, double* T_do, double* TT, int* i, cudaStream_t st) {
    funk_time_kernel<<<1, 1, 0, st>>>(T, T_do, TT, i);
    return cudaGetLastError();
}

cudaError_t launch_set_end(Scalars* sc, double t_end, cudaStream_t st) {
    set_end_kernel<<<1, 1, 0, st>>>(sc, t_end);
    return cudaGetLastError();
}

cudaError_t launch_set_time(Scalars* sc, double T_do, double TT, cudaStream_t st) {
    set_time_kernel<<<1, 1, 0, st>>>(sc, T_do, TT);
    return cudaGetLastError();
}

cudaError_t launch_batch_set_time(BatchGrid* grids, int ngrids, double T_do, double TT,
                                  cudaStream_t st) {
    batch_set_time_kernel<<<(ngrids + 127) / 128, 128, 0, st>>>(grids, ngrids, T_do, TT);
    return cudaGetLastError();
}

cudaError_t launch_batch_reset_T(BatchGrid* grids, int ngrids, cudaStream_t st) {
    batch_reset_T_kernel<<<(ngrids + 127) / 128, 128, 0, st>>>(grids, ngrids);
    return cudaGetLastError();
}

cudaError_t launch_batch_dt_commit(BatchGrid* grids, int ngrids, cudaStream_t st) {
    batch_dt_commit_kernel<<<(ngrids + 127) / 128, 128, 0, st>>>(grids, ngrids);
    return cudaGetLastError();
}

cudaError_t launch_dt_commit(Scalars* sc, cudaStream_t st) {
    dt_commit_kernel<<<1, 1, 0, st>>>(sc);
    return cudaGetLastError();
}

cudaError_t launch_reset_T(Scalars* sc, cudaStream_t st) {
    reset_T_kernel<<<1, 1, 0, st>>>(sc);
    return cudaGetLastError();
}

namespace {
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {  // splitmix64
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
// imul against the FP64 unit's multiply on n seeded operand pairs per thread, in four
// classes: any bit pattern; exponents near 1; a subnormal operand; products near the
// overflow and underflow limits.  counts: mismatches, NaN-payload differences, pairs outside
// the integer fast path, pairs checked.
__global__ void check_imul_kernel(unsigned long long* counts, unsigned long long seed, int n) {
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    unsigned long long bad = 0, nanpay = 0, slow = 0;
    for (int i = 0; i < n; ++i) {
        const unsigned long long r1 = mix64(seed + 3 * (t * n + i)), r2 = mix64(r1 + 1),
                                 r3 = mix64(r2 + 2);
        unsigned long long A = r1, B = r2;
        const unsigned long long keep = 0x800fffffffffffffULL;
        switch ((int)(r3 & 3)) {
            case 1:
                A = (A & keep) | ((1003 + (r3 >> 8) % 40) << 52);
                B = (B & keep) | ((1003 + (r3 >> 20) % 40) << 52);
                break;
            case 2:
                A = (A & keep) >> (r3 >> 58);
                break;
            case 3: {
                const unsigned long long ea = 1 + (r3 >> 8) % 2046;
                const unsigned long long eb = ((r3 >> 40) & 1) ? 3067 - ea + (r3 >> 48) % 9 - 4
                                                               : 1024 - ea + (r3 >> 48) % 61 - 30;
                A = (A & keep) | (ea << 52);
                B = (B & keep) | ((eb & 0x7ff) << 52);
                break;
            }
            default:
                break;
        }
        const double a = from_bits((long long)A), b = from_bits((long long)B);
        bool ok;
        (void)swfp::dmul_fast(a, b, ok);
        slow += !ok;
        const double s = imul(a, b);
        double h;
        asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(h) : "d"(a), "d"(b));
        if (bits(s) != bits(h)) {
            if (isnan(s) && isnan(h)) ++nanpay;
            else ++bad;
        }
    }
    atomicAdd(counts + 0, bad);
    atomicAdd(counts + 1, nanpay);
    atomicAdd(counts + 2, slow);
    atomicAdd(counts + 3, (unsigned long long)n);
}
}  // namespace

// The two-operation reciprocal and root against IEEE division and square root on seeded
// values (reciprocals of +-[2^-100, 2^100], roots sqrt(a / r) of a, r in [2^-50, 2^50]):
// the largest distance in units of the last place of the IEEE result.  The IEEE sqrt(a / r)
// rounds twice (the quotient, then the root), so it is itself within one unit of the exact
// root.  out: max ulp of rcp_2op, of sqrt_over_2op, of the three-operation sqrt_over, count.
__device__ __forceinline__ double ulp_dist(double x, double ref) {
    const long long d = bits(x) - bits(ref);
    return (double)(d < 0 ? -d : d);
}
__global__ void check_roots_kernel(unsigned long long* out, unsigned long long seed, int n) {
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    double m0 = 0, m1 = 0, m2 = 0;
    for (int i = 0; i < n; ++i) {
        const unsigned long long r1 = mix64(seed + 3 * (t * n + i)), r2 = mix64(r1 + 1),
                                 r3 = mix64(r2 + 2);
        const double x = from_bits((long long)((r1 & 0x800fffffffffffffULL) |
                                               ((923ULL + (r3 >> 8) % 201) << 52)));
        const double a = from_bits((long long)((r2 & 0x000fffffffffffffULL) |
                                               ((973ULL + (r3 >> 20) % 101) << 52)));
        const double r = from_bits((long long)((r3 & 0x000fffffffffffffULL) |
                                               ((973ULL + (r1 >> 52) % 101) << 52)));
        double q;
        asm volatile("div.rn.f64 %0, %1, %2;" : "=d"(q) : "d"(1.0), "d"(x));
        m0 = fmax(m0, ulp_dist(rcp_2op(x), q));
        double ar, sr;
        asm volatile("div.rn.f64 %0, %1, %2;" : "=d"(ar) : "d"(a), "d"(r));
        asm volatile("sqrt.rn.f64 %0, %1;" : "=d"(sr) : "d"(ar));
        m1 = fmax(m1, ulp_dist(sqrt_over_2op(a, r), sr));
        m2 = fmax(m2, ulp_dist(sqrt_over(a, r), sr));
    }
    atomicMax(out + 0, (unsigned long long)m0);
    atomicMax(out + 1, (unsigned long long)m1);
    atomicMax(out + 2, (unsigned long long)m2);
    atomicAdd(out + 3, (unsigned long long)n);
}

cudaError_t check_roots(long long count, unsigned long long seed, long long* out) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 4, threads = 256;
    const long long per = (count + (long long)blocks * threads - 1) / ((long long)blocks * threads);
    unsigned long long* c = nullptr;
    e = gd::dev_alloc(&c, 4 * sizeof(unsigned long long));
    if (e != cudaSuccess) return e;
    e = cudaMemset(c, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) {
        check_roots_kernel<<<blocks, threads>>>(c, seed, (int)(per < 1 ? 1 : per));
        e = cudaGetLastError();
    }
    unsigned long long h[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, c, sizeof h, cudaMemcpyDeviceToHost);
    gd::dev_free(c);
    for (int i = 0; i < 4; ++i) out[i] = (long long)h[i];
    return e;
}

cudaError_t check_imul(long long pairs, unsigned long long seed, long long* out) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 4, threads = 256;
    const long long per = (pairs + (long long)blocks * threads - 1) / ((long long)blocks * threads);
    unsigned long long* counts = nullptr;
    e = gd::dev_alloc(&counts, 4 * sizeof(unsigned long long));
    if (e != cudaSuccess) return e;
    e = cudaMemset(counts, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) {
        check_imul_kernel<<<blocks, threads>>>(counts, seed, (int)(per < 1 ? 1 : per));
        e = cudaGetLastError();
    }
    unsigned long long h[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, counts, sizeof h, cudaMemcpyDeviceToHost);
    gd::dev_free(counts);
    for (int i = 0; i < 4; ++i) out[i] = (long long)h[i];
    return e;
}

cudaError_t probe_fp64_peak(double* flops) {
    constexpr int ITER = 4096;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    double* sink = nullptr;
    e = gd::dev_alloc(&sink, 1024 * sizeof(double));
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 4, threads = 256;
    fp64_fma_kernel<ITER><<<blocks, threads>>>(sink, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(a);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) fp64_fma_kernel<ITER><<<blocks, threads>>>(sink, 0.999999, 1e-7);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    gd::dev_free(sink);
    if (e != cudaSuccess) return e;
    const double fmas = (double)reps * blocks * threads * 8.0 * ITER;
    *flops = 2.0 * fmas / (ms * 1e-3);
    return cudaGetLastError();
}

}  // namespace gd
