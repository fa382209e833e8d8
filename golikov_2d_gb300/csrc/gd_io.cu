// gd_io.cu -- the reference's state file formats, produced and parsed on the GPU
// (include/gd2d.h: gd_format_text / gd_write_text / gd_parse_text / gd_read_text,
// gd_write_binary / gd_read_binary, gd_format_tecplot / gd_write_tecplot).
//
// Writers: one thread per output line formats it into a fixed-width slot (gd_text.cuh,
// exact "%.6g"), an exclusive scan of the line lengths gives every line's offset, a
// compaction kernel packs the slots into the file image, and the image goes to the host
// in pinned chunks.  Readers: the text goes to the device, one thread per 1 KiB chunk
// counts token starts, a scan numbers the tokens, and the same threads parse their tokens
// (correctly rounded) straight into the state planes.  Text formatting and parsing are
// byte and integer work on the integer pipes; the FP64 pipe only sees the fast path's one
// multiply or divide per number.
#include <cstdio>
#include <cstring>
#include <new>

#include "../../include/gd2d.h"
#include "gd_ctx.h"
#include "gd_text.cuh"

namespace gd {

void io_free(gd_ctx* ctx) {
    IoScratch* io = ctx->io;
    if (!io) return;
    cudaFree(io->dev);
    cudaFreeHost(io->host);
    delete io;
    ctx->io = nullptr;
}

}  // namespace gd

namespace {

using gd::text::format_g6;
using gd::text::parse_double;
using gd::text::put_uint;

#define IO_TRY(call)                                  \
    do {                                              \
        if ((call) != cudaSuccess) return GD_ERR_CUDA; \
    } while (0)

constexpr int NT = 256;
constexpr size_t kAlign = 256;
constexpr int kTextSlot = 128;     // 9 numbers of <= 13 chars, 8 spaces, newline: <= 126
constexpr int kTecSlot = 256;      // 11 numbers: <= 154; the header: < 256
constexpr int kChunk = 1024;       // bytes of text per reader thread
constexpr size_t kStage = 32u << 20;  // pinned staging chunk for file transfers

size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// ---- exclusive scan of uint32 (or uint64) counts into uint64 offsets ---------------------
constexpr int kScanItems = 8;
constexpr int kScanTile = NT * kScanItems;

__device__ __forceinline__ unsigned long long block_exclusive(unsigned long long v,
                                                              unsigned long long* total) {
    __shared__ unsigned long long warp_sum[NT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long s = lane < NT / 32 ? warp_sum[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < NT / 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < NT / 32) warp_sum[lane] = s;
    }
    __syncthreads();
    const unsigned long long pre = warp > 0 ? warp_sum[warp - 1] : 0ull;
    *total = warp_sum[NT / 32 - 1];
    __syncthreads();
    return pre + x - v;
}

template <class T>
__global__ void __launch_bounds__(NT) scan_reduce_kernel(const T* in, long long n,
                                                         unsigned long long* bsum) {
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += (unsigned long long)in[base + i];
    unsigned long long tot;
    block_exclusive(s, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

template <class T>
__global__ void __launch_bounds__(NT) scan_down_kernel(const T* in, long long n,
                                                       const unsigned long long* bpre,
                                                       unsigned long long* out) {
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned long long v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? (unsigned long long)in[base + i] : 0ull;
        s += v[i];
    }
    unsigned long long tot;
    unsigned long long run = block_exclusive(s, &tot) + (bpre ? bpre[blockIdx.x] : 0ull);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

// out[i] = sum of in[0..i); scratch holds scan_scratch_bytes(n)
template <class T>
cudaError_t exclusive_scan(const T* in, long long n, unsigned long long* out,
                           unsigned long long* scratch, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const long long nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        scan_down_kernel<T><<<1, NT, 0, st>>>(in, n, nullptr, out);
        return cudaGetLastError();
    }
    unsigned long long* bsum = scratch;
    unsigned long long* bpre = scratch + nb;  // scan of bsum; deeper levels follow
    scan_reduce_kernel<T><<<(unsigned)nb, NT, 0, st>>>(in, n, bsum);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the partial sums' own scan writes into bpre, using the space after it
    e = exclusive_scan<unsigned long long>(bsum, nb, bpre, bpre + nb, st);
    if (e != cudaSuccess) return e;
    scan_down_kernel<T><<<(unsigned)nb, NT, 0, st>>>(in, n, bpre, out);
    return cudaGetLastError();
}

size_t scan_scratch_bytes(long long n) {
    // exclusive_scan places bsum (nb) and bpre (nb) per level, recursively
    size_t total = 0;
    long long m = n;
    while (m > kScanTile) {
        m = (m + kScanTile - 1) / kScanTile;
        total += 2 * (size_t)m;
    }
    return (total + 2) * sizeof(unsigned long long);
}

// ---- writers: line formatting --------------------------------------------------------------

__device__ __forceinline__ int put_values(char* o, const double* v, int nv) {
    int len = 0;
    for (int i = 0; i < nv; ++i) {
        if (i) o[len++] = ' ';
        len += format_g6(v[i], o + len);
    }
    o[len++] = '\n';
    return len;
}

// restart text: x y rho p vx vy Bx By Bz per cell
__global__ void __launch_bounds__(NT) restart_lines_kernel(Params P, CPlanes U, int nf,
                                                           char* slots, unsigned* lens) {
    const long long K = (long long)P.N * P.M;
    const long long k = (long long)blockIdx.x * NT + threadIdx.x;
    if (k >= K) return;
    const int n = (int)(k % P.N), m = (int)(k / P.N);
    double v[9];
    // x = x_min + n * dx, y = y_min + m * dy: rounded as written (no contraction)
    v[0] = __dadd_rn(P.x0, __dmul_rn((double)n, P.dx));
    v[1] = __dadd_rn(P.y0, __dmul_rn((double)m, P.dy));
#pragma unroll
    for (int f = 0; f < 7; ++f) v[2 + f] = f < nf ? U.f[f][k] : 0.0;
    lens[k] = (unsigned)put_values(slots + (size_t)k * kTextSlot, v, 9);
}

struct TecShape {
    int N, M, nmin, nn, mm;
    long long npts, nconn;
};

__device__ int put_str(char* o, const char* s) {
    int n = 0;
    while (s[n]) {
        o[n] = s[n];
        ++n;
    }
    return n;
}

// Tecplot: line 0 the header, lines 1..npts the points, then the connectivity
__global__ void __launch_bounds__(NT) tecplot_lines_kernel(Params P, CPlanes U, int nf,
                                                           TecShape S, gd_tecplot_opts O,
                                                           char* slots, unsigned* lens) {
    const long long i = (long long)blockIdx.x * NT + threadIdx.x;
    const long long nlines = 1 + S.npts + S.nconn;
    if (i >= nlines) return;
    char* o = slots + (size_t)i * kTecSlot;
    int len = 0;
    if (i == 0) {
        len += put_str(o + len,
                       nf == 7 ? "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", \"Vx\", "
                                 "\"Vy\", \"Bx\", \"By\", \"Bz\", \"Max\", \"T\", ZONE T = \"HP\", "
                                 "N = "
                               : "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", \"Vx\", "
                                 "\"Vy\", \"Max\", \"T\", ZONE T = \"HP\", N = ");
        len += put_uint(o + len, (unsigned long long)S.npts);
        len += put_str(o + len, " , E = ");
        len += put_uint(o + len, (unsigned long long)((long long)(S.nn - 1) * (S.mm - 1)));
        len += put_str(o + len, ", F = FEPOINT, ET = quadrilateral");
        if (O.with_time) {
            len += put_str(o + len, ", SOLUTIONTIME = ");
            len += format_g6(O.time, o + len);
        }
        o[len++] = '\n';
    } else if (i <= S.npts) {
        const long long j = i - 1;
        const int n = (int)(j % S.nn) * S.nmin, m = (int)(j / S.nn) * S.nmin;
        const long long k = (long long)m * S.N + n;
        double v[11];
        // y = y_min + m (y_max - y_min) / (M - 1), x likewise, in the written order
        v[1] = __dadd_rn(O.y_min, __ddiv_rn(__dmul_rn((double)m, __dsub_rn(O.y_max, O.y_min)),
                                            (double)(S.M - 1)));
        v[0] = __dadd_rn(O.x_min, __ddiv_rn(__dmul_rn((double)n, __dsub_rn(O.x_max, O.x_min)),
                                            (double)(S.N - 1)));
        const double r = U.f[0][k], p = U.f[1][k], vx = U.f[2][k], vy = U.f[3][k];
        double Max = 0.0, T = 0.0;
        if (r > 0.0) {
            // sqrt((vx vx + vy vy) / (gamma p / rho)), p / rho: rounded as written
            const double a = __dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy));
            Max = __dsqrt_rn(__ddiv_rn(a, __ddiv_rn(__dmul_rn(P.gamma, p), r)));
            T = __ddiv_rn(p, r);
        }
        int c = 0;
        v[c++] = v[0];
        v[c++] = v[1];
        v[c++] = r;
        v[c++] = p;
        v[c++] = vx;
        v[c++] = vy;
        if (nf == 7) {
            v[c++] = U.f[4][k];
            v[c++] = U.f[5][k];
            v[c++] = U.f[6][k];
        }
        v[c++] = Max;
        v[c++] = T;
        len = put_values(o, v, c);
    } else {
        const long long q = i - 1 - S.npts;
        const long long n = q % (S.nn - 1), m = q / (S.nn - 1);
        const long long a = m * S.nn + n;
        const unsigned long long c4[4] = {(unsigned long long)(a + 1), (unsigned long long)(a + 2),
                                          (unsigned long long)(a + S.nn + 2),
                                          (unsigned long long)(a + S.nn + 1)};
        for (int t = 0; t < 4; ++t) {
            if (t) o[len++] = ' ';
            len += put_uint(o + len, c4[t]);
        }
        o[len++] = '\n';
    }
    lens[i] = (unsigned)len;
}

// pack slot lines into the file image; a warp copies one line, 8 bytes a lane where the
// line allows
__global__ void __launch_bounds__(NT) compact_kernel(const char* slots, int slot, long long nlines,
                                                     const unsigned* lens,
                                                     const unsigned long long* offs, char* out) {
    const long long line = ((long long)blockIdx.x * NT + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (line >= nlines) return;
    const char* src = slots + (size_t)line * slot;
    char* dst = out + offs[line];
    const int len = (int)lens[line];
    for (int b = lane; b < len; b += 32) dst[b] = src[b];
}

// ---- readers -------------------------------------------------------------------------------

__device__ __forceinline__ bool is_ws(char c) {
    return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f';
}

__global__ void __launch_bounds__(NT) count_tokens_kernel(const char* t, long long L,
                                                          long long nchunks, unsigned* counts) {
    const long long c = (long long)blockIdx.x * NT + threadIdx.x;
    if (c >= nchunks) return;
    const long long b0 = c * kChunk, b1 = b0 + kChunk < L ? b0 + kChunk : L;
    unsigned n = 0;
    bool prev_ws = b0 == 0 ? true : is_ws(t[b0 - 1]);
    for (long long p = b0; p < b1; ++p) {
        const bool w = is_ws(t[p]);
        if (!w && prev_ws) ++n;
        prev_ws = w;
    }
    counts[c] = n;
}

// token j -> cell j / 9, column j % 9 (x, y, rho, p, vx, vy, Bx, By, Bz)
__global__ void __launch_bounds__(NT) parse_tokens_kernel(const char* t, long long L,
                                                          long long nchunks,
                                                          const unsigned long long* first,
                                                          long long ntok_needed, int nf,
                                                          Planes out, long long* bad) {
    const long long c = (long long)blockIdx.x * NT + threadIdx.x;
    if (c >= nchunks) return;
    const long long b0 = c * kChunk, b1 = b0 + kChunk < L ? b0 + kChunk : L;
    long long j = (long long)first[c];
    if (j >= ntok_needed) return;
    bool prev_ws = b0 == 0 ? true : is_ws(t[b0 - 1]);
    for (long long p = b0; p < b1 && j < ntok_needed; ++p) {
        const bool w = is_ws(t[p]);
        if (!w && prev_ws) {
            long long e = p;
            while (e < L && !is_ws(t[e])) ++e;
            double v = 0.0;
            const bool ok = (e - p) < 4096 && parse_double(t + p, (int)(e - p), v);
            if (!ok) {
                atomicMin((unsigned long long*)bad, (unsigned long long)j);
            } else {
                const int col = (int)(j % 9);
                const long long k = j / 9;
                const int f = col - 2;
                if (f >= 0 && f < nf) out.f[f][k] = v;
            }
            ++j;
        }
        prev_ws = w;
    }
}

// binary dump: x, y, rho, p, vx, vy, Bz per cell
__global__ void __launch_bounds__(NT) pack_binary_kernel(Params P, CPlanes U, int nf, double* o) {
    const long long K = (long long)P.N * P.M;
    const long long k = (long long)blockIdx.x * NT + threadIdx.x;
    if (k >= K) return;
    const int n = (int)(k % P.N), m = (int)(k / P.N);
    double* r = o + (size_t)k * 7;
    r[0] = __dadd_rn(P.x0, __dmul_rn((double)n, P.dx));
    r[1] = __dadd_rn(P.y0, __dmul_rn((double)m, P.dy));
    r[2] = U.f[0][k];
    r[3] = U.f[1][k];
    r[4] = U.f[2][k];
    r[5] = U.f[3][k];
    r[6] = nf == 7 ? U.f[6][k] : 0.0;
}

__global__ void __launch_bounds__(NT) unpack_binary_kernel(long long K, int nf, const double* in,
                                                           Planes U) {
    const long long k = (long long)blockIdx.x * NT + threadIdx.x;
    if (k >= K) return;
    const double* r = in + (size_t)k * 7;
    U.f[0][k] = r[2];
    U.f[1][k] = r[3];
    U.f[2][k] = r[4];
    U.f[3][k] = r[5];
    if (nf == 7) {
        U.f[4][k] = 0.0;
        U.f[5][k] = 0.0;
        U.f[6][k] = r[6];
    }
}

// ---- host side -----------------------------------------------------------------------------

unsigned blocks(long long n, int per = NT) { return (unsigned)((n + per - 1) / per); }

gd_status ensure_dev(gd_ctx* ctx, size_t bytes) {
    if (!ctx->io) {
        ctx->io = new (std::nothrow) gd::IoScratch();
        if (!ctx->io) return GD_ERR_INVALID_ARG;
    }
    gd::IoScratch* io = ctx->io;
    if (io->dev_cap >= bytes) return GD_OK;
    cudaFree(io->dev);
    io->dev = nullptr;
    io->dev_cap = 0;
    IO_TRY(cudaMalloc(&io->dev, bytes));
    io->dev_cap = bytes;
    return GD_OK;
}

gd_status ensure_host(gd_ctx* ctx, size_t bytes) {
    gd::IoScratch* io = ctx->io;
    if (io->host_cap >= bytes) return GD_OK;
    cudaFreeHost(io->host);
    io->host = nullptr;
    io->host_cap = 0;
    IO_TRY(cudaMallocHost(&io->host, bytes));
    io->host_cap = bytes;
    return GD_OK;
}

// Formats nlines lines of `slot` bytes with `launch` and packs them; on return the image
// (len bytes) is at *image on the device.
template <class Launch>
gd_status format_lines(gd_ctx* ctx, long long nlines, int slot, Launch launch, char** image,
                       size_t* len, cudaStream_t st) {
    const size_t b_slots = up((size_t)nlines * slot);
    const size_t b_lens = up((size_t)nlines * sizeof(unsigned));
    const size_t b_offs = up((size_t)nlines * sizeof(unsigned long long));
    const size_t b_scan = up(scan_scratch_bytes(nlines));
    const size_t b_img = up((size_t)nlines * slot);  // upper bound of the image
    gd_status r = ensure_dev(ctx, b_slots + b_lens + b_offs + b_scan + b_img);
    if (r != GD_OK) return r;
    char* base = ctx->io->dev;
    char* slots = base;
    unsigned* lens = (unsigned*)(base + b_slots);
    unsigned long long* offs = (unsigned long long*)(base + b_slots + b_lens);
    unsigned long long* scr = (unsigned long long*)(base + b_slots + b_lens + b_offs);
    char* img = base + b_slots + b_lens + b_offs + b_scan;
    IO_TRY(launch(slots, lens));
    ctx->launches += 1;
    IO_TRY(exclusive_scan<unsigned>(lens, nlines, offs, scr, st));
    ctx->launches += 1;
    unsigned long long last_off = 0;
    unsigned last_len = 0;
    IO_TRY(cudaMemcpyAsync(&last_off, offs + nlines - 1, sizeof(last_off), cudaMemcpyDeviceToHost,
                           st));
    IO_TRY(cudaMemcpyAsync(&last_len, lens + nlines - 1, sizeof(last_len), cudaMemcpyDeviceToHost,
                           st));
    IO_TRY(cudaStreamSynchronize(st));
    compact_kernel<<<blocks(nlines * 32), NT, 0, st>>>(slots, slot, nlines, lens, offs, img);
    IO_TRY(cudaGetLastError());
    ctx->launches += 1;
    *image = img;
    *len = (size_t)last_off + last_len;
    return GD_OK;
}

// device image -> caller memory (or only its length)
gd_status deliver(const char* img, size_t n, char* buf, size_t cap, size_t* len,
                  cudaStream_t st) {
    *len = n;
    if (!buf) {
        IO_TRY(cudaStreamSynchronize(st));
        return GD_OK;
    }
    if (cap < n) return GD_ERR_INVALID_ARG;
    IO_TRY(cudaMemcpyAsync(buf, img, n, cudaMemcpyDeviceToHost, st));
    IO_TRY(cudaStreamSynchronize(st));
    return GD_OK;
}

// device image -> file, through pinned chunks
gd_status to_file(gd_ctx* ctx, const char* img, size_t n, const char* path, cudaStream_t st) {
    gd_status r = ensure_host(ctx, kStage);
    if (r != GD_OK) return r;
    FILE* f = std::fopen(path, "wb");
    if (!f) return GD_ERR_INVALID_ARG;
    for (size_t o = 0; o < n; o += kStage) {
        const size_t c = n - o < kStage ? n - o : kStage;
        if (cudaMemcpyAsync(ctx->io->host, img + o, c, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            std::fclose(f);
            return GD_ERR_CUDA;
        }
        if (std::fwrite(ctx->io->host, 1, c, f) != c) {
            std::fclose(f);
            return GD_ERR_INVALID_ARG;
        }
    }
    return std::fclose(f) == 0 ? GD_OK : GD_ERR_INVALID_ARG;
}

gd_status format_text_image(gd_ctx* ctx, char** img, size_t* n, cudaStream_t st) {
    const Params P = ctx->P;
    const CPlanes U = gd_ctx::cplanes(ctx->planes(ctx->cur));
    const int nf = ctx->nf;
    const long long K = ctx->K;
    return format_lines(
        ctx, K, kTextSlot,
        [&](char* slots, unsigned* lens) {
            restart_lines_kernel<<<blocks(K), NT, 0, st>>>(P, U, nf, slots, lens);
            return cudaGetLastError();
        },
        img, n, st);
}

bool tec_shape(const gd_ctx* ctx, const gd_tecplot_opts* o, TecShape* S) {
    if (!o || o->nmin < 1) return false;
    S->N = ctx->cfg.N;
    S->M = ctx->cfg.M;
    S->nmin = o->nmin;
    S->nn = (S->N + o->nmin - 1) / o->nmin;
    S->mm = (S->M + o->nmin - 1) / o->nmin;
    S->npts = (long long)S->nn * S->mm;
    S->nconn = (S->nn > 1 && S->mm > 1) ? (long long)(S->nn - 1) * (S->mm - 1) : 0;
    return true;
}

gd_status format_tecplot_image(gd_ctx* ctx, const gd_tecplot_opts* opts, char** img, size_t* n,
                               cudaStream_t st) {
    TecShape S;
    if (!tec_shape(ctx, opts, &S)) return GD_ERR_INVALID_ARG;
    const Params P = ctx->P;
    const CPlanes U = gd_ctx::cplanes(ctx->planes(ctx->cur));
    const int nf = ctx->nf;
    const gd_tecplot_opts O = *opts;
    const long long nlines = 1 + S.npts + S.nconn;
    return format_lines(
        ctx, nlines, kTecSlot,
        [&](char* slots, unsigned* lens) {
            tecplot_lines_kernel<<<blocks(nlines), NT, 0, st>>>(P, U, nf, S, O, slots, lens);
            return cudaGetLastError();
        },
        img, n, st);
}

// text on the device (L bytes at dtext) -> state
gd_status parse_device_text(gd_ctx* ctx, const char* dtext, long long L, char* work,
                            cudaStream_t st) {
    const long long K = ctx->K;
    const long long need = 9 * K;
    const long long nchunks = (L + kChunk - 1) / kChunk;
    unsigned* counts = (unsigned*)work;
    unsigned long long* first =
        (unsigned long long*)(work + up((size_t)nchunks * sizeof(unsigned)));
    unsigned long long* scr = first + up((size_t)nchunks * sizeof(unsigned long long)) / 8;
    long long* bad = (long long*)(scr + up(scan_scratch_bytes(nchunks)) / 8);
    if (nchunks == 0) return GD_ERR_INVALID_ARG;
    count_tokens_kernel<<<blocks(nchunks), NT, 0, st>>>(dtext, L, nchunks, counts);
    IO_TRY(cudaGetLastError());
    IO_TRY(exclusive_scan<unsigned>(counts, nchunks, first, scr, st));
    unsigned long long last_first = 0;
    unsigned last_count = 0;
    IO_TRY(cudaMemcpyAsync(&last_first, first + nchunks - 1, 8, cudaMemcpyDeviceToHost, st));
    IO_TRY(cudaMemcpyAsync(&last_count, counts + nchunks - 1, 4, cudaMemcpyDeviceToHost, st));
    const long long none = 0x7fffffffffffffffLL;
    IO_TRY(cudaMemcpyAsync(bad, &none, sizeof(none), cudaMemcpyHostToDevice, st));
    IO_TRY(cudaStreamSynchronize(st));
    ctx->launches += 2;
    if ((long long)(last_first + last_count) < need) return GD_ERR_INVALID_ARG;  // too short
    parse_tokens_kernel<<<blocks(nchunks), NT, 0, st>>>(dtext, L, nchunks, first, need, ctx->nf,
                                                        ctx->planes(ctx->cur), bad);
    IO_TRY(cudaGetLastError());
    ctx->launches += 1;
    long long first_bad = none;
    IO_TRY(cudaMemcpyAsync(&first_bad, bad, sizeof(first_bad), cudaMemcpyDeviceToHost, st));
    IO_TRY(cudaStreamSynchronize(st));
    return first_bad == none ? GD_OK : GD_ERR_INVALID_ARG;
}

size_t parse_work_bytes(long long L) {
    const long long nchunks = (L + kChunk - 1) / kChunk;
    return up((size_t)nchunks * sizeof(unsigned)) + up((size_t)nchunks * 8) +
           up(scan_scratch_bytes(nchunks)) + kAlign;
}

}  // namespace

extern "C" {

gd_status gd_format_text(gd_ctx* ctx, char* buf, size_t cap, size_t* len, gd_stream stream) {
    if (!ctx || !len) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    char* img = nullptr;
    size_t n = 0;
    gd_status r = format_text_image(ctx, &img, &n, st);
    if (r != GD_OK) return r;
    return deliver(img, n, buf, cap, len, st);
}

gd_status gd_write_text(gd_ctx* ctx, const char* path, gd_stream stream) {
    if (!ctx || !path) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    char* img = nullptr;
    size_t n = 0;
    gd_status r = format_text_image(ctx, &img, &n, st);
    if (r != GD_OK) return r;
    return to_file(ctx, img, n, path, st);
}

gd_status gd_format_tecplot(gd_ctx* ctx, const gd_tecplot_opts* opts, char* buf, size_t cap,
                            size_t* len, gd_stream stream) {
    if (!ctx || !opts || !len) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    char* img = nullptr;
    size_t n = 0;
    gd_status r = format_tecplot_image(ctx, opts, &img, &n, st);
    if (r != GD_OK) return r;
    return deliver(img, n, buf, cap, len, st);
}

gd_status gd_write_tecplot(gd_ctx* ctx, const char* path, const gd_tecplot_opts* opts,
                           gd_stream stream) {
    if (!ctx || !path || !opts) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    char* img = nullptr;
    size_t n = 0;
    gd_status r = format_tecplot_image(ctx, opts, &img, &n, st);
    if (r != GD_OK) return r;
    return to_file(ctx, img, n, path, st);
}

gd_status gd_parse_text(gd_ctx* ctx, const char* text, size_t len, gd_stream stream) {
    if (!ctx || (!text && len)) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t b_text = up(len + 1);
    gd_status r = ensure_dev(ctx, b_text + parse_work_bytes((long long)len));
    if (r != GD_OK) return r;
    char* dtext = ctx->io->dev;
    if (len) IO_TRY(cudaMemcpyAsync(dtext, text, len, cudaMemcpyHostToDevice, st));
    return parse_device_text(ctx, dtext, (long long)len, dtext + b_text, st);
}

gd_status gd_read_text(gd_ctx* ctx, const char* path, gd_stream stream) {
    if (!ctx || !path) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    FILE* f = std::fopen(path, "rb");
    if (!f) return GD_ERR_INVALID_ARG;
    std::fseek(f, 0, SEEK_END);
    const long long L = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (L < 0) {
        std::fclose(f);
        return GD_ERR_INVALID_ARG;
    }
    const size_t b_text = up((size_t)L + 1);
    gd_status r = ensure_dev(ctx, b_text + parse_work_bytes(L));
    if (r == GD_OK) r = ensure_host(ctx, kStage);
    if (r != GD_OK) {
        std::fclose(f);
        return r;
    }
    char* dtext = ctx->io->dev;
    for (long long o = 0; o < L; o += (long long)kStage) {
        const size_t c = (size_t)(L - o) < kStage ? (size_t)(L - o) : kStage;
        if (std::fread(ctx->io->host, 1, c, f) != c ||
            cudaMemcpyAsync(dtext + o, ctx->io->host, c, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            std::fclose(f);
            return GD_ERR_INVALID_ARG;
        }
    }
    std::fclose(f);
    return parse_device_text(ctx, dtext, L, dtext + b_text, st);
}

gd_status gd_write_binary(gd_ctx* ctx, const char* path, gd_stream stream) {
    if (!ctx || !path) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)ctx->K * 7 * sizeof(double);
    gd_status r = ensure_dev(ctx, up(n));
    if (r != GD_OK) return r;
    pack_binary_kernel<<<blocks(ctx->K), NT, 0, st>>>(
        ctx->P, gd_ctx::cplanes(ctx->planes(ctx->cur)), ctx->nf, (double*)ctx->io->dev);
    IO_TRY(cudaGetLastError());
    ctx->launches += 1;
    return to_file(ctx, ctx->io->dev, n, path, st);
}

gd_status gd_read_binary(gd_ctx* ctx, const char* path, gd_stream stream) {
    if (!ctx || !path) return GD_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)ctx->K * 7 * sizeof(double);
    FILE* f = std::fopen(path, "rb");
    if (!f) return GD_ERR_INVALID_ARG;
    gd_status r = ensure_dev(ctx, up(n));
    if (r == GD_OK) r = ensure_host(ctx, kStage);
    if (r != GD_OK) {
        std::fclose(f);
        return r;
    }
    for (size_t o = 0; o < n; o += kStage) {
        const size_t c = n - o < kStage ? n - o : kStage;
        if (std::fread(ctx->io->host, 1, c, f) != c ||
            cudaMemcpyAsync(ctx->io->dev + o, ctx->io->host, c, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            std::fclose(f);
            return GD_ERR_INVALID_ARG;
        }
    }
    std::fclose(f);
    unpack_binary_kernel<<<blocks(ctx->K), NT, 0, st>>>(ctx->K, ctx->nf, (const double*)ctx->io->dev,
                                                        ctx->planes(ctx->cur));
    IO_TRY(cudaGetLastError());
    ctx->launches += 1;
    IO_TRY(cudaStreamSynchronize(st));
    return GD_OK;
}

}  // extern "C"
