// gd_io.cu -- the reference's state file formats, produced and parsed on the GPU
// (include/gd2d.h: gd_format_text / gd_write_text / gd_parse_text / gd_read_text,
// gd_write_binary / gd_read_binary, gd_format_tecplot / gd_write_tecplot).
//
// Writers: one thread per output line formats it into its row of shared memory (gd_text.cuh,
// exact "%.6g"), the block packs its lines (block-wide scan of the lengths) and writes them
// with 16-byte stores to its own stage region; a scan of the block totals gives every
// block's file offset and a gather kernel moves the regions into the file image, which goes
// to the host in pinned chunks.  Readers: the text goes to the device, each block finds the
// token starts of a 4 KiB tile from 16-byte loads, a scan of the tile counts numbers the
// tokens, a second pass writes every token's position, and one thread per token parses it
// (correctly rounded) straight into the state planes.  Text formatting and
// parsing are byte and integer work on the integer pipes; the FP64 pipe sees about four
// operations per printed number and one multiply or divide per parsed one.
#include <cstdio>
#include <cstring>
#include <new>

#include "../../include/gd2d.h"
#include "gd_ctx.h"
#include "gd_kernels.h"
#include "gd_text.cuh"

namespace gd {

void io_free(gd_ctx* ctx) {
    IoScratch* io = ctx->io;
    if (!io) return;
    gd::dev_free(io->dev);
    gd::host_free(io->host);
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
        const cudaError_t e_ = (call);                \
        if (e_ != cudaSuccess) return gd::cuda_error(e_); \
    } while (0)

constexpr int NT = 256;
constexpr size_t kAlign = 256;
constexpr size_t kStage = 32u << 20;  // pinned staging chunk for file transfers

size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// ---- exclusive scan of uint32 (or uint64) counts into uint64 offsets ---------------------
constexpr int kScanItems = 8;
constexpr int kScanTile = NT * kScanItems;

template <int NTB = NT>
__device__ __forceinline__ unsigned long long block_exclusive(unsigned long long v,
                                                              unsigned long long* total) {
    constexpr int NW = NTB / 32;
    __shared__ unsigned long long warp_sum[NW];
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
        unsigned long long s = lane < NW ? warp_sum[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < NW; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < NW) warp_sum[lane] = s;
    }
    __syncthreads();
    const unsigned long long pre = warp > 0 ? warp_sum[warp - 1] : 0ull;
    *total = warp_sum[NW - 1];
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

__device__ int put_str(char* o, const char* s) {
    int n = 0;
    while (s[n]) {
        o[n] = s[n];
        ++n;
    }
    return n;
}

// restart text: x y rho p vx vy Bx By Bz per cell
struct RestartLine {
    Params P;
    CPlanes U;
    int nf;
    static constexpr int kSlot = 128;  // 9 numbers of <= 13 chars, 8 spaces, newline: <= 126
    __device__ int operator()(long long k, char* o) const {
        const int n = (int)(k % P.N), m = (int)(k / P.N);
        double v[9];
        // x = x_min + n * dx, y = y_min + m * dy: rounded as written (no contraction)
        v[0] = __dadd_rn(P.x0, __dmul_rn((double)n, P.dx));
        v[1] = __dadd_rn(P.y0, __dmul_rn((double)m, P.dy));
#pragma unroll
        for (int f = 0; f < 7; ++f) v[2 + f] = f < nf ? U.f[f][k] : 0.0;
        return put_values(o, v, 9);
    }
};

struct TecShape {
    int N, M, nmin, nn, mm;
    long long npts, nconn;
};

// Tecplot: line 0 the header, lines 1..npts the points, then the connectivity
struct TecLine {
    Params P;
    CPlanes U;
    int nf;
    TecShape S;
    gd_tecplot_opts O;
    static constexpr int kSlot = 256;  // 11 numbers: <= 154; the header: < 256
    __device__ int operator()(long long i, char* o) const {
        int len = 0;
        if (i == 0) {
            len += put_str(o + len,
                           nf == 7 ? "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", "
                                     "\"Vx\", \"Vy\", \"Bx\", \"By\", \"Bz\", \"Max\", \"T\", "
                                     "ZONE T = \"HP\", N = "
                                   : "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", "
                                     "\"Vx\", \"Vy\", \"Max\", \"T\", ZONE T = \"HP\", N = ");
            len += put_uint(o + len, (unsigned long long)S.npts);
            len += put_str(o + len, " , E = ");
            len += put_uint(o + len, (unsigned long long)((long long)(S.nn - 1) * (S.mm - 1)));
            len += put_str(o + len, ", F = FEPOINT, ET = quadrilateral");
            if (O.with_time) {
                len += put_str(o + len, ", SOLUTIONTIME = ");
                len += format_g6(O.time, o + len);
            }
            o[len++] = '\n';
            return len;
        }
        if (i <= S.npts) {
            const long long j = i - 1;
            const int n = (int)(j % S.nn) * S.nmin, m = (int)(j / S.nn) * S.nmin;
            const long long k = (long long)m * S.N + n;
            double v[11];
            // y = y_min + m (y_max - y_min) / (M - 1), x likewise, in the written order
            const double y = __dadd_rn(
                O.y_min, __ddiv_rn(__dmul_rn((double)m, __dsub_rn(O.y_max, O.y_min)),
                                   (double)(S.M - 1)));
            const double x = __dadd_rn(
                O.x_min, __ddiv_rn(__dmul_rn((double)n, __dsub_rn(O.x_max, O.x_min)),
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
            v[c++] = x;
            v[c++] = y;
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
            return put_values(o, v, c);
        }
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
        return len;
    }
};

// Lines per block of the formatting kernel and its shared memory: the lines (rows padded
// by 4 bytes so that the threads' byte stores fall in different banks) and the packed
// block image (16-byte aligned).
template <class Line>
struct StageShape {
    static constexpr int kSlot = Line::kSlot;
    static constexpr int kLines = kSlot <= 128 ? 128 : 64;
    static constexpr int kStride = kSlot + 4;
    static constexpr int kPackedAt = (kLines * kStride + 15) / 16 * 16;
    static constexpr int kSmem = kPackedAt + kLines * kSlot;
    static constexpr size_t kRegion = (size_t)kLines * kSlot;  // stage bytes per block
};

template <class Line>
__global__ void __launch_bounds__(StageShape<Line>::kLines)
    format_stage_kernel(Line line, long long nlines, char* stage, unsigned* block_len) {
    using SS = StageShape<Line>;
    extern __shared__ __align__(16) char sm[];
    char* mine = sm + threadIdx.x * SS::kStride;
    char* packed = sm + SS::kPackedAt;
    const long long i = (long long)blockIdx.x * SS::kLines + threadIdx.x;
    const int len = i < nlines ? line(i, mine) : 0;
    unsigned long long tot;
    const unsigned off = (unsigned)block_exclusive<SS::kLines>((unsigned long long)len, &tot);
    for (int b = 0; b < len; ++b) packed[off + b] = mine[b];
    __syncthreads();
    uint4* dst = reinterpret_cast<uint4*>(stage + (size_t)blockIdx.x * SS::kRegion);
    const uint4* src = reinterpret_cast<const uint4*>(packed);
    for (int w = threadIdx.x; w * 16 < (int)tot; w += SS::kLines) dst[w] = src[w];
    if (threadIdx.x == 0) block_len[blockIdx.x] = (unsigned)tot;
}

// The blocks' packed regions -> the file image at the scanned offsets.  A region starts
// 16-byte aligned in the stage; its destination offset is arbitrary.  The destination's
// whole aligned 16-byte words inside the block's range are assembled from two aligned source
// words with funnel shifts (R = the byte shift, uniform over the block) and stored as uint4;
// the partial words at both ends (< 16 bytes each) are written byte by byte, so no two
// blocks write the same byte.
template <int R>
__device__ __forceinline__ uint4 shifted16(const uint4* src, long long q) {
    // bytes [16 q + R, 16 q + R + 16) of src
    const uint4 a = src[q];
    if (R == 0) return a;
    const uint4 b = src[q + 1];
    const unsigned w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    constexpr int Q = R / 4, T = (R % 4) * 8;
    uint4 o;
    o.x = T ? __funnelshift_r(w[Q], w[Q + 1], T) : w[Q];
    o.y = T ? __funnelshift_r(w[Q + 1], w[Q + 2], T) : w[Q + 1];
    o.z = T ? __funnelshift_r(w[Q + 2], w[Q + 3], T) : w[Q + 2];
    o.w = T ? __funnelshift_r(w[Q + 3], w[Q + 4], T) : w[Q + 3];
    return o;
}

template <int R>
__device__ __forceinline__ void copy_words(const uint4* src, uint4* dst, long long w0, long long w1,
                                           long long src_shift_words) {
    // dst word w (w0 <= w < w1) takes source bytes [16 w - off, +16) = word (w + shift), R
    for (long long w = w0 + threadIdx.x; w < w1; w += NT) dst[w] = shifted16<R>(src, w + src_shift_words);
}

__global__ void __launch_bounds__(NT) gather_stage_kernel(const char* stage, size_t region,
                                                          const unsigned* block_len,
                                                          const unsigned long long* offs,
                                                          char* out) {
    const char* src = stage + (size_t)blockIdx.x * region;
    const unsigned long long off = offs[blockIdx.x];
    const long long len = (long long)block_len[blockIdx.x];
    // aligned destination words fully inside [off, off + len)
    const long long w0 = (long long)((off + 15) / 16), w1 = (long long)((off + len) / 16);
    const long long head = w0 < w1 ? w0 * 16 - (long long)off : len;  // bytes before word w0
    const long long tail0 = w0 < w1 ? w1 * 16 - (long long)off : len;  // first byte after w1
    for (long long b = threadIdx.x; b < head; b += NT) out[off + b] = src[b];
    for (long long b = tail0 + threadIdx.x; b < len; b += NT) out[off + b] = src[b];
    if (w0 >= w1) return;
    // source byte of destination word w: 16 w - off = 16 (w - w0) + head
    const int R = (int)(head % 16);
    const long long shift = head / 16 - w0;  // source word index = w + shift (+ R bytes)
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(out);
    switch (R) {
#define GD_COPY_CASE(r) \
    case r:             \
        copy_words<r>(s4, d4, w0, w1, shift); \
        break;
        GD_COPY_CASE(0) GD_COPY_CASE(1) GD_COPY_CASE(2) GD_COPY_CASE(3)
        GD_COPY_CASE(4) GD_COPY_CASE(5) GD_COPY_CASE(6) GD_COPY_CASE(7)
        GD_COPY_CASE(8) GD_COPY_CASE(9) GD_COPY_CASE(10) GD_COPY_CASE(11)
        GD_COPY_CASE(12) GD_COPY_CASE(13) GD_COPY_CASE(14) GD_COPY_CASE(15)
#undef GD_COPY_CASE
    }
}

// ---- readers -------------------------------------------------------------------------------

__device__ __forceinline__ bool is_ws(char c) {
    return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f';
}

// Token starts of one 4 KiB tile per block: thread t owns bytes [16 t, 16 t + 16) of the
// tile (one 16-byte load) and returns them as a 16-bit mask.  The text is padded with
// whitespace past its end, so tiles and tokens need no bounds checks.
constexpr int kTile = NT * 16;

__device__ __forceinline__ unsigned token_mask(const char* t, long long p0) {
    const uint4 v = *reinterpret_cast<const uint4*>(t + p0);
    const unsigned w[4] = {v.x, v.y, v.z, v.w};
    bool prev = p0 == 0 ? true : is_ws(t[p0 - 1]);
    unsigned m = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const bool ws = is_ws((char)(w[i >> 2] >> (8 * (i & 3))));
        if (!ws && prev) m |= 1u << i;
        prev = ws;
    }
    return m;
}

__global__ void __launch_bounds__(NT) token_count_kernel(const char* t, unsigned* tile_count) {
    const long long p0 = (long long)blockIdx.x * kTile + threadIdx.x * 16;
    unsigned long long tot;
    block_exclusive((unsigned long long)__popc(token_mask(t, p0)), &tot);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = (unsigned)tot;
}

// position of every token j < need, in text order
__global__ void __launch_bounds__(NT) token_place_kernel(const char* t,
                                                         const unsigned long long* tile_first,
                                                         long long need,
                                                         unsigned long long* tokpos) {
    const long long p0 = (long long)blockIdx.x * kTile + threadIdx.x * 16;
    unsigned m = token_mask(t, p0);
    unsigned long long tot;
    long long j = (long long)(tile_first[blockIdx.x] +
                              block_exclusive((unsigned long long)__popc(m), &tot));
    while (m && j < need) {
        const int i = __ffs(m) - 1;
        m &= m - 1;
        tokpos[j++] = (unsigned long long)(p0 + i);
    }
}

// token j -> cell j / 9, column j % 9 (x, y, rho, p, vx, vy, Bx, By, Bz)
constexpr int kMaxToken = 4096;

__global__ void __launch_bounds__(NT) token_parse_kernel(const char* t,
                                                         const unsigned long long* tokpos,
                                                         long long need, int nf, Planes out,
                                                         long long* bad) {
    const long long j = (long long)blockIdx.x * NT + threadIdx.x;
    if (j >= need) return;
    const long long p = (long long)tokpos[j];
    int len = 0;
    while (len < kMaxToken && !is_ws(t[p + len])) ++len;
    double v = 0.0;
    if (len >= kMaxToken || !parse_double(t + p, len, v)) {
        atomicMin((unsigned long long*)bad, (unsigned long long)j);
        return;
    }
    const int f = (int)(j % 9) - 2;
    if (f >= 0 && f < nf) out.f[f][j / 9] = v;
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
    gd::dev_free(io->dev);
    io->dev = nullptr;
    io->dev_cap = 0;
    IO_TRY(gd::dev_alloc(&io->dev, bytes));
    io->dev_cap = bytes;
    return GD_OK;
}

gd_status ensure_host(gd_ctx* ctx, size_t bytes) {
    gd::IoScratch* io = ctx->io;
    if (io->host_cap >= bytes) return GD_OK;
    gd::host_free(io->host);
    io->host = nullptr;
    io->host_cap = 0;
    IO_TRY(gd::host_alloc(&io->host, bytes));
    io->host_cap = bytes;
    return GD_OK;
}

// Formats nlines lines with `line` and packs them; on return the file image (len bytes) is
// at *image on the device.
template <class Line>
gd_status format_lines(gd_ctx* ctx, const Line& line, long long nlines, char** image, size_t* len,
                       cudaStream_t st) {
    using SS = StageShape<Line>;
    const long long nb = (nlines + SS::kLines - 1) / SS::kLines;
    const size_t b_stage = up((size_t)nb * SS::kRegion);
    const size_t b_lens = up((size_t)nb * sizeof(unsigned));
    const size_t b_offs = up((size_t)nb * sizeof(unsigned long long));
    const size_t b_scan = up(scan_scratch_bytes(nb));
    const size_t b_img = up((size_t)nb * SS::kRegion);  // upper bound of the image
    gd_status r = ensure_dev(ctx, b_stage + b_lens + b_offs + b_scan + b_img);
    if (r != GD_OK) return r;
    char* base = ctx->io->dev;
    char* stage = base;
    unsigned* blen = (unsigned*)(base + b_stage);
    unsigned long long* offs = (unsigned long long*)(base + b_stage + b_lens);
    unsigned long long* scr = (unsigned long long*)(base + b_stage + b_lens + b_offs);
    char* img = base + b_stage + b_lens + b_offs + b_scan;
    format_stage_kernel<Line><<<(unsigned)nb, SS::kLines, SS::kSmem, st>>>(line, nlines, stage, blen);
    IO_TRY(cudaGetLastError());
    IO_TRY(exclusive_scan<unsigned>(blen, nb, offs, scr, st));
    unsigned long long last_off = 0;
    unsigned last_len = 0;
    IO_TRY(cudaMemcpyAsync(&last_off, offs + nb - 1, sizeof(last_off), cudaMemcpyDeviceToHost, st));
    IO_TRY(cudaMemcpyAsync(&last_len, blen + nb - 1, sizeof(last_len), cudaMemcpyDeviceToHost, st));
    gather_stage_kernel<<<(unsigned)nb, NT, 0, st>>>(stage, SS::kRegion, blen, offs, img);
    IO_TRY(cudaGetLastError());
    IO_TRY(cudaStreamSynchronize(st));
    ctx->launches += 3;
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
        cudaError_t e = cudaMemcpyAsync(ctx->io->host, img + o, c, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            std::fclose(f);
            return gd::cuda_error(e);
        }
        if (std::fwrite(ctx->io->host, 1, c, f) != c) {
            std::fclose(f);
            return GD_ERR_INVALID_ARG;
        }
    }
    return std::fclose(f) == 0 ? GD_OK : GD_ERR_INVALID_ARG;
}

gd_status format_text_image(gd_ctx* ctx, char** img, size_t* n, cudaStream_t st) {
    const RestartLine line{ctx->P, gd_ctx::cplanes(ctx->planes(ctx->cur)), ctx->nf};
    return format_lines(ctx, line, ctx->K, img, n, st);
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
    const TecLine line{ctx->P, gd_ctx::cplanes(ctx->planes(ctx->cur)), ctx->nf, S, *opts};
    return format_lines(ctx, line, 1 + S.npts + S.nconn, img, n, st);
}

// text buffer on the device: L bytes and a whitespace pad of one tile (parse_device_text
// writes the pad)
size_t text_bytes(long long L) { return up((size_t)L + kTile + 16); }

// text on the device (L bytes at dtext, buffer of text_bytes(L)) -> state
gd_status parse_device_text(gd_ctx* ctx, char* dtext, long long L, char* work, cudaStream_t st) {
    const long long K = ctx->K;
    const long long need = 9 * K;
    if (L <= 0) return GD_ERR_INVALID_ARG;
    const long long ntiles = (L + kTile - 1) / kTile;
    unsigned* tile_count = (unsigned*)work;
    char* w = work + up((size_t)ntiles * sizeof(unsigned));
    unsigned long long* tile_first = (unsigned long long*)w;
    w += up((size_t)ntiles * 8);
    unsigned long long* scr = (unsigned long long*)w;
    w += up(scan_scratch_bytes(ntiles));
    unsigned long long* tokpos = (unsigned long long*)w;
    w += up((size_t)need * 8);
    long long* bad = (long long*)w;
    IO_TRY(cudaMemsetAsync(dtext + L, ' ', text_bytes(L) - (size_t)L, st));
    token_count_kernel<<<(unsigned)ntiles, NT, 0, st>>>(dtext, tile_count);
    IO_TRY(cudaGetLastError());
    IO_TRY(exclusive_scan<unsigned>(tile_count, ntiles, tile_first, scr, st));
    unsigned long long last_first = 0;
    unsigned last_count = 0;
    IO_TRY(cudaMemcpyAsync(&last_first, tile_first + ntiles - 1, 8, cudaMemcpyDeviceToHost, st));
    IO_TRY(cudaMemcpyAsync(&last_count, tile_count + ntiles - 1, 4, cudaMemcpyDeviceToHost, st));
    const long long none = 0x7fffffffffffffffLL;
    IO_TRY(cudaMemcpyAsync(bad, &none, sizeof(none), cudaMemcpyHostToDevice, st));
    IO_TRY(cudaStreamSynchronize(st));
    ctx->launches += 2;
    if ((long long)(last_first + last_count) < need) return GD_ERR_INVALID_ARG;  // too short
    token_place_kernel<<<(unsigned)ntiles, NT, 0, st>>>(dtext, tile_first, need, tokpos);
    IO_TRY(cudaGetLastError());
    // parsed into the other plane set, which every cell's nf fields overwrite; the context
    // switches to it only when every token parsed, so a failed parse leaves the state as it was
    token_parse_kernel<<<blocks(need), NT, 0, st>>>(dtext, tokpos, need, ctx->nf,
                                                    ctx->planes(1 - ctx->cur), bad);
    IO_TRY(cudaGetLastError());
    ctx->launches += 2;
    long long first_bad = none;
    IO_TRY(cudaMemcpyAsync(&first_bad, bad, sizeof(first_bad), cudaMemcpyDeviceToHost, st));
    IO_TRY(cudaStreamSynchronize(st));
    if (first_bad != none) return GD_ERR_INVALID_ARG;
    ctx->cur = 1 - ctx->cur;
    return GD_OK;
}

size_t parse_work_bytes(long long L, long long K) {
    const long long ntiles = (L + kTile - 1) / kTile;
    return up((size_t)ntiles * sizeof(unsigned)) + up((size_t)ntiles * 8) +
           up(scan_scratch_bytes(ntiles)) + up((size_t)9 * K * 8) + kAlign;
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
    const size_t b_text = text_bytes((long long)len);
    gd_status r = ensure_dev(ctx, b_text + parse_work_bytes((long long)len, ctx->K));
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
    const size_t b_text = text_bytes(L);
    gd_status r = ensure_dev(ctx, b_text + parse_work_bytes(L, ctx->K));
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
