// gd_hancock.cu -- the MUSCL-Hancock step of Kernel_GKR (kernel.cu:2663-3284) for
// GD_MODE_PARITY: one thread per cell, each cell computed as the reference computes it
// (gd_hancock_cell.cuh).  This translation unit is compiled with --fmad=false, so with IEEE
// division and square root its results are bit-identical to the reference's.
#include "gd_hancock_cell.cuh"
#include "gd_internal.cuh"
#include "gd_kernels.h"

namespace gd {
namespace {

constexpr int HTX = 32, HTY = 4, HNT = HTX * HTY;

template <bool VYP>
__global__ void __launch_bounds__(HNT) hancock_parity_kernel(Params P, CPlanes in, Planes out,
                                                             const double* __restrict__ T_do_ptr,
                                                             unsigned long long* T_bits,
                                                             Scalars* rot, Scalars* ctr,
                                                             int dt_only) {
    const int n = blockIdx.x * HTX + (threadIdx.x % HTX);
    const int m = (blockIdx.y + P.tile_row0) * HTY + (threadIdx.x / HTX);
    double tmin = kCellTmin0;
    bool active = false;
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    if (n < P.N && m < P.M) {
        const long long k = (long long)m * P.N + n;
        const double y = hancock_y(P, m);
        if (hancock_frozen(P, n, y)) {
            if (!dt_only)
                for (int f = 0; f < 7; ++f) store_f(out, f, k, load_f(in, f, k));
        } else {
            active = true;
            double res[7];
            tmin = hancock_cell<VYP>(P, in, n, m, y, *T_do_ptr, res, nfl_r, nfl_p);
            if (!dt_only) {
                for (int f = 0; f < 7; ++f) {
                    if (!isfinite(res[f])) {
                        ++nbad;
                        break;
                    }
                }
                for (int f = 0; f < 7; ++f) store_f(out, f, k, res[f]);
            }
        }
    }
    if (ctr != nullptr && !dt_only && (nfl_r | nfl_p | nbad)) {
        if (nfl_r) atomicAdd(&ctr->rho_floor, (unsigned long long)nfl_r);
        if (nfl_p) atomicAdd(&ctr->p_floor, (unsigned long long)nfl_p);
        if (nbad) atomicAdd(&ctr->nonfinite, (unsigned long long)nbad);
    }
    block_tmin_and_rotate<HNT>(tmin, active, T_bits, rot, P.tile_nblocks);
}

}  // namespace

cudaError_t launch_hancock_parity(const Params& P, const CPlanes& in, const Planes& out,
                                  const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                  Scalars* ctr, int dt_only, cudaStream_t st) {
    const dim3 grid((P.N + HTX - 1) / HTX, P.tile_rows ? P.tile_rows : (P.M + HTY - 1) / HTY);
    if (P.scheme == GD_SCHEME_HANCOCK_REF)
        hancock_parity_kernel<true><<<grid, HNT, 0, st>>>(P, in, out, T_do, T_bits, rot, ctr,
                                                           dt_only);
    else
        hancock_parity_kernel<false><<<grid, HNT, 0, st>>>(P, in, out, T_do, T_bits, rot, ctr,
                                                            dt_only);
    return cudaGetLastError();
}

}  // namespace gd
