// gd_fast_mhd.cu -- fused minmod-TVD + HLLD / HLLC-MHD + update step for 2-D ideal MHD,
// face-once tiles.  (Kernel body added in the next revision.)
#include "gd_internal.cuh"
#include "gd_kernels.h"

namespace gd {

cudaError_t prepare_mhd_fast() { return cudaSuccess; }

cudaError_t launch_mhd_fast(const Params&, const CPlanes&, const Planes&, const double*,
                            unsigned long long*, Scalars*, Scalars*, int, cudaStream_t) {
    return cudaErrorNotSupported;
}

}  // namespace gd
