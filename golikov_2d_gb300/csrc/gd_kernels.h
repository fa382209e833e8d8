// gd_kernels.h -- host-side launch functions of the step kernels (internal).
#pragma once

#include <cuda_runtime.h>

#include "gd_internal.cuh"

namespace gd {

// One-time function attributes (dynamic shared memory) of the fast kernels; called when a
// context is created, outside any stream capture.
cudaError_t prepare_euler_fast();
cudaError_t prepare_mhd_fast();

// Fast face-once step.  `rot` (may be null) receives the fused funk_time rotation by the
// last block; `ctr` (may be null) receives floor / non-finite counters.  dt_only != 0
// computes only the dt minimum.
// Tangent of one Euler step (value and derivative planes), dt read from *T_do.
cudaError_t launch_euler_tangent(const Params& P, const CPlanes& in, const CPlanes& din,
                                 const Planes& out, const Planes& dout, const double* T_do,
                                 cudaStream_t st);
// The Euler step (variant 0, as gd_advance launches it) writing its flux differences d[0..3] per cell to `aux`.
cudaError_t launch_euler_fast_aux(const Params& P, const CPlanes& in, const Planes& out,
                                  const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                  Scalars* ctr, double* aux, cudaStream_t st);
// The step's face solvers on n independent faces (gd_probe_faces).
cudaError_t launch_euler_face_probe(const Params& P, long long n, int axis, const double* L,
                                    const double* R, double* flux, double* speed,
                                    cudaStream_t st);
cudaError_t launch_mhd_face_probe(const Params& P, long long n, int axis, const double* L,
                                  const double* R, double* flux, double* speed,
                                  cudaStream_t st);
cudaError_t launch_euler_fast(const Params& P, const CPlanes& in, const Planes& out,
                              const double* T_do, unsigned long long* T_bits, Scalars* rot,
                              Scalars* ctr, int dt_only, cudaStream_t st);
cudaError_t launch_mhd_fast(const Params& P, const CPlanes& in, const Planes& out,
                            const double* T_do, unsigned long long* T_bits, Scalars* rot,
                            Scalars* ctr, int dt_only, cudaStream_t st);
// Rows of a tile of launch_mhd_fast (the Euler step's are euler_tile_shape(0)).  Both fast
// launches honour Params::tile_row0 / tile_rows / tile_nblocks (a band of tile rows).
int mhd_tile_height();
// Rows of the blocks of the per-cell parity kernels (launch_parity, launch_hancock_parity),
// which honour the same band parameters; their blocks are 32 cells wide.
constexpr int kParityBlockRows = 4;

// Tile-shape variants of the fast Euler kernels (0: 16x16, the single-grid step's; 1: 32x8;
// 2: 32x16; 3: 64x8).
constexpr int kEulerVariants = 4;
void euler_tile_shape(int variant, int* tx, int* ty);
size_t euler_smem_bytes(int order, int variant);
cudaError_t launch_euler_fast_v(int variant, const Params& P, const CPlanes& in,
                                const Planes& out, const double* T_do,
                                unsigned long long* T_bits, Scalars* rot, Scalars* ctr,
                                int dt_only, cudaStream_t st);
// Resident CTAs per SM of the persistent batched kernel of a variant.
int euler_batch_blocks_per_sm(int order, int variant);
// Per-grid scalar kernels of a batch (gd_util.cu).
cudaError_t launch_batch_set_time(BatchGrid* grids, int ngrids, double T_do, double TT,
                                  cudaStream_t st);
cudaError_t launch_batch_reset_T(BatchGrid* grids, int ngrids, cudaStream_t st);
cudaError_t launch_batch_dt_commit(BatchGrid* grids, int ngrids, cudaStream_t st);
// Persistent batched step over the (grid, tile) list `items` with `ctas` CTAs.
cudaError_t launch_euler_batch(int variant, int order, const BatchGrid* grids, const int2* items,
                               int nitems, int cur, int dt_only, Scalars* sc_override, int ctas,
                               cudaStream_t st);

// Tangent (forward-mode JVP) of one fast MHD step with the dt read from *T_do:
// (in, din) -> (out, dout).
cudaError_t launch_mhd_tangent(const Params& P, const CPlanes& in, const CPlanes& din,
                               const Planes& out, const Planes& dout, const double* T_do,
                               cudaStream_t st);

// Fast MHD step that also stores, per cell, the flux differences and the Powell term the
// update used (8 planes of N*M in `aux`), for the adjoint.  `rot` / `ctr` as in
// launch_mhd_fast (null: no dt rotation, no counters).
cudaError_t launch_mhd_fast_aux(const Params& P, const CPlanes& in, const Planes& out,
                                const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                Scalars* ctr, double* aux, cudaStream_t st);
// One reverse step of the fast MHD step (HLLD, order 2, Cartesian, periodic):
// lam_in = S'(U)^T lam_out, with U, aux of the forward step and the dt *T_do.
// `scratch` holds adjoint_scratch_planes() planes of N*M.
int adjoint_scratch_planes();
// The Euler (HLLC) reverse step, the same roles as launch_adjoint_step with four fields and
// aux d[0..3] per cell; its scratch holds adjoint_euler_scratch_planes() planes.
int adjoint_euler_scratch_planes();
cudaError_t launch_adjoint_step_euler(const Params& P, const CPlanes& U, const double* aux,
                                      const CPlanes& lam_out, const Planes& lam_in,
                                      double* scratch, const double* T_do, cudaStream_t st);
cudaError_t prepare_adjoint();
// Branch switches between two runs of the MHD step (gd_adj_switches): per step, the face
// choices of the two input states (counters 0-4: minmod, rho/p fallback, wave-speed picks,
// HLLD region, guards; (step, face) pairs; faces mark their two cells in step_mark), then
// the update floors of both steps (counter 5, (step, cell) pairs) and the marked cells
// (counter 6; moved into ever_mark); at the end the cells marked at any step (counter 7).
int switch_kinds();
cudaError_t launch_switch_faces(const Params& P, const CPlanes& Ua, const CPlanes& Ub,
                                unsigned long long* ctr, unsigned char* step_mark,
                                cudaStream_t st);
cudaError_t launch_switch_cells(const Params& P, const CPlanes& Ua, const double* auxa,
                                const CPlanes& Ub, const double* auxb, unsigned long long* ctr,
                                unsigned char* step_mark, unsigned char* ever_mark,
                                cudaStream_t st);
cudaError_t launch_switch_total(long long K, const unsigned char* ever_mark,
                                unsigned long long* ctr, cudaStream_t st);
cudaError_t launch_adjoint_step(const Params& P, const CPlanes& U, const double* aux,
                                const CPlanes& lam_out, const Planes& lam_in, double* scratch,
                                const double* T_do, cudaStream_t st);

// Parity step: per-cell faces in the reference's arithmetic order (built without FMA
// contraction); bit-identical to the reference step.
cudaError_t launch_parity(const Params& P, const CPlanes& in, const Planes& out,
                          const double* T_do, unsigned long long* T_bits, Scalars* rot,
                          Scalars* ctr, int dt_only, cudaStream_t st);

// MUSCL-Hancock step of Kernel_GKR (P.scheme GD_SCHEME_HANCOCK_REF / GD_SCHEME_HANCOCK).
// Parity: every cell as the reference computes it (built without FMA contraction;
// bit-identical).  Fast: face-once tiles for the cells away from the edges, the per-cell
// evaluation for the two-cell band along the edges (two launches, concurrent when a side
// stream is given).
cudaError_t launch_hancock_parity(const Params& P, const CPlanes& in, const Planes& out,
                                  const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                  Scalars* ctr, int dt_only, cudaStream_t st);
cudaError_t launch_hancock_fast(const Params& P, const CPlanes& in, const Planes& out,
                                const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                Scalars* ctr, int dt_only, cudaStream_t st,
                                const HancockStreams* side = nullptr);
cudaError_t prepare_hancock_fast();
// The fast Hancock step on rows [r0, r1) only, for a step cut into bands: `parts` 1 launches
// the edge cells, 2 the interior tiles, 3 both (in that order on `st`); r0 and r1 are 0, M or
// 2 + a multiple of hancock_tile_height() (the interior tiles start at row 2).  All launches
// of the step share one rotation ticket of `nblocks` blocks: the sum over the launches of
// hancock_fast_blocks(P, r0, r1, parts).
int hancock_tile_height();
unsigned int hancock_fast_blocks(const Params& P, int r0, int r1, int parts);
cudaError_t launch_hancock_fast_rows(const Params& P, const CPlanes& in, const Planes& out,
                                     const double* T_do, unsigned long long* T_bits,
                                     Scalars* rot, Scalars* ctr, int r0, int r1,
                                     unsigned int nblocks, int parts, cudaStream_t st);

// Utilities (gd_util.cu).
cudaError_t launch_aos_to_soa(const double* s, const double* u, const double* b, Planes out,
                              long long K, int nf, cudaStream_t st);
cudaError_t launch_soa_to_aos(CPlanes in, double* s, double* u, double* b, long long K, int nf,
                              cudaStream_t st);
cudaError_t launch_funk_time(double* T, double* T_do, double* TT, int* i, cudaStream_t st);
cudaError_t launch_set_time(Scalars* sc, double T_do, double TT, cudaStream_t st);
cudaError_t launch_set_end(Scalars* sc, double t_end, cudaStream_t st);
cudaError_t launch_dt_commit(Scalars* sc, cudaStream_t st);
cudaError_t launch_reset_T(Scalars* sc, cudaStream_t st);
cudaError_t probe_fp64_peak(double* flops);
cudaError_t check_imul(long long pairs, unsigned long long seed, long long* out);
cudaError_t check_roots(long long count, unsigned long long seed, long long* out);

// Every device and pinned-host allocation and release the library makes goes through these
// (gd_api.cu), which count them for gd_alloc_counts.
cudaError_t dev_alloc_bytes(void** p, size_t bytes);
cudaError_t host_alloc_bytes(void** p, size_t bytes);
cudaError_t dev_free(void* p);
cudaError_t host_free(void* p);
template <class T>
cudaError_t dev_alloc(T** p, size_t bytes) {
    return dev_alloc_bytes(reinterpret_cast<void**>(p), bytes);
}
template <class T>
cudaError_t host_alloc(T** p, size_t bytes) {
    return host_alloc_bytes(reinterpret_cast<void**>(p), bytes);
}

// Records e as the process's last CUDA error (gd_last_cuda_error) and returns GD_ERR_CUDA;
// every entry point reports a failed CUDA call through it.
gd_status cuda_error(cudaError_t e);

// Configuration checks and launch parameters (gd_api.cu), shared with entry points that
// work without a context.
gd_status validate_config(const gd_config* c);
Params params_from_config(const gd_config& c);

}  // namespace gd
