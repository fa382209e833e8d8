/*
 * gd2d.h -- C ABI of the GB300-native finite-volume step (2-D Euler and ideal MHD).
 *
 * Drop-in boundary for the reference's explicit step: minmod TVD reconstruction, HLLC
 * (Euler) / HLLD and HLLC-MHD (ideal MHD) interface fluxes, the conservative update with
 * positivity floors, and the CFL time-step minimum.  Plain C types only; every pointer
 * argument named "device" is a CUDA device pointer, `gd_stream` is a cudaStream_t (NULL
 * selects the legacy default stream).  Every call is asynchronous on its stream unless it
 * says otherwise, returns a gd_status and never exits the process.
 *
 * The reference has no library interface.  Its de-facto API is the kernel launch
 * protocol of main() in kernel.cu; each entry point below names the part it replaces.
 */
#ifndef GD2D_H
#define GD2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GD_ABI_VERSION 3

typedef void* gd_stream; /* cudaStream_t */

typedef enum {
    GD_OK = 0,
    GD_ERR_INVALID_ARG = 1,  /* bad configuration or argument; nothing was launched      */
    GD_ERR_CUDA = 2,         /* a CUDA call failed; see gd_last_cuda_error()              */
    GD_ERR_NONPHYSICAL = 3,  /* non-finite state detected (gd_stats.nonfinite > 0)        */
    GD_ERR_TIMEOUT = 4,      /* reserved for a bounded device-side wait that gives up; no
                                kernel here waits on another block, so none returns it    */
    GD_ERR_UNSUPPORTED = 5   /* combination not implemented                               */
} gd_status;

/* physics */
enum { GD_EULER = 0, GD_MHD = 1 };
/* geometry: Cartesian, or axisymmetric with y the radius (kernel.cu:2615, 2619-2648) */
enum { GD_CARTESIAN = 0, GD_AXISYM = 1 };
/* flux method codes are the reference's `method` argument (Ker_Dekard kernel.cu:1795 and
 * Kernel_TVD_old kernel.cu:3547 for Euler, Kernel_TVD's HLLDQ_Korolkov metod for MHD):
 * 0 = HLL (Euler, kernel.cu:1485), 1 = HLLC (Euler, HLLC_Aleksashov kernel.cu:853; the
 * reference's method 1 switches to HLL only on faces below hx = -3288, hy = 0, kernel.cu:26-27,
 * i.e. nowhere on its domains), 2 = HLLC-MHD (Gas_Dinamic.cu:1137), 3 = HLLD
 * (Gas_Dinamic.cu:1303).  GD_METHOD_CONFIG (-1) in a per-call argument means the context's
 * configured method. */
enum { GD_METHOD_HLL = 0, GD_METHOD_HLLC = 1, GD_METHOD_HLLC_MHD = 2, GD_METHOD_HLLD = 3 };
#define GD_METHOD_CONFIG (-1)
/* boundary conditions, one per side (left, right, bottom, top); two ghost layers each */
enum {
    GD_BC_PERIODIC = 0,      /* wrap; both sides of an axis must be periodic              */
    GD_BC_TRANSMISSIVE = 1,  /* ghosts copy the edge cell                                 */
    GD_BC_MIRROR_X = 2,      /* reflection, vx, Bx, By odd    (kernel.cu:2268-2281)        */
    GD_BC_AXIS = 3,          /* reflection, vy, Bz odd        (kernel.cu:2291-2302)        */
    GD_BC_AMBIENT = 4,       /* rho=1, p=1/gamma, v=0, B=0    (kernel.cu:2234-2242)        */
    GD_BC_OUTFLOW = 5,       /* edge cell, vx<0 -> 0.01       (kernel.cu:2249-2256)        */
    GD_BC_AMBIENT_KEEPB = 6  /* AMBIENT with B of the edge cell (kernel.cu:1935-1940)      */
};
/* spatial scheme */
enum {
    GD_SCHEME_TVD = 0,          /* cfg.order 1: add2 / Ker_Dekard; 2: minmod TVD Kernel_TVD    */
    GD_SCHEME_HANCOCK_REF = 1,  /* MUSCL-Hancock predictor-corrector, Kernel_GKR
                                   (kernel.cu:2663-3284) as written: the v_y slopes are taken
                                   from the pressures (kernel.cu:2966, 2974, 3006, 3038, ...)  */
    GD_SCHEME_HANCOCK = 2       /* the same scheme with v_y slopes taken from v_y             */
};
/* execution mode */
enum {
    GD_MODE_FAST = 0,   /* face-once tiles, hoisted reciprocals, FMA: within 1e-12 per step */
    GD_MODE_PARITY = 1  /* per-cell faces in the reference's arithmetic order, no FMA:
                           bit-identical to the reference's own step                      */
};

/* Grid, physics and boundaries.  Replaces the compile-time constants of Header.h:3-38
 * and kernel.cu:11-30. */
typedef struct gd_config {
    int N, M;              /* cells along x (fastest in memory) and y; N, M >= 3          */
    double dx, dy;         /* cell sizes (kernel.cu:19-20)                                 */
    double x0, y0;         /* centre of cell (0,0): x = x0 + n*dx (kernel.cu:2203-2204)      */
    double gamma;          /* adiabatic index (Header.h:4-5)                               */
    double krit;           /* per-face Courant number (Header.h:3)                         */
    int physics;           /* GD_EULER or GD_MHD                                           */
    int geometry;          /* GD_CARTESIAN or GD_AXISYM                                    */
    int order;             /* 1: first order (add2, Ker_Dekard); 2: minmod TVD (Kernel_TVD) */
    int method;            /* default flux code (GD_METHOD_*)                              */
    int bc[4];             /* left, right, bottom, top                                     */
    double frozen_radius;  /* cells with sqrt(x^2+y^2) < r are copied, 0 = none (ddist,
                              Header.h:36; kernel.cu:2218-2225; Kernel_GKR uses 2.0,
                              kernel.cu:2692)                                              */
    int mode;              /* GD_MODE_FAST or GD_MODE_PARITY                               */
    /* Added in ABI 3; zero keeps the ABI 2 behaviour. */
    int scheme;            /* GD_SCHEME_*.  The Hancock schemes are Kernel_GKR's own setting:
                              MHD, GD_AXISYM, method HLLD (its metod 3), bc = {MIRROR_X,
                              OUTFLOW, AXIS, AMBIENT_KEEPB}; anything else is
                              GD_ERR_UNSUPPORTED.  order is not used by them.              */
    double x_max, y_max;   /* domain extents (kernel.cu:15, 17); the Hancock schemes place
                              cell (n, m) at x = x0 + n (x_max - x0)/(N - 1),
                              y = y0 + m y_max / M (kernel.cu:2669-2670)                   */
} gd_config;

typedef struct gd_stats {
    double t;                   /* simulated time TT (kernel.cu:1725)                       */
    double dt;                  /* dt the next step will use (T_do)                         */
    double dt_next;             /* running minimum being accumulated (T)                    */
    long long steps;            /* steps taken (the reference's device counter i)           */
    long long rho_floor_hits;   /* cells whose density was floored (kernel.cu:1862, 2622)   */
    long long p_floor_hits;     /* cells whose pressure was floored (kernel.cu:1872, 2657)  */
    long long nonfinite;        /* cells that produced a non-finite value                   */
    /* Added in ABI 3. */
    double t_state;             /* time of the current state: the sum of the dt every step
                                   used (t lags the reference's way: TT already includes the
                                   dt of the next step, kernel.cu:1724-1725)                  */
} gd_stats;

typedef struct gd_ctx gd_ctx;

/* ---- lifetime ------------------------------------------------------------------------ */

/* Validates cfg (everything the reference assumed silently: sizes, positive h, BC pairs,
 * method vs physics) and allocates the resident state on the current device.
 * Replaces main()'s cudaMalloc block (kernel.cu:3838-3847). */
gd_status gd_create(const gd_config* cfg, gd_ctx** out);
gd_status gd_destroy(gd_ctx* ctx);
gd_status gd_get_config(const gd_ctx* ctx, gd_config* out);
const char* gd_status_string(gd_status s);
/* the last cudaError_t seen by any call in this process (0 = none) */
int gd_last_cuda_error(void);
int gd_abi_version(void);

/* ---- compat: the reference's launch protocol, reference AoS layout ------------------- */

/* One step over the whole grid, reference layout (kernel.cu:3814-3825):
 *   s = double2[K] {rho, p}, u = double2[K] {vx, vy}, b = double3[K] {Bx, By, Bz}
 *   (b = NULL for Euler), K = N*M, index m*N + n.
 * Reads *T_do (dt of this step), min-combines this step's CFL dt into *T.  Same roles as
 *   Kernel_TVD<<<K/256,256>>>(s,u,b,s2,u2,b2,T,T_do,i,method)  (kernel.cu:2198, 4113)
 *   add2<<<...>>>(...)            when cfg.order == 1, physics MHD (kernel.cu:1877, 4042)
 *   Ker_Dekard<<<...>>>(...)      when cfg.order == 1, physics Euler (kernel.cu:1736)
 *   Kernel_GKR<<<...>>>(...)      when cfg.scheme is a Hancock scheme (kernel.cu:2663)
 * method is the reference's code (GD_METHOD_*), GD_METHOD_CONFIG (-1) uses cfg.method.  `i`
 * is the reference's step counter (unused, as there).
 * All pointers are device pointers; s/s2 etc. must not alias.  Unlike the reference, the
 * dt minimum is exact and deterministic (no racy read-compare-write, kernel.cu:2607-2611),
 * and the launch needs no K % 256 == 0. */
gd_status gd_step_ref(gd_ctx* ctx, const double* s, const double* u, const double* b,
                      double* s2, double* u2, double* b2, double* T, const double* T_do,
                      int i, int method, gd_stream stream);

/* funk_time<<<1,1>>>(T, T_do, TT, i) (kernel.cu:1722-1733): T_do <- T, TT += T_do,
 * T <- 1e7, ++i.  Device pointers. */
gd_status gd_funk_time(gd_ctx* ctx, double* T, double* T_do, double* TT, int* i,
                       gd_stream stream);

/* ---- resident state (SoA planes owned by the context) -------------------------------- */

/* Load / store the state in the reference AoS layout from host (is_host != 0, pageable or
 * pinned) or device memory.  b is ignored (may be NULL) for Euler.  Replaces main()'s
 * cudaMemcpy blocks (kernel.cu:4005-4014, 4181-4188). */
gd_status gd_import(gd_ctx* ctx, const double* s, const double* u, const double* b,
                    int is_host, gd_stream stream);
gd_status gd_export(gd_ctx* ctx, double* s, double* u, double* b, int is_host,
                    gd_stream stream);

/* Set the dt of the next step and the simulated time (main() starts T_do = 1e-8, TT = 0,
 * kernel.cu:3860-3863). */
gd_status gd_set_time(gd_ctx* ctx, double T_do, double TT, gd_stream stream);

/* dt-only pass over the current state: T_do <- min over faces of krit*rad/max(|SL|,|SR|)
 * (capped at 1000 as the reference's per-cell start value), without updating the state. */
gd_status gd_init_dt(gd_ctx* ctx, gd_stream stream);

/* nsteps iterations of { step(cfg.method); funk_time } with ping-pong buffers, the
 * reference's production loop (kernel.cu:4102-4174).  The dt reduction and the
 * funk_time rotation are fused into the step kernel; one launch per step.
 * use_graph != 0 captures the nsteps launches in a CUDA graph on first use and replays
 * it (the graph is cached per nsteps). */
gd_status gd_advance(gd_ctx* ctx, int nsteps, int use_graph, gd_stream stream);

/* Time-step policy of gd_advance / gd_advance_to.
 *   GD_DT_LAGGED (default): the reference's protocol -- a step uses the dt reduced during the
 *     previous step (kernel.cu:2607-2611 + funk_time), i.e. the CFL dt of the state before.
 *   GD_DT_CURRENT: a step uses the CFL dt of its own input state (a dt-only pass and a
 *     commit launch before every step; ~2x the work per step).
 * Changing the policy drops the cached graphs. */
enum { GD_DT_LAGGED = 0, GD_DT_CURRENT = 1 };
gd_status gd_set_dt_policy(gd_ctx* ctx, int policy);

/* Advances until the time of the state (gd_stats.t_state) reaches t_end or max_steps steps
 * were taken: each step's dt is limited to what is left to t_end, so the last step lands
 * on it (to rounding).  Runs chunks of gd_advance (graphs when use_graph != 0) sized from
 * the current dt, reading the time back between chunks (one synchronisation each; about
 * log2 of the step count in all).  *steps_taken (may be NULL) receives the steps run.
 * Afterwards t_end is cleared.  t_end must be larger than the current t_state. */
gd_status gd_advance_to(gd_ctx* ctx, double t_end, long long max_steps, int use_graph,
                        long long* steps_taken, gd_stream stream);

/* One step of the resident loop (as gd_advance(1)) whose state comes from host memory and
 * whose result goes back to host memory: s, u, b in, s2, u2, b2 out, the reference AoS
 * layout (as gd_import / gd_export with is_host = 1).  Same result, dt and time as
 * gd_import + gd_advance(1) + gd_export.  With the lagged dt and pinned (page-locked) host
 * buffers the grid is moved in bands of tile rows, each band's upload, step and download
 * overlapping the others' on two copy streams, `stream` and two more compute streams;
 * otherwise (GD_DT_CURRENT, pageable buffers, grids of fewer than four tile rows) the three
 * calls run in turn.  The banded step is captured into a CUDA graph the first time a set
 * of buffer addresses is used with each of the two internal state buffers, and replayed
 * after that (the last four such graphs are kept): the buffers are checked to be pinned
 * at every call.
 * Returns after the result is in s2, u2, b2. */
gd_status gd_step_host(gd_ctx* ctx, const double* s, const double* u, const double* b,
                       double* s2, double* u2, double* b2, gd_stream stream);

/* A limit on the floor hits (density and pressure floors together, gd_stats
 * rho_floor_hits + p_floor_hits, counted since gd_create): when it is exceeded,
 * gd_get_stats returns GD_ERR_NONPHYSICAL, as it does for non-finite cells.  0 (the
 * default) sets no limit. */
gd_status gd_set_floor_limit(gd_ctx* ctx, long long max_floor_hits);

/* Synchronises `stream` and reads time, dt and the floor / non-finite counters. */
gd_status gd_get_stats(gd_ctx* ctx, gd_stats* out, gd_stream stream);

/* Device pointer of resident field f (0 rho, 1 p, 2 vx, 3 vy, 4 Bx, 5 By, 6 Bz) of the
 * current state; plane of N*M doubles, index m*N + n.  Valid until the next advance. */
gd_status gd_field_ptr(gd_ctx* ctx, int f, const double** out);

/* ---- differentiation: discrete adjoint and tangent ------------------------------------
 * No counterpart in the reference.  The map differentiated is n steps of the fast step
 * with the dt sequence of a recorded forward run held fixed (the CFL minimum is not
 * differentiated); minmod, wave-speed min/max, HLLC / HLLD region and guard choices and
 * floors are differentiated along the branch the forward values take.  Supported: MHD with
 * HLLD or Euler with HLLC, order 2, Cartesian, periodic on all sides, fast mode, no frozen
 * cells (the Orszag-Tang and Kelvin-Helmholtz configurations), with the dt policy
 * GD_DT_LAGGED (the recorded dt of a step is the one rotated by the step before it);
 * other configurations, and a context set to GD_DT_CURRENT, return GD_ERR_UNSUPPORTED from
 * gd_adj_forward.  All vectors are device pointers in
 * the reference AoS layout (d/ds: K x 2, d/du: K x 2, d/dB: K x 3, Gaussian B; for Euler
 * the d/dB pointers may be null).
 *
 * gd_adj_forward: advance nsteps from the current state (as gd_advance), recording the dt
 *   of every step and a checkpoint of the state every ckpt_every steps.
 * gd_adj_backward: given dL/dU at the final state, return dL/dU at the recorded initial
 *   state; each checkpoint segment is recomputed once, then stepped back in reverse.
 * gd_tangent: J v, the derivative of the recorded map at the initial state along v.
 * gd_adj_replay: the recorded map (same dt sequence) applied to another initial state. */
gd_status gd_adj_forward(gd_ctx* ctx, int nsteps, int ckpt_every, gd_stream stream);
gd_status gd_adj_backward(gd_ctx* ctx, const double* gs, const double* gu, const double* gb,
                          double* os, double* ou, double* ob, gd_stream stream);
gd_status gd_tangent(gd_ctx* ctx, const double* vs, const double* vu, const double* vb,
                     double* os, double* ou, double* ob, gd_stream stream);
gd_status gd_adj_replay(gd_ctx* ctx, const double* s, const double* u, const double* b,
                        double* os, double* ou, double* ob, gd_stream stream);
/* Diagnostic of the central-difference check (MHD; Euler contexts: GD_ERR_UNSUPPORTED):
 * replays the recorded map from two initial states (U0 + eps v and U0 - eps v) side by
 * side, writes both final states (as gd_adj_replay would) and counts where the two runs
 * take different branches of a non-smooth choice, step by step.  counts[0..7]:
 *   0 minmod pick of a cell's slope           (step, face) pairs, each slope at one face
 *   1 rho / p face-state fallback             (step, face) pairs
 *   2 HLLD wave-speed picks (min u, max u, max cf, max |S|)   (step, face) pairs
 *   3 HLLD upwind side and fan region                          (step, face) pairs
 *   4 HLLD guards (disc <= 0, |tt| >= 1e-5 either side, |bn| > 1e-6, sign bn)  pairs
 *   5 update floors rho <= 0, p <= 0          (step, cell) pairs
 *   6 cells touched by any of these           (step, cell) pairs
 *   7 cells touched at any step               cells
 * A difference quotient is the derivative of the branch the adjoint differentiates only
 * where all counts are 0.  Blocking (returns with the counts on the host). */
gd_status gd_adj_switches(gd_ctx* ctx, const double* sp, const double* up, const double* bp,
                          const double* sm, const double* um, const double* bm, double* osp,
                          double* oup, double* obp, double* osm, double* oum, double* obm,
                          long long* counts, gd_stream stream);

/* ---- batched: many independent grids --------------------------------------------------
 * No counterpart in the reference (it advances one grid, kernel.cu:4102).  A batch holds
 * ngrids independent grids of any sizes (same physics, order and mode; Euler, fast mode),
 * each with its own boundaries, dt reduction, dt rotation and time.  Schedules:
 *   GD_BATCH_PERSISTENT  one persistent launch per step walks the tiles of every grid
 *   GD_BATCH_LOOPED      one plain launch per grid per step (the baseline)
 *   GD_BATCH_LOOPED_SYNC as GD_BATCH_LOOPED, the host waiting for each launch to finish
 *                        before the next, as the reference's main loop synchronises after
 *                        each of its launches (kernel.cu:4113-4137); no graph (use_graph 0)
 * gd_batch_autotune times every compiled tile shape (16x16, 32x8, 32x16, 64x8; the halo
 * width is the stencil's, 2 cells for order 2) on the batch's own grids without changing
 * their state or time, and keeps the fastest for GD_BATCH_PERSISTENT. */
enum { GD_BATCH_PERSISTENT = 0, GD_BATCH_LOOPED = 1, GD_BATCH_LOOPED_SYNC = 2 };
typedef struct gd_batch gd_batch;
typedef struct gd_batch_info {
    int ngrids;
    long long total_cells;
    int tile_x, tile_y;        /* tile shape in use for the persistent schedule */
    int ctas;                  /* CTAs of the persistent launch */
    long long tiles;           /* work items per persistent step */
    double tuned_ms[4];        /* autotuner: ms per step of the tile shapes 16x16, 32x8,
                                  32x16, 64x8 (0 = not timed) */
} gd_batch_info;

gd_status gd_batch_create(const gd_config* cfgs, int ngrids, gd_batch** out);
gd_status gd_batch_destroy(gd_batch* b);
gd_status gd_batch_import(gd_batch* b, int grid, const double* s, const double* u,
                          const double* bfield, int is_host, gd_stream stream);
gd_status gd_batch_export(gd_batch* b, int grid, double* s, double* u, double* bfield,
                          int is_host, gd_stream stream);
gd_status gd_batch_set_time(gd_batch* b, double T_do, double TT, gd_stream stream);
gd_status gd_batch_init_dt(gd_batch* b, gd_stream stream);
gd_status gd_batch_advance(gd_batch* b, int nsteps, int schedule, int use_graph,
                           gd_stream stream);
gd_status gd_batch_autotune(gd_batch* b, int reps, gd_stream stream);
gd_status gd_batch_get_stats(gd_batch* b, int grid, gd_stats* out, gd_stream stream);
gd_status gd_batch_get_info(const gd_batch* b, gd_batch_info* out);
long long gd_batch_launch_count(const gd_batch* b);

/* ---- one step without device allocation ----------------------------------------------
 * No counterpart in the reference.  For callers that must not let a library allocate
 * device memory: a host program that owns all device memory through its own pool (a
 * coupled multi-physics driver, an in-situ analysis framework) or that runs on a
 * latency-critical path, where cudaMalloc would allocate outside the owner's budget and
 * cudaFree would synchronise the whole device.
 *
 * Same arguments and results as gd_step_ref, but no context: the grid is given by `cfg`,
 * and the scratch (SoA staging planes and floor counters) lives in one file-scope device
 * array of GD_STATIC_SCRATCH_BYTES that every GPU which loads this library holds until the
 * process exits.  Grids with N*M > GD_STATIC_MAX_CELLS are rejected with
 * GD_ERR_INVALID_ARG before anything is launched.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and sets kernel attributes, with that
 * device current; make that first call before any stream capture.  Every call shares the
 * one array and it keeps the last call's contents (the counters are cleared at the start
 * of each call): calls that overlap on the GPU (other streams, other host threads) race, so
 * serialise them.  Calls no cudaMalloc, cudaFree or other allocating routine
 * (gd_alloc_counts shows it).  It reports no non-physical state: the floor and non-finite
 * counts of the step stay in the device array and are not read back (that would
 * synchronise the stream), so GD_OK says nothing about the values; a caller that needs to
 * know checks the output itself or steps through a context (gd_step_ref + gd_get_stats). */
#define GD_STATIC_MAX_CELLS 65536
#define GD_STATIC_SCRATCH_BYTES (256 + 2 * 7 * 8 * GD_STATIC_MAX_CELLS)
gd_status gd_step_ref_static(const gd_config* cfg, const double* s, const double* u,
                             const double* b, double* s2, double* u2, double* b2, double* T,
                             const double* T_do, int method, gd_stream stream);

/* ---- state I/O -------------------------------------------------------------------------
 * The reference's file formats, produced and parsed on the GPU (formatting into per-line
 * slots, a prefix sum of line lengths, compaction, one copy to the host).  Numbers are
 * written as `ostream << double` writes them at its default format (printf "%.6g",
 * correctly rounded) and read as `istream >> double` reads them (correctly rounded);
 * files are byte-identical to the reference's writers.  Cells are in the reference order
 * k = m*N + n.  The gd_format_* / gd_parse_* forms work on host memory: with buf == NULL
 * (or cap too small) they only report the length in *len (GD_ERR_INVALID_ARG if buf was
 * given but too small).  All are blocking (they synchronise `stream`).
 *
 * Text restart file (kernel.cu:4245-4254 writer, kernel.cu:3944-3996 reader): one line
 * per cell, "x y rho p vx vy Bx By Bz", x = x0 + n*dx, y = y0 + m*dy (the config's cell
 * centres, the reference's x_min + n*dx), B in the stored Gaussian units; Euler contexts
 * write 0 for B.  The reader takes whitespace-separated numbers in order as the
 * reference's `fin >> c1 >> c2 >> a1 ... >> a7` does, ignores x and y, and fails on a
 * malformed or missing number or an overflowing value. */
gd_status gd_format_text(gd_ctx* ctx, char* buf, size_t cap, size_t* len, gd_stream stream);
gd_status gd_write_text(gd_ctx* ctx, const char* path, gd_stream stream);
gd_status gd_parse_text(gd_ctx* ctx, const char* text, size_t len, gd_stream stream);
gd_status gd_read_text(gd_ctx* ctx, const char* path, gd_stream stream);

/* Binary dump save_b3.dat (kernel.cu:4233-4261): per cell the raw doubles x, y, rho, p, vx,
 * vy, Bz (host byte order).  The reference writes no reader; gd_read_binary restores rho,
 * p, vx, vy and Bz from such a file and sets Bx = By = 0 (the file has no Bx, By). */
gd_status gd_write_binary(gd_ctx* ctx, const char* path, gd_stream stream);
gd_status gd_read_binary(gd_ctx* ctx, const char* path, gd_stream stream);

/* Tecplot FEPOINT snapshot (print_file_mini kernel.cu:3682-3722 for Euler,
 * print_file_mini2 kernel.cu:3724-3808 for MHD; with_time adds SOLUTIONTIME as the
 * second print_file_mini2 does): every nmin-th point in x and y (the reference's Nmin),
 * x = x_min + n (x_max - x_min) / (N - 1) with the reference's x_min / x_max (and y),
 * columns X Y Ro P Vx Vy [Bx By Bz] Max T with Max = |v| / sqrt(gamma p / rho) and
 * T = p / rho (0 where rho <= 0), then the quadrilateral connectivity (1-based). */
typedef struct {
    int nmin;
    double x_min, x_max, y_min, y_max;
    int with_time;
    double time;
} gd_tecplot_opts;
gd_status gd_format_tecplot(gd_ctx* ctx, const gd_tecplot_opts* opts, char* buf, size_t cap,
                            size_t* len, gd_stream stream);
gd_status gd_write_tecplot(gd_ctx* ctx, const char* path, const gd_tecplot_opts* opts,
                           gd_stream stream);

/* ---- measurement helpers -------------------------------------------------------------- */

/* Number of kernel launches the library issued on behalf of this context so far. */
long long gd_launch_count(const gd_ctx* ctx);

/* Measures the device's FP64 FMA throughput (FLOP/s, FMA = 2) with a register-resident
 * DFMA loop on every SM; blocking, ~50 ms. */
gd_status gd_probe_fp64_peak(double* flops_out);

/* Diagnostic (no reference counterpart): checks, on the device, the step kernels' IEEE-754
 * binary64 multiplication on the integer pipes against the FP64 unit's multiply on about
 * `pairs` seeded operand pairs (any bit patterns, exponents near 1, subnormal operands,
 * products near the overflow and underflow limits).  counts_out[0]: results whose bits
 * differ (NaN results excepted), [1]: NaN results whose payloads differ, [2]: pairs outside
 * the integer fast path, [3]: pairs checked.  Blocking. */
gd_status gd_check_int_mul(long long pairs, unsigned long long seed, long long* counts_out);

/* Diagnostic (no reference counterpart): the Euler step's two-operation reciprocal and root
 * against IEEE division and square root on about `count` seeded values (reciprocals of
 * +-[2^-100, 2^100]; sqrt(a / r) for a, r in [2^-50, 2^50], whose IEEE form rounds twice).
 * out[0]: largest distance of the reciprocal in units of the last place, out[1]: of the
 * root, out[2]: of the three-operation root the MHD step uses, out[3]: values checked.
 * Blocking. */
gd_status gd_check_fast_roots(long long count, unsigned long long seed, long long* out);

/* Diagnostic (no reference counterpart): how many device or pinned-host allocations
 * (cudaMalloc, cudaMallocHost) and releases (cudaFree, cudaFreeHost) this library has made
 * in this process, over all contexts and threads.  Every allocation of the library goes
 * through the two counted helpers; a caller that must not let the library allocate can
 * check that a call left both counts unchanged. */
gd_status gd_alloc_counts(long long* allocs, long long* frees);

/* Test entry point (no reference counterpart): the fast step's own face solver on n
 * independent faces, for per-face checks against the reference's HLLC_Aleksashov /
 * HLL (kernel.cu:853-1165, 1485-1609) and HLLDQ_Korolkov (Gas_Dinamic.cu:964-1510).
 * Device pointers; axis 0: the face normal is +x, 1: +y.
 *   physics GD_EULER, method GD_METHOD_HLL or GD_METHOD_HLLC: L, R n x 4 (rho, p, vx, vy);
 *     flux n x 4 (mass, energy, x momentum, y momentum).
 *   physics GD_MHD, method GD_METHOD_HLLC_MHD or GD_METHOD_HLLD: L, R n x 8 (rho, p, vx, vy,
 *     vz, Bx, By, Bz; Gaussian B; vz is taken as 0, as the 2-D step does); flux n x 8 (mass,
 *     x, y, z momentum, Bx, By, Bz, energy; Gaussian field fluxes; the z-momentum flux is not
 *     formed by the 2-D step and is written as 0).
 * speed: n values max(|S_L|, |S_R|) (the reference's dt estimate is krit * rad / speed).
 * Asynchronous on stream. */
gd_status gd_probe_faces(int physics, int method, double gamma, int axis, long long n,
                         const double* L, const double* R, double* flux, double* speed,
                         gd_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* GD2D_H */
