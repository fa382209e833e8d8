/*
 * gd_oracle.h -- CPU restatement of the reference's explicit finite-volume step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library is checked against.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and only as
 * the oracle or the timed CPU baseline; the product never calls it.
 *
 * Every function restates a reference routine (file:line given at each definition) with
 * the reference's arithmetic order, so that, compiled with -ffp-contract=off, it reproduces
 * the reference bit for bit.  That claim is tested against the reference's own code built
 * for the host (oracle/_ref/libgdref.so) and against the golden vectors in tests/golden/.
 *
 * State layout is the reference's AoS layout (kernel.cu:3814-3825), cell index k = m*N + n
 * with n along x (fastest):
 *   s[2k..2k+1] = {rho, p}, u[2k..2k+1] = {vx, vy}, b[3k..3k+2] = {Bx, By, Bz} (Gaussian).
 */
#ifndef GD_ORACLE_H
#define GD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { GDO_EULER = 0, GDO_MHD = 1 };
enum { GDO_CARTESIAN = 0, GDO_AXISYM = 1 };
enum {
    GDO_BC_PERIODIC = 0,      /* wrap around (both sides of the axis must be periodic)      */
    GDO_BC_TRANSMISSIVE = 1,  /* both ghosts = edge cell                                    */
    GDO_BC_MIRROR_X = 2,      /* reflect, vx, Bx, By odd        (kernel.cu:2268-2281)       */
    GDO_BC_AXIS = 3,          /* reflect, vy, Bz odd            (kernel.cu:2291-2302)       */
    GDO_BC_AMBIENT = 4,       /* rho=1, p=1/gamma, v=0, B=0     (kernel.cu:2234-2242)       */
    GDO_BC_OUTFLOW = 5,       /* edge cell with vx<0 -> 0.01    (kernel.cu:2249-2256)       */
    GDO_BC_AMBIENT_KEEPB = 6  /* as AMBIENT but B = edge cell B (kernel.cu:1935-1940, add2) */
};

typedef struct {
    int N, M;              /* cells along x and y                                         */
    double dx, dy;         /* cell sizes                                                  */
    double x0, y0;         /* centre of cell (0,0): x = x0 + n*dx (kernel.cu:2203-2204)     */
    double gamma, krit;    /* adiabatic index (Header.h:4-5), per-face CFL (Header.h:3)     */
    int physics;           /* GDO_EULER / GDO_MHD                                         */
    int geometry;          /* GDO_CARTESIAN / GDO_AXISYM (y is the radius)                 */
    int order;             /* 1: first order (Ker_Dekard, add2); 2: minmod TVD             */
    int method;            /* flux code: Euler 1 = HLLC; MHD 2 = HLLC-MHD, 3 = HLLD         */
    int bc[4];             /* left, right, bottom, top                                    */
    double frozen_radius;  /* cells with sqrt(x^2+y^2) < this are copied (kernel.cu:2218)  */
    int scheme;            /* 0: TVD step by order; 1: MUSCL-Hancock Kernel_GKR
                              (kernel.cu:2663) as written (v_y slopes from p, :2966);
                              2: the same with v_y slopes from v_y                        */
    double x_max, y_max;   /* the reference's x_max, y_max (kernel.cu:15, 17): Kernel_GKR
                              places cells at x_min + n (x_max - x_min)/(N - 1),
                              y_min + m y_max / M                                        */
} gdo_config;

/* kernel.cu:51-84 */
double gdo_minmod(double a, double b);
double gdo_linear(double x1, double t1, double x2, double t2, double x3, double t3, double y);
void gdo_linear2(double x1, double t1, double x2, double t2, double x3, double t3, double y1,
                 double y2, double* A, double* B);

/* Euler HLLC, kernel.cu:853-1165.  L, R = {rho, p, vx, vy}; normal (n1, n2) axis-aligned.
 * out = {F_rho, F_E, F_mx, F_my}.  Returns krit*rad/max(|SL|,|SR|). */
double gdo_hll(const double* L, const double* R, double n1, double n2, double rad,
               double gamma, double krit, double* out);
double gdo_hllc(const double* L, const double* R, double n1, double n2, double rad,
                double gamma, double krit, double* out);

/* MHD HLLD (method 3) / HLLC-MHD (method 2), Gas_Dinamic.cu:964-1510.
 * L, R = {rho, p, vx, vy, vz, Bx, By, Bz}.  P = {F_rho, F_mx, F_my, F_mz, F_Bx, F_By, F_Bz, F_E}.
 * Returns krit*rad/max(|SL|,|SR|). */
double gdo_hlld(const double* L, const double* R, double n1, double n2, double n3, double rad,
                int method, double gamma, double krit, double* P);

/* One step over the whole grid.  Reads (s,u,b), writes (s2,u2,b2) for every cell the
 * reference writes.  dt_only != 0 computes only the dt minimum and writes nothing.
 * Returns min(T_in, min over active cells of the per-cell dt, which starts at 1000). */
double gdo_step(const gdo_config* cfg, const double* s, const double* u, const double* b,
                double* s2, double* u2, double* b2, double T_do, double T_in, int dt_only);

/* Host threads used by gdo_step (0 = leave unchanged); returns the count in effect. */
int gdo_set_threads(int n);

/* Reference funk_time, kernel.cu:1722-1733 (without its progress print). */
void gdo_funk_time(double* T, double* T_do, double* TT, int* i);

/* State files (kernel.cu:3682-3808, 4233-4261): the reference's writers restated with C
 * stdio.  `os << double` at the stream's default format is printf "%g" (precision 6) and
 * `os << int` is "%d", so the bytes are the reference's.  Return 0 on success. */
int gdo_write_restart(const gdo_config* cfg, const double* s, const double* u, const double* b,
                      const char* path);
int gdo_write_binary(const gdo_config* cfg, const double* s, const double* u, const double* b,
                     const char* path);
/* The restart reader (kernel.cu:3944-3996): nine numbers per cell read in order, x and y
 * dropped; b may be NULL (Euler).  Returns 0 on success, 1 if a number is missing. */
int gdo_read_restart(const gdo_config* cfg, const char* path, double* s, double* u, double* b);
int gdo_write_tecplot(const gdo_config* cfg, const double* s, const double* u, const double* b,
                      int nmin, double x_min, double x_max, double y_min, double y_max,
                      int with_time, double time, const char* path);

#ifdef __cplusplus
}
#endif
#endif
