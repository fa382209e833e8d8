/*
 * gdref_wrap.cpp -- C-ABI over the reference's OWN functions, compiled for the host.
 *
 * TEST INFRASTRUCTURE ONLY (oracle).  The symbols declared below are defined by the
 * reference's Gas_Dinamic.cu and kernel.cu, compiled unmodified through gdref_prelude.h
 * (see the Makefile in this directory).  Tests use this library to pin the project's C
 * restatement (oracle/gd_oracle.c) bit for bit, and tests/golden/make_golden.py uses it to
 * write the committed golden vectors.  The library exists only where the reference
 * sources exist; nothing in the product links against it.
 *
 * Layout of the state arrays is the reference's (kernel.cu:3814-3825):
 *   s = double2[K] {rho, p}, u = double2[K] {vx, vy}, b = double3[K] {Bx, By, Bz}.
 */
#include "gdref_prelude.h"
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <omp.h>

thread_local gdref_dim3 threadIdx = {0, 0, 0};
thread_local gdref_dim3 blockIdx = {0, 0, 0};
thread_local gdref_dim3 blockDim = {1, 1, 1};

double gdref_gamma = 5.0 / 3.0;
double gdref_krit = 0.25;
int gdref_N = 3226;
int gdref_M = 1792;
double gdref_xmax = 9.0;
double gdref_ymax = 5.0;

/* Reference functions (kernel.cu), declared with the reference's own signatures. */
double minmod(double x, double y);                                              /* kernel.cu:51  */
double linear(double x1, double t1, double x2, double t2, double x3, double t3,
              double y);                                                        /* kernel.cu:69  */
void linear2(double x1, double t1, double x2, double t2, double x3, double t3,
             double y1, double y2, double& A, double& B);                       /* kernel.cu:75  */
double HLLC_Aleksashov(double2& Ls, double2& Lu, double2& Rs, double2& Ru,
                       double n1, double n2, double2& Ps, double2& Pu,
                       double rad);                                             /* kernel.cu:853 */
double HLL(double2& Ls, double2& Lu, double2& Rs, double2& Ru, double n1, double n2,
           double2& Ps, double2& Pu, double rad);                               /* kernel.cu:1485 */
void funk_time(double* T, double* T_do, double* TT, int* i);                    /* kernel.cu:1722 */
void Ker_Dekard(double2* s, double2* u, double2* s2, double2* u2, double* T,
                double* T_do, int method);                                      /* kernel.cu:1736 */
void add2(double2* s, double2* u, double3* b, double2* s2, double2* u2, double3* b2,
          double* T, double* T_do, int i, int method);                          /* kernel.cu:1877 */
void Kernel_TVD(double2* s, double2* u, double3* b, double2* s2, double2* u2,
                double3* b2, double* T, double* T_do, int i, int method);       /* kernel.cu:2198 */
void Kernel_TVD_old(double2* s, double2* u, double2* s2, double2* u2, double* T,
                    double* T_do, int method);                                  /* kernel.cu:3286 */
void Kernel_GKR(double2* s, double2* u, double3* b, double2* s2, double2* u2, double3* b2,
                double* T, double* T_do, int i, int method);                    /* kernel.cu:2663 */
void print_file_mini(double2* s, double2* u, std::string name);                 /* kernel.cu:3682 */
void print_file_mini2(double2* s, double2* u, double3* b, std::string name);    /* kernel.cu:3724 */
void print_file_mini2(double2* s, double2* u, double3* b, std::string name,
                      double TTT);                                              /* kernel.cu:3767 */

namespace {

/* Run one __global__ body over every flat cell index, in parallel over host threads.
 * Each thread keeps its own copy of the dt accumulator (the reference's `*T > tmin`
 * write is a data race on the GPU); the copies are min-combined afterwards, which is the
 * value the race approximates.  Inputs are copied into buffers one element longer than
 * the grid because the reference reads s[K] / u[K] for the last cell (kernel.cu:2226). */
template <class Body>
void for_each_cell(double* T, Body body) {
    const long K = (long)gdref_N * gdref_M;
    double tmin = *T;
#pragma omp parallel
    {
        double t_local = *T;
#pragma omp for schedule(static)
        for (long idx = 0; idx < K; ++idx) {
            blockIdx.x = (unsigned)idx;
            blockDim.x = 1;
            threadIdx.x = 0;
            body(&t_local);
        }
#pragma omp critical
        {
            if (t_local < tmin) tmin = t_local;
        }
    }
    *T = tmin;
}

template <class V>
std::vector<V> padded(const double* src, long K) {
    std::vector<V> v((size_t)K + 1);
    std::memset(v.data(), 0, sizeof(V) * v.size());
    std::memcpy(v.data(), src, sizeof(V) * (size_t)K);
    return v;
}

}  // namespace

extern "C" {

void gdref_set_params(double gamma, double krit_, int N, int M, double xmax, double ymax) {
    gdref_gamma = gamma;
    gdref_krit = krit_;
    gdref_N = N;
    gdref_M = M;
    gdref_xmax = xmax;
    gdref_ymax = ymax;
}

int gdref_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

double gdref_minmod(double a, double b) { return minmod(a, b); }

double gdref_linear(double x1, double t1, double x2, double t2, double x3, double t3, double y) {
    return linear(x1, t1, x2, t2, x3, t3, y);
}

void gdref_linear2(double x1, double t1, double x2, double t2, double x3, double t3,
                   double y1, double y2, double* A, double* B) {
    linear2(x1, t1, x2, t2, x3, t3, y1, y2, *A, *B);
}

/* L, R = {rho, p, vx, vy}; out = {Ps.x, Ps.y, Pu.x, Pu.y} = {F_rho, F_E, F_mx, F_my}. */
double gdref_hllc(const double* L, const double* R, double n1, double n2, double rad,
                  double* out) {
    double2 Ls = {L[0], L[1]}, Lu = {L[2], L[3]};
    double2 Rs = {R[0], R[1]}, Ru = {R[2], R[3]};
    double2 Ps = {0.0, 0.0}, Pu = {0.0, 0.0};
    double t = HLLC_Aleksashov(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad);
    out[0] = Ps.x; out[1] = Ps.y; out[2] = Pu.x; out[3] = Pu.y;
    return t;
}

double gdref_hll(const double* L, const double* R, double n1, double n2, double rad,
                 double* out) {
    double2 Ls = {L[0], L[1]}, Lu = {L[2], L[3]};
    double2 Rs = {R[0], R[1]}, Ru = {R[2], R[3]};
    double2 Ps = {0.0, 0.0}, Pu = {0.0, 0.0};
    double t = HLL(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad);
    out[0] = Ps.x; out[1] = Ps.y; out[2] = Pu.x; out[3] = Pu.y;
    return t;
}

/* L, R = {rho, p, vx, vy, vz, Bx, By, Bz} (Gaussian B); P = the reference's P[8] after its
 * final permutation: {F_rho, F_mx, F_my, F_mz, F_Bx, F_By, F_Bz, F_E}. */
double gdref_hlld(const double* L, const double* R, double n1, double n2, double n3,
                  double rad, int metod, double* P) {
    double Q = 1.0, PQ = 0.0;
    for (int k = 0; k < 8; ++k) P[k] = 0.0;
    return HLLDQ_Korolkov(L[0], Q, L[1], L[2], L[3], L[4], L[5], L[6], L[7],
                          R[0], Q, R[1], R[2], R[3], R[4], R[5], R[6], R[7],
                          P, PQ, n1, n2, n3, rad, metod);
}

void gdref_funk_time(double* T, double* T_do, double* TT, int* i) { funk_time(T, T_do, TT, i); }

/* Whole-grid kernels.  s,u: 2*K doubles; b: 3*K doubles; outputs are in/out (cells the
 * reference does not write keep their contents).  *T is the running dt minimum. */
void gdref_kernel_tvd(const double* s, const double* u, const double* b, double* s2, double* u2,
                      double* b2, double* T, double T_do, int i, int method) {
    const long K = (long)gdref_N * gdref_M;
    auto ps = padded<double2>(s, K);
    auto pu = padded<double2>(u, K);
    auto pb = padded<double3>(b, K);
    double tdo = T_do;
    for_each_cell(T, [&](double* t) {
        Kernel_TVD(ps.data(), pu.data(), pb.data(), (double2*)s2, (double2*)u2, (double3*)b2, t,
                   &tdo, i, method);
    });
}

/* MUSCL-Hancock step (Kernel_GKR, kernel.cu:2663-3284) over all cells. */
void gdref_kernel_gkr(const double* s, const double* u, const double* b, double* s2, double* u2,
                      double* b2, double* T, double T_do, int i, int method) {
    const long K = (long)gdref_N * gdref_M;
    auto ps = padded<double2>(s, K);
    auto pu = padded<double2>(u, K);
    auto pb = padded<double3>(b, K);
    double tdo = T_do;
    for_each_cell(T, [&](double* t) {
        Kernel_GKR(ps.data(), pu.data(), pb.data(), (double2*)s2, (double2*)u2, (double3*)b2, t,
                   &tdo, i, method);
    });
}

void gdref_add2(const double* s, const double* u, const double* b, double* s2, double* u2,
                double* b2, double* T, double T_do, int i, int method) {
    const long K = (long)gdref_N * gdref_M;
    auto ps = padded<double2>(s, K);
    auto pu = padded<double2>(u, K);
    auto pb = padded<double3>(b, K);
    double tdo = T_do;
    for_each_cell(T, [&](double* t) {
        add2(ps.data(), pu.data(), pb.data(), (double2*)s2, (double2*)u2, (double3*)b2, t, &tdo,
             i, method);
    });
}

void gdref_ker_dekard(const double* s, const double* u, double* s2, double* u2, double* T,
                      double T_do, int method) {
    const long K = (long)gdref_N * gdref_M;
    auto ps = padded<double2>(s, K);
    auto pu = padded<double2>(u, K);
    double tdo = T_do;
    for_each_cell(T, [&](double* t) {
        Ker_Dekard(ps.data(), pu.data(), (double2*)s2, (double2*)u2, t, &tdo, method);
    });
}

void gdref_kernel_tvd_old(const double* s, const double* u, double* s2, double* u2, double* T,
                          double T_do, int method) {
    const long K = (long)gdref_N * gdref_M;
    auto ps = padded<double2>(s, K);
    auto pu = padded<double2>(u, K);
    double tdo = T_do;
    for_each_cell(T, [&](double* t) {
        Kernel_TVD_old(ps.data(), pu.data(), (double2*)s2, (double2*)u2, t, &tdo, method);
    });
}

/* Tecplot snapshots through the reference's own writers (Nmin, x_min = x_max / (2 N) and
 * y_min are the reference's compile-time values; x_max, y_max, N, M, gamma are the ones set
 * by gdref_set_params).  with_b = 0: print_file_mini (s, u); with_b = 1: print_file_mini2;
 * with_b = 2: print_file_mini2 with SOLUTIONTIME = ttt. */
void gdref_print_tecplot(const double* s, const double* u, const double* b, int with_b,
                         double ttt, const char* path) {
    const long K = (long)gdref_N * gdref_M;
    auto ps = padded<double2>(s, K);
    auto pu = padded<double2>(u, K);
    if (with_b == 0) {
        print_file_mini(ps.data(), pu.data(), std::string(path));
        return;
    }
    auto pb = padded<double3>(b, K);
    if (with_b == 1) print_file_mini2(ps.data(), pu.data(), pb.data(), std::string(path));
    else print_file_mini2(ps.data(), pu.data(), pb.data(), std::string(path), ttt);
}

/* The restart dump of the reference's main loop (kernel.cu:4245-4254, the
 * "instable_for_inner_b3.txt" stream): the same stream statements over every cell, at the
 * reference's x_min + n dx, y_min + m dy. */
void gdref_write_restart(const double* s, const double* u, const double* b, const char* path) {
    const long K = (long)gdref_N * gdref_M;
    const double xmin = gdref_xmax / (2.0 * gdref_N), ymin = gdref_ymax / (2.0 * gdref_M);
    const double dxr = gdref_xmax / gdref_N, dyr = gdref_ymax / gdref_M;
    std::ofstream fout(path);
    for (long k = 0; k < K; k++) {
        const int n = (int)(k % gdref_N);
        const int m = (int)((k - n) / gdref_N);
        const double y = ymin + m * dyr;
        const double x = xmin + n * dxr;
        fout << x << " " << y << " " << s[2 * k] << " " << s[2 * k + 1] << " " << u[2 * k] << " "
             << u[2 * k + 1] << " " << b[3 * k] << " " << b[3 * k + 1] << " " << b[3 * k + 2]
             << std::endl;
    }
}

}  // extern "C"
