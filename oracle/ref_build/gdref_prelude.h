/*
 * gdref_prelude.h -- host shim that lets the reference's CUDA sources compile as plain C++.
 *
 * TEST INFRASTRUCTURE ONLY.  This is part of the oracle: it is force-included (g++ -include)
 * in front of the reference's own Gas_Dinamic.cu and kernel.cu, which are compiled where they
 * lie, unmodified except for the grid-size lines of kernel.cu (N, M, x_max, y_max, see the
 * Makefile).  Nothing in the product links against the library this builds.
 *
 * What it provides:
 *   - empty CUDA qualifiers, double2 / double3 aggregates and __dsqrt_rn -> std::sqrt;
 *   - thread-local blockIdx / blockDim / threadIdx so that a host loop can call a __global__
 *     body once per flat cell index (index = blockIdx.x, blockDim.x = 1, threadIdx.x = 0);
 *   - run-time gamma and CFL: Header.h (pragma once) is included here first, then its
 *     compile-time constants `ga`, `ggg` (Header.h:4-5) and `krit` (Header.h:3) are redefined
 *     to read globals.  Every derived macro (g1, gg1, U8, ...) follows automatically.
 */
#pragma once
/* Every standard header the reference includes, ahead of Header.h: Header.h defines short
 * object-like macros (alpha, step, ...) that must not leak into the standard library. */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cfloat>
#include <math.h>
#include <stdio.h>
#include <algorithm>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>
#include <omp.h>

struct double2 { double x, y; };
struct double3 { double x, y, z; };
struct gdref_dim3 { unsigned int x, y, z; };

extern thread_local gdref_dim3 threadIdx;
extern thread_local gdref_dim3 blockIdx;
extern thread_local gdref_dim3 blockDim;

#define __device__
#define __global__
#define __host__
#define __forceinline__ inline

static inline double __dsqrt_rn(double v) { return std::sqrt(v); }

extern double gdref_gamma;
extern double gdref_krit;
extern int gdref_N;
extern int gdref_M;
extern double gdref_xmax;
extern double gdref_ymax;

#include "Header.h"

#undef krit
#define krit (gdref_krit)
#undef ggg
#define ggg (gdref_gamma)
#undef ga
#define ga (gdref_gamma)
