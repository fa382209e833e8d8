// A C++ host program bound to libgd2d through include/gd2d.h and the CUDA runtime only, as
// the reference's main would be (kernel.cu:3838-4174): it owns the device buffers in the
// reference's AoS layout (double2 s, u; double3 b), runs the reference's phase-2 loop
// protocol -- the step into the other buffer, then funk_time, twice per iteration
// (kernel.cu:4110-4137) -- through gd_step_ref / gd_funk_time, and writes the final state
// and times to a file for the test to compare with the same loop driven from Python.
//
//   capi_client <physics 0|1> <mode 0|1> <N> <M> <iterations> <in.bin> <out.bin>
//
// in.bin: N*M cells of s (2 doubles), u (2), then b (3) for MHD, as the reference stores
// them.  out.bin: the same layout after 2*iterations steps, then T_do and TT.
// Exit status 0 on success; a failed call prints its gd_status string.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gd2d.h"

namespace {

bool ok(gd_status s, const char* what) {
    if (s == GD_OK) return true;
    std::fprintf(stderr, "%s: %s\n", what, gd_status_string(s));
    return false;
}

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    return false;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: capi_client physics mode N M iterations in.bin out.bin\n");
        return 2;
    }
    const int physics = std::atoi(argv[1]), mode = std::atoi(argv[2]);
    const int N = std::atoi(argv[3]), M = std::atoi(argv[4]), iters = std::atoi(argv[5]);
    const size_t K = (size_t)N * M;
    const bool mhd = physics == GD_MHD;

    // the benchmark setting of each physics on the unit square, periodic (Euler: HLLC,
    // gamma 1.4; MHD: HLLD, gamma 5/3), CFL 0.4
    gd_config cfg = {};
    cfg.N = N;
    cfg.M = M;
    cfg.dx = 1.0 / N;
    cfg.dy = 1.0 / M;
    cfg.x0 = 0.5 / N;
    cfg.y0 = 0.5 / M;
    cfg.gamma = mhd ? 5.0 / 3.0 : 1.4;
    cfg.krit = 0.4;
    cfg.physics = physics;
    cfg.geometry = GD_CARTESIAN;
    cfg.order = 2;
    cfg.method = mhd ? GD_METHOD_HLLD : GD_METHOD_HLLC;
    for (int k = 0; k < 4; ++k) cfg.bc[k] = GD_BC_PERIODIC;
    cfg.mode = mode;
    gd_ctx* ctx = nullptr;
    if (!ok(gd_create(&cfg, &ctx), "gd_create")) return 1;

    const size_t ns = 2 * K, nu = 2 * K, nb = mhd ? 3 * K : 0;
    std::vector<double> host(ns + nu + nb);
    FILE* f = std::fopen(argv[6], "rb");
    if (!f || std::fread(host.data(), sizeof(double), host.size(), f) != host.size()) {
        std::fprintf(stderr, "cannot read %s\n", argv[6]);
        return 1;
    }
    std::fclose(f);

    // the reference's device buffers (kernel.cu:3838-3847): two states, T, T_do, TT, i
    double *s = nullptr, *u = nullptr, *b = nullptr, *s2 = nullptr, *u2 = nullptr, *b2 = nullptr;
    double *T = nullptr, *T_do = nullptr, *TT = nullptr;
    int* dev_i = nullptr;
    bool good = cuda_ok(cudaMalloc(&s, ns * sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&u, nu * sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&s2, ns * sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&u2, nu * sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&T, sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&T_do, sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&TT, sizeof(double)), "cudaMalloc") &&
                cuda_ok(cudaMalloc(&dev_i, sizeof(int)), "cudaMalloc");
    if (good && mhd)
        good = cuda_ok(cudaMalloc(&b, nb * sizeof(double)), "cudaMalloc") &&
               cuda_ok(cudaMalloc(&b2, nb * sizeof(double)), "cudaMalloc");
    if (!good) return 1;
    cudaMemcpy(s, host.data(), ns * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(u, host.data() + ns, nu * sizeof(double), cudaMemcpyHostToDevice);
    if (mhd) cudaMemcpy(b, host.data() + ns + nu, nb * sizeof(double), cudaMemcpyHostToDevice);
    // the reference's initial values (kernel.cu:3855-3866): T = 1e7 (the min-accumulator),
    // T_do the first dt, TT = 0, i = 0
    const double T0 = 1e7, Tdo0 = 1e-4, TT0 = 0.0;
    const int i0 = 0;
    cudaMemcpy(T, &T0, sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(T_do, &Tdo0, sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(TT, &TT0, sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dev_i, &i0, sizeof(int), cudaMemcpyHostToDevice);

    for (int it = 0; it < iters; ++it) {
        // was: Kernel_TVD<<<K/256, 256>>>(s, u, b, s2, u2, b2, T, T_do, i, meth);
        if (!ok(gd_step_ref(ctx, s, u, b, s2, u2, b2, T, T_do, it, GD_METHOD_CONFIG, nullptr),
                "gd_step_ref"))
            return 1;
        // was: funk_time<<<1, 1>>>(T, T_do, TT, dev_i);
        if (!ok(gd_funk_time(ctx, T, T_do, TT, dev_i, nullptr), "gd_funk_time")) return 1;
        if (!ok(gd_step_ref(ctx, s2, u2, b2, s, u, b, T, T_do, it, GD_METHOD_CONFIG, nullptr),
                "gd_step_ref"))
            return 1;
        if (!ok(gd_funk_time(ctx, T, T_do, TT, dev_i, nullptr), "gd_funk_time")) return 1;
    }
    if (!cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) return 1;

    double Tdo_h = 0.0, TT_h = 0.0;
    cudaMemcpy(host.data(), s, ns * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(host.data() + ns, u, nu * sizeof(double), cudaMemcpyDeviceToHost);
    if (mhd) cudaMemcpy(host.data() + ns + nu, b, nb * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(&Tdo_h, T_do, sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(&TT_h, TT, sizeof(double), cudaMemcpyDeviceToHost);
    if (!cuda_ok(cudaGetLastError(), "copies")) return 1;
    FILE* o = std::fopen(argv[7], "wb");
    if (!o) return 1;
    std::fwrite(host.data(), sizeof(double), host.size(), o);
    std::fwrite(&Tdo_h, sizeof(double), 1, o);
    std::fwrite(&TT_h, sizeof(double), 1, o);
    std::fclose(o);

    for (double* p : {s, u, b, s2, u2, b2, T, T_do, TT}) cudaFree(p);
    cudaFree(dev_i);
    gd_destroy(ctx);
    return 0;
}
