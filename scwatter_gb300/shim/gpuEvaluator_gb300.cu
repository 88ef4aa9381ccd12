// gpuEvaluator_gb300.cu -- drop-in replacement of the reference viewer's gpuEvaluator.cu.
//
// Keeps the two entry points of gpuEvaluator.h:8-18 and their meaning, and runs them on the
// GB300 library through its C ABI (include/scwatter.h):
//   gpu_initialize()      (gpuEvaluator.cu:15-26)  uploads the unpacked wave table that
//                         cw_allocate / cw_unpack left in the globals layers, z_layers,
//                         waves_begin, waves_end, W (cpuEvaluator.cpp:3-7, 34-102);
//   gpu_cw_evaluate(...)  (gpuEvaluator.cu:131-165) evaluates the xy plane at z, the xz plane at y
//                         and the yz plane at x into the caller's host arrays, [N][N][3] complex64
//                         each with the second axis as the row.
// A viewer build replaces gpuEvaluator.cu with this file and links -lscwatter_gb300; the globals
// stay where cpuEvaluator.cpp defines them.  Like the reference (HANDLE_ERROR), a failing call
// prints the library's message and stops the program.  The reference reads `device` only for
// its launch shape; here the context is opened on the device current at gpu_initialize().
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>
#include <thrust/complex.h>

#include "gpuEvaluator.h"   // the reference's declarations: the definitions below must match them
#include "scwatter.h"

static scw_ctx g_ctx = nullptr;
static scw_waves g_waves = nullptr;
static int g_device = 0;

static void check(scw_status s) {
    if (s != SCW_OK) {
        std::fprintf(stderr, "scwatter_gb300: %s\n", scw_last_error());
        std::exit(1);
    }
}

void gpu_initialize() {
    if (!g_ctx) {
        if (cudaGetDevice(&g_device) != cudaSuccess) g_device = 0;
        check(scw_ctx_create(g_device, nullptr, &g_ctx));
    }
    if (g_waves) {
        check(scw_waves_destroy(g_waves));
        g_waves = nullptr;
    }
    // UnpackedWave<float> is {complex<float> E0[3], k[3]}: the 12-float record the ABI takes
    static_assert(sizeof(UnpackedWave<float>) == 12 * sizeof(float), "UnpackedWave<float> layout");
    check(scw_gpu_initialize(g_ctx, layers, z_layers.data(), waves_begin.data(), waves_end.data(),
                             reinterpret_cast<const float*>(W.data()), (int64_t)W.size(), &g_waves));
}

void gpu_cw_evaluate(thrust::complex<float>* E_xy, thrust::complex<float>* E_xz, thrust::complex<float>* E_yz,
                     float x_start, float y_start, float z_start, float x, float y, float z, float d, int N,
                     int device) {
    (void)device;
    if (!g_waves) {
        std::fprintf(stderr, "scwatter_gb300: gpu_cw_evaluate before gpu_initialize\n");
        std::exit(1);
    }
    check(scw_gpu_cw_evaluate(g_waves, reinterpret_cast<float*>(E_xy), reinterpret_cast<float*>(E_xz),
                              reinterpret_cast<float*>(E_yz), x_start, y_start, z_start, x, y, z, d, N, g_device));
}
