// Test harness around the reference viewer's GPU evaluator interface (gpuEvaluator.h:8-18).
//
// Test infrastructure only.  It plays the part of sCWatterView: it owns the unpacked-wave
// globals that cpuEvaluator.cpp:3-7 defines and cw_allocate / cw_unpack fill
// (cpuEvaluator.cpp:34-102), then calls gpu_initialize() and gpu_cw_evaluate(...) the way
// EvaluateVectorSlices does (sCWatterView.cpp:363-370).  The same file is linked twice:
//   * with the reference's own gpuEvaluator.cu (copied unchanged into oracle/_ref/src), which
//     pins the FP64 oracle and the GB300 evaluator to the reference's own kernels, and
//   * with the drop-in shim scwatter_gb300/shim/gpuEvaluator_gb300.cu, which shows that the
//     shim keeps the reference's interface and results.
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>

#include <thrust/complex.h>

#include "gpuEvaluator.h"

int layers = 0;
std::vector<float> z_layers;
std::vector<int> waves_begin;
std::vector<int> waves_end;
std::vector<UnpackedWave<float>> W;
size_t free_gpu_memory = 0;     // defined by the viewer (sCWatterView.cpp:102-103)
size_t total_gpu_memory = 0;

static std::string g_error;

extern "C" {

__attribute__((visibility("default"))) const char* scwref_last_error(void) { return g_error.c_str(); }

// waves: n_waves records of 12 floats (UnpackedWave<float>); begin / end: n_layers + 1 region
// offsets; zl: n_layers boundaries.  The three planes are N*N*6 floats each.  0 on success.
__attribute__((visibility("default"))) int scwref_evaluate(int n_layers, const float* zl, const int* begin,
                                                           const int* end, const float* waves, int64_t n_waves,
                                                           float* E_xy, float* E_xz, float* E_yz, float x_start,
                                                           float y_start, float z_start, float x, float y, float z,
                                                           float d, int N, int device) {
    try {
        layers = n_layers;
        z_layers.assign(zl, zl + n_layers);
        waves_begin.assign(begin, begin + n_layers + 1);
        waves_end.assign(end, end + n_layers + 1);
        W.resize((size_t)n_waves);
        if (n_waves) std::memcpy(W.data(), waves, (size_t)n_waves * sizeof(UnpackedWave<float>));
        gpu_initialize();
        gpu_cw_evaluate(reinterpret_cast<thrust::complex<float>*>(E_xy), reinterpret_cast<thrust::complex<float>*>(E_xz),
                        reinterpret_cast<thrust::complex<float>*>(E_yz), x_start, y_start, z_start, x, y, z, d, N,
                        device);
        const cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            g_error = cudaGetErrorString(e);
            return 2;
        }
    } catch (const std::exception& ex) {
        g_error = ex.what();
        return 1;
    }
    return 0;
}

}  // extern "C"
