// Internal definitions shared by the scwatter_gb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/scwatter.h"

namespace scw {

// Thread-local last-error message behind scw_last_error().
void set_error(const std::string& msg);
scw_status fail(scw_status st, const std::string& msg);

#define SCW_CUDA_TRY(expr)                                                                \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return ::scw::fail(SCW_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Makes `device` current for the enclosing scope and gives the caller's current device back
// when the scope ends, so no entry point changes the calling thread's device as a side effect.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int device) {
        if (device < 0) return;
        int cur = -1;
        if (cudaGetDevice(&cur) != cudaSuccess) {
            cudaGetLastError();
            cur = -1;
        }
        if (cur != device) {
            err = cudaSetDevice(device);
            if (err == cudaSuccess) prev = cur;
        }
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

#define SCW_CAT2_(a, b) a##b
#define SCW_CAT_(a, b) SCW_CAT2_(a, b)
// the device of a context current until the end of the enclosing scope; returns on failure
#define SCW_ON_DEVICE(dev)                                                                          \
    ::scw::DeviceScope SCW_CAT_(scw_dev_scope_, __LINE__)(dev);                                     \
    if (SCW_CAT_(scw_dev_scope_, __LINE__).err != cudaSuccess)                                      \
    return ::scw::fail(SCW_ERR_CUDA, std::string("cudaSetDevice: ") +                               \
                                         cudaGetErrorString(SCW_CAT_(scw_dev_scope_, __LINE__).err))

// Device buffer (of a context or a call); grows on demand, never shrinks, freed on destruction.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    scw_status reserve(size_t n);
    void release();
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
};

// Pinned host staging buffer for small per-call descriptor uploads.
struct PinnedBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    scw_status reserve(size_t n);
    void release();
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { release(); }
};

}  // namespace scw

// Optional per-kernel CUDA-event timing (scw_ctx_set_timing): one record per launch.
struct KernelTiming {
    const char* name;
    cudaEvent_t start, stop;
};

struct scw_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 0;
    int synth_ctas = 0;         // > 0: CTAs of the tensor-core output GEMM (a pipelined caller leaves SMs free)
    int64_t launches = 0;
    scw::DevBuf scratch;        // split-K partial sums of the plain evaluator
    scw::DevBuf desc;           // per-call work descriptors
    scw::DevBuf planes_out;     // device staging of gpu_cw_evaluate's three planes
    scw::DevBuf sep_scratch;    // separable evaluator: phases, coefficients C, row products T, tables
    scw::PinnedBuf host_desc;   // pinned staging of the descriptors
    cudaEvent_t desc_done = nullptr;  // the last descriptor upload has been consumed
    void* static_scratch = nullptr;   // device address of the allocation-free entry point's array
    int* tc_err = nullptr;            // device flag: a tensor-core kernel's bounded wait gave up
    bool tc_pending_check = false;    // a tensor-core kernel ran since the flag was last read
    bool timing = false;
    std::vector<KernelTiming> timings;
    std::vector<cudaEvent_t> event_pool;
};

namespace scw {
// brackets one kernel launch with events when the context's timing is on
struct LaunchTimer {
    scw_ctx ctx;
    const char* name;
    cudaEvent_t a = nullptr, b = nullptr;
    LaunchTimer(scw_ctx c, const char* n);
    ~LaunchTimer();
};
}  // namespace scw

struct scw_cw_s {
    uint64_t sizeof_T = 8;
    std::vector<double> Pi;                 // n * 12
    struct Layer {
        double z = 0.0;
        std::vector<double> Pr, Pt;         // n * 12 each
    };
    std::vector<Layer> layers;
};

struct scw_waves_s {
    scw_ctx ctx = nullptr;
    int layers = 0;
    int64_t n = 0;
    int rule = 0;                           // 0: z >= z_l - 0.001, 1: z >= z_l
    std::vector<float> z_layers;
    std::vector<int64_t> begin, end;        // layers + 1 regions
    // device SoA tables (n entries each)
    double* kre = nullptr;                  // [3][n] Re k
    double* kim = nullptr;                  // [3][n] Im k
    double* zref = nullptr;                 // [n] reference plane of the amplitude
    float2* amp = nullptr;                  // [3][n] E0 at the reference plane
};

namespace scw {
// Implemented in eval_plain.cu
scw_status waves_upload(scw_waves w, const std::vector<double>& kre, const std::vector<double>& kim,
                        const std::vector<double>& zref, const std::vector<float2>& amp);
}
