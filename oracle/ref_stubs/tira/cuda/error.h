// Stand-in for tira's cuda/error.h (STIM-Lab/tiralib; not vendored by the reference): the
// HANDLE_ERROR macro that gpuEvaluator.cu wraps around every CUDA call.  tira prints the error
// and stops the program; this harness version throws instead, so that a failed allocation or
// copy ends the call before any kernel runs on a bad pointer, and the harness reports it.
#pragma once

#include <cuda_runtime.h>
#include <stdexcept>
#include <string>

struct ScwRefCudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void scwref_handle_error(cudaError_t err, const char* file, int line) {
    if (err != cudaSuccess)
        throw ScwRefCudaError(std::string(cudaGetErrorString(err)) + " in " + file + " at line " + std::to_string(line));
}

#define HANDLE_ERROR(err) (scwref_handle_error((err), __FILE__, __LINE__))
