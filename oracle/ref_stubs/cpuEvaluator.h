// Stand-in for the reference's cpuEvaluator.h (cpuEvaluator.h:1-35), for compiling the
// reference's gpuEvaluator.cu (and the drop-in shim) without Eigen, FFTW, MKL, glm or tira.
// Test infrastructure: it declares only what gpuEvaluator.cu and gpuEvaluator.h use -- the
// unpacked wave record (cpuEvaluator.h:6-10) and the globals cw_allocate / cw_unpack fill
// (cpuEvaluator.cpp:3-7, cpuEvaluator.h:12-16).
#pragma once

#include <cmath>
#include <complex>
#include <iostream>
#include <vector>

template <typename T>
struct UnpackedWave {
    std::complex<T> E0[3];
    std::complex<T> k[3];
};

extern int layers;
extern std::vector<float> z_layers;
extern std::vector<int> waves_begin;
extern std::vector<int> waves_end;
extern std::vector<UnpackedWave<float>> W;
