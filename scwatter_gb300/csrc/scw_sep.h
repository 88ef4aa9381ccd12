// Separable-form coefficient set and shared declarations of the GEMM-form evaluator.
#pragma once

#include <cuda_runtime.h>
#include <vector>

#include "scw_internal.h"

namespace scw {

constexpr int kMaxGroup = 8;   // z-planes contracted together in stage 1

// z-planes of one region handled by one stage-1 pass
struct PGroup {
    int region;
    int nk;
    int zi[kMaxGroup];
};

// output GEMM of stage 2: E[r][col][c] = sum_m T[r][c][m] F[m][col]
scw_status sep_synth(scw_ctx ctx, const float2* T, const float2* F, int nrows, int ncols, int Mk, float* out,
                     int method);
// tensor-core version (eval_sep_tc.cu); SCW_ERR_UNSUPPORTED when the shape is outside it
scw_status sep_synth_tc(scw_ctx ctx, const float2* T, const float2* F, int nrows, int ncols, int Mk, float* out,
                        int method);

}  // namespace scw

struct scw_sep_s {
    scw_ctx ctx = nullptr;
    int M0 = 0, M1 = 0, MF = 0, Z = 0, J = 0;
    int Jp = 0;                            // J rounded up to even: row stride of Q / kz on the device (zero padded)
    int rule = 0;
    std::vector<double> kx, ky, zb;
    std::vector<float> z_layers;           // Z + 1 boundaries as float (region rule)
    double* dkx = nullptr;
    double* dky = nullptr;
    double* dzb = nullptr;
    double2* dExt = nullptr;               // inc[3][MF], refl[3][MF], trans[3][MF], kz_inc, kz_refl, kz_trans
    double2* dKz = nullptr;                // [Z][2][Jp] kz of the downward / upward modes
    float2* dQ = nullptr;                  // [Z][2][3][MF][Jp] amplitudes at the modes' reference planes
    bool own_Q = false;
};
