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

// A planned evaluation of a separable set: the z-planes, their stage-1 grouping, the device
// descriptor block (groups, exterior planes, z-values) and the scratch it needs.
struct SepEvalPlan {
    int kind = 0, Na = 0, Nb = 0, Nz = 0, method = 0;
    float a0 = 0, b0 = 0, c = 0, da = 0, db = 0, dz = 0;
    std::vector<float> zlist;
    std::vector<PGroup> groups;
    std::vector<int2> ext;
    int max_nk = 1;
    size_t off_e = 0, off_z = 0, desc_bytes = 0;
    int nrows = 0, ncols = 0, Mk = 0;
    size_t phi_bytes = 0, c_bytes = 0, t_bytes = 0, tab_bytes = 0, scratch_bytes = 0;
};
// kind 0: Nz xy planes (a = x, b = y); 1: xz plane at y = c; 2: yz plane at x = c
scw_status sep_eval_plan(const scw_sep_s* s, int kind, float a0, float b0, float c, float da, float db, float dz,
                         int Na, int Nb, int Nz, int method, SepEvalPlan& p);
void sep_eval_desc(const SepEvalPlan& p, char* host);
// launches only, on the set's context stream
scw_status sep_eval_record(scw_sep_s* s, const SepEvalPlan& p, const char* d_desc, char* scratch, float* dE);

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
    // Interior amplitudes, in one of two forms:
    //   halves = 2: dQ [Z][2][3][MF][Jp], the downward and upward blocks Q_dn, Q_up as given;
    //   halves = 1 ("paired"): dQ [Z][3][MF][Jp] holds one block V and dBeta [Z][2][Jp] the mode
    //     amplitudes, with Q_dn = V diag(beta_dn) and Q_up = S V diag(beta_up), S = diag(+1, +1, -1)
    //     over (Ex, Ey, Ez) -- the structure of the solver's modes, whose E rows are the same
    //     eigenvector for the two roots +-gamma and whose H rows (hence Ez) change sign.
    int halves = 2;
    // contraction tile shape: 0 = the default rows per warp for the launch's planes per group
    // (8, 8, 4, 2 for 1, 2, 4, 8 planes), 1 = half as many rows per warp (twice the CTAs);
    // chosen by the batch autotuner
    int ctr_shape = 0;
    float2* dQ = nullptr;
    double2* dBeta = nullptr;
    bool own_Q = false;
    // host-streamed evaluation (scw_sep_eval_volume_host): copy streams, events, output slabs
    cudaStream_t up_stream = nullptr, down_stream = nullptr;
    std::vector<cudaEvent_t> events;
    // pipelined device volumes: stage 2 of one chunk of planes on hi_stream (high priority) while
    // stage 1 of the next runs on the context stream
    cudaStream_t hi_stream = nullptr;
    std::vector<cudaEvent_t> pevents;
    int pipe_chunks = 0;                   // chunks of a pipelined slab (0 or 1: one pass)
    int pipe_synth_div = 2;                // the pipelined output GEMM runs on sm_count / pipe_synth_div SMs
    void* dslab = nullptr;                 // output slab ring (device)
    size_t slab_bytes = 0;
    size_t chunk_bytes = 0, slab_target = 0;   // scw_sep_set_streaming (0: defaults)
};
