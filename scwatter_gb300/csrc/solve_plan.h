// Planning / recording interface of the GPU coupled-wave solve (solve.cu), shared by the
// single-sample entry point and the batched graph (batch.cu).
//
// A solve is split into
//   plan_solve    host only: harmonic counts, k grids, incident field, twiddle tables
//   carve         the device buffers, carved from caller-provided blocks (or sized, base = null)
//   upload_inputs host -> device copies of the sample and the plan's tables
//   record_solve  launches only: no allocation, no host synchronisation, no host reads, so a
//                 stream capture of it is a valid CUDA graph
// The status words (eigen-solver convergence, zero pivots) stay on the device and are read
// after the stream (or graph) has finished.
#pragma once

#include <complex>
#include <vector>

#include "scw_dense.h"
#include "scw_eigmix.h"

namespace scw {
namespace sv {

using cd = std::complex<double>;

struct SolvePlan {
    int Z = 0, Y = 0, X = 0;
    int M0 = 0, M1 = 0, MF = 0, n = 0;      // n = 2 MF
    double k = 0, n0 = 1, n1 = 1;
    bool external = false, pz = true;
    bool eig_mixed = true;                  // FP32 QR + FP64 refinement (else FP64 QR throughout)
    bool wide_hess = false;                 // Hessenberg reductions over the whole GPU (single solves)
    std::vector<double> zb, dz;             // Z + 1 boundaries, Z thicknesses
    std::vector<int> ps, qs;                // integer harmonic series
    std::vector<double> up, wq;             // k grids (reference PI)
    std::vector<double> up_pz, wq_pz;       // per harmonic m = q M0 + p (M_PI), Ez step
    std::vector<double> Sx, Sy;             // flattened meshes (column-major, sCWatter.cpp:677-680)
    std::vector<cd> Sz0, Sz1, EF, f1EF;     // MF, MF, 3MF, 4MF
    std::vector<cd> tw1, tw2;               // DFT twiddles of the cropped bins: [Y][M1], [M0][X]
};

// bump allocator over one device block; base == nullptr only measures
struct Carver {
    char* base = nullptr;
    size_t off = 0;
    template <typename T>
    T* take(size_t count) {
        off = (off + 255) / 256 * 256;
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += std::max<size_t>(count, 1) * sizeof(T);
        return p;
    }
};

struct SolveIn {                            // uploaded once
    double2 *data, *tw1, *tw2, *Sz0, *Sz1, *f1EF, *EF;
    int *qs, *ps;
    double *up, *wq, *dz, *Sx, *Sy, *uppz, *wqpz;
};

struct SolveWs {                            // scratch, reusable once the solve has finished
    double2 *coef, *P, *Q, *PQ, *U, *W, *lam, *E, *beta, *v;
    int* piv;
    // temporary region: DFT stage (data planes, T) / cascade + boundary (X, A1, A2, A, b) / modes (Kn, Hm, Qtmp)
    double2 *F, *T, *X, *A1, *A2, *A, *b, *Kn, *Hm, *Qtmp;
    // mixed-precision eigen-solver: FP32 slots overlay P and W (free during the eigen-solve)
    mx::EigMixWs mix;
};

struct SolveOut {                           // results
    double2* x;                             // 6MF
    double2* gam;                           // Z x 2MF
    int* status;                            // [0, Z): eigen-solver, [Z, 2Z): U pivots, [2Z, 3Z): W pivots, [3Z]: boundary
    double2* Q64;                           // [Z][2][3MF][2MF] FP64 mode amplitudes, or null
    float2* Qsep;                           // [Z][2][3][MF][2MF] complex64 (separable layout), or null
    double2* sepKz;                         // [Z][2][2MF] kz = +-gamma k for the separable set, or null
    double2* sepExt;                        // [12 MF] exterior blocks of the separable set, or null
    float2* Vsep = nullptr;                 // [Z][3][MF][2MF] complex64 mode block V of the paired set, or null
    double2* sepBeta = nullptr;             // [Z][2][2MF] its amplitudes beta_dn, beta_up (with Vsep)
    int* eig;                               // mixed eigen-solver per slice: [0, Z) state, [Z, 2Z) steps, or null
    double* eig_res;                        // [Z] last relative residual, or null
};

// Summary of the mixed eigen-solver's per-slice record (state 1 = accepted): accepted slices,
// most steps, largest accepted residual, FP64 residual GEMMs issued.
struct EigSummary {
    int accepted = 0, max_steps = -1, checks = 0;
    double max_res = 0.0;
};
EigSummary eig_summary(const int* state, const int* steps, const double* res, int Z);

scw_status plan_solve(const scw_solve_params* prm, int Z, int Y, int X, SolvePlan& p);
void carve_in(const SolvePlan& p, Carver& c, SolveIn& in);
void carve_ws(const SolvePlan& p, Carver& c, SolveWs& ws);
void carve_out(const SolvePlan& p, Carver& c, SolveOut& out, bool q64, bool sep);
scw_status upload_inputs(const SolvePlan& p, const double* sample, const SolveIn& in, cudaStream_t st);
// number of kernels launched is added to *launches
scw_status record_solve(const SolvePlan& p, const SolveIn& in, const SolveWs& ws, const SolveOut& out,
                        cudaStream_t st, long long* launches);

}  // namespace sv
}  // namespace scw
