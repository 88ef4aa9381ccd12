// Per-layer coupled-wave solve on the GPU in FP64: the computation of the reference program
// sCWatter (sCWatter.cpp:569-885, FourierWave.h:152-397), producing the reflected and
// transmitted amplitudes and the per-slice mode amplitudes that the evaluators consume.
//
// Reduced eigenproblem.  Per slice the reference builds the 4MF x 4MF matrix
// Phi = [[0, P], [Q, 0]] (FourierWave.h:336-397) and runs zgeev on it.  Phi^2 = diag(PQ, QP),
// so here the 2MF x 2MF matrix PQ is decomposed instead: PQ u = lambda u gives the two Phi
// modes gamma = +-sqrt(lambda) with eigenvectors [u; +-Q u / gamma].  The member the
// reference files in its even ("downward") slots, i.e. the larger imaginary part
// (sCWatter.cpp:185-225), is the root with Im > 0 (Re > 0 when Im == 0).  With U = [u_j],
// W = [Q u_j / gamma_j], E = diag(exp(i k gamma dz)) and V = [[U, U], [W, -W]]:
//   Gd = V diag(I, E),  Gc = V diag(E, I)                         (sCWatter.cpp:281-316)
//   V^-1 = 1/2 [[U^-1, W^-1], [U^-1, -W^-1]]
// so every product with Gd, Gc or their inverses is two 2MF GEMMs plus an elementwise mix.
//
// Boundary system.  The reference forms Gc_static = Gc_{Z-1} Gd_{Z-1}^-1 ... Gc_1 Gd_1^-1 Gc_0
// (sCWatter.cpp:321-330) and then needs Gd_0 Gc_static^-1 f3 (:393-461).  That product equals
//   prod_{l = 0 .. Z-1} [V_l diag(E_l^-1, E_l) V_l^-1]  f3
// which is applied here from the right to the 4MF x 3MF matrix f3: no 4MF x 4MF matrix is
// formed or inverted.  The 6MF system (:722), the beta recursion (:743-777), Q_check / Q_hat
// and the Ez rows from the magnetic field (:781-871) follow the reference, including its index
// conventions (column-major flattening of the Sx / Sy meshes, wrapped harmonic differences,
// the column-major read of the 1/n^2 coefficients in the Ez step).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include <string>

#include "scw_dense.h"
#include "scw_sep.h"
#include "solve_plan.h"

using cd = std::complex<double>;

struct scw_solution_s {
    scw_ctx ctx = nullptr;
    int M0 = 0, M1 = 0, MF = 0, Z = 0;
    double k = 0, n0 = 1, n1 = 1;
    bool external = false;
    std::vector<double> zb;                // Z + 1 boundaries
    std::vector<double> Sx, Sy;            // direction components of the flattened meshes
    std::vector<cd> Sz0, Sz1, EF, x;       // MF, MF, 3MF incident, 6MF boundary solution
    std::vector<cd> gam;                   // Z x 2MF downward roots
    double2* dQ = nullptr;                 // device [Z][2][3MF][2MF]: Q_check, Q_hat (FP64)
    float2* dV = nullptr;                  // device [Z][3][MF][2MF] complex64: the paired set's block V
    double2* dBeta = nullptr;              // device [Z][2][2MF]: beta_dn, beta_up
    // mixed eigen-solver per slice: state (1 accepted, else FP64 fallback), refinement steps
    // used, last relative residual; empty when the FP64 solver ran throughout
    std::vector<int> eig_state, eig_steps;
    std::vector<double> eig_res;
    ~scw_solution_s() {
        if (dQ || dV || dBeta) {
            ::scw::DeviceScope dev_scope_(ctx->device);
            if (dQ) cudaFree(dQ);
            if (dV) cudaFree(dV);
            if (dBeta) cudaFree(dBeta);
        }
    }
};

namespace scw {
namespace sv {

constexpr double kPiRef = 3.141592653;     // the reference's PI (FourierWave.h:18)

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cinv(double2 a) {
    const double d = a.x * a.x + a.y * a.y;
    return make_double2(a.x / d, -a.y / d);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 chalf(double2 a) { return make_double2(0.5 * a.x, 0.5 * a.y); }

// n^2 and n^-2 of every sample value, two planes per slice
__global__ void n2_kernel(const double2* __restrict__ data, long long per, int Z, double2* __restrict__ F) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= per * Z) return;
    const int l = (int)(e / per);
    const long long i = e % per;
    const double2 n = data[e];
    const double2 n2 = cmul(n, n);
    F[(2LL * l) * per + i] = n2;
    F[(2LL * l + 1) * per + i] = cinv(n2);
}

// P (rows Ex, Ey; columns Hx, Hy) and Q (rows Hx, Hy; columns Ex, Ey) of Phi
// (FourierWave.h:359-394); harmonic m = q M0 + p.  coef: per slice the M1 x M0 crops of
// n^2 and n^-2, stored column-major (index a + b M1).
__global__ void build_pq_kernel(const double2* __restrict__ coef, const double* __restrict__ up,
                                const double* __restrict__ wq, const int* __restrict__ qs, const int* __restrict__ ps,
                                int M0, int M1, double k, double2* __restrict__ P, double2* __restrict__ Qm) {
    const int l = blockIdx.z;
    const int MF = M0 * M1, n = 2 * MF;
    const int i = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double2* Nf = coef + (long long)l * 2 * MF;
    const double2* Ni = Nf + MF;
    const int mi = i % MF, mj = j % MF;
    const int qi = mi / M0, pi_ = mi % M0, qj = mj / M0, pj = mj % M0;
    // wrapped index differences with C++ remainders (FourierWave.h:366-372)
    const int R = ((((qs[qi] % M1) - (qs[qj] % M1) + M1) % M1) + M1 / 2) % M1;
    const int C = ((((ps[pi_] % M0) - (ps[pj] % M0) + M0) % M0) + M0 / 2) % M0;
    const double2 nf = Nf[R + C * M1], ni = Ni[R + C * M1];
    const double kin = 1.0 / (k * k);
    const double upi = up[pi_], wqi = wq[qi], upj = up[pj], wqj = wq[qj];
    const bool bi = i >= MF, bj = j >= MF;
    const double d = (mi == mj) ? 1.0 : 0.0;
    double2 p, q;
    if (!bi && !bj) p = make_double2(upi * kin * wqj * ni.x, upi * kin * wqj * ni.y);
    else if (!bi && bj) p = make_double2(-upi * kin * upj * ni.x + d, -upi * kin * upj * ni.y);
    else if (bi && !bj) p = make_double2(wqi * kin * wqj * ni.x - d, wqi * kin * wqj * ni.y);
    else p = make_double2(-wqi * kin * upj * ni.x, -wqi * kin * upj * ni.y);
    if (!bi && !bj) q = make_double2(-upi * wqi * kin * d, 0.0);
    else if (!bi && bj) q = make_double2(-nf.x + upi * upi * kin * d, -nf.y);
    else if (bi && !bj) q = make_double2(nf.x - wqi * wqi * kin * d, nf.y);
    else q = make_double2(upi * wqi * kin * d, 0.0);
    const long long o = ((long long)l * n + i) * n + j;
    P[o] = p;
    Qm[o] = q;
}

// gamma = sqrt(lambda) with Im > 0 (Re > 0 when Im == 0);  E = exp(i k gamma dz)
__global__ void roots_kernel(const double2* __restrict__ lam, int n, int Z, const double* __restrict__ dz, double k,
                             double2* __restrict__ gam, double2* __restrict__ E) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)n * Z) return;
    const int l = (int)(e / n);
    const double2 root = zsqrt(lam[e]);
    double gr = root.x, gi = root.y;
    if (gi < 0 || (gi == 0 && gr < 0)) {
        gr = -gr;
        gi = -gi;
    }
    gam[e] = make_double2(gr, gi);
    const double m = exp(-k * gi * dz[l]);
    double s, c;
    sincos(k * gr * dz[l], &s, &c);
    E[e] = make_double2(m * c, m * s);
}

// X[b][:, j] /= f[b][j]
__global__ void coldiv_kernel(double2* __restrict__ X, int n, const double2* __restrict__ f, int batch) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * n;
    if (e >= per * batch) return;
    const int b = (int)(e / per), j = (int)(e % n);
    X[e] = cmul(X[e], cinv(f[(long long)b * n + j]));
}

__global__ void identity_kernel(double2* __restrict__ X, int n, int batch) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n * n;
    if (e >= per * batch) return;
    const long long r = e % per;
    X[e] = make_double2((r / n) == (r % n) ? 1.0 : 0.0, 0.0);
}

// [Yt; Yb] from A1 = U^-1 Xt, A2 = W^-1 Xb (rows i scaled by E_i):
//   mode 0 (Gd Gc^-1 step):  Yt = E^-1 (A1 + A2)/2,  Yb = E (A1 - A2)/2,
//                            then St = Yt + Yb,  Sb = Yt - Yb   (written over A1, A2)
//   mode 1 (Gd^-1):          A1 <- (A1 + A2)/2,  A2 <- E^-1 (A1 - A2)/2
//   mode 2 (Gc):             A1 <- E A1 + A2,    A2 <- E A1 - A2
__global__ void mix_kernel(double2* __restrict__ A1, double2* __restrict__ A2, const double2* __restrict__ E, int n,
                           int ncol, int mode) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)n * ncol) return;
    const int i = (int)(e / ncol);
    const double2 a1 = A1[e], a2 = A2[e], Ei = E[i];
    if (mode == 0) {
        const double2 yt = cmul(cinv(Ei), chalf(cadd(a1, a2)));
        const double2 yb = cmul(Ei, chalf(csub(a1, a2)));
        A1[e] = cadd(yt, yb);
        A2[e] = csub(yt, yb);
    } else if (mode == 1) {
        A1[e] = chalf(cadd(a1, a2));
        A2[e] = cmul(cinv(Ei), chalf(csub(a1, a2)));
    } else {
        const double2 ea = cmul(Ei, a1);
        A1[e] = cadd(ea, a2);
        A2[e] = csub(ea, a2);
    }
}

// f3 (4MF x 3MF, sCWatter.cpp:372-389)
__global__ void f3_kernel(const double* __restrict__ Sx, const double* __restrict__ Sy, const double2* __restrict__ Sz1,
                          int MF, double2* __restrict__ F) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int ncol = 3 * MF;
    if (e >= 4LL * MF * ncol) return;
    const int r = (int)(e / ncol), c = (int)(e % ncol);
    const int blk = r / MF, m = r % MF;
    double2 v = make_double2(0, 0);
    if (blk == 0 && c == m) v = make_double2(-1, 0);
    else if (blk == 1 && c == MF + m) v = make_double2(-1, 0);
    else if (blk == 2 && c == MF + m) v = Sz1[m];
    else if (blk == 2 && c == 2 * MF + m) v = make_double2(-Sy[m], 0);
    else if (blk == 3 && c == m) v = make_double2(-Sz1[m].x, -Sz1[m].y);
    else if (blk == 3 && c == 2 * MF + m) v = make_double2(Sx[m], 0);
    F[e] = v;
}

// the 6MF x 6MF boundary matrix (sCWatter.cpp:143-146, 393-461): divergence constraints,
// then [f2 | T3] with T3 = Gd_0 Gc_static^-1 f3 (4MF x 3MF)
__global__ void bc_matrix_kernel(const double* __restrict__ Sx, const double* __restrict__ Sy,
                                 const double2* __restrict__ Sz0, const double2* __restrict__ Sz1,
                                 const double2* __restrict__ T3, int MF, double2* __restrict__ A) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int N6 = 6 * MF;
    if (e >= (long long)N6 * N6) return;
    const int r = (int)(e / N6), c = (int)(e % N6);
    double2 v = make_double2(0, 0);
    if (r < MF) {
        const int m = r;
        if (c == m) v = make_double2(Sx[m], 0);
        else if (c == MF + m) v = make_double2(Sy[m], 0);
        else if (c == 2 * MF + m) v = make_double2(-Sz0[m].x, -Sz0[m].y);
    } else if (r < 2 * MF) {
        const int m = r - MF;
        if (c == 3 * MF + m) v = make_double2(Sx[m], 0);
        else if (c == 4 * MF + m) v = make_double2(Sy[m], 0);
        else if (c == 5 * MF + m) v = Sz1[m];
    } else {
        const int rr = r - 2 * MF;
        if (c >= 3 * MF) {
            v = T3[(long long)rr * 3 * MF + (c - 3 * MF)];
        } else {
            const int blk = rr / MF, m = rr % MF;
            if (blk == 0 && c == m) v = make_double2(1, 0);
            else if (blk == 1 && c == MF + m) v = make_double2(1, 0);
            else if (blk == 2 && c == MF + m) v = Sz0[m];
            else if (blk == 2 && c == 2 * MF + m) v = make_double2(Sy[m], 0);
            else if (blk == 3 && c == m) v = make_double2(-Sz0[m].x, -Sz0[m].y);
            else if (blk == 3 && c == 2 * MF + m) v = make_double2(-Sx[m], 0);
        }
    }
    A[e] = v;
}

// Kn[m_i][m_j] = scale * NIf[lin] with lin the wrapped difference index read column-major
// (sCWatter.cpp:839-871 reads NIf(lin) on a column-major Eigen matrix)
__global__ void kn_kernel(const double2* __restrict__ NiF, int M0, int M1, double scale, double2* __restrict__ Kn) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int MF = M0 * M1;
    if (e >= (long long)MF * MF) return;
    const int mi = (int)(e / MF), mj = (int)(e % MF);
    const int qi = mi / M0, pi_ = mi % M0, qj = mj / M0, pj = mj % M0;
    const int lin = (((qi - qj + M1) % M1 + M1 / 2) % M1) * M0 + ((pi_ - pj + M0) % M0 + M0 / 2) % M0;
    const double2 v = NiF[lin];
    Kn[e] = make_double2(v.x * scale, v.y * scale);
}

// rows Ex, Ey of Q_check / Q_hat: U diag(beta);  Hm = sign (up_m Hy - wq_m Hx) for the Ez step,
// with Hx, Hy = rows of W diag(beta) (sign -1 for the upward modes, whose H rows are -W).
// beta == null: unit amplitudes (the paired set's block V = [U; Kn (up W_y - wq W_x)])
__global__ void q_rows_kernel(const double2* __restrict__ U, const double2* __restrict__ Wm,
                              const double2* __restrict__ beta, int MF, double sign, const double* __restrict__ up_pz,
                              const double* __restrict__ wq_pz, double2* __restrict__ Qout, double2* __restrict__ Hm) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = 2 * MF;
    if (e >= (long long)n * n) return;
    const int r = (int)(e / n), j = (int)(e % n);
    const double2 b = beta ? beta[j] : make_double2(1.0, 0.0);
    Qout[e] = cmul(U[e], b);
    if (Hm && r < MF) {
        const double2 hx = cmul(Wm[e], b);
        const double2 hy = cmul(Wm[(long long)(MF + r) * n + j], b);
        Hm[e] = make_double2(sign * (up_pz[r] * hy.x - wq_pz[r] * hx.x), sign * (up_pz[r] * hy.y - wq_pz[r] * hx.y));
    }
}

__global__ void to_c64_kernel(const double2* __restrict__ a, float2* __restrict__ b, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) b[e] = make_float2((float)a[e].x, (float)a[e].y);
}

// b = [0 (2MF); -f1 EF (4MF)]  (sCWatter.cpp:459-460)
__global__ void bc_rhs_kernel(const double2* __restrict__ f1EF, int MF, double2* __restrict__ b) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 6 * MF) return;
    b[e] = e < 2 * MF ? make_double2(0.0, 0.0) : make_double2(-f1EF[e - 2 * MF].x, -f1EF[e - 2 * MF].y);
}

// v = f1 EF + f2 R with R = x[0, 3MF)  (sCWatter.cpp:745-747)
__global__ void beta_init_kernel(const double2* __restrict__ f1EF, const double2* __restrict__ x,
                                 const double* __restrict__ Sx, const double* __restrict__ Sy,
                                 const double2* __restrict__ Sz0, int MF, double2* __restrict__ v) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= MF) return;
    const double2 rx = x[m], ry = x[MF + m], rz = x[2 * MF + m], s0 = Sz0[m];
    v[m] = cadd(f1EF[m], rx);
    v[MF + m] = cadd(f1EF[MF + m], ry);
    v[2 * MF + m] = cadd(cadd(f1EF[2 * MF + m], cmul(s0, ry)), make_double2(Sy[m] * rz.x, Sy[m] * rz.y));
    v[3 * MF + m] = csub(csub(f1EF[3 * MF + m], cmul(s0, rx)), make_double2(Sx[m] * rz.x, Sx[m] * rz.y));
}

// kz of the separable set: [l][0][j] = gamma k, [l][1][j] = -gamma k
__global__ void sep_kz_kernel(const double2* __restrict__ gam, int Z, int n, double k, double2* __restrict__ kz) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Z * n) return;
    const int l = (int)(e / n), j = (int)(e % n);
    const double2 g = gam[e];
    kz[((long long)l * 2) * n + j] = make_double2(g.x * k, g.y * k);
    kz[((long long)l * 2 + 1) * n + j] = make_double2(-g.x * k, -g.y * k);
}

// exterior blocks of the separable set: incident, reflected, transmitted amplitudes [3][MF]
// each, then kz of the three (reflected -Sz0 k n0, transmitted Sz1 k n1: sCWatter.cpp:471-475)
__global__ void sep_ext_kernel(const double2* __restrict__ EF, const double2* __restrict__ x,
                               const double2* __restrict__ Sz0, const double2* __restrict__ Sz1, int MF, double k,
                               double n0, double n1, double2* __restrict__ ext) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * MF) return;
    ext[e] = EF[e];
    ext[3 * MF + e] = x[e];
    ext[6 * MF + e] = x[3 * MF + e];
    if (e < MF) {
        const double2 a = Sz0[e], b = Sz1[e];
        ext[9 * MF + e] = make_double2(a.x * k, a.y * k);
        ext[10 * MF + e] = make_double2(-a.x * k * n0, -a.y * k * n0);
        ext[11 * MF + e] = make_double2(b.x * k * n1, b.y * k * n1);
    }
}

static unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// FourierWave.h:82-145: the source index of each shifted row / column, including the column
// index it builds when the row count is even and the column count odd
static void fft_shift_index(int m, int n, std::vector<int>& indx, std::vector<int>& indy) {
    int p, q;
    if (m % 2 == 1) {
        p = m / 2;
        q = n / 2;
    } else {
        p = (m + 1) / 2;
        q = (n + 1) / 2;
    }
    indx.resize(m);
    indy.resize(n);
    for (int i = 0; i < m; i++) {
        if (m % 2 == 1) indx[i] = i < m - p - 1 ? (m - p) + i : i - (m - p - 1);
        else indx[i] = i < m - p ? p + i : i - (m - p);
    }
    for (int i = 0; i < n; i++) {
        if (n % 2 == 1) indy[i] = i < n - q - 1 ? (n - q) + i : i - (n - q - 1);
        else indy[i] = i < n - q ? q + i : i - (n - q);
    }
}

#define SCW_TRY(expr)                          \
    do {                                       \
        const scw_status s_ = (expr);          \
        if (s_ != SCW_OK) return s_;           \
    } while (0)

const double2 kOne = {1.0, 0.0};
const double2 kZero = {0.0, 0.0};

// ---------------------------------------------------------------------------------------
// Planning (host): sCWatter.cpp:569-680
// ---------------------------------------------------------------------------------------
scw_status plan_solve(const scw_solve_params* prm, int Zs, int Y, int X, SolvePlan& p) {
    if (!prm || Zs < 1 || Y < 1 || X < 1) return fail(SCW_ERR_ARG, "scw_solve: bad arguments");
    if (!(prm->lambda > 0) || !(prm->size[0] > 0) || !(prm->size[1] > 0) || !(prm->size[2] > 0))
        return fail(SCW_ERR_ARG, "scw_solve: wavelength and sizes must be positive");
    const double dn = std::sqrt(prm->direction[0] * prm->direction[0] + prm->direction[1] * prm->direction[1] +
                                prm->direction[2] * prm->direction[2]);
    if (!(dn > 0)) return fail(SCW_ERR_ARG, "scw_solve: zero direction");
    const double dvec[3] = {prm->direction[0] / dn, prm->direction[1] / dn, prm->direction[2] / dn};
    cd e[3] = {cd(prm->ex[0], prm->ex[1]), cd(prm->ey[0], prm->ey[1]), cd(prm->ez[0], prm->ez[1])};
    {   // orthogonalize (FourierWave.h:32-39): |E| is the complex sqrt of sum(E_i^2)
        const cd mag = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        for (auto& c : e) c /= mag;
        const cd d[3] = {dvec[0], dvec[1], dvec[2]};
        const cd s[3] = {e[1] * d[2] - e[2] * d[1], e[2] * d[0] - e[0] * d[2], e[0] * d[1] - e[1] * d[0]};
        e[0] = d[1] * s[2] - d[2] * s[1];
        e[1] = d[2] * s[0] - d[0] * s[2];
        e[2] = d[0] * s[1] - d[1] * s[0];
    }
    const double n0 = prm->n[0], n1r = prm->n[1];
    const double dir[3] = {dvec[0] * n0, dvec[1] * n0, dvec[2] * n0};
    const double k = 2 * kPiRef / prm->lambda;
    const cd ni0(n0, 0.0), ni1(n1r, prm->kappa);
    const int ZL = Zs + 1;
    p.Z = Zs;
    p.Y = Y;
    p.X = X;
    p.k = k;
    p.n0 = n0;
    p.n1 = n1r;
    p.external = prm->external != 0;
    p.pz = prm->pz != 0;
    p.eig_mixed = prm->eig_fp64 == 0 && 2 * (long long)p.MF <= mx::kMaxN;
    p.zb.resize(ZL);
    p.zb[0] = prm->z - prm->size[2] / 2.0;
    for (int i = 1; i < ZL; i++) p.zb[i] = p.zb[i - 1] + prm->size[2] / Zs;
    p.dz.resize(Zs);
    for (int l = 0; l < Zs; l++) p.dz[l] = (Zs == 1) ? p.zb[ZL - 1] - p.zb[0] : p.zb[l + 1] - p.zb[l];
    int M0 = prm->coef[0] > 0 ? prm->coef[0] : X, M1 = prm->coef[1] > 0 ? prm->coef[1] : Y;
    {   // harmonic count clamping (sCWatter.cpp:607-645)
        const double lam = prm->lambda;
        auto sq = [](double v) { return v * v; };
        if (sq(double(M0 / 2) / prm->size[0] * lam + dir[0]) + sq(double(M1 / 2) / prm->size[1] * lam + dir[1]) >=
            n0 * n0) {
            if (M0 != 1 && M1 != 1) {
                if ((double(M0 / 2) / prm->size[0] * lam + dir[0]) > 0.71 * n0)
                    M0 = int(0.707 * n0 * 2 * prm->size[0] / lam) - 1;
                if ((double(M1 / 2) / prm->size[1] * lam + dir[1]) > 0.71 * n0)
                    M1 = int(0.707 * n1r * 2 * prm->size[1] / lam) - 1;
            }
            if (M0 == 1 && (double(M1 / 2) / prm->size[1] * lam + std::fabs(dir[1])) >= n0) {
                M1 = int(n1r * 2 * prm->size[1] / lam - 1e-10);
                if (M1 % 2 == 0) M1 -= 1;
            }
            if (M1 == 1 && (double(M0 / 2) / prm->size[1] * lam + std::fabs(dir[0])) >= n0) {
                M0 = int(n0 * 2 * prm->size[0] / lam - 1e-10);
                if (M0 % 2 == 0) M0 -= 1;
            }
        }
        M0 = std::min(M0, X);
        M1 = std::min(M1, Y);
        if (M0 < 1 || M1 < 1) return fail(SCW_ERR_ARG, "scw_solve: no Fourier coefficients left after clamping");
    }
    const int MF = M0 * M1;
    if ((long long)6 * MF * 6 * MF > (1LL << 31)) return fail(SCW_ERR_ARG, "scw_solve: too many Fourier coefficients");
    p.M0 = M0;
    p.M1 = M1;
    p.MF = MF;
    p.n = 2 * MF;
    // k grids (FourierWave.h:319-334): integer series -(M/2) .. (M-1)/2
    p.ps.resize(M0);
    p.qs.resize(M1);
    p.up.resize(M0);
    p.wq.resize(M1);
    for (int i = 0; i < M0; i++) {
        p.ps[i] = -(M0 / 2) + i;
        p.up[i] = 2 * kPiRef * p.ps[i] / prm->size[0] + dir[0] * k;
    }
    for (int i = 0; i < M1; i++) {
        p.qs[i] = -(M1 / 2) + i;
        p.wq[i] = 2 * kPiRef * p.qs[i] / prm->size[1] + dir[1] * k;
    }
    p.up_pz.resize(MF);
    p.wq_pz.resize(MF);
    for (int m = 0; m < MF; m++) {      // the Ez step builds its grids with M_PI (sCWatter.cpp:806-812)
        p.up_pz[m] = 2.0 * p.ps[m % M0] * M_PI / prm->size[0] + dir[0] * k;
        p.wq_pz[m] = 2.0 * p.qs[m / M0] * M_PI / prm->size[1] + dir[1] * k;
    }
    p.Sx.resize(MF);
    p.Sy.resize(MF);
    p.Sz0.resize(MF);
    p.Sz1.resize(MF);
    for (int f = 0; f < MF; f++) {      // column-major flattening of the M1 x M0 meshes
        const double sx = p.up[f / M1] / k, sy = p.wq[f % M1] / k;
        p.Sx[f] = sx;
        p.Sy[f] = sy;
        p.Sz0[f] = std::sqrt(ni0 * ni0 - cd(sx * sx) - cd(sy * sy));
        p.Sz1[f] = std::sqrt(ni1 * ni1 - cd(sx * sx) - cd(sy * sy));
    }
    // the DFT rows / columns that land in the centred crop after the shift
    std::vector<int> ix, iy;
    fft_shift_index(Y, X, ix, iy);
    const int r0 = Y / 2 - M1 / 2, c0 = X / 2 - M0 / 2;
    std::vector<int> du(M1), dv(M0);
    for (int a = 0; a < M1; a++) du[a] = ix[r0 + a];
    for (int b = 0; b < M0; b++) dv[b] = iy[c0 + b];
    // incident field: the transform of a constant lands on the DC bin (sCWatter.cpp:656-674);
    // --psf puts E0 on every harmonic (:665-669)
    p.EF.assign(3 * MF, cd(0, 0));
    for (int c = 0; c < 3; c++)
        for (int a = 0; a < M1; a++)
            for (int b = 0; b < M0; b++)
                if (prm->psf || (du[a] == 0 && dv[b] == 0)) p.EF[c * MF + a + b * M1] = e[c];
    p.f1EF.resize(4 * MF);
    for (int m = 0; m < MF; m++) {      // f1 EF (sCWatter.cpp:334-357)
        const cd ph = std::exp(cd(0, 1) * k * p.zb[0] * p.Sz0[m]);
        const cd ex = p.EF[m], ey = p.EF[MF + m], ez = p.EF[2 * MF + m];
        p.f1EF[m] = ph * ex;
        p.f1EF[MF + m] = ph * ey;
        p.f1EF[2 * MF + m] = -ph * p.Sz0[m] * ey + ph * p.Sy[m] * ez;
        p.f1EF[3 * MF + m] = ph * p.Sz0[m] * ex - ph * p.Sx[m] * ez;
    }
    // twiddles of the cropped DFT bins, phases reduced with integers
    p.tw1.resize((size_t)Y * M1);
    p.tw2.resize((size_t)M0 * X);
    for (int r = 0; r < Y; r++)
        for (int a = 0; a < M1; a++) {
            const double t = (double)(((long long)du[a] * r) % Y) / Y;
            p.tw1[(size_t)r * M1 + a] = cd(std::cos(2 * M_PI * t), -std::sin(2 * M_PI * t));
        }
    for (int b = 0; b < M0; b++)
        for (int c = 0; c < X; c++) {
            const double t = (double)(((long long)dv[b] * c) % X) / X;
            p.tw2[(size_t)b * X + c] = cd(std::cos(2 * M_PI * t), -std::sin(2 * M_PI * t));
        }
    return SCW_OK;
}

void carve_in(const SolvePlan& p, Carver& c, SolveIn& in) {
    const int MF = p.MF;
    in.data = c.take<double2>((size_t)p.Z * p.Y * p.X);
    in.tw1 = c.take<double2>(p.tw1.size());
    in.tw2 = c.take<double2>(p.tw2.size());
    in.Sz0 = c.take<double2>(MF);
    in.Sz1 = c.take<double2>(MF);
    in.f1EF = c.take<double2>(4 * MF);
    in.EF = c.take<double2>(3 * MF);
    in.qs = c.take<int>(p.M1);
    in.ps = c.take<int>(p.M0);
    in.up = c.take<double>(p.M0);
    in.wq = c.take<double>(p.M1);
    in.dz = c.take<double>(p.Z);
    in.Sx = c.take<double>(MF);
    in.Sy = c.take<double>(MF);
    in.uppz = c.take<double>(MF);
    in.wqpz = c.take<double>(MF);
}

void carve_ws(const SolvePlan& p, Carver& c, SolveWs& ws) {
    const size_t Z = p.Z, MF = p.MF, n = p.n, nn = n * n, N4 = 4 * MF, M3 = 3 * MF, M6 = 6 * MF;
    ws.coef = c.take<double2>(Z * 2 * MF);
    ws.P = c.take<double2>(Z * (nn + 3 * n));     // P, then eigen-solver work, then U^-1
    ws.Q = c.take<double2>(Z * nn);               // Q, then LU factors
    ws.PQ = c.take<double2>(Z * nn);              // PQ, then W^-1
    ws.U = c.take<double2>(Z * nn);
    ws.W = c.take<double2>(Z * nn);
    ws.lam = c.take<double2>(Z * n);
    ws.E = c.take<double2>(Z * n);
    ws.beta = c.take<double2>(Z * N4);
    ws.v = c.take<double2>(N4);
    ws.piv = c.take<int>(std::max(Z * n, M6));
    // mixed eigen-solver: small buffers of its own; S0, S1 (adjacent), its QR work and the FP32
    // eigenvalues inside P (Z (n^2 + 3 n) double2 >= 2 Z n^2 + 4 Z n float2), S2, S3 inside W
    if (p.eig_mixed) {
        char* small = c.take<char>(mx::eigmix_small_bytes((int)n, (int)Z));
        mx::eigmix_carve_small(ws.mix, small, (int)n, (int)Z);
        float2* Pf = reinterpret_cast<float2*>(ws.P);
        float2* Wf = reinterpret_cast<float2*>(ws.W);
        ws.mix.S0 = Pf;
        ws.mix.S1 = Pf + Z * nn;
        ws.mix.hw = Pf + 2 * Z * nn;
        ws.mix.lam32 = ws.mix.hw + 3 * Z * n;
        ws.mix.S2 = Wf;
        ws.mix.S3 = Wf + Z * nn;
    }
    // temporary region, three overlays
    const size_t t0 = (c.off + 255) / 256 * 256;
    Carver ca{c.base, t0};
    ws.F = ca.take<double2>(2 * Z * (size_t)p.Y * p.X);
    ws.T = ca.take<double2>(2 * Z * (size_t)p.X * p.M1);
    Carver cc{c.base, t0};
    ws.X = cc.take<double2>(N4 * M3);
    ws.A1 = cc.take<double2>(n * M3);
    ws.A2 = cc.take<double2>(n * M3);
    const size_t tA = (cc.off + 255) / 256 * 256;
    ws.A = cc.take<double2>(M6 * M6);
    ws.b = cc.take<double2>(M6);
    Carver cm{c.base, tA};
    ws.Kn = cm.take<double2>(MF * MF);
    ws.Hm = cm.take<double2>(MF * n);
    ws.Qtmp = cm.take<double2>(M3 * n);
    c.off = std::max(ca.off, std::max(cc.off, cm.off));
}

void carve_out(const SolvePlan& p, Carver& c, SolveOut& out, bool q64, bool sep) {
    const size_t Z = p.Z, MF = p.MF, n = p.n;
    out.x = c.take<double2>(6 * MF);
    out.gam = c.take<double2>(Z * n);
    out.status = c.take<int>(3 * Z + 1);
    out.Q64 = (q64 && !p.external) ? c.take<double2>(Z * 2 * 3 * MF * n) : nullptr;
    out.Qsep = (sep && !p.external) ? c.take<float2>(Z * 2 * 3 * MF * n) : nullptr;
    out.sepKz = (sep && !p.external) ? c.take<double2>(Z * 2 * n) : nullptr;
    out.sepExt = sep ? c.take<double2>(12 * MF) : nullptr;
    out.eig = p.eig_mixed ? c.take<int>(2 * Z) : nullptr;
    out.eig_res = p.eig_mixed ? c.take<double>(Z) : nullptr;
}

EigSummary eig_summary(const int* state, const int* steps, const double* res, int Z) {
    EigSummary e;
    for (int b = 0; b < Z; b++) {
        if (state[b] == 1) {
            e.accepted++;
            e.max_steps = std::max(e.max_steps, steps[b]);
            e.max_res = std::max(e.max_res, res[b]);
            e.checks += steps[b] + 1;
        } else {
            e.checks += mx::EigMixParams{}.steps + 1;
        }
    }
    return e;
}

scw_status upload_inputs(const SolvePlan& p, const double* sample, const SolveIn& in, cudaStream_t st) {
    auto up = [&](void* dst, const void* src, size_t bytes) -> scw_status {
        SCW_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
        return SCW_OK;
    };
    const size_t MF = p.MF;
    // the sample may be in host or device memory
    SCW_CUDA_TRY(cudaMemcpyAsync(in.data, sample, sizeof(double2) * p.Z * p.Y * p.X, cudaMemcpyDefault, st));
    SCW_TRY(up(in.tw1, p.tw1.data(), sizeof(double2) * p.tw1.size()));
    SCW_TRY(up(in.tw2, p.tw2.data(), sizeof(double2) * p.tw2.size()));
    SCW_TRY(up(in.Sz0, p.Sz0.data(), sizeof(double2) * MF));
    SCW_TRY(up(in.Sz1, p.Sz1.data(), sizeof(double2) * MF));
    SCW_TRY(up(in.f1EF, p.f1EF.data(), sizeof(double2) * 4 * MF));
    SCW_TRY(up(in.EF, p.EF.data(), sizeof(double2) * 3 * MF));
    SCW_TRY(up(in.qs, p.qs.data(), sizeof(int) * p.M1));
    SCW_TRY(up(in.ps, p.ps.data(), sizeof(int) * p.M0));
    SCW_TRY(up(in.up, p.up.data(), sizeof(double) * p.M0));
    SCW_TRY(up(in.wq, p.wq.data(), sizeof(double) * p.M1));
    SCW_TRY(up(in.dz, p.dz.data(), sizeof(double) * p.Z));
    SCW_TRY(up(in.Sx, p.Sx.data(), sizeof(double) * MF));
    SCW_TRY(up(in.Sy, p.Sy.data(), sizeof(double) * MF));
    SCW_TRY(up(in.uppz, p.up_pz.data(), sizeof(double) * MF));
    SCW_TRY(up(in.wqpz, p.wq_pz.data(), sizeof(double) * MF));
    return SCW_OK;
}

// ---------------------------------------------------------------------------------------
// Recording (launches only): sCWatter.cpp:248-871 restated on the reduced problem
// ---------------------------------------------------------------------------------------
scw_status record_solve(const SolvePlan& p, const SolveIn& in, const SolveWs& ws, const SolveOut& out,
                        cudaStream_t st, long long* launches) {
    const int Zs = p.Z, Y = p.Y, X = p.X, M0 = p.M0, M1 = p.M1, MF = p.MF, n = p.n;
    const int N4 = 4 * MF, M3 = 3 * MF, M6 = 6 * MF;
    const long long nn = (long long)n * n, YX = (long long)Y * X;
    const double k = p.k;
    long long L = 0;
    // Fourier coefficients of n^2 and n^-2 (FourierWave.h:152-195, 283-301): the slice read as
    // the X x Y row-major matrix F^T (F[r][c] = data[r + c Y]); the 2-D DFT crop is
    // tw2^T (M0 x X) . (F^T (X x Y) . tw1^T (Y x M1)), the M1 x M0 crop stored column-major
    n2_kernel<<<nblk(Zs * YX), 256, 0, st>>>(in.data, YX, Zs, ws.F);
    SCW_CUDA_TRY(cudaGetLastError());
    SCW_TRY(zgemm(st, X, M1, Y, kOne, ws.F, Y, YX, in.tw1, M1, 0, kZero, ws.T, M1, (long long)X * M1, 2 * Zs));
    SCW_TRY(zgemm(st, M0, M1, X, make_double2(1.0 / (double)YX, 0.0), in.tw2, X, 0, ws.T, M1, (long long)X * M1, kZero,
                  ws.coef, M1, MF, 2 * Zs));
    // P, Q and the reduced eigenproblem
    build_pq_kernel<<<dim3(nblk(n), n, Zs), 256, 0, st>>>(ws.coef, in.up, in.wq, in.qs, in.ps, M0, M1, k, ws.P, ws.Q);
    SCW_CUDA_TRY(cudaGetLastError());
    SCW_TRY(zgemm(st, n, n, n, kOne, ws.P, n, nn, ws.Q, n, nn, kZero, ws.PQ, n, nn, Zs));
    if (p.eig_mixed) {
        mx::EigMixParams prm;
        prm.wide = p.wide_hess;
        SCW_TRY(mx::geev_mixed(st, ws.PQ, ws.lam, ws.U, n, Zs, ws.mix, ws.P, out.status, prm, &L));
        if (out.eig) {
            SCW_CUDA_TRY(cudaMemcpyAsync(out.eig, ws.mix.state, sizeof(int) * Zs, cudaMemcpyDeviceToDevice, st));
            SCW_CUDA_TRY(cudaMemcpyAsync(out.eig + Zs, ws.mix.steps, sizeof(int) * Zs, cudaMemcpyDeviceToDevice, st));
            SCW_CUDA_TRY(cudaMemcpyAsync(out.eig_res, ws.mix.res, sizeof(double) * Zs, cudaMemcpyDeviceToDevice, st));
        }
    } else {
        SCW_TRY(zgeev(st, ws.PQ, ws.lam, ws.U, n, Zs, ws.P, out.status, p.wide_hess));
        L += 5;
    }
    roots_kernel<<<nblk((long long)n * Zs), 256, 0, st>>>(ws.lam, n, Zs, in.dz, k, out.gam, ws.E);
    SCW_CUDA_TRY(cudaGetLastError());
    // W = Q U Gamma^-1
    SCW_TRY(zgemm(st, n, n, n, kOne, ws.Q, n, nn, ws.U, n, nn, kZero, ws.W, n, nn, Zs));
    coldiv_kernel<<<nblk(nn * Zs), 256, 0, st>>>(ws.W, n, out.gam, Zs);
    SCW_CUDA_TRY(cudaGetLastError());
    L += 8;
    // U^-1 into P, W^-1 into PQ (LU factors in Q)
    double2* Uinv = ws.P;
    double2* Winv = ws.PQ;
    for (int which = 0; which < 2; which++) {
        double2* inv = which == 0 ? Uinv : Winv;
        identity_kernel<<<nblk(nn * Zs), 256, 0, st>>>(inv, n, Zs);
        SCW_CUDA_TRY(cudaGetLastError());
        SCW_CUDA_TRY(cudaMemcpyAsync(ws.Q, which == 0 ? ws.U : ws.W, sizeof(double2) * nn * Zs,
                                     cudaMemcpyDeviceToDevice, st));
        SCW_TRY(zgetrf(st, ws.Q, n, nn, ws.piv, n, out.status + (1 + which) * Zs, Zs, nullptr));
        SCW_TRY(zgetrs(st, ws.Q, n, nn, ws.piv, n, inv, n, nn, Zs));
        L += 2 + 3 * ((n + 31) / 32);
    }
    // T3 = Gd_0 Gc_static^-1 f3 = prod_l V_l diag(E_l^-1, E_l) V_l^-1 f3
    f3_kernel<<<nblk((long long)N4 * M3), 256, 0, st>>>(in.Sx, in.Sy, in.Sz1, MF, ws.X);
    SCW_CUDA_TRY(cudaGetLastError());
    for (int l = Zs - 1; l >= 0; l--) {
        const long long o = (long long)l * nn;
        SCW_TRY(zgemm(st, n, M3, n, kOne, Uinv + o, n, 0, ws.X, M3, 0, kZero, ws.A1, M3, 0, 1));
        SCW_TRY(zgemm(st, n, M3, n, kOne, Winv + o, n, 0, ws.X + (size_t)n * M3, M3, 0, kZero, ws.A2, M3, 0, 1));
        mix_kernel<<<nblk((long long)n * M3), 256, 0, st>>>(ws.A1, ws.A2, ws.E + (size_t)l * n, n, M3, 0);
        SCW_CUDA_TRY(cudaGetLastError());
        SCW_TRY(zgemm(st, n, M3, n, kOne, ws.U + o, n, 0, ws.A1, M3, 0, kZero, ws.X, M3, 0, 1));
        SCW_TRY(zgemm(st, n, M3, n, kOne, ws.W + o, n, 0, ws.A2, M3, 0, kZero, ws.X + (size_t)n * M3, M3, 0, 1));
        L += 5;
    }
    // boundary system and its solve (sCWatter.cpp:393-461, 722)
    bc_matrix_kernel<<<nblk((long long)M6 * M6), 256, 0, st>>>(in.Sx, in.Sy, in.Sz0, in.Sz1, ws.X, MF, ws.A);
    SCW_CUDA_TRY(cudaGetLastError());
    bc_rhs_kernel<<<nblk(M6), 256, 0, st>>>(in.f1EF, MF, ws.b);
    SCW_CUDA_TRY(cudaGetLastError());
    SCW_TRY(zgetrf(st, ws.A, M6, 0, ws.piv, 0, out.status + 3 * Zs, 1, nullptr));
    SCW_TRY(zgetrs(st, ws.A, M6, 0, ws.piv, 0, ws.b, 1, 0, 1));
    SCW_CUDA_TRY(cudaMemcpyAsync(out.x, ws.b, sizeof(double2) * M6, cudaMemcpyDeviceToDevice, st));
    L += 4 + 3 * ((M6 + 31) / 32);
    if (out.sepExt) {
        sep_ext_kernel<<<nblk(M3), 256, 0, st>>>(in.EF, out.x, in.Sz0, in.Sz1, MF, k, p.n0, p.n1, out.sepExt);
        SCW_CUDA_TRY(cudaGetLastError());
        L++;
    }
    if (p.external) {
        if (launches) *launches += L;
        return SCW_OK;
    }
    // beta: beta_0 = Gd_0^-1 (f1 EF + f2 R),  beta_l = Gd_l^-1 Gc_{l-1} beta_{l-1} (sCWatter.cpp:743-777)
    beta_init_kernel<<<nblk(MF), 256, 0, st>>>(in.f1EF, out.x, in.Sx, in.Sy, in.Sz0, MF, ws.v);
    SCW_CUDA_TRY(cudaGetLastError());
    for (int l = 0; l < Zs; l++) {
        const long long o = (long long)l * nn;
        double2* bl = ws.beta + (size_t)l * N4;
        if (l > 0) {   // v = Gc_{l-1} beta_{l-1} = [U (E bt + bb); W (E bt - bb)]
            const double2* bp = ws.beta + (size_t)(l - 1) * N4;
            SCW_CUDA_TRY(cudaMemcpyAsync(ws.A1, bp, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
            SCW_CUDA_TRY(cudaMemcpyAsync(ws.A2, bp + n, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
            mix_kernel<<<nblk(n), 256, 0, st>>>(ws.A1, ws.A2, ws.E + (size_t)(l - 1) * n, n, 1, 2);
            SCW_CUDA_TRY(cudaGetLastError());
            SCW_TRY(zgemm(st, n, 1, n, kOne, ws.U + o - nn, n, 0, ws.A1, 1, 0, kZero, ws.v, 1, 0, 1));
            SCW_TRY(zgemm(st, n, 1, n, kOne, ws.W + o - nn, n, 0, ws.A2, 1, 0, kZero, ws.v + n, 1, 0, 1));
            L += 3;
        }
        SCW_TRY(zgemm(st, n, 1, n, kOne, Uinv + o, n, 0, ws.v, 1, 0, kZero, bl, 1, 0, 1));
        SCW_TRY(zgemm(st, n, 1, n, kOne, Winv + o, n, 0, ws.v + n, 1, 0, kZero, bl + n, 1, 0, 1));
        mix_kernel<<<nblk(n), 256, 0, st>>>(bl, bl + n, ws.E + (size_t)l * n, n, 1, 1);
        SCW_CUDA_TRY(cudaGetLastError());
        L += 3;
    }
    // Q_check / Q_hat with Ez from the magnetic field (sCWatter.cpp:781-871)
    for (int l = 0; l < Zs; l++) {
        const long long o = (long long)l * nn;
        if (p.pz) {
            kn_kernel<<<nblk((long long)MF * MF), 256, 0, st>>>(ws.coef + (size_t)l * 2 * MF + MF, M0, M1, -1.0 / k,
                                                                ws.Kn);
            SCW_CUDA_TRY(cudaGetLastError());
            L++;
        }
        for (int h = 0; h < 2; h++) {
            double2* Qo = out.Q64 ? out.Q64 + ((size_t)l * 2 + h) * M3 * n : ws.Qtmp;
            const double2* beta = ws.beta + (size_t)l * N4 + (h ? n : 0);
            q_rows_kernel<<<nblk(nn), 256, 0, st>>>(ws.U + o, ws.W + o, beta, MF, h ? -1.0 : 1.0, in.uppz, in.wqpz, Qo,
                                                   p.pz ? ws.Hm : nullptr);
            SCW_CUDA_TRY(cudaGetLastError());
            if (p.pz) {
                SCW_TRY(zgemm(st, MF, n, MF, kOne, ws.Kn, MF, 0, ws.Hm, n, 0, kZero, Qo + (size_t)n * n, n, 0, 1));
            } else {
                SCW_CUDA_TRY(cudaMemsetAsync(Qo + (size_t)n * n, 0, sizeof(double2) * MF * n, st));
            }
            if (out.Qsep) {
                const long long cnt = (long long)M3 * n;
                to_c64_kernel<<<nblk(cnt), 256, 0, st>>>(Qo, out.Qsep + ((size_t)l * 2 + h) * M3 * n, cnt);
                SCW_CUDA_TRY(cudaGetLastError());
                L++;
            }
            L += 2;
        }
        if (out.Vsep) {      // the paired set: V = [U; Kn (up W_y - wq W_x)] and beta_dn, beta_up
            q_rows_kernel<<<nblk(nn), 256, 0, st>>>(ws.U + o, ws.W + o, nullptr, MF, 1.0, in.uppz, in.wqpz, ws.Qtmp,
                                                   p.pz ? ws.Hm : nullptr);
            SCW_CUDA_TRY(cudaGetLastError());
            if (p.pz) {
                SCW_TRY(zgemm(st, MF, n, MF, kOne, ws.Kn, MF, 0, ws.Hm, n, 0, kZero, ws.Qtmp + (size_t)n * n, n, 0, 1));
            } else {
                SCW_CUDA_TRY(cudaMemsetAsync(ws.Qtmp + (size_t)n * n, 0, sizeof(double2) * MF * n, st));
            }
            const long long cnt = (long long)M3 * n;
            to_c64_kernel<<<nblk(cnt), 256, 0, st>>>(ws.Qtmp, out.Vsep + (size_t)l * M3 * n, cnt);
            SCW_CUDA_TRY(cudaGetLastError());
            SCW_CUDA_TRY(cudaMemcpyAsync(out.sepBeta + (size_t)l * 2 * n, ws.beta + (size_t)l * N4,
                                         sizeof(double2) * 2 * n, cudaMemcpyDeviceToDevice, st));
            L += 3;
        }
    }
    if (out.sepKz) {
        sep_kz_kernel<<<nblk((long long)Zs * n), 256, 0, st>>>(out.gam, Zs, n, k, out.sepKz);
        SCW_CUDA_TRY(cudaGetLastError());
        L++;
    }
    if (launches) *launches += L;
    return SCW_OK;
}

}  // namespace sv
}  // namespace scw

using scw::fail;

static std::string solve_status_message(const std::vector<int>& status, int Z) {
    for (int l = 0; l < Z; l++)
        if (status[l]) return "scw_solve: eigen-solver did not converge for slice " + std::to_string(l);
    for (int l = 0; l < Z; l++)
        if (status[Z + l]) return "scw_solve: singular U mode matrix in slice " + std::to_string(l);
    for (int l = 0; l < Z; l++)
        if (status[2 * Z + l]) return "scw_solve: singular W mode matrix in slice " + std::to_string(l);
    if (status[3 * Z]) return "scw_solve: singular boundary system";
    return "";
}

extern "C" {

scw_status scw_solution_destroy(scw_solution s) {
    delete s;
    return SCW_OK;
}

// sCWatter main (sCWatter.cpp:569-885) on the context's GPU.
scw_status scw_solve(scw_ctx ctx, const double* sample, int Zs, int Y, int X, const scw_solve_params* prm,
                     scw_solution* out) {
    using namespace scw::sv;
    if (!ctx || !sample || !prm || !out) return fail(SCW_ERR_ARG, "scw_solve: bad arguments");
    *out = nullptr;
    SolvePlan p;
    scw_status st = plan_solve(prm, Zs, Y, X, p);
    if (st != SCW_OK) return st;
    p.wide_hess = true;          // one sample: spread the Hessenberg reductions over the GPU
    SCW_ON_DEVICE(ctx->device);
    std::unique_ptr<scw_solution_s> sol(new (std::nothrow) scw_solution_s());
    if (!sol) return fail(SCW_ERR_NOMEM, "host allocation");
    sol->ctx = ctx;
    sol->M0 = p.M0;
    sol->M1 = p.M1;
    sol->MF = p.MF;
    sol->Z = Zs;
    sol->k = p.k;
    sol->zb = p.zb;
    sol->external = p.external;
    sol->n0 = p.n0;
    sol->n1 = p.n1;
    sol->Sx = p.Sx;
    sol->Sy = p.Sy;
    sol->Sz0 = p.Sz0;
    sol->Sz1 = p.Sz1;
    sol->EF = p.EF;
    // one block for inputs, scratch and the small results; the FP64 mode amplitudes in their own
    // allocation, owned by the solution
    SolveIn in{};
    SolveWs ws{};
    SolveOut o{};
    Carver sz;
    carve_in(p, sz, in);
    carve_ws(p, sz, ws);
    carve_out(p, sz, o, false, false);
    char* blk = nullptr;
    if (cudaMalloc(&blk, sz.off) != cudaSuccess) {
        cudaGetLastError();
        return fail(SCW_ERR_NOMEM, "scw_solve: cudaMalloc of " + std::to_string(sz.off >> 20) + " MiB");
    }
    std::unique_ptr<char, void (*)(char*)> blk_guard(blk, [](char* q) { cudaFree(q); });
    Carver c{blk, 0};
    carve_in(p, c, in);
    carve_ws(p, c, ws);
    carve_out(p, c, o, false, false);
    if (!p.external) {
        const size_t qbytes = sizeof(double2) * (size_t)Zs * 2 * 3 * p.MF * p.n;
        if (cudaMalloc(&sol->dQ, qbytes) != cudaSuccess) {
            cudaGetLastError();
            sol->dQ = nullptr;
            return fail(SCW_ERR_NOMEM, "scw_solve: cudaMalloc of the mode amplitudes");
        }
        o.Q64 = sol->dQ;
        const size_t vbytes = sizeof(float2) * (size_t)Zs * 3 * p.MF * p.n;
        const size_t bbytes = sizeof(double2) * (size_t)Zs * 2 * p.n;
        if (cudaMalloc(&sol->dV, vbytes) != cudaSuccess || cudaMalloc(&sol->dBeta, bbytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(SCW_ERR_NOMEM, "scw_solve: cudaMalloc of the paired mode blocks");
        }
        o.Vsep = sol->dV;
        o.sepBeta = sol->dBeta;
    }
    cudaStream_t s = ctx->stream;
    if ((st = upload_inputs(p, sample, in, s)) != SCW_OK) return st;
    long long launches = 0;
    if ((st = record_solve(p, in, ws, o, s, &launches)) != SCW_OK) return st;
    std::vector<int> status(3 * Zs + 1);
    sol->x.resize(6 * p.MF);
    sol->gam.resize((size_t)Zs * p.n);
    SCW_CUDA_TRY(cudaMemcpyAsync(status.data(), o.status, sizeof(int) * status.size(), cudaMemcpyDeviceToHost, s));
    SCW_CUDA_TRY(cudaMemcpyAsync(sol->x.data(), o.x, sizeof(double2) * sol->x.size(), cudaMemcpyDeviceToHost, s));
    SCW_CUDA_TRY(cudaMemcpyAsync(sol->gam.data(), o.gam, sizeof(double2) * sol->gam.size(), cudaMemcpyDeviceToHost, s));
    if (p.eig_mixed) {
        sol->eig_state.resize(Zs);
        sol->eig_steps.resize(Zs);
        sol->eig_res.resize(Zs);
        SCW_CUDA_TRY(cudaMemcpyAsync(sol->eig_state.data(), o.eig, sizeof(int) * Zs, cudaMemcpyDeviceToHost, s));
        SCW_CUDA_TRY(cudaMemcpyAsync(sol->eig_steps.data(), o.eig + Zs, sizeof(int) * Zs, cudaMemcpyDeviceToHost, s));
        SCW_CUDA_TRY(cudaMemcpyAsync(sol->eig_res.data(), o.eig_res, sizeof(double) * Zs, cudaMemcpyDeviceToHost, s));
    }
    SCW_CUDA_TRY(cudaStreamSynchronize(s));
    ctx->launches += launches;
    const std::string msg = solve_status_message(status, Zs);
    if (!msg.empty()) return fail(SCW_ERR_NUMERIC, msg);
    *out = sol.release();
    return SCW_OK;
}

// The layer problems of a sample without solving them: per slice the M1 x M0 Fourier crops
// of n^2 and n^-2 (column-major, FourierWave.h:152-195) and the reduced matrix PQ
// (2MF x 2MF, FourierWave.h:336-397), written to caller-provided DEVICE buffers
// (coef: Z x 2 x MF complex, PQ: Z x 2MF x 2MF complex).  Either may be NULL (M0 / M1 only).
scw_status scw_layer_problem(scw_ctx ctx, const double* sample, int Zs, int Y, int X, const scw_solve_params* prm,
                             int* M0, int* M1, void* coef, void* PQ) {
    using namespace scw::sv;
    if (!ctx || !prm) return fail(SCW_ERR_ARG, "scw_layer_problem: bad arguments");
    SolvePlan p;
    scw_status st = plan_solve(prm, Zs, Y, X, p);
    if (st != SCW_OK) return st;
    if (M0) *M0 = p.M0;
    if (M1) *M1 = p.M1;
    if (!coef && !PQ) return SCW_OK;
    if (!sample) return fail(SCW_ERR_ARG, "scw_layer_problem: null sample");
    SCW_ON_DEVICE(ctx->device);
    SolveIn in{};
    SolveWs ws{};
    Carver sz;
    carve_in(p, sz, in);
    carve_ws(p, sz, ws);
    char* blk = nullptr;
    if (cudaMalloc(&blk, sz.off) != cudaSuccess) {
        cudaGetLastError();
        return fail(SCW_ERR_NOMEM, "scw_layer_problem: cudaMalloc");
    }
    std::unique_ptr<char, void (*)(char*)> guard(blk, [](char* q) { cudaFree(q); });
    Carver c{blk, 0};
    carve_in(p, c, in);
    carve_ws(p, c, ws);
    cudaStream_t s = ctx->stream;
    if ((st = upload_inputs(p, sample, in, s)) != SCW_OK) return st;
    const int MF = p.MF, n = p.n;
    const long long nn = (long long)n * n, YX = (long long)Y * X;
    n2_kernel<<<nblk(Zs * YX), 256, 0, s>>>(in.data, YX, Zs, ws.F);
    SCW_CUDA_TRY(cudaGetLastError());
    if ((st = scw::zgemm(s, X, p.M1, Y, kOne, ws.F, Y, YX, in.tw1, p.M1, 0, kZero, ws.T, p.M1, (long long)X * p.M1, 2 * Zs)) !=
        SCW_OK)
        return st;
    if ((st = scw::zgemm(s, p.M0, p.M1, X, make_double2(1.0 / (double)YX, 0.0), in.tw2, X, 0, ws.T, p.M1, (long long)X * p.M1,
                    kZero, ws.coef, p.M1, MF, 2 * Zs)) != SCW_OK)
        return st;
    if (PQ) {
        build_pq_kernel<<<dim3(nblk(n), n, Zs), 256, 0, s>>>(ws.coef, in.up, in.wq, in.qs, in.ps, p.M0, p.M1, p.k, ws.P,
                                                              ws.Q);
        SCW_CUDA_TRY(cudaGetLastError());
        if ((st = scw::zgemm(s, n, n, n, kOne, ws.P, n, nn, ws.Q, n, nn, kZero, (double2*)PQ, n, nn, Zs)) != SCW_OK) return st;
    }
    if (coef)
        SCW_CUDA_TRY(cudaMemcpyAsync(coef, ws.coef, sizeof(double2) * (size_t)Zs * 2 * MF, cudaMemcpyDeviceToDevice, s));
    SCW_CUDA_TRY(cudaStreamSynchronize(s));
    ctx->launches += PQ ? 5 : 3;
    return SCW_OK;
}

scw_status scw_solution_info(scw_solution s, int* M0, int* M1, int* n_slices, double* k) {
    if (!s) return fail(SCW_ERR_ARG, "null solution");
    if (M0) *M0 = s->M0;
    if (M1) *M1 = s->M1;
    if (n_slices) *n_slices = s->Z;
    if (k) *k = s->k;
    return SCW_OK;
}

scw_status scw_solution_eig_slices(scw_solution s, int* state, int* steps, double* residual) {
    if (!s) return fail(SCW_ERR_ARG, "null solution");
    if (s->eig_state.empty()) return fail(SCW_ERR_STATE, "scw_solution_eig_slices: the FP64 eigen-solver ran throughout");
    const size_t Z = s->eig_state.size();
    if (state) std::copy(s->eig_state.begin(), s->eig_state.end(), state);
    if (steps) std::copy(s->eig_steps.begin(), s->eig_steps.begin() + Z, steps);
    if (residual) std::copy(s->eig_res.begin(), s->eig_res.begin() + Z, residual);
    return SCW_OK;
}

scw_status scw_solution_eig_info(scw_solution s, int* mixed, int* accepted, int* max_steps, double* max_residual,
                                 int* residual_checks) {
    if (!s) return fail(SCW_ERR_ARG, "null solution");
    const scw::sv::EigSummary e =
        scw::sv::eig_summary(s->eig_state.data(), s->eig_steps.data(), s->eig_res.data(), (int)s->eig_state.size());
    if (mixed) *mixed = s->eig_state.empty() ? 0 : 1;
    if (accepted) *accepted = e.accepted;
    if (max_steps) *max_steps = e.max_steps;
    if (max_residual) *max_residual = e.max_res;
    if (residual_checks) *residual_checks = e.checks;
    return SCW_OK;
}

scw_status scw_solution_get(scw_solution s, double* gamma, double* x, double* ef, double* z_boundaries) {
    if (!s) return fail(SCW_ERR_ARG, "null solution");
    if (gamma) std::memcpy(gamma, s->gam.data(), sizeof(cd) * s->gam.size());
    if (x) std::memcpy(x, s->x.data(), sizeof(cd) * s->x.size());
    if (ef) std::memcpy(ef, s->EF.data(), sizeof(cd) * s->EF.size());
    if (z_boundaries) std::memcpy(z_boundaries, s->zb.data(), sizeof(double) * s->zb.size());
    return SCW_OK;
}

scw_status scw_solution_get_modes(scw_solution s, int l, double* Q_check, double* Q_hat) {
    if (!s || l < 0 || l >= s->Z) return fail(SCW_ERR_ARG, "scw_solution_get_modes: slice out of range");
    if (!s->dQ) return fail(SCW_ERR_STATE, "scw_solution_get_modes: no mode amplitudes (external solve)");
    const size_t blk = (size_t)3 * s->MF * 2 * s->MF;
    SCW_ON_DEVICE(s->ctx->device);
    if (Q_check)
        SCW_CUDA_TRY(cudaMemcpy(Q_check, s->dQ + (size_t)l * 2 * blk, sizeof(double2) * blk, cudaMemcpyDeviceToHost));
    if (Q_hat)
        SCW_CUDA_TRY(cudaMemcpy(Q_hat, s->dQ + ((size_t)l * 2 + 1) * blk, sizeof(double2) * blk, cudaMemcpyDeviceToHost));
    return SCW_OK;
}

// The separable coefficient set of a solution, on the solution's device.
scw_status scw_solution_to_sep(scw_solution s, scw_sep* out) {
    if (!s || !out) return fail(SCW_ERR_ARG, "null argument");
    *out = nullptr;
    scw_ctx ctx = s->ctx;
    SCW_ON_DEVICE(ctx->device);
    const int MF = s->MF, n = 2 * MF, M0 = s->M0, M1 = s->M1, Z = s->Z;
    const double k = s->k;
    std::vector<double> kx(M0), ky(M1);
    for (int a = 0; a < M0; a++) kx[a] = s->Sx[(size_t)a * M1] * k;
    for (int b = 0; b < M1; b++) ky[b] = s->Sy[(size_t)b] * k;
    std::vector<double> zb = s->zb;
    if (s->external)      // interior layers of an external-only structure sit at z = 0 with no waves
        for (int l = 1; l < Z; l++) zb[l] = 0.0;
    scw_sep sp = nullptr;
    // interior modes as a paired set: one block V per slice and the amplitudes beta (half the
    // coefficient bytes of the two blocks Q_check, Q_hat)
    const bool paired = !s->external && s->dV && s->dBeta;
    scw_status st = paired ? scw_sep_create_paired(ctx, M0, M1, Z, n, kx.data(), ky.data(), zb.data(), &sp)
                           : scw_sep_create(ctx, M0, M1, Z, s->external ? 0 : n, kx.data(), ky.data(), zb.data(), &sp);
    if (st != SCW_OK) return st;
    std::unique_ptr<scw_sep_s, scw_status (*)(scw_sep)> guard(sp, scw_sep_destroy);
    std::vector<cd> inc(3 * MF), refl(3 * MF), trans(3 * MF), kzi(MF), kzr(MF), kzt(MF);
    for (int p = 0; p < MF; p++) {
        for (int c = 0; c < 3; c++) {
            inc[c * MF + p] = s->EF[c * MF + p];
            refl[c * MF + p] = s->x[c * MF + p];
            trans[c * MF + p] = s->x[3 * MF + c * MF + p];
        }
        kzi[p] = s->Sz0[p] * k;
        kzr[p] = -s->Sz0[p] * k * s->n0;     // sCWatter.cpp:471-475 multiplies by n0 once more
        kzt[p] = s->Sz1[p] * k * s->n1;
    }
    st = scw_sep_set_exterior(sp, (const double*)inc.data(), (const double*)kzi.data(), (const double*)refl.data(),
                              (const double*)kzr.data(), (const double*)trans.data(), (const double*)kzt.data());
    if (st != SCW_OK) return st;
    if (paired) {
        std::vector<cd> kzd(n), kzu(n), beta(2 * (size_t)n);
        for (int l = 0; l < Z && st == SCW_OK; l++) {
            for (int j = 0; j < n; j++) {
                kzd[j] = s->gam[(size_t)l * n + j] * k;
                kzu[j] = -s->gam[(size_t)l * n + j] * k;
            }
            SCW_CUDA_TRY(cudaMemcpy(beta.data(), s->dBeta + (size_t)l * 2 * n, sizeof(double2) * 2 * n,
                                    cudaMemcpyDeviceToHost));
            st = scw_sep_set_slice_paired(sp, l, (const double*)kzd.data(), (const double*)kzu.data(),
                                          s->dV + (size_t)l * 3 * MF * n, (const double*)beta.data(),
                                          (const double*)(beta.data() + n));
        }
        if (st != SCW_OK) return st;
        SCW_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    } else if (!s->external) {
        const size_t blk = (size_t)3 * MF * n;
        float2* tmp = nullptr;
        if (cudaMalloc(&tmp, sizeof(float2) * 2 * blk) != cudaSuccess) {
            cudaGetLastError();
            return fail(SCW_ERR_NOMEM, "scw_solution_to_sep: cudaMalloc");
        }
        std::vector<cd> kzd(n), kzu(n);
        for (int l = 0; l < Z && st == SCW_OK; l++) {
            for (int j = 0; j < n; j++) {
                kzd[j] = s->gam[(size_t)l * n + j] * k;
                kzu[j] = -s->gam[(size_t)l * n + j] * k;
            }
            scw::sv::to_c64_kernel<<<scw::sv::nblk(2 * blk), 256, 0, ctx->stream>>>(s->dQ + (size_t)l * 2 * blk, tmp,
                                                                                   (long long)(2 * blk));
            st = scw_sep_set_slice_device(sp, l, (const double*)kzd.data(), tmp, (const double*)kzu.data(), tmp + blk);
            if (st == SCW_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
                st = fail(SCW_ERR_CUDA, "scw_solution_to_sep: stream error");
        }
        cudaFree(tmp);
        if (st != SCW_OK) return st;
    }
    *out = guard.release();
    return SCW_OK;
}

// The .cw structure written by sCWatter (sCWatter.cpp:890-956): per harmonic p the incident
// wave, the reflected wave (wound to z_0), the transmitted wave (wound to z_Z) and, unless
// external, the 2MF downward / upward modes of each slice wound to their boundary.
extern "C++" {
// One .cw record (tira::planewave<double>: E0 xyz, k xyz as re/im pairs) of a wave wound to z = 0
// from its reference plane zw: E0 exp(-i kz zw) (wind(0, 0, -z), sCWatter.cpp:469-482).
static void cw_record(double* v, cd ex, cd ey, cd ez, cd kx, cd ky, cd kz, double zw) {
    const cd f = std::exp(cd(0, -1) * kz * zw);
    const cd E[3] = {ex * f, ey * f, ez * f};
    const cd K[3] = {kx, ky, kz};
    for (int c = 0; c < 3; c++) {
        v[2 * c] = E[c].real();
        v[2 * c + 1] = E[c].imag();
    }
    for (int c = 0; c < 3; c++) {
        v[6 + 2 * c] = K[c].real();
        v[6 + 2 * c + 1] = K[c].imag();
    }
}

// The waves of one .cw layer in the order sCWatter writes them (sCWatter.cpp:890-956): harmonic
// p outer; per p either the one exterior wave or the 2MF modes of the adjacent slice half.
// Qup / Qdn: [3MF][2MF] amplitudes of slice l-1's upward / slice l's downward half (host), or
// null where the layer has none.  emit(record) is called once per wave.
template <typename Emit>
static void cw_layer_waves(const scw_solution_s* s, int l, bool reflected, const cd* Qup, const cd* Qdn, Emit&& emit) {
    const int MF = s->MF, n = 2 * MF, ZL = s->Z + 1;
    const double k = s->k;
    double r[12];
    for (int p = 0; p < MF; p++) {
        const cd kx = s->Sx[p] * k, ky = s->Sy[p] * k;
        if (reflected) {                       // Pr
            if (l == 0) {
                cw_record(r, s->x[p], s->x[MF + p], s->x[2 * MF + p], kx, ky, -s->Sz0[p] * k * s->n0, s->zb[0]);
                emit(r);
            } else if (Qup) {
                const cd* gam = s->gam.data() + (size_t)(l - 1) * n;
                for (int j = 0; j < n; j++) {
                    cw_record(r, Qup[(size_t)p * n + j], Qup[(size_t)(MF + p) * n + j], Qup[(size_t)(2 * MF + p) * n + j],
                              kx, ky, -1.0 * gam[j] * k, s->zb[l]);
                    emit(r);
                }
            }
        } else {                               // Pt
            if (l == ZL - 1) {
                cw_record(r, s->x[3 * MF + p], s->x[4 * MF + p], s->x[5 * MF + p], kx, ky, s->Sz1[p] * k * s->n1,
                          s->zb[l]);
                emit(r);
            } else if (Qdn) {
                const cd* gam = s->gam.data() + (size_t)l * n;
                for (int j = 0; j < n; j++) {
                    cw_record(r, Qdn[(size_t)p * n + j], Qdn[(size_t)(MF + p) * n + j], Qdn[(size_t)(2 * MF + p) * n + j],
                              kx, ky, 1.0 * gam[j] * k, s->zb[l]);
                    emit(r);
                }
            }
        }
    }
}

static double cw_layer_z(const scw_solution_s* s, int l) {
    const int ZL = s->Z + 1;
    return (l == 0 || l == ZL - 1 || !s->external) ? s->zb[l] : 0.0;
}

}  // extern "C++"

scw_status scw_solution_to_cw(scw_solution s, scw_cw* out) {
    if (!s || !out) return fail(SCW_ERR_ARG, "null argument");
    *out = nullptr;
    const int MF = s->MF, n = 2 * MF, Z = s->Z, ZL = Z + 1;
    const size_t blk = (size_t)3 * MF * n;
    std::vector<cd> Qh;
    try {
        if (!s->external) Qh.resize((size_t)Z * 2 * blk);
    } catch (const std::bad_alloc&) {
        return fail(SCW_ERR_NOMEM, "host allocation of the mode amplitudes");
    }
    if (!s->external) {
        SCW_ON_DEVICE(s->ctx->device);
        SCW_CUDA_TRY(cudaMemcpy(Qh.data(), s->dQ, sizeof(double2) * Qh.size(), cudaMemcpyDeviceToHost));
    }
    std::unique_ptr<scw_cw_s> cw(new (std::nothrow) scw_cw_s());
    if (!cw) return fail(SCW_ERR_NOMEM, "host allocation");
    try {
        double r[12];
        for (int p = 0; p < MF; p++) {
            cw_record(r, s->EF[p], s->EF[MF + p], s->EF[2 * MF + p], s->Sx[p] * s->k, s->Sy[p] * s->k, s->Sz0[p] * s->k,
                      0.0);
            cw->Pi.insert(cw->Pi.end(), r, r + 12);
        }
        cw->layers.resize(ZL);
        for (int l = 0; l < ZL; l++) {
            auto& L = cw->layers[l];
            L.z = cw_layer_z(s, l);
            const cd* Qup = (!s->external && l > 0) ? Qh.data() + ((size_t)(l - 1) * 2 + 1) * blk : nullptr;
            const cd* Qdn = (!s->external && l < ZL - 1) ? Qh.data() + (size_t)l * 2 * blk : nullptr;
            cw_layer_waves(s, l, true, Qup, Qdn, [&](const double* w) { L.Pr.insert(L.Pr.end(), w, w + 12); });
            cw_layer_waves(s, l, false, Qup, Qdn, [&](const double* w) { L.Pt.insert(L.Pt.end(), w, w + 12); });
        }
    } catch (const std::bad_alloc&) {
        return fail(SCW_ERR_NOMEM, "host allocation of the wave lists");
    }
    *out = cw.release();
    return SCW_OK;
}

// Streaming writer of the same .cw file (CoupledWaveStructure.h:72-100 layout): one layer's
// two slice halves on the host at a time, records written in chunks, so host memory stays
// O(slice) whatever the file size (about 63 GB at MF = 1600, 64 slices).
scw_status scw_solution_write_cw(scw_solution s, const char* path) {
    if (!s || !path) return fail(SCW_ERR_ARG, "null argument");
    const int MF = s->MF, n = 2 * MF, Z = s->Z, ZL = Z + 1;
    const size_t blk = (size_t)3 * MF * n;
    FILE* f = fopen(path, "wb");
    if (!f) return fail(SCW_ERR_IO, std::string("cannot create ") + path);
    std::unique_ptr<FILE, int (*)(FILE*)> guard(f, fclose);
    std::vector<cd> Qup, Qdn;
    std::vector<double> chunk;
    try {
        if (!s->external) {
            Qup.resize(blk);
            Qdn.resize(blk);
        }
        chunk.reserve(12 * 65536);
    } catch (const std::bad_alloc&) {
        return fail(SCW_ERR_NOMEM, "host allocation of one slice");
    }
    bool ok = true;
    auto put = [&](const void* p, size_t bytes) { ok = ok && fwrite(p, 1, bytes, f) == bytes; };
    auto flush = [&]() {
        put(chunk.data(), chunk.size() * sizeof(double));
        chunk.clear();
    };
    auto emit = [&](const double* w) {
        chunk.insert(chunk.end(), w, w + 12);
        if (chunk.size() >= 12 * 65536) flush();
    };
    const uint64_t sz = 8, nPi = (uint64_t)MF, nL = (uint64_t)ZL;
    put(&sz, 8);
    put(&nPi, 8);
    double r[12];
    for (int p = 0; p < MF; p++) {
        cw_record(r, s->EF[p], s->EF[MF + p], s->EF[2 * MF + p], s->Sx[p] * s->k, s->Sy[p] * s->k, s->Sz0[p] * s->k,
                  0.0);
        emit(r);
    }
    flush();
    put(&nL, 8);
    SCW_ON_DEVICE(s->external ? -1 : s->ctx->device);
    for (int l = 0; l < ZL && ok; l++) {
        const bool up = !s->external && l > 0, dn = !s->external && l < ZL - 1;
        if (up)
            SCW_CUDA_TRY(cudaMemcpy(Qup.data(), s->dQ + ((size_t)(l - 1) * 2 + 1) * blk, sizeof(double2) * blk,
                                    cudaMemcpyDeviceToHost));
        if (dn)
            SCW_CUDA_TRY(cudaMemcpy(Qdn.data(), s->dQ + (size_t)l * 2 * blk, sizeof(double2) * blk,
                                    cudaMemcpyDeviceToHost));
        const double z = cw_layer_z(s, l);
        put(&z, 8);
        for (int half = 0; half < 2; half++) {
            const bool refl = half == 0;
            const uint64_t cnt = refl ? (l == 0 ? (uint64_t)MF : (up ? (uint64_t)MF * n : 0))
                                      : (l == ZL - 1 ? (uint64_t)MF : (dn ? (uint64_t)MF * n : 0));
            put(&cnt, 8);
            cw_layer_waves(s, l, refl, up ? Qup.data() : nullptr, dn ? Qdn.data() : nullptr, emit);
            flush();
        }
    }
    if (!ok || fflush(f) != 0) return fail(SCW_ERR_IO, std::string("write failed: ") + path);
    return SCW_OK;
}

}  // extern "C"
