// Small fully connected network (FP32) with its own forward, backward and Adam kernels:
//   h1 = relu(W1 x + b1),  h2 = relu(W2 h1 + b2),  y = W3 h2 + b3
// Used to propose eigenvalue shifts from a layer's Fourier coefficients (warm.cu); trained on
// the GPU with a mean-squared-error loss.  Row-major batches: X [B][n_in], Y [B][n_out].
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "scw_internal.h"

namespace scw {
namespace nn {

constexpr int kT = 64;      // C tile
constexpr int kK = 16;      // K step

// C[M][N] = alpha op(A) op(B) + beta C (+ bias[n] if bias), row-major.
// op(A): ta == 0 -> A[M][K] (lda), ta == 1 -> A stored [K][M];
// op(B): tb == 0 -> B[K][N] (ldb), tb == 1 -> B stored [N][K].
__global__ void __launch_bounds__(256)
sgemm_kernel(int M, int N, int K, float alpha, const float* __restrict__ A, int lda, int ta,
             const float* __restrict__ B, int ldb, int tb, float beta, float* __restrict__ C, int ldc,
             const float* __restrict__ bias, int relu) {
    __shared__ float As[kK][kT + 1];
    __shared__ float Bs[kK][kT + 1];
    const int i0 = blockIdx.y * kT, j0 = blockIdx.x * kT;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kK) {
        for (int e = threadIdx.x; e < kK * kT; e += 256) {
            // A tile: rows i0.., k k0..
            int r, kk;
            if (!ta) { r = e / kK; kk = e % kK; } else { kk = e / kT; r = e % kT; }
            const int gi = i0 + r, gk = k0 + kk;
            float a = 0.f;
            if (gi < M && gk < K) a = ta ? A[(long long)gk * lda + gi] : A[(long long)gi * lda + gk];
            As[kk][r] = a;
            int c, kb;
            if (!tb) { kb = e / kT; c = e % kT; } else { c = e / kK; kb = e % kK; }
            const int gj = j0 + c, gk2 = k0 + kb;
            float b = 0.f;
            if (gj < N && gk2 < K) b = tb ? B[(long long)gj * ldb + gk2] : B[(long long)gk2 * ldb + gj];
            Bs[kb][c] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const int gi = i0 + ty + 16 * p;
        if (gi >= M) continue;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int gj = j0 + tx + 16 * q;
            if (gj >= N) continue;
            float* c = C + (long long)gi * ldc + gj;
            float v = alpha * acc[p][q];
            if (beta != 0.f) v = fmaf(beta, *c, v);
            if (bias) v += bias[gj];
            if (relu) v = fmaxf(v, 0.f);
            *c = v;
        }
    }
}

// dY = (2 / (B n_out)) (Y - T);  loss partial sums of (Y - T)^2 into sums (one per block)
__global__ void mse_grad_kernel(const float* __restrict__ Y, const float* __restrict__ T, long long n, float scale,
                                float* __restrict__ dY, double* __restrict__ sums) {
    __shared__ double sh[8];
    double s = 0.0;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float d = Y[e] - T[e];
        dY[e] = scale * d;
        s += (double)d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        sums[blockIdx.x] = t;
    }
}

// dH *= (H > 0)
__global__ void relu_back_kernel(const float* __restrict__ H, float* __restrict__ dH, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n && H[e] <= 0.f) dH[e] = 0.f;
}

// db[o] = sum_b dY[b][o]
__global__ void bias_grad_kernel(const float* __restrict__ dY, int B, int N, float* __restrict__ db) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= N) return;
    float s = 0.f;
    for (int b = 0; b < B; b++) s += dY[(long long)b * N + o];
    db[o] = s;
}

// Adam (Kingma & Ba 2015) with bias correction folded into the step size
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr_t, float b1, float b2, float eps) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.f - b1) * gi;
    const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    p[e] -= lr_t * mi / (sqrtf(vi) + eps);
}

}  // namespace nn
}  // namespace scw

using scw::fail;

struct scw_mlp_s {
    scw_ctx ctx = nullptr;
    int n_in = 0, width = 0, n_out = 0;
    long long n_par = 0;
    long long off[6] = {};          // W1 b1 W2 b2 W3 b3 offsets in the parameter vector
    float* P = nullptr;             // parameters
    float* G = nullptr;             // gradients
    float* Mv = nullptr;            // Adam first moment
    float* Vv = nullptr;            // Adam second moment
    long long step = 0;
    // activations / work for the largest batch seen
    int cap = 0;
    float *H1 = nullptr, *H2 = nullptr, *Y = nullptr, *dY = nullptr, *dH2 = nullptr, *dH1 = nullptr;
    double* sums = nullptr;
    ~scw_mlp_s() {
        ::scw::DeviceScope dev_scope_(ctx ? ctx->device : -1);
        for (void* p : {(void*)P, (void*)G, (void*)Mv, (void*)Vv, (void*)H1, (void*)H2, (void*)Y, (void*)dY,
                        (void*)dH2, (void*)dH1, (void*)sums})
            cudaFree(p);
    }
};

namespace {

unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

scw_status gemm(cudaStream_t st, int M, int N, int K, const float* A, int lda, int ta, const float* B, int ldb, int tb,
                float beta, float* C, int ldc, const float* bias, int relu) {
    dim3 grid((N + scw::nn::kT - 1) / scw::nn::kT, (M + scw::nn::kT - 1) / scw::nn::kT);
    scw::nn::sgemm_kernel<<<grid, 256, 0, st>>>(M, N, K, 1.f, A, lda, ta, B, ldb, tb, beta, C, ldc, bias, relu);
    SCW_CUDA_TRY(cudaGetLastError());
    return SCW_OK;
}

scw_status reserve(scw_mlp m, int B) {
    if (B <= m->cap) return SCW_OK;
    for (float** p : {&m->H1, &m->H2, &m->dH2, &m->dH1}) {
        cudaFree(*p);
        *p = nullptr;
        if (cudaMalloc(p, sizeof(float) * (size_t)B * m->width) != cudaSuccess) return fail(SCW_ERR_NOMEM, "mlp work");
    }
    for (float** p : {&m->Y, &m->dY}) {
        cudaFree(*p);
        *p = nullptr;
        if (cudaMalloc(p, sizeof(float) * (size_t)B * m->n_out) != cudaSuccess) return fail(SCW_ERR_NOMEM, "mlp work");
    }
    if (!m->sums && cudaMalloc(&m->sums, sizeof(double) * 256) != cudaSuccess) return fail(SCW_ERR_NOMEM, "mlp work");
    m->cap = B;
    return SCW_OK;
}

scw_status forward(scw_mlp m, const float* X, int B, float* Y) {
    cudaStream_t st = m->ctx->stream;
    const float* P = m->P;
    scw_status s;
    if ((s = gemm(st, B, m->width, m->n_in, X, m->n_in, 0, P + m->off[0], m->n_in, 1, 0.f, m->H1, m->width,
                  P + m->off[1], 1)) != SCW_OK)
        return s;
    if ((s = gemm(st, B, m->width, m->width, m->H1, m->width, 0, P + m->off[2], m->width, 1, 0.f, m->H2, m->width,
                  P + m->off[3], 1)) != SCW_OK)
        return s;
    if ((s = gemm(st, B, m->n_out, m->width, m->H2, m->width, 0, P + m->off[4], m->width, 1, 0.f, Y, m->n_out,
                  P + m->off[5], 0)) != SCW_OK)
        return s;
    m->ctx->launches += 3;
    return SCW_OK;
}

// forward + MSE + backward into m->G; loss (mean squared error) to *loss if not null
scw_status backward(scw_mlp m, const float* X, const float* T, int B, double* loss) {
    cudaStream_t st = m->ctx->stream;
    scw_status s = forward(m, X, B, m->Y);
    if (s != SCW_OK) return s;
    const long long ny = (long long)B * m->n_out;
    scw::nn::mse_grad_kernel<<<256, 256, 0, st>>>(m->Y, T, ny, 2.f / (float)ny, m->dY, m->sums);
    SCW_CUDA_TRY(cudaGetLastError());
    float* G = m->G;
    const float* P = m->P;
    // layer 3: dW3 = dY^T H2, db3, dH2 = dY W3
    if ((s = gemm(st, m->n_out, m->width, B, m->dY, m->n_out, 1, m->H2, m->width, 0, 0.f, G + m->off[4], m->width,
                  nullptr, 0)) != SCW_OK)
        return s;
    scw::nn::bias_grad_kernel<<<nb(m->n_out), 256, 0, st>>>(m->dY, B, m->n_out, G + m->off[5]);
    if ((s = gemm(st, B, m->width, m->n_out, m->dY, m->n_out, 0, P + m->off[4], m->width, 0, 0.f, m->dH2, m->width,
                  nullptr, 0)) != SCW_OK)
        return s;
    scw::nn::relu_back_kernel<<<nb((long long)B * m->width), 256, 0, st>>>(m->H2, m->dH2, (long long)B * m->width);
    // layer 2
    if ((s = gemm(st, m->width, m->width, B, m->dH2, m->width, 1, m->H1, m->width, 0, 0.f, G + m->off[2], m->width,
                  nullptr, 0)) != SCW_OK)
        return s;
    scw::nn::bias_grad_kernel<<<nb(m->width), 256, 0, st>>>(m->dH2, B, m->width, G + m->off[3]);
    if ((s = gemm(st, B, m->width, m->width, m->dH2, m->width, 0, P + m->off[2], m->width, 0, 0.f, m->dH1, m->width,
                  nullptr, 0)) != SCW_OK)
        return s;
    scw::nn::relu_back_kernel<<<nb((long long)B * m->width), 256, 0, st>>>(m->H1, m->dH1, (long long)B * m->width);
    // layer 1
    if ((s = gemm(st, m->width, m->n_in, B, m->dH1, m->width, 1, X, m->n_in, 0, 0.f, G + m->off[0], m->n_in, nullptr,
                  0)) != SCW_OK)
        return s;
    scw::nn::bias_grad_kernel<<<nb(m->width), 256, 0, st>>>(m->dH1, B, m->width, G + m->off[1]);
    SCW_CUDA_TRY(cudaGetLastError());
    m->ctx->launches += 12;
    if (loss) {
        std::vector<double> h(256);
        SCW_CUDA_TRY(cudaMemcpyAsync(h.data(), m->sums, sizeof(double) * 256, cudaMemcpyDeviceToHost, st));
        SCW_CUDA_TRY(cudaStreamSynchronize(st));
        double t = 0;
        for (double v : h) t += v;
        *loss = t / (double)ny;
    }
    return SCW_OK;
}

}  // namespace

extern "C" {

scw_status scw_mlp_create(scw_ctx ctx, int n_in, int width, int n_out, uint64_t seed, scw_mlp* out) {
    if (!ctx || !out || n_in < 1 || width < 1 || n_out < 1) return fail(SCW_ERR_ARG, "scw_mlp_create: bad arguments");
    *out = nullptr;
    SCW_ON_DEVICE(ctx->device);
    scw_mlp m = new (std::nothrow) scw_mlp_s();
    if (!m) return fail(SCW_ERR_NOMEM, "host allocation");
    m->ctx = ctx;
    m->n_in = n_in;
    m->width = width;
    m->n_out = n_out;
    const long long sizes[6] = {(long long)width * n_in, width, (long long)width * width, width,
                                (long long)n_out * width, n_out};
    long long o = 0;
    for (int i = 0; i < 6; i++) {
        m->off[i] = o;
        o += sizes[i];
    }
    m->n_par = o;
    // He-uniform weights, zero biases
    std::vector<float> h((size_t)o, 0.f);
    std::mt19937_64 rng(seed);
    const int fan_in[3] = {n_in, width, width};
    for (int l = 0; l < 3; l++) {
        const float lim = std::sqrt(6.f / (float)fan_in[l]) * (l == 2 ? 0.5f : 1.f);
        std::uniform_real_distribution<float> U(-lim, lim);
        for (long long i = 0; i < sizes[2 * l]; i++) h[(size_t)(m->off[2 * l] + i)] = U(rng);
    }
    const size_t bytes = sizeof(float) * (size_t)o;
    if (cudaMalloc(&m->P, bytes) != cudaSuccess || cudaMalloc(&m->G, bytes) != cudaSuccess ||
        cudaMalloc(&m->Mv, bytes) != cudaSuccess || cudaMalloc(&m->Vv, bytes) != cudaSuccess) {
        delete m;
        return fail(SCW_ERR_NOMEM, "scw_mlp_create: cudaMalloc");
    }
    cudaMemcpy(m->P, h.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemset(m->Mv, 0, bytes);
    cudaMemset(m->Vv, 0, bytes);
    cudaMemset(m->G, 0, bytes);
    *out = m;
    return SCW_OK;
}

scw_status scw_mlp_destroy(scw_mlp m) {
    delete m;
    return SCW_OK;
}

scw_status scw_mlp_info(scw_mlp m, int* n_in, int* width, int* n_out, int64_t* n_params) {
    if (!m) return fail(SCW_ERR_ARG, "null network");
    if (n_in) *n_in = m->n_in;
    if (width) *width = m->width;
    if (n_out) *n_out = m->n_out;
    if (n_params) *n_params = m->n_par;
    return SCW_OK;
}

// parameters as one host vector: W1 [width][n_in], b1, W2 [width][width], b2, W3 [n_out][width], b3
scw_status scw_mlp_get_params(scw_mlp m, float* host) {
    if (!m || !host) return fail(SCW_ERR_ARG, "null argument");
    SCW_ON_DEVICE(m->ctx->device);
    SCW_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
    SCW_CUDA_TRY(cudaMemcpy(host, m->P, sizeof(float) * m->n_par, cudaMemcpyDeviceToHost));
    return SCW_OK;
}

scw_status scw_mlp_set_params(scw_mlp m, const float* host) {
    if (!m || !host) return fail(SCW_ERR_ARG, "null argument");
    SCW_ON_DEVICE(m->ctx->device);
    SCW_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
    SCW_CUDA_TRY(cudaMemcpy(m->P, host, sizeof(float) * m->n_par, cudaMemcpyHostToDevice));
    return SCW_OK;
}

// Y (device, [B][n_out]) from X (device, [B][n_in]); asynchronous
scw_status scw_mlp_forward(scw_mlp m, const float* X, int B, float* Y) {
    if (!m || !X || !Y || B < 1) return fail(SCW_ERR_ARG, "scw_mlp_forward: bad arguments");
    SCW_ON_DEVICE(m->ctx->device);
    scw_status s = reserve(m, B);
    if (s != SCW_OK) return s;
    return forward(m, X, B, Y);
}

// gradients of the mean squared error over the batch (device X, T) into host grad (n_params)
scw_status scw_mlp_gradients(scw_mlp m, const float* X, const float* T, int B, float* grad_host, double* loss) {
    if (!m || !X || !T || B < 1) return fail(SCW_ERR_ARG, "scw_mlp_gradients: bad arguments");
    SCW_ON_DEVICE(m->ctx->device);
    scw_status s = reserve(m, B);
    if (s != SCW_OK) return s;
    if ((s = backward(m, X, T, B, loss)) != SCW_OK) return s;
    if (grad_host) {
        SCW_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
        SCW_CUDA_TRY(cudaMemcpy(grad_host, m->G, sizeof(float) * m->n_par, cudaMemcpyDeviceToHost));
    }
    return SCW_OK;
}

// one Adam step on the batch; loss (before the step) to *loss if not null
scw_status scw_mlp_train_step(scw_mlp m, const float* X, const float* T, int B, float lr, double* loss) {
    if (!m || !X || !T || B < 1 || !(lr > 0)) return fail(SCW_ERR_ARG, "scw_mlp_train_step: bad arguments");
    SCW_ON_DEVICE(m->ctx->device);
    scw_status s = reserve(m, B);
    if (s != SCW_OK) return s;
    if ((s = backward(m, X, T, B, loss)) != SCW_OK) return s;
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float lr_t = lr * std::sqrt(1.f - std::pow(b2, (float)m->step)) / (1.f - std::pow(b1, (float)m->step));
    scw::nn::adam_kernel<<<nb(m->n_par), 256, 0, m->ctx->stream>>>(m->P, m->G, m->Mv, m->Vv, m->n_par, lr_t, b1, b2,
                                                                  1e-8f);
    SCW_CUDA_TRY(cudaGetLastError());
    m->ctx->launches++;
    return SCW_OK;
}

}  // extern "C"
