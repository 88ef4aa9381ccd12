/*
 * CPU oracle for scwatter's plane-wave field evaluation.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA evaluators, and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * --impl reference legs load this library.  The product never links it.
 *
 * Two families of functions:
 *
 *  orc_cpu_eval_{xy,yz,xz}_f32  -- restatement of the reference CPU evaluator
 *      cpu_cw_evaluate_xy / _yz / _xz (cpuEvaluator.cpp:294-407) in its shipped FP32
 *      form: float coordinates, complex<float> k.r, std::exp(complex<float>), complex<float>
 *      accumulation (xy, yz) and complex<double> accumulation of complex<float>
 *      products for xz (cpuEvaluator.cpp:395).  Region lookup "z >= z_layers[li]", last
 *      satisfied layer wins (cpuEvaluator.cpp:302-306, 348-352, 385-389).  Rows are
 *      split over nthreads POSIX threads; every row is computed exactly as the serial
 *      loop computes it, so the output does not depend on the thread count.
 *
 *  orc_eval_points_f64  -- the FP64 oracle: the same sum E = sum_w E0_w exp(i k_w . r)
 *      (gpuEvaluator.cu:28-68, cpuEvaluator.cpp:317-323) in double precision over the
 *      double-precision wave table read from a .cw file, at caller-supplied float
 *      coordinates, with caller-supplied region thresholds (GPU rule
 *      z >= z_l - 0.001 of gpuEvaluator.cu:34, or the CPU rule z >= z_l).
 *
 * Wave tables: f32 = 12 floats per wave  (E0x re, im, E0y, E0z, kx, ky, kz) as
 * UnpackedWave<float> (cpuEvaluator.h:6-10); f64 = 12 doubles per wave, same order
 * (the .cw record order of CoupledWaveStructure.h:11-22).
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared -pthread (contraction off so x86 and
 * aarch64 hosts give identical FP32 results).
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------ */
/* FP32 restatement of cpu_cw_evaluate_{xy,yz,xz}                                  */
/* ------------------------------------------------------------------------------ */
typedef struct {
    const float* W;
    const int64_t* begin;
    const int64_t* end;
    const float* z_layers;
    int64_t layers;
    float a_start, b_start, c_fixed, d;
    int64_t N;
    int axis;           /* 0 = xy (a=x,b=y,c=z), 1 = yz (a=y,b=z,c=x), 2 = xz (a=x,b=z,c=y) */
    float* out;         /* N*N*6 floats: [row][col][Ex re, im, Ey re, im, Ez re, im] */
    int64_t row0, row1;
} f32_job;

static int64_t region_f32(const float* z_layers, int64_t layers, float z) {
    int64_t l = 0;
    for (int64_t li = 0; li < layers; li++)
        if (z >= z_layers[li]) l = li + 1;
    return l;
}

static inline float complex load_c(const float* p) { return CMPLXF(p[0], p[1]); }

static void* f32_worker(void* arg) {
    f32_job* j = (f32_job*)arg;
    const float complex I1 = CMPLXF(0.0f, 1.0f);
    int64_t N = j->N;
    if (j->axis == 0) {
        /* cpu_cw_evaluate_xy: one region for the whole plane (cpuEvaluator.cpp:300-309) */
        int64_t l = region_f32(j->z_layers, j->layers, j->c_fixed);
        int64_t b = j->begin[l], e = j->end[l];
        float z = j->c_fixed;
        for (int64_t iy = j->row0; iy < j->row1; iy++) {
            float y = j->b_start + (float)(unsigned)iy * j->d;
            for (int64_t ix = 0; ix < N; ix++) {
                float x = j->a_start + (float)(unsigned)ix * j->d;
                float complex E0 = 0, E1 = 0, E2 = 0;
                for (int64_t w = b; w < e; w++) {
                    const float* r = j->W + 12 * w;
                    float complex kdr = x * load_c(r + 6) + y * load_c(r + 8) + z * load_c(r + 10);
                    float complex ph = cexpf(I1 * kdr);
                    E0 += load_c(r + 0) * ph;
                    E1 += load_c(r + 2) * ph;
                    E2 += load_c(r + 4) * ph;
                }
                float* o = j->out + 6 * (iy * N + ix);
                o[0] = crealf(E0); o[1] = cimagf(E0);
                o[2] = crealf(E1); o[3] = cimagf(E1);
                o[4] = crealf(E2); o[5] = cimagf(E2);
            }
        }
    } else {
        /* cpu_cw_evaluate_yz (axis 1) / _xz (axis 2): region per z row.  The reference
         * carries `l` across rows without resetting it (cpuEvaluator.cpp:345-352); a row
         * whose z satisfies no threshold therefore keeps the previous row's region.
         * Reproduced by replaying the scan from row 0. */
        int64_t l = 0;
        for (int64_t iz = 0; iz < j->row0; iz++) {
            float z = j->b_start + (float)(unsigned)iz * j->d;
            for (int64_t li = 0; li < j->layers; li++)
                if (z >= j->z_layers[li]) l = li + 1;
        }
        for (int64_t iz = j->row0; iz < j->row1; iz++) {
            float z = j->b_start + (float)(unsigned)iz * j->d;
            for (int64_t li = 0; li < j->layers; li++)
                if (z >= j->z_layers[li]) l = li + 1;
            int64_t b = j->begin[l], e = j->end[l];
            for (int64_t ia = 0; ia < N; ia++) {
                float a = j->a_start + (float)(unsigned)ia * j->d;
                float x, y;
                if (j->axis == 1) { x = j->c_fixed; y = a; }
                else { x = a; y = j->c_fixed; }
                float* o = j->out + 6 * (iz * N + ia);
                if (j->axis == 1) {
                    float complex E0 = 0, E1 = 0, E2 = 0;
                    for (int64_t w = b; w < e; w++) {
                        const float* r = j->W + 12 * w;
                        float complex kdr = x * load_c(r + 6) + y * load_c(r + 8) + z * load_c(r + 10);
                        float complex ph = cexpf(I1 * kdr);
                        E0 += load_c(r + 0) * ph;
                        E1 += load_c(r + 2) * ph;
                        E2 += load_c(r + 4) * ph;
                    }
                    o[0] = crealf(E0); o[1] = cimagf(E0);
                    o[2] = crealf(E1); o[3] = cimagf(E1);
                    o[4] = crealf(E2); o[5] = cimagf(E2);
                } else {
                    double complex E0 = 0, E1 = 0, E2 = 0;   /* cpuEvaluator.cpp:395 */
                    for (int64_t w = b; w < e; w++) {
                        const float* r = j->W + 12 * w;
                        float complex kdr = x * load_c(r + 6) + y * load_c(r + 8) + z * load_c(r + 10);
                        float complex ph = cexpf(I1 * kdr);
                        E0 += (double complex)(load_c(r + 0) * ph);
                        E1 += (double complex)(load_c(r + 2) * ph);
                        E2 += (double complex)(load_c(r + 4) * ph);
                    }
                    o[0] = (float)creal(E0); o[1] = (float)cimag(E0);
                    o[2] = (float)creal(E1); o[3] = (float)cimag(E1);
                    o[4] = (float)creal(E2); o[5] = (float)cimag(E2);
                }
            }
        }
    }
    return NULL;
}

static int run_f32(f32_job proto, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > proto.N) nthreads = (int)(proto.N > 0 ? proto.N : 1);
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    f32_job* jobs = (f32_job*)calloc((size_t)nthreads, sizeof(f32_job));
    if (!th || !jobs) { free(th); free(jobs); return -1; }
    int64_t chunk = (proto.N + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = proto;
        jobs[t].row0 = t * chunk < proto.N ? t * chunk : proto.N;
        jobs[t].row1 = (t + 1) * chunk < proto.N ? (t + 1) * chunk : proto.N;
        pthread_create(&th[t], NULL, f32_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
    return 0;
}

/* Rows [row0, row1) only: lets a caller time a bounded sample of a plane. */
int orc_cpu_eval_plane_f32(int axis, const float* W, const int64_t* begin, const int64_t* end,
                           const float* z_layers, int64_t layers,
                           float a_start, float b_start, float c_fixed, float d, int64_t N,
                           int64_t row0, int64_t row1, float* out, int nthreads) {
    f32_job p;
    memset(&p, 0, sizeof(p));
    p.W = W; p.begin = begin; p.end = end; p.z_layers = z_layers; p.layers = layers;
    p.a_start = a_start; p.b_start = b_start; p.c_fixed = c_fixed; p.d = d; p.N = N;
    p.axis = axis; p.out = out;
    if (row0 < 0) row0 = 0;
    if (row1 > N) row1 = N;
    if (row1 <= row0) return 0;
    /* split [row0, row1) over threads */
    if (nthreads < 1) nthreads = 1;
    int64_t rows = row1 - row0;
    if (nthreads > rows) nthreads = (int)rows;
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    f32_job* jobs = (f32_job*)calloc((size_t)nthreads, sizeof(f32_job));
    if (!th || !jobs) { free(th); free(jobs); return -1; }
    int64_t chunk = (rows + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = p;
        int64_t r0 = row0 + t * chunk, r1 = row0 + (t + 1) * chunk;
        jobs[t].row0 = r0 < row1 ? r0 : row1;
        jobs[t].row1 = r1 < row1 ? r1 : row1;
        pthread_create(&th[t], NULL, f32_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
    (void)run_f32;
    return 0;
}

/* ------------------------------------------------------------------------------ */
/* FP64 oracle over an arbitrary point list                                        */
/* ------------------------------------------------------------------------------ */
typedef struct {
    const double* W;
    const int64_t* begin;
    const int64_t* end;
    const double* thr;
    int64_t layers;
    const float* pts;
    double* out;
    int64_t p0, p1;
} f64_job;

static void* f64_worker(void* arg) {
    f64_job* j = (f64_job*)arg;
    for (int64_t p = j->p0; p < j->p1; p++) {
        double x = (double)j->pts[3 * p + 0];
        double y = (double)j->pts[3 * p + 1];
        double z = (double)j->pts[3 * p + 2];
        int64_t l = 0;
        for (int64_t li = 0; li < j->layers; li++)
            if (z >= j->thr[li]) l = li + 1;
        double complex E0 = 0, E1 = 0, E2 = 0;
        for (int64_t w = j->begin[l]; w < j->end[l]; w++) {
            const double* r = j->W + 12 * w;
            double complex kdr = x * CMPLX(r[6], r[7]) + y * CMPLX(r[8], r[9]) + z * CMPLX(r[10], r[11]);
            double complex ph = cexp(CMPLX(-cimag(kdr), creal(kdr)));
            E0 += CMPLX(r[0], r[1]) * ph;
            E1 += CMPLX(r[2], r[3]) * ph;
            E2 += CMPLX(r[4], r[5]) * ph;
        }
        double* o = j->out + 6 * p;
        o[0] = creal(E0); o[1] = cimag(E0);
        o[2] = creal(E1); o[3] = cimag(E1);
        o[4] = creal(E2); o[5] = cimag(E2);
    }
    return NULL;
}

int orc_eval_points_f64(const double* W, const int64_t* begin, const int64_t* end,
                        const double* thresholds, int64_t layers,
                        const float* pts, int64_t npts, double* out, int nthreads) {
    if (npts <= 0) return 0;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > npts) nthreads = (int)npts;
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    f64_job* jobs = (f64_job*)calloc((size_t)nthreads, sizeof(f64_job));
    if (!th || !jobs) { free(th); free(jobs); return -1; }
    int64_t chunk = (npts + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        f64_job* jb = &jobs[t];
        jb->W = W; jb->begin = begin; jb->end = end; jb->thr = thresholds; jb->layers = layers;
        jb->pts = pts; jb->out = out;
        jb->p0 = t * chunk < npts ? t * chunk : npts;
        jb->p1 = (t + 1) * chunk < npts ? (t + 1) * chunk : npts;
        pthread_create(&th[t], NULL, f64_worker, jb);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
    return 0;
}

/* ------------------------------------------------------------------------------ */
/* FP64 oracle for the separable (factored) form of one region                     */
/*   E_c(x,y,z) = sum_{a,b} e^{i kx_a x} e^{i ky_b y} sum_j Q_c(a*Mb+b, j)          */
/*                 e^{i kz_j (z - zref_j)}                                          */
/* kx, ky real; kz complex.  Used to check the GEMM-form evaluator on the same      */
/* coefficients without materialising a 4 MF^2 wave list.  Points sharing a z       */
/* (consecutive in the list) reuse the contracted coefficients C_c(m; z).           */
/* ------------------------------------------------------------------------------ */
typedef struct {
    int64_t Ma, Mb, J;
    const double* kx;      /* Ma */
    const double* ky;      /* Mb */
    const double* kz;      /* J complex (2J doubles) */
    const double* zref;    /* J */
    const double* Q;       /* [3][Ma*Mb][J] complex */
    const float* pts;
    double* out;
    int64_t p0, p1;
} sep_job;

static void* sep_worker(void* arg) {
    sep_job* j = (sep_job*)arg;
    int64_t MF = j->Ma * j->Mb;
    double complex* C = (double complex*)malloc(sizeof(double complex) * (size_t)(3 * MF));
    double complex* ph = (double complex*)malloc(sizeof(double complex) * (size_t)(j->J > 0 ? j->J : 1));
    double zlast = NAN;
    for (int64_t p = j->p0; p < j->p1; p++) {
        double x = j->pts[3 * p], y = j->pts[3 * p + 1], z = j->pts[3 * p + 2];
        if (!(z == zlast)) {   /* C_c(m; z) = sum_j Q_c(m, j) exp(i kz_j (z - zref_j)), cached per z */
            for (int64_t jj = 0; jj < j->J; jj++) {
                double complex kz = CMPLX(j->kz[2 * jj], j->kz[2 * jj + 1]);
                double complex arg2 = kz * (z - j->zref[jj]);
                ph[jj] = cexp(CMPLX(-cimag(arg2), creal(arg2)));
            }
            for (int c = 0; c < 3; c++)
                for (int64_t m = 0; m < MF; m++) {
                    const double* q = j->Q + 2 * ((c * MF + m) * j->J);
                    double complex s = 0;
                    for (int64_t jj = 0; jj < j->J; jj++) s += CMPLX(q[2 * jj], q[2 * jj + 1]) * ph[jj];
                    C[c * MF + m] = s;
                }
            zlast = z;
        }
        double complex E[3] = {0, 0, 0};
        for (int64_t a = 0; a < j->Ma; a++) {
            for (int64_t b = 0; b < j->Mb; b++) {
                double ang = j->kx[a] * x + j->ky[b] * y;
                double complex exy = CMPLX(cos(ang), sin(ang));
                int64_t m = a * j->Mb + b;
                for (int c = 0; c < 3; c++) E[c] += C[c * MF + m] * exy;
            }
        }
        for (int c = 0; c < 3; c++) {
            j->out[6 * p + 2 * c] = creal(E[c]);
            j->out[6 * p + 2 * c + 1] = cimag(E[c]);
        }
    }
    free(ph);
    free(C);
    return NULL;
}

int orc_eval_separable_f64(int64_t Ma, int64_t Mb, int64_t J, const double* kx, const double* ky,
                           const double* kz, const double* zref, const double* Q,
                           const float* pts, int64_t npts, double* out, int nthreads) {
    if (npts <= 0) return 0;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > npts) nthreads = (int)npts;
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    sep_job* jobs = (sep_job*)calloc((size_t)nthreads, sizeof(sep_job));
    if (!th || !jobs) { free(th); free(jobs); return -1; }
    int64_t chunk = (npts + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        sep_job* jb = &jobs[t];
        jb->Ma = Ma; jb->Mb = Mb; jb->J = J; jb->kx = kx; jb->ky = ky; jb->kz = kz;
        jb->zref = zref; jb->Q = Q; jb->pts = pts; jb->out = out;
        jb->p0 = t * chunk < npts ? t * chunk : npts;
        jb->p1 = (t + 1) * chunk < npts ? (t + 1) * chunk : npts;
        pthread_create(&th[t], NULL, sep_worker, jb);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
    return 0;
}
