/*
 * scwatter_gb300 -- C ABI of the GB300 (sm_103a) build of scwatter's plane-wave field
 * evaluation and per-layer coupled-wave solve.
 *
 * Every entry point returns an scw_status; SCW_OK is 0.  scw_last_error() gives a
 * message for the calling thread's last failure.  No entry point exits the process.
 * Plain pointers and sizes only.  Complex numbers are (re, im) pairs of float or
 * double, interleaved.
 *
 * Wave records ("planewave") are 12 values: E0.x re, im, E0.y re, im, E0.z re, im,
 * k.x re, im, k.y re, im, k.z re, im -- the record of the .cw file format
 * (CoupledWaveStructure.h:7-55) and of UnpackedWave<float> (cpuEvaluator.h:6-10).
 *
 * Field outputs are N x N arrays of 3 complex64 values per point, row-major with the
 * second axis as the row (E_xy[iy*N+ix], E_xz[iz*N+ix], E_yz[iz*N+iy]), exactly the
 * layout written by gpu_cw_evaluate (gpuEvaluator.cu:76-88).
 */
#ifndef SCWATTER_GB300_H
#define SCWATTER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SCW_API __attribute__((visibility("default")))
#else
#define SCW_API
#endif

typedef enum scw_status {
    SCW_OK = 0,
    SCW_ERR_ARG = 1,        /* bad argument (null pointer, size out of range, wrong device) */
    SCW_ERR_IO = 2,         /* file cannot be opened / read / written */
    SCW_ERR_FORMAT = 3,     /* truncated or inconsistent .cw data */
    SCW_ERR_CUDA = 4,       /* a CUDA runtime call failed */
    SCW_ERR_NOMEM = 5,      /* host or device allocation failed */
    SCW_ERR_STATE = 6,      /* object not initialised / wrong object kind */
    SCW_ERR_NUMERIC = 7,    /* singular system, non-finite values, eigen-solver did not converge */
    SCW_ERR_TIMEOUT = 8,    /* a bounded device-side wait gave up */
    SCW_ERR_UNSUPPORTED = 9 /* the requested shape is outside what the kernel supports */
} scw_status;

typedef struct scw_ctx_s* scw_ctx;       /* one CUDA device + one stream + cached scratch */
typedef struct scw_cw_s* scw_cw;         /* host CoupledWaveStructure<double> */
typedef struct scw_waves_s* scw_waves;   /* device-resident unpacked wave set */
typedef struct scw_sep_s* scw_sep;       /* device-resident separable (factored) coefficient set */
typedef struct scw_solution_s* scw_solution; /* result of the per-layer coupled-wave solve */
typedef struct scw_batch_s* scw_batch;       /* many samples solved + evaluated by one CUDA graph */
typedef struct scw_mlp_s* scw_mlp;           /* small fully connected network (FP32) */

/* Output-GEMM methods of the separable evaluator */
#define SCW_SEP_FP32 1      /* FP32 SIMT */
#define SCW_SEP_TF32X3 2    /* tcgen05 kind::tf32, 3 products of hi/lo splits, FP32 accumulation */
#define SCW_SEP_BF16X3 3    /* tcgen05 kind::f16 (bf16), 3 products of hi/lo splits, FP32 accumulation */

SCW_API const char* scw_last_error(void);
SCW_API const char* scw_version(void);

/* ---------------------------------------------------------------------------------- */
/* Context                                                                             */
/* ---------------------------------------------------------------------------------- */
/* stream: a cudaStream_t to run on, or NULL to create a private non-blocking stream. */
SCW_API scw_status scw_ctx_create(int device, void* stream, scw_ctx* out);
SCW_API scw_status scw_ctx_destroy(scw_ctx ctx);
SCW_API scw_status scw_ctx_synchronize(scw_ctx ctx);
SCW_API scw_status scw_ctx_stream(scw_ctx ctx, void** stream);
/* Number of kernels this context has launched since creation (evidence of GPU work). */
SCW_API scw_status scw_ctx_launch_count(scw_ctx ctx, int64_t* count);
/* Per-kernel CUDA-event timing of every launch while on; the report synchronises the stream,
 * sums milliseconds and launch counts per kernel name ('\n'-separated in names) and clears. */
SCW_API scw_status scw_ctx_set_timing(scw_ctx ctx, int on);
SCW_API scw_status scw_ctx_timing_report(scw_ctx ctx, char* names, int64_t name_bytes, double* ms,
                                         int64_t* counts, int max_entries, int* n);

/* ---------------------------------------------------------------------------------- */
/* .cw coefficient files -- replaces CoupledWaveStructure<T>::save / load /            */
/* getPlaneIndex (CoupledWaveStructure.h:72-147).  Records are read as double; the     */
/* header's precision field is read and ignored, as the reference does (:107-108).     */
/* ---------------------------------------------------------------------------------- */
SCW_API scw_status scw_cw_create(scw_cw* out);
SCW_API scw_status scw_cw_destroy(scw_cw cw);
SCW_API scw_status scw_cw_load(const char* path, scw_cw* out);              /* CoupledWaveStructure.h:103-134 */
SCW_API scw_status scw_cw_save(scw_cw cw, const char* path);                /* CoupledWaveStructure.h:72-101 */
SCW_API scw_status scw_cw_set_incident(scw_cw cw, int64_t n, const double* waves);
SCW_API scw_status scw_cw_set_layer_count(scw_cw cw, int64_t n_layers);
SCW_API scw_status scw_cw_set_layer(scw_cw cw, int64_t l, double z, int64_t n_pr, const double* pr,
                                    int64_t n_pt, const double* pt);
SCW_API scw_status scw_cw_counts(scw_cw cw, int64_t* n_incident, int64_t* n_layers);
SCW_API scw_status scw_cw_layer_counts(scw_cw cw, int64_t l, double* z, int64_t* n_pr, int64_t* n_pt);
SCW_API scw_status scw_cw_get_incident(scw_cw cw, double* waves);
SCW_API scw_status scw_cw_get_layer(scw_cw cw, int64_t l, double* pr, double* pt);
SCW_API scw_status scw_cw_get_plane_index(scw_cw cw, double z, int64_t* index); /* CoupledWaveStructure.h:141-147 */

/* ---------------------------------------------------------------------------------- */
/* Unpacking -- replaces cw_allocate / cw_unpack (cpuEvaluator.cpp:34-102).            */
/* waves_begin / waves_end have layers+1 entries; W has total_waves*12 floats.         */
/* ---------------------------------------------------------------------------------- */
SCW_API scw_status scw_cw_allocate(scw_cw cw, int* layers, int64_t* total_waves);
SCW_API scw_status scw_cw_unpack(scw_cw cw, float* W, int* waves_begin, int* waves_end, float* z_layers);

/* ---------------------------------------------------------------------------------- */
/* GPU field evaluator -- replaces gpu_initialize / gpu_cw_evaluate                    */
/* (gpuEvaluator.h:8-18, gpuEvaluator.cu:15-26, 131-165).                              */
/* ---------------------------------------------------------------------------------- */
/* gpu_initialize (gpuEvaluator.cu:15-26): uploads the unpacked float wave table, exactly
 * as the reference globals hold it (waves wound to the origin). */
SCW_API scw_status scw_gpu_initialize(scw_ctx ctx, int layers, const float* z_layers,
                                      const int* waves_begin, const int* waves_end,
                                      const float* W, int64_t n_waves, scw_waves* out);
/* Same set from the double-precision .cw structure: each wave of layer l is re-referenced
 * ("un-wound") to z_l in FP64 so no float exponent over- or under-flows. */
SCW_API scw_status scw_gpu_initialize_cw(scw_ctx ctx, scw_cw cw, scw_waves* out);
SCW_API scw_status scw_waves_destroy(scw_waves waves);
/* Region rule: 0 = gpuEvaluator rule z >= z_l - 0.001 (default, gpuEvaluator.cu:34),
 *              1 = cpuEvaluator rule z >= z_l (cpuEvaluator.cpp:303). */
SCW_API scw_status scw_waves_set_region_rule(scw_waves waves, int rule);
SCW_API scw_status scw_waves_info(scw_waves waves, int* layers, int64_t* n_waves);

/* gpu_cw_evaluate (gpuEvaluator.cu:131-165): three N x N planes into HOST arrays
 * (each N*N*6 floats); blocks until the results are in host memory. */
SCW_API scw_status scw_gpu_cw_evaluate(scw_waves waves, float* E_xy, float* E_xz, float* E_yz,
                                       float x_start, float y_start, float z_start,
                                       float x, float y, float z, float d, int N, int device);
/* One plane into DEVICE memory, asynchronous on the context stream.
 * axis 0: xy plane at z = c (a = x, b = y); 1: yz plane at x = c (a = y, b = z);
 * 2: xz plane at y = c (a = x, b = z).  Output [N][N][3] complex64, row = b. */
SCW_API scw_status scw_eval_plane_device(scw_waves waves, int axis, float a_start, float b_start,
                                         float c, float d, int N, float* dE);
/* Nz x Ny x Nx grid into DEVICE memory [Nz][Ny][Nx][3] complex64, asynchronous;
 * point (ix, iy, iz) = (x_start + dx*ix, y_start + dy*iy, z_start + dz*iz), each product
 * and sum rounded to float separately. */
SCW_API scw_status scw_eval_volume_device(scw_waves waves, float x_start, float y_start, float z_start,
                                          float dx, float dy, float dz, int Nx, int Ny, int Nz, float* dE);
/* Allocation-free variant of scw_eval_plane_device (no counterpart in the reference).
 * Same arguments, output and stream behaviour, for callers that must not allocate GPU memory
 * while they run: applications that pre-size one device pool and count any other cudaMalloc
 * as a leak, frame loops that may not stall on the allocator, plug-in hosts that forbid device
 * allocation.  It calls no cudaMalloc, cudaMallocHost, cudaFree or allocating library routine:
 * its split-K partial sums live in a 12 MiB array compiled into the library (held on every
 * GPU that loads it until exit) and its region table travels as kernel parameters.
 * Limits: N <= 16384 and at most 160 layers (SCW_ERR_ARG beyond either); planes of more
 * than 1024 tiles of 16 x 32 points run without the split.
 * The first call through a context looks up the array's address on the context's device (and may
 * load the library's GPU module there) and keeps it in the context; make that first call before
 * any stream capture on that device.  After a cudaDeviceReset, create a new context.
 * All calls share the one array per device: calls that overlap on the GPU (other streams,
 * other contexts on the same device) race.  Calls on one stream are ordered and safe; each
 * call writes every scratch element it reads, so nothing needs clearing between calls. */
SCW_API scw_status scw_eval_plane_device_static(scw_waves waves, int axis, float a_start, float b_start,
                                                float c, float d, int N, float* dE);

/* ---------------------------------------------------------------------------------- */
/* Separable ("GEMM form") evaluator -- no reference counterpart; evaluates the same    */
/* field as gpu_cw_evaluate when the waves come from the volume solver (sCWatter.cpp:  */
/* 890-956): inside slice l every wave is (harmonic p = (a, b), mode j) with           */
/* kx = kx_a, ky = ky_b, kz = kz_j, so E = sum_a e^{i kx_a x} sum_b e^{i ky_b y} C(a,b;z). */
/* Complex arrays are (re, im) doubles; Q blocks are [3][MF][J] with row p = a*M1 + b.  */
/* ---------------------------------------------------------------------------------- */
SCW_API scw_status scw_sep_create(scw_ctx ctx, int M0, int M1, int n_slices, int modes_per_half,
                                  const double* kx, const double* ky, const double* z_boundaries, scw_sep* out);
SCW_API scw_status scw_sep_destroy(scw_sep s);
/* Paired set (no reference counterpart): per slice ONE block V [3][MF][J] and the mode amplitudes
 * beta_dn, beta_up [J], standing for Q_dn = V diag(beta_dn) and Q_up = diag(1, 1, -1) V diag(beta_up).
 * That is the structure of the solver's modes (sCWatter.cpp:781-871: the E rows of a mode are the
 * same eigenvector for the roots +gamma and -gamma, its H rows -- hence Ez -- change sign), so the
 * evaluator streams one block per slice instead of two: half the coefficient bytes.  The amplitudes
 * are folded into the FP64 mode phases. */
SCW_API scw_status scw_sep_create_paired(scw_ctx ctx, int M0, int M1, int n_slices, int modes_per_half,
                                         const double* kx, const double* ky, const double* z_boundaries,
                                         scw_sep* out);
/* kz_dn, kz_up, beta_dn, beta_up: [J] complex (HOST); V: [3][MF][J] complex64 in host or device memory. */
SCW_API scw_status scw_sep_set_slice_paired(scw_sep s, int l, const double* kz_dn, const double* kz_up,
                                            const void* V_c64, const double* beta_dn, const double* beta_up);
/* 2: two-half set (scw_sep_create), 1: paired set (scw_sep_create_paired). */
SCW_API scw_status scw_sep_form(scw_sep s, int* halves);
/* incident (referenced at z = 0), reflected (at z_0), transmitted (at z_Z): [3][MF] complex;
 * kz_*: [MF] complex. */
SCW_API scw_status scw_sep_set_exterior(scw_sep s, const double* inc, const double* kz_inc, const double* refl,
                                        const double* kz_refl, const double* trans, const double* kz_trans);
/* slice l: downward modes referenced at z_l, upward modes at z_{l+1}; kz: [J] complex, Q: [3][MF][J] */
SCW_API scw_status scw_sep_set_slice(scw_sep s, int l, const double* kz_dn, const double* Q_dn,
                                     const double* kz_up, const double* Q_up);
/* same with Q already in complex64 (host or device memory) */
SCW_API scw_status scw_sep_set_slice_device(scw_sep s, int l, const double* kz_dn, const void* Q_dn_c64,
                                            const double* kz_up, const void* Q_up_c64);
/* factors a .cw written by the volume solver; SCW_ERR_UNSUPPORTED if its waves do not have
 * the separable structure (use the plain evaluator then). */
SCW_API scw_status scw_sep_from_cw(scw_ctx ctx, scw_cw cw, scw_sep* out);
/* Compact factored coefficient file (.cwf; no reference counterpart): the separable set as it is
 * -- "SCWSEP01", int32 M0, M1, Z, J, region rule, 0; float64 kx[M0], ky[M1], z[Z+1];
 * complex128 exterior[12 MF], kz[Z][2][Jp]; complex64 Q[Z][2][3][MF][Jp] (Jp = J rounded up to
 * even), little-endian -- streamed one slice at a time.  A paired set is written as "SCWSEP02":
 * the same header and blocks up to kz, then complex128 beta[Z][2][Jp] and complex64 V[Z][3][MF][Jp].
 * Load checks the magic and that the file size matches the header (SCW_ERR_FORMAT otherwise). */
SCW_API scw_status scw_sep_save(scw_sep s, const char* path);
SCW_API scw_status scw_sep_load(scw_ctx ctx, const char* path, scw_sep* out);
SCW_API scw_status scw_sep_info(scw_sep s, int* M0, int* M1, int* n_slices, int* modes_per_half);
/* kx [M0], ky [M1] (the separable harmonic grid) and the Z + 1 slice boundaries; any may be NULL. */
SCW_API scw_status scw_sep_get_grid(scw_sep s, double* kx, double* ky, double* z_boundaries);
SCW_API scw_status scw_sep_set_region_rule(scw_sep s, int rule);
SCW_API scw_status scw_sep_eval_volume_device(scw_sep s, float x_start, float y_start, float z_start,
                                              float dx, float dy, float dz, int Nx, int Ny, int Nz,
                                              float* dE, int method);
/* The same volume from HOST amplitudes, end to end (no reference counterpart; the reference
 * uploads its wave table once in gpu_initialize, gpuEvaluator.cu:15-26, and reads each plane back
 * in gpu_cw_evaluate, :131-165).  Q_host: [Z][2][3][MF][J] complex64 (per slice the downward then
 * the upward block, as in the .cwf file but without the even padding; a paired set takes its one block
 * per slice, [Z][3][MF][J], and keeps its kz and beta from scw_sep_set_slice_paired); E_host: [Nz][Ny][Nx][3]
 * complex64.  Slices go up on one stream while the planes of the slices already up are evaluated
 * on the context stream, and finished planes come back on a third stream; use page-locked host
 * buffers for full link speed.  The set's device copy of each slice that a grid plane lies in is
 * overwritten (after the work already queued on the context stream); blocks until E_host is
 * written. */
SCW_API scw_status scw_sep_eval_volume_host(scw_sep s, const void* Q_host, float x_start, float y_start,
                                            float z_start, float dx, float dy, float dz, int Nx, int Ny, int Nz,
                                            float* E_host, int method);
/* Planes k_begin .. k_end-1 of the volume above (plane k at z = z_start + dz*k, the value the whole
 * volume gives it): output [k_end - k_begin][Ny][Nx][3] complex64.  One process per GPU evaluates
 * its own z-slab this way; the slabs put together are the whole volume.  The host form reads only
 * the slices its planes lie in from Q_host (still the whole [Z][2][3][MF][J] array). */
SCW_API scw_status scw_sep_eval_slab_device(scw_sep s, float x_start, float y_start, float z_start, float dx,
                                            float dy, float dz, int Nx, int Ny, int k_begin, int k_end, float* dE,
                                            int method);
SCW_API scw_status scw_sep_eval_slab_host(scw_sep s, const void* Q_host, float x_start, float y_start,
                                          float z_start, float dx, float dy, float dz, int Nx, int Ny, int k_begin,
                                          int k_end, float* E_host, int method);
/* Granularity of scw_sep_eval_volume_host: Q bytes per upload (whole slices, at least one; default
 * 192 MiB) and output bytes per read-back slab (whole planes, at least one; default 64 MiB; three
 * slabs are kept on the device).  0 restores a default. */
SCW_API scw_status scw_sep_set_streaming(scw_sep s, int64_t chunk_bytes, int64_t slab_bytes);
/* Tile shape of the coefficient contraction: 0 (default) = 8, 8, 4, 2 mode rows per warp for
 * launches of 1, 2, 4, 8 planes per group; 1 = half as many.  Results are bit-identical; the
 * batch autotuner picks it for its items. */
SCW_API scw_status scw_sep_set_tiles(scw_sep s, int ctr_shape);
/* Device slabs of >= 32 planes in `chunks` chunks whose stages overlap on two streams (stage 1 of
 * a chunk beside stage 2 of the previous, its output GEMM on SM count / synth_sm_div SMs);
 * chunks 0 or 1 (the default): one pass.  Results are bit-identical either way. */
SCW_API scw_status scw_sep_set_pipeline(scw_sep s, int chunks, int synth_sm_div);
SCW_API scw_status scw_sep_eval_plane_device(scw_sep s, int axis, float a_start, float b_start, float c,
                                             float d, int N, float* dE, int method);
SCW_API scw_status scw_sep_gpu_cw_evaluate(scw_sep s, float* E_xy, float* E_xz, float* E_yz,
                                           float x_start, float y_start, float z_start,
                                           float x, float y, float z, float d, int N, int device, int method);

/* ---------------------------------------------------------------------------------- */
/* FP64 complex dense linear algebra on DEVICE buffers (row-major, batched back to     */
/* back) -- GPU replacements of the reference's LAPACK wrappers                         */
/* MKL_multiply / MKL_linearsolve / MKL_eigensolve (third_Lapack.h:38-87).              */
/* Complex values are (re, im) doubles.                                                 */
/* ---------------------------------------------------------------------------------- */
/* C = alpha A B + beta C; A: M x K, B: K x N, C: M x N per batch entry. */
SCW_API scw_status scw_zgemm(scw_ctx ctx, int M, int N, int K, const double* alpha, const void* A, const void* B,
                             const double* beta, void* C, int batch);
/* B := A^-1 B (A n x n overwritten by its LU factors, B n x nrhs); SCW_ERR_NUMERIC if singular;
 * info_host (optional, batch ints) receives the first zero pivot + 1 per matrix. */
SCW_API scw_status scw_zgesv(scw_ctx ctx, int n, int nrhs, void* A, void* B, int batch, int* info_host);
/* eigenvalues W (n) and right eigenvectors V (n x n, column k = eigenvector k) of A (n x n,
 * overwritten); SCW_ERR_NUMERIC if the QR iteration does not converge. */
SCW_API scw_status scw_zgeev(scw_ctx ctx, int n, void* A, void* W, void* V, int batch, int* status_host);
/* Same contract as scw_zgeev (n <= 4096), computed by the mixed-precision solver: FP32
 * Householder + QR + triangular eigenvectors, then Newton refinement of all eigenpairs with FP64
 * residuals (clusters of close eigenvalues solved as small FP64 Schur problems).  Refinement stops
 * once max_i ||A x_i - lambda_i x_i|| / (||A||_1 ||x_i||) <= 1e-14; a matrix at or below 1e-12 from
 * step 10 on is accepted, and one still above 1e-12 after 10 steps (16 for n >= 1600) is solved by
 * the FP64 QR solver instead (and only then overwritten).  Optional per-matrix
 * outputs: accepted_host (1 = refined result; else why the FP64 solver took it: 2 FP32 QR not
 * converged, 3 a cluster above 64 eigenvalues, 4 singular FP32 eigenvector matrix, 5 a cluster's
 * small Schur solve not converged, 6 residual above 1e-12 after the last step), steps_host
 * (refinement steps), residual_host (last relative residual of the refined result). */
/* FP32 counterpart of scw_zgeev (complex64 A, W, V; LAPACK cgeev semantics), the first stage of
 * scw_zgeev_mixed.  No reference counterpart. */
SCW_API scw_status scw_cgeev(scw_ctx ctx, int n, void* A, void* W, void* V, int batch, int* status_host);
/* CTAs per matrix of the QR sweeps in scw_zgeev, scw_cgeev, scw_zgeev_mixed and scw_solve, for the
 * whole process: 0 (default) chooses per call (a thread-block cluster of up to 8 CTAs per matrix
 * where all matrices' clusters fit on the GPU at once, else one CTA), 1 one CTA per matrix, 2..8
 * a cluster of that size where it fits.  Results agree to rounding in every setting.
 * Batches (scw_batch_*) always use one CTA per matrix.  No reference counterpart. */
SCW_API scw_status scw_set_qr_cluster(int ctas);
SCW_API scw_status scw_zgeev_mixed(scw_ctx ctx, int n, void* A, void* W, void* V, int batch, int* accepted_host,
                                   int* steps_host, double* residual_host);

/* ---------------------------------------------------------------------------------- */
/* Per-layer coupled-wave solve (FP64, on the GPU) -- the computation of the reference  */
/* program sCWatter (sCWatter.cpp:569-956; its options sCWatter.cpp:506-527).           */
/* ---------------------------------------------------------------------------------- */
typedef struct scw_solve_params {
    double lambda;        /* --lambda: vacuum wavelength */
    double direction[3];  /* --direction: incident direction (normalised here) */
    double ex[2], ey[2], ez[2]; /* --ex/--ey/--ez: incident field components (re, im) */
    double n[2];          /* --n: real refractive index of the upper and lower media */
    double kappa;         /* --kappa: absorbance of the lower medium */
    double size[3];       /* --size: sample extent x, y, z */
    double z;             /* --z: sample centre along z */
    int coef[2];          /* --coef: harmonics along x, y (<= 0: the sample's X, Y) */
    int external;         /* --external: keep only the exterior waves */
    int pz;               /* 1 = compute Ez of the modes; 0 = the reference's --npz */
    int psf;              /* --psf: every harmonic carries the incident field (sCWatter.cpp:665-669) */
    int eig_fp64;         /* no reference counterpart.  0 (default): FP32 Householder + QR eigen-solve
                           * refined to FP64 residuals by Newton steps, FP64 QR for any slice that
                           * does not converge; 1: FP64 Householder + QR for every slice */
} scw_solve_params;

/* sample: [Z][Y][X] complex128 refractive index in host or device memory (the .npy volume;
 * unified addressing tells them apart).  Runs the
 * whole solve on the context's device and blocks until it is done.  SCW_ERR_NUMERIC when an
 * eigen-solve does not converge or a mode / boundary matrix is singular. */
/* Sample volumes on the device (no reference counterpart; the reference reads the .npy on the
 * host, FourierWave.h:269, and generates samples with tilesample.py).  out: [Z][Y][X]
 * complex128 device buffer.
 * scw_gen_spheres: background index, then each sphere (spheres[4 s ..]: cz, cy, cx, r in voxel
 * units) overwrites the voxels with (z-cz)^2 + (y-cy)^2 + (x-cx)^2 <= r^2, in order.
 * scw_gen_grf: Gaussian random field -- counter-based normal noise (splitmix64 of seed and index,
 * Box-Muller), periodic separable Gaussian filter exp(-t^2 / (2 corr^2)) truncated at 4 corr,
 * min-max normalised to t in [0, 1]; n = n_lo + (n_hi - n_lo) t + i kappa t with kappa drawn from
 * the seed in [0, kappa_max].
 * scw_npy_read: dims[3] = Z, Y, X of a 2-D or 3-D '<c16' / '<f8' .npy; with out != NULL the
 * volume is streamed into out (ctx needed then). */
SCW_API scw_status scw_gen_spheres(scw_ctx ctx, int Z, int Y, int X, int n_spheres, const double* spheres,
                                   const double* n_background, const double* n_sphere, void* out);
SCW_API scw_status scw_gen_grf(scw_ctx ctx, int Z, int Y, int X, double corr_px, double n_lo, double n_hi,
                               double kappa_max, uint64_t seed, void* out);
SCW_API scw_status scw_npy_read(scw_ctx ctx, const char* path, int* dims, void* out);

SCW_API scw_status scw_solve(scw_ctx ctx, const double* sample, int Z, int Y, int X, const scw_solve_params* prm,
                             scw_solution* out);
SCW_API scw_status scw_solution_destroy(scw_solution s);
SCW_API scw_status scw_solution_info(scw_solution s, int* M0, int* M1, int* n_slices, double* k);
/* No reference counterpart: how the eigen-solves went.  mixed = 1 when the FP32 + refinement
 * path ran; accepted = slices it finished (the others went through the FP64 QR solver);
 * max_steps = most refinement steps an accepted slice needed; max_residual = largest
 * accepted max_i ||A x_i - lambda_i x_i|| / (||A||_1 ||x_i||); residual_checks = FP64 residual
 * products (one n x n x n GEMM each) summed over the slices. */
SCW_API scw_status scw_solution_eig_info(scw_solution s, int* mixed, int* accepted, int* max_steps,
                                         double* max_residual, int* residual_checks);
/* Per slice (Z entries each, any may be NULL): state 1 = the mixed eigen-solver's refined result
 * was accepted, else the reason code of scw_zgeev_mixed for the FP64 fallback; refinement steps;
 * last relative residual.  SCW_ERR_STATE when the FP64 solver ran for every slice. */
SCW_API scw_status scw_solution_eig_slices(scw_solution s, int* state, int* steps, double* residual);
/* gamma: Z x 2MF complex downward roots (the reference's even-slot eigenvalues); x: 6MF
 * complex reflected / transmitted amplitudes (sCWatter.cpp:722); ef: 3MF incident Fourier
 * amplitudes; z_boundaries: Z + 1.  Any pointer may be NULL. */
SCW_API scw_status scw_solution_get(scw_solution s, double* gamma, double* x, double* ef, double* z_boundaries);
/* Q_check / Q_hat of slice l: 3MF x 2MF complex each (row-major; rows Ex, Ey, Ez blocks). */
SCW_API scw_status scw_solution_get_modes(scw_solution s, int l, double* Q_check, double* Q_hat);
/* Separable coefficient set for the evaluators, on the solution's device. */
SCW_API scw_status scw_solution_to_sep(scw_solution s, scw_sep* out);
/* The .cw structure that sCWatter writes (sCWatter.cpp:890-956). */
SCW_API scw_status scw_solution_to_cw(scw_solution s, scw_cw* out);
/* The same structure written straight to a .cw file (CoupledWaveStructure.h:72-100 layout),
 * layer by layer: host memory stays at one slice's mode amplitudes.  Byte-identical to
 * scw_solution_to_cw + scw_cw_save. */
SCW_API scw_status scw_solution_write_cw(scw_solution s, const char* path);

/* ---------------------------------------------------------------------------------- */
/* Batched solve + evaluate (no counterpart in the reference, which solves one sample   */
/* per sCWatter run): every item is solved (FP64) and its field volume evaluated with   */
/* the separable evaluator; the whole batch is captured once into a CUDA graph.         */
/* ---------------------------------------------------------------------------------- */
typedef struct scw_batch_item {
    const double* sample;  /* [Z][Y][X] complex128 refractive index, host; read during create */
    int Z, Y, X;
    scw_solve_params prm;
    float x0, y0, z0;      /* evaluation grid: point (i, j, k) = (x0 + dx i, y0 + dy j, z0 + dz k) */
    float dx, dy, dz;
    int Nx, Ny, Nz;
} scw_batch_item;
/* lanes: concurrent streams (0 = autotune); method: SCW_SEP_* output GEMM (0 = autotune); the
 * contraction tile shape is always autotuned.  Plans, uploads, autotunes on stratified subsets,
 * and captures the graph. */
SCW_API scw_status scw_batch_create(scw_ctx ctx, const scw_batch_item* items, int count, int lanes, int method,
                                    scw_batch* out);
/* One cudaGraphLaunch on the context stream (asynchronous). */
SCW_API scw_status scw_batch_run(scw_batch b);
/* Waits; item_status (count ints, may be NULL): 0, SCW_ERR_NUMERIC or SCW_ERR_TIMEOUT. */
SCW_API scw_status scw_batch_wait(scw_batch b, int* item_status);
/* x: 6MF complex; gamma: Z x 2MF complex; field_host: [Nz][Ny][Nx][3] complex64; any may be NULL. */
SCW_API scw_status scw_batch_get(scw_batch b, int i, double* x, double* gamma, float* field_host, float** field_device);
/* harmonics, slices and points x modes of the item's volume */
SCW_API scw_status scw_batch_item_info(scw_batch b, int i, int* M0, int* M1, int* n_slices, int64_t* points_modes);
/* The mixed eigen-solver's record of item i after a run, as scw_solution_eig_info. */
SCW_API scw_status scw_batch_item_eig(scw_batch b, int i, int* mixed, int* accepted, int* max_steps,
                                      double* max_residual, int* residual_checks);
/* Per slice of item i after a run, as scw_solution_eig_slices (n_slices entries each, any may be
 * NULL); SCW_ERR_STATE when the item's FP64 solver ran for every slice. */
SCW_API scw_status scw_batch_item_eig_slices(scw_batch b, int i, int* state, int* steps, double* residual);
/* chosen lanes / method / contraction tile shape (0: default rows per warp, 1: half), graph
 * nodes, kernels per launch, tuning time and its log (quadruples lanes, method, tile shape, ms;
 * n_tune entries, at most 16). */
SCW_API scw_status scw_batch_info(scw_batch b, int* lanes, int* method, int* ctr_shape, int64_t* graph_nodes,
                                  int64_t* kernels, double* tune_ms, double* tune_log, int* n_tune);
SCW_API scw_status scw_batch_destroy(scw_batch b);

/* ---------------------------------------------------------------------------------- */
/* Learned eigen warm start (no counterpart in the reference, whose eigen-solve is one   */
/* zgeev per slice, sCWatter.cpp:248-272)                                               */
/* ---------------------------------------------------------------------------------- */
/* Layer problems of a sample without the solve: Fourier crops of n^2 and n^-2 per slice
 * (coef: DEVICE Z x 2 x MF complex, column-major M1 x M0 crops) and the reduced matrices PQ
 * (DEVICE Z x 2MF x 2MF complex); both may be NULL (harmonic counts only). */
SCW_API scw_status scw_layer_problem(scw_ctx ctx, const double* sample, int Z, int Y, int X,
                                     const scw_solve_params* prm, int* M0, int* M1, void* coef, void* PQ);
/* Network y = W3 relu(W2 relu(W1 x + b1) + b2) + b3 (FP32), He-uniform initialisation. */
SCW_API scw_status scw_mlp_create(scw_ctx ctx, int n_in, int width, int n_out, uint64_t seed, scw_mlp* out);
SCW_API scw_status scw_mlp_destroy(scw_mlp m);
SCW_API scw_status scw_mlp_info(scw_mlp m, int* n_in, int* width, int* n_out, int64_t* n_params);
/* parameters as one host vector: W1 [width][n_in], b1, W2 [width][width], b2, W3 [n_out][width], b3 */
SCW_API scw_status scw_mlp_get_params(scw_mlp m, float* host);
SCW_API scw_status scw_mlp_set_params(scw_mlp m, const float* host);
/* X: DEVICE [B][n_in] float, Y: DEVICE [B][n_out] float (asynchronous) */
SCW_API scw_status scw_mlp_forward(scw_mlp m, const float* X, int B, float* Y);
/* gradient of the mean squared error against T (DEVICE [B][n_out]) into grad_host (n_params) */
SCW_API scw_status scw_mlp_gradients(scw_mlp m, const float* X, const float* T, int B, float* grad_host, double* loss);
/* one Adam step (beta 0.9 / 0.999); loss before the step to *loss (may be NULL; synchronises if not) */
SCW_API scw_status scw_mlp_train_step(scw_mlp m, const float* X, const float* T, int B, float lr, double* loss);
/* Eigenpairs of a batch of n x n matrices (DEVICE, not modified) from one shift per eigenvalue
 * (DEVICE batch x n complex) and optionally one proposed mode per eigenvalue (DEVICE batch x n
 * ints: the start vector is that unit vector of A's basis; NULL or -1: pseudo-random):
 * Rayleigh-quotient iteration on the Hessenberg form, one warp per eigenpair; tasks that land on
 * another task's eigenvector restart with it projected out.  A matrix is accepted when every pair
 * has ||A v - lambda v|| <= tol ||A||_F ||v|| and no two pairs share an eigenvector; otherwise
 * the plain eigen-solver replaces it.  W: DEVICE batch x n, V: DEVICE batch x n x n (columns).
 * accepted_host: batch ints (may be NULL); stats_host (5 doubles, may be NULL): mean iterations,
 * largest accepted residual, accepted, fallen back, repaired tasks. */
SCW_API scw_status scw_eig_warm(scw_ctx ctx, int n, const void* A, int batch, const void* shifts,
                                const int* start_index, int max_it, double tol, void* W, void* V,
                                int* accepted_host, double* stats_host);

/* ---------------------------------------------------------------------------------- */
/* Viewer display processing on DEVICE buffers -- replaces EvaluateScalarSlices,       */
/* CalculateMinMax and EvaluateColorValue / EvaluateColorSlices (sCWatterView.cpp:200-352) */
/* ---------------------------------------------------------------------------------- */
/* S[i] (complex64) = E[i][mode] for mode 0/1/2 (x, y, z), or |Ex|^2 + |Ey|^2 + |Ez|^2 for 3. */
SCW_API scw_status scw_view_scalar(scw_ctx ctx, const float* E, int64_t n, int mode, float* S);
/* out4 = real min, real max, imaginary min, imaginary max over the n complex64 values (synchronises). */
SCW_API scw_status scw_view_minmax(scw_ctx ctx, const float* S, int64_t n, float* out4);
/* rgb (n x 3 bytes): params = real_low, real_high, imag_low, imag_high, real_color[3],
 * imag_color[3], show_real, show_imag (12 floats, HOST). */
SCW_API scw_status scw_view_color(scw_ctx ctx, const float* S, int64_t n, const float* params, unsigned char* rgb);

/* ---------------------------------------------------------------------------------- */
/* Homogeneous multilayer solve -- the computation of the reference program            */
/* sCWatterLayer (sCWatterLayer.cpp:119-267), batched over incident plane waves         */
/* ---------------------------------------------------------------------------------- */
/* ri: L complex refractive indices (HOST, layer 0 = incident medium); z: L - 1 interfaces;
 * n0 = Re ri[0]; k: vacuum wavenumber; waves: count HOST records of 12 doubles (incident
 * plane waves); x: count x 6L complex (HOST; per layer the transmitted then the reflected
 * amplitude, xyz); info: count ints (1 = singular system).  2 <= L <= 16. */
SCW_API scw_status scw_layer_solve(scw_ctx ctx, int L, const double* ri, const double* z, double n0, double k,
                                   int count, const double* waves, double* x, int* info);

/* ---------------------------------------------------------------------------------- */
/* Diagnostics (no reference counterpart)                                              */
/* ---------------------------------------------------------------------------------- */
/* Measured issue peaks of this GPU (any output may be NULL): MUFU operations per second for
 * sin.approx / cos.approx (the plain evaluator issues one of each per point and wave) and for
 * ex2.approx (issued only where a wave's k has an imaginary part in the evaluated plane), FP32 and
 * FP64 FMA FLOP/s; independent dependency chains on every SM, event-timed; synchronises. */
SCW_API scw_status scw_measure_peaks(scw_ctx ctx, double* sincos_ops_per_s, double* ex2_ops_per_s, double* fp32_flops,
                                     double* fp64_flops);

#ifdef __cplusplus
}
#endif
#endif /* SCWATTER_GB300_H */
