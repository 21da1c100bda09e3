/*
 * s2kit_gb300.h -- C ABI of the GB300 (sm_103a) seminaive spherical harmonic transform library.
 *
 * Part 1 is a drop-in for S2kit 1.1's memo path: every function keeps the reference
 * signature (the headers in include/s2kit/), argument meaning and coefficient layout, takes HOST
 * buffers, and runs on the GPU (CUDA device 0 unless S2G_DEVICE selects another).
 * FFTW plans are accepted and ignored (NULL is fine).  Tables produced by the table
 * builders below are generated on the GPU and copied into the caller's buffers.
 *
 * Part 2 adds status-returning entry points on DEVICE pointers, batched over functions,
 * with an explicit CUDA stream, and a split-precision (tensor core) real-field path.
 *
 * Coefficient layout (both parts): f(m,l) at IndexOfHarmonicCoeff(m,l,bw), real and
 * imaginary parts in separate arrays of bw*bw doubles (util.c:42-49).
 * Sample layout: (2bw)^2 values, latitude-major [theta_j][phi_k],
 * theta_j = pi (2j+1) / (4bw), phi_k = 2 pi k / (2bw).
 */
#ifndef S2KIT_GB300_H
#define S2KIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* include/s2kit/util.h:16-19 */
#ifndef _UTIL_H
typedef enum {
    COMPLEX = 0, /* data is complex */
    REAL         /* data is real */
} DataFormat;
#endif

/* FFTW plan handle as seen by the reference signatures.  When <fftw3.h> is included
 * first its own definition is used; the library never dereferences plans. */
#ifndef FFTW3_H
typedef struct fftw_plan_s* fftw_plan;
#endif

/* =============================== Part 1: drop-in ================================ */

/* Replaces FSTSemiMemo, src/FST_semi_memo.c:68-202 (include/s2kit/FST_semi_memo.h:8-9).
 * The table argument is uploaded on first use and cached by address (see
 * s2g_cache_clear); workspace, plans and weights are not needed (device copies). */
void FSTSemiMemo(double* rdata, double* idata, double* rcoeffs, double* icoeffs, const int bw,
                 double** seminaive_naive_table, double* workspace, DataFormat data_format, const int cutoff,
                 fftw_plan* DCT_plan, fftw_plan* FFT_plan, double* weights);

/* Replaces InvFSTSemiMemo, src/FST_semi_memo.c:228-351 (FST_semi_memo.h:11-12). */
void InvFSTSemiMemo(double* rcoeffs, double* icoeffs, double* rdata, double* idata, const int bw,
                    double** transpose_seminaive_naive_table, double* workspace, DataFormat data_format,
                    const int cutoff, fftw_plan* inv_DCT_plan, fftw_plan* inv_FFT_plan);

/* Replaces FZTSemiMemo, src/FST_semi_memo.c:374-407 (FST_semi_memo.h:14).  As in the
 * reference, REAL data writes 2*bw zeros to ires. */
void FZTSemiMemo(double* rdata, double* idata, double* rres, double* ires, const int bw, double* cos_pml_table,
                 double* workspace, DataFormat data_format, fftw_plan* DCT_plan, double* weights);

/* Replaces ConvOn2SphereSemiMemo, src/FST_semi_memo.c:439-518 (FST_semi_memo.h:16).
 * Device tables for bw are generated once and cached (the reference rebuilds them
 * on every call); workspace is unused. */
void ConvOn2SphereSemiMemo(double* rdata, double* idata, double* rfilter, double* ifilter, double* rres,
                           double* ires, const int bw, double* workspace);

/* Replace the on-the-fly family, src/FST_semi_fly.c (include/s2kit/FST_semi_fly.h:8-16):
 * FSTSemiFly :67-211, InvFSTSemiFly :235-369, FZTSemiFly :390-425, ConvOn2SphereSemiFly :454-519.
 * The reference generates each order's Legendre table inside every call and frees it; here no
 * table exists on the device at all: the associated Legendre recurrence runs inside the
 * contraction kernels, which apply the reference's naive Legendre transform (its form for the
 * orders >= cutoff) to every order.  Results equal the memo family's to rounding; cutoff is
 * validated and otherwise has no effect.  Device memory per call: the samples, coefficients and
 * a row-DFT workspace (2 x rows x 2bw doubles), no O(bw^3) table.  Workspace and plans are
 * ignored; weights are used when given. */
void FSTSemiFly(double* rdata, double* idata, double* rcoeffs, double* icoeffs, const int bw, double* workspace,
                DataFormat data_format, const int cutoff, fftw_plan* DCT_plan, fftw_plan* FFT_plan,
                double* weights);
void InvFSTSemiFly(double* rcoeffs, double* icoeffs, double* rdata, double* idata, const int bw, double* workspace,
                   DataFormat data_format, const int cutoff, fftw_plan* inv_DCT_plan, fftw_plan* inv_FFT_plan);
void FZTSemiFly(double* rdata, double* idata, double* rres, double* ires, const int bw, double* workspace,
                DataFormat data_format, fftw_plan* DCT_plan, double* weights);
void ConvOn2SphereSemiFly(double* rdata, double* idata, double* rfilter, double* ifilter, double* rres,
                          double* ires, const int bw, double* workspace);

/* Replaces DLTSemi, src/legendre_transform/seminaive.c:153-198 (seminaive.h:6). */
void DLTSemi(double* data, const int bw, const int m, double* result, double* workspace, double* cos_pml_table,
             double* weights, fftw_plan* plan);

/* Replaces InvDLTSemi, src/legendre_transform/seminaive.c:56-115 (seminaive.h:8). */
void InvDLTSemi(double* coeffs, const int bw, const int m, double* result, double* trans_cos_pml_table,
                double* sin_values, double* workspace, fftw_plan* plan);

/* Replace DLTNaive / InvDLTNaive, src/legendre_transform/naive.c:34-59, 78-96 (naive.h:4-6). */
void DLTNaive(double* data, const int bw, const int m, double* weights, double* result, double* pml_table,
              double* workspace);
void InvDLTNaive(double* coeffs, const int bw, const int m, double* result, double* pml_table);

/* Replaces GenerateWeightsForDLT, src/legendre_transform/weights.c:32-47 (weights.h:4). */
void GenerateWeightsForDLT(const int bw, double* weights);

/* Table builders, src/legendre_polynomials/cospml.c and pml.c (cospml.h:6-30, pml.h:4). */
void GenerateCosPmlTable(const int bw, const int m, double* tablespace, double* workspace); /* cospml.c:161-242 */
void TransposeCosPmlTable(const int bw, const int m, double* cos_pml_table, double* result); /* cospml.c:301-362 */
double** Spharmonic_Pml_Table(const int bw, double* resultspace, double* workspace);     /* cospml.c:387-401 */
double** Transpose_Spharmonic_Pml_Table(double** spharmonic_pml_table, const int bw,
                                        double* resultspace);                                /* cospml.c:415-428 */
double** SemiNaive_Naive_Pml_Table(const int bw, const int m, double* resultspace,
                                   double* workspace);                                        /* cospml.c:451-475 */
double** Transpose_SemiNaive_Naive_Pml_Table(double** seminaive_naive_pml_table, const int bw, const int m,
                                             double* resultspace, double* workspace);        /* cospml.c:490-518 */
void GeneratePmlTable(const int bw, const int m, double* pml_table, double* workspace);     /* pml.c:41-79 */
void Pmm_L2(const int m, double* eval_points, const int n, double* result);                /* pmm.c:21-34 */

/* Size / layout helpers (integer arithmetic only), cospml.c:39-288. */
int TableSize(const int m, const int bw);                    /* cospml.c:39-59 */
int Spharmonic_TableSize(const int bw);                      /* cospml.c:85-92 */
int Reduced_SpharmonicTableSize(const int bw, const int m);  /* cospml.c:107-115 */
int Reduced_Naive_TableSize(const int bw, const int m);      /* cospml.c:434-440 */
int TableOffset(int m, int l);                               /* cospml.c:123-134 */
int RowSize(const int m, const int l);                       /* cospml.c:250-258 */
int Transpose_RowSize(const int row, const int m, const int bw); /* cospml.c:270-288 */

/* src/util/util.c:42-49 and :68-103 (util.h:15-17) */
int IndexOfHarmonicCoeff(const int m, const int l, const int bw);
void TransMult(double* rdatacoeffs, double* idatacoeffs, double* rfiltercoeffs, double* ifiltercoeffs,
               double* rres, double* ires, const int bw);

/* src/util/chebyshev_nodes.c:15-34 (chebyshev_nodes.h:4-6) */
void AcosOfChebyshevNodes(const int n, double* eval_points);
void ChebyshevNodes(const int n, double* eval_points);

/* ============================ Part 2: device API ================================== */

typedef enum {
    S2G_OK = 0,
    S2G_ERR_ARG = 1,         /* invalid argument (bw, cutoff, batch, NULL pointer, precision) */
    S2G_ERR_NOMEM = 2,       /* device or host allocation failed */
    S2G_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    S2G_ERR_UNSUPPORTED = 4, /* valid request this build does not implement (e.g. odd bw on tensor cores) */
    S2G_ERR_TIMEOUT = 5,     /* a bounded device-side wait expired */
    S2G_ERR_NOGPU = 6        /* no usable CUDA device */
} s2g_status;

typedef enum {
    S2G_PREC_FP64 = 0,   /* plain FP64 everywhere (parity path) */
    S2G_PREC_BF16X3 = 1, /* FP32 FFT/DCT, Legendre contraction as 3-term split BF16 on tcgen05, FP32 accumulate */
    S2G_PREC_BF16X2 = 2, /* as above with 2-term splits (3 products) */
    S2G_PREC_FP16X2 = 3  /* 2-term split FP16 (3 products), rows and table scaled by powers of two */
} s2g_precision;

/* Last error message of the calling thread ("" if none). */
const char* s2g_last_error(void);
/* Library version string. */
const char* s2g_version(void);
/* Drops every cached device table and uploaded caller table (all devices). */
int s2g_cache_clear(void);

/* Table files: the device's FP64 seminaive/naive tables for (bw, cutoff) -- the forward
 * (SemiNaive_Naive_Pml_Table, cospml.c:451-475) and transposed (cospml.c:490-518) layouts --
 * written to `path` (generated first if needed), and read back into the current device's table
 * cache in another process, so that plans and drop-ins for (bw, cutoff) use them without
 * generating.  The file holds a 64-byte header (magic "S2GTAB1", bw, cutoff, doubles per table,
 * an FNV-1a hash of the payload) and both tables; loading rejects a wrong magic, sizes that do
 * not match bw and cutoff, a short file or a hash mismatch, and tables that already exist on
 * the device.  No counterpart in the reference, which regenerates its tables in every
 * process. */
int s2g_tables_save(int bw, int cutoff, const char* path);
int s2g_tables_load(const char* path, int* bw, int* cutoff);

typedef struct s2g_plan_s* s2g_plan;

/* Creates a plan for bandwidth bw (2 <= bw <= 2048 for powers of two, any bw <= 512 otherwise) and a
 * seminaive/naive cutoff (1 <= cutoff <= bw).  Tables are generated on the current device
 * (FP64 recurrence and DCT, cospml.c:161-242) and shared by every plan with the same
 * (device, bw, cutoff).  A plan owns scratch buffers and streams: use it from one host thread at
 * a time (one plan per thread for concurrent callers; the tables stay shared). */
int s2g_plan_create(s2g_plan* plan, int bw, int cutoff);
int s2g_plan_destroy(s2g_plan plan);
/* A plan for the on-the-fly family (src/FST_semi_fly.c, as the Fly drop-ins above): it holds no
 * Legendre table, only weights and twiddles.  s2g_fst, s2g_inv_fst, s2g_fzt and s2g_conv on it
 * run the on-the-fly kernels; the split-precision entry points reject it (S2G_ERR_ARG). */
int s2g_plan_create_fly(s2g_plan* plan, int bw);
/* Device bytes of scratch a call with this batch needs (the plan grows its own scratch
 * on demand when the caller passes none). */
size_t s2g_plan_workspace_size(s2g_plan plan, int batch, int precision);

/* Batched FP64 transforms on device pointers.  Function f of the batch uses
 * rdata + f*(2bw)^2 and rcoeffs + f*bw*bw (likewise for the imaginary arrays).
 * REAL with idata == NULL (forward) or idata == NULL (inverse output) selects the
 * real-field fast path (imaginary samples taken as zero / not written).  `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Asynchronous with respect to the host. */
int s2g_fst(s2g_plan plan, const double* rdata, const double* idata, double* rcoeffs, double* icoeffs, int batch,
            DataFormat data_format, void* stream);
int s2g_inv_fst(s2g_plan plan, const double* rcoeffs, const double* icoeffs, double* rdata, double* idata,
                int batch, DataFormat data_format, void* stream);
/* Zonal transform of `batch` functions: rres/ires hold bw values per function (REAL
 * zeroes the imaginary part; the host drop-in FZTSemiMemo zeroes 2*bw as the reference). */
int s2g_fzt(s2g_plan plan, const double* rdata, const double* idata, double* rres, double* ires, int batch,
            DataFormat data_format, void* stream);
/* Coefficient-space product with a zonal filter (TransMult), batched. */
int s2g_transmult(int bw, const double* rdatacoeffs, const double* idatacoeffs, const double* rfiltercoeffs,
                  const double* ifiltercoeffs, double* rres, double* ires, int batch, void* stream);
/* Convolution of `batch` pairs (data_f, filter_f), each as ConvOn2SphereSemiMemo, both
 * grids batch*(2bw)^2; the plan must have cutoff == bw. */
int s2g_conv(s2g_plan plan, const double* rdata, const double* idata, const double* rfilter,
             const double* ifilter, double* rres, double* ires, int batch, void* stream);

/* Real-field batched transforms with FP32 samples/coefficients and a selectable
 * precision for the Legendre contraction (s2g_precision); any bw in [16, 256] and the powers
 * of two up to 1024 (lengths 2bw that no warp FFT takes, odd bw among them, run as chirp-z
 * transforms), plan cutoff == bw.  grid: batch*(2bw)^2 floats;
 * rcoeffs/icoeffs: batch*bw*bw floats in the reference layout, negative orders filled by
 * f(l,-m) = (-1)^m conj f(l,m) on output and ignored on input. */
int s2g_fst_real_f32(s2g_plan plan, const float* grid, float* rcoeffs, float* icoeffs, int batch, int precision,
                     void* stream);
int s2g_inv_fst_real_f32(s2g_plan plan, const float* rcoeffs, const float* icoeffs, float* grid, int batch,
                         int precision, void* stream);

/* COMPLEX data (FSTSemiMemo / InvFSTSemiMemo with DataFormat COMPLEX, FST_semi_memo.c:146-200 and
 * :290-333) on the split path: rgrid/igrid are the real and imaginary samples, batch*(2bw)^2
 * floats each; rcoeffs/icoeffs batch*bw*bw floats with every order in the reference layout (the
 * inverse reads all of them).  The field is taken as two real fields, f = g + i h, each through the
 * real-field transforms above (same precisions, bandwidths and cutoff rule), and combined per
 * coefficient: f(l, m) = g(l, m) + i h(l, m).  The plan holds 16*batch*bw^2 bytes of extra scratch. */
int s2g_fst_complex_f32(s2g_plan plan, const float* rgrid, const float* igrid, float* rcoeffs, float* icoeffs,
                        int batch, int precision, void* stream);
int s2g_inv_fst_complex_f32(s2g_plan plan, const float* rcoeffs, const float* icoeffs, float* rgrid, float* igrid,
                            int batch, int precision, void* stream);

/* Real-field transforms with FP64 samples and coefficients whose Legendre contraction runs as
 * split products (precision: S2G_PREC_BF16X3, _BF16X2 or _FP16X2) followed by one refinement
 * step with an FP64 residual: forward a1 = F(f), a = a1 + F(f - I64(a1)); inverse g1 = I(a),
 * g = g1 + I(a - F64(g1)), where I64/F64 are the FP64 transforms on the GPU.  Forward: the
 * coefficient error falls from about e (the split path's) to about e^2 (below 1e-10 with
 * BF16X3).  Inverse: the band-limited part of the sample error -- what a forward transform of
 * the output sees, F64(g) - a -- falls to about e^2 as well, but the split synthesis rounds its
 * samples to FP32, and that rounding noise lies outside the band the residual can see, so the
 * pointwise sample error stays at the FP32 level (about 1e-7).  Both cost one FP64 transform
 * (the residual) plus two split transforms.  Layouts as
 * s2g_fst_real_f32 (the inverse reads the non-negative orders); bandwidths as s2g_fst_real_f32,
 * plan cutoff == bw.  The plan grows its own scratch. */
int s2g_fst_refined(s2g_plan plan, const double* grid, double* rcoeffs, double* icoeffs, int batch, int precision,
                    void* stream);
int s2g_inv_fst_refined(s2g_plan plan, const double* rcoeffs, const double* icoeffs, double* grid, int batch,
                        int precision, void* stream);

/* Forward FP64 transform of ONE function that allocates no device memory (no counterpart in
 * the reference).  For callers that cannot call cudaMalloc/cudaFree -- code running inside a
 * framework that has already reserved its device memory budget, or latency-critical code that
 * cannot accept the implicit synchronisation of allocation -- the intermediate buffer and the
 * twiddle factors live in a fixed __device__ array of about 4 MiB held by every GPU that loads
 * the library.  All pointers are device pointers: samples, coefficients (as s2g_fst), the
 * seminaive/naive table in the SemiNaive_Naive_Pml_Table layout with its bw int64 order offsets,
 * and the 4*bw quadrature weights.  bw <= 256 (any such bw: when 2*bw is not a power of two
 * the Bluestein tables of its DFTs are rewritten into the array on every call); larger bw is
 * rejected with S2G_ERR_ARG.  The first
 * call on a device looks up the array's device address (make that first call before any stream
 * capture).  Calls share the array, so calls that overlap on the GPU race: serialise them. */
int s2g_fst_noalloc(const double* rdata, const double* idata, double* rcoeffs, double* icoeffs, int bw,
                    const double* table, const int64_t* table_offsets, const double* weights,
                    DataFormat data_format, int cutoff, void* stream);

/* Same on HOST buffers: copies in, transforms, copies out (chunked, copies overlapped with
 * compute on the plan's streams); returns when the results are in host memory. */
int s2g_fst_real_f32_host(s2g_plan plan, const float* grid, float* rcoeffs, float* icoeffs, int batch,
                          int precision);
int s2g_inv_fst_real_f32_host(s2g_plan plan, const float* rcoeffs, const float* icoeffs, float* grid, int batch,
                              int precision);

/* The same, queued without waiting: each call returns once its copies and transforms are queued
 * on the plan's streams, so the uploads of one call overlap the downloads of the one before (the
 * host link carries both directions at once).  Host memory that a queued call reads or writes is
 * tracked per chunk: a later call's upload from memory an earlier call downloads into waits for
 * that download, and a later download into memory an earlier call uploads from waits for that
 * upload, so chained calls on aliased buffers are ordered.  The caller leaves the buffers alone
 * until s2g_plan_wait returns.  Calls on the plan that take device buffers wait for queued
 * host-buffer work first (they share its scratch). */
int s2g_fst_real_f32_host_async(s2g_plan plan, const float* grid, float* rcoeffs, float* icoeffs, int batch,
                                int precision);
int s2g_inv_fst_real_f32_host_async(s2g_plan plan, const float* rcoeffs, const float* icoeffs, float* grid,
                                    int batch, int precision);
/* Waits for every host-buffer call queued on the plan. */
int s2g_plan_wait(s2g_plan plan);

/* Waits for the plan's device work and reports a failure recorded on the device by the
 * tensor-core kernels (S2G_ERR_TIMEOUT when a bounded wait expired); clears the record. */
int s2g_plan_sync_status(s2g_plan plan);

/* Grouped transforms of many real functions of uneven bandwidth (no counterpart in the
 * reference, which transforms one function per call).  Function f has bandwidth bw[f], any
 * bandwidth of the split path (16 .. 256, or a power of two up to 512), at most 16 distinct ones
 * per group; precision is a split mode (S2G_PREC_BF16X3, _BF16X2 or _FP16X2).  Layout
 * on the device: the functions back to back in the order given, function f's grid taking
 * (2 bw[f])^2 floats and its coefficients bw[f]^2 floats in each of rcoeffs/icoeffs (the
 * reference layout per function, negative orders written by symmetry as s2g_fst_real_f32);
 * s2g_group_layout returns the offsets.  A call runs each phi-FFT and DCT stage as at most two
 * grouped launches over the power-of-two classes (short transforms, bw <= 64, and long ones, run
 * concurrently) plus one launch per other class, and ONE persistent tensor-core contraction
 * launch over all classes; the sequence
 * is captured as a CUDA graph on the first call with a given set of pointers and replayed on later
 * calls with the same pointers.  Calls on one group must be serialised (they share the group's
 * intermediate buffers). */
typedef struct s2g_group_s* s2g_group;
int s2g_group_create(s2g_group* group, int nfunc, const int* bw, int precision);
int s2g_group_destroy(s2g_group group);
int s2g_group_layout(s2g_group group, int64_t* grid_offsets, int64_t* coeff_offsets, int64_t* grid_total,
                     int64_t* coeff_total);
int s2g_group_fst(s2g_group group, const float* grid, float* rcoeffs, float* icoeffs, void* stream);
int s2g_group_inv_fst(s2g_group group, const float* rcoeffs, const float* icoeffs, float* grid, void* stream);
/* forward of grid into the coefficients, then inverse of those into grid_out, one graph */
int s2g_group_fst_inv(s2g_group group, const float* grid, float* rcoeffs, float* icoeffs, float* grid_out,
                      void* stream);
/* Times candidate shapes (N extent of each class's contraction tile, depth of the contraction's
 * table-copy ring, resident blocks per SM the DCT stages are sized for) on the group's
 * whole forward + inverse sequence and keeps the fastest.  Results are cached per
 * (device, precision, class sizes); force != 0 re-measures.  $S2G_TUNE_CACHE, when set, names a
 * file that keeps them across processes.  Synchronous. */
int s2g_group_autotune(s2g_group group, int force);
/* Sets the shapes by hand: table_stages (the contraction's table-copy ring depth: 0 = as many as
 * fit, else 2..8) and one tile N per bandwidth class
 * in increasing bandwidth (0 = the class's whole table-row extent; NULL = all 0). */
int s2g_group_set_tiles(s2g_group group, int table_stages, const int* tile_n);
/* Sets the resident blocks per SM the grouped DCT stages are sized for (0 = as many as fit). */
int s2g_group_set_dct_ctas(s2g_group group, int dct_ctas_per_sm);
/* JSON description: classes [bw, count], chosen tiles, kernels per captured graph. */
int s2g_group_describe(s2g_group group, char* buf, size_t len);
/* Waits for the device and reports a failure recorded by the tensor-core kernels. */
int s2g_group_sync_status(s2g_group group);

/* ========================== Part 3: diagnostics =================================== */

/* Runs the split-BF16 tcgen05 machinery on one tile: D[128 x N] = A[128 x K] * B[N x K]^T
 * (row-major FP32 device arrays, N and K multiples of 16, N <= 256, K <= 128) with `nprod`
 * of the six split products (1 = plain BF16 ... 6 = 3-term split).  Synchronous. */
int s2g_selftest_tc(int N, int K, int nprod, const float* A, const float* B, float* D);

/* Selects the tensor-core contraction's data path for later calls (process-wide): 1 (default) =
 * the warp-specialised persistent kernel (scheduler/table-copy warp, MMA warp, A-producer warps,
 * epilogue warps; one CTA per SM) moving its A operand -- and the inverse its output -- by
 * tensor-map TMA where it can (one bandwidth class, BF16 terms, bw >= 64); 2 = the same kernel
 * with per-thread asynchronous copies only.  Both do the same arithmetic per work item and give
 * identical results. */
int s2g_set_contraction_kernel(int which);

/* Test hook for the failure path of the tensor-core contraction (off by default): with on != 0,
 * the warp-specialised contraction's scheduler publishes no work, so every other role's bounded
 * wait runs out (about half a second); the kernel then records S2G_ERR_TIMEOUT in the plan's
 * device word, frees its tensor memory and returns.  No fault, trap or hang is involved, and the
 * context stays usable: s2g_plan_sync_status reports the timeout and clears it. */
int s2g_test_stall_contraction(int on);

/* Kernel timing: while enabled, every kernel the library launches is bracketed by CUDA
 * events on the stream it is launched on.  s2g_prof_enable() also discards earlier records.
 * s2g_prof_report() waits for the recorded events and writes a JSON object
 * {"kernel": [launches, total_ms], ...} into buf. */
int s2g_prof_enable(int on);
int s2g_prof_report(char* buf, size_t len);
/* Number of kernels the library has launched in this process. */
unsigned long long s2g_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* S2KIT_GB300_H */
