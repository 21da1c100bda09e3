/*
 * s2oracle.h -- CPU restatement of S2kit 1.1's seminaive "memo" spherical harmonic
 * transform path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * implementation in s2kit_gb300/ and the timed CPU baseline ("port") in bench.py.
 * It is never linked into, loaded by or called from the product path.
 *
 * Parity pinning: the restatement is checked against
 *   - the reference's golden convolution outputs data/o{64,128}_conv_semi_memo_original.dat
 *     (produced by the reference with real FFTW3),
 *   - the analytic known-answer inputs data/y20_bw8.dat, y31_bw8.dat (and the odd-bandwidth
 *     y43_bw23.dat / yMix_bw17.dat forward cases),
 *   - outputs of the reference C sources compiled here against oracle/fftw_shim
 *     (the tests/golden/ref_*.npz fixtures, generated by tests/golden/make_golden.py).
 *
 * Every function cites the reference file:line it restates (paths relative to the
 * S2kit repository root).  All arithmetic is FP64, as in the reference.
 */
#ifndef S2ORACLE_H
#define S2ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* DataFormat values, include/s2kit/util.h:16-19 */
enum { ORC_COMPLEX = 0, ORC_REAL = 1 };

/* ---- index / size helpers (src/util/util.c:42-49, src/legendre_polynomials/cospml.c) ---- */
int orc_index_of_harmonic_coeff(int m, int l, int bw);
int64_t orc_table_size(int m, int bw);
int64_t orc_table_offset(int m, int l);
int orc_row_size(int m, int l);
int orc_transpose_row_size(int row, int m, int bw);
int64_t orc_reduced_spharmonic_table_size(int bw, int cutoff);
int64_t orc_reduced_naive_table_size(int bw, int cutoff);

/* ---- 1-D transforms with FFTW's documented conventions ---- */
/* unnormalised DFT, sign = -1 (forward) or +1, in place on split re/im */
void orc_dft(int n, double* re, double* im, int sign);
/* FFTW_REDFT10: out[k] = 2 sum_j in[j] cos(pi (j+1/2) k / n) */
void orc_redft10(int n, const double* in, double* out);
/* FFTW_REDFT01: out[k] = in[0] + 2 sum_{j>=1} in[j] cos(pi j (k+1/2) / n) */
void orc_redft01(int n, const double* in, double* out);
/* O(n^2) definitions of the same, used to pin the fast versions in tests */
void orc_redft10_direct(int n, const double* in, double* out);
void orc_redft01_direct(int n, const double* in, double* out);

/* ---- table generation ---- */
void orc_pmm_l2(int m, const double* eval_points, int n, double* result);
double orc_l2_an(int m, int l);
double orc_l2_cn(int m, int l);
void orc_generate_weights(int bw, double* weights);                 /* 4*bw doubles */
void orc_generate_cos_pml_table(int bw, int m, double* table);      /* TableSize(m,bw) */
void orc_transpose_cos_pml_table(int bw, int m, const double* table, double* result);
void orc_generate_pml_table(int bw, int m, double* table);          /* 2*bw*(bw-m) */

/* Full memo table set (forward + transposed) in the reference's packed layout:
 * order m starts at offsets[m] in both buffers (SemiNaive_Naive_Pml_Table,
 * cospml.c:451-475 and Transpose_SemiNaive_Naive_Pml_Table, cospml.c:490-518). */
typedef struct {
    int bw, cutoff;
    int64_t total;     /* doubles in each buffer */
    int64_t* offsets;  /* bw entries */
    double* fwd;
    double* inv;
} orc_tables;

orc_tables* orc_tables_new(int bw, int cutoff);
/* Same tables, the orders generated by `nthreads` threads (orders interleaved across them). */
orc_tables* orc_tables_new_mt(int bw, int cutoff, int nthreads);
void orc_tables_free(orc_tables* t);
/* Accessors for ctypes callers */
int64_t orc_tables_total(const orc_tables* t);
const double* orc_tables_fwd(const orc_tables* t);
const double* orc_tables_inv(const orc_tables* t);
const int64_t* orc_tables_offsets(const orc_tables* t);

/* ---- Legendre transforms ---- */
void orc_dlt_semi(const double* data, int bw, int m, double* result, const double* cos_pml_table,
                  const double* weights);
void orc_inv_dlt_semi(const double* coeffs, int bw, int m, double* result, const double* trans_cos_pml_table,
                      const double* sin_values);
void orc_dlt_naive(const double* data, int bw, int m, const double* weights, double* result,
                   const double* pml_table);
void orc_inv_dlt_naive(const double* coeffs, int bw, int m, double* result, const double* pml_table);

/* ---- sphere transforms ---- */
void orc_fst(const double* rdata, const double* idata, double* rcoeffs, double* icoeffs, int bw,
             const orc_tables* t, const double* weights, int data_format, int cutoff);
void orc_inv_fst(const double* rcoeffs, const double* icoeffs, double* rdata, double* idata, int bw,
                 const orc_tables* t, int data_format, int cutoff);
void orc_fzt(const double* rdata, const double* idata, double* rres, double* ires, int bw,
             const double* cos_pml_table_m0, const double* weights, int data_format);
void orc_transmult(const double* rdatacoeffs, const double* idatacoeffs, const double* rfiltercoeffs,
                   const double* ifiltercoeffs, double* rres, double* ires, int bw);
void orc_conv(const double* rdata, const double* idata, const double* rfilter, const double* ifilter,
              double* rres, double* ires, int bw);
/* orc_conv on tables built beforehand (orc_tables_new*(bw, bw)) instead of per call. */
void orc_conv_tables(const double* rdata, const double* idata, const double* rfilter, const double* ifilter,
                     double* rres, double* ires, int bw, const orc_tables* t);

/* ---- timed CPU baseline: nfunc independent REAL round trips (InvFST then FST, cutoff=bw),
 * one function per thread at a time, private workspaces, shared read-only tables.
 * coeffs_in: nfunc*2*bw*bw (re plane then im plane per function); coeffs_out same.
 * Returns wall-clock seconds of the transform loop (tables excluded). */
double orc_bench_roundtrip(int bw, int nfunc, int nthreads, const double* coeffs_in, double* coeffs_out);

#ifdef __cplusplus
}
#endif
#endif
