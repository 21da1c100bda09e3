// s2g_internal.h -- internal (non-exported) declarations of the GB300 seminaive SHT library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <initializer_list>
#include <mutex>
#include <string>

#include "../../include/s2kit_gb300.h"

namespace s2g {

// Records a formatted message for s2g_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);
// cudaError_t -> status (records the CUDA error string)
int cuda_fail(cudaError_t e, const char* what);

#define S2G_CUDA(call)                                           \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ::s2g::cuda_fail(e_, #call); \
    } while (0)

#define S2G_TRY(call)            \
    do {                         \
        int r_ = (call);         \
        if (r_ != S2G_OK) return r_; \
    } while (0)

// Kernel launch accounting: every launch is counted; when profiling is enabled
// (s2g_prof_enable) it is also bracketed by CUDA events on its own stream.
void prof_begin(const char* name, cudaStream_t st);
void prof_end(cudaStream_t st);

// Graph capture on this thread: launches counted into the graph (see launches_add for replays).
void capture_count_begin();
unsigned long long capture_count_end();
void launches_add(unsigned long long n);

struct ProfScope {
    cudaStream_t st;
    ProfScope(const char* name, cudaStream_t s) : st(s) { prof_begin(name, s); }
    ~ProfScope() { prof_end(st); }
};

// Device tables and constants for one (bandwidth, cutoff) on one device.
struct Tables {
    int bw = 0, cutoff = 0, device = -1;
    int64_t total = 0;          // doubles in each of fwd / inv
    double* fwd = nullptr;      // reference layout: SemiNaive_Naive_Pml_Table (cospml.c:451-475)
    double* inv = nullptr;      // Transpose_SemiNaive_Naive_Pml_Table layout (cospml.c:490-518)
    int64_t* off = nullptr;     // bw offsets (device)
    int64_t* h_off = nullptr;   // same, host copy
    double* weights = nullptr;  // 4*bw (weights.c:32-47)
    double* sinv = nullptr;     // sin(theta_j), 2*bw
    double2* tw_S = nullptr;    // exp(2 pi i k / 2bw), k < 2bw   (cos, sin)
    double2* tw_D = nullptr;    // exp(i pi k / (2 * 2bw)), k < 2bw (DCT pre/post twiddle)
    // split-precision (tensor core) operands, built on first use
    void* split = nullptr;
    int refs = 0;               // references (cache, plans, groups, calls in flight); under the cache lock
};

// Device scratch owned by a plan; grown on demand.
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t need);
    void release();
};

// The FP32 transforms move samples and coefficients as float4 and through TMA, so their device
// pointers must be 16-byte aligned (every cudaMalloc pointer is); others are rejected up front.
inline int check_aligned16(std::initializer_list<const void*> ps) {
    for (const void* q : ps)
        if ((uintptr_t)q & 15) return fail(S2G_ERR_ARG, "device pointer %p is not 16-byte aligned", q);
    return S2G_OK;
}

// Build / fetch device tables (cached per device, bw, cutoff); the caller gets a reference and
// returns it with put_tables.  cutoff 0 gives the weights, nodes and twiddles of bw without any
// Legendre table (fwd, inv and off null), for the on-the-fly family.
int get_tables(int bw, int cutoff, Tables** out);
void put_tables(Tables* t);
struct TabRef {
    Tables* t;
    ~TabRef() { put_tables(t); }
};
// Build tables into caller-visible device buffers (used by the host table builders).
// Allocates and fills t's device tables; with h_fwd/h_inv (host copies of total doubles each,
// e.g. read from a table file) the Legendre tables are uploaded instead of generated.
int build_tables(Tables* t, cudaStream_t st, const double* h_fwd = nullptr, const double* h_inv = nullptr);
int generate_weights_device(int bw, double* d_weights, cudaStream_t st);
int generate_cos_pml_device(int bw, int m_begin, int m_end, double* d_fwd, const int64_t* d_off,
                            cudaStream_t st);
int transpose_cos_pml_device(int bw, int m_begin, int m_end, const double* d_fwd, double* d_inv,
                             const int64_t* d_off, cudaStream_t st);
int generate_pml_device(int bw, int m_begin, int m_end, double* d_fwd, const int64_t* d_off, cudaStream_t st);
int pmm_device(int m, const double* d_eval, int n, double* d_out, cudaStream_t st);
int nodes_device(int n, double* d_out, int acos_only, cudaStream_t st);

// ---- FP64 pipeline (sht_fp64.cu) ----
struct F64Work {
    double* Xr;  // [batch][rows][2bw]
    double* Xi;
    int rows;    // rows per function in X (bw for REAL, 2bw for COMPLEX)
};
size_t f64_work_bytes(int bw, int batch, int data_format);
int fst_f64(const Tables* t, const double* rdata, const double* idata, double* rc, double* ic, int batch,
            int data_format, int cutoff, void* work, cudaStream_t st);
// fst_f64 with the DFT geometry of length 2bw (Bluestein tables included when 2bw is not a
// power of two) supplied by the caller instead of looked up in the per-device length cache,
// which builds missing tables with cudaMalloc.  Null `len_S` behaves like fst_f64.
struct Len;
int fst_f64_len(const Tables* t, const Len* len_S, const double* rdata, const double* idata, double* rc,
                double* ic, int batch, int data_format, int cutoff, void* work, cudaStream_t st);
int inv_fst_f64(const Tables* t, const double* rc, const double* ic, double* rdata, double* idata, int batch,
                int data_format, int cutoff, void* work, cudaStream_t st);
// On-the-fly family (FST_semi_fly.c): the Legendre functions are generated inside the
// contraction kernels, so `t` needs only its weights and twiddles (tables of cutoff 0, see
// get_tables); work as f64_work_bytes.
int fst_f64_fly(const Tables* t, const double* rdata, const double* idata, double* rc, double* ic, int batch,
                int data_format, void* work, cudaStream_t st);
int inv_fst_f64_fly(const Tables* t, const double* rc, const double* ic, double* rdata, double* idata, int batch,
                    int data_format, void* work, cudaStream_t st);
int fzt_f64_fly(const Tables* t, const double* rdata, const double* idata, double* rres, double* ires, int batch,
                int data_format, void* work, cudaStream_t st);
int fzt_f64(const Tables* t, const double* rdata, const double* idata, double* rres, double* ires, int batch,
            int data_format, void* work, cudaStream_t st);
int transmult_f64(const double* rd, const double* id, const double* rf, const double* iff, double* rr,
                  double* ir, int bw, int batch, cudaStream_t st);
// 1-D transforms with caller-provided (device) tables for a single order m
int dlt_semi_f64(const double* data, int bw, int m, double* result, const double* table, const double* weights,
                 const double2* tw_S, const double2* tw_D, cudaStream_t st);
int inv_dlt_semi_f64(const double* coeffs, int bw, int m, double* result, const double* ttable,
                     const double* sinv, const double2* tw_S, const double2* tw_D, cudaStream_t st);
int dlt_naive_f64(const double* data, int bw, int m, const double* weights, double* result, const double* ptable,
                  cudaStream_t st);
int inv_dlt_naive_f64(const double* coeffs, int bw, int m, double* result, const double* ptable,
                      cudaStream_t st);
int twiddles_device(int n, double2* d_tw_full, double2* d_tw_quarter, cudaStream_t st);

// ---- split-precision pipeline (sht_split.cu, czt_split.cu) ----
// Orders the split path computes with the naive transform: odd m below 32.  For these the cosine
// series of G = P/sin(theta) has large coefficients, and FP32 rounding of the DCT output is
// amplified by them (the reference's seminaive/naive hybrid, FST_semi_memo.c:96-120, makes the
// same trade at the other end of the order range).
constexpr int kSplitNaiveOddBelow = 32;
__host__ __device__ __forceinline__ bool split_naive_order(int m) { return (m & 1) && m < kSplitNaiveOddBelow; }
// Layout of the split path's intermediate arrays at bandwidth bw, per plane (re, im), function
// and order m < bw: X and F rows of SX floats (latitudes theta < 2bw; a naive order's folded
// halves at t BN, t = 0, 1), C and Fc rows of 2 BH floats (cosine frequency k = 2j + t at t BH + j).
// bw itself (BH = bw/2, BN = bw, SX = 2bw) where the warp FFTs take length 2bw; at the chirp-z
// bandwidths BN and BH are rounded up to multiples of 8, the padding held at zero.
struct SplitLayout {
    int BH, BN, SX;
};
SplitLayout split_layout(int bw);
// True where the split path's length-2bw DFTs run as chirp-z transforms (czt_split.cu): bw in
// [17, 256] and 2bw not a warp-FFT length.
bool split_czt(int bw);
// Length M of the chirp-z convolution at bandwidth bw: the power of two >= 4 bw - 1 (at least 128).
int czt_len(int bw);
// Device tables of one chirp-z bandwidth (the first three from czt_build_tables, the rest the
// split path's FP32 weights, sin(theta) and DCT twiddles).
struct CztTabs {
    int B, M;
    const float2* h;     // exp(-i pi (n^2 mod 2S) / S), n < S = 2B
    const float2* K;     // DFT_M of b_j = conj(h_|j|) (|j| < S, j mod M), divided by M
    const float2* twM;   // exp(2 pi i k / M), k < M
    const float* w32;    // quadrature weights, 2S (even orders, then odd)
    const float* sin32;  // sin(theta_j), S
    const float2* twD;   // (cos, sin)(pi k / 2S), k < S
};
int czt_build_tables(int bw, float2** d_h, float2** d_K, float2** d_tw);
// One FFT stage (which: 0 rows forward, 1 weighted DCT-II, 2 DCT-III, 3 rows inverse) of N
// functions at a chirp-z bandwidth; in/out, scale and gmap as the warp-FFT stages.
int czt_stage(int which, const CztTabs& g, const void* in, void* out, int N, float scale, const int64_t* gmap,
              cudaStream_t st);
size_t split_work_bytes(int bw, int batch);
int fst_split(Tables* t, const float* grid, float* rc, float* ic, int batch, int precision, void* work,
              cudaStream_t st);
int inv_fst_split(Tables* t, const float* rc, const float* ic, float* grid, int batch, int precision, void* work,
                  cudaStream_t st);
// COMPLEX data as two real fields (cwork: split_complex_bytes of scratch besides work).
size_t split_complex_bytes(int bw, int batch);
int fst_split_complex(Tables* t, const float* rgrid, const float* igrid, float* rc, float* ic, int batch,
                      int precision, void* work, void* cwork, cudaStream_t st);
int inv_fst_split_complex(Tables* t, const float* rc, const float* ic, float* rgrid, float* igrid, int batch,
                          int precision, void* work, void* cwork, cudaStream_t st);
// One FFT stage of several bandwidth classes (split path, power-of-two bw <= 512) in ONE launch:
// which 0 rows forward (grid -> X), 1 weighted DCT-II (X -> C), 2 DCT-III (Fc -> F), 3 rows
// inverse (F -> grid); in/out as the per-class kernels, gmap per-function grid offsets for the
// rows stages.  dct_ctas_per_sm bounds the resident blocks the DCT stages are sized for (0: as
// many as fit).
struct StageSpec {
    Tables* t;
    int N;
    const void* in;
    void* out;
    const int64_t* gmap;
};
int split_stage_group(int which, const StageSpec* spec, int ncls, int dct_ctas_per_sm, cudaStream_t st);
// The same stage for one class of any split-path bandwidth, as its own launch.
int split_stage_one(int which, Tables* t, int N, const void* in, void* out, const int64_t* gmap, cudaStream_t st);
// Reads (and optionally clears) the device error word of the tensor-core kernels.
int split_device_status(Tables* t, int clear);

// One bandwidth class of a (grouped) tensor-core contraction launch.  Intermediate arrays are
// class-contiguous: X/F [2][N][B][SX], C/Fc [2][N][B][2 BH] floats (split_layout(B)).
struct LegSpec {
    Tables* t;
    int N;                    // functions of this class
    int NB;                   // table rows per work item (0: the largest the class needs)
    const float* C;           // forward: DCT output
    const float* X;           // forward: phi-DFT output (naive orders)
    const float* rc_in;       // inverse: input coefficients
    const float* ic_in;
    float* rc;                // forward: output coefficients
    float* ic;
    float* Fc;                // inverse: cosine-series output
    float* F;                 // inverse: naive-order output
    const int64_t* cmap;      // function -> coefficient offset (null: f * B * B)
};
// One persistent launch over every class; counter: one device int (zeroed on `st` here);
// table_stages: depth of the kernel's table-copy ring, 0 = as many stages as fit.
int split_leg(bool fwd, int precision, const LegSpec* cls, int ncls, int* counter, int table_stages,
              cudaStream_t st);
// Packs the tensor-core operands of `t` for `precision` now (they are otherwise packed on first use).
int split_prepare(Tables* t, int precision);
int split_fwd_head(Tables* t, const float* grid, float* X, float* C, int batch, const int64_t* gmap,
                   cudaStream_t st);
int split_inv_tail(Tables* t, float* F, float* Fc, float* grid, int batch, const int64_t* gmap, cudaStream_t st);

// ---- split transforms with one FP64-residual refinement step (refine.cu) ----
size_t refine_io_bytes(int bw, int batch);
size_t refine_work_bytes(int bw, int batch);
int fst_refined(Tables* t, const double* grid, double* rc, double* ic, int batch, int precision, void* io,
                void* work, cudaStream_t st);
int inv_fst_refined(Tables* t, const double* rc, const double* ic, double* grid, int batch, int precision, void* io,
                    void* work, cudaStream_t st);

}  // namespace s2g
