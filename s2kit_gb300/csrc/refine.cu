// refine.cu -- split-precision transforms with one FP64-residual refinement step.
//
// Forward:  a1 = F_split(f);  r = f - I_fp64(a1);  a = a1 + F_split(r)
// Inverse:  g1 = I_split(a);  r = a - F_fp64(g1);  g = g1 + I_split(r)
// F and I are exact inverses on band-limited data (the Driscoll-Healy sampling theorem the
// reference's round trips rest on), so if the split transform has relative error e, the
// residual is -I(E1) with |E1| <= e|a|, and the corrected result has error about e^2: one step
// takes the 3-term split BF16 path (e ~ 1e-6) below 1e-10.  The residual and the sums are FP64;
// the two split transforms read FP32 samples/coefficients (the residual is small, so FP32 keeps
// its relative precision).
// The forward result is exact to e^2 only if the split forward leaves nothing the FP64 inverse
// ignores: for a real field that is Im f(l,0), which the split DCT writes as exact zeros.
// The inverse's samples g1 carry FP32 rounding noise that is not band-limited; F64 sees only
// its band-limited part, so the refined samples are exact to e^2 in that part (F64(g) = a to
// about e^2) while their pointwise error keeps the FP32 rounding of the split synthesis.
#include "s2g_internal.h"

namespace s2g {

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_f2d(const float* __restrict__ a, double* __restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// r = (float)(x - y)
__global__ void k_resid(const double* __restrict__ x, const double* __restrict__ y, float* __restrict__ r, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        r[i] = (float)(x[i] - y[i]);
}

// x += (double)d
__global__ void k_accum(double* __restrict__ x, const float* __restrict__ d, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        x[i] += (double)d[i];
}

static int ew_grid(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

#define S2G_EW(name, kern, n, st, ...)                                   \
    do {                                                                 \
        ProfScope ps_(name, st);                                         \
        kern<<<ew_grid(n), 256, 0, st>>>(__VA_ARGS__, n);                \
        S2G_CUDA(cudaGetLastError());                                    \
    } while (0)

static size_t rnd(size_t x) { return (x + 255) & ~(size_t)255; }

size_t refine_io_bytes(int bw, int batch) {
    const size_t ng = 4 * (size_t)bw * bw * batch, nc = (size_t)bw * bw * batch;
    // FP32 samples, 2 x FP32 coefficients, FP64 samples or 2 x FP64 coefficients
    return rnd(4 * ng) + 2 * rnd(4 * nc) + std::max(rnd(8 * ng), 2 * rnd(8 * nc)) + 256;
}

size_t refine_work_bytes(int bw, int batch) {
    return std::max(split_work_bytes(bw, batch), f64_work_bytes(bw, batch, REAL) + 256);
}

int fst_refined(Tables* t, const double* grid, double* rc, double* ic, int batch, int precision, void* io,
                void* work, cudaStream_t st) {
    const int B = t->bw;
    const size_t ng = 4 * (size_t)B * B * batch, nc = (size_t)B * B * batch;
    char* p = (char*)io;
    float* g32 = (float*)p;
    p += rnd(4 * ng);
    float* c32r = (float*)p;
    p += rnd(4 * nc);
    float* c32i = (float*)p;
    p += rnd(4 * nc);
    double* g64 = (double*)p;
    // a1 = F_split(f)
    S2G_EW("refine_d2f", k_d2f, ng, st, grid, g32);
    S2G_TRY(fst_split(t, g32, c32r, c32i, batch, precision, work, st));
    S2G_EW("refine_f2d", k_f2d, nc, st, c32r, rc);
    S2G_EW("refine_f2d", k_f2d, nc, st, c32i, ic);
    // r = f - I_fp64(a1)
    S2G_TRY(inv_fst_f64(t, rc, ic, g64, nullptr, batch, REAL, t->cutoff, work, st));
    S2G_EW("refine_resid", k_resid, ng, st, grid, g64, g32);
    // a = a1 + F_split(r)
    S2G_TRY(fst_split(t, g32, c32r, c32i, batch, precision, work, st));
    S2G_EW("refine_accum", k_accum, nc, st, rc, c32r);
    S2G_EW("refine_accum", k_accum, nc, st, ic, c32i);
    return S2G_OK;
}

int inv_fst_refined(Tables* t, const double* rc, const double* ic, double* grid, int batch, int precision, void* io,
                    void* work, cudaStream_t st) {
    const int B = t->bw;
    const size_t ng = 4 * (size_t)B * B * batch, nc = (size_t)B * B * batch;
    char* p = (char*)io;
    float* g32 = (float*)p;
    p += rnd(4 * ng);
    float* c32r = (float*)p;
    p += rnd(4 * nc);
    float* c32i = (float*)p;
    p += rnd(4 * nc);
    double* a64r = (double*)p;
    double* a64i = (double*)(p + rnd(8 * nc));
    // g1 = I_split(a)
    S2G_EW("refine_d2f", k_d2f, nc, st, rc, c32r);
    S2G_EW("refine_d2f", k_d2f, nc, st, ic, c32i);
    S2G_TRY(inv_fst_split(t, c32r, c32i, g32, batch, precision, work, st));
    S2G_EW("refine_f2d", k_f2d, ng, st, g32, grid);
    // r = a - F_fp64(g1)
    S2G_TRY(fst_f64(t, grid, nullptr, a64r, a64i, batch, REAL, t->cutoff, work, st));
    S2G_EW("refine_resid", k_resid, nc, st, rc, a64r, c32r);
    S2G_EW("refine_resid", k_resid, nc, st, ic, a64i, c32i);
    // g = g1 + I_split(r)
    S2G_TRY(inv_fst_split(t, c32r, c32i, g32, batch, precision, work, st));
    S2G_EW("refine_accum", k_accum, ng, st, grid, g32);
    return S2G_OK;
}

}  // namespace s2g
