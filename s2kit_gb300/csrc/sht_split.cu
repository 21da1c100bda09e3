// sht_split.cu -- real-field SHT with FP32 samples/coefficients and the seminaive Legendre
// contraction on the 5th-generation tensor cores as split-BF16 products (FP32 accumulation in TMEM).
//
// Forward (FSTSemiMemo, REAL, cutoff = bw; FST_semi_memo.c:68-145):
//   k_rows_fwd_w       : DFT along phi (warp FFT, two real latitudes per warp), X[p][f][m][theta]
//   k_dct_fwd_w        : weights (even/odd order) + REDFT10 + normalisation (seminaive.c:161-176)
//                        -> C[p][f][m][k], k < bw
//   k_leg_fwd_tc       : per (order m, 64 functions): for each parity t of (l - m), the dense
//                        trapezoid T_{m,t}[i][j] = T(m, l = m+t+2i, k = 2j+t) times C (seminaive.c:183-197)
//                        as D[128 x N] = A[128 x K] * B[N x K]^T on tcgen05, A = 64 functions x
//                        (re, im) rows, B = table rows; epilogue writes f(l, m) and f(l, -m).
// Inverse (InvFSTSemiMemo, REAL; FST_semi_memo.c:228-351):
//   k_leg_inv_tc       : fcos[2j+t] = sum_i T_{m,t}[i][j] a(m + t + 2i) (seminaive.c:74-98), scaled
//   k_dct_inv_w        : REDFT01, sin(theta) for odd m, 1/sqrt(2 pi)
//   k_naive_combine    : naive orders (odd m < 32): even/odd latitude halves back to samples
//   k_rows_inv_w       : DFT with sign +1 over m, Hermitian rows, two latitudes per warp
//
// Precision: x = x0 + x1 + x2 with BF16 terms (each the rounded residual of the previous);
// the table is split the same way from FP64.  S2G_PREC_BF16X3 sums the six products
// x_a t_b with a + b <= 2, S2G_PREC_BF16X2 the three with a + b <= 1.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "s2g_common.cuh"
#include "s2g_internal.h"
#include "fft32.cuh"
#include "tc_sm103.cuh"

namespace s2g {

static constexpr double kPi = 3.14159265358979323846;

struct Split {
    int B = 0, KC = 0;
    float* w32 = nullptr;        // 4B weights
    float* sin32 = nullptr;      // 2B
    float2* twS = nullptr;       // exp(2 pi i k / S), k < S
    float2* twD = nullptr;       // (cos, sin)(pi k / 2S), k < S
    uint8_t* fwd_blob = nullptr;
    uint8_t* inv_blob = nullptr;
    int64_t* fwd_off = nullptr;  // device, bytes, per order
    int64_t* inv_off = nullptr;
    int* err = nullptr;          // device error word (S2G_ERR_TIMEOUT on an expired wait)
    size_t fwd_bytes = 0, inv_bytes = 0;
};

static std::mutex g_split_mu;

void free_split(Tables* t) {
    Split* s = (Split*)t->split;
    if (!s) return;
    cudaFree(s->w32);
    cudaFree(s->sin32);
    cudaFree(s->twS);
    cudaFree(s->twD);
    cudaFree(s->fwd_blob);
    cudaFree(s->inv_blob);
    cudaFree(s->fwd_off);
    cudaFree(s->inv_off);
    cudaFree(s->err);
    delete s;
    t->split = nullptr;
}

__host__ __device__ __forceinline__ int round16(int x) { return (x + 15) & ~15; }
__host__ __device__ __forceinline__ int nr_par(int B, int m, int t) { return (B - m - t + 1) / 2; }

// Orders computed with the naive transform in the split path: odd m below 32.  For these the
// cosine series of G = P/sin(theta) has large coefficients, and FP32 rounding of the DCT
// output is amplified by them (the reference's seminaive/naive hybrid, FST_semi_memo.c:96-120,
// makes the same trade at the other end of the order range).
static constexpr int kNaiveOddBelow = 32;
__host__ __device__ __forceinline__ bool naive_order(int m) { return (m & 1) && m < kNaiveOddBelow; }

static constexpr int kKC = 32;   // K columns per pipeline chunk (two K=16 MMA steps)
static constexpr int kNBN = 128; // latitude block of the naive inverse (N per CTA)

// Geometry of the tensor-core contraction for one (direction, order): rows of the table
// operand per CTA (N), K extent, K chunks and latitude blocks.
struct Geo {
    int NP, KX, nch, nblk;
};

__host__ __device__ __forceinline__ Geo geo(bool fwd, int B, int m) {
    Geo g;
    const bool nv = naive_order(m);
    const int nr0 = nr_par(B, m, 0);
    if (fwd) {
        g.NP = round16(nr0);
        g.KX = nv ? B : B / 2;
        g.nblk = 1;
    } else {
        g.KX = nr0;
        const int nbn = B < kNBN ? B : kNBN;
        g.NP = nv ? nbn : round16(B / 2);
        g.nblk = nv ? B / nbn : 1;
    }
    g.nch = (g.KX + kKC - 1) / kKC;
    return g;
}

__host__ __device__ __forceinline__ int64_t blob_bytes(bool fwd, int B, int m) {
    const Geo g = geo(fwd, B, m);
    return (int64_t)2 * g.nblk * g.nch * 3 * g.NP * kKC * 2;
}

// ------------------------------------------------------------------------------------
// Operand packing: table operands in the tcgen05 smem layout, three BF16 terms, one
// contiguous blob per (order, parity, latitude block, K-chunk): [term][NP rows][KC].
//   forward seminaive : rows i (l = m+t+2i), cols j (cosine frequency k = 2j+t)
//   forward naive     : rows i, cols j (latitude j < B): P(m,l)(x_j) w_j  (even/odd folded)
//   inverse seminaive : rows j, cols i
//   inverse naive     : rows theta (block nb), cols i: P(m,l_i)(x_theta)
__device__ __forceinline__ double tz(const double* tab, int m, int B, int t, int i, int j) {
    const int l = m + t + 2 * i;
    if (l >= B || j > m / 2 + i) return 0.0;
    return tab[table_offset(m, l) + j];
}

__device__ __forceinline__ void split3d(double v, __nv_bfloat16* h) {
    h[0] = __double2bfloat16(v);
    const double r1 = v - (double)__bfloat162float(h[0]);
    h[1] = __double2bfloat16(r1);
    const double r2 = r1 - (double)__bfloat162float(h[1]);
    h[2] = __double2bfloat16(r2);
}

struct Pack {
    int B;
    const double* fwd;      // seminaive tables (reference layout)
    const int64_t* off;
    const double* pml;      // sampled P(m,l)(x_j), [l-m][2B] per naive order
    const int64_t* pml_off;
    const double* w;        // quadrature weights
    uint8_t* blob;
    const int64_t* blob_off;
};

template <bool FWD>
__global__ void k_pack(Pack p) {
    const int B = p.B, S = 2 * B;
    const int m = blockIdx.x, c = blockIdx.y;
    const int t = blockIdx.z & 1, nb = blockIdx.z >> 1;
    const Geo g = geo(FWD, B, m);
    if (c >= g.nch || nb >= g.nblk) return;
    const bool nv = naive_order(m);
    const size_t tile = (size_t)g.NP * kKC * 2;
    uint8_t* out = p.blob + p.blob_off[m] + ((size_t)(t * g.nblk + nb) * g.nch + c) * 3 * tile;
    const double* tab = p.fwd + p.off[m];
    const double* pml = nv ? p.pml + p.pml_off[m] : nullptr;
    for (int e = threadIdx.x; e < g.NP * kKC; e += blockDim.x) {
        const int n = e / kKC, kk = e - n * kKC;
        const int kidx = c * kKC + kk;
        double v = 0.0;
        if (FWD) {
            const int i = n, l = m + t + 2 * i;
            if (!nv) v = tz(tab, m, B, t, i, kidx);
            else if (l < B && kidx < B) v = pml[(size_t)(l - m) * S + kidx] * p.w[kidx];
        } else {
            const int i = kidx, l = m + t + 2 * i;
            if (!nv) v = tz(tab, m, B, t, i, n);
            else {
                const int th = nb * g.NP + n;
                if (l < B && th < B) v = pml[(size_t)(l - m) * S + th];
            }
        }
        __nv_bfloat16 h[3];
        split3d(v, h);
        for (int s = 0; s < 3; ++s) *(__nv_bfloat16*)(out + s * tile + tc::tile_off(n, kk, kKC)) = h[s];
    }
}

__global__ void k_to_f32(const double* a, float* b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

__global__ void k_tw_f32(const double2* a, float2* b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

static int build_split(Tables* t) {
    std::lock_guard<std::mutex> lk(g_split_mu);
    if (t->split) return S2G_OK;
    const int B = t->bw, S = 2 * B;
    if ((B & (B - 1)) || B < 16 || B > 512)
        return fail(S2G_ERR_UNSUPPORTED, "split-precision path needs a power-of-two bw in [16, 512] (got %d)", B);
    if (t->cutoff != B) return fail(S2G_ERR_UNSUPPORTED, "split-precision path is seminaive at every order (cutoff == bw)");
    Split* s = new Split();
    s->B = B;
    s->KC = kKC;
    std::vector<int64_t> fo(B), io(B), po(B, 0);
    int64_t fb = 0, ib = 0, pb = 0;
    for (int m = 0; m < B; ++m) {
        fo[m] = fb;
        io[m] = ib;
        fb += blob_bytes(true, B, m);
        ib += blob_bytes(false, B, m);
        if (naive_order(m)) {
            po[m] = pb;
            pb += (int64_t)(B - m) * S;
        }
    }
    s->fwd_bytes = fb;
    s->inv_bytes = ib;
    cudaStream_t st;
    S2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int r = S2G_OK;
    auto ck = [&](cudaError_t e, const char* w) {
        if (e != cudaSuccess && r == S2G_OK) r = cuda_fail(e, w);
    };
    double* pml = nullptr;
    int64_t* d_po = nullptr;
    ck(cudaMalloc(&s->w32, sizeof(float) * 4 * B), "cudaMalloc");
    ck(cudaMalloc(&s->sin32, sizeof(float) * S), "cudaMalloc");
    ck(cudaMalloc(&s->twS, sizeof(float2) * S), "cudaMalloc");
    ck(cudaMalloc(&s->twD, sizeof(float2) * S), "cudaMalloc");
    ck(cudaMalloc(&s->fwd_blob, fb), "cudaMalloc");
    ck(cudaMalloc(&s->inv_blob, ib), "cudaMalloc");
    ck(cudaMalloc(&s->fwd_off, sizeof(int64_t) * B), "cudaMalloc");
    ck(cudaMalloc(&s->inv_off, sizeof(int64_t) * B), "cudaMalloc");
    ck(cudaMalloc(&s->err, sizeof(int)), "cudaMalloc");
    ck(cudaMalloc(&pml, sizeof(double) * (size_t)(pb > 0 ? pb : 1)), "cudaMalloc");
    ck(cudaMalloc(&d_po, sizeof(int64_t) * B), "cudaMalloc");
    if (r == S2G_OK) {
        ck(cudaMemsetAsync(s->err, 0, sizeof(int), st), "memset");
        ck(cudaMemcpyAsync(s->fwd_off, fo.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st), "copy");
        ck(cudaMemcpyAsync(s->inv_off, io.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st), "copy");
        ck(cudaMemcpyAsync(d_po, po.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st), "copy");
        {
            ProfScope ps_("to_f32", st);
            k_to_f32<<<(4 * B + 255) / 256, 256, 0, st>>>(t->weights, s->w32, 4 * B);
        }
        {
            ProfScope ps_("to_f32", st);
            k_to_f32<<<(S + 255) / 256, 256, 0, st>>>(t->sinv, s->sin32, S);
        }
        {
            ProfScope ps_("tw_f32", st);
            k_tw_f32<<<(S + 255) / 256, 256, 0, st>>>(t->tw_S, s->twS, S);
        }
        {
            ProfScope ps_("tw_f32", st);
            k_tw_f32<<<(S + 255) / 256, 256, 0, st>>>(t->tw_D, s->twD, S);
        }
        ck(cudaGetLastError(), "conversion kernels");
    }
    // sampled P(m,l) of the naive orders (pml.c:41-79), one order at a time
    for (int m = 1; r == S2G_OK && m < B && m < kNaiveOddBelow; m += 2) {
        int rr = generate_pml_device(B, m, m + 1, pml, d_po, st);
        if (rr != S2G_OK) r = rr;
    }
    if (r == S2G_OK) {
        Pack pk{B, t->fwd, t->off, pml, d_po, t->weights, s->fwd_blob, s->fwd_off};
        int maxch = 0;
        for (int m = 0; m < B; ++m) maxch = std::max(maxch, geo(true, B, m).nch);
        {
            ProfScope ps_("pack_fwd", st);
            k_pack<true><<<dim3(B, maxch, 2), 256, 0, st>>>(pk);
        }
        pk.blob = s->inv_blob;
        pk.blob_off = s->inv_off;
        maxch = 0;
        int maxblk = 1;
        for (int m = 0; m < B; ++m) {
            maxch = std::max(maxch, geo(false, B, m).nch);
            maxblk = std::max(maxblk, geo(false, B, m).nblk);
        }
        {
            ProfScope ps_("pack_inv", st);
            k_pack<false><<<dim3(B, maxch, 2 * maxblk), 256, 0, st>>>(pk);
        }
        ck(cudaGetLastError(), "pack kernels");
        ck(cudaStreamSynchronize(st), "pack kernels");
    }
    cudaFree(pml);
    cudaFree(d_po);
    cudaStreamDestroy(st);
    t->split = s;
    if (r != S2G_OK) free_split(t);
    return r;
}

// ------------------------------------------------------------------------------------
// Warp-FFT kernels (fft32.cuh), S = 2B = 32 R.  One warp owns one complex sequence; layout
// changes go through padded shared memory.

// Loads tw[k] = exp(2 pi i k / S), twD[k] = (cos, sin)(pi k / 2S) for k < S into shared memory.
// (tw padded as padtw(k), see fft32.cuh; twD unpadded)
__device__ __forceinline__ void load_tw(float2* tw, float2* twD, const float2* gS, const float2* gD, int S) {
    for (int k = threadIdx.x; k < S; k += blockDim.x) {
        tw[padtw(k)] = gS[k];
        if (twD) twD[k] = gD[k];
    }
}

static constexpr int kWarps = 8;       // warps per CTA in the FFT kernels
static constexpr int kLatPerCta = 16;  // latitudes per CTA in the row kernels (2 per warp)

// DFT along phi of 16 latitudes (two real rows per warp), transposed to X[p][f][m][theta], m < B.
template <int R>
__global__ void __launch_bounds__(256) k_rows_fwd_w(const float* __restrict__ grid, float* __restrict__ X, int N,
                                                    float scale, const float2* __restrict__ gtw) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int PS = S + S / 32;        // padded spectrum length
    constexpr int RS = B + B / 32 + 1;    // padded stage row (odd)
    constexpr int TWL = twtab_len(S);
    extern __shared__ __align__(16) float fsm[];
    float2* tw = reinterpret_cast<float2*>(fsm);
    float* spr = fsm + 2 * TWL;                    // [warps][PS] re
    float* spi = spr + kWarps * PS;                // [warps][PS] im
    float* str = spi + kWarps * PS;                // [16][RS] re
    float* sti = str + kLatPerCta * RS;            // [16][RS] im
    const int f = blockIdx.y, th0 = blockIdx.x * kLatPerCta;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    load_tw(tw, nullptr, gtw, nullptr, S);
    __syncthreads();
    const int la = th0 + 2 * warp;
    if (la < S) {
        const float* ra = grid + ((size_t)f * S + la) * S;
        const float* rb = ra + S;
        float2 v[R];
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = make_float2(ra[lane + 32 * i], (la + 1 < S) ? rb[lane + 32 * i] : 0.f);
        WarpFFT<R>::run(v, tw, -1.f);
        float* wr = spr + warp * PS;
        float* wi = spi + warp * PS;
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            const int o = pad32(WarpFFT<R>::out_index(k1));
            wr[o] = v[k1].x;
            wi[o] = v[k1].y;
        }
        __syncwarp();
        for (int m = lane; m < B; m += 32) {
            const int mm = (S - m) & (S - 1);
            const float zr = wr[pad32(m)], zi = wi[pad32(m)], xr = wr[pad32(mm)], xi = wi[pad32(mm)];
            str[(2 * warp) * RS + pad32(m)] = 0.5f * (zr + xr) * scale;
            sti[(2 * warp) * RS + pad32(m)] = 0.5f * (zi - xi) * scale;
            str[(2 * warp + 1) * RS + pad32(m)] = 0.5f * (zi + xi) * scale;
            sti[(2 * warp + 1) * RS + pad32(m)] = -0.5f * (zr - xr) * scale;
        }
    }
    __syncthreads();
    const int nlat = min(kLatPerCta, S - th0);
    const size_t plane = (size_t)N * B * S;
    for (int e = threadIdx.x; e < B * kLatPerCta; e += blockDim.x) {
        const int m = e / kLatPerCta, q = e - m * kLatPerCta;
        if (q >= nlat) continue;
        const size_t o = ((size_t)f * B + m) * S + th0 + q;
        X[o] = str[q * RS + pad32(m)];
        X[plane + o] = sti[q * RS + pad32(m)];
    }
}

// Weighted REDFT10 per (function, seminaive order) row: C[p][f][m][k], k < B.
template <int R>
__global__ void __launch_bounds__(256) k_dct_fwd_w(const float* __restrict__ X, float* __restrict__ Cout, int nrows,
                                                   const float* __restrict__ gw, const float2* __restrict__ gtw,
                                                   const float2* __restrict__ gtwD) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int PS = S + S / 32;
    constexpr int TWL = twtab_len(S);
    extern __shared__ __align__(16) float fsm[];
    float2* tw = reinterpret_cast<float2*>(fsm);
    float2* twD = tw + TWL;
    float* w = fsm + 2 * TWL + 2 * S;    // 2S weights (even orders, then odd)
    float* spr = w + 2 * S;
    float* spi = spr + kWarps * PS;
    load_tw(tw, twD, gtw, gtwD, S);
    for (int q = threadIdx.x; q < 2 * S; q += blockDim.x) w[q] = gw[q];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * kWarps + warp;
    if (row >= nrows) return;
    const int m = row % B;
    if (naive_order(m)) return;
    const float* ws = w + ((m & 1) ? S : 0);
    const float* xr = X + (size_t)row * S;
    const float* xi = xr + (size_t)nrows * S;
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int j = lane + 32 * i;                        // v[j] = x[2j] | x[2(S-1-j)+1]
        const int q = (j < S / 2) ? 2 * j : 2 * (S - 1 - j) + 1;
        v[i] = make_float2(xr[q] * ws[q], xi[q] * ws[q]);
    }
    WarpFFT<R>::run(v, tw, -1.f);
    float* wr = spr + warp * PS;
    float* wi = spi + warp * PS;
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        const int o = pad32(WarpFFT<R>::out_index(k1));
        wr[o] = v[k1].x;
        wi[o] = v[k1].y;
    }
    __syncwarp();
    const float nrm = rsqrtf(2.f * S);
    const float nrm0 = 0.70710678118654752440f * nrm;
    float* cr = Cout + (size_t)row * B;
    float* ci = cr + (size_t)nrows * B;
    for (int k = lane; k < B; k += 32) {
        const int kk = (S - k) & (S - 1);
        const float ar = wr[pad32(k)], ai = wi[pad32(k)], br = wr[pad32(kk)], bi = wi[pad32(kk)];
        const float c = twD[k].x, sn = twD[k].y;
        const float fct = (k == 0) ? nrm0 : nrm;
        cr[k] = ((ar + br) * c + (ai - bi) * sn) * fct;
        ci[k] = ((ai + bi) * c - (ar - br) * sn) * fct;
    }
}

// REDFT01 per (function, seminaive order) row, sin(theta) for odd m, scale: F[p][f][m][theta].
template <int R>
__global__ void __launch_bounds__(256) k_dct_inv_w(const float* __restrict__ Fc, float* __restrict__ F, int nrows,
                                                   const float* __restrict__ gsin, const float2* __restrict__ gtw,
                                                   const float2* __restrict__ gtwD, float scale) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int PS = S + S / 32;
    constexpr int TWL = twtab_len(S);
    extern __shared__ __align__(16) float fsm[];
    float2* tw = reinterpret_cast<float2*>(fsm);
    float2* twD = tw + TWL;
    float* sn = fsm + 2 * TWL + 2 * S;
    float* spr = sn + S;
    float* spi = spr + kWarps * PS;
    load_tw(tw, twD, gtw, gtwD, S);
    for (int q = threadIdx.x; q < S; q += blockDim.x) sn[q] = gsin[q];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * kWarps + warp;
    if (row >= nrows) return;
    const int m = row % B;
    if (naive_order(m)) return;
    const float* xa = Fc + (size_t)row * B;
    const float* xb = xa + (size_t)nrows * B;
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int k = lane + 32 * i;
        const int r = S - k;
        const float ak = (k < B) ? xa[k] : 0.f, bk = (k < B) ? xb[k] : 0.f;
        const float ar = (k > 0 && r < B) ? xa[r] : 0.f, br = (k > 0 && r < B) ? xb[r] : 0.f;
        const float wr = ak + br, wi = bk - ar;
        const float2 d = twD[k];
        v[i] = make_float2(wr * d.x - wi * d.y, wr * d.y + wi * d.x);
    }
    WarpFFT<R>::run(v, tw, 1.f);
    float* zr = spr + warp * PS;
    float* zi = spi + warp * PS;
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        const int o = pad32(WarpFFT<R>::out_index(k1));
        zr[o] = v[k1].x;
        zi[o] = v[k1].y;
    }
    __syncwarp();
    float* fr = F + (size_t)row * S;
    float* fi = fr + (size_t)nrows * S;
    const bool odd = m & 1;
    for (int q = lane; q < S; q += 32) {
        const int src = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
        const float g = odd ? sn[q] * scale : scale;
        fr[q] = zr[pad32(src)] * g;
        fi[q] = zi[pad32(src)] * g;
    }
}

// DFT with sign +1 over the orders for 16 latitudes (two real output rows per warp).
template <int R>
__global__ void __launch_bounds__(256) k_rows_inv_w(const float* __restrict__ F, float* __restrict__ grid, int N,
                                                    const float2* __restrict__ gtw) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int PS = S + S / 32;
    constexpr int TS = kLatPerCta + 1;  // padded tile row (odd)
    constexpr int TWL = twtab_len(S);
    extern __shared__ __align__(16) float fsm[];
    float2* tw = reinterpret_cast<float2*>(fsm);
    float* tr = fsm + 2 * TWL;           // [B][TS]
    float* ti = tr + B * TS;
    float* spr = ti + B * TS;            // [warps][PS]
    float* spi = spr + kWarps * PS;
    const int f = blockIdx.y, th0 = blockIdx.x * kLatPerCta;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    load_tw(tw, nullptr, gtw, nullptr, S);
    const int nlat = min(kLatPerCta, S - th0);
    const size_t plane = (size_t)N * B * S;
    for (int e = threadIdx.x; e < B * kLatPerCta; e += blockDim.x) {
        const int m = e / kLatPerCta, q = e - m * kLatPerCta;
        const size_t o = ((size_t)f * B + m) * S + th0 + q;
        tr[m * TS + q] = (q < nlat) ? F[o] : 0.f;
        ti[m * TS + q] = (q < nlat) ? F[plane + o] : 0.f;
    }
    __syncthreads();
    const int a = 2 * warp, b = a + 1;
    if (th0 + a >= S) return;
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int m = lane + 32 * i;
        float ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
        if (m < B) {
            ar = tr[m * TS + a];
            ai = (m == 0) ? 0.f : ti[m * TS + a];
            br = tr[m * TS + b];
            bi = (m == 0) ? 0.f : ti[m * TS + b];
        } else if (m > B) {
            const int mm = S - m;
            ar = tr[mm * TS + a];
            ai = -ti[mm * TS + a];
            br = tr[mm * TS + b];
            bi = -ti[mm * TS + b];
        }
        v[i] = make_float2(ar - bi, ai + br);  // F_a + i F_b
    }
    WarpFFT<R>::run(v, tw, 1.f);
    float* zr = spr + warp * PS;
    float* zi = spi + warp * PS;
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        const int o = pad32(WarpFFT<R>::out_index(k1));
        zr[o] = v[k1].x;
        zi[o] = v[k1].y;
    }
    __syncwarp();
    float* ga = grid + ((size_t)f * S + th0 + a) * S;
    for (int k = lane; k < S; k += 32) {
        ga[k] = zr[pad32(k)];
        if (th0 + b < S) ga[S + k] = zi[pad32(k)];
    }
}

// Naive inverse orders: the contraction left D0 (even l-m) in F[..][0, B) and D1 (odd l-m)
// in F[..][B, 2B) for the northern latitudes; P(m,l)(-x) = (-1)^(l-m) P(m,l)(x) gives
// F[theta] = D0 + D1 and F[2B-1-theta] = D0 - D1 (times 1/sqrt(2 pi)).
__global__ void k_naive_combine(float* F, int N, int B, float scale) {
    extern __shared__ __align__(16) float fsm[];
    const int S = 2 * B;
    const int nnaive = (B < kNaiveOddBelow ? B : kNaiveOddBelow) / 2;
    const int f = blockIdx.x / nnaive, m = 2 * (blockIdx.x % nnaive) + 1;
    const int part = blockIdx.y;
    float* row = F + (((size_t)part * N + f) * B + m) * S;
    for (int q = threadIdx.x; q < S; q += blockDim.x) fsm[q] = row[q];
    __syncthreads();
    for (int th = threadIdx.x; th < B; th += blockDim.x) {
        const float d0 = fsm[th], d1 = fsm[B + th];
        row[th] = (d0 + d1) * scale;
        row[S - 1 - th] = (d0 - d1) * scale;
    }
}

// ------------------------------------------------------------------------------------
// Tensor-core Legendre contraction, one (order, 64 functions, parity, latitude block) per CTA:
// D[128 x NP] = A[128 x K] * B[NP x K]^T, A = 64 functions x (re, im) rows in three BF16
// terms (exact for FP32), B = the packed table blob, FP32 accumulation in TMEM.
struct Leg {
    const float* C;          // forward seminaive: C[p][f][m][k]
    const float* X;          // forward naive: latitude samples X[p][f][m][theta]
    const float* rc_in;      // inverse: coefficients
    const float* ic_in;
    float* rc;               // forward output coefficients
    float* ic;
    float* Fc;               // inverse seminaive output Fcos[p][f][m][k]
    float* F;                // inverse naive output (D0 | D1) in F[p][f][m][.]
    const uint8_t* blob;
    const int64_t* blob_off;
    int* err;
    int B, N, nprod;
};

__constant__ int c_prod_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_prod_b[6] = {0, 1, 0, 2, 1, 0};

static constexpr int kTPB = 256;
static constexpr uint32_t kATile = 128u * kKC * 2u;  // bytes of one A term tile

static size_t leg_smem(int B, bool fwd) {
    int npmax = 16;
    for (int m = 0; m < B; ++m) npmax = std::max(npmax, geo(fwd, B, m).NP);
    const size_t stage = 3 * (size_t)kATile + 3 * (size_t)npmax * kKC * 2;
    return 1024 + 2 * stage;
}

// 8 consecutive K entries of parity t for row r, segment seg of chunk c, as FP32.
template <bool FWD>
__device__ __forceinline__ void load_seg(const Leg& p, int m, bool nv, int t, int f, int part, int c, int seg,
                                         float* v) {
    const int B = p.B, S = 2 * B;
    if (f >= p.N) {
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = 0.f;
        return;
    }
    if (FWD && nv) {
        // folded latitudes: x[j] +/- x[S-1-j], j = c*KC + seg*8 + q < B
        const int j0 = c * kKC + seg * 8;
        if (j0 >= B) {
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = 0.f;
            return;
        }
        const float* row = p.X + (((size_t)part * p.N + f) * B + m) * S;
        const float4 a0 = reinterpret_cast<const float4*>(row + j0)[0];
        const float4 a1 = reinterpret_cast<const float4*>(row + j0)[1];
        const float4 b0 = reinterpret_cast<const float4*>(row + S - 8 - j0)[0];
        const float4 b1 = reinterpret_cast<const float4*>(row + S - 8 - j0)[1];
        const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float b[8] = {b1.w, b1.z, b1.y, b1.x, b0.w, b0.z, b0.y, b0.x};  // x[S-1-j0-q]
        const float sg = t ? -1.f : 1.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = a[q] + sg * b[q];
        return;
    }
    // 16 consecutive source entries, parity t taken: forward C[k], k = 2j + t; inverse a(l), l-m = 2i + t
    const int kb = 2 * (c * kKC + seg * 8);
    if (FWD) {
        const float* src = p.C + (((size_t)part * p.N + f) * B + m) * B + kb;
        if (kb < B) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 x = reinterpret_cast<const float4*>(src)[q];
                v[2 * q] = t ? x.y : x.x;
                v[2 * q + 1] = t ? x.w : x.z;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = 0.f;
        }
    } else {
        const float* src = (part ? p.ic_in : p.rc_in) + (size_t)f * B * B + index_of_harmonic_coeff(m, m, B);
        const int lim = B - m;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int d = kb + 2 * q + t;
            v[q] = (d < lim) ? src[d] : 0.f;
        }
    }
}

// A operand of one chunk, split into loads (issued early, held in registers across the
// barrier and the MMA issue of the previous chunk) and the BF16 split + shared-memory store.
static constexpr int kTasks = 128 * (kKC / 8) / kTPB;  // (row, 8-column segment) tasks per thread

template <bool FWD>
__device__ __forceinline__ void load_a(const Leg& p, int m, bool nv, int t, int f0, int c, float (&v)[kTasks][8]) {
    constexpr int segs = kKC / 8;
#pragma unroll
    for (int q = 0; q < kTasks; ++q) {
        const int task = threadIdx.x + q * kTPB;
        const int r = task / segs, seg = task - r * segs;
        load_seg<FWD>(p, m, nv, t, f0 + (r & 63), r >> 6, c, seg, v[q]);
    }
}

__device__ __forceinline__ void store_a(uint8_t* st, const float (&v)[kTasks][8]) {
    constexpr int segs = kKC / 8;
#pragma unroll
    for (int q = 0; q < kTasks; ++q) {
        const int task = threadIdx.x + q * kTPB;
        const int r = task / segs, seg = task - r * segs;
        uint32_t w[3][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            __nv_bfloat16 a0, a1, a2, b0, b1, b2;
            tc::split3(v[q][2 * j], a0, a1, a2);
            tc::split3(v[q][2 * j + 1], b0, b1, b2);
            w[0][j] = (uint32_t)__bfloat16_as_ushort(a0) | ((uint32_t)__bfloat16_as_ushort(b0) << 16);
            w[1][j] = (uint32_t)__bfloat16_as_ushort(a1) | ((uint32_t)__bfloat16_as_ushort(b1) << 16);
            w[2][j] = (uint32_t)__bfloat16_as_ushort(a2) | ((uint32_t)__bfloat16_as_ushort(b2) << 16);
        }
        const uint32_t o = tc::tile_off(r, seg * 8, kKC);
#pragma unroll
        for (int s = 0; s < 3; ++s)
            *reinterpret_cast<uint4*>(st + s * kATile + o) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
}

// 16 columns of the leading-product accumulator plus the matching correction columns.
__device__ __forceinline__ void ld_sum(uint32_t taddr, int NP, bool corr, float* v) {
    tc::tmem_ld16(taddr, v);
    if (corr) {
        float u[16];
        tc::tmem_ld16(taddr + NP, u);
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] += u[q];
    }
}

template <bool FWD>
__global__ void __launch_bounds__(kTPB, 1) k_leg_tc(Leg p, uint32_t stage_bytes) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)dsm + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t bars[4];  // [0,1] table bytes landed, [2,3] MMAs of the stage done
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int B = p.B;
    // parity is the fastest grid index: the two CTAs that write the interleaved (stride-2)
    // halves of the same coefficient rows run back to back, so their sectors merge in L2
    const int t = blockIdx.x & 1, nb = blockIdx.x >> 1;
    const int m = blockIdx.y, f0 = blockIdx.z * 64;
    const Geo g = geo(FWD, B, m);
    if (nb >= g.nblk) return;  // uniform per CTA, before any barrier or TMEM use
    const bool nv = naive_order(m);
    const int NP = g.NP, nchunks = g.nch;
    const uint32_t bt = (uint32_t)NP * kKC * 2;
    // two accumulators: columns [0, NP) take the leading product x0*t0, [NP, 2NP) the
    // correction products; each FP32 accumulation step in TMEM truncates relative to the
    // accumulator's own magnitude, so the small terms are not rounded against the large sum
    uint32_t ncols = 32;
    while (ncols < (uint32_t)(2 * NP)) ncols <<= 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint8_t* blob = p.blob + p.blob_off[m] + (size_t)(t * g.nblk + nb) * nchunks * 3 * bt;

    if (threadIdx.x == 0) {
        for (int i = 0; i < 4; ++i) tc::mbar_init(&bars[i], 1);
        tc::fence_mbar_init();
        s_abort = 0;
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16_f32(128, NP);
    constexpr uint32_t sbo = (kKC / 8) * 128;

    // Table chunks: 0 and 1 are issued here; chunk c+1 is issued right after the MMAs of chunk
    // c, as soon as those of chunk c-1 (the previous user of that stage) have retired.
    if (threadIdx.x == 0) {
        for (int c = 0; c < 2 && c < nchunks; ++c) {
            tc::mbar_arrive_expect_tx(&bars[c], 3 * bt);
            tc::bulk_g2s(smem + c * stage_bytes + 3 * kATile, blob + (size_t)c * 3 * bt, 3 * bt, &bars[c]);
        }
    }
    float va[kTasks][8];
    load_a<FWD>(p, m, nv, t, f0, 0, va);
    for (int c = 0; c < nchunks; ++c) {
        const int s = c & 1;
        uint8_t* st = smem + s * stage_bytes;
        // the A part of stage s was last read by the MMAs of chunk c-2; thread 0 waited for them
        // at the end of iteration c-1, before it issued the table copy of chunk c into stage s
        __syncthreads();
        if (s_abort) break;
        store_a(st, va);
        if (c + 1 < nchunks) load_a<FWD>(p, m, nv, t, f0, c + 1, va);  // in flight across the MMA issue
        tc::fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            if (!tc::mbar_wait(&bars[s], (c >> 1) & 1)) {
                s_abort = 1;
            } else {
                tc::tc_fence_after();
                const uint32_t sa = tc::smem_u32(st), sb = tc::smem_u32(st + 3 * kATile);
                for (int ks = 0; ks < kKC / 16; ++ks) {
                    for (int pr = 0; pr < p.nprod; ++pr) {
                        const uint64_t da = tc::sdesc(sa + c_prod_a[pr] * kATile + ks * 256, 128, sbo);
                        const uint64_t db = tc::sdesc(sb + c_prod_b[pr] * bt + ks * 256, 128, sbo);
                        const bool first = (c == 0 && ks == 0 && pr <= 1);  // first write of either accumulator
                        tc::mma_bf16(tmem + (pr ? NP : 0), da, db, idesc, first ? 0u : 1u);
                    }
                }
                tc::mma_commit(&bars[2 + s]);
                // stage s^1 is free once the MMAs of chunk c-1 retire: fetch chunk c+1 into it
                if (c + 1 < nchunks && c >= 1) {
                    if (!tc::mbar_wait(&bars[2 + (s ^ 1)], ((c - 1) >> 1) & 1)) {
                        s_abort = 1;
                    } else {
                        uint8_t* sn = smem + (s ^ 1) * stage_bytes;
                        tc::mbar_arrive_expect_tx(&bars[s ^ 1], 3 * bt);
                        tc::bulk_g2s(sn + 3 * kATile, blob + (size_t)(c + 1) * 3 * bt, 3 * bt, &bars[s ^ 1]);
                    }
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && !s_abort) {
        const int last = nchunks - 1;
        if (!tc::mbar_wait(&bars[2 + (last & 1)], (last >> 1) & 1)) s_abort = 1;
    }
    __syncthreads();
    // Epilogue: TMEM -> registers (warps 0-3, one accumulator row per thread) -> padded smem
    // tile D[r][i] (stage buffers are free once the last commit has arrived) -> all 8 warps
    // write the outputs with consecutive threads on consecutive columns.
    float* dt = reinterpret_cast<float*>(smem);
    const int DS = NP + 1;  // odd row stride
    if (!s_abort && warp < 4) {
        tc::tc_fence_after();
        const int r = warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int cb = 0; cb < NP; cb += 16) {
            float v[16];
            ld_sum(trow + cb, NP, p.nprod > 1, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) dt[r * DS + cb + q] = v[q];
        }
    }
    __syncthreads();
    if (!s_abort) {
        if (FWD) {
            const int base = index_of_harmonic_coeff(m, m, B) + t;
            const int nbase = index_of_harmonic_coeff(-m, m, B) + t;
            const int nv_ = (B - m - t + 1) / 2;  // degrees of this parity
            for (int e = threadIdx.x; e < 128 * nv_; e += kTPB) {
                const int r = e / nv_, i = e - r * nv_;
                const int f = f0 + (r & 63), part = r >> 6;
                if (f >= p.N) continue;
                const float v = dt[r * DS + i];
                float* out = (part ? p.ic : p.rc) + (size_t)f * B * B;
                out[base + 2 * i] = v;
                if (m) out[nbase + 2 * i] = (((m & 1) ? -1.f : 1.f) * (part ? -1.f : 1.f)) * v;
            }
        } else if (!nv) {
            const float sc = (float)(0.5 / sqrt((double)B)), sc0 = (float)(1.0 / sqrt(2.0 * B));
            const int nj = B / 2;
            for (int e = threadIdx.x; e < 128 * nj; e += kTPB) {
                const int r = e / nj, j = e - r * nj;
                const int f = f0 + (r & 63), part = r >> 6;
                if (f >= p.N) continue;
                const int k = 2 * j + t;
                p.Fc[(((size_t)part * p.N + f) * B + m) * B + k] = dt[r * DS + j] * (k == 0 ? sc0 : sc);
            }
        } else {
            for (int e = threadIdx.x; e < 128 * NP; e += kTPB) {
                const int r = e / NP, i = e - r * NP;
                const int f = f0 + (r & 63), part = r >> 6;
                if (f >= p.N) continue;
                p.F[(((size_t)part * p.N + f) * B + m) * (2 * B) + t * B + nb * NP + i] = dt[r * DS + i];
            }
        }
    }
    if (s_abort && threadIdx.x == 0) atomicExch(p.err, S2G_ERR_TIMEOUT);
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, ncols);
    }
}

// ------------------------------------------------------------------------------------
size_t split_work_bytes(int bw, int batch) {
    const size_t B = bw, S = 2 * B;
    return 2 * (size_t)batch * B * (S + B) * sizeof(float) + 1024;
}

static int set_smem(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) S2G_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return S2G_OK;
}

static int check_prec(int precision, int* nprod) {
    if (precision == S2G_PREC_BF16X3) *nprod = 6;
    else if (precision == S2G_PREC_BF16X2) *nprod = 3;
    else return fail(S2G_ERR_ARG, "precision %d is not a split-BF16 mode", precision);
    return S2G_OK;
}

static int launch_leg(bool fwd, Leg& p, cudaStream_t st) {
    const size_t smem = leg_smem(p.B, fwd);
    const uint32_t stage = (uint32_t)((smem - 1024) / 2);
    const void* fn = fwd ? (const void*)k_leg_tc<true> : (const void*)k_leg_tc<false>;
    S2G_TRY(set_smem(fn, smem));
    int nblk = 1;
    for (int m = 0; m < p.B; ++m) nblk = std::max(nblk, geo(fwd, p.B, m).nblk);
    dim3 grid(2 * nblk, p.B, (p.N + 63) / 64);
    if (fwd)
        {
            ProfScope ps_("leg_tc_fwd", st);
            k_leg_tc<true><<<grid, kTPB, smem, st>>>(p, stage);
        }
    else
        {
            ProfScope ps_("leg_tc_inv", st);
            k_leg_tc<false><<<grid, kTPB, smem, st>>>(p, stage);
        }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

// ---- warp-FFT kernel launchers (dispatch on R = S / 32) ----
template <int R>
static int launch_fft_kernels(int which, const void* in, void* out, int N, const Split* s, cudaStream_t st,
                              float scale) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int PS = S + S / 32;
    const int nrows = N * B;
    size_t smem = 0;
    if (which == 0) {  // rows forward
        smem = sizeof(float) * (2 * twtab_len(S) + 2 * kWarps * PS + 2 * kLatPerCta * (B + B / 32 + 1));
        S2G_TRY(set_smem((const void*)k_rows_fwd_w<R>, smem));
        dim3 g((S + kLatPerCta - 1) / kLatPerCta, N);
        ProfScope ps_("rows_fwd_f32", st);
        k_rows_fwd_w<R><<<g, 256, smem, st>>>((const float*)in, (float*)out, N, scale, s->twS);
    } else if (which == 1) {  // DCT-II
        smem = sizeof(float) * (2 * twtab_len(S) + 2 * S + 2 * S + 2 * kWarps * PS);
        S2G_TRY(set_smem((const void*)k_dct_fwd_w<R>, smem));
        ProfScope ps_("dct_fwd_f32", st);
        k_dct_fwd_w<R><<<(nrows + kWarps - 1) / kWarps, 256, smem, st>>>((const float*)in, (float*)out, nrows, s->w32,
                                                                        s->twS, s->twD);
    } else if (which == 2) {  // DCT-III
        smem = sizeof(float) * (2 * twtab_len(S) + 2 * S + S + 2 * kWarps * PS);
        S2G_TRY(set_smem((const void*)k_dct_inv_w<R>, smem));
        ProfScope ps_("dct_inv_f32", st);
        k_dct_inv_w<R><<<(nrows + kWarps - 1) / kWarps, 256, smem, st>>>((const float*)in, (float*)out, nrows,
                                                                        s->sin32, s->twS, s->twD, scale);
    } else {  // rows inverse
        smem = sizeof(float) * (2 * twtab_len(S) + 2 * B * (kLatPerCta + 1) + 2 * kWarps * PS);
        S2G_TRY(set_smem((const void*)k_rows_inv_w<R>, smem));
        dim3 g((S + kLatPerCta - 1) / kLatPerCta, N);
        ProfScope ps_("rows_inv_f32", st);
        k_rows_inv_w<R><<<g, 256, smem, st>>>((const float*)in, (float*)out, N, s->twS);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

static int fft_kernels(int which, int B, const void* in, void* out, int N, const Split* s, cudaStream_t st,
                       float scale) {
    switch (2 * B / 32) {
        case 1: return launch_fft_kernels<1>(which, in, out, N, s, st, scale);
        case 2: return launch_fft_kernels<2>(which, in, out, N, s, st, scale);
        case 4: return launch_fft_kernels<4>(which, in, out, N, s, st, scale);
        case 8: return launch_fft_kernels<8>(which, in, out, N, s, st, scale);
        case 16: return launch_fft_kernels<16>(which, in, out, N, s, st, scale);
        case 32: return launch_fft_kernels<32>(which, in, out, N, s, st, scale);
        default: return fail(S2G_ERR_UNSUPPORTED, "no warp FFT for bandwidth %d", B);
    }
}

int fst_split(Tables* t, const float* grid, float* rc, float* ic, int batch, int precision, void* work,
              cudaStream_t st) {
    int nprod;
    S2G_TRY(check_prec(precision, &nprod));
    S2G_TRY(build_split(t));
    Split* s = (Split*)t->split;
    const int B = t->bw, S = 2 * B;
    float* X = (float*)work;
    float* Cb = X + 2 * (size_t)batch * B * S;
    // 1. DFT along phi (two real latitudes per warp), scaled by sqrt(2 pi)/S   (FST_semi_memo.c:81-90)
    S2G_TRY(fft_kernels(0, B, grid, X, batch, s, st, (float)(sqrt(2.0 * kPi) / S)));
    // 2. weighted DCT-II per (function, seminaive order)                      (seminaive.c:161-176)
    S2G_TRY(fft_kernels(1, B, X, Cb, batch, s, st, 1.f));
    // 3. tensor-core contraction (seminaive orders from C, naive orders from X)
    Leg p{};
    p.C = Cb;
    p.X = X;
    p.rc = rc;
    p.ic = ic;
    p.blob = s->fwd_blob;
    p.blob_off = s->fwd_off;
    p.err = s->err;
    p.B = B;
    p.N = batch;
    p.nprod = nprod;
    return launch_leg(true, p, st);
}

int inv_fst_split(Tables* t, const float* rc, const float* ic, float* grid, int batch, int precision, void* work,
                  cudaStream_t st) {
    int nprod;
    S2G_TRY(check_prec(precision, &nprod));
    S2G_TRY(build_split(t));
    Split* s = (Split*)t->split;
    const int B = t->bw, S = 2 * B;
    float* F = (float*)work;
    float* Fc = F + 2 * (size_t)batch * B * S;
    const float scale = (float)(1.0 / sqrt(2.0 * kPi));
    Leg p{};
    p.rc_in = rc;
    p.ic_in = ic;
    p.Fc = Fc;
    p.F = F;
    p.blob = s->inv_blob;
    p.blob_off = s->inv_off;
    p.err = s->err;
    p.B = B;
    p.N = batch;
    p.nprod = nprod;
    S2G_TRY(launch_leg(false, p, st));
    // REDFT01 (+ sin(theta) for odd m), scaled by 1/sqrt(2 pi)              (seminaive.c:105-114)
    S2G_TRY(fft_kernels(2, B, Fc, F, batch, s, st, scale));
    {
        const int nnaive = std::min(B, kNaiveOddBelow) / 2;
        ProfScope ps_("naive_combine_f32", st);
        k_naive_combine<<<dim3(batch * nnaive, 2), 256, S * sizeof(float), st>>>(F, batch, B, scale);
        S2G_CUDA(cudaGetLastError());
    }
    // DFT with sign +1 over the orders, Hermitian rows                      (FST_semi_memo.c:334-350)
    return fft_kernels(3, B, F, grid, batch, s, st, 1.f);
}

int split_device_status(Tables* t, int clear) {
    Split* s = (Split*)t->split;
    if (!s) return S2G_OK;
    int v = 0;
    S2G_CUDA(cudaMemcpy(&v, s->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (clear && v) S2G_CUDA(cudaMemset(s->err, 0, sizeof(int)));
    if (v) return fail(v, "a bounded wait in the tensor-core kernel expired");
    return S2G_OK;
}

// ------------------------------------------------------------------------------------
// Self-test of the tensor-core machinery: D[128 x N] = A[128 x K] * B[N x K]^T with split-BF16
// products (nprod 1..6), FP32 accumulation.  One CTA; operands written with st.shared.
__global__ void __launch_bounds__(128, 1) k_tc_selftest(int N, int K, int nprod, const float* A, const float* Bm,
                                                      float* D, int* err) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)dsm + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_slot;
    const uint32_t at = 128u * K * 2, bt = (uint32_t)N * K * 2;
    uint32_t ncols = 32;
    while (ncols < (uint32_t)N) ncols <<= 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
    for (int e = threadIdx.x; e < 128 * K; e += blockDim.x) {
        const int r = e / K, k = e - r * K;
        __nv_bfloat16 h[3];
        tc::split3(A[e], h[0], h[1], h[2]);
        for (int s = 0; s < 3; ++s) *(__nv_bfloat16*)(smem + s * at + tc::tile_off(r, k, K)) = h[s];
    }
    for (int e = threadIdx.x; e < N * K; e += blockDim.x) {
        const int r = e / K, k = e - r * K;
        __nv_bfloat16 h[3];
        tc::split3(Bm[e], h[0], h[1], h[2]);
        for (int s = 0; s < 3; ++s) *(__nv_bfloat16*)(smem + 3 * at + s * bt + tc::tile_off(r, k, K)) = h[s];
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_slot;
    bool ok = true;
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc::idesc_bf16_f32(128, N);
        const uint32_t sa = tc::smem_u32(smem), sb = tc::smem_u32(smem + 3 * at);
        const uint32_t sbo = (uint32_t)(K / 8) * 128;
        for (int ks = 0; ks < K / 16; ++ks)
            for (int pr = 0; pr < nprod; ++pr) {
                const uint64_t da = tc::sdesc(sa + c_prod_a[pr] * at + ks * 256, 128, sbo);
                const uint64_t db = tc::sdesc(sb + c_prod_b[pr] * bt + ks * 256, 128, sbo);
                tc::mma_bf16(tmem, da, db, idesc, (ks > 0 || pr > 0) ? 1u : 0u);
            }
        tc::mma_commit(&bar);
        ok = tc::mbar_wait(&bar, 0);
        if (!ok) atomicExch(err, S2G_ERR_TIMEOUT);
    }
    __syncthreads();
    tc::tc_fence_after();
    const int r = warp * 32 + lane;
    for (int cb = 0; cb < N; cb += 16) {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + cb, v);
        for (int q = 0; q < 16; ++q) D[(size_t)r * N + cb + q] = v[q];
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, ncols);
    }
}

}  // namespace s2g

extern "C" int s2g_selftest_tc(int N, int K, int nprod, const float* dA, const float* dB, float* dD) {
    using namespace s2g;
    if (N < 16 || N > 256 || N % 16 || K < 16 || K > 128 || K % 16 || nprod < 1 || nprod > 6 || !dA || !dB || !dD)
        return fail(S2G_ERR_ARG, "selftest: N in [16,256] step 16, K in [16,128] step 16, nprod in [1,6]");
    if (1024 + 3 * (128 * (size_t)K * 2) + 3 * ((size_t)N * K * 2) > 227 * 1024)
        return fail(S2G_ERR_ARG, "selftest: operands exceed shared memory (reduce N or K)");
    int* err = nullptr;
    S2G_CUDA(cudaMalloc(&err, sizeof(int)));
    S2G_CUDA(cudaMemset(err, 0, sizeof(int)));
    const size_t smem = 1024 + 3 * (128 * (size_t)K * 2) + 3 * ((size_t)N * K * 2);
    S2G_TRY(set_smem((const void*)k_tc_selftest, smem));
    {
        ProfScope ps_("tc_selftest", 0);
        k_tc_selftest<<<1, 128, smem>>>(N, K, nprod, dA, dB, dD, err);
    }
    S2G_CUDA(cudaGetLastError());
    int v = 0;
    S2G_CUDA(cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(err);
    if (v) return fail(v, "selftest: bounded wait expired");
    return S2G_OK;
}
