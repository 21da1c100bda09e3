// sht_split.cu -- real-field SHT with FP32 samples/coefficients and the seminaive Legendre
// contraction on the 5th-generation tensor cores as split-BF16 products (FP32 accumulation in TMEM).
//
// Forward (FSTSemiMemo, REAL, cutoff = bw; FST_semi_memo.c:68-145):
//   (the FFT stages below run as chirp-z transforms, czt_split.cu, at lengths 2 bw the warp FFTs
//   do not take; the intermediate layout is then split_layout's padded one)
//   k_rows_fwd_w       : DFT along phi (warp FFT, two real latitudes per warp), X[p][f][m][theta]
//   k_dct_fwd_w        : weights (even/odd order) + REDFT10 + normalisation (seminaive.c:161-176)
//                        -> C[p][f][m][t][j], cosine frequency k = 2j + t (parity-split)
//   k_leg_ws (forward) : per (order m, 64 functions): for each parity t of (l - m), the dense
//                        trapezoid T_{m,t}[i][j] = T(m, l = m+t+2i, k = 2j+t) times C (seminaive.c:183-197)
//                        as D[128 x N] = A[128 x K] * B[N x K]^T on tcgen05, A = 64 functions x
//                        (re, im) rows, B = table rows; epilogue writes f(l, m) and f(l, -m).
// Inverse (InvFSTSemiMemo, REAL; FST_semi_memo.c:228-351):
//   k_leg_ws (inverse) : fcos[2j+t] = sum_i T_{m,t}[i][j] a(m + t + 2i) (seminaive.c:74-98), scaled
//   k_dct_inv_w        : REDFT01, sin(theta) for odd m, 1/sqrt(2 pi); naive orders (odd m < 32):
//                        even/odd latitude halves back to samples
//   k_rows_inv_w       : DFT with sign +1 over m, Hermitian rows, two latitudes per warp
//
// Precision: x = x0 + x1 + x2 with BF16 terms (each the rounded residual of the previous);
// the table is split the same way from FP64.  S2G_PREC_BF16X3 sums the six products
// x_a t_b with a + b <= 2, S2G_PREC_BF16X2 the three with a + b <= 1.
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include <cuda.h>  // CUtensorMap and its encoder's types (the encoder is fetched at run time)
#include <cudaTypedefs.h>

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
    // FP16 two-term blobs (built on first use), table scaled by tab16 = 2^k
    uint8_t* fwd16 = nullptr;
    uint8_t* inv16 = nullptr;
    int64_t* fwd16_off = nullptr;
    int64_t* inv16_off = nullptr;
    double tab16 = 0.0;
    // chirp-z bandwidths (split_czt): chirp, kernel spectrum and length-M twiddles; czM = 0 otherwise
    int czM = 0;
    float2* czh = nullptr;
    float2* czK = nullptr;
    float2* cztw = nullptr;
    // per (direction, tile N extent NB): the work items of one 64-function tile, in order, as
    // (order m, index j within the order) -- item decoding is one load
    std::vector<std::pair<int, int2*>> itab[2];
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
    cudaFree(s->fwd16);
    cudaFree(s->inv16);
    cudaFree(s->fwd16_off);
    cudaFree(s->inv16_off);
    cudaFree(s->czh);
    cudaFree(s->czK);
    cudaFree(s->cztw);
    for (auto& v : s->itab)
        for (auto& e : v) cudaFree(e.second);
    cudaFree(s->err);
    delete s;
    t->split = nullptr;
}

__host__ __device__ __forceinline__ int round16(int x) { return (x + 15) & ~15; }
__host__ __device__ __forceinline__ int nr_par(int B, int m, int t) { return (B - m - t + 1) / 2; }

// Orders computed with the naive transform in the split path (split_naive_order, s2g_internal.h).
static constexpr int kNaiveOddBelow = kSplitNaiveOddBelow;
__host__ __device__ __forceinline__ bool naive_order(int m) { return split_naive_order(m); }

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
    // (B + 1) / 2: the cosine frequencies k = 2j + t < B of parity 0 (at odd B parity 1 has one fewer)
    if (fwd) {
        g.NP = round16(nr0);
        g.KX = nv ? B : (B + 1) / 2;
        g.nblk = 1;
    } else {
        g.KX = nr0;
        // latitude blocks of the naive orders: the MMA's N must be a multiple of 16
        const int nbn = B < kNBN ? round16(B) : kNBN;
        g.NP = nv ? nbn : round16((B + 1) / 2);
        g.nblk = nv ? (B + nbn - 1) / nbn : 1;  // the last block is partial when B is not a multiple of it
    }
    g.nch = (g.KX + kKC - 1) / kKC;
    return g;
}

__host__ __device__ __forceinline__ int64_t blob_bytes(bool fwd, int B, int m, int nterms) {
    const Geo g = geo(fwd, B, m);
    return (int64_t)2 * g.nblk * g.nch * nterms * g.NP * kKC * 2;
}

// ------------------------------------------------------------------------------------
// Operand packing: table operands in the tcgen05 smem layout, one contiguous blob per
// (order, parity, latitude block, K-chunk): [term][NP rows][KC], three BF16 terms or two FP16
// terms of the table scaled by a power of two.
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
    double scale;           // FP16 terms: table scale
    unsigned long long* maxbits;  // kPackMax: largest |entry| as the bits of a double
};

enum { kPackBF16 = 0, kPackMax = 1, kPackF16 = 2 };

template <bool FWD, int MODE>
__global__ void k_pack(Pack p) {
    constexpr int NT = MODE == kPackF16 ? 2 : 3;
    const int B = p.B, S = 2 * B;
    const int m = blockIdx.x, c = blockIdx.y;
    const int t = blockIdx.z & 1, nb = blockIdx.z >> 1;
    const Geo g = geo(FWD, B, m);
    if (c >= g.nch || nb >= g.nblk) return;
    const bool nv = naive_order(m);
    const size_t tile = (size_t)g.NP * kKC * 2;
    uint8_t* out = MODE == kPackMax ? nullptr
                                    : p.blob + p.blob_off[m] + ((size_t)(t * g.nblk + nb) * g.nch + c) * NT * tile;
    const double* tab = p.fwd + p.off[m];
    const double* pml = nv ? p.pml + p.pml_off[m] : nullptr;
    double mx = 0.0;
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
        if (MODE == kPackMax) {
            mx = fmax(mx, fabs(v));
        } else if (MODE == kPackF16) {
            const double x = v * p.scale;
            const __half h0 = __double2half(x);
            const __half h1 = __double2half(x - (double)__half2float(h0));
            *(__half*)(out + tc::tile_off(n, kk, kKC)) = h0;
            *(__half*)(out + tile + tc::tile_off(n, kk, kKC)) = h1;
        } else {
            __nv_bfloat16 h[3];
            split3d(v, h);
            for (int s = 0; s < 3; ++s) *(__nv_bfloat16*)(out + s * tile + tc::tile_off(n, kk, kKC)) = h[s];
        }
    }
    if (MODE == kPackMax && mx > 0.0) atomicMax(p.maxbits, (unsigned long long)__double_as_longlong(mx));
}

__global__ void k_to_f32(const double* a, float* b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

__global__ void k_tw_f32(const double2* a, float2* b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// Packs both directions' table blobs of `t` into s (BF16: three terms; FP16: two terms of the
// table scaled by 2^k, k chosen from the largest entry so that it stays below 2^14).
static int pack_blobs(Tables* t, Split* s, bool f16, cudaStream_t st) {
    const int B = t->bw, S = 2 * B, nt = f16 ? 2 : 3;
    std::vector<int64_t> fo(B), io(B), po(B, 0);
    int64_t fb = 0, ib = 0, pb = 0;
    for (int m = 0; m < B; ++m) {
        fo[m] = fb;
        io[m] = ib;
        fb += blob_bytes(true, B, m, nt);
        ib += blob_bytes(false, B, m, nt);
        if (naive_order(m)) {
            po[m] = pb;
            pb += (int64_t)(B - m) * S;
        }
    }
    uint8_t*& fblob = f16 ? s->fwd16 : s->fwd_blob;
    uint8_t*& iblob = f16 ? s->inv16 : s->inv_blob;
    int64_t*& foff = f16 ? s->fwd16_off : s->fwd_off;
    int64_t*& ioff = f16 ? s->inv16_off : s->inv_off;
    int r = S2G_OK;
    auto ck = [&](cudaError_t e, const char* w) {
        if (e != cudaSuccess && r == S2G_OK) r = cuda_fail(e, w);
    };
    double* pml = nullptr;
    int64_t* d_po = nullptr;
    unsigned long long* d_max = nullptr;
    ck(cudaMalloc(&fblob, fb), "cudaMalloc");
    ck(cudaMalloc(&iblob, ib), "cudaMalloc");
    ck(cudaMalloc(&foff, sizeof(int64_t) * B), "cudaMalloc");
    ck(cudaMalloc(&ioff, sizeof(int64_t) * B), "cudaMalloc");
    ck(cudaMalloc(&pml, sizeof(double) * (size_t)(pb > 0 ? pb : 1)), "cudaMalloc");
    ck(cudaMalloc(&d_po, sizeof(int64_t) * B), "cudaMalloc");
    ck(cudaMalloc(&d_max, sizeof(unsigned long long)), "cudaMalloc");
    if (r == S2G_OK) {
        ck(cudaMemcpyAsync(foff, fo.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st), "copy");
        ck(cudaMemcpyAsync(ioff, io.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st), "copy");
        ck(cudaMemcpyAsync(d_po, po.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st), "copy");
        ck(cudaMemsetAsync(d_max, 0, sizeof(unsigned long long), st), "memset");
    }
    // sampled P(m,l) of the naive orders (pml.c:41-79), one order at a time
    for (int m = 1; r == S2G_OK && m < B && m < kNaiveOddBelow; m += 2) {
        int rr = generate_pml_device(B, m, m + 1, pml, d_po, st);
        if (rr != S2G_OK) r = rr;
    }
    int fch = 0, ich = 0, iblk = 1;
    for (int m = 0; m < B; ++m) {
        fch = std::max(fch, geo(true, B, m).nch);
        ich = std::max(ich, geo(false, B, m).nch);
        iblk = std::max(iblk, geo(false, B, m).nblk);
    }
    const dim3 gf(B, fch, 2), gi(B, ich, 2 * iblk);
    Pack pk{B, t->fwd, t->off, pml, d_po, t->weights, fblob, foff, 1.0, d_max};
    if (r == S2G_OK && f16) {
        // inverse blobs hold the same table entries as the forward ones, plus the naive samples
        {
            ProfScope ps_("pack_max", st);
            k_pack<true, kPackMax><<<gf, 256, 0, st>>>(pk);
        }
        {
            ProfScope ps_("pack_max", st);
            k_pack<false, kPackMax><<<gi, 256, 0, st>>>(pk);
        }
        unsigned long long bits = 0;
        ck(cudaMemcpyAsync(&bits, d_max, sizeof(bits), cudaMemcpyDeviceToHost, st), "copy");
        ck(cudaStreamSynchronize(st), "pack max");
        double mx = 0.0;
        memcpy(&mx, &bits, sizeof(mx));
        int e = 0;
        frexp(mx > 0.0 ? mx : 1.0, &e);  // mx < 2^e
        s->tab16 = ldexp(1.0, 14 - e);
        pk.scale = s->tab16;
    }
    if (r == S2G_OK) {
        {
            ProfScope ps_("pack_fwd", st);
            if (f16) k_pack<true, kPackF16><<<gf, 256, 0, st>>>(pk);
            else k_pack<true, kPackBF16><<<gf, 256, 0, st>>>(pk);
        }
        pk.blob = iblob;
        pk.blob_off = ioff;
        {
            ProfScope ps_("pack_inv", st);
            if (f16) k_pack<false, kPackF16><<<gi, 256, 0, st>>>(pk);
            else k_pack<false, kPackBF16><<<gi, 256, 0, st>>>(pk);
        }
        ck(cudaGetLastError(), "pack kernels");
        ck(cudaStreamSynchronize(st), "pack kernels");
    }
    cudaFree(pml);
    cudaFree(d_po);
    cudaFree(d_max);
    if (!f16) {
        s->fwd_bytes = fb;
        s->inv_bytes = ib;
    }
    return r;
}

// Bandwidths of the split path: powers of two 16 .. 1024 (transform lengths 32 R, R a power of
// two), the multiples of 16 from 48 to 240 (R = 3 .. 15: the warp FFT's direct register DFT), and
// every other bandwidth from 17 to 255 through chirp-z transforms (czt_split.cu).
static bool split_bw_ok(int B) {
    if (B < 16 || B > 1024) return false;
    if ((B & (B - 1)) == 0) return true;
    return (B % 16 == 0 && B / 16 <= 15) || split_czt(B);
}

static int build_split(Tables* t) {
    std::lock_guard<std::mutex> lk(g_split_mu);
    if (t->split) return S2G_OK;
    const int B = t->bw, S = 2 * B;
    if (!split_bw_ok(B))
        return fail(S2G_ERR_UNSUPPORTED,
                    "split-precision path needs a bw in [16, 256] or a power of two up to 1024 (got %d)",
                    B);
    if (t->cutoff != B) return fail(S2G_ERR_UNSUPPORTED, "split-precision path is seminaive at every order (cutoff == bw)");
    // every work item's N extent (table rows) must be a valid tcgen05 N: a multiple of 16, at most 256
    for (int m = 0; m < B; ++m)
        for (int d = 0; d < 2; ++d) {
            const Geo g = geo(d == 0, B, m);
            if (g.NP % 16 || g.NP < 16 || g.KX < 1)
                return fail(S2G_ERR_UNSUPPORTED, "contraction geometry of bw %d, order %d: N extent %d", B, m, g.NP);
        }
    Split* s = new Split();
    s->B = B;
    s->KC = kKC;
    cudaStream_t st;
    S2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int r = S2G_OK;
    auto ck = [&](cudaError_t e, const char* w) {
        if (e != cudaSuccess && r == S2G_OK) r = cuda_fail(e, w);
    };
    ck(cudaMalloc(&s->w32, sizeof(float) * 4 * B), "cudaMalloc");
    ck(cudaMalloc(&s->sin32, sizeof(float) * S), "cudaMalloc");
    ck(cudaMalloc(&s->twS, sizeof(float2) * S), "cudaMalloc");
    ck(cudaMalloc(&s->twD, sizeof(float2) * S), "cudaMalloc");
    ck(cudaMalloc(&s->err, sizeof(int)), "cudaMalloc");
    if (r == S2G_OK) {
        ck(cudaMemsetAsync(s->err, 0, sizeof(int), st), "memset");
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
    if (r == S2G_OK && split_czt(B)) {
        r = czt_build_tables(B, &s->czh, &s->czK, &s->cztw);
        if (r == S2G_OK) s->czM = czt_len(B);
    }
    if (r == S2G_OK) r = pack_blobs(t, s, false, st);
    cudaStreamDestroy(st);
    t->split = s;
    if (r != S2G_OK) free_split(t);
    return r;
}

// FP16 blobs, packed on first use of S2G_PREC_FP16X2 for this table set.
static int build_split16(Tables* t) {
    S2G_TRY(build_split(t));
    std::lock_guard<std::mutex> lk(g_split_mu);
    Split* s = (Split*)t->split;
    if (s->fwd16) return S2G_OK;
    cudaStream_t st;
    S2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int r = pack_blobs(t, s, true, st);
    cudaStreamDestroy(st);
    if (r != S2G_OK) {
        cudaFree(s->fwd16);
        cudaFree(s->inv16);
        cudaFree(s->fwd16_off);
        cudaFree(s->inv16_off);
        s->fwd16 = s->inv16 = nullptr;
        s->fwd16_off = s->inv16_off = nullptr;
    }
    return r;
}

// ------------------------------------------------------------------------------------
// Warp-FFT kernels (fft32.cuh), S = 2B = 32 R.  One warp owns one complex sequence; layout
// changes go through padded shared memory.

// Loads tw[k] = exp(2 pi i k / S) (padded as padtw(k)), its (register, lane) copy
// twb[32 k1 + lane] = tw[(lane k1) mod S] for the warp FFT's stage (b) (see fft32.cuh), and
// twD[k] = (cos, sin)(pi k / 2S) (unpadded, optional) for k < S into shared memory.
__device__ __forceinline__ void load_tw(float2* tw, float2* twb, float2* twD, const float2* gS, const float2* gD,
                                        int S) {
    for (int k = threadIdx.x; k < S; k += blockDim.x) {
        tw[padtw(k)] = gS[k];
        twb[k] = gS[((k & 31) * (k >> 5)) % S];
        if (twD) twD[k] = gD[k];
    }
}

// Tables of the length-2048 transforms (R = 64), which run as two length-1024 four-step FFTs and
// a radix-2 step (WarpFFT2048): tw[padtw(k)] = exp(2 pi i k / 1024), its (register, lane) copy twb,
// and twc[k] = exp(2 pi i k / 2048), k < 1024; gS is the length-2048 table.
__device__ __forceinline__ void load_tw_split(float2* tw, float2* twb, float2* twc, const float2* gS) {
    for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
        tw[padtw(k)] = gS[2 * k];
        twb[k] = gS[2 * (((k & 31) * (k >> 5)) & 1023)];
        twc[k] = gS[k];
    }
}

// CTA shape of the FFT kernels: W warps (one sequence each), LAT = 2W latitudes per CTA in the
// row kernels.  At S = 2048 (R = 64) one such CTA takes 170-195 KB of shared memory (one per SM).
template <int R>
struct FftShape {
    static constexpr int W = 8;
    static constexpr int LAT = 2 * W;
    static constexpr int T = 32 * W;
    // resident CTAs per SM the rows-inverse kernel is compiled for: register budgets of 128
    // (R = 32), 64 (R = 16), 48 (R = 8) and 32 (R <= 4) per thread; lengths that are not powers
    // of two (R = 3 .. 15, the lane-butterfly form with a direct register DFT) 80 above R = 8,
    // 64 above R = 4, 48 below
    static constexpr bool kPow2 = (R & (R - 1)) == 0;
    static constexpr int kMinCtasInv = kPow2 ? (R == 64 ? 1 : R == 32 ? 2 : R == 16 ? 4 : R == 8 ? 5 : 8)
                                             : (R > 8 ? 3 : R > 4 ? 4 : 5);
    // the rows-forward kernel: 48 registers at R = 8 (5 CTAs per SM; unbounded it takes 62 and
    // runs 4% slower); 0 leaves the other lengths unbounded
    static constexpr int kMinCtasFwd = R == 8 ? 5 : 0;
};

// Shared-memory layouts of the FFT kernels put the 16-byte staged buffers first (per-warp
// spectrum buffers padded to PSA floats, a multiple of 4) and the twiddle tables last.
template <int R>
struct FftSmem {
    static constexpr int S = 32 * R, B = S / 2;
    // per-warp spectrum stride: >= pad32(S), a multiple of 4, and 4 mod 32 so that the same
    // element of different warps' spectra falls in different banks
    static constexpr int PSA = (((S + S / 32) + 31) & ~31) + 4;
    static constexpr int RS = B + B / 32 + 1;                    // padded transpose row (odd)
    static constexpr int TILE = (FftShape<R>::LAT * RS + 3) & ~3; // one plane of the row kernels' tile
    // rows-inverse tile, latitude-major [LAT][TS] per plane: TS = B + 2 (2 mod 32 for B >= 32, 18 at
    // B = 16) spreads a warp's float4-component stores (8 orders x 4 latitude groups) over 32 banks,
    // and the per-warp gathers of one latitude over consecutive orders are conflict-free
    static constexpr int TS = B + 2;
    // the inverse DCT kernel's per-warp prefetch rows: two planes of PB floats.  R <= 16 only: at
    // R = 32 the 34 KB they add leave one CTA per SM (+4% there against -7% at R = 16)
    static constexpr bool kDctInvPf = R <= 16;
    static constexpr int PB = B + 16;
    // the four-step warp FFT exchanges through the warp's spectrum rows
    static_assert((R != 8 && R != 16 && R != 32) || R * (32 + 32 / R) <= PSA, "exchange planes fit the spectrum rows");
    // R = 64 (WarpFFT2048): the odd pass exchanges in [OFF, OFF + 32 * 33), the spectrum reaches pad32(2047)
    static_assert(R != 64 || (WarpFFT2048::OFF + 32 * 33 <= PSA && pad32(S - 1) < PSA), "split 2048 buffers fit");
};

// DFT along phi of LAT latitudes (two real rows per warp), transposed to X[p][f][m][theta], m < B.
// Each warp leaves its spectrum in shared memory; the separation of the two packed real rows,
// X_a = (Z[m] + conj Z[S-m]) / 2 and X_b = (Z[m] - conj Z[S-m]) / 2i, is done by the threads
// that write the transposed tile, each a float4 run of 4 latitudes of one order.
// The FFT kernels' bodies: with G the block index vb and block count vgrid come as arguments, so
// that the grouped stage kernels (k_stage_group) run the same code over several bandwidth classes;
// without G they are blockIdx.x and gridDim.x, used where and as (unsigned) the per-length
// kernels always used them, which keeps those kernels' register allocation.
template <bool G>
__device__ __forceinline__ auto vblock(int vb) {
    if constexpr (G) return vb;
    else return blockIdx.x;
}
template <bool G>
__device__ __forceinline__ auto vgridn(int vgrid) {
    if constexpr (G) return vgrid;
    else return gridDim.x;
}

template <int R, bool G>
__device__ __forceinline__ void rows_fwd_body(const float* __restrict__ grid, float* __restrict__ X, int N,
                                              float scale, const float2* __restrict__ gtw,
                                              const int64_t* __restrict__ gmap, int vb, int vgrid) {
    using L = FftSmem<R>;
    constexpr int S = L::S, B = L::B, PSA = L::PSA;
    constexpr int W = FftShape<R>::W, LAT = FftShape<R>::LAT, T = FftShape<R>::T;
    static_assert(S % LAT == 0 && LAT % 4 == 0, "row tiling");
    extern __shared__ __align__(16) float fsm[];
    float* spr = fsm;                  // [W][PSA] re
    float* spi = spr + W * PSA;        // [W][PSA] im
    float2* tw = reinterpret_cast<float2*>(spi + W * PSA);
    float2* twb = tw + (R == 64 ? twtab_len(S / 2) : twtab_len(S));
    float2* twc = twb + S / 2;  // R = 64 only
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if constexpr (R == 64)
        load_tw_split(tw, twb, twc, gtw);
    else
        load_tw(tw, twb, nullptr, gtw, nullptr, S);
    __syncthreads();
    // CTA-strided (function, latitude block) tiles; launched with one tile per CTA
    constexpr int NLB = S / LAT;
    for (int tile = vblock<G>(vb); tile < N * NLB; tile += vgridn<G>(vgrid)) {
    const int f = tile / NLB, th0 = (tile - f * NLB) * LAT;
    const float* ra = grid + (gmap ? gmap[f] : (int64_t)f * S * S) + (size_t)(th0 + 2 * warp) * S;
    float* wr = spr + warp * PSA;
    float* wi = spi + warp * PSA;
    // R = 8, 16, 32: the spectrum as (re, im) pairs, Z[k] (k < B) at wr[2 pad32(k)] and Z[k]
    // (k >= B) at wi[2 pad32(k - B)] (the warp's two plane segments), so that the output phase
    // reads each value with one 8-byte load (-1 to -2%).  Otherwise planes wr/wi[pad32(k)] (at
    // R <= 4 the pairs cost registers and occupancy: +14% at R = 4).
    constexpr bool kPairSpec = R == 8 || R == 16 || R == 32;
    if constexpr (R == 64) {
        WarpFFT2048::to_spectrum([&](int j) { return make_float2(ra[j], ra[S + j]); }, tw, twb, twc, wr, wi, -1.f);
    } else {
        float2 v[R];
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = make_float2(ra[lane + 32 * i], ra[S + lane + 32 * i]);
        WarpFFTSel<R>::run(v, tw, twb, wr, wi, -1.f);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            const int o = WarpFFTSel<R>::out_index(k1);
            if constexpr (kPairSpec) {
                *reinterpret_cast<float2*>((o < B ? wr + 2 * pad32(o) : wi + 2 * pad32(o - B))) = v[k1];
            } else {
                wr[pad32(o)] = v[k1].x;
                wi[pad32(o)] = v[k1].y;
            }
        }
    }
    __syncthreads();
    const size_t plane = (size_t)N * B * S;
    constexpr int Q4 = LAT / 4;
    const float hs = 0.5f * scale;
    for (int e = threadIdx.x; e < B * Q4; e += T) {
        const int m = e / Q4, q = 4 * (e - m * Q4);
        const int pm = pad32(m);
        float re[4], im[4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // latitude pair q/2 + h is warp q/2 + h's (a, b) rows
            const float* zr = spr + (q / 2 + h) * PSA;
            const float* zi = spi + (q / 2 + h) * PSA;
            float ar, ai, br, bi;
            if constexpr (!kPairSpec) {
                const int pmm = pad32((S - m) % S);
                ar = zr[pm], ai = zi[pm], br = zr[pmm], bi = zi[pmm];
            } else {
                // Z[m] (m < B) and Z[S - m] (S - m > B, or Z[0] for m = 0)
                const float2 zm = *reinterpret_cast<const float2*>(zr + 2 * pm);
                const float2 zn = m == 0 ? zm : *reinterpret_cast<const float2*>(zi + 2 * pad32(B - m));
                ar = zm.x, ai = zm.y, br = zn.x, bi = zn.y;
            }
            re[2 * h] = (ar + br) * hs;
            im[2 * h] = (ai - bi) * hs;
            re[2 * h + 1] = (ai + bi) * hs;
            im[2 * h + 1] = (br - ar) * hs;
        }
        const size_t o = ((size_t)f * B + m) * S + th0 + q;
        *reinterpret_cast<float4*>(X + o) = make_float4(re[0], re[1], re[2], re[3]);
        *reinterpret_cast<float4*>(X + plane + o) = make_float4(im[0], im[1], im[2], im[3]);
    }
    __syncthreads();  // every warp's spectrum has been read before the next tile overwrites it
    }
}

template <int R>
__global__ void __launch_bounds__(FftShape<R>::T, FftShape<R>::kMinCtasFwd)
    k_rows_fwd_w(const float* __restrict__ grid, float* __restrict__ X, int N, float scale,
                 const float2* __restrict__ gtw, const int64_t* __restrict__ gmap) {
    rows_fwd_body<R, false>(grid, X, N, scale, gtw, gmap, 0, 0);
}

// Weighted REDFT10 per (function, seminaive order) row, stored by parity of the cosine index:
// C[p][f][m][t][j] holds frequency k = 2j + t (j < B/2), so that the contraction's operand rows
// of one parity are contiguous.  Naive orders are folded in place in X for their contraction:
// X[p][f][m][t][j] = x[j] + (-1)^t x[S-1-j], j < B (the even/odd latitude halves).
// Seminaive rows are read straight into the FFT's registers (4- or 8-byte loads) and leave in
// 16-byte pieces through the warp's spectrum buffer; naive rows go through it both ways.
template <int R, bool G>
__device__ __forceinline__ void dct_fwd_body(float* __restrict__ X, float* __restrict__ Cout, int nrows,
                                             const float* __restrict__ gw, const float2* __restrict__ gtw,
                                             const float2* __restrict__ gtwD, int vb, int vgrid) {
    using L = FftSmem<R>;
    constexpr int S = L::S, B = L::B, PSA = L::PSA;
    constexpr int W = FftShape<R>::W;
    extern __shared__ __align__(16) float fsm[];
    float* spr = fsm;                  // [W][PSA]
    float* spi = spr + W * PSA;        // [W][PSA]
    float* w = spi + W * PSA;          // 2S weights (even orders, then odd)
    float2* twP = reinterpret_cast<float2*>(w + 2 * S);  // B output twiddles, see below
    float2* tw = twP + B;
    float2* twb = tw + (R == 64 ? twtab_len(S / 2) : twtab_len(S));
    float2* twc = twb + S / 2;  // R = 64 only
    if constexpr (R == 64)
        load_tw_split(tw, twb, twc, gtw);
    else
        load_tw(tw, twb, nullptr, gtw, nullptr, S);
    // (cos, sin)(pi k / 2S) of output o (k = 2o, or 2(o - B/2) + 1 for o >= B/2), stored at
    // (o % 4) B/4 + o / 4: the output loop's lanes (4 consecutive o each) read consecutive entries
    for (int o = threadIdx.x; o < B; o += blockDim.x)
        twP[(o & 3) * (B / 4) + (o >> 2)] = gtwD[o < B / 2 ? 2 * o : 2 * (o - B / 2) + 1];
    for (int q = threadIdx.x; q < 2 * S; q += blockDim.x) w[q] = gw[q];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // persistent: the tables are loaded once, then each warp walks rows
    for (int row = vblock<G>(vb) * W + warp; row < nrows; row += vgridn<G>(vgrid) * W) {
    const int m = row % B;
    float* xr = X + (size_t)row * S;
    float* xi = xr + (size_t)nrows * S;
    float* wr = spr + warp * PSA;
    float* wi = spi + warp * PSA;
    if (naive_order(m)) {
        for (int e = lane; e < S / 4; e += 32) {
            reinterpret_cast<float4*>(wr)[e] = reinterpret_cast<const float4*>(xr)[e];
            reinterpret_cast<float4*>(wi)[e] = reinterpret_cast<const float4*>(xi)[e];
        }
        __syncwarp();
        for (int e = lane; e < B / 4; e += 32) {
            float a[4], b[4], c[4], d[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = 4 * e + u;
                const float ar = wr[j], br = wr[S - 1 - j], ai = wi[j], bi = wi[S - 1 - j];
                a[u] = ar + br, b[u] = ar - br, c[u] = ai + bi, d[u] = ai - bi;
            }
            reinterpret_cast<float4*>(xr)[e] = make_float4(a[0], a[1], a[2], a[3]);
            reinterpret_cast<float4*>(xr + B)[e] = make_float4(b[0], b[1], b[2], b[3]);
            reinterpret_cast<float4*>(xi)[e] = make_float4(c[0], c[1], c[2], c[3]);
            reinterpret_cast<float4*>(xi + B)[e] = make_float4(d[0], d[1], d[2], d[3]);
        }
        __syncwarp();  // the staged row is read before the next row overwrites it
        continue;
    }
    const float* ws = w + ((m & 1) ? S : 0);
    auto in = [&](int j) {  // v[j] = x[2j] | x[2(S-1-j)+1]
        const int q = (j < S / 2) ? 2 * j : 2 * (S - 1 - j) + 1;
        return make_float2(xr[q] * ws[q], xi[q] * ws[q]);
    };
    if constexpr (R == 64) {
        WarpFFT2048::to_spectrum(in, tw, twb, twc, wr, wi, -1.f);
    } else {
        float2 v[R];
        if constexpr (R == 8 || R == 32) {
            // input j = L + 32 i < S/2 is sample 2j; sample 2j + 1 is the input S-1-j = (31-L) +
            // 32 (R-1-i) of lane 31 - L.  One 8-byte load per plane feeds both, the odd half
            // crossing lanes by one shuffle.  Measured faster at R = 8 and 32 (-7%, -9%); at
            // R = 16 the 4-byte loads below are (-7%: that kernel then keeps 80 registers, 3 CTAs)
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
                const int q = 2 * (lane + 32 * i);
                const float2 a = *reinterpret_cast<const float2*>(xr + q);
                const float2 b = *reinterpret_cast<const float2*>(xi + q);
                const float2 w2 = *reinterpret_cast<const float2*>(ws + q);
                v[i] = make_float2(a.x * w2.x, b.x * w2.x);
                v[R - 1 - i].x = __shfl_xor_sync(0xffffffffu, a.y * w2.y, 31);
                v[R - 1 - i].y = __shfl_xor_sync(0xffffffffu, b.y * w2.y, 31);
            }
        } else {
#pragma unroll
            for (int i = 0; i < R; ++i) v[i] = in(lane + 32 * i);
        }
        WarpFFTSel<R>::run(v, tw, twb, wr, wi, -1.f);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            const int o = pad32(WarpFFTSel<R>::out_index(k1));
            wr[o] = v[k1].x;
            wi[o] = v[k1].y;
        }
    }
    __syncwarp();
    const float nrm = rsqrtf(2.f * S);
    const float nrm0 = 0.70710678118654752440f * nrm;
    float* cr = Cout + (size_t)row * B;
    float* ci = cr + (size_t)nrows * B;
    // Order 0 of a real field has a real spectrum: its imaginary plane is zero on input, but the
    // packed FFT's Hermitian halves do not cancel exactly in FP32, so store exact zeros (the
    // reference's REDFT10 of the zero imaginary row gives exact zeros, FST_semi_memo.c:96-120).
    const bool im_zero = (m == 0);
    for (int e = lane; e < B / 4; e += 32) {
        float a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int o = 4 * e + u;                         // o = (k & 1) * B/2 + k/2
            const int k = o < B / 2 ? 2 * o : 2 * (o - B / 2) + 1;
            const int kk = (S - k) % S;
            const float ar = wr[pad32(k)], ai = wi[pad32(k)], br = wr[pad32(kk)], bi = wi[pad32(kk)];
            const float2 cs = twP[u * (B / 4) + e];
            const float c = cs.x, sn = cs.y;
            const float fct = (k == 0) ? nrm0 : nrm;
            a[u] = ((ar + br) * c + (ai - bi) * sn) * fct;
            b[u] = im_zero ? 0.f : ((ai + bi) * c - (ar - br) * sn) * fct;
        }
        reinterpret_cast<float4*>(cr)[e] = make_float4(a[0], a[1], a[2], a[3]);
        reinterpret_cast<float4*>(ci)[e] = make_float4(b[0], b[1], b[2], b[3]);
    }
    __syncwarp();  // the spectrum is read before the next row's transform overwrites it
    }
}

template <int R>
__global__ void __launch_bounds__(FftShape<R>::T) k_dct_fwd_w(float* __restrict__ X, float* __restrict__ Cout, int nrows,
                                                   const float* __restrict__ gw, const float2* __restrict__ gtw,
                                                   const float2* __restrict__ gtwD) {
    dct_fwd_body<R, false>(X, Cout, nrows, gw, gtw, gtwD, 0, 0);
}

// REDFT01 per (function, seminaive order) row, sin(theta) for odd m, scale: F[p][f][m][theta].
// Seminaive rows arrive through the warp's cp.async prefetch buffer (R <= 16) or straight from
// global memory, and leave in 16-byte pieces through the warp's spectrum buffer.
template <int R, bool G>
__device__ __forceinline__ void dct_inv_body(const float* __restrict__ Fc, float* __restrict__ F, int nrows,
                                             const float* __restrict__ gsin, const float2* __restrict__ gtw,
                                             const float2* __restrict__ gtwD, float scale, int vb, int vgrid) {
    using L = FftSmem<R>;
    constexpr int S = L::S, B = L::B, PSA = L::PSA;
    constexpr int W = FftShape<R>::W;
    extern __shared__ __align__(16) float fsm[];
    // R <= 16: each warp's next row of Fc is copied into its prefetch buffer while the current
    // row is transformed (the global loads' latency was this kernel's main stall).  Per plane:
    // the t = 0 half at 0, the t = 1 half at B/2 + 16 (PB floats per plane), so that the even and
    // odd lanes' reads fall in different banks.
    constexpr bool kPf = L::kDctInvPf;
    constexpr int PB = L::PB;
    float* spr = fsm;                  // [W][PSA]
    float* spi = spr + W * PSA;        // [W][PSA]
    float* pfb = spi + W * PSA;        // [W][2][PB] (kPf)
    float* sn = pfb + (kPf ? W * 2 * PB : 0);  // S
    float2* twD = reinterpret_cast<float2*>(sn + S);
    float2* tw = twD + S;
    float2* twb = tw + (R == 64 ? twtab_len(S / 2) : twtab_len(S));
    float2* twc = twb + S / 2;  // R = 64 only
    if constexpr (R == 64) {
        load_tw_split(tw, twb, twc, gtw);
        for (int k = threadIdx.x; k < S; k += blockDim.x) twD[k] = gtwD[k];
    } else {
        load_tw(tw, twb, twD, gtw, gtwD, S);
    }
    for (int q = threadIdx.x; q < S; q += blockDim.x) sn[q] = gsin[q];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* zr = spr + warp * PSA;
    float* zi = spi + warp * PSA;
    float* pf = pfb + warp * 2 * PB;
    const int rstride = vgridn<G>(vgrid) * W;
    // asynchronous copy of row r's two planes (B/4 16-byte pieces each) into the warp's buffer;
    // naive-order rows and rows past the end copy nothing.  One commit group per call.
    auto prefetch = [&](int r) {
        if (r < nrows && !naive_order(r % B)) {
            for (int c = lane; c < B / 2; c += 32) {
                const int pl = c >= B / 4, q = 4 * (c - pl * (B / 4));
                tc::cp_async16(pf + pl * PB + q + (q >= B / 2 ? 16 : 0), Fc + (size_t)(pl * nrows + r) * B + q, 16u);
            }
        }
        tc::cp_async_commit();
    };
    if constexpr (kPf) prefetch(vblock<G>(vb) * W + warp);
    // persistent: the tables are loaded once, then each warp walks rows
    for (int row = vblock<G>(vb) * W + warp; row < nrows; row += rstride) {
    const int m = row % B;
    if (naive_order(m)) {
        // the buffer is idle during a naive row: the next row's copy starts now
        if constexpr (kPf) prefetch(row + rstride);
        // Naive orders: the contraction left D0 (even l - m) in F[..][0, B) and D1 (odd l - m) in
        // F[..][B, 2B) for the northern latitudes; P(m,l)(-x) = (-1)^(l-m) P(m,l)(x) gives
        // F[theta] = D0 + D1 and F[2B-1-theta] = D0 - D1 (times 1/sqrt(2 pi)), in place.
        float* fr = F + (size_t)row * S;
        float* fi = fr + (size_t)nrows * S;
        for (int e = lane; e < S / 4; e += 32) {
            reinterpret_cast<float4*>(zr)[e] = reinterpret_cast<const float4*>(fr)[e];
            reinterpret_cast<float4*>(zi)[e] = reinterpret_cast<const float4*>(fi)[e];
        }
        __syncwarp();
        for (int e = lane; e < B / 4; e += 32) {
            float lo[4], hi[4], lo2[4], hi2[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float d0 = zr[4 * e + u], d1 = zr[B + 4 * e + u], c0 = zi[4 * e + u], c1 = zi[B + 4 * e + u];
                lo[u] = (d0 + d1) * scale, hi[u] = (d0 - d1) * scale;
                lo2[u] = (c0 + c1) * scale, hi2[u] = (c0 - c1) * scale;
            }
            reinterpret_cast<float4*>(fr)[e] = make_float4(lo[0], lo[1], lo[2], lo[3]);
            reinterpret_cast<float4*>(fi)[e] = make_float4(lo2[0], lo2[1], lo2[2], lo2[3]);
            // F[S-1-(4e+u)] for u = 3..0 is the aligned run starting at S-4-4e
            reinterpret_cast<float4*>(fr + S - 4 - 4 * e)[0] = make_float4(hi[3], hi[2], hi[1], hi[0]);
            reinterpret_cast<float4*>(fi + S - 4 - 4 * e)[0] = make_float4(hi2[3], hi2[2], hi2[1], hi2[0]);
        }
        __syncwarp();
        continue;
    }
    // Fc[p][f][m][t][j]: cosine coefficient k = 2j + t at (k & 1) * B/2 + k/2 (in the prefetch
    // buffer: (k & 1) * (B/2 + 16) + k/2)
    const float* xa = kPf ? pf : Fc + (size_t)row * B;
    const float* xb = kPf ? pf + PB : Fc + (size_t)(nrows + row) * B;
    constexpr int HO = kPf ? B / 2 + 16 : B / 2;
    auto in = [&](int k) {
        const int r = S - k;
        const int ok = (k & 1) * HO + (k >> 1), orr = (r & 1) * HO + (r >> 1);
        const float ak = (k < B) ? xa[ok] : 0.f, bk = (k < B) ? xb[ok] : 0.f;
        const float ar = (k > 0 && r < B) ? xa[orr] : 0.f, br = (k > 0 && r < B) ? xb[orr] : 0.f;
        const float wr = ak + br, wi = bk - ar;
        const float2 d = twD[k];
        return make_float2(wr * d.x - wi * d.y, wr * d.y + wi * d.x);
    };
    if constexpr (R == 64) {
        WarpFFT2048::to_spectrum(in, tw, twb, twc, zr, zi, 1.f);
    } else {
        float2 v[R];
        if constexpr (kPf) {
            tc::cp_async_wait(0);  // this lane's copies of the row have landed
            __syncwarp();          // and every lane's
        }
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = in(lane + 32 * i);
        if constexpr (kPf) {
            __syncwarp();  // the buffer is read: the next row's copy may overwrite it
            prefetch(row + rstride);
        }
        WarpFFTSel<R>::run(v, tw, twb, zr, zi, 1.f);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            const int o = pad32(WarpFFTSel<R>::out_index(k1));
            zr[o] = v[k1].x;
            zi[o] = v[k1].y;
        }
    }
    __syncwarp();
    float* fr = F + (size_t)row * S;
    float* fi = fr + (size_t)nrows * S;
    const bool odd = m & 1;
    for (int e = lane; e < S / 4; e += 32) {
        float a[4], b[4];
        const float4 s4 = reinterpret_cast<const float4*>(sn)[e];
        const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = 4 * e + u;
            const int src = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
            const float g = odd ? sv[u] * scale : scale;
            a[u] = zr[pad32(src)] * g;
            b[u] = zi[pad32(src)] * g;
        }
        reinterpret_cast<float4*>(fr)[e] = make_float4(a[0], a[1], a[2], a[3]);
        reinterpret_cast<float4*>(fi)[e] = make_float4(b[0], b[1], b[2], b[3]);
    }
    __syncwarp();  // the spectrum is read before the next row's transform overwrites it
    }
}

// DFT with sign +1 over the orders for LAT latitudes (two real output rows per warp).  The
// order-major input arrives as float4 runs of 4 latitudes; output rows leave as 128-byte lines
// from registers (R = 8, 16, 32) or as float4 through the warp's spectrum buffer.
template <int R, bool G>
__device__ __forceinline__ void rows_inv_body(const float* __restrict__ F, float* __restrict__ grid, int N,
                                              const float2* __restrict__ gtw, const int64_t* __restrict__ gmap,
                                              int vb, int vgrid) {
#include "rows_inv_body.inc"
}

template <int R>
__global__ void __launch_bounds__(FftShape<R>::T, FftShape<R>::kMinCtasInv)
    k_rows_inv_w(const float* __restrict__ F, float* __restrict__ grid, int N, const float2* __restrict__ gtw,
                 const int64_t* __restrict__ gmap) {
    constexpr bool G = false;
    constexpr int vb = 0, vgrid = 0;
#include "rows_inv_body.inc"
}

template <int R>
__global__ void __launch_bounds__(FftShape<R>::T) k_dct_inv_w(const float* __restrict__ Fc, float* __restrict__ F, int nrows,
                                                   const float* __restrict__ gsin, const float2* __restrict__ gtw,
                                                   const float2* __restrict__ gtwD, float scale) {
    dct_inv_body<R, false>(Fc, F, nrows, gsin, gtw, gtwD, scale, 0, 0);
}

// Dynamic shared memory of FFT kernel `which` (0 rows forward, 1 DCT-II, 2 DCT-III, 3 rows inverse)
// at length S = 32 R.
template <int R>
static size_t fft_smem(int which) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int kWarps = FftShape<R>::W, kLatPerCta = FftShape<R>::LAT;
    using L = FftSmem<R>;
    const size_t tw_bytes = sizeof(float2) * (twtab_len(S) + S), spec = sizeof(float) * 2 * kWarps * L::PSA;
    switch (which) {
        case 0: return spec + tw_bytes;
        case 1: return spec + sizeof(float) * 2 * S + sizeof(float2) * B + tw_bytes;
        case 2:
            return spec + (L::kDctInvPf ? sizeof(float) * kWarps * 2 * L::PB : 0) + sizeof(float) * S +
                   sizeof(float2) * S + tw_bytes;
        default: return std::max(sizeof(float) * 2 * kLatPerCta * L::TS, spec) + tw_bytes;
    }
}

// ---- grouped stage kernels: one launch runs one FFT stage of several bandwidth classes ----
// Blocks [blk0, blk0 + nblk) belong to class c; each class runs the body of its own length with
// block index blockIdx.x - blk0 among nblk.  The row kernels take one (function, latitude block)
// tile per block; the DCT kernels stride their blocks over the class's rows, so a class's block
// count sets how many rows share one load of its twiddle tables.
static constexpr int kStageMaxClasses = 6;

struct StageCls {
    int R, blk0, nblk, N;
    const void* in;
    void* out;
    const int64_t* gmap;   // rows kernels: per-function grid offsets (null: f * S * S)
    const float* w32;      // DCT-II: weights
    const float* sin32;    // DCT-III: sin(theta)
    const float2* twS;
    const float2* twD;
    float scale;
};

struct StageArgs {
    int ncls;
    StageCls c[kStageMaxClasses];
};

template <int WHICH, int R>
__device__ __forceinline__ void stage_body(const StageCls& k, int vb) {
    const int B = 16 * R;
    if constexpr (WHICH == 0)
        rows_fwd_body<R, true>((const float*)k.in, (float*)k.out, k.N, k.scale, k.twS, k.gmap, vb, k.nblk);
    else if constexpr (WHICH == 1)
        dct_fwd_body<R, true>((float*)k.in, (float*)k.out, k.N * B, k.w32, k.twS, k.twD, vb, k.nblk);
    else if constexpr (WHICH == 2)
        dct_inv_body<R, true>((const float*)k.in, (float*)k.out, k.N * B, k.sin32, k.twS, k.twD, k.scale, vb, k.nblk);
    else
        rows_inv_body<R, true>((const float*)k.in, (float*)k.out, k.N, k.twS, k.gmap, vb, k.nblk);
}

// Resident CTAs per SM a grouped stage kernel is compiled for.  RMAX is the longest transform
// (32 RMAX points) it carries, and only lengths up to RMAX are compiled in, so the short tier
// (RMAX 4: bw <= 64) keeps the per-length kernels' small register budgets; the long tiers take
// three CTAs (RMAX 16, bw <= 256; at four the row stages spill, the dispatch over lengths costing
// registers the per-length kernels do not spend) and two (RMAX 32, bw 512).
template <int WHICH, int RMAX>
struct StageOcc {
    static constexpr int v = RMAX <= 4 ? ((WHICH == 1 || WHICH == 2) ? 5 : 8) : RMAX <= 16 ? 3 : 2;
};

template <int WHICH, int RMAX>
__global__ void __launch_bounds__(256, StageOcc<WHICH, RMAX>::v) k_stage_group(const __grid_constant__ StageArgs a) {
    int ci = 0;
    while (ci + 1 < a.ncls && (int)blockIdx.x >= a.c[ci + 1].blk0) ++ci;
    const StageCls& k = a.c[ci];
    const int vb = (int)blockIdx.x - k.blk0;
    switch (k.R) {
        case 1: stage_body<WHICH, 1>(k, vb); break;
        case 2: stage_body<WHICH, 2>(k, vb); break;
        case 4: stage_body<WHICH, 4>(k, vb); break;
        case 8:
            if constexpr (RMAX >= 8) stage_body<WHICH, 8>(k, vb);
            break;
        case 16:
            if constexpr (RMAX >= 16) stage_body<WHICH, 16>(k, vb);
            break;
        default:
            if constexpr (RMAX >= 32) stage_body<WHICH, 32>(k, vb);
            break;
    }
}

// ------------------------------------------------------------------------------------
// Tensor-core Legendre contraction.  A persistent kernel: each CTA takes work items from a
// counter; an item is (bandwidth class, 64 functions, order m, latitude block nb, table-row
// sub-block, parity t of l-m) and computes D[128 x NB] = A[128 x K] * B[NB x K]^T, A = 64
// functions x (re, im) rows in split terms, B = rows [n0, n0 + NB) of the packed table blob,
// FP32 accumulation in TMEM.  NB (the N extent of the tile) is chosen per class at launch.
// Barriers and TMEM are set up once per CTA; the stage and phase of every chunk follow a
// running per-CTA chunk count, so consecutive items keep the two-stage pipeline.
//
// FP16 terms (S2G_PREC_FP16X2): each A row is scaled by a power of two 2^e_r chosen from the
// row's largest magnitude (|x| 2^e_r < 2^14) and the table blob by one power of two per
// bandwidth, so that FP16's exponent range holds both; the epilogue undoes both scales.
static constexpr int kMaxClasses = 16;  // bandwidth classes of one contraction launch

struct LegClass {
    int B, N, ntiles;         // bandwidth, functions, 64-function tiles
    int BH, BN, SX;           // intermediate layout (SplitLayout): C/Fc half rows, folded halves, X/F rows
    int NB;                   // table rows per work item (N extent of the tile)
    int per_tile;             // work items per 64-function tile
    const int2* itab;         // per_tile entries: (order m, index of the item within the order)
    int64_t item0;            // first work item of the class
    float tab_inv;            // inverse of the table blob's scale
    const float* C;           // forward seminaive input C[p][f][m][t][j] (k = 2j + t), rows of 2 BH
    const float* X;           // forward naive input, folded halves X[p][f][m][t][j], j < B, rows of SX
    const float* rc_in;       // inverse input coefficients
    const float* ic_in;
    float* rc;                // forward output coefficients
    float* ic;
    float* Fc;                // inverse seminaive output Fcos[p][f][m][t][j] (k = 2j + t)
    float* F;                 // inverse naive output (D0 | D1) in F[p][f][m][.]
    const int64_t* cmap;      // function -> element offset of its coefficients (null: f * B * B)
    const uint8_t* blob;
    const int64_t* blob_off;
};

// Tensor-map TMA path (one bandwidth class, BF16 terms, no coefficient map, bw a multiple of 64): the A
// operand of every chunk is one or two tiled TMA loads into a staging ring, and the inverse's
// seminaive output leaves through tiled TMA stores.  Boxes (innermost first):
//   forward seminaive: C      [p][f][m][t*B/2 + j]  box {32, 1, 64, 2}, 128-byte swizzle
//   forward naive    : X      [p][f][m][t*B + j]    box {32, 1, 64, 2}, 128-byte swizzle
//   inverse          : rc, ic [f][bw*bw]            box {kInvBox, 64} from the 16-byte aligned
//                      element below the chunk's first coefficient (no swizzle)
//   inverse output   : Fc     [p][f][m][t*B/2 + j]  box {32, 1, 64, 2}, 128-byte swizzle
static constexpr int kInvBox = 68;     // 64 coefficients (both parities of 32 degrees) + 4 of alignment slack

struct Leg {
    LegClass cls[kMaxClasses];
    int ncls;
    int nprod;
    long long nitems;
    int* counter;             // work counter, zero at launch
    int* err;
    int tma;                  // 1: tensor-map TMA path (below)
    uint32_t a_chunk_bytes;   // TMA bytes of one A chunk
    int pair;                 // forward: items come in parity pairs; the odd item writes both (see k_leg_ws)
    int stall;                // test hook: the scheduler publishes no work (every other wait runs out)
    uint32_t stash_off;       // forward pairs: shared-memory offset of the even parity's results (group 0)
    uint32_t epi_stride;      // bytes between the two epilogue groups' staging (and stash) areas
    int stash_stride;         // ... and their row stride in floats (odd)
    CUtensorMap tmA0, tmA1;   // forward: C, folded X; inverse: rc, ic
    CUtensorMap tmO;          // inverse: Fc
};

__constant__ int c_prod_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_prod_b[6] = {0, 1, 0, 2, 1, 0};

static constexpr int kTPB = 256;  // A-producer threads: two (row, 8-column segment) tasks each
static constexpr uint32_t kATile = 128u * kKC * 2u;  // bytes of one A term tile
static constexpr uint32_t kSBO = (kKC / 8) * 128;    // byte stride of 8-row groups in a tile

static int leg_npmax(int B, bool fwd) {
    int npmax = 16;
    for (int m = 0; m < B; ++m) npmax = std::max(npmax, geo(fwd, B, m).NP);
    return npmax;
}

__device__ __forceinline__ int64_t coef_base(const LegClass& k, int f) {
    return k.cmap ? k.cmap[f] : (int64_t)f * k.B * k.B;
}

// 8 consecutive K entries of parity t for row r, segment seg of chunk c, as FP32.
//   forward seminaive: C[p][f][m][t][j], j < B/2 (parity-split DCT output)
//   forward naive    : X[p][f][m][t][j], j < B (latitude halves folded by the DCT kernel)
//   inverse          : a(l), l - m = 2i + t, from the coefficient arrays (stride 2)
template <bool FWD>
__device__ __forceinline__ const float* fwd_row(const LegClass& k, int m, bool nv, int t, int f, int part) {
    const size_t row = ((size_t)part * k.N + f) * k.B + m;
    return nv ? k.X + row * k.SX + t * k.BN : k.C + row * (2 * k.BH) + t * k.BH;
}

template <bool FWD>
__device__ __forceinline__ void load_seg(const LegClass& k, int m, bool nv, int t, int f, int part, int c, int seg,
                                         float* v) {
    const int B = k.B;
    if (f >= k.N) {
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = 0.f;
        return;
    }
    const int j0 = c * kKC + seg * 8;
    if (FWD) {
        if (j0 >= (nv ? k.BN : k.BH)) {
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = 0.f;
            return;
        }
        const float4* src = reinterpret_cast<const float4*>(fwd_row<FWD>(k, m, nv, t, f, part) + j0);
        const float4 a = src[0], b = src[1];
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
        const float* src = (part ? k.ic_in : k.rc_in) + coef_base(k, f) + index_of_harmonic_coeff(m, m, B);
        const int lim = B - m;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int d = 2 * (j0 + q) + t;
            v[q] = (d < lim) ? src[d] : 0.f;
        }
    }
}

// Task q of producer thread tid: A-tile row r (function f0 + r % 64, plane r / 64) and 8-column
// segment seg of the chunk.  Eight consecutive lanes take the eight rows of one core matrix (one
// contiguous 128-byte block of the tile), so each quarter-warp's 16-byte shared-memory stores hit
// 32 distinct banks; the four tasks of a row (seg 0..3) are lanes l, l + 8, l + 16, l + 24.
__device__ __forceinline__ void task_rs(int tid, int q, int& r, int& seg) {
    const int lane = tid & 31;
    seg = lane >> 3;
    r = q * 64 + (tid >> 5) * 8 + (lane & 7);
}

// A operand of one chunk, split into loads (issued early, held in registers across the
// barrier and the MMA issue of the previous chunk) and the split + shared-memory store.
static constexpr int kTasks = 128 * (kKC / 8) / kTPB;  // (row, 8-column segment) tasks per thread

template <bool FWD>
__device__ __forceinline__ void load_a(const LegClass& k, int m, bool nv, int t, int f0, int c,
                                       float (&v)[kTasks][8], int tid) {
#pragma unroll
    for (int q = 0; q < kTasks; ++q) {
        int r, seg;
        task_rs(tid, q, r, seg);
        load_seg<FWD>(k, m, nv, t, f0 + (r & 63), r >> 6, c, seg, v[q]);
    }
}

// FP32 -> 16-bit terms: three BF16 (each the rounded residual of the previous; exact for FP32
// data) or two FP16.
template <bool F16>
__device__ __forceinline__ void split_terms(float x, uint16_t& h0, uint16_t& h1, uint16_t& h2) {
    if (F16) {
        const __half a = __float2half_rn(x);
        const __half b = __float2half_rn(x - __half2float(a));
        h0 = __half_as_ushort(a);
        h1 = __half_as_ushort(b);
        h2 = 0;
    } else {
        __nv_bfloat16 a, b, c;
        tc::split3(x, a, b, c);
        h0 = __bfloat16_as_ushort(a);
        h1 = __bfloat16_as_ushort(b);
        h2 = __bfloat16_as_ushort(c);
    }
}

template <bool F16>
__device__ __forceinline__ void store_a(uint8_t* st, const float (&v)[kTasks][8], const float (&sc)[kTasks],
                                        int tid) {
#pragma unroll
    for (int q = 0; q < kTasks; ++q) {
        int r, seg;
        task_rs(tid, q, r, seg);
        uint32_t w[3][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            uint16_t a0, a1, a2, b0, b1, b2;
            split_terms<F16>(v[q][2 * j] * sc[q], a0, a1, a2);
            split_terms<F16>(v[q][2 * j + 1] * sc[q], b0, b1, b2);
            w[0][j] = (uint32_t)a0 | ((uint32_t)b0 << 16);
            w[1][j] = (uint32_t)a1 | ((uint32_t)b1 << 16);
            w[2][j] = (uint32_t)a2 | ((uint32_t)b2 << 16);
        }
        const uint32_t o = tc::tile_off(r, seg * 8, kKC);
#pragma unroll
        for (int s = 0; s < (F16 ? 2 : 3); ++s)
            *reinterpret_cast<uint4*>(st + s * kATile + o) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
}

// 16 columns of the leading-product accumulator plus the matching correction columns.
__device__ __forceinline__ void ld_sum(uint32_t taddr, uint32_t corr_off, bool corr, float* v) {
    if (corr) {
        float u[16];
        tc::tmem_ld16x2(taddr, taddr + corr_off, v, u);
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] += u[q];
    } else {
        tc::tmem_ld16(taddr, v);
    }
}

// Epilogue stores of one staged block: rows r (function f0 + r % 64, part r / 64) of the
// staging tile `ep` (row stride ES floats), columns [0, w) of table-row block c0 = n0 + cb0.
// Warps take rows, lanes take consecutive columns (coalesced; no per-element division).
template <bool FWD>
__device__ __forceinline__ void epi_store(const LegClass& K, int m, int t, int nb, int NP, int f0, int c0, int w,
                                          const float* ep, int ES, int wid, int nw, int lane) {
    const int B = K.B;
    if (FWD) {
        const int base = index_of_harmonic_coeff(m, m, B) + t + 2 * c0;
        const int nbase = index_of_harmonic_coeff(-m, m, B) + t + 2 * c0;
        const int nv_ = min(w, nr_par(B, m, t) - c0);
        const float sgn = (m & 1) ? -1.f : 1.f;
        // Rows in groups of RU per warp: all of a group's shared-memory loads are issued before
        // its global stores.  The staging tile is reached through a generic pointer, so a load
        // placed after a global store waits for that store's address to be resolved; loads that
        // go first overlap their latencies.  Two values per lane cover a row (w <= 64).
        constexpr int RU = 4;
        for (int r0 = wid; r0 < 128; r0 += RU * nw) {
            float v[RU][2];
#pragma unroll
            for (int u = 0; u < RU; ++u) {
                const int r = r0 + u * nw;
                const float* src = ep + (r < 128 ? r : 0) * ES;
                v[u][0] = lane < nv_ ? src[lane] : 0.f;
                v[u][1] = lane + 32 < nv_ ? src[lane + 32] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < RU; ++u) {
                const int r = r0 + u * nw;
                const int f = f0 + (r & 63), part = r >> 6;
                if (r >= 128 || f >= K.N) continue;
                float* out = (part ? K.ic : K.rc) + coef_base(K, f);
                const float s2 = part ? -sgn : sgn;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int i = lane + 32 * h;
                    if (i < nv_) {
                        out[base + 2 * i] = v[u][h];
                        if (m) out[nbase + 2 * i] = s2 * v[u][h];
                    }
                }
            }
        }
    } else {
        // inverse: Fcos of a seminaive order (scaled), or a naive order's latitude block; rows in
        // groups of RU as in the forward
        const bool nv = naive_order(m);
        const float sc_ = (float)(0.5 / sqrt((double)B)), sc0 = (float)(1.0 / sqrt(2.0 * B));
        const int nj = nv ? min(w, B - nb * NP - c0)  // latitudes of a partial last block end at B
                          : min(w, (B + 1) / 2 - c0);
        constexpr int RU = 4;
        for (int r0 = wid; r0 < 128; r0 += RU * nw) {
            float v[RU][2];
#pragma unroll
            for (int u = 0; u < RU; ++u) {
                const int r = r0 + u * nw;
                const float* src = ep + (r < 128 ? r : 0) * ES;
                v[u][0] = lane < nj ? src[lane] : 0.f;
                v[u][1] = lane + 32 < nj ? src[lane + 32] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < RU; ++u) {
                const int r = r0 + u * nw;
                const int f = f0 + (r & 63), part = r >> 6;
                if (r >= 128 || f >= K.N) continue;
                const size_t row = ((size_t)part * K.N + f) * B + m;
                float* dst = nv ? K.F + row * K.SX + t * K.BN + nb * NP + c0 : K.Fc + row * (2 * K.BH) + t * K.BH + c0;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int j = lane + 32 * h;
                    if (j < nj) dst[j] = nv ? v[u][h] : v[u][h] * ((c0 + j + t) == 0 ? sc0 : sc_);
                }
            }
        }
    }
}

// Forward stores of one interleaved block of a parity pair: row r of `ep` (stride ES) holds the
// coefficients l = m + 2 i0 + u, u < 32 (both parities), of function f0 + r % 64, part r / 64;
// a warp writes a row's run as one contiguous store (and its mirror at order -m).
__device__ __forceinline__ void epi_store_pair(const LegClass& K, int m, int f0, int i0, const float* ep, int ES,
                                               int wid, int nw, int lane) {
    const int B = K.B;
    const int nl = min(32, B - m - 2 * i0);
    if (lane >= nl) return;
    const int base = index_of_harmonic_coeff(m, m, B) + 2 * i0 + lane;
    const int nbase = index_of_harmonic_coeff(-m, m, B) + 2 * i0 + lane;
    const float sgn = (m & 1) ? -1.f : 1.f;
    constexpr int RU = 4;  // rows per group: the group's shared-memory loads go before its stores (see epi_store)
    for (int r0 = wid; r0 < 128; r0 += RU * nw) {
        float v[RU];
#pragma unroll
        for (int u = 0; u < RU; ++u) {
            const int r = r0 + u * nw;
            v[u] = ep[(r < 128 ? r : 0) * ES + lane];
        }
#pragma unroll
        for (int u = 0; u < RU; ++u) {
            const int r = r0 + u * nw;
            const int f = f0 + (r & 63), part = r >> 6;
            if (r >= 128 || f >= K.N) continue;
            float* out = (part ? K.ic : K.rc) + coef_base(K, f);
            out[base] = v[u];
            if (m) out[nbase] = (part ? -sgn : sgn) * v[u];
        }
    }
}

// Bulk copies of table rows [n0, n0 + rows) of chunk c, all terms, into stage buffer sb.
template <bool F16>
__device__ __forceinline__ void issue_table(uint8_t* sb, const uint8_t* blob, int NP, int n0, int rows, int c,
                                            uint64_t* bar) {
    constexpr int NT = F16 ? 2 : 3;
    const uint32_t tile = (uint32_t)NP * kKC * 2, part = (uint32_t)rows * kKC * 2;
    const uint8_t* src = blob + (size_t)c * NT * tile + (size_t)(n0 / 8) * kSBO;
    tc::mbar_arrive_expect_tx(bar, NT * part);
#pragma unroll
    for (int s = 0; s < NT; ++s) tc::bulk_g2s(sb + s * part, src + (size_t)s * tile, part, bar);
}

// ------------------------------------------------------------------------------------
// Warp-specialised contraction: the stages of consecutive work items overlapped.  16 warps, one
// CTA per SM:
//   warp 0     : scheduler (fetches and decodes items into a kNI-entry ring in shared memory)
//                and table producer (bulk copies into an nbs-stage ring);
//   warp 1     : MMA issuer (one thread; two accumulator pairs in TMEM when they fit, so the
//                epilogue of item k overlaps the MMAs of item k+1);
//   warps 4-7 and 16-19: two epilogue groups taking alternate work items (alternate parity pairs
//                in pair mode); warp 4+q (16+q) reads TMEM lanes 32q..32q+31 = accumulator rows,
//                stages column blocks in its group's shared memory, writes them coalesced.  One
//                group was the busiest role of the kernel (82-91% busy against 40-58% for the MMA
//                thread and the A producers, measured with per-role clock counters);
//   warps 8-15 : A producers (FP32 loads one chunk ahead, split, store into a kNAS-stage ring);
//   warp 2     : on the tensor-map path, A loader: one TMA per chunk into the FP32 staging ring,
//                paced by that ring alone, so the A operand (from HBM) runs up to nstg chunks
//                ahead of the MMAs while the table (from L2) keeps its own nbs-stage ring;
//   warp 3     : no role.
// Every mbarrier wait is bounded; on expiry the role records the abort and leaves its loop,
// the table producer waits (bounded) for its copies in flight, the MMA thread for its MMAs,
// and the CTA frees TMEM and returns.
static constexpr int kWsThreads = 640;
static constexpr int kNI = 8;          // item ring entries (8 against 4: bw 64 x 4096 forward -6%, inverse -3%)
static constexpr int kNAS = 2;         // A stages
static constexpr int kMaxNBS = 8;      // table stages (upper bound)
static constexpr int kEpiCols = 64;    // epilogue staging width
static_assert(kEpiCols <= 64, "epi_store holds two staged values per lane and row");
static constexpr int kMaxStg = 8;      // FP32 staging stages of the BF16 A producers (upper bound)
static constexpr int kAProd = 256;     // A-producer threads
static constexpr int kEpi = 128;       // epilogue threads
static constexpr uint32_t kStgBytes = kAProd * kTasks * 8 * sizeof(float);  // one staging stage (16 KB)

struct WsItem {
    int ci, m, t, sub, nb, f0;
};

// The TMEM accumulator pair of item k and how many items used that pair before it.  A pair's
// mbarriers are waited on by parity, so every use of one pair must go to the same epilogue group
// (a group waiting for use u while use u-1 is still open would see use u-2's parity and pass):
// with two pairs and two groups, group g owns pair g; in forward pair mode a parity pair (k, k+1)
// shares one accumulator pair, since the even item frees it at once after stashing its results.
// With one pair (wide blocks) there is one epilogue group.
struct AccUse {
    int buf, use;
};
__device__ __forceinline__ AccUse acc_use(int k, int nacc, bool pair) {
    if (nacc == 1) return {0, k};
    if (pair) return {(k >> 1) & 1, ((k >> 2) << 1) | (k & 1)};
    return {k & 1, k >> 1};
}

// The K chunks an item multiplies, [c0, c1), and per chunk the N rows [r0, r0 + n) its MMAs cover.
// The seminaive table of order m is zero where the cosine frequency index j exceeds m/2 + i, i the
// degree index (tz above; seminaive.c:183-197 stops each degree's sum at its last frequency): the
// forward's row i (N = degrees) has non-zero entries only in chunks up to (m/2 + i) / 32, the
// inverse's row j (N = frequencies) only from chunk (j - m/2) / 32 on.  Chunks no row of the item
// reaches are skipped (no A or table load, no MMA), and within a chunk the MMAs leave out the
// 16-row blocks that are zero there.  The first chunk of an item covers every row, since it
// starts the accumulators; skipped products are exact zeros, so the sums do not change.  Naive
// orders are dense.
struct Span {
    int c0, c1;
};

__device__ __forceinline__ Span item_span(bool fwd, int nch, int m, int n0, int rows) {
    if (naive_order(m)) return Span{0, nch};
    const int h = m / 2;
    if (fwd) return Span{0, min(nch, (h + n0 + rows - 1) / kKC + 1)};
    const int lo = n0 - h - (kKC - 1);  // the first chunk c with h + 32 c + 31 >= n0
    return Span{lo > 0 ? (lo + kKC - 1) / kKC : 0, nch};
}

template <bool FWD>
__device__ __forceinline__ Span item_span(const Leg& p, const WsItem& e) {
    const LegClass& K = p.cls[e.ci];
    const Geo g = geo(FWD, K.B, e.m);
    const int n0 = e.sub * K.NB;
    return item_span(FWD, g.nch, e.m, n0, min(K.NB, g.NP - n0));
}

// Rows of chunk c's MMAs: r0 (a multiple of 16) and the count n, within the item's `rows`.
__device__ __forceinline__ void chunk_rows(bool fwd, int m, int n0, int rows, int c, bool first, int& r0, int& n) {
    r0 = 0;
    n = rows;
    if (first || naive_order(m)) return;
    const int h = m / 2;
    if (fwd) {
        const int z = kKC * c - h - n0;  // rows below z (item-relative) are zero in chunk c
        r0 = z > 0 ? (z & ~15) : 0;
        n = rows - r0;
    } else {
        const int last = h + kKC * c + kKC - n0;  // rows at or above `last` are zero in chunk c
        n = min(rows, (last + 15) & ~15);
    }
}

template <bool FWD>
__device__ __forceinline__ WsItem decode_item(const Leg& p, long long item) {
    WsItem e;
    if (item >= p.nitems) {
        e.ci = -1;
        return e;
    }
    int ci = 0;
    while (ci + 1 < p.ncls && item >= p.cls[ci + 1].item0) ++ci;
    const LegClass& K = p.cls[ci];
    const long long li = item - K.item0;
    const int rem = (int)(li % K.per_tile);
    const int2 mj = K.itab[rem];
    const int lo = mj.x, j = mj.y;
    const int nsub = (geo(FWD, K.B, lo).NP + K.NB - 1) / K.NB;
    e.ci = ci;
    e.m = lo;
    e.t = j & 1;
    e.sub = (j >> 1) % nsub;
    e.nb = (j >> 1) / nsub;
    e.f0 = (int)(li / K.per_tile) * 64;
    return e;
}

// BF16 A producers with asynchronous copies.  Each producer thread owns the same two
// (row, 8-column segment) tasks of every chunk and stages their FP32 values through a private
// ring of `nstg` stages in shared memory (cp.async, 16-byte pieces for the contiguous forward
// rows, 4-byte pieces for the inverse's stride-2 coefficient gathers), so up to nstg chunks of
// this CTA's A operand are in flight at once, across item boundaries.  A thread reads back only
// what it copied itself, so its own cp.async groups order everything; no cross-thread barrier.
__device__ __forceinline__ float4* stg_at(float4* stg, int s, int q, int h, int tid) {
    return stg + ((s * kTasks + q) * 2 + h) * kAProd + tid;
}

template <bool FWD>
__device__ __forceinline__ void issue_chunk(const LegClass& K, const WsItem& e, int c, float4* stg, int s, int tid) {
    const int B = K.B;
    const bool nv = FWD && naive_order(e.m);
#pragma unroll
    for (int q = 0; q < kTasks; ++q) {
        int r, seg;
        task_rs(tid, q, r, seg);
        const int f = e.f0 + (r & 63), part = r >> 6;
        const int j0 = c * kKC + seg * 8;
        float4* d0 = stg_at(stg, s, q, 0, tid);
        float4* d1 = stg_at(stg, s, q, 1, tid);
        if (FWD) {
            // rows are 32-byte aligned: C rows are BH floats apart, folded X rows BN (both multiples
            // of 8), and j0 % 8 == 0
            const bool ok = f < K.N && j0 < (nv ? K.BN : K.BH);
            const float* src = ok ? fwd_row<FWD>(K, e.m, nv, e.t, f, part) + j0 : (nv ? K.X : K.C);
            tc::cp_async16(d0, src, ok ? 16u : 0u);
            tc::cp_async16(d1, ok ? src + 4 : src, ok ? 16u : 0u);
        } else {
            const bool fok = f < K.N;
            const float* row =
                fok ? (part ? K.ic_in : K.rc_in) + coef_base(K, f) + index_of_harmonic_coeff(e.m, e.m, B) : K.rc_in;
            const int lim = B - e.m;
            float* a = reinterpret_cast<float*>(d0);
            float* b = reinterpret_cast<float*>(d1);
#pragma unroll
            for (int x = 0; x < 8; ++x) {
                const int d = 2 * (j0 + x) + e.t;
                const bool ok = fok && d < lim;
                tc::cp_async4((x < 4 ? a : b) + (x & 3), ok ? row + d : K.rc_in, ok ? 4u : 0u);
            }
        }
    }
}

template <bool FWD>
__device__ __forceinline__ void produce_a_async(const Leg& p, uint8_t* smem, float4* stg, int nstg,
                                                const WsItem* items, uint64_t* item_full, uint64_t* item_empty,
                                                uint64_t* a_full, uint64_t* a_empty, volatile int* s_abort, int tid) {
    constexpr uint32_t kAStage = 3 * kATile;
    const unsigned full = 0xffffffffu;
    uint32_t ac = 0;                 // A tiles produced (position in the A ring)
    uint32_t n_iss = 0, n_con = 0;   // chunks issued into / consumed from the staging ring
    int ki = 0, ci = 0, nch_i = 0;   // issue cursor: item, chunk, chunks of that item
    WsItem ei{};
    bool have_ei = false, iss_done = false;
    float sc[kTasks];
#pragma unroll
    for (int q = 0; q < kTasks; ++q) sc[q] = 1.f;
    // Fill free staging stages.  Waits (bounded) for an unpublished item only when nothing is in
    // flight; every decision is warp-uniform.  Returns false when a wait expired.
    auto top_up = [&]() -> bool {
        while (!iss_done && n_iss - n_con < (uint32_t)nstg) {
            if (!have_ei) {
                const int sl = ki % kNI;
                const uint32_t ph = (ki / kNI) & 1;
                if (!__all_sync(full, tc::mbar_test_wait(&item_full[sl], ph))) {
                    if (n_iss != n_con) return true;
                    if (!__all_sync(full, tc::mbar_wait(&item_full[sl], ph))) return false;
                }
                ei = items[sl];
                if (ei.ci < 0) {
                    iss_done = true;
                    break;
                }
                have_ei = true;
                const Span sp = item_span<FWD>(p, ei);
                ci = sp.c0;
                nch_i = sp.c1;
            }
            issue_chunk<FWD>(p.cls[ei.ci], ei, ci, stg, (int)(n_iss % (uint32_t)nstg), tid);
            tc::cp_async_commit();
            ++n_iss;
            if (++ci == nch_i) {
                have_ei = false;
                ++ki;
            }
        }
        return true;
    };
    for (int k = 0; !*s_abort; ++k) {
        const int slot = k % kNI;
        if (!__all_sync(full, tc::mbar_wait(&item_full[slot], (k / kNI) & 1))) {
            *s_abort = 1;
            break;
        }
        const WsItem e = items[slot];
        tc::mbar_arrive(&item_empty[slot]);
        if (e.ci < 0) break;
        const Span sp = item_span<FWD>(p, e);
        bool ok = true;
        for (int c = sp.c0; c < sp.c1; ++c, ++ac) {
            // chunk (k, c) is the oldest one issued: the issue cursor never falls behind
            if (!top_up() || n_iss == n_con) {
                ok = false;
                break;
            }
            tc::cp_async_wait((int)(n_iss - n_con) - 1);
            float va[kTasks][8];
            const int ss = (int)(n_con % (uint32_t)nstg);
#pragma unroll
            for (int q = 0; q < kTasks; ++q) {
                const float4 a = *stg_at(stg, ss, q, 0, tid), b = *stg_at(stg, ss, q, 1, tid);
                va[q][0] = a.x, va[q][1] = a.y, va[q][2] = a.z, va[q][3] = a.w;
                va[q][4] = b.x, va[q][5] = b.y, va[q][6] = b.z, va[q][7] = b.w;
            }
            ++n_con;
            const int s = ac % kNAS;
            if (!tc::mbar_wait(&a_empty[s], ((ac / kNAS) & 1) ^ 1)) {
                ok = false;
                break;
            }
            store_a<false>(smem + s * kAStage, va, sc, tid);
            tc::fence_proxy_async_smem();
            tc::mbar_arrive(&a_full[s]);
        }
        if (!ok) {
            *s_abort = 1;
            break;
        }
    }
    tc::cp_async_wait(0);  // no copy lands in shared memory after this role has left
}

// v[x] = w[u + 2x], x < 8, for a run-time u in [0, 4] (one unrolled copy per u, no local memory).
template <int U>
__device__ __forceinline__ void pick_u(const float (&w)[20], float* v) {
#pragma unroll
    for (int x = 0; x < 8; ++x) v[x] = w[U + 2 * x];
}
__device__ __forceinline__ void pick_stride2(const float (&w)[20], int u, float* v) {
    switch (u) {
        case 0: pick_u<0>(w, v); break;
        case 1: pick_u<1>(w, v); break;
        case 2: pick_u<2>(w, v); break;
        case 3: pick_u<3>(w, v); break;
        default: pick_u<4>(w, v); break;
    }
}

// BF16 A producers fed by tensor-map TMA: the scheduler warp loads each chunk's A operand
// (FP32) into a staging ring; the producers split their two tasks' values into BF16 terms.
template <bool FWD>
__device__ __forceinline__ void produce_a_tma(const Leg& p, uint8_t* smem, const uint8_t* stg, uint32_t stg_stride,
                                              int nstg, const WsItem* items, uint64_t* item_full, uint64_t* item_empty,
                                              uint64_t* stg_full, uint64_t* stg_empty, uint64_t* a_full,
                                              uint64_t* a_empty, volatile int* s_abort, int tid) {
    constexpr uint32_t kAStage = 3 * kATile;
    const unsigned full = 0xffffffffu;
    uint32_t ac = 0, sc = 0;  // A tiles produced, staging chunks consumed
    int ss = 0;               // staging stage of chunk sc (running: no division per chunk)
    uint32_t sph = 0;         // its phase parity
    float one[kTasks];
#pragma unroll
    for (int q = 0; q < kTasks; ++q) one[q] = 1.f;
    for (int k = 0; !*s_abort; ++k) {
        const int slot = k % kNI;
        if (!__all_sync(full, tc::mbar_wait(&item_full[slot], (k / kNI) & 1))) {
            *s_abort = 1;
            break;
        }
        const WsItem e = items[slot];
        tc::mbar_arrive(&item_empty[slot]);
        if (e.ci < 0) break;
        const LegClass& K = p.cls[e.ci];
        const int B = K.B, m = e.m, t = e.t;
        const bool nv = FWD && naive_order(m);
        const Span sp = item_span<FWD>(p, e);
        const int base = FWD ? 0 : index_of_harmonic_coeff(m, m, B);
        bool ok = true;
        for (int c = sp.c0; c < sp.c1; ++c, ++ac, ++sc) {
            if (!tc::mbar_wait(&stg_full[ss], sph)) {
                ok = false;
                break;
            }
            const uint8_t* sb = stg + (size_t)ss * stg_stride;
            float va[kTasks][8];
#pragma unroll
            for (int q = 0; q < kTasks; ++q) {
                int r, seg;
                task_rs(tid, q, r, seg);
                const int j0 = c * kKC + seg * 8;
                if (FWD) {
                    // 128-byte rows (p, f), 16-byte chunk u of row r stored at chunk u ^ (r % 8)
                    const bool valid = j0 < (nv ? K.BN : K.BH);
                    const float4 a = *reinterpret_cast<const float4*>(sb + r * 128 + (((2 * seg) ^ (r & 7)) << 4));
                    const float4 b = *reinterpret_cast<const float4*>(sb + r * 128 + (((2 * seg + 1) ^ (r & 7)) << 4));
                    va[q][0] = valid ? a.x : 0.f, va[q][1] = valid ? a.y : 0.f;
                    va[q][2] = valid ? a.z : 0.f, va[q][3] = valid ? a.w : 0.f;
                    va[q][4] = valid ? b.x : 0.f, va[q][5] = valid ? b.y : 0.f;
                    va[q][6] = valid ? b.z : 0.f, va[q][7] = valid ? b.w : 0.f;
                } else {
                    // planes [p][64 functions][kInvBox]; the box starts at the 16-byte aligned element
                    // at or below the chunk's first coefficient base + 64 c.  The task's eight
                    // stride-2 values lie in the 20 floats from 16 seg on, read as five aligned
                    // float4: a quarter-warp's eight rows then fall in eight distinct 16-byte bank
                    // groups (rows are 272 bytes apart), where scalar reads of the same values
                    // collided four ways (the segments 0 and 2, 1 and 3 of a row share banks)
                    const int o = (base + c * 64) & 3;
                    const float4* row4 = reinterpret_cast<const float4*>(
                        reinterpret_cast<const float*>(sb) + (r >> 6) * (64 * kInvBox) + (r & 63) * kInvBox +
                        16 * seg);
                    float w[20];
#pragma unroll
                    for (int k4 = 0; k4 < 5; ++k4) {
                        const float4 f4 = row4[k4];
                        w[4 * k4] = f4.x, w[4 * k4 + 1] = f4.y, w[4 * k4 + 2] = f4.z, w[4 * k4 + 3] = f4.w;
                    }
                    pick_stride2(w, o + t, va[q]);
                    const int lim = B - m - c * 64;
#pragma unroll
                    for (int x = 0; x < 8; ++x)
                        if (2 * (seg * 8 + x) + t >= lim) va[q][x] = 0.f;
                }
            }
            // the next chunk's TMA (async proxy) overwrites this staging buffer once the release
            // below is seen: order this thread's generic-proxy reads of it before that write
            tc::fence_proxy_async_smem();
            tc::mbar_arrive(&stg_empty[ss]);
            if (++ss == nstg) {
                ss = 0;
                sph ^= 1;
            }
            const int s = ac % kNAS;
            if (!tc::mbar_wait(&a_empty[s], ((ac / kNAS) & 1) ^ 1)) {
                ok = false;
                break;
            }
            store_a<false>(smem + s * kAStage, va, one, tid);
            tc::fence_proxy_async_smem();
            tc::mbar_arrive(&a_full[s]);
        }
        if (!ok) {
            *s_abort = 1;
            break;
        }
    }
}

// TMA loads of the A operand of chunk c of item e into staging buffer dst (scheduler thread).
template <bool FWD>
__device__ __forceinline__ void issue_a_tma(const Leg& p, const WsItem& e, int c, uint8_t* dst, uint64_t* bar) {
    const int B = p.cls[0].B;
    tc::mbar_arrive_expect_tx(bar, p.a_chunk_bytes);
    if (FWD) {
        const bool nv = naive_order(e.m);
        const int x = (nv ? e.t * p.cls[0].BN : e.t * p.cls[0].BH) + c * kKC;
        tc::tma_load_4d(dst, nv ? (const void*)&p.tmA1 : (const void*)&p.tmA0, x, e.m, e.f0, 0, bar);
    } else {
        const int x0 = (index_of_harmonic_coeff(e.m, e.m, B) + c * 64) & ~3;
        tc::tma_load_2d(dst, &p.tmA0, x0, e.f0, bar);
        tc::tma_load_2d(dst + 64 * kInvBox * sizeof(float), &p.tmA1, x0, e.f0, bar);
    }
}

// The MMAs of one 32-deep chunk: for each 16-deep step, the products x_a t_b of the split terms
// (lead x0 t0 into the accumulator at d0, the rest into the correction accumulator at d0 + corr);
// a first chunk starts both accumulators.
template <int NP>
__device__ __forceinline__ void mma_chunk(uint32_t d0, uint32_t corr, uint64_t da0, uint64_t db0, uint64_t bstep,
                                          uint32_t idesc, bool first_chunk) {
    constexpr int PA[6] = {0, 0, 1, 0, 1, 2}, PB[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
    for (int ks = 0; ks < kKC / 16; ++ks)
#pragma unroll
        for (int pr = 0; pr < NP; ++pr)
            tc::mma_bf16(d0 + (pr ? corr : 0u), da0 + (uint64_t)((PA[pr] * kATile + ks * 256) >> 4),
                         db0 + PB[pr] * bstep + (uint64_t)((ks * 256) >> 4), idesc,
                         (first_chunk && ks == 0 && pr <= 1) ? 0u : 1u);
}

template <bool FWD, bool F16>
__global__ void __launch_bounds__(kWsThreads, 1)
    k_leg_ws(const __grid_constant__ Leg p, uint32_t b_off, uint32_t b_stage, int nbs, uint32_t epi_off,
             uint32_t ncols, int nacc, uint32_t stg_off, int nstg, uint32_t stg_stride) {
    constexpr int NT = F16 ? 2 : 3;
    constexpr uint32_t kAStage = NT * kATile;
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)dsm + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t item_full[kNI], item_empty[kNI], sc_full[kNI];
    __shared__ uint64_t a_full[kNAS], a_empty[kNAS], b_full[kMaxNBS], b_empty[kMaxNBS];
    __shared__ uint64_t acc_full[2], acc_empty[2], fin;
    __shared__ uint64_t stg_full[kMaxStg], stg_empty[kMaxStg];  // tensor-map path: A staging ring
    __shared__ WsItem items[kNI];
    __shared__ float s_rinv[kNI][128];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool a_loader = !F16 && p.tma;  // warp 2 issues the A operand's TMA loads

    if (threadIdx.x == 0) {
        for (int i = 0; i < kNI; ++i) {
            tc::mbar_init(&item_full[i], 1);
            tc::mbar_init(&item_empty[i], 1 + kAProd + kEpi + (a_loader ? 1 : 0));
            tc::mbar_init(&sc_full[i], kAProd);
        }
        for (int i = 0; i < kNAS; ++i) {
            tc::mbar_init(&a_full[i], kAProd);
            tc::mbar_init(&a_empty[i], 1);
        }
        for (int i = 0; i < nbs; ++i) {
            tc::mbar_init(&b_full[i], 1);
            tc::mbar_init(&b_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&acc_full[i], 1);
            tc::mbar_init(&acc_empty[i], kEpi);
        }
        tc::mbar_init(&fin, 1);
        for (int i = 0; i < kMaxStg; ++i) {
            tc::mbar_init(&stg_full[i], 1);
            tc::mbar_init(&stg_empty[i], kAProd);
        }
        tc::fence_mbar_init();
        s_abort = 0;
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t accw = ncols / nacc;  // columns of one accumulator pair
    const uint32_t corr = accw / 2;      // offset of the correction accumulator

    if (warp == 0) {
        // ---------------- scheduler + table producer ----------------
        if (lane == 0) {
            uint32_t bc = 0;  // table chunks issued
            int bs = 0;       // stage of chunk bc (running: no division per chunk)
            uint32_t bph = 0; // its phase parity
            WsItem odd{};     // parity pairs: the odd item of the pair fetched at the last even k
            // The next claim on the work counter is issued before the current item's table copies,
            // so the atomic's round trip overlaps them (its result is read only when the next item
            // is decoded).  Item tables list the parities of an (order, block) next to each other
            // and every class holds an even number of items, so in pair mode an even index starts a
            // pair and one claim takes both.
            const int claim = p.pair ? 2 : 1;
            long long next_idx = p.stall ? 0 : atomicAdd(p.counter, claim);
            for (int k = 0; !s_abort && !p.stall; ++k) {
                const int slot = k % kNI;
                if (!tc::mbar_wait(&item_empty[slot], ((k / kNI) & 1) ^ 1)) {
                    s_abort = 1;
                    break;
                }
                WsItem e;
                bool claimed = false;
                if (p.pair && (k & 1)) {
                    e = odd;
                } else {
                    const long long idx = next_idx;
                    e = decode_item<FWD>(p, idx);
                    if (p.pair) odd = decode_item<FWD>(p, idx + 1);
                    claimed = true;
                }
                items[slot] = e;
                tc::mbar_arrive(&item_full[slot]);
                if (e.ci < 0) {
                    // each epilogue group stops at the first end marker it sees: publish the marker
                    // for the next three items too, so the other group meets one whichever items
                    // (or, in pair mode, parity pairs) it takes
                    for (int x = 1; x <= 3 && !s_abort; ++x) {
                        const int sl = (k + x) % kNI;
                        if (!tc::mbar_wait(&item_empty[sl], (((k + x) / kNI) & 1) ^ 1)) {
                            s_abort = 1;
                            break;
                        }
                        items[sl] = e;
                        tc::mbar_arrive(&item_full[sl]);
                    }
                    break;
                }
                if (claimed) next_idx = atomicAdd(p.counter, claim);
                const LegClass& K = p.cls[e.ci];
                const Geo g = geo(FWD, K.B, e.m);
                const int n0 = e.sub * K.NB, rows = min(K.NB, g.NP - n0);
                const uint8_t* blob =
                    K.blob + K.blob_off[e.m] + (size_t)(e.t * g.nblk + e.nb) * g.nch * NT * g.NP * kKC * 2;
                const Span sp = item_span(FWD, g.nch, e.m, n0, rows);
                for (int c = sp.c0; c < sp.c1; ++c, ++bc) {
                    if (!tc::mbar_wait(&b_empty[bs], bph ^ 1)) {
                        s_abort = 1;
                        break;
                    }
                    issue_table<F16>(smem + b_off + bs * b_stage, blob, g.NP, n0, rows, c, &b_full[bs]);
                    if (++bs == nbs) {
                        bs = 0;
                        bph ^= 1;
                    }
                }
            }
            // copies in flight land before the CTA leaves (immediate on the normal path)
            for (uint32_t j = bc > (uint32_t)nbs ? bc - nbs : 0; j < bc; ++j)
                tc::mbar_wait(&b_full[j % nbs], (j / nbs) & 1);
        }
    } else if (warp == 2 && a_loader) {
        // ---------------- A loader (tensor-map path) ----------------
        if (lane == 0) {
            uint32_t stc = 0;  // A chunks issued
            int ss = 0;        // stage of chunk stc (running: no division per chunk)
            uint32_t sph = 0;  // its phase parity
            for (int k = 0; !s_abort; ++k) {
                const int slot = k % kNI;
                if (!tc::mbar_wait(&item_full[slot], (k / kNI) & 1)) {
                    s_abort = 1;
                    break;
                }
                const WsItem e = items[slot];
                tc::mbar_arrive(&item_empty[slot]);
                if (e.ci < 0) break;
                const Span sp = item_span<FWD>(p, e);
                for (int c = sp.c0; c < sp.c1; ++c, ++stc) {
                    if (!tc::mbar_wait(&stg_empty[ss], sph ^ 1)) {
                        s_abort = 1;
                        break;
                    }
                    issue_a_tma<FWD>(p, e, c, smem + stg_off + (size_t)ss * stg_stride, &stg_full[ss]);
                    if (++ss == nstg) {
                        ss = 0;
                        sph ^= 1;
                    }
                }
            }
            for (uint32_t j = stc > (uint32_t)nstg ? stc - nstg : 0; j < stc; ++j)
                tc::mbar_wait(&stg_full[j % nstg], (j / nstg) & 1);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t ac = 0;            // A chunks consumed
            int sb = 0;                 // table stage (running, no division per chunk)
            uint32_t bph = 0;           // its phase parity
            for (int k = 0; !s_abort; ++k) {
                const int slot = k % kNI;
                if (!tc::mbar_wait(&item_full[slot], (k / kNI) & 1)) {
                    s_abort = 1;
                    break;
                }
                const WsItem e = items[slot];
                tc::mbar_arrive(&item_empty[slot]);
                if (e.ci < 0) break;
                const LegClass& K = p.cls[e.ci];
                const Geo g = geo(FWD, K.B, e.m);
                const int n0 = e.sub * K.NB, rows = min(K.NB, g.NP - n0);
                const Span sp = item_span(FWD, g.nch, e.m, n0, rows);
                const uint32_t bpart = (uint32_t)rows * kKC * 2;
                const AccUse au = acc_use(k, nacc, FWD && p.pair);
                const int buf = au.buf;
                if (!tc::mbar_wait(&acc_empty[buf], (au.use & 1) ^ 1)) {
                    s_abort = 1;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t d0 = tmem + buf * accw;
                bool ok = true;
                for (int c = sp.c0; c < sp.c1; ++c, ++ac) {
                    const int sa = ac % kNAS;
                    if (!tc::mbar_wait(&a_full[sa], (ac / kNAS) & 1) || !tc::mbar_wait(&b_full[sb], bph)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t sa_addr = tc::smem_u32(smem + sa * kAStage);
                    const uint32_t sb_addr = tc::smem_u32(smem + b_off + sb * b_stage);
                    // the issue rate of this single thread bounds the kernel: the product loop is
                    // unrolled for the 6- and 3-product modes, and the operand descriptors are the
                    // chunk's base descriptors plus constant offsets (start address >> 4 in bits 0-13;
                    // shared-memory addresses stay below 2^18, so the sums do not carry)
                    // rows [r0, r0 + nr) of this chunk: D columns and table rows offset by r0 (a table
                    // row is 64 bytes of the K-major core-matrix layout, 4 descriptor units)
                    int r0, nr;
                    chunk_rows(FWD, e.m, n0, rows, c, c == sp.c0, r0, nr);
                    const uint32_t idesc = F16 ? tc::idesc_f16_f32(128, nr) : tc::idesc_bf16_f32(128, nr);
                    const uint64_t da0 = tc::sdesc(sa_addr, 128, kSBO),
                                   db0 = tc::sdesc(sb_addr, 128, kSBO) + (uint64_t)(4 * r0);
                    const uint64_t bstep = bpart >> 4;
                    const uint32_t dr = d0 + (uint32_t)r0;
                    if (p.nprod == 6)
                        mma_chunk<6>(dr, corr, da0, db0, bstep, idesc, c == sp.c0);
                    else if (p.nprod == 3)
                        mma_chunk<3>(dr, corr, da0, db0, bstep, idesc, c == sp.c0);
                    else
                        mma_chunk<1>(dr, corr, da0, db0, bstep, idesc, c == sp.c0);
                    tc::mma_commit(&a_empty[sa]);
                    tc::mma_commit(&b_empty[sb]);
                    if (++sb == nbs) {
                        sb = 0;
                        bph ^= 1;
                    }
                }
                if (!ok) {
                    s_abort = 1;
                    break;
                }
                tc::mma_commit(&acc_full[buf]);
            }
            // every MMA issued has completed before TMEM is freed
            tc::mma_commit(&fin);
            tc::mbar_wait(&fin, 0);
        }
    } else if ((warp >= 4 && warp < 8) || (warp >= 16 && nacc == 2)) {
        // ---------------- epilogue (two groups with two accumulator pairs, else one) ----------------
        const int grp = warp >= 16 ? 1 : 0;
        const int ebar = 1 + grp;                        // the group's named barrier
        const int et = ((warp & 3) << 5) | lane;         // accumulator row = TMEM lane
        float* ep = reinterpret_cast<float*>(smem + epi_off + grp * p.epi_stride);
        constexpr int ES = kEpiCols + 1;   // odd row stride
        uint32_t eblk = 0;                 // TMA-store blocks written (staging buffer eblk & 1)
        for (int i = 0;; ++i) {
            // this group's i-th item: every item with one group; else alternate items, or
            // alternate parity pairs in pair mode (the items of the group's accumulator pair)
            const int k = nacc == 1 ? i : (FWD && p.pair) ? 4 * (i >> 1) + 2 * grp + (i & 1) : 2 * i + grp;
            const int slot = k % kNI;
            const AccUse au = acc_use(k, nacc, FWD && p.pair);
            const int buf = au.buf;
            bool ok = tc::mbar_wait(&item_full[slot], (k / kNI) & 1);
            WsItem e = items[slot];
            if (ok && e.ci >= 0) {
                ok = tc::mbar_wait(&acc_full[buf], au.use & 1);
                if (ok && F16) ok = tc::mbar_wait(&sc_full[slot], (k / kNI) & 1);
            }
            // the group's 128 threads take every decision below together (they share named barriers)
            if (!tc::named_bar_and(ebar, kEpi, ok && !s_abort)) {
                s_abort = 1;
                break;
            }
            if (e.ci < 0) {
                tc::mbar_arrive(&item_empty[slot]);
                break;
            }
            const LegClass K = p.cls[e.ci];
            const int B = K.B, m = e.m, t = e.t;
            const Geo g = geo(FWD, B, m);
            const int n0 = e.sub * K.NB, rows = min(K.NB, g.NP - n0);
            const float rs = F16 ? s_rinv[slot][et] * K.tab_inv : 1.f;
            tc::tc_fence_after();
            const uint32_t trow = tmem + buf * accw + ((uint32_t)((warp & 3) * 32) << 16);
            if (FWD && p.pair) {
                // parity pairs: the even item (k even) parks its results in the stash and frees its
                // accumulator at once; the odd item interleaves both parities in l and stores whole runs
                float* stash = reinterpret_cast<float*>(smem + p.stash_off + grp * p.epi_stride);
                const int SST = p.stash_stride;
                if (t != (k & 1)) {  // not a pair in order (never expected): abort, reported as a device error
                    s_abort = 1;
                    tc::tc_fence_before();
                    tc::mbar_arrive(&acc_empty[buf]);
                    tc::mbar_arrive(&item_empty[slot]);
                    break;
                }
                if (t == 0) {
                    for (int cb = 0; cb < rows; cb += 16) {
                        float v[16];
                        ld_sum(trow + cb, corr, p.nprod > 1, v);
#pragma unroll
                        for (int q = 0; q < 16; ++q) stash[et * SST + cb + q] = v[q] * rs;
                    }
                    tc::tc_fence_before();
                    tc::mbar_arrive(&acc_empty[buf]);
                    tc::mbar_arrive(&item_empty[slot]);
                    continue;
                }
                constexpr int PS = 33;  // interleave tile: 32 values of l per row, odd stride
                for (int cb0 = 0; cb0 < rows; cb0 += 16) {
                    float v[16];
                    ld_sum(trow + cb0, corr, p.nprod > 1, v);
                    if (cb0 + 16 >= rows) {  // last TMEM read of this item: release the buffer
                        tc::tc_fence_before();
                        tc::mbar_arrive(&acc_empty[buf]);
                    }
                    // the even parity's 16 values are read before any store (generic pointers:
                    // a load after a store would wait for it)
                    float ev[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) ev[q] = stash[et * SST + cb0 + q];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        ep[et * PS + 2 * q] = ev[q];
                        ep[et * PS + 2 * q + 1] = v[q] * rs;
                    }
                    tc::named_bar_sync(ebar, kEpi);
                    epi_store_pair(K, m, e.f0, n0 + cb0, ep, PS, warp & 3, 4, lane);
                    tc::named_bar_sync(ebar, kEpi);
                }
                tc::mbar_arrive(&item_empty[slot]);
                continue;
            }
            if (!FWD && p.tma && !naive_order(m)) {
                // 32-column blocks: TMEM -> 128-byte swizzled staging (two buffers) -> one TMA store
                const float sc_ = (float)(0.5 / sqrt((double)B)), sc0 = (float)(1.0 / sqrt(2.0 * B));
                for (int cb0 = 0; cb0 < rows; cb0 += 32, ++eblk) {
                    uint8_t* eb = reinterpret_cast<uint8_t*>(ep) + (eblk & 1) * 16384;
                    if (et == 0) tc::bulk_wait_read1();  // the store that last read this buffer is done
                    tc::named_bar_sync(ebar, kEpi);
                    float v[32];
                    ld_sum(trow + cb0, corr, p.nprod > 1, v);
                    ld_sum(trow + cb0 + 16, corr, p.nprod > 1, v + 16);
                    if (cb0 + 32 >= rows) {  // last TMEM read of this item: release the buffer
                        tc::tc_fence_before();
                        tc::mbar_arrive(&acc_empty[buf]);
                    }
                    const int j0 = n0 + cb0;
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        float4 w4 = make_float4(v[4 * u] * sc_, v[4 * u + 1] * sc_, v[4 * u + 2] * sc_,
                                                v[4 * u + 3] * sc_);
                        if (u == 0 && j0 == 0 && t == 0) w4.x = v[0] * sc0;
                        *reinterpret_cast<float4*>(eb + et * 128 + ((u ^ (et & 7)) << 4)) = w4;
                    }
                    tc::fence_proxy_async_smem();
                    tc::named_bar_sync(ebar, kEpi);
                    if (et == 0) {
                        tc::tma_store_4d(&p.tmO, t * K.BH + j0, m, e.f0, 0, eb);
                        tc::bulk_commit();
                    }
                }
                tc::mbar_arrive(&item_empty[slot]);
                continue;
            }
            if (!FWD && p.tma) {  // the plain path below reuses the staging: no store may still read it
                if (et == 0) tc::bulk_wait_read0();
                tc::named_bar_sync(ebar, kEpi);
            }
            for (int cb0 = 0; cb0 < rows; cb0 += kEpiCols) {
                const int w = min(kEpiCols, rows - cb0);
                for (int cb = 0; cb < w; cb += 16) {
                    float v[16];
                    ld_sum(trow + cb0 + cb, corr, p.nprod > 1, v);
#pragma unroll
                    for (int q = 0; q < 16; ++q) ep[et * ES + cb + q] = v[q] * rs;
                }
                if (cb0 + kEpiCols >= rows) {  // last TMEM read of this item: release the buffer
                    tc::tc_fence_before();
                    tc::mbar_arrive(&acc_empty[buf]);
                }
                tc::named_bar_sync(ebar, kEpi);
                epi_store<FWD>(K, m, t, e.nb, g.NP, e.f0, n0 + cb0, w, ep, ES, warp & 3, 4, lane);
                tc::named_bar_sync(ebar, kEpi);
            }
            tc::mbar_arrive(&item_empty[slot]);
        }
        if (et == 0) tc::bulk_wait_all();  // TMA stores complete before the CTA leaves
    } else if (warp >= 8 && warp < 16 && !F16 && p.tma) {
        // ---------------- A producers (BF16 terms): staging filled by tensor-map TMA ----------------
        produce_a_tma<FWD>(p, smem, smem + stg_off, stg_stride, nstg, items, item_full, item_empty, stg_full,
                           stg_empty, a_full, a_empty, &s_abort, threadIdx.x - 256);
    } else if (warp >= 8 && warp < 16 && !F16) {
        // ---------------- A producers (BF16 terms): asynchronous staging ----------------
        produce_a_async<FWD>(p, smem, reinterpret_cast<float4*>(smem + stg_off), nstg, items, item_full, item_empty,
                             a_full, a_empty, &s_abort, threadIdx.x - 256);
    } else if (warp >= 8 && warp < 16) {
        // ---------------- A producers (FP16 terms): row scales first, loads in registers ----------------
        const int tid = threadIdx.x - 256;
        uint32_t ac = 0;
        float va[kTasks][8];
        float sc[kTasks];
        for (int k = 0; !s_abort; ++k) {
            const int slot = k % kNI;
            // warp-uniform: the F16 row scales below use full-warp shuffles
            if (!__all_sync(0xffffffffu, tc::mbar_wait(&item_full[slot], (k / kNI) & 1))) {
                s_abort = 1;
                break;
            }
            const WsItem e = items[slot];
            tc::mbar_arrive(&item_empty[slot]);
            if (e.ci < 0) break;
            const LegClass K = p.cls[e.ci];
            const int m = e.m, t = e.t, f0 = e.f0;
            const Geo g = geo(FWD, K.B, m);
            const bool nv = naive_order(m);
            if (F16) {
                float mx[kTasks];
#pragma unroll
                for (int q = 0; q < kTasks; ++q) mx[q] = 0.f;
                for (int c = g.nch - 1; c >= 0; --c) {
                    load_a<FWD>(K, m, nv, t, f0, c, va, tid);
#pragma unroll
                    for (int q = 0; q < kTasks; ++q)
#pragma unroll
                        for (int x = 0; x < 8; ++x) mx[q] = fmaxf(mx[q], fabsf(va[q][x]));
                }
#pragma unroll
                for (int q = 0; q < kTasks; ++q) {
                    mx[q] = fmaxf(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], 8));
                    mx[q] = fmaxf(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], 16));
                    int ex = 0;
                    frexpf(mx[q], &ex);  // mx < 2^ex
                    const int sh = mx[q] > 0.f ? min(14 - ex, 120) : 0;
                    sc[q] = ldexpf(1.f, sh);
                    int r, seg;
                    task_rs(tid, q, r, seg);
                    if (seg == 0) s_rinv[slot][r] = ldexpf(1.f, -sh);
                }
                tc::mbar_arrive(&sc_full[slot]);
            } else {
#pragma unroll
                for (int q = 0; q < kTasks; ++q) sc[q] = 1.f;
            }
            const Span sp = item_span<FWD>(p, e);
            load_a<FWD>(K, m, nv, t, f0, sp.c0, va, tid);
            bool ok = true;
            for (int c = sp.c0; c < sp.c1; ++c, ++ac) {
                const int s = ac % kNAS;
                if (!tc::mbar_wait(&a_empty[s], ((ac / kNAS) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                store_a<F16>(smem + s * kAStage, va, sc, tid);
                tc::fence_proxy_async_smem();
                tc::mbar_arrive(&a_full[s]);
                if (c + 1 < sp.c1) load_a<FWD>(K, m, nv, t, f0, c + 1, va, tid);
            }
            if (!ok) {
                s_abort = 1;
                break;
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, ncols);
    }
    if (threadIdx.x == 0 && s_abort) atomicExch(p.err, S2G_ERR_TIMEOUT);
}

// ------------------------------------------------------------------------------------
size_t split_work_bytes(int bw, int batch) {
    const SplitLayout L = split_layout(bw);
    return 2 * (size_t)batch * bw * ((size_t)L.SX + 2 * (size_t)L.BH) * sizeof(float) + 1024;
}

static int set_smem(const void* fn, size_t bytes) {
    // always set: the 48 KiB default covers static plus dynamic shared memory
    S2G_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return S2G_OK;
}

static int check_prec(int precision, int* nprod, bool* f16) {
    *f16 = false;
    if (precision == S2G_PREC_BF16X3) *nprod = 6;
    else if (precision == S2G_PREC_BF16X2) *nprod = 3;
    else if (precision == S2G_PREC_FP16X2) *nprod = 3, *f16 = true;
    else return fail(S2G_ERR_ARG, "precision %d is not a split (tensor-core) mode", precision);
    return S2G_OK;
}

static std::atomic<int> g_leg_stall{0};  // test hook, see s2g_test_stall_contraction

// table_stages: the depth of the table-copy ring (0: as many stages as fit, up to kMaxNBS).
static int launch_leg_ws(bool fwd, bool f16, Leg& p, int nbmax, long long items, int* counter, int table_stages,
                         cudaStream_t st) {
    const void* fn = fwd ? (f16 ? (const void*)k_leg_ws<true, true> : (const void*)k_leg_ws<true, false>)
                         : (f16 ? (const void*)k_leg_ws<false, true> : (const void*)k_leg_ws<false, false>);
    const int nt = f16 ? 2 : 3;
    uint32_t pair = 32;
    while (pair < 2u * nbmax) pair <<= 1;
    const int nacc = 2 * pair <= 512 ? 2 : 1;
    const uint32_t ncols = pair * nacc;
    const size_t a_bytes = (size_t)kNAS * nt * kATile;
    const size_t b_stage = (size_t)nt * nbmax * kKC * 2;
    // epilogue staging: the padded tile of the plain stores (and, on the tensor-map path of the
    // inverse, two 16 KB swizzled TMA-store buffers in the same place), 1024-byte multiple
    size_t epi = ((size_t)128 * (kEpiCols + 1) * sizeof(float) + 1023) & ~(size_t)1023;
    int dev = 0, optin = 0, nsm = 0;
    S2G_CUDA(cudaGetDevice(&dev));
    S2G_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    S2G_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaFuncAttributes fa{};
    S2G_CUDA(cudaFuncGetAttributes(&fa, fn));
    const long long budget = (long long)optin - (long long)fa.sharedSizeBytes - 1024;
    // A staging: tensor-map path, one TMA box per stage (1024-byte multiple: swizzled boxes);
    // cp.async path, per-thread slots.  As many stages as leave room for two table stages.
    const size_t stg_stride = p.tma ? ((size_t)p.a_chunk_bytes + 1023) & ~(size_t)1023 : kStgBytes;
    // forward parity pairs (whole sectors in the coefficient stores): the even parity's results
    // wait in a stash of 128 rows x (nbmax + 1) floats and the interleave tile is 128 x 33, one of
    // each per epilogue group; taken when that still leaves two table stages and four A staging
    // stages (at bw 256 the stash would cut the staging to two, and the shallower A prefetch costs
    // more than the whole sectors gain)
    const int ngrp = nacc;  // epilogue groups: one per accumulator pair (see acc_use)
    p.pair = 0;
    if (fwd && nbmax <= 128) {
        const size_t stash = ((size_t)128 * (nbmax + 1) * sizeof(float) + 1023) & ~(size_t)1023;
        const size_t tile = ((size_t)128 * 33 * sizeof(float) + 1023) & ~(size_t)1023;
        const long long need =
            (long long)(a_bytes + (f16 ? 0 : 4 * stg_stride) + 2 * b_stage + ngrp * (tile + stash));
        if (need <= budget) {
            p.pair = 1;
            p.stash_stride = nbmax + 1;
            epi = tile + stash;  // the stash follows the tile inside the epilogue area
        }
    }
    int nstg = f16 ? 0 : kMaxStg;
    const int nstg_min = p.tma ? 1 : 2;
    long long nbs_fit = 0;
    for (;;) {
        nbs_fit = (budget - (long long)a_bytes - (long long)nstg * (long long)stg_stride - ngrp * (long long)epi) /
                  (long long)b_stage;
        if (nbs_fit >= 2 || nstg <= nstg_min || f16) break;
        --nstg;
    }
    const int nbs = (int)std::min<long long>(table_stages > 0 ? std::min(table_stages, kMaxNBS) : kMaxNBS, nbs_fit);
    if (nbs < 2) return fail(S2G_ERR_UNSUPPORTED, "warp-specialised contraction does not fit in shared memory");
    const size_t stg_bytes = (size_t)nstg * stg_stride;
    const size_t smem = 1024 + a_bytes + stg_bytes + (size_t)nbs * b_stage + ngrp * epi;
    p.epi_stride = (uint32_t)epi;
    S2G_TRY(set_smem(fn, smem));
    const int grid = (int)std::min<long long>(items, nsm);
    S2G_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
    const uint32_t stg_off = (uint32_t)a_bytes, b_off = (uint32_t)(a_bytes + stg_bytes),
                   epi_off = (uint32_t)(a_bytes + stg_bytes + nbs * b_stage);
    if (p.pair) p.stash_off = epi_off + (uint32_t)(((size_t)128 * 33 * sizeof(float) + 1023) & ~(size_t)1023);
    const uint32_t bs = (uint32_t)b_stage, ss = (uint32_t)stg_stride;
    {
        ProfScope ps_(fwd ? "leg_tc_fwd" : "leg_tc_inv", st);
        if (fwd && f16)
            k_leg_ws<true, true><<<grid, kWsThreads, smem, st>>>(p, b_off, bs, nbs, epi_off, ncols, nacc, stg_off, nstg, ss);
        else if (fwd)
            k_leg_ws<true, false><<<grid, kWsThreads, smem, st>>>(p, b_off, bs, nbs, epi_off, ncols, nacc, stg_off, nstg, ss);
        else if (f16)
            k_leg_ws<false, true><<<grid, kWsThreads, smem, st>>>(p, b_off, bs, nbs, epi_off, ncols, nacc, stg_off, nstg, ss);
        else
            k_leg_ws<false, false><<<grid, kWsThreads, smem, st>>>(p, b_off, bs, nbs, epi_off, ncols, nacc, stg_off, nstg,
                                                                   ss);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

// cuTensorMapEncodeTiled from the driver (fetched once through the runtime; no libcuda link).
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
    });
    return fn;
}

// FP32 tiled map: dims/strides innermost first (strides in bytes for dims 1..rank-1).
static bool encode_map(CUtensorMap* m, const void* base, int rank, const uint64_t* dims, const uint64_t* strides,
                       const uint32_t* box, bool swz) {
    auto fn = tmap_encoder();
    if (!fn || ((uintptr_t)base & 15)) return false;
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, const_cast<void*>(base), (const cuuint64_t*)dims,
              (const cuuint64_t*)strides, (const cuuint32_t*)box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              swz ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Sets up the tensor-map path for a one-class launch; false leaves the launch on the other path.
static bool setup_tma(Leg& p, bool fwd, const LegSpec& q) {
    const int B = q.t->bw;
    const uint64_t N = (uint64_t)q.N, b = (uint64_t)B;
    const uint32_t box4[4] = {32, 1, 64, 2};
    if (fwd) {
        const uint64_t dc[4] = {b, b, N, 2}, sc[3] = {b * 4, b * b * 4, N * b * b * 4};
        const uint64_t dx[4] = {2 * b, b, N, 2}, sx[3] = {2 * b * 4, 2 * b * b * 4, 2 * N * b * b * 4};
        if (!encode_map(&p.tmA0, q.C, 4, dc, sc, box4, true) || !encode_map(&p.tmA1, q.X, 4, dx, sx, box4, true))
            return false;
        p.a_chunk_bytes = 32 * 64 * 2 * sizeof(float);
    } else {
        const uint64_t dcoef[2] = {b * b, N}, scoef[1] = {b * b * 4};
        const uint32_t boxc[2] = {(uint32_t)kInvBox, 64};
        const uint64_t dc[4] = {b, b, N, 2}, sc[3] = {b * 4, b * b * 4, N * b * b * 4};
        if (!encode_map(&p.tmA0, q.rc_in, 2, dcoef, scoef, boxc, false) ||
            !encode_map(&p.tmA1, q.ic_in, 2, dcoef, scoef, boxc, false) ||
            !encode_map(&p.tmO, q.Fc, 4, dc, sc, box4, true))
            return false;
        p.a_chunk_bytes = 2 * 64 * kInvBox * sizeof(float);
    }
    return true;
}

// The tensor-map path is off for everything but the plain one-class BF16 launch at bw >= 64
// (s2g_set_contraction_kernel(2) keeps the warp-specialised kernel on its cp.async path).
static std::atomic<int> g_leg_tma{1};

// Device table of the work items of one 64-function tile for tile N extent NB: order m has
// 2 (parities) x nblk(m) (latitude blocks) x ceil(NP(m) / NB) (sub-blocks) items, orders in
// increasing m (largest first); entry = (m, index of the item within its order).
static int get_itab(Split* s, bool fwd, int NB, const int2** out, int* per_tile) {
    std::lock_guard<std::mutex> lk(g_split_mu);
    const int B = s->B;
    std::vector<int2> h;
    for (int m = 0; m < B; ++m) {
        const Geo g = geo(fwd, B, m);
        const int n = 2 * g.nblk * ((g.NP + NB - 1) / NB);
        for (int j = 0; j < n; ++j) h.push_back(make_int2(m, j));
    }
    *per_tile = (int)h.size();
    for (auto& e : s->itab[fwd])
        if (e.first == NB) return (*out = e.second), S2G_OK;
    int2* d = nullptr;
    S2G_CUDA(cudaMalloc(&d, sizeof(int2) * h.size()));
    const cudaError_t e = cudaMemcpy(d, h.data(), sizeof(int2) * h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "cudaMemcpy");
    }
    s->itab[fwd].push_back({NB, d});
    *out = d;
    return S2G_OK;
}

int split_leg(bool fwd, int precision, const LegSpec* spec, int ncls, int* counter, int table_stages,
              cudaStream_t st) {
    int nprod = 0;
    bool f16 = false;
    S2G_TRY(check_prec(precision, &nprod, &f16));
    if (ncls < 1 || ncls > kMaxClasses) return fail(S2G_ERR_ARG, "%d bandwidth classes (1..%d)", ncls, kMaxClasses);
    Leg p{};
    p.ncls = ncls;
    p.nprod = nprod;
    p.counter = counter;
    p.stall = g_leg_stall.load();
    long long items = 0;
    int nbmax = 16;
    // tensor-map TMA path: one class, BF16 terms, contiguous batches, bw a multiple of 64 (the
    // inverse's 32-column output boxes then never reach into the other parity's half row, and every
    // row of the maps is a multiple of 16 bytes), warp-specialised kernel
    const bool want_tma = g_leg_tma && !f16 && ncls == 1 && !spec[0].cmap && spec[0].t->bw >= 64 &&
                          spec[0].t->bw % 64 == 0;
    for (int c = 0; c < ncls; ++c) {
        const LegSpec& q = spec[c];
        S2G_TRY(f16 ? build_split16(q.t) : build_split(q.t));
        Split* s = (Split*)q.t->split;
        LegClass& k = p.cls[c];
        const int B = q.t->bw, npmax = leg_npmax(B, fwd);
        int NB = q.NB > 0 ? std::min(q.NB, npmax) : npmax;
        NB = std::max(16, std::min(256, NB) & ~15);  // the MMA's N is at most 256
        // inverse TMA stores take 32-column blocks, and its staging leaves room for 128-row tables
        if (want_tma && !fwd) NB = std::max(32, std::min(128, NB) & ~31);
        k.B = B;
        const SplitLayout lay = split_layout(B);
        k.BH = lay.BH;
        k.BN = lay.BN;
        k.SX = lay.SX;
        k.N = q.N;
        k.ntiles = (q.N + 63) / 64;
        k.NB = NB;
        S2G_TRY(get_itab(s, fwd, NB, &k.itab, &k.per_tile));
        k.item0 = items;
        k.tab_inv = f16 ? (float)(1.0 / s->tab16) : 1.f;
        k.C = q.C;
        k.X = q.X;
        k.rc_in = q.rc_in;
        k.ic_in = q.ic_in;
        k.rc = q.rc;
        k.ic = q.ic;
        k.Fc = q.Fc;
        k.F = q.F;
        k.cmap = q.cmap;
        k.blob = fwd ? (f16 ? s->fwd16 : s->fwd_blob) : (f16 ? s->inv16 : s->inv_blob);
        k.blob_off = fwd ? (f16 ? s->fwd16_off : s->fwd_off) : (f16 ? s->inv16_off : s->inv_off);
        if (c == 0) p.err = s->err;
        items += (long long)k.ntiles * k.per_tile;
        nbmax = std::max(nbmax, NB);
    }
    p.nitems = items;
    if (items == 0) return S2G_OK;
    p.tma = want_tma && setup_tma(p, fwd, spec[0]) ? 1 : 0;
    if (items > 0x7fffffffLL) return fail(S2G_ERR_ARG, "contraction of %lld work items is too large", items);
    return launch_leg_ws(fwd, f16, p, nbmax, items, counter, table_stages, st);
}

// Grid of a persistent kernel: the CTAs that fit on the GPU at once (cached per kernel and
// shared-memory size), at most `blocks`.
static int persistent_grid(const void* fn, int threads, size_t smem, long long blocks, int* grid) {
    static std::mutex mu;
    static std::vector<std::pair<std::pair<const void*, size_t>, int>> cache;
    int per_gpu = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        for (auto& e : cache)
            if (e.first.first == fn && e.first.second == smem) per_gpu = e.second;
    }
    if (!per_gpu) {
        int occ = 0, dev = 0, nsm = 0;
        S2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem));
        S2G_CUDA(cudaGetDevice(&dev));
        S2G_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        per_gpu = std::max(1, occ) * nsm;
        std::lock_guard<std::mutex> lk(mu);
        cache.push_back({{fn, smem}, per_gpu});
    }
    *grid = (int)std::max<long long>(1, std::min<long long>(blocks, per_gpu));
    return S2G_OK;
}

// ---- warp-FFT kernel launchers (dispatch on R = S / 32) ----
template <int R>
static int launch_fft_kernels(int which, const void* in, void* out, int N, const Split* s, cudaStream_t st,
                              float scale, const int64_t* gmap) {
    constexpr int S = 32 * R, B = S / 2;
    constexpr int kWarps = FftShape<R>::W, kLatPerCta = FftShape<R>::LAT, kThreads = FftShape<R>::T;
    const int nrows = N * B;
    const size_t smem = fft_smem<R>(which);
    if (which == 0) {  // rows forward
        S2G_TRY(set_smem((const void*)k_rows_fwd_w<R>, smem));
        const int g = N * (S / kLatPerCta);  // one tile per CTA: fresh CTAs overlap loads better than a loop
        ProfScope ps_("rows_fwd_f32", st);
        k_rows_fwd_w<R><<<g, kThreads, smem, st>>>((const float*)in, (float*)out, N, scale, s->twS, gmap);
    } else if (which == 1) {  // DCT-II
        S2G_TRY(set_smem((const void*)k_dct_fwd_w<R>, smem));
        int g;
        S2G_TRY(persistent_grid((const void*)k_dct_fwd_w<R>, kThreads, smem, (nrows + kWarps - 1) / kWarps, &g));
        ProfScope ps_("dct_fwd_f32", st);
        k_dct_fwd_w<R><<<g, kThreads, smem, st>>>((float*)in, (float*)out, nrows, s->w32,
                                                                        s->twS, s->twD);
    } else if (which == 2) {  // DCT-III
        S2G_TRY(set_smem((const void*)k_dct_inv_w<R>, smem));
        int g;
        S2G_TRY(persistent_grid((const void*)k_dct_inv_w<R>, kThreads, smem, (nrows + kWarps - 1) / kWarps, &g));
        ProfScope ps_("dct_inv_f32", st);
        k_dct_inv_w<R><<<g, kThreads, smem, st>>>((const float*)in, (float*)out, nrows,
                                                                        s->sin32, s->twS, s->twD, scale);
    } else {  // rows inverse
        S2G_TRY(set_smem((const void*)k_rows_inv_w<R>, smem));
        const int g = N * (S / kLatPerCta);  // one tile per CTA: fresh CTAs overlap loads better than a loop
        ProfScope ps_("rows_inv_f32", st);
        k_rows_inv_w<R><<<g, kThreads, smem, st>>>((const float*)in, (float*)out, N, s->twS, gmap);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

static int fft_kernels(int which, int B, const void* in, void* out, int N, const Split* s, cudaStream_t st,
                       float scale, const int64_t* gmap = nullptr) {
    if (s->czM) {
        const CztTabs g{B, s->czM, s->czh, s->czK, s->cztw, s->w32, s->sin32, s->twD};
        return czt_stage(which, g, in, out, N, scale, gmap, st);
    }
    if ((2 * B) % 32) return fail(S2G_ERR_UNSUPPORTED, "no warp FFT for bandwidth %d", B);
    switch (2 * B / 32) {
        case 1: return launch_fft_kernels<1>(which, in, out, N, s, st, scale, gmap);
        case 3: return launch_fft_kernels<3>(which, in, out, N, s, st, scale, gmap);
        case 5: return launch_fft_kernels<5>(which, in, out, N, s, st, scale, gmap);
        case 6: return launch_fft_kernels<6>(which, in, out, N, s, st, scale, gmap);
        case 7: return launch_fft_kernels<7>(which, in, out, N, s, st, scale, gmap);
        case 9: return launch_fft_kernels<9>(which, in, out, N, s, st, scale, gmap);
        case 10: return launch_fft_kernels<10>(which, in, out, N, s, st, scale, gmap);
        case 11: return launch_fft_kernels<11>(which, in, out, N, s, st, scale, gmap);
        case 12: return launch_fft_kernels<12>(which, in, out, N, s, st, scale, gmap);
        case 13: return launch_fft_kernels<13>(which, in, out, N, s, st, scale, gmap);
        case 14: return launch_fft_kernels<14>(which, in, out, N, s, st, scale, gmap);
        case 15: return launch_fft_kernels<15>(which, in, out, N, s, st, scale, gmap);
        case 2: return launch_fft_kernels<2>(which, in, out, N, s, st, scale, gmap);
        case 4: return launch_fft_kernels<4>(which, in, out, N, s, st, scale, gmap);
        case 8: return launch_fft_kernels<8>(which, in, out, N, s, st, scale, gmap);
        case 16: return launch_fft_kernels<16>(which, in, out, N, s, st, scale, gmap);
        case 32: return launch_fft_kernels<32>(which, in, out, N, s, st, scale, gmap);
        case 64: return launch_fft_kernels<64>(which, in, out, N, s, st, scale, gmap);
        default: return fail(S2G_ERR_UNSUPPORTED, "no warp FFT for bandwidth %d", B);
    }
}

static size_t fft_smem_rt(int R, int which) {
    switch (R) {
        case 1: return fft_smem<1>(which);
        case 2: return fft_smem<2>(which);
        case 4: return fft_smem<4>(which);
        case 8: return fft_smem<8>(which);
        case 16: return fft_smem<16>(which);
        case 32: return fft_smem<32>(which);
        default: return fft_smem<64>(which);
    }
}

template <int WHICH>
static const void* stage_kernel(int rmax) {
    return rmax <= 4 ? (const void*)k_stage_group<WHICH, 4>
         : rmax <= 16 ? (const void*)k_stage_group<WHICH, 16> : (const void*)k_stage_group<WHICH, 32>;
}

int split_stage_group(int which, const StageSpec* spec, int ncls, int dct_ctas_per_sm, cudaStream_t st) {
    if (ncls < 1 || ncls > kStageMaxClasses) return fail(S2G_ERR_ARG, "%d classes in one stage launch", ncls);
    if (which < 0 || which > 3) return fail(S2G_ERR_ARG, "stage %d", which);
    StageArgs a{};
    a.ncls = ncls;
    int rmax = 1;
    size_t smem = 0;
    double wsum = 0.0;
    for (int c = 0; c < ncls; ++c) {
        const StageSpec& q = spec[c];
        S2G_TRY(build_split(q.t));
        const Split* sp = (const Split*)q.t->split;
        const int B = q.t->bw, S = 2 * B, R = S / 32;
        if (R > 32) return fail(S2G_ERR_UNSUPPORTED, "grouped stages take bw <= 512 (got %d)", B);
        StageCls& k = a.c[c];
        k.R = R;
        k.N = q.N;
        k.in = q.in;
        k.out = q.out;
        k.gmap = q.gmap;
        k.w32 = sp->w32;
        k.sin32 = sp->sin32;
        k.twS = sp->twS;
        k.twD = sp->twD;
        k.scale = which == 0 ? (float)(sqrt(2.0 * kPi) / S) : which == 2 ? (float)(1.0 / sqrt(2.0 * kPi)) : 1.f;
        rmax = std::max(rmax, R);
        smem = std::max(smem, fft_smem_rt(R, which));
        wsum += (double)q.N * B * R;
    }
    const void* fn = which == 0 ? stage_kernel<0>(rmax) : which == 1 ? stage_kernel<1>(rmax)
                   : which == 2 ? stage_kernel<2>(rmax) : stage_kernel<3>(rmax);
    S2G_TRY(set_smem(fn, smem));
    int budget = 0;  // DCT stages: blocks shared out by work (rows x length), as many as fit at once
    if (which == 1 || which == 2) {
        int occ = 0, dev = 0, nsm = 0;
        S2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 256, smem));
        S2G_CUDA(cudaGetDevice(&dev));
        S2G_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        if (dct_ctas_per_sm > 0) occ = std::min(std::max(occ, 1), dct_ctas_per_sm);
        budget = std::max(1, occ) * nsm;
    }
    // blocks of the longest transforms first: they take longest, and starting them first leaves
    // the short classes' blocks for the tail of the launch
    int order[kStageMaxClasses];
    for (int c = 0; c < ncls; ++c) order[c] = c;
    std::sort(order, order + ncls, [&](int x, int y) { return a.c[x].R > a.c[y].R; });
    const StageArgs unsorted = a;
    for (int c = 0; c < ncls; ++c) a.c[c] = unsorted.c[order[c]];
    int blk = 0;
    for (int c = 0; c < ncls; ++c) {
        StageCls& k = a.c[c];
        const int B = 16 * k.R, S = 2 * B;
        long long nb;
        if (which == 0 || which == 3) {
            nb = (long long)k.N * (S / FftShape<1>::LAT);
        } else {
            const long long rows = (long long)k.N * B, most = (rows + FftShape<1>::W - 1) / FftShape<1>::W;
            nb = std::llround(budget * ((double)k.N * B * k.R / wsum));
            nb = std::max(1LL, std::min(nb, most));
        }
        if (blk + nb > INT_MAX / 2) return fail(S2G_ERR_UNSUPPORTED, "grouped stage too large");
        k.blk0 = blk;
        k.nblk = (int)nb;
        blk += (int)nb;
    }
    static const char* names[4] = {"rows_fwd_f32_group", "dct_fwd_f32_group", "dct_inv_f32_group",
                                   "rows_inv_f32_group"};
    {
        ProfScope ps_(names[which], st);
        void* args[] = {&a};
        S2G_CUDA(cudaLaunchKernel(fn, dim3(blk), dim3(256), args, smem, st));
    }
    return S2G_OK;
}

// Work counter of the contraction kernel: the int after the two intermediate arrays.
static int* work_counter(void* work, int B, int batch) {
    const SplitLayout L = split_layout(B);
    const size_t used = 2 * (size_t)batch * B * ((size_t)L.SX + 2 * (size_t)L.BH) * sizeof(float);
    return (int*)((char*)work + ((used + 255) & ~(size_t)255));
}

int fst_split(Tables* t, const float* grid, float* rc, float* ic, int batch, int precision, void* work,
              cudaStream_t st) {
    int nprod = 0;
    bool f16 = false;
    S2G_TRY(check_prec(precision, &nprod, &f16));
    S2G_TRY(build_split(t));
    Split* s = (Split*)t->split;
    const int B = t->bw, S = 2 * B;
    float* X = (float*)work;
    float* Cb = X + 2 * (size_t)batch * B * split_layout(B).SX;
    // 1. DFT along phi (two real latitudes per warp), scaled by sqrt(2 pi)/S   (FST_semi_memo.c:81-90)
    S2G_TRY(fft_kernels(0, B, grid, X, batch, s, st, (float)(sqrt(2.0 * kPi) / S)));
    // 2. weighted DCT-II per (function, seminaive order)                      (seminaive.c:161-176)
    S2G_TRY(fft_kernels(1, B, X, Cb, batch, s, st, 1.f));
    // 3. tensor-core contraction (seminaive orders from C, naive orders from X)
    LegSpec q{};
    q.t = t;
    q.N = batch;
    q.C = Cb;
    q.X = X;
    q.rc = rc;
    q.ic = ic;
    return split_leg(true, precision, &q, 1, work_counter(work, B, batch), 0, st);
}

int inv_fst_split(Tables* t, const float* rc, const float* ic, float* grid, int batch, int precision, void* work,
                  cudaStream_t st) {
    int nprod = 0;
    bool f16 = false;
    S2G_TRY(check_prec(precision, &nprod, &f16));
    const int B = t->bw;
    float* F = (float*)work;
    float* Fc = F + 2 * (size_t)batch * B * split_layout(B).SX;
    LegSpec q{};
    q.t = t;
    q.N = batch;
    q.rc_in = rc;
    q.ic_in = ic;
    q.Fc = Fc;
    q.F = F;
    S2G_TRY(split_leg(false, precision, &q, 1, work_counter(work, B, batch), 0, st));
    return split_inv_tail(t, F, Fc, grid, batch, nullptr, st);
}

// ---- COMPLEX data (FST_semi_memo.c:146-200, 290-333) as two real fields ----
// A complex field f = g + i h has real fields g (rdata) and h (idata), so f(l, m) = g(l, m) + i h(l, m)
// for every order, and the real fields' symmetry g(l, -m) = (-1)^m conj g(l, m) gives the negative
// orders from the non-negative ones: f(l, -m) = (-1)^m (conj g(l, m) + i conj h(l, m)).  The real
// path's packed row DFT (two real latitudes per complex FFT) makes the two real transforms cost what
// one complex transform would: the same FFT, DCT and contraction work per function.

// Order and degree of position j of the coefficient layout (util.c:42-49): orders 0 .. B-1 with
// l = m .. B-1, then orders -(B-1) .. -1 with l = |m| .. B-1.
__device__ __forceinline__ void coeff_order_degree(int j, int B, int* m, int* l) {
    const int nn = B * (B + 1) / 2;
    if (j < nn) {  // start(m) = m (2B + 1 - m) / 2
        const float b = 2.f * B + 1.f;
        int mm = (int)((b - sqrtf(fmaxf(b * b - 8.f * (float)j, 0.f))) * 0.5f);
        mm = max(0, min(mm, B - 1));
        while (mm > 0 && mm * (2 * B + 1 - mm) / 2 > j) --mm;
        while (mm + 1 < B && (mm + 1) * (2 * B - mm) / 2 <= j) ++mm;
        *m = mm;
        *l = mm + j - mm * (2 * B + 1 - mm) / 2;
    } else {  // block k = B-1-|m| starts at k (k+1) / 2 and holds k+1 degrees
        const int jj = j - nn;
        int k = (int)((sqrtf(8.f * (float)jj + 1.f) - 1.f) * 0.5f);
        k = max(0, min(k, B - 2));
        while (k > 0 && k * (k + 1) / 2 > jj) --k;
        while (k + 1 <= B - 2 && (k + 1) * (k + 2) / 2 <= jj) ++k;
        *m = -(B - 1 - k);
        *l = (B - 1 - k) + jj - k * (k + 1) / 2;
    }
}

__device__ __forceinline__ void coeff_next(int B, int* m, int* l) {
    if (++*l < B) return;
    if (*m >= 0) {
        ++*m;
        if (*m == B) *m = -(B - 1);
        *l = *m >= 0 ? *m : -*m;
    } else {
        ++*m;
        *l = -*m;
    }
}

// Forward: g, h are [batch][B*B] (re then im arrays, each batch*B*B) from the real path; writes
// f into rc/ic, four consecutive positions per thread (float4 stores).
__global__ void __launch_bounds__(256) k_cplx_combine(const float* __restrict__ gr, const float* __restrict__ gi,
                                                      const float* __restrict__ hr, const float* __restrict__ hi,
                                                      float* __restrict__ rc, float* __restrict__ ic, int B,
                                                      long long nquads) {
    const int BB = B * B, qpf = (BB + 3) / 4;  // quads per function, the last partial when 4 does not divide B^2
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nquads;
         q += (long long)gridDim.x * blockDim.x) {
        const long long f = q / qpf;
        const int j0 = 4 * (int)(q - f * qpf);
        const int ne = min(4, BB - j0);
        const size_t base = (size_t)f * BB;
        int m, l;
        coeff_order_degree(j0, B, &m, &l);
        float orr[4] = {0.f, 0.f, 0.f, 0.f}, oi[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            if (e >= ne) break;
            const int am = m >= 0 ? m : -m;
            const size_t src = base + am * B - (am * (am - 1)) / 2 + (l - am);
            const float a = __ldg(gr + src), b = __ldg(gi + src), c = __ldg(hr + src), d = __ldg(hi + src);
            if (m >= 0) {
                orr[e] = a - d;
                oi[e] = b + c;
            } else {
                const float s = (am & 1) ? -1.f : 1.f;
                orr[e] = s * (a + d);
                oi[e] = s * (c - b);
            }
            coeff_next(B, &m, &l);
        }
        if ((BB & 3) == 0) {  // every function starts 16-byte aligned, every quad is whole
            *(float4*)(rc + base + j0) = make_float4(orr[0], orr[1], orr[2], orr[3]);
            *(float4*)(ic + base + j0) = make_float4(oi[0], oi[1], oi[2], oi[3]);
        } else {
            for (int e = 0; e < ne; ++e) {
                rc[base + j0 + e] = orr[e];
                ic[base + j0 + e] = oi[e];
            }
        }
    }
}

// Inverse: from f (all orders) the non-negative orders of g = (f(l,m) + (-1)^m conj f(l,-m)) / 2 and
// h = (f(l,m) - (-1)^m conj f(l,-m)) / 2i, four consecutive positions per thread.  The real-field
// inverse reads only the non-negative orders, so the negative-order slots of g and h stay unwritten.
__global__ void __launch_bounds__(256) k_cplx_split(const float* __restrict__ rc, const float* __restrict__ ic,
                                                    float* __restrict__ gr, float* __restrict__ gi,
                                                    float* __restrict__ hr, float* __restrict__ hi, int B,
                                                    long long nquads) {
    // quads of the non-negative orders per function (the last partial when 4 does not divide nn)
    const int BB = B * B, nn = B * (B + 1) / 2, qpf = (nn + 3) / 4;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nquads;
         q += (long long)gridDim.x * blockDim.x) {
        const long long f = q / qpf;
        const int j0 = 4 * (int)(q - f * qpf);
        const int ne = min(4, nn - j0);
        const size_t base = (size_t)f * BB;
        const bool vec = (BB & 3) == 0 && ne == 4;  // a whole quad at a 16-byte aligned position
        int m, l;
        coeff_order_degree(j0, B, &m, &l);
        float far_[4] = {0.f, 0.f, 0.f, 0.f}, fai[4] = {0.f, 0.f, 0.f, 0.f};
        if (vec) {
            const float4 ar = *(const float4*)(rc + base + j0), ai = *(const float4*)(ic + base + j0);
            far_[0] = ar.x, far_[1] = ar.y, far_[2] = ar.z, far_[3] = ar.w;
            fai[0] = ai.x, fai[1] = ai.y, fai[2] = ai.z, fai[3] = ai.w;
        } else {
            for (int e = 0; e < ne; ++e) {
                far_[e] = rc[base + j0 + e];
                fai[e] = ic[base + j0 + e];
            }
        }
        float o[4][4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            if (e >= ne) break;
            const int L = B - 1;
            const size_t neg = m == 0 ? base + j0 + e
                                      : base + (L * (L + 3)) / 2 + 1 + ((L - m) * (L - m + 1)) / 2 + (l - m);
            const float s = (m & 1) ? -1.f : 1.f;
            const float br = s * __ldg(rc + neg), bi = -s * __ldg(ic + neg);  // (-1)^m conj f(l, -m)
            o[0][e] = 0.5f * (far_[e] + br);
            o[1][e] = 0.5f * (fai[e] + bi);
            o[2][e] = 0.5f * (fai[e] - bi);
            o[3][e] = -0.5f * (far_[e] - br);
            coeff_next(B, &m, &l);
        }
        if (vec) {
            *(float4*)(gr + base + j0) = make_float4(o[0][0], o[0][1], o[0][2], o[0][3]);
            *(float4*)(gi + base + j0) = make_float4(o[1][0], o[1][1], o[1][2], o[1][3]);
            *(float4*)(hr + base + j0) = make_float4(o[2][0], o[2][1], o[2][2], o[2][3]);
            *(float4*)(hi + base + j0) = make_float4(o[3][0], o[3][1], o[3][2], o[3][3]);
        } else {
            for (int e = 0; e < ne; ++e) {
                gr[base + j0 + e] = o[0][e];
                gi[base + j0 + e] = o[1][e];
                hr[base + j0 + e] = o[2][e];
                hi[base + j0 + e] = o[3][e];
            }
        }
    }
}

size_t split_complex_bytes(int bw, int batch) { return 4 * (size_t)batch * bw * bw * sizeof(float) + 256; }

static int launch_grid_stride(long long n, int* grid) {
    int dev = 0, nsm = 0;
    S2G_CUDA(cudaGetDevice(&dev));
    S2G_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    *grid = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)nsm * 8));
    return S2G_OK;
}

int fst_split_complex(Tables* t, const float* rgrid, const float* igrid, float* rc, float* ic, int batch,
                      int precision, void* work, void* cwork, cudaStream_t st) {
    const int B = t->bw;
    const size_t n = (size_t)batch * B * B;
    float* g = (float*)cwork;
    float* h = g + 2 * n;
    S2G_TRY(fst_split(t, rgrid, g, g + n, batch, precision, work, st));
    S2G_TRY(fst_split(t, igrid, h, h + n, batch, precision, work, st));
    const long long nq = (long long)batch * ((B * B + 3) / 4);  // quads per function, see k_cplx_combine
    int grid;
    S2G_TRY(launch_grid_stride(nq, &grid));
    ProfScope ps_("cplx_combine", st);
    k_cplx_combine<<<grid, 256, 0, st>>>(g, g + n, h, h + n, rc, ic, B, nq);
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

int inv_fst_split_complex(Tables* t, const float* rc, const float* ic, float* rgrid, float* igrid, int batch,
                          int precision, void* work, void* cwork, cudaStream_t st) {
    int nprod = 0;
    bool f16 = false;
    S2G_TRY(check_prec(precision, &nprod, &f16));
    const int B = t->bw;
    const size_t n = (size_t)batch * B * B;
    float* g = (float*)cwork;
    float* h = g + 2 * n;
    const long long nq = (long long)batch * ((B * (B + 1) / 2 + 3) / 4);  // see k_cplx_split
    int grid;
    S2G_TRY(launch_grid_stride(nq, &grid));
    {
        ProfScope ps_("cplx_split", st);
        k_cplx_split<<<grid, 256, 0, st>>>(rc, ic, g, g + n, h, h + n, B, nq);
        S2G_CUDA(cudaGetLastError());
    }
    S2G_TRY(inv_fst_split(t, g, g + n, rgrid, batch, precision, work, st));
    return inv_fst_split(t, h, h + n, igrid, batch, precision, work, st);
}

// One FFT stage of one bandwidth class on its own launch (the per-length warp-FFT or chirp-z
// kernels), with the scale of that stage; in/out and gmap as split_stage_group.
int split_stage_one(int which, Tables* t, int N, const void* in, void* out, const int64_t* gmap, cudaStream_t st) {
    if (which < 0 || which > 3) return fail(S2G_ERR_ARG, "stage %d", which);
    S2G_TRY(build_split(t));
    const Split* s = (const Split*)t->split;
    const int B = t->bw, S = 2 * B;
    const float scale = which == 0 ? (float)(sqrt(2.0 * kPi) / S) : which == 2 ? (float)(1.0 / sqrt(2.0 * kPi)) : 1.f;
    return fft_kernels(which, B, in, out, N, s, st, scale, (which == 0 || which == 3) ? gmap : nullptr);
}

// Inverse stages after the contraction: REDFT01 (+ sin(theta) for odd m), naive-order
// recombination, DFT over the orders into the grid (gmap: per-function grid offsets or null).
int split_inv_tail(Tables* t, float* F, float* Fc, float* grid, int batch, const int64_t* gmap, cudaStream_t st) {
    S2G_TRY(build_split(t));
    Split* s = (Split*)t->split;
    const int B = t->bw;
    const float scale = (float)(1.0 / sqrt(2.0 * kPi));
    // REDFT01 (+ sin(theta) for odd m), scaled by 1/sqrt(2 pi), and the naive orders' even/odd
    // latitude halves recombined                                             (seminaive.c:105-114)
    S2G_TRY(fft_kernels(2, B, Fc, F, batch, s, st, scale));
    // DFT with sign +1 over the orders, Hermitian rows                      (FST_semi_memo.c:334-350)
    return fft_kernels(3, B, F, grid, batch, s, st, 1.f, gmap);
}

int split_prepare(Tables* t, int precision) {
    int nprod = 0;
    bool f16 = false;
    S2G_TRY(check_prec(precision, &nprod, &f16));
    return f16 ? build_split16(t) : build_split(t);
}

// Forward stages before the contraction: DFT along phi and the weighted DCT-II.
int split_fwd_head(Tables* t, const float* grid, float* X, float* C, int batch, const int64_t* gmap,
                   cudaStream_t st) {
    S2G_TRY(build_split(t));
    Split* s = (Split*)t->split;
    const int B = t->bw, S = 2 * B;
    S2G_TRY(fft_kernels(0, B, grid, X, batch, s, st, (float)(sqrt(2.0 * kPi) / S), gmap));
    return fft_kernels(1, B, X, C, batch, s, st, 1.f);
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

extern "C" int s2g_test_stall_contraction(int on) {
    s2g::g_leg_stall = on ? 1 : 0;
    return S2G_OK;
}

extern "C" int s2g_set_contraction_kernel(int which) {
    if (which < 1 || which > 2) return s2g::fail(S2G_ERR_ARG, "contraction data path %d (1 or 2)", which);
    s2g::g_leg_tma = which == 1 ? 1 : 0;
    return S2G_OK;
}

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
