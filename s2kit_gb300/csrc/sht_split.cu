// sht_split.cu -- real-field SHT with FP32 samples/coefficients and the seminaive Legendre
// contraction on the 5th-generation tensor cores as split-BF16 products (FP32 accumulation in TMEM).
//
// Forward (FSTSemiMemo, REAL, cutoff = bw; FST_semi_memo.c:68-145):
//   k_rows_fwd<float>  : DFT along phi, two real latitudes per complex DFT, X[p][f][m][theta]
//   k_dct_fwd32        : weights (even/odd order) + REDFT10 + normalisation (seminaive.c:161-176)
//                        -> C[p][f][m][k], k < bw
//   k_leg_fwd_tc       : per (order m, 64 functions): for each parity t of (l - m), the dense
//                        trapezoid T_{m,t}[i][j] = T(m, l = m+t+2i, k = 2j+t) times C (seminaive.c:183-197)
//                        as D[128 x N] = A[128 x K] * B[N x K]^T on tcgen05, A = 64 functions x
//                        (re, im) rows, B = table rows; epilogue writes f(l, m) and f(l, -m).
// Inverse (InvFSTSemiMemo, REAL; FST_semi_memo.c:228-351):
//   k_leg_inv_tc       : fcos[2j+t] = sum_i T_{m,t}[i][j] a(m + t + 2i) (seminaive.c:74-98), scaled
//   k_dct_inv32        : REDFT01, sin(theta) for odd m, 1/sqrt(2 pi)
//   k_rows_inv<float>  : DFT with sign +1 over m, Hermitian rows, two latitudes per DFT
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

#include "rows.cuh"
#include "s2g_common.cuh"
#include "s2g_internal.h"
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
static constexpr int kNBN = 256; // latitude block of the naive inverse (N per CTA)

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
// FP32 DCTs over latitude for R (function, order) rows per CTA; rows of naive orders are
// skipped (their Legendre transform reads / writes latitude samples directly).
__global__ void k_dct_fwd32(const float* __restrict__ X, float* __restrict__ Cout, int nrows, int B, int logS, int R,
                            const float* __restrict__ w, const float2* __restrict__ twS,
                            const float2* __restrict__ twD) {
    extern __shared__ __align__(16) float fsm[];
    const int S = 2 * B;
    const Len L{S, logS};
    const int SP = S + 1;
    float* zr = fsm;
    float* zi = zr + (size_t)R * SP;
    const int row0 = blockIdx.x * R;
    const int nr = min(R, nrows - row0);
    const size_t plane = (size_t)nrows * S;
    for (int e = threadIdx.x; e < nr * S; e += blockDim.x) {
        const int r = e / S, q = e - r * S;
        const int m = (row0 + r) % B;
        const float wq = w[q + ((m & 1) ? S : 0)];
        const int d = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
        const size_t src = (size_t)(row0 + r) * S + q;
        const bool skip = naive_order(m);
        zr[r * SP + L.pos(d)] = skip ? 0.f : X[src] * wq;
        zi[r * SP + L.pos(d)] = skip ? 0.f : X[plane + src] * wq;
    }
    __syncthreads();
    block_dft<float, float2>(zr, zi, L, nr, SP, twS, -1.0f, nullptr);
    const float nrm = (float)(1.0 / sqrt(2.0 * S));
    const float nrm0 = (float)(0.70710678118654752440 / sqrt(2.0 * S));
    const size_t cplane = (size_t)nrows * B;
    for (int e = threadIdx.x; e < nr * B; e += blockDim.x) {
        const int r = e / B, k = e - r * B;
        if (naive_order((row0 + r) % B)) continue;
        const int kk = (k == 0) ? 0 : S - k;
        const float ar = zr[r * SP + k], ai = zi[r * SP + k], br = zr[r * SP + kk], bi = zi[r * SP + kk];
        const float c = twD[k].x, s = twD[k].y;
        const float f = (k == 0) ? nrm0 : nrm;
        Cout[(size_t)(row0 + r) * B + k] = ((ar + br) * c + (ai - bi) * s) * f;
        Cout[cplane + (size_t)(row0 + r) * B + k] = ((ai + bi) * c - (ar - br) * s) * f;
    }
}

__global__ void k_dct_inv32(const float* __restrict__ Fc, float* __restrict__ F, int nrows, int B, int logS, int R,
                            const float* __restrict__ sinv, const float2* __restrict__ twS,
                            const float2* __restrict__ twD, float scale) {
    extern __shared__ __align__(16) float fsm[];
    const int S = 2 * B;
    const Len L{S, logS};
    const int SP = S + 1;
    float* zr = fsm;
    float* zi = zr + (size_t)R * SP;
    const int row0 = blockIdx.x * R;
    const int nr = min(R, nrows - row0);
    const size_t cplane = (size_t)nrows * B;
    for (int e = threadIdx.x; e < nr * S; e += blockDim.x) {
        const int r = e / S, k = e - r * S;
        const bool skip = naive_order((row0 + r) % B);
        const float* xa = Fc + (size_t)(row0 + r) * B;
        const float* xb = xa + cplane;
        const float ak = (!skip && k < B) ? xa[k] : 0.f, bk = (!skip && k < B) ? xb[k] : 0.f;
        const int q = S - k;
        const float ar = (!skip && k > 0 && q < B) ? xa[q] : 0.f, br = (!skip && k > 0 && q < B) ? xb[q] : 0.f;
        const float wr = ak + br, wi = bk - ar;
        const float c = twD[k].x, s = twD[k].y;
        zr[r * SP + L.pos(k)] = wr * c - wi * s;
        zi[r * SP + L.pos(k)] = wr * s + wi * c;
    }
    __syncthreads();
    block_dft<float, float2>(zr, zi, L, nr, SP, twS, 1.0f, nullptr);
    const size_t plane = (size_t)nrows * S;
    for (int e = threadIdx.x; e < nr * S; e += blockDim.x) {
        const int r = e / S, q = e - r * S;
        const int m = (row0 + r) % B;
        if (naive_order(m)) continue;
        const int src = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
        const float g = (m & 1) ? sinv[q] * scale : scale;
        F[(size_t)(row0 + r) * S + q] = zr[r * SP + src] * g;
        F[plane + (size_t)(row0 + r) * S + q] = zi[r * SP + src] * g;
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

template <bool FWD>
__device__ __forceinline__ void produce_a(const Leg& p, uint8_t* st, int m, bool nv, int t, int f0, int c) {
    constexpr int segs = kKC / 8;
    for (int task = threadIdx.x; task < 128 * segs; task += kTPB) {
        const int r = task / segs, seg = task - r * segs;
        float v[8];
        load_seg<FWD>(p, m, nv, t, f0 + (r & 63), r >> 6, c, seg, v);
        uint32_t w[3][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            __nv_bfloat16 a0, a1, a2, b0, b1, b2;
            tc::split3(v[2 * q], a0, a1, a2);
            tc::split3(v[2 * q + 1], b0, b1, b2);
            w[0][q] = (uint32_t)__bfloat16_as_ushort(a0) | ((uint32_t)__bfloat16_as_ushort(b0) << 16);
            w[1][q] = (uint32_t)__bfloat16_as_ushort(a1) | ((uint32_t)__bfloat16_as_ushort(b1) << 16);
            w[2][q] = (uint32_t)__bfloat16_as_ushort(a2) | ((uint32_t)__bfloat16_as_ushort(b2) << 16);
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
    const int m = blockIdx.x, f0 = blockIdx.y * 64;
    const int t = blockIdx.z & 1, nb = blockIdx.z >> 1;
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

    for (int c = 0; c < nchunks; ++c) {
        const int s = c & 1;
        uint8_t* st = smem + s * stage_bytes;
        if (threadIdx.x == 0) {
            if (c >= 2 && !tc::mbar_wait(&bars[2 + s], ((c - 2) >> 1) & 1)) s_abort = 1;
            if (!s_abort) {
                tc::mbar_arrive_expect_tx(&bars[s], 3 * bt);
                tc::bulk_g2s(st + 3 * kATile, blob + (size_t)c * 3 * bt, 3 * bt, &bars[s]);
            }
        }
        __syncthreads();
        if (s_abort) break;
        produce_a<FWD>(p, st, m, nv, t, f0, c);
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
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && !s_abort) {
        const int last = nchunks - 1;
        if (!tc::mbar_wait(&bars[2 + (last & 1)], (last >> 1) & 1)) s_abort = 1;
    }
    __syncthreads();
    if (!s_abort && warp < 4) {
        tc::tc_fence_after();
        const int r = warp * 32 + lane;
        const int f = f0 + (r & 63), part = r >> 6;
        const bool live = f < p.N;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        if (FWD) {
            float* out = (part ? p.ic : p.rc) + (size_t)f * B * B;
            const int base = index_of_harmonic_coeff(m, m, B) + t;
            const int nbase = index_of_harmonic_coeff(-m, m, B) + t;
            const float sneg = ((m & 1) ? -1.f : 1.f) * (part ? -1.f : 1.f);
            const int lim = B - m - t;  // valid 2i
            for (int cb = 0; cb < NP; cb += 16) {
                float v[16];
                ld_sum(trow + cb, NP, p.nprod > 1, v);
                if (live) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int d = 2 * (cb + q);
                        if (d < lim) {
                            out[base + d] = v[q];
                            if (m) out[nbase + d] = sneg * v[q];
                        }
                    }
                }
            }
        } else if (!nv) {
            float* out = p.Fc + (((size_t)part * p.N + f) * B + m) * B + t;
            const float sc = (float)(0.5 / sqrt((double)B)), sc0 = (float)(1.0 / sqrt(2.0 * B));
            for (int cb = 0; cb < NP; cb += 16) {
                float v[16];
                ld_sum(trow + cb, NP, p.nprod > 1, v);
                if (live) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int k = 2 * (cb + q);
                        if (k < B) out[k] = v[q] * ((k + t == 0) ? sc0 : sc);
                    }
                }
            }
        } else {
            float* out = p.F + (((size_t)part * p.N + f) * B + m) * (2 * B) + t * B + nb * NP;
            for (int cb = 0; cb < NP; cb += 16) {
                float v[16];
                ld_sum(trow + cb, NP, p.nprod > 1, v);
                if (live) {
#pragma unroll
                    for (int q = 0; q < 16; q += 4)
                        *reinterpret_cast<float4*>(out + cb + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                }
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

static int dct_rows_per_cta(int S) {
    int R = 8192 / S;
    return R < 1 ? 1 : (R > 32 ? 32 : R);
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
    dim3 grid(p.B, (p.N + 63) / 64, 2 * nblk);
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

static int rows_r(int S) { return (4096 / S) < 1 ? 1 : ((4096 / S) > 32 ? 32 : 4096 / S); }

int fst_split(Tables* t, const float* grid, float* rc, float* ic, int batch, int precision, void* work,
              cudaStream_t st) {
    int nprod;
    S2G_TRY(check_prec(precision, &nprod));
    S2G_TRY(build_split(t));
    Split* s = (Split*)t->split;
    const int B = t->bw, S = 2 * B;
    const Len L = make_len(S);
    float* X = (float*)work;
    float* Cb = X + 2 * (size_t)batch * B * S;
    // 1. DFT along phi (two real latitudes per complex DFT), scaled by sqrt(2 pi)/S
    {
        const int R = rows_r(S);
        const size_t smem = (size_t)2 * R * (S + 1) * sizeof(float);
        S2G_TRY(set_smem((const void*)k_rows_fwd<float, float2>, smem));
        dim3 grid2((S + 2 * R - 1) / (2 * R), batch);
        {
            ProfScope ps_("rows_fwd_f32", st);
            k_rows_fwd<float, float2><<<grid2, 256, smem, st>>>(grid, nullptr, X, X + (size_t)batch * B * S, S, L.logn, B,
                                                               R, (float)(sqrt(2.0 * kPi) / S), s->twS);
        }
        S2G_CUDA(cudaGetLastError());
    }
    // 2. weighted DCT-II per (function, seminaive order)
    {
        const int nrows = batch * B;
        const int R = dct_rows_per_cta(S);
        const size_t smem = (size_t)2 * R * (S + 1) * sizeof(float);
        S2G_TRY(set_smem((const void*)k_dct_fwd32, smem));
        {
            ProfScope ps_("dct_fwd_f32", st);
            k_dct_fwd32<<<(nrows + R - 1) / R, 256, smem, st>>>(X, Cb, nrows, B, L.logn, R, s->w32, s->twS, s->twD);
        }
        S2G_CUDA(cudaGetLastError());
    }
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
    const Len L = make_len(S);
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
    {
        const int nrows = batch * B;
        const int R = dct_rows_per_cta(S);
        const size_t smem = (size_t)2 * R * (S + 1) * sizeof(float);
        S2G_TRY(set_smem((const void*)k_dct_inv32, smem));
        {
            ProfScope ps_("dct_inv_f32", st);
            k_dct_inv32<<<(nrows + R - 1) / R, 256, smem, st>>>(Fc, F, nrows, B, L.logn, R, s->sin32, s->twS, s->twD,
                                                                 scale);
        }
        S2G_CUDA(cudaGetLastError());
        const int nnaive = std::min(B, kNaiveOddBelow) / 2;
        {
            ProfScope ps_("naive_combine_f32", st);
            k_naive_combine<<<dim3(batch * nnaive, 2), 256, S * sizeof(float), st>>>(F, batch, B, scale);
        }
        S2G_CUDA(cudaGetLastError());
    }
    {
        const int R = rows_r(S);
        const size_t smem = (size_t)2 * R * (S + 1) * sizeof(float);
        S2G_TRY(set_smem((const void*)k_rows_inv<float, float2>, smem));
        dim3 grid2((S + 2 * R - 1) / (2 * R), batch);
        {
            ProfScope ps_("k_rows_inv<float, float2>", st);
            k_rows_inv<float, float2><<<grid2, 256, smem, st>>>(F, F + (size_t)batch * B * S, B, 0, grid, nullptr, S,
                                                               L.logn, R, s->twS);
        }
        S2G_CUDA(cudaGetLastError());
    }
    return S2G_OK;
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
