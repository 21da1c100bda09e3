// czt_split.cu -- FFT stages of the split-precision path at the bandwidths whose transform length
// S = 2B is not a warp-FFT length (32 R for the R the warp FFTs of fft32.cuh take): odd bandwidths,
// and even ones that are neither powers of two nor multiples of 16 in [48, 240].  Every length-S
// DFT there is Bluestein's chirp-z transform over a power-of-two warp FFT of length M = 32 RM,
// M >= 2S - 1 (L. Bluestein, "A linear filtering approach to the computation of discrete Fourier
// transform", 1970):
//   X_k = sum_n x_n w^(n k), w = exp(sign 2 pi i / S).  With n k = (n^2 + k^2 - (k - n)^2) / 2 and
//   the chirp c_n = exp(sign i pi n^2 / S),  X_k = c_k sum_n (x_n c_n) conj(c_(k-n)):  a cyclic
//   convolution of length M of a_n = x_n c_n (n < S, zero beyond) with b_j = conj(c_|j|)
//   (|j| < S, j taken mod M), evaluated as X_k = c_k IDFT_M(DFT_M(a) DFT_M(b))_k, k < S.
// DFT_M(b) / M is a table per bandwidth, built on the host in FP64 with exact angle reduction.  The
// sign +1 chirp and kernel spectrum are the complex conjugates of the sign -1 ones (b is even in
// j), so one pair of tables serves all four stages.  n^2 is reduced mod 2S in integers before the
// angle is formed, so the chirp is exact to FP64 rounding at every n.
//
// The four stage kernels compute what the warp-FFT stage kernels of sht_split.cu compute
// (FST_semi_memo.c:81-90 and 334-350 for the longitude DFTs, seminaive.c:161-176 and 105-114 for
// the weighted REDFT10 and the REDFT01), with the transform length a run-time value and the
// intermediate layout of split_layout(B): rows padded to multiples of 8 floats (every row starts
// 32-byte aligned, as the contraction's 16-byte operand copies need), the padding written as zeros.
#include <math.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "s2g_common.cuh"
#include "s2g_internal.h"
#include "fft32.cuh"

namespace s2g {

namespace {

constexpr int kW = 8;          // warps per CTA, one sequence each
constexpr int kT = 32 * kW;
constexpr int kLat = 2 * kW;   // latitudes per CTA in the row kernels (two real rows per warp)

// Per-warp spectrum / exchange rows: >= pad32(M) floats (the spectrum at pad32(k), k < M, and the
// four-step FFT's exchange, R (32 + 32/R) = pad32(M) floats per plane), 4 mod 32 so that the same
// element of different warps' rows falls in different banks.
template <int RM>
struct CztShape {
    static constexpr int M = 32 * RM;
    static constexpr int PSA = (((M + M / 32) + 31) & ~31) + 4;
};

// Shared-memory tables every stage kernel loads: the warp FFT's twiddles for length M (padded
// table and its (register, lane) copy, see fft32.cuh), the kernel spectrum in register order
// (kq[32 k1 + lane] = K[out_index(k1)] of that lane) and the chirp.
struct CztSm {
    float2* tw;
    float2* twb;
    float2* kq;
    float2* h;
};

template <int RM>
__device__ __forceinline__ size_t czt_tab_floats(int S) {
    constexpr int M = 32 * RM;
    return 2 * ((size_t)twtab_len(M) + 2 * M + S);
}

template <int RM>
__device__ __forceinline__ CztSm czt_load(float* base, const CztTabs& g) {
    constexpr int M = 32 * RM;
    CztSm t;
    t.tw = reinterpret_cast<float2*>(base);
    t.twb = t.tw + twtab_len(M);
    t.kq = t.twb + M;
    t.h = t.kq + M;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        t.tw[padtw(k)] = g.twM[k];
        t.twb[k] = g.twM[((k & 31) * (k >> 5)) % M];
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k1 = warp; k1 < RM; k1 += blockDim.x >> 5) t.kq[32 * k1 + lane] = g.K[WarpFFTSel<RM>::out_index(k1)];
    for (int n = threadIdx.x; n < 2 * g.B; n += blockDim.x) t.h[n] = g.h[n];
    return t;
}

// chirp c_n of the given sign: the table holds the sign -1 chirp
__device__ __forceinline__ float2 chirp(const CztSm& t, int n, float sign) {
    const float2 c = t.h[n];
    return make_float2(c.x, -sign * c.y);
}

// Chirp-z transform of the warp's sequence.  On entry v holds a_n = x_n c_n in natural order
// (register i of lane L is n = L + 32 i, zero for n >= S); on return zr/zi[pad32(k)] hold
// X_k = sum_n x_n exp(sign 2 pi i n k / S) for k < S.  zr/zi are the warp's own rows.
template <int RM>
__device__ __forceinline__ void czt_warp(float2 (&v)[RM], const CztSm& t, float* zr, float* zi, int S, float sign) {
    const int lane = threadIdx.x & 31;
    WarpFFTSel<RM>::run(v, t.tw, t.twb, zr, zi, -1.f);  // DFT_M(a)
#pragma unroll
    for (int k1 = 0; k1 < RM; ++k1) {
        float2 q = t.kq[32 * k1 + lane];
        q.y *= -sign;
        v[k1] = cmulf(v[k1], q);
    }
    // to natural order through the warp's rows.  At RM = 32 the four-step FFT's output order is
    // its input order already (one lane per column: register s of lane L holds index L + 32 s),
    // so the product goes straight into the second FFT.
    if constexpr (RM != 32) {
        __syncwarp();
#pragma unroll
        for (int k1 = 0; k1 < RM; ++k1) {
            const int o = pad32(WarpFFTSel<RM>::out_index(k1));
            zr[o] = v[k1].x;
            zi[o] = v[k1].y;
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < RM; ++i) {
            const int o = pad32(lane + 32 * i);
            v[i] = make_float2(zr[o], zi[o]);
        }
        __syncwarp();
    }
    WarpFFTSel<RM>::run(v, t.tw, t.twb, zr, zi, 1.f);  // M IDFT_M (the 1/M is in the kernel spectrum)
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < RM; ++k1) {
        const int o = WarpFFTSel<RM>::out_index(k1);
        if (o < S) {
            const float2 x = cmulf(v[k1], chirp(t, o, sign));
            zr[pad32(o)] = x.x;
            zi[pad32(o)] = x.y;
        }
    }
    __syncwarp();
}

// DFT along phi of kLat latitudes (two real rows per warp, packed as one complex sequence),
// separated and transposed to X[p][f][m][theta] (rows of SX floats; latitudes S .. SX-1 zero).
template <int RM>
__global__ void __launch_bounds__(kT) k_czt_rows_fwd(const float* __restrict__ grid, float* __restrict__ X, int N,
                                                     int B, int SX, float scale, const CztTabs g,
                                                     const int64_t* __restrict__ gmap) {
    using Sh = CztShape<RM>;
    constexpr int PSA = Sh::PSA;
    const int S = 2 * B;
    extern __shared__ __align__(16) float fsm[];
    float* spr = fsm;
    float* spi = spr + kW * PSA;
    const CztSm t = czt_load<RM>(spi + kW * PSA, g);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NT = SX / kLat;
    const int f = blockIdx.x / NT, th0 = (blockIdx.x - f * NT) * kLat;
    const int a = th0 + 2 * warp;  // this warp's latitudes a, a + 1 (S is even: both or neither exist)
    float* zr = spr + warp * PSA;
    float* zi = spi + warp * PSA;
    if (a < S) {
        const float* ra = grid + (gmap ? gmap[f] : (int64_t)f * S * S) + (size_t)a * S;
        float2 v[RM];
#pragma unroll
        for (int i = 0; i < RM; ++i) {
            const int n = lane + 32 * i;
            v[i] = n < S ? cmulf(make_float2(ra[n], ra[S + n]), chirp(t, n, -1.f)) : make_float2(0.f, 0.f);
        }
        czt_warp<RM>(v, t, zr, zi, S, -1.f);
    }
    __syncthreads();
    const size_t plane = (size_t)N * B * SX;
    const float hs = 0.5f * scale;
    for (int e = threadIdx.x; e < B * (kLat / 4); e += kT) {
        const int m = e / (kLat / 4), q = 4 * (e - m * (kLat / 4));
        float re[4], im[4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // latitude pair q/2 + h is warp q/2 + h's (a, b) rows
            const int w = q / 2 + h;
            if (th0 + 2 * w < S) {
                const float* zwr = spr + w * PSA;
                const float* zwi = spi + w * PSA;
                const int pm = pad32(m), pn = pad32((S - m) % S);
                const float ar = zwr[pm], ai = zwi[pm], br = zwr[pn], bi = zwi[pn];
                re[2 * h] = (ar + br) * hs;
                im[2 * h] = (ai - bi) * hs;
                re[2 * h + 1] = (ai + bi) * hs;
                im[2 * h + 1] = (br - ar) * hs;
            } else {
                re[2 * h] = im[2 * h] = re[2 * h + 1] = im[2 * h + 1] = 0.f;
            }
        }
        const size_t o = ((size_t)f * B + m) * SX + th0 + q;
        *reinterpret_cast<float4*>(X + o) = make_float4(re[0], re[1], re[2], re[3]);
        *reinterpret_cast<float4*>(X + plane + o) = make_float4(im[0], im[1], im[2], im[3]);
    }
}

// Weighted REDFT10 per (function, seminaive order) row (Makhoul's reordering: v_n = x_(2n),
// v_(S-1-n) = x_(2n+1), then one length-S DFT), stored by parity of the cosine index:
// C[p][f][m][t][j] holds k = 2j + t < B at t BH + j (rows of 2 BH floats, zeros past B).  Naive
// orders are folded in place in X: X[p][f][m][t BN + j] = x_j + (-1)^t x_(S-1-j), j < B, zeros
// up to BN.  Persistent: each warp walks rows.
template <int RM>
__global__ void __launch_bounds__(kT, 2) k_czt_dct_fwd(float* __restrict__ X, float* __restrict__ Cout, int nrows,
                                                    int B, int BH, int BN, int SX, const CztTabs g) {
    using Sh = CztShape<RM>;
    constexpr int PSA = Sh::PSA;
    const int S = 2 * B;
    extern __shared__ __align__(16) float fsm[];
    float* spr = fsm;
    float* spi = spr + kW * PSA;
    float* tabs = spi + kW * PSA;
    const CztSm t = czt_load<RM>(tabs, g);
    float* w = tabs + czt_tab_floats<RM>(S);             // 2S weights (even orders, then odd)
    float2* twD = reinterpret_cast<float2*>(w + 2 * S);  // (cos, sin)(pi k / 2S), k < B
    for (int q = threadIdx.x; q < 2 * S; q += blockDim.x) w[q] = g.w32[q];
    for (int k = threadIdx.x; k < B; k += blockDim.x) twD[k] = g.twD[k];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* zr = spr + warp * PSA;
    float* zi = spi + warp * PSA;
    const float nrm = rsqrtf(2.f * S);
    const float nrm0 = 0.70710678118654752440f * nrm;
    for (int row = blockIdx.x * kW + warp; row < nrows; row += gridDim.x * kW) {
        const int m = row % B;
        float* xr = X + (size_t)row * SX;
        float* xi = xr + (size_t)nrows * SX;
        if (split_naive_order(m)) {
            for (int n = lane; n < S; n += 32) {
                zr[n] = xr[n];
                zi[n] = xi[n];
            }
            __syncwarp();
            for (int o4 = lane; o4 < BN / 2; o4 += 32) {  // 2 BN / 4 float4 pieces
                const int tt = (4 * o4) >= BN, j0 = 4 * o4 - tt * BN;
                const float sg = tt ? -1.f : 1.f;
                float a[4], c[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = j0 + u;
                    a[u] = j < B ? zr[j] + sg * zr[S - 1 - j] : 0.f;
                    c[u] = j < B ? zi[j] + sg * zi[S - 1 - j] : 0.f;
                }
                reinterpret_cast<float4*>(xr)[o4] = make_float4(a[0], a[1], a[2], a[3]);
                reinterpret_cast<float4*>(xi)[o4] = make_float4(c[0], c[1], c[2], c[3]);
            }
            __syncwarp();  // the staged row is read before the next row overwrites it
            continue;
        }
        const float* ws = w + ((m & 1) ? S : 0);
        // the weighted row goes through the warp's rows (coalesced loads, few registers in flight),
        // then into the registers in Makhoul's order
        for (int q = lane; q < S; q += 32) {
            zr[q] = xr[q] * ws[q];
            zi[q] = xi[q] * ws[q];
        }
        __syncwarp();
        float2 v[RM];
#pragma unroll
        for (int i = 0; i < RM; ++i) {
            const int n = lane + 32 * i;
            if (n < S) {
                const int q = n < B ? 2 * n : 2 * (S - 1 - n) + 1;
                v[i] = cmulf(make_float2(zr[q], zi[q]), chirp(t, n, -1.f));
            } else {
                v[i] = make_float2(0.f, 0.f);
            }
        }
        __syncwarp();  // every lane has read the staged row before the transform reuses the rows
        czt_warp<RM>(v, t, zr, zi, S, -1.f);
        float* cr = Cout + (size_t)row * (2 * BH);
        float* ci = cr + (size_t)nrows * (2 * BH);
        // order 0 of a real field: exact zeros in the imaginary plane (see k_dct_fwd_w)
        const bool im_zero = (m == 0);
        for (int o4 = lane; o4 < BH / 2; o4 += 32) {  // 2 BH / 4 float4 pieces
            float a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int o = 4 * o4 + u;
                const int tt = o >= BH, k = 2 * (o - tt * BH) + tt;
                a[u] = b[u] = 0.f;
                if (k < B) {
                    const int kk = (S - k) % S;
                    const float ar = zr[pad32(k)], ai = zi[pad32(k)], br = zr[pad32(kk)], bi = zi[pad32(kk)];
                    const float2 cs = twD[k];
                    const float fct = (k == 0) ? nrm0 : nrm;
                    a[u] = ((ar + br) * cs.x + (ai - bi) * cs.y) * fct;
                    b[u] = im_zero ? 0.f : ((ai + bi) * cs.x - (ar - br) * cs.y) * fct;
                }
            }
            reinterpret_cast<float4*>(cr)[o4] = make_float4(a[0], a[1], a[2], a[3]);
            reinterpret_cast<float4*>(ci)[o4] = make_float4(b[0], b[1], b[2], b[3]);
        }
        __syncwarp();  // the spectrum is read before the next row's transform overwrites it
    }
}

// REDFT01 per (function, seminaive order) row, sin(theta) for odd m, scale: F[p][f][m][theta]
// (rows of SX floats).  Naive orders: the contraction left D0 (even l - m) at [0, B) and D1 (odd
// l - m) at [BN, BN + B) for the northern latitudes; F[theta] = D0 + D1 and F[S-1-theta] = D0 - D1.
// Compiled for two CTAs per SM: unbounded it takes 225 registers at M = 1024 (one CTA), and the
// bound took bw 255 from 0.65 to 0.40 ms at 256 functions (the forward DCT measured 5% slower
// under the same bound and stays unbounded).
template <int RM>
__global__ void __launch_bounds__(kT, 2) k_czt_dct_inv(const float* __restrict__ Fc, float* __restrict__ F, int nrows,
                                                    int B, int BH, int BN, int SX, float scale, const CztTabs g) {
    using Sh = CztShape<RM>;
    constexpr int PSA = Sh::PSA;
    const int S = 2 * B;
    extern __shared__ __align__(16) float fsm[];
    float* spr = fsm;
    float* spi = spr + kW * PSA;
    float* tabs = spi + kW * PSA;
    const CztSm t = czt_load<RM>(tabs, g);
    float* sn = tabs + czt_tab_floats<RM>(S);             // sin(theta), S
    float2* twD = reinterpret_cast<float2*>(sn + S + (S & 2));  // (cos, sin)(pi k / 2S), k < S (8-byte aligned)
    for (int q = threadIdx.x; q < S; q += blockDim.x) {
        sn[q] = g.sin32[q];
        twD[q] = g.twD[q];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* zr = spr + warp * PSA;
    float* zi = spi + warp * PSA;
    for (int row = blockIdx.x * kW + warp; row < nrows; row += gridDim.x * kW) {
        const int m = row % B;
        float* fr = F + (size_t)row * SX;
        float* fi = fr + (size_t)nrows * SX;
        if (split_naive_order(m)) {
            for (int n = lane; n < 2 * BN; n += 32) {
                zr[n] = fr[n];
                zi[n] = fi[n];
            }
            __syncwarp();
            for (int j = lane; j < B; j += 32) {
                const float d0 = zr[j], d1 = zr[BN + j], c0 = zi[j], c1 = zi[BN + j];
                fr[j] = (d0 + d1) * scale;
                fi[j] = (c0 + c1) * scale;
                fr[S - 1 - j] = (d0 - d1) * scale;
                fi[S - 1 - j] = (c0 - c1) * scale;
            }
            __syncwarp();
            continue;
        }
        // Fc[p][f][m][t][j]: cosine coefficient k = 2j + t at t BH + j
        const float* xa = Fc + (size_t)row * (2 * BH);
        const float* xb = xa + (size_t)nrows * (2 * BH);
        float2 v[RM];
#pragma unroll
        for (int i = 0; i < RM; ++i) {
            const int k = lane + 32 * i;
            if (k < S) {
                const int r = S - k;
                const int ok = (k & 1) * BH + (k >> 1), orr = (r & 1) * BH + (r >> 1);
                const float ak = (k < B) ? xa[ok] : 0.f, bk = (k < B) ? xb[ok] : 0.f;
                const float ar = (k > 0 && r < B) ? xa[orr] : 0.f, br = (k > 0 && r < B) ? xb[orr] : 0.f;
                const float wr = ak + br, wi = bk - ar;
                const float2 d = twD[k];
                v[i] = cmulf(make_float2(wr * d.x - wi * d.y, wr * d.y + wi * d.x), chirp(t, k, 1.f));
            } else {
                v[i] = make_float2(0.f, 0.f);
            }
        }
        czt_warp<RM>(v, t, zr, zi, S, 1.f);
        const bool odd = m & 1;
        for (int q = lane; q < S; q += 32) {
            const int src = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
            const float gq = odd ? sn[q] * scale : scale;
            fr[q] = zr[pad32(src)] * gq;
            fi[q] = zi[pad32(src)] * gq;
        }
        __syncwarp();  // the spectrum is read before the next row's transform overwrites it
    }
}

// DFT with sign +1 over the orders for kLat latitudes (two real output rows per warp): the
// order-major input arrives as float4 runs of 4 latitudes into a latitude-major tile, which the
// warps' spectrum rows reuse once every warp holds its inputs.
template <int RM>
__global__ void __launch_bounds__(kT) k_czt_rows_inv(const float* __restrict__ F, float* __restrict__ grid, int N,
                                                     int B, int SX, const CztTabs g,
                                                     const int64_t* __restrict__ gmap) {
    using Sh = CztShape<RM>;
    constexpr int PSA = Sh::PSA;
    const int S = 2 * B;
    const int TS = (B + 1) | 1;  // odd tile row stride
    extern __shared__ __align__(16) float fsm[];
    const int U = max(2 * kW * PSA, 2 * kLat * TS);
    float* tr = fsm;
    float* ti = tr + kLat * TS;
    float* spr = fsm;
    float* spi = spr + kW * PSA;
    const CztSm t = czt_load<RM>(fsm + ((U + 3) & ~3), g);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NT = SX / kLat;
    const int f = blockIdx.x / NT, th0 = (blockIdx.x - f * NT) * kLat;
    const size_t plane = (size_t)N * B * SX;
    for (int e = threadIdx.x; e < B * (kLat / 4); e += kT) {
        const int m = e / (kLat / 4), q = 4 * (e - m * (kLat / 4));
        const size_t o = ((size_t)f * B + m) * SX + th0 + q;
        const float4 a = *reinterpret_cast<const float4*>(F + o);
        const float4 b = *reinterpret_cast<const float4*>(F + plane + o);
        float* pr = tr + q * TS + m;
        float* pi = ti + q * TS + m;
        pr[0] = a.x, pr[TS] = a.y, pr[2 * TS] = a.z, pr[3 * TS] = a.w;
        pi[0] = b.x, pi[TS] = b.y, pi[2 * TS] = b.z, pi[3 * TS] = b.w;
    }
    __syncthreads();
    const int a = 2 * warp, b = a + 1;
    const bool live = th0 + a < S;
    float2 v[RM];
#pragma unroll
    for (int i = 0; i < RM; ++i) {
        const int n = lane + 32 * i;
        float ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
        if (live && n < S) {
            if (n < B) {
                ar = tr[a * TS + n], br = tr[b * TS + n];
                ai = n == 0 ? 0.f : ti[a * TS + n];
                bi = n == 0 ? 0.f : ti[b * TS + n];
            } else if (n > B) {  // Hermitian rows: order n - S
                const int s = S - n;
                ar = tr[a * TS + s], br = tr[b * TS + s];
                ai = -ti[a * TS + s], bi = -ti[b * TS + s];
            }
        }
        v[i] = (live && n < S) ? cmulf(make_float2(ar - bi, ai + br), chirp(t, n, 1.f)) : make_float2(0.f, 0.f);
    }
    __syncthreads();  // the tile is dead: the warps' spectrum rows overwrite it
    if (!live) return;
    float* zr = spr + warp * PSA;
    float* zi = spi + warp * PSA;
    czt_warp<RM>(v, t, zr, zi, S, 1.f);
    float* ga = grid + (gmap ? gmap[f] : (int64_t)f * S * S) + (size_t)(th0 + a) * S;
    for (int k2 = lane; k2 < B; k2 += 32) {  // S / 2 pairs per row; rows start 8-byte aligned
        const int k = 2 * k2;
        reinterpret_cast<float2*>(ga)[k2] = make_float2(zr[pad32(k)], zr[pad32(k + 1)]);
        reinterpret_cast<float2*>(ga + S)[k2] = make_float2(zi[pad32(k)], zi[pad32(k + 1)]);
    }
}

template <int RM>
size_t czt_smem(int which, int B) {
    constexpr int M = 32 * RM, PSA = CztShape<RM>::PSA;
    const int S = 2 * B;
    const size_t tabs = sizeof(float) * 2 * ((size_t)twtab_len(M) + 2 * M + S);
    const size_t spec = sizeof(float) * 2 * kW * PSA;
    switch (which) {
        case 0: return spec + tabs;
        case 1: return spec + tabs + sizeof(float) * 2 * S + sizeof(float2) * B;
        case 2: return spec + tabs + sizeof(float) * (S + 2) + sizeof(float2) * S;
        default: {
            const int TS = (B + 1) | 1;
            const size_t U = (size_t)std::max(2 * kW * PSA, 2 * kLat * TS);
            return sizeof(float) * ((U + 3) & ~(size_t)3) + tabs;
        }
    }
}

// Grid of a persistent stage kernel: the CTAs that fit on the GPU at once, at most `blocks`
// (resident CTAs cached per device, kernel and shared-memory size).
int grid_for(const void* fn, size_t smem, long long blocks, int* g) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void*, size_t>, int> cache;
    int dev = 0;
    S2G_CUDA(cudaGetDevice(&dev));
    const auto key = std::make_tuple(dev, fn, smem);
    int per_gpu = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) per_gpu = it->second;
    }
    if (!per_gpu) {
        int occ = 0, nsm = 0;
        S2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kT, smem));
        S2G_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        per_gpu = std::max(occ, 1) * nsm;
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = per_gpu;
    }
    *g = (int)std::max<long long>(1, std::min<long long>(blocks, per_gpu));
    return S2G_OK;
}

template <int RM>
int czt_launch(int which, const CztTabs& g, const void* in, void* out, int N, float scale, const int64_t* gmap,
               cudaStream_t st) {
    const int B = g.B;
    const SplitLayout L = split_layout(B);
    const size_t smem = czt_smem<RM>(which, B);
    const int nrows = N * B;
    const void* fn = which == 0 ? (const void*)k_czt_rows_fwd<RM>
                   : which == 1 ? (const void*)k_czt_dct_fwd<RM>
                   : which == 2 ? (const void*)k_czt_dct_inv<RM> : (const void*)k_czt_rows_inv<RM>;
    S2G_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long tiles = (long long)N * (L.SX / kLat);
    if (which == 0) {
        ProfScope ps_("rows_fwd_czt", st);
        k_czt_rows_fwd<RM><<<(unsigned)tiles, kT, smem, st>>>((const float*)in, (float*)out, N, B, L.SX, scale, g,
                                                              gmap);
    } else if (which == 1) {
        int grid = 0;
        S2G_TRY(grid_for(fn, smem, (nrows + kW - 1) / kW, &grid));
        ProfScope ps_("dct_fwd_czt", st);
        k_czt_dct_fwd<RM><<<grid, kT, smem, st>>>((float*)in, (float*)out, nrows, B, L.BH, L.BN, L.SX, g);
    } else if (which == 2) {
        int grid = 0;
        S2G_TRY(grid_for(fn, smem, (nrows + kW - 1) / kW, &grid));
        ProfScope ps_("dct_inv_czt", st);
        k_czt_dct_inv<RM><<<grid, kT, smem, st>>>((const float*)in, (float*)out, nrows, B, L.BH, L.BN, L.SX, scale,
                                                  g);
    } else {
        ProfScope ps_("rows_inv_czt", st);
        k_czt_rows_inv<RM><<<(unsigned)tiles, kT, smem, st>>>((const float*)in, (float*)out, N, B, L.SX, g, gmap);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

}  // namespace

// Bandwidths 17 .. 256 whose length 2B no warp FFT takes: the warp FFTs run lengths 32 R for
// R = 1 .. 15 (any R up to 15) and the powers of two up to 64.
bool split_czt(int bw) {
    if (bw < 17 || bw > 256) return false;
    if ((bw & (bw - 1)) == 0) return false;
    return !(bw % 16 == 0 && bw / 16 <= 15);
}

int czt_len(int bw) {
    int M = 128;
    while (M < 4 * bw - 1) M <<= 1;
    return M;
}

SplitLayout split_layout(int bw) {
    SplitLayout L;
    if (split_czt(bw)) {
        L.BN = (bw + 7) & ~7;
        L.BH = ((bw + 1) / 2 + 7) & ~7;
        L.SX = 2 * L.BN;
    } else {
        L.BN = bw;
        L.BH = bw / 2;
        L.SX = 2 * bw;
    }
    return L;
}

int czt_build_tables(int bw, float2** d_h, float2** d_K, float2** d_tw) {
    const int S = 2 * bw, M = czt_len(bw);
    const double pi = 3.14159265358979323846;
    std::vector<double> hr(S), hi(S);
    for (int n = 0; n < S; ++n) {
        const long long r = ((long long)n * n) % (2 * S);  // exp(-i pi n^2 / S) depends on n^2 mod 2S
        hr[n] = cos(pi * (double)r / S);
        hi[n] = -sin(pi * (double)r / S);
    }
    // b_j = conj(c_|j|), j mod M; K_k = (1/M) sum_j b_j exp(-2 pi i j k / M)
    std::vector<double> rr(M), ri(M);
    for (int q = 0; q < M; ++q) {
        rr[q] = cos(2.0 * pi * q / M);
        ri[q] = -sin(2.0 * pi * q / M);
    }
    std::vector<float2> h(S), K(M), tw(M);
    for (int n = 0; n < S; ++n) h[n] = make_float2((float)hr[n], (float)hi[n]);
    for (int k = 0; k < M; ++k) {
        double sr = 0.0, si = 0.0;
        for (int j = -(S - 1); j < S; ++j) {
            const int a = j < 0 ? -j : j;
            const double br = hr[a], bi = -hi[a];
            const int q = (int)(((long long)((j + M) % M) * k) % M);
            sr += br * rr[q] - bi * ri[q];
            si += br * ri[q] + bi * rr[q];
        }
        K[k] = make_float2((float)(sr / M), (float)(si / M));
        tw[k] = make_float2((float)rr[k], (float)-ri[k]);  // exp(+2 pi i k / M)
    }
    *d_h = *d_K = *d_tw = nullptr;
    cudaError_t e = cudaMalloc(d_h, sizeof(float2) * S);
    if (e == cudaSuccess) e = cudaMalloc(d_K, sizeof(float2) * M);
    if (e == cudaSuccess) e = cudaMalloc(d_tw, sizeof(float2) * M);
    if (e == cudaSuccess) e = cudaMemcpy(*d_h, h.data(), sizeof(float2) * S, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(*d_K, K.data(), sizeof(float2) * M, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(*d_tw, tw.data(), sizeof(float2) * M, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(*d_h);
        cudaFree(*d_K);
        cudaFree(*d_tw);
        *d_h = *d_K = *d_tw = nullptr;
        return cuda_fail(e, "chirp-z tables");
    }
    return S2G_OK;
}

int czt_stage(int which, const CztTabs& g, const void* in, void* out, int N, float scale, const int64_t* gmap,
              cudaStream_t st) {
    if (which < 0 || which > 3) return fail(S2G_ERR_ARG, "stage %d", which);
    switch (g.M) {
        case 128: return czt_launch<4>(which, g, in, out, N, scale, gmap, st);
        case 256: return czt_launch<8>(which, g, in, out, N, scale, gmap, st);
        case 512: return czt_launch<16>(which, g, in, out, N, scale, gmap, st);
        case 1024: return czt_launch<32>(which, g, in, out, N, scale, gmap, st);
        default: return fail(S2G_ERR_UNSUPPORTED, "no chirp-z length %d", g.M);
    }
}

}  // namespace s2g
