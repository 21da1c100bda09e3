// sht_fp64.cu -- plain FP64 seminaive SHT on the GPU (the parity path).
//
// Forward (FSTSemiMemo, FST_semi_memo.c:68-202):
//   k_rows_fwd : DFT along phi of every latitude row, scaled by sqrt(2 pi)/2bw and stored
//                transposed X[f][m][theta]          (FST_semi_memo.c:81-90)
//   k_fwd_dlt  : per (order row, group of functions): weights, REDFT10 of length 2bw,
//                normalisation, then the seminaive triangular contraction against the
//                cosine-series table (DLTSemi, seminaive.c:153-198) or, for orders >= cutoff,
//                the naive sampled-Pml product (DLTNaive, naive.c:34-59); writes the
//                coefficients at IndexOfHarmonicCoeff positions (+ REAL mirror, :131-145)
// Inverse (InvFSTSemiMemo, FST_semi_memo.c:228-351):
//   k_inv_dlt  : per (order row, group): transposed contraction (InvDLTSemi, seminaive.c:56-115)
//                or naive synthesis (InvDLTNaive, naive.c:78-96), REDFT01, sin(theta) for odd m,
//                sign for odd negative rows, 1/sqrt(2 pi)  -> Fourier rows F[f][m][theta]
//   k_rows_inv : per latitude, DFT with sign +1 over m (the reference's swapped re/im forward
//                DFT, FST_semi_memo.c:350) -> samples
// The real-field fast path (no imaginary samples) packs two latitudes into one complex DFT.
#include <math.h>

#include <map>
#include <mutex>
#include <vector>

#include "rows.cuh"
#include "s2g_common.cuh"
#include "s2g_internal.h"

namespace s2g {

static constexpr double kPi = 3.14159265358979323846;
static constexpr double kSqrtHalf = 0.70710678118654752440;

// ------------------------------------------------------------------------------------
__global__ void k_twiddles(int n, double2* full, double2* quarter) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double s, c;
    if (full) {
        sincospi(2.0 * (double)k / (double)n, &s, &c);
        full[k] = make_double2(c, s);
    }
    if (quarter) {
        sincospi((double)k / (2.0 * (double)n), &s, &c);
        quarter[k] = make_double2(c, s);
    }
}

int twiddles_device(int n, double2* d_full, double2* d_quarter, cudaStream_t st) {
    {
        ProfScope ps_("twiddles", st);
        k_twiddles<<<(n + 255) / 256, 256, 0, st>>>(n, d_full, d_quarter);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

static int set_smem(const void* fn, size_t bytes) {
    // always set: the 48 KiB default covers static plus dynamic shared memory
    S2G_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return S2G_OK;
}

// ------------------------------------------------------------------------------------
struct FwdDlt {
    const double* Xr;
    const double* Xi;      // may be null (imaginary input zero)
    int xrows;             // rows per function in X
    double* rc;
    double* ic;            // may be null (imaginary output not wanted)
    int64_t c_stride;      // doubles between functions in rc/ic
    const double* tab;
    const int64_t* off;    // null: `tab` is the table of order m1d
    const double* w;
    const double2* twS;
    const double2* twD;
    int B, S, cutoff, nfunc, G;
    Len L;                 // DFT length S (with Bluestein tables when S is not a power of two)
    int complex_rows;      // rows 0..B-1 and B+1..S-1 (COMPLEX) else 0..B-1
    int real_mirror;       // fill f(l,-m) = (-1)^m conj f(l,m)
    int one_d, m1d;        // single order from row 0 of X, output contiguous result[l-m]
};

__global__ void k_fwd_dlt(FwdDlt p) {
    extern __shared__ double sm[];
    const int B = p.B, S = p.S;
    const Len L = p.L;
    const int Ge = (p.G + 1) & ~1;
    int row, m;
    bool neg = false;
    if (p.one_d) {
        row = 0;
        m = p.m1d;
    } else {
        row = blockIdx.x;
        if (p.complex_rows && row >= B) row += 1;
        neg = row > B;
        m = neg ? S - row : row;
    }
    const bool semi = m < p.cutoff;
    const double sgn = (neg && (row & 1)) ? -1.0 : 1.0;
    const int f0 = blockIdx.y * p.G;

    double* zr = sm;
    double* zi = zr + S;
    double* tmp = zi + S;
    double* cbuf = tmp + L.tmp_len();
    const int clen = semi ? B : S;  // per function per part
    double* cre = cbuf;                          // [Ge][clen]
    double* cim = cbuf + (size_t)Ge * clen;      // [Ge][clen]
    const double* w = p.w + ((semi && (m & 1)) ? S : 0);
    const int xrow = p.one_d ? 0 : row;

    for (int g = 0; g < Ge; ++g) {
        const int f = f0 + g;
        const bool live = (g < p.G) && (f < p.nfunc);
        const double* xr = p.Xr + ((size_t)f * p.xrows + xrow) * S;
        const double* xi = p.Xi ? p.Xi + ((size_t)f * p.xrows + xrow) * S : nullptr;
        if (!semi) {
            for (int q = threadIdx.x; q < S; q += blockDim.x) {
                cre[(size_t)g * S + q] = live ? xr[q] * w[q] : 0.0;
                cim[(size_t)g * S + q] = (live && xi) ? xi[q] * w[q] : 0.0;
            }
            continue;
        }
        if (!live) {
            for (int k = threadIdx.x; k < B; k += blockDim.x) {
                cre[(size_t)g * B + k] = 0.0;
                cim[(size_t)g * B + k] = 0.0;
            }
            continue;
        }
        // weighted data, Makhoul reorder (v[j] = x[2j], v[S-1-j] = x[2j+1]) into bit-reversed slots
        for (int q = threadIdx.x; q < S; q += blockDim.x) {
            const int d = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
            zr[L.pos(d)] = xr[q] * w[q];
            zi[L.pos(d)] = xi ? xi[q] * w[q] : 0.0;
        }
        __syncthreads();
        block_dft<double, double2>(zr, zi, L, 1, S, p.twS, -1.0, tmp);
        // REDFT10 of both parts, c[0] *= sqrt(1/2), c *= 1/sqrt(2S)   (seminaive.c:170-176)
        const double nrm = 1.0 / sqrt(2.0 * S);
        for (int k = threadIdx.x; k < B; k += blockDim.x) {
            const int kk = (k == 0) ? 0 : S - k;
            const double ar = zr[k], ai = zi[k], br = zr[kk], bi = zi[kk];
            const double c = p.twD[k].x, s = p.twD[k].y;
            double va = (ar + br) * c + (ai - bi) * s;
            double vb = (ai + bi) * c - (ar - br) * s;
            const double f = (k == 0) ? kSqrtHalf * nrm : nrm;
            cre[(size_t)g * B + k] = va * f;
            cim[(size_t)g * B + k] = vb * f;
        }
        __syncthreads();
    }
    __syncthreads();

    const int nrows = B - m;
    const int nch = Ge / 2;
    const int64_t tab0 = p.off ? p.off[m] : 0;
    const double* tab = p.tab + tab0;
    for (int task = threadIdx.x; task < nrows * nch; task += blockDim.x) {
        const int li = task % nrows, ch = task / nrows;
        const int l = m + li;
        const int g0 = 2 * ch, g1 = g0 + 1;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        if (semi) {
            const int t = li & 1;
            const int rs = row_size(m, l);
            const double* trow = tab + table_offset(m, l);
            const double* c0 = cre + (size_t)g0 * B + t;
            const double* c1 = cim + (size_t)g0 * B + t;
            const double* c2 = cre + (size_t)g1 * B + t;
            const double* c3 = cim + (size_t)g1 * B + t;
            for (int j = 0; j < rs; ++j) {
                const double v = trow[j];
                a0 = fma(v, c0[2 * j], a0);
                a1 = fma(v, c1[2 * j], a1);
                a2 = fma(v, c2[2 * j], a2);
                a3 = fma(v, c3[2 * j], a3);
            }
        } else {
            const double* prow = tab + (size_t)li * S;
            const double* c0 = cre + (size_t)g0 * S;
            const double* c1 = cim + (size_t)g0 * S;
            const double* c2 = cre + (size_t)g1 * S;
            const double* c3 = cim + (size_t)g1 * S;
            for (int j = 0; j < S; ++j) {
                const double v = prow[j];
                a0 = fma(c0[j], v, a0);
                a1 = fma(c1[j], v, a1);
                a2 = fma(c2[j], v, a2);
                a3 = fma(c3[j], v, a3);
            }
        }
        for (int h = 0; h < 2; ++h) {
            const int g = g0 + h;
            const int f = f0 + g;
            if (g >= p.G || f >= p.nfunc) continue;
            const double vr = sgn * (h ? a2 : a0), vi = sgn * (h ? a3 : a1);
            double* rc = p.rc + (size_t)f * p.c_stride;
            double* ic = p.ic ? p.ic + (size_t)f * p.c_stride : nullptr;
            const int idx = p.one_d ? li : index_of_harmonic_coeff(neg ? -m : m, l, B);
            rc[idx] = vr;
            if (ic) ic[idx] = vi;
            if (p.real_mirror && m > 0) {
                const int i2 = index_of_harmonic_coeff(-m, l, B);
                const double s = (m & 1) ? -1.0 : 1.0;
                rc[i2] = s * vr;
                if (ic) ic[i2] = -s * vi;
            }
        }
    }
}

// ------------------------------------------------------------------------------------
struct InvDlt {
    const double* rc;
    const double* ic;      // may be null (zero)
    int64_t c_stride;
    double* Fr;
    double* Fi;
    int frows;
    const double* tab;     // transposed cosine tables / sampled Pml
    const int64_t* off;    // null: `tab` is the table of order m1d
    const double* sinv;
    const double2* twS;
    const double2* twD;
    int B, S, cutoff, nfunc, G;
    Len L;                 // DFT length S (with Bluestein tables when S is not a power of two)
    int complex_rows;
    int one_d, m1d;
    double out_scale;
};

__global__ void k_inv_dlt(InvDlt p) {
    extern __shared__ double sm[];
    const int B = p.B, S = p.S;
    const Len L = p.L;
    const int Ge = (p.G + 1) & ~1;
    int row, m;
    bool neg = false;
    if (p.one_d) {
        row = 0;
        m = p.m1d;
    } else {
        row = blockIdx.x;
        if (p.complex_rows && row >= B) row += 1;
        neg = row > B;
        m = neg ? S - row : row;
    }
    const bool semi = m < p.cutoff;
    const double sgn = ((neg && (row & 1)) ? -1.0 : 1.0) * p.out_scale;
    const int f0 = blockIdx.y * p.G;
    const int nl = B - m;

    double* zr = sm;
    double* zi = zr + S;
    double* tmp = zi + S;
    double* are = tmp + L.tmp_len();              // [Ge][B]
    double* aim = are + (size_t)Ge * B;           // [Ge][B]
    double* fre = aim + (size_t)Ge * B;           // [Ge][B]  (semi only)
    double* fim = fre + (size_t)Ge * B;
    int* toff = (int*)(fim + (size_t)Ge * B);     // B + 1 ints
    int* wtot = toff + B + 1;                     // 32 ints

    for (int t = threadIdx.x; t < Ge * nl; t += blockDim.x) {
        const int g = t / nl, li = t - g * nl;
        const int f = f0 + g;
        double vr = 0.0, vi = 0.0;
        if (g < p.G && f < p.nfunc) {
            const int idx = p.one_d ? li : index_of_harmonic_coeff(neg ? -m : m, m + li, B);
            vr = p.rc[(size_t)f * p.c_stride + idx];
            vi = p.ic ? p.ic[(size_t)f * p.c_stride + idx] : 0.0;
        }
        are[(size_t)g * B + li] = vr;
        aim[(size_t)g * B + li] = vi;
    }
    const int64_t tab0 = p.off ? p.off[m] : 0;
    const double* tab = p.tab + tab0;
    const int nch = Ge / 2;

    if (!semi) {
        __syncthreads();
        // naive synthesis: F[q] = sum_l a[l-m] P(m,l)(x_q)
        for (int task = threadIdx.x; task < S * nch; task += blockDim.x) {
            const int q = task % S, ch = task / S;
            const int g0 = 2 * ch;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            for (int li = 0; li < nl; ++li) {
                const double v = tab[(size_t)li * S + q];
                a0 = fma(are[(size_t)g0 * B + li], v, a0);
                a1 = fma(aim[(size_t)g0 * B + li], v, a1);
                a2 = fma(are[(size_t)(g0 + 1) * B + li], v, a2);
                a3 = fma(aim[(size_t)(g0 + 1) * B + li], v, a3);
            }
            for (int h = 0; h < 2; ++h) {
                const int f = f0 + g0 + h;
                if (g0 + h >= p.G || f >= p.nfunc) continue;
                const size_t o = ((size_t)f * p.frows + (p.one_d ? 0 : row)) * S + q;
                p.Fr[o] = sgn * (h ? a2 : a0);
                if (p.Fi) p.Fi[o] = sgn * (h ? a3 : a1);
            }
        }
        return;
    }

    // transposed-table row offsets: exclusive scan of Transpose_RowSize(i, m, B)
    for (int i = threadIdx.x; i < B; i += blockDim.x) toff[i] = transpose_row_size(i, m, B);
    __syncthreads();
    block_exclusive_scan(toff, B, wtot);

    const double scale = 0.5 / sqrt((double)B);
    const double scale0 = 1.0 / sqrt((double)S);
    for (int task = threadIdx.x; task < B * nch; task += blockDim.x) {
        const int i = task % B, ch = task / B;
        const int g0 = 2 * ch;
        const int rs = transpose_row_size(i, m, B);
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        if (rs > 0) {
            const int base = trans_first_l(i, m) - m;
            const double* trow = tab + toff[i];
            const double* c0 = are + (size_t)g0 * B + base;
            const double* c1 = aim + (size_t)g0 * B + base;
            const double* c2 = are + (size_t)(g0 + 1) * B + base;
            const double* c3 = aim + (size_t)(g0 + 1) * B + base;
            for (int j = 0; j < rs; ++j) {
                const double v = trow[j];
                a0 = fma(c0[2 * j], v, a0);
                a1 = fma(c1[2 * j], v, a1);
                a2 = fma(c2[2 * j], v, a2);
                a3 = fma(c3[2 * j], v, a3);
            }
        }
        const double s = (i == 0) ? scale0 : scale;
        fre[(size_t)g0 * B + i] = a0 * s;
        fim[(size_t)g0 * B + i] = a1 * s;
        fre[(size_t)(g0 + 1) * B + i] = a2 * s;
        fim[(size_t)(g0 + 1) * B + i] = a3 * s;
    }
    __syncthreads();

    // REDFT01 of (fre + i fim) per function, zero-padded from B to S   (seminaive.c:107)
    for (int g = 0; g < Ge; ++g) {
        const int f = f0 + g;
        if (g >= p.G || f >= p.nfunc) break;
        const double* xa = fre + (size_t)g * B;
        const double* xb = fim + (size_t)g * B;
        for (int k = threadIdx.x; k < S; k += blockDim.x) {
            const double ak = (k < B) ? xa[k] : 0.0, bk = (k < B) ? xb[k] : 0.0;
            const int r = S - k;  // X[S] = 0
            const double ar = (k > 0 && r < B) ? xa[r] : 0.0, br = (k > 0 && r < B) ? xb[r] : 0.0;
            const double wr = ak + br, wi = bk - ar;
            const double c = p.twD[k].x, s = p.twD[k].y;
            zr[L.pos(k)] = wr * c - wi * s;
            zi[L.pos(k)] = wr * s + wi * c;
        }
        __syncthreads();
        block_dft<double, double2>(zr, zi, L, 1, S, p.twS, 1.0, tmp);
        const size_t ob = ((size_t)f * p.frows + (p.one_d ? 0 : row)) * S;
        for (int q = threadIdx.x; q < S; q += blockDim.x) {
            const int src = (q & 1) ? S - 1 - (q >> 1) : (q >> 1);
            double vr = zr[src], vi = zi[src];
            if (m & 1) {
                vr *= p.sinv[q];
                vi *= p.sinv[q];
            }
            p.Fr[ob + q] = sgn * vr;
            if (p.Fi) p.Fi[ob + q] = sgn * vi;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------
// FZT row sums (FST_semi_memo.c:386-398): X0[f][theta] = sqrt(2 pi)/S * sum_phi data
__global__ void k_rowsum(const double* __restrict__ rdata, const double* __restrict__ idata, double* Xr, double* Xi,
                         int S, double scale) {
    const int f = blockIdx.y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + warp;
    if (row >= S) return;
    const size_t b = (size_t)f * S * S + (size_t)row * S;
    double sr = 0.0, si = 0.0;
    for (int k = lane; k < S; k += 32) {
        sr += rdata[b + k];
        if (idata) si += idata[b + k];
    }
    for (int o = 16; o; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
        Xr[(size_t)f * S + row] = sr * scale;
        Xi[(size_t)f * S + row] = si * scale;
    }
}

// TransMult (util.c:68-103): out = (filter (x) data) * sqrt(4 pi / (2l+1)), with the
// reference's ComplexMult imaginary part x*v - y*u (util.c:23-27).
__global__ void k_transmult(const double* __restrict__ rd, const double* __restrict__ id,
                            const double* __restrict__ rf, const double* __restrict__ iff, double* rr, double* ir,
                            int B) {
    const int f = blockIdx.y;
    const int m = (int)blockIdx.x - (B - 1);
    const int am = m < 0 ? -m : m;
    const size_t cb = (size_t)f * B * B;
    for (int l = am + threadIdx.x; l < B; l += blockDim.x) {
        const int idx = index_of_harmonic_coeff(m, l, B);
        const double x = rf[(size_t)f * B + l], y = iff[(size_t)f * B + l];
        const double u = rd[cb + idx], v = id[cb + idx];
        const double s = sqrt(4.0 * kPi / (2.0 * l + 1.0));
        rr[cb + idx] = (x * u - y * v) * s;
        ir[cb + idx] = (x * v - y * u) * s;
    }
}

// ------------------------------------------------------------------------------------
// Host-side launchers.

static int rows_per_cta(int S) {
    int R = 4096 / S;
    if (R < 1) R = 1;
    if (R > 32) R = 32;
    return R;
}

// DFT length n with, when n is not a power of two, Bluestein tables on the current device
// (built once per device and n, host arithmetic in long double; see Len and block_dft).
static int dft_len(int n, Len* out) {
    Len L = make_len(n);
    if (L.pow2() || n < 2) {
        *out = L;
        return S2G_OK;
    }
    int dev = 0;
    S2G_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<std::pair<int, int>, Len> cache;
    std::lock_guard<std::mutex> lk(mu);
    const auto it = cache.find({dev, n});
    if (it != cache.end()) {
        *out = it->second;
        return S2G_OK;
    }
    int M = 1, lM = 0;
    while (M < 2 * n - 1) M <<= 1, ++lM;
    const long double pi = 3.141592653589793238462643383279502884L;
    std::vector<double2> h(n), tab((size_t)n + 2 * (size_t)M + M / 2);
    std::vector<long double> rc(M), rs(M);
    for (int k = 0; k < M; ++k) rc[k] = cosl(2 * pi * k / M), rs[k] = sinl(2 * pi * k / M);
    std::vector<long double> hc(n), hsn(n);  // exp(-i pi j^2 / n), angle reduced exactly: j^2 mod 2n
    for (int j = 0; j < n; ++j) {
        const long double a = pi * (long double)(((long long)j * j) % (2LL * n)) / n;
        hc[j] = cosl(a), hsn[j] = -sinl(a);
        tab[j] = make_double2((double)hc[j], (double)hsn[j]);
    }
    for (int sg = 0; sg < 2; ++sg) {  // sg 0: sign -1 (h = chirp), 1: sign +1 (h = conj chirp)
        // kernel b[m] = conj(h_m) at m and M - m (|m| < n); its DFT (sign -1) / M, bit-reversed order
        const long double bi_sign = sg == 0 ? -1.0L : 1.0L;  // imaginary part of conj(h) = -(+-hsn)
        for (int k = 0; k < M; ++k) {
            long double sr = 0, si = 0;
            for (int m = -(n - 1); m <= n - 1; ++m) {
                const int am = m < 0 ? -m : m, pm = m < 0 ? M + m : m;
                const long double br = hc[am], bim = bi_sign * hsn[am];
                const int idx = (int)(((long long)pm * k) % M);
                const long double c = rc[idx], s_ = -rs[idx];
                sr += br * c - bim * s_;
                si += br * s_ + bim * c;
            }
            int rk = 0;
            for (int b = 0; b < lM; ++b) rk |= ((k >> b) & 1) << (lM - 1 - b);
            tab[(size_t)n + (size_t)sg * M + rk] = make_double2((double)(sr / M), (double)(si / M));
        }
    }
    for (int k = 0; k < M / 2; ++k) tab[(size_t)n + 2 * (size_t)M + k] = make_double2((double)rc[k], (double)rs[k]);
    double2* d = nullptr;
    S2G_CUDA(cudaMalloc(&d, sizeof(double2) * tab.size()));
    const cudaError_t e = cudaMemcpy(d, tab.data(), sizeof(double2) * tab.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "cudaMemcpy");
    }
    L.M = M;
    L.logM = lM;
    L.chirp = d;
    L.bfwd = d + n;
    L.binv = d + n + M;
    L.twM = d + n + 2 * M;
    cache[{dev, n}] = L;
    *out = L;
    return S2G_OK;
}

static size_t rows_smem(const Len& L, int R) {
    return ((size_t)2 * R * (L.n + 1) + L.tmp_len()) * sizeof(double);
}

// `given`: the geometry of length 2B (with its Bluestein tables) built by the caller; null looks
// it up (and builds it on first use) with dft_len.
static int launch_rows_fwd(const double* rdata, const double* idata, double* Xr, double* Xi, int B, int rows_out,
                           int batch, const double2* tw, cudaStream_t st, const Len* given = nullptr) {
    const int S = 2 * B;
    Len L;
    if (given)
        L = *given;
    else
        S2G_TRY(dft_len(S, &L));
    const int R = rows_per_cta(S);
    const int lat_per = idata ? R : 2 * R;
    const size_t smem = rows_smem(L, R);
    S2G_TRY(set_smem((const void*)k_rows_fwd<double, double2>, smem));
    dim3 grid((S + lat_per - 1) / lat_per, batch);
    {
        ProfScope ps_("rows_fwd_f64", st);
        k_rows_fwd<double, double2><<<grid, 256, smem, st>>>(rdata, idata, Xr, Xi, S, L, rows_out, R, sqrt(2.0 * kPi) / S, tw);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

static int pick_group(int B, int S, bool naive, int tmp_len, size_t* smem_out, size_t per_g_extra = 0) {
    const size_t fixed = ((size_t)2 * S + tmp_len) * sizeof(double);
    const size_t per_g = (size_t)2 * (naive ? S : B) * sizeof(double) + per_g_extra;
    const size_t budget = 160 * 1024;
    int G = 8;
    while (G > 2 && fixed + (size_t)G * per_g > budget) G -= 2;
    if (fixed + (size_t)G * per_g > 220 * 1024) return 0;
    *smem_out = fixed + (size_t)G * per_g;
    return G;
}

static int launch_fwd_dlt(FwdDlt p, int nrows_grid, cudaStream_t st, const Len* given = nullptr) {
    Len L;
    if (given)
        L = *given;
    else
        S2G_TRY(dft_len(p.S, &L));
    size_t smem = 0;
    const bool any_naive = p.one_d ? (p.m1d >= p.cutoff) : (p.cutoff < p.B);
    const int G = pick_group(p.B, p.S, any_naive, L.tmp_len(), &smem);
    if (!G) return fail(S2G_ERR_UNSUPPORTED, "bandwidth %d too large for the FP64 DLT kernel", p.B);
    p.G = G;
    p.L = L;
    S2G_TRY(set_smem((const void*)k_fwd_dlt, smem));
    dim3 grid(nrows_grid, (p.nfunc + G - 1) / G);
    {
        ProfScope ps_("fwd_dlt_f64", st);
        k_fwd_dlt<<<grid, 256, smem, st>>>(p);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

static int launch_inv_dlt(InvDlt p, int nrows_grid, cudaStream_t st) {
    Len L;
    S2G_TRY(dft_len(p.S, &L));
    // are, aim, fre, fim: 4*B per function; plus B+33 ints
    const size_t fixed = ((size_t)2 * p.S + L.tmp_len()) * sizeof(double) +
                         (size_t)(p.B + 1 + 32) * sizeof(int);
    const size_t per_g = (size_t)4 * p.B * sizeof(double);
    int G = 8;
    while (G > 2 && fixed + (size_t)G * per_g > 160 * 1024) G -= 2;
    const size_t smem = fixed + (size_t)G * per_g;
    if (smem > 220 * 1024) return fail(S2G_ERR_UNSUPPORTED, "bandwidth %d too large for the FP64 DLT kernel", p.B);
    p.G = G;
    p.L = L;
    S2G_TRY(set_smem((const void*)k_inv_dlt, smem));
    dim3 grid(nrows_grid, (p.nfunc + G - 1) / G);
    {
        ProfScope ps_("inv_dlt_f64", st);
        k_inv_dlt<<<grid, 256, smem, st>>>(p);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

// Inverse row DFT over the orders of each latitude: F [batch][rows][2B] -> samples.
static int launch_rows_inv(const double* Fr, const double* Fi, int rows, int data_format, double* rdata,
                           double* idata, int B, int batch, const double2* tw, cudaStream_t st) {
    const int S = 2 * B;
    Len L;
    S2G_TRY(dft_len(S, &L));
    const int R = rows_per_cta(S);
    const int lat_per = idata ? R : 2 * R;
    const size_t smem = rows_smem(L, R);
    S2G_TRY(set_smem((const void*)k_rows_inv<double, double2>, smem));
    dim3 grid((S + lat_per - 1) / lat_per, batch);
    {
        ProfScope ps_("rows_inv_f64", st);
        k_rows_inv<double, double2><<<grid, 256, smem, st>>>(Fr, Fi, rows, data_format == COMPLEX, rdata, idata, S, L, R,
                                                              tw);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

size_t f64_work_bytes(int bw, int batch, int data_format) {
    const size_t S = 2 * (size_t)bw;
    const size_t rows = (data_format == COMPLEX) ? S : (size_t)bw;
    return 2 * (size_t)batch * rows * S * sizeof(double);
}

int fst_f64(const Tables* t, const double* rdata, const double* idata, double* rc, double* ic, int batch,
            int data_format, int cutoff, void* work, cudaStream_t st) {
    return fst_f64_len(t, nullptr, rdata, idata, rc, ic, batch, data_format, cutoff, work, st);
}

int fst_f64_len(const Tables* t, const Len* len_S, const double* rdata, const double* idata, double* rc,
                double* ic, int batch, int data_format, int cutoff, void* work, cudaStream_t st) {
    const int B = t->bw, S = 2 * B;
    const int rows = (data_format == COMPLEX) ? S : B;
    double* Xr = (double*)work;
    double* Xi = Xr + (size_t)batch * rows * S;
    // REAL data with no imaginary samples: the packed real path (imaginary part zero)
    S2G_TRY(launch_rows_fwd(rdata, idata, Xr, Xi, B, rows, batch, t->tw_S, st, len_S));
    FwdDlt p{};
    p.Xr = Xr;
    p.Xi = Xi;
    p.xrows = rows;
    p.rc = rc;
    p.ic = ic;
    p.c_stride = (int64_t)B * B;
    p.tab = t->fwd;
    p.off = t->off;
    p.w = t->weights;
    p.twS = t->tw_S;
    p.twD = t->tw_D;
    p.B = B;
    p.S = S;
    p.cutoff = cutoff;
    p.nfunc = batch;
    p.complex_rows = (data_format == COMPLEX);
    p.real_mirror = (data_format != COMPLEX);
    return launch_fwd_dlt(p, (data_format == COMPLEX) ? S - 1 : B, st, len_S);
}

int inv_fst_f64(const Tables* t, const double* rc, const double* ic, double* rdata, double* idata, int batch,
                int data_format, int cutoff, void* work, cudaStream_t st) {
    const int B = t->bw, S = 2 * B;
    const int rows = (data_format == COMPLEX) ? S : B;
    double* Fr = (double*)work;
    double* Fi = Fr + (size_t)batch * rows * S;
    InvDlt p{};
    p.rc = rc;
    p.ic = ic;
    p.c_stride = (int64_t)B * B;
    p.Fr = Fr;
    p.Fi = Fi;
    p.frows = rows;
    p.tab = t->inv;
    p.off = t->off;
    p.sinv = t->sinv;
    p.twS = t->tw_S;
    p.twD = t->tw_D;
    p.B = B;
    p.S = S;
    p.cutoff = cutoff;
    p.nfunc = batch;
    p.complex_rows = (data_format == COMPLEX);
    p.out_scale = 1.0 / sqrt(2.0 * kPi);  // FST_semi_memo.c:344-348
    S2G_TRY(launch_inv_dlt(p, (data_format == COMPLEX) ? S - 1 : B, st));
    return launch_rows_inv(Fr, Fi, rows, data_format, rdata, idata, B, batch, t->tw_S, st);
}

int fzt_f64(const Tables* t, const double* rdata, const double* idata, double* rres, double* ires, int batch,
            int data_format, void* work, cudaStream_t st) {
    const int B = t->bw, S = 2 * B;
    double* Xr = (double*)work;
    double* Xi = Xr + (size_t)batch * S;
    dim3 g1((S + 7) / 8, batch);
    {
        ProfScope ps_("rowsum_f64", st);
        k_rowsum<<<g1, 256, 0, st>>>(rdata, idata, Xr, Xi, S, sqrt(2.0 * kPi) / S);
    }
    S2G_CUDA(cudaGetLastError());
    FwdDlt p{};
    p.Xr = Xr;
    p.Xi = (data_format == COMPLEX) ? Xi : nullptr;
    p.xrows = 1;
    p.rc = rres;
    p.ic = (data_format == COMPLEX) ? ires : nullptr;
    p.c_stride = B;
    p.tab = t->fwd;   // order 0 starts at offset 0 (cutoff >= 1)
    p.off = nullptr;
    p.w = t->weights;
    p.twS = t->tw_S;
    p.twD = t->tw_D;
    p.B = B;
    p.S = S;
    p.cutoff = B;  // FZT is always seminaive (DLTSemi, FST_semi_memo.c:401)
    p.nfunc = batch;
    p.one_d = 1;
    p.m1d = 0;
    S2G_TRY(launch_fwd_dlt(p, 1, st));
    if (data_format != COMPLEX) S2G_CUDA(cudaMemsetAsync(ires, 0, sizeof(double) * (size_t)batch * B, st));
    return S2G_OK;
}

int transmult_f64(const double* rd, const double* id, const double* rf, const double* iff, double* rr, double* ir,
                  int bw, int batch, cudaStream_t st) {
    dim3 grid(2 * bw - 1, batch);
    {
        ProfScope ps_("transmult_f64", st);
        k_transmult<<<grid, 128, 0, st>>>(rd, id, rf, iff, rr, ir, bw);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

// 1-D transforms (DLTSemi etc.) on device buffers; `table` is the caller's table for order m.
int dlt_semi_f64(const double* data, int bw, int m, double* result, const double* table, const double* weights,
                 const double2* twS, const double2* twD, cudaStream_t st) {
    FwdDlt p{};
    p.Xr = data;
    p.xrows = 1;
    p.rc = result;
    p.c_stride = bw;
    p.tab = table;
    p.w = weights;
    p.twS = twS;
    p.twD = twD;
    p.B = bw;
    p.S = 2 * bw;
    p.cutoff = bw;
    p.nfunc = 1;
    p.one_d = 1;
    p.m1d = m;
    return launch_fwd_dlt(p, 1, st);
}

int dlt_naive_f64(const double* data, int bw, int m, const double* weights, double* result, const double* ptable,
                  cudaStream_t st) {
    FwdDlt p{};
    p.Xr = data;
    p.xrows = 1;
    p.rc = result;
    p.c_stride = bw;
    p.tab = ptable;
    p.w = weights;
    p.B = bw;
    p.S = 2 * bw;
    p.cutoff = 0;  // naive
    p.nfunc = 1;
    p.one_d = 1;
    p.m1d = m;
    return launch_fwd_dlt(p, 1, st);
}

int inv_dlt_semi_f64(const double* coeffs, int bw, int m, double* result, const double* ttable, const double* sinv,
                     const double2* twS, const double2* twD, cudaStream_t st) {
    InvDlt p{};
    p.rc = coeffs;
    p.c_stride = bw;
    p.Fr = result;
    p.frows = 1;
    p.tab = ttable;
    p.sinv = sinv;
    p.twS = twS;
    p.twD = twD;
    p.B = bw;
    p.S = 2 * bw;
    p.cutoff = bw;
    p.nfunc = 1;
    p.one_d = 1;
    p.m1d = m;
    p.out_scale = 1.0;
    return launch_inv_dlt(p, 1, st);
}

int inv_dlt_naive_f64(const double* coeffs, int bw, int m, double* result, const double* ptable, cudaStream_t st) {
    InvDlt p{};
    p.rc = coeffs;
    p.c_stride = bw;
    p.Fr = result;
    p.frows = 1;
    p.tab = ptable;
    p.B = bw;
    p.S = 2 * bw;
    p.cutoff = 0;
    p.nfunc = 1;
    p.one_d = 1;
    p.m1d = m;
    p.out_scale = 1.0;
    return launch_inv_dlt(p, 1, st);
}

// ------------------------------------------------------------------------------------
// On-the-fly family (FST_semi_fly.c).  The reference builds every order's Legendre table inside
// each call (GenerateCosPmlTable / GeneratePmlTable per order, FST_semi_fly.c:94-96, 257-261)
// and keeps none of them.  Here no table is written at all: each thread runs the three-term
// recurrence P(m,l) -> P(m,l+1) (pml.c:41-79: L2-normalised, seeded with P(m,m) of pmm.c:21-34)
// at its own latitude nodes and contracts every value with the data as it is produced.  The
// contraction is the reference's naive Legendre transform (DLTNaive / InvDLTNaive, naive.c:34-96,
// which FST_semi_fly.c applies to the orders >= cutoff); in exact arithmetic it equals the
// seminaive one that the reference applies below the cutoff, so every order runs naive here and
// `cutoff` changes nothing but its validation.  Latitudes theta_j and pi - theta_j share
// P(m,l) up to the sign (-1)^(l-m), so the data are folded into even and odd halves and only
// the bw northern nodes carry a recurrence.  Device memory: the row-DFT workspace, no table.
//
// Forward: one CTA per (order row, G functions).  A tile of T = 16/G degrees gives each thread
// T * 2G = 32 partial sums (degree x function x re/im) over its nodes; a warp reduce-scatter
// leaves sum `lane` on each lane, and the warps' sums are added through shared memory.
// Inverse: one thread per node and function group, summing a(l) P(m,l) over the degrees
// (even and odd degrees apart, then unfolded), no reduction.

constexpr int kFlyThreads = 256;
constexpr int kFlyMaxPasses = 8;  // nodes per thread: bw <= 8 * 256

struct FlyArgs {
    const double* Xr;     // forward: row-DFT output [f][xrows][S]
    const double* Xi;     // may be null (imaginary samples zero)
    int xrows;
    double* rc;           // forward: coefficients
    double* ic;           // may be null
    const double* crc;    // inverse: coefficients
    const double* cic;    // may be null
    int64_t c_stride;     // doubles between functions' coefficients
    double* Fr;           // inverse: [f][frows][S] latitude vectors per order
    double* Fi;           // may be null
    int frows;
    const double* w;      // forward: the 2B quadrature weights (weights.c:32-47)
    int B, S, nfunc;
    int complex_rows;     // rows 0..B-1 and B+1..S-1 (COMPLEX) else 0..B-1
    int real_mirror;      // forward: fill f(l,-m) = (-1)^m conj f(l,m)
    int one_d;            // order 0 from row 0, output result[l] (FZT)
    double out_scale;     // inverse: FST_semi_memo.c:344-348
};

__device__ __forceinline__ void fly_row(const FlyArgs& p, int& row, int& m, bool& neg) {
    neg = false;
    if (p.one_d) {
        row = 0;
        m = 0;
        return;
    }
    row = blockIdx.x;
    if (p.complex_rows && row >= p.B) row += 1;
    neg = row > p.B;
    m = neg ? p.S - row : row;
}

template <int G>
__global__ void __launch_bounds__(kFlyThreads) k_fly_fwd(FlyArgs p) {
    constexpr int T = 16 / G;  // degrees per tile (even, so l - m = d mod 2 inside a tile)
    constexpr int V = 2 * G;   // values per degree: function x (re, im)
    extern __shared__ double sm[];
    const int B = p.B, S = p.S;
    int row, m;
    bool neg;
    fly_row(p, row, m, neg);
    const double sgn = (neg && (row & 1)) ? -1.0 : 1.0;
    const int f0 = blockIdx.y * G;
    const int NT = blockDim.x, nw = NT >> 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* sv = sm;                      // [B][2 parities][V] folded weighted data
    double* an = sv + (size_t)B * 2 * V;  // [B] recurrence coefficients of this order
    double* cn = an + B;
    double* red = cn + B;                 // [nw][32]
    __shared__ double cpmm;
    if (threadIdx.x == 0) cpmm = (m == 0) ? 0.0 : pmm_const(m);
    for (int l = m + threadIdx.x; l < B; l += NT) {
        an[l] = l2_an(m, l);
        cn[l] = l2_cn(m, l);
    }
    const int xrow = p.one_d ? 0 : row;
    for (int i = threadIdx.x; i < B * G; i += NT) {
        const int j = i % B, g = i / B, f = f0 + g;
        double er = 0.0, ei = 0.0, orr = 0.0, oi = 0.0;
        if (f < p.nfunc) {
            const size_t base = ((size_t)f * p.xrows + xrow) * S;
            const double wa = p.w[j], wb = p.w[S - 1 - j];
            const double a = p.Xr[base + j] * wa, b = p.Xr[base + S - 1 - j] * wb;
            er = a + b;
            orr = a - b;
            if (p.Xi) {
                const double c = p.Xi[base + j] * wa, d = p.Xi[base + S - 1 - j] * wb;
                ei = c + d;
                oi = c - d;
            }
        }
        double* q = sv + (size_t)j * 2 * V;
        q[2 * g] = er;
        q[2 * g + 1] = ei;
        q[V + 2 * g] = orr;
        q[V + 2 * g + 1] = oi;
    }
    __syncthreads();
    // this thread's nodes j = threadIdx.x + r * NT: x = cos(theta_j), P(m,l) and P(m,l-1)
    const int R = (B + NT - 1) / NT;
    double x[kFlyMaxPasses], pc[kFlyMaxPasses], pp[kFlyMaxPasses];
#pragma unroll
    for (int r = 0; r < kFlyMaxPasses; ++r) {
        x[r] = pc[r] = pp[r] = 0.0;
        const int j = threadIdx.x + r * NT;
        if (r < R && j < B) {
            double sn, cs;
            sincospi((2.0 * j + 1.0) / (2.0 * S), &sn, &cs);
            x[r] = cs;
            pc[r] = (m == 0) ? kSqrtHalf : cpmm * pow(sn, (double)m);
        }
    }
    for (int l0 = m; l0 < B; l0 += T) {
        double acc[T * V];
#pragma unroll
        for (int k = 0; k < T * V; ++k) acc[k] = 0.0;
#pragma unroll
        for (int r = 0; r < kFlyMaxPasses; ++r) {
            const int j = threadIdx.x + r * NT;
            if (r >= R || j >= B) continue;
            const double* q = sv + (size_t)j * 2 * V;
            double se[V], so[V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                se[v] = q[v];
                so[v] = q[V + v];
            }
#pragma unroll
            for (int d = 0; d < T; ++d) {
                const int l = l0 + d;
                if (l >= B) break;
                double val = pc[r];
                if (l > m) {
                    val = an[l - 1] * (pc[r] * x[r]) + cn[l - 1] * pp[r];
                    pp[r] = pc[r];
                    pc[r] = val;
                }
#pragma unroll
                for (int v = 0; v < V; ++v) acc[d * V + v] = fma(val, (d & 1) ? so[v] : se[v], acc[d * V + v]);
            }
        }
        // reduce-scatter over the warp: after the step of width h a lane keeps the half of its
        // values whose index bit h equals its own lane bit, so lane L ends with value L
#pragma unroll
        for (int h = 16; h >= 1; h >>= 1) {
            const bool up = (lane & h) != 0;
#pragma unroll
            for (int k = 0; k < h; ++k) {
                const double send = up ? acc[k] : acc[k + h];
                const double keep = up ? acc[k + h] : acc[k];
                acc[k] = keep + __shfl_xor_sync(0xffffffffu, send, h);
            }
        }
        red[warp * 32 + lane] = acc[0];
        __syncthreads();
        if (warp == 0) {
            double tot = 0.0;
            for (int w2 = 0; w2 < nw; ++w2) tot += red[w2 * 32 + lane];
            const int d = lane / V, v = lane % V, g = v >> 1, f = f0 + g;
            const int l = l0 + d;
            if (l < B && f < p.nfunc) {
                const double val = sgn * tot;
                if (p.one_d) {
                    double* out = (v & 1) ? p.ic : p.rc;
                    if (out) out[(size_t)f * p.c_stride + l] = val;
                } else {
                    const int idx = index_of_harmonic_coeff(neg ? -m : m, l, B);
                    double* out = (v & 1) ? p.ic : p.rc;
                    if (out) {
                        out[(size_t)f * p.c_stride + idx] = val;
                        if (p.real_mirror && m > 0) {
                            // f(l,-m) = (-1)^m conj f(l,m)   (FST_semi_memo.c:131-145)
                            const double sm_ = (m & 1) ? -1.0 : 1.0;
                            out[(size_t)f * p.c_stride + index_of_harmonic_coeff(-m, l, B)] =
                                (v & 1) ? -sm_ * val : sm_ * val;
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <int G>
__global__ void __launch_bounds__(kFlyThreads) k_fly_inv(FlyArgs p) {
    constexpr int V = 2 * G;
    extern __shared__ double sm[];
    const int B = p.B, S = p.S;
    int row, m;
    bool neg;
    fly_row(p, row, m, neg);
    const double sgn = ((neg && (row & 1)) ? -1.0 : 1.0) * p.out_scale;
    const int f0 = blockIdx.y * G;
    const int NT = blockDim.x;
    const int nl = B - m;
    double* a = sm;                    // [nl][V] coefficients of this order
    double* an = a + (size_t)B * V;    // [B]
    double* cn = an + B;
    __shared__ double cpmm;
    if (threadIdx.x == 0) cpmm = (m == 0) ? 0.0 : pmm_const(m);
    for (int l = m + threadIdx.x; l < B; l += NT) {
        an[l] = l2_an(m, l);
        cn[l] = l2_cn(m, l);
    }
    for (int i = threadIdx.x; i < nl * G; i += NT) {
        const int li = i % nl, g = i / nl, f = f0 + g;
        double vr = 0.0, vi = 0.0;
        if (f < p.nfunc) {
            const int idx = p.one_d ? li : index_of_harmonic_coeff(neg ? -m : m, m + li, B);
            vr = p.crc[(size_t)f * p.c_stride + idx];
            vi = p.cic ? p.cic[(size_t)f * p.c_stride + idx] : 0.0;
        }
        a[(size_t)li * V + 2 * g] = vr;
        a[(size_t)li * V + 2 * g + 1] = vi;
    }
    __syncthreads();
    const int frow = p.one_d ? 0 : row;
    for (int j = threadIdx.x; j < B; j += NT) {
        double sn, x;
        sincospi((2.0 * j + 1.0) / (2.0 * S), &sn, &x);
        double pc = (m == 0) ? kSqrtHalf : cpmm * pow(sn, (double)m);
        double pp = 0.0;
        double ev[V], od[V];
#pragma unroll
        for (int v = 0; v < V; ++v) ev[v] = od[v] = 0.0;
        // degrees in pairs: l - m even into ev, odd into od
        for (int l = m; l < B; l += 2) {
            const double* al = a + (size_t)(l - m) * V;
#pragma unroll
            for (int v = 0; v < V; ++v) ev[v] = fma(pc, al[v], ev[v]);
            if (l + 1 >= B) break;
            double nx = an[l] * (pc * x) + cn[l] * pp;
            pp = pc;
            pc = nx;
#pragma unroll
            for (int v = 0; v < V; ++v) od[v] = fma(pc, al[V + v], od[v]);
            if (l + 2 >= B) break;
            nx = an[l + 1] * (pc * x) + cn[l + 1] * pp;
            pp = pc;
            pc = nx;
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int f = f0 + g;
            if (f >= p.nfunc) break;
            const size_t o = ((size_t)f * p.frows + frow) * S;
            p.Fr[o + j] = sgn * (ev[2 * g] + od[2 * g]);
            p.Fr[o + S - 1 - j] = sgn * (ev[2 * g] - od[2 * g]);
            if (p.Fi) {
                p.Fi[o + j] = sgn * (ev[2 * g + 1] + od[2 * g + 1]);
                p.Fi[o + S - 1 - j] = sgn * (ev[2 * g + 1] - od[2 * g + 1]);
            }
        }
    }
}

static size_t fly_fwd_smem(int B, int G) {
    return ((size_t)B * 4 * G + 2 * (size_t)B + (kFlyThreads / 32) * 32) * sizeof(double);
}
static size_t fly_inv_smem(int B, int G) { return ((size_t)B * 2 * G + 2 * (size_t)B) * sizeof(double); }

// Functions per CTA: as many (up to 4) as the batch has, within 200 KiB of shared memory.
template <typename SmemFn>
static int fly_group(int B, int nfunc, SmemFn smem) {
    int G = nfunc >= 4 ? 4 : (nfunc >= 2 ? 2 : 1);
    while (G > 1 && smem(B, G) > 200 * 1024) G /= 2;
    return G;
}

static int launch_fly(bool fwd, FlyArgs p, int nrows, cudaStream_t st) {
    if (p.B > kFlyMaxPasses * kFlyThreads)
        return fail(S2G_ERR_UNSUPPORTED, "bandwidth %d too large for the on-the-fly kernels", p.B);
    const int G = fwd ? fly_group(p.B, p.nfunc, fly_fwd_smem) : fly_group(p.B, p.nfunc, fly_inv_smem);
    const size_t smem = fwd ? fly_fwd_smem(p.B, G) : fly_inv_smem(p.B, G);
    const int nt = p.B >= kFlyThreads ? kFlyThreads : ((p.B + 31) / 32) * 32;
    dim3 grid(nrows, (p.nfunc + G - 1) / G);
    const void* fn = fwd ? (G == 4 ? (const void*)k_fly_fwd<4> : G == 2 ? (const void*)k_fly_fwd<2>
                                                                        : (const void*)k_fly_fwd<1>)
                         : (G == 4 ? (const void*)k_fly_inv<4> : G == 2 ? (const void*)k_fly_inv<2>
                                                                        : (const void*)k_fly_inv<1>);
    S2G_TRY(set_smem(fn, smem));
    {
        ProfScope ps_(fwd ? "fly_fwd_f64" : "fly_inv_f64", st);
        if (fwd) {
            if (G == 4) k_fly_fwd<4><<<grid, nt, smem, st>>>(p);
            else if (G == 2) k_fly_fwd<2><<<grid, nt, smem, st>>>(p);
            else k_fly_fwd<1><<<grid, nt, smem, st>>>(p);
        } else {
            if (G == 4) k_fly_inv<4><<<grid, nt, smem, st>>>(p);
            else if (G == 2) k_fly_inv<2><<<grid, nt, smem, st>>>(p);
            else k_fly_inv<1><<<grid, nt, smem, st>>>(p);
        }
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

int fst_f64_fly(const Tables* t, const double* rdata, const double* idata, double* rc, double* ic, int batch,
                int data_format, void* work, cudaStream_t st) {
    const int B = t->bw, S = 2 * B;
    const int rows = (data_format == COMPLEX) ? S : B;
    double* Xr = (double*)work;
    double* Xi = Xr + (size_t)batch * rows * S;
    S2G_TRY(launch_rows_fwd(rdata, idata, Xr, Xi, B, rows, batch, t->tw_S, st));
    FlyArgs p{};
    p.Xr = Xr;
    p.Xi = Xi;
    p.xrows = rows;
    p.rc = rc;
    p.ic = ic;
    p.c_stride = (int64_t)B * B;
    p.w = t->weights;
    p.B = B;
    p.S = S;
    p.nfunc = batch;
    p.complex_rows = (data_format == COMPLEX);
    p.real_mirror = (data_format != COMPLEX);
    return launch_fly(true, p, (data_format == COMPLEX) ? S - 1 : B, st);
}

int inv_fst_f64_fly(const Tables* t, const double* rc, const double* ic, double* rdata, double* idata, int batch,
                    int data_format, void* work, cudaStream_t st) {
    const int B = t->bw, S = 2 * B;
    const int rows = (data_format == COMPLEX) ? S : B;
    double* Fr = (double*)work;
    double* Fi = Fr + (size_t)batch * rows * S;
    FlyArgs p{};
    p.crc = rc;
    p.cic = ic;
    p.c_stride = (int64_t)B * B;
    p.Fr = Fr;
    p.Fi = Fi;
    p.frows = rows;
    p.B = B;
    p.S = S;
    p.nfunc = batch;
    p.complex_rows = (data_format == COMPLEX);
    p.out_scale = 1.0 / sqrt(2.0 * kPi);  // FST_semi_memo.c:344-348
    S2G_TRY(launch_fly(false, p, (data_format == COMPLEX) ? S - 1 : B, st));
    return launch_rows_inv(Fr, Fi, rows, data_format, rdata, idata, B, batch, t->tw_S, st);
}

int fzt_f64_fly(const Tables* t, const double* rdata, const double* idata, double* rres, double* ires, int batch,
                int data_format, void* work, cudaStream_t st) {
    const int B = t->bw, S = 2 * B;
    double* Xr = (double*)work;
    double* Xi = Xr + (size_t)batch * S;
    dim3 g1((S + 7) / 8, batch);
    {
        ProfScope ps_("rowsum_f64", st);
        k_rowsum<<<g1, 256, 0, st>>>(rdata, idata, Xr, Xi, S, sqrt(2.0 * kPi) / S);
    }
    S2G_CUDA(cudaGetLastError());
    FlyArgs p{};
    p.Xr = Xr;
    p.Xi = (data_format == COMPLEX) ? Xi : nullptr;
    p.xrows = 1;
    p.rc = rres;
    p.ic = (data_format == COMPLEX) ? ires : nullptr;
    p.c_stride = B;
    p.w = t->weights;
    p.B = B;
    p.S = S;
    p.nfunc = batch;
    p.one_d = 1;
    S2G_TRY(launch_fly(true, p, 1, st));
    if (data_format != COMPLEX) S2G_CUDA(cudaMemsetAsync(ires, 0, sizeof(double) * (size_t)batch * B, st));
    return S2G_OK;
}

}  // namespace s2g
