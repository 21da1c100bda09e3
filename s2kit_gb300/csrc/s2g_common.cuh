// s2g_common.cuh -- shared device helpers for the GB300 seminaive SHT library.
//
// Block-cooperative transforms in shared memory with FFTW's documented conventions
// (the reference S2kit calls FFTW3 for these; FST_semi_memo.c:81,350, seminaive.c:107,170,
// cospml.c:203-224):
//   DFT sign -1 : X[k] = sum_j x[j] exp(-2 pi i j k / n)     (unnormalised)
//   REDFT10     : Y[k] = 2 sum_j x[j] cos(pi (j+1/2) k / n)  (DCT-II)
//   REDFT01     : Y[k] = x[0] + 2 sum_{j>=1} x[j] cos(pi j (k+1/2) / n)  (DCT-III)
// Power-of-two lengths use an in-place radix-2 decimation-in-time FFT whose input is
// stored in bit-reversed order; other lengths use a direct O(n^2) DFT.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace s2g {

// ---------------------------------------------------------------------------------
// Geometry of one transform length n.
struct Len {
    int n;      // length
    int logn;   // log2(n) when n is a power of two, else -1
    // Non power-of-two n with tables (Bluestein's chirp-z transform, see block_dft): M, a power of
    // two >= 2n - 1, and device tables chirp[j] = exp(-i pi j^2 / n) (j < n), the spectra of the
    // convolution kernel for sign -1 and +1 (M entries in bit-reversed order, 1/M folded in) and
    // twM[k] = exp(2 pi i k / M) (k < M/2).  Without tables (M = 0) the DFT is direct, O(n^2).
    int M = 0, logM = -1;
    const double2* chirp = nullptr;
    const double2* bfwd = nullptr;
    const double2* binv = nullptr;
    const double2* twM = nullptr;
    __host__ __device__ bool pow2() const { return logn >= 0; }
    // reals of scratch block_dft needs (`tmp`)
    __host__ __device__ int tmp_len() const { return pow2() ? 0 : (M > 0 ? 2 * M : 2 * n); }
    // position at which input element k must be stored before block_dft()
    __device__ __forceinline__ int pos(int k) const {
        return logn > 0 ? (int)(__brev((unsigned)k) >> (32 - logn)) : k;
    }
};

inline Len make_len(int n) {
    int lg = -1;
    if (n > 0 && (n & (n - 1)) == 0) {
        lg = 0;
        while ((1 << lg) < n) ++lg;
    }
    return Len{n, lg};
}

// ---------------------------------------------------------------------------------
// In-place DFT of `cnt` sequences re/im[s*stride + k], k < L.n (input in L.pos order).
// tw[k] = (cos(2 pi k / n), sin(2 pi k / n)) for k < n.  Ends with __syncthreads().
// For non power-of-two n, `tmp` holds L.tmp_len() reals (used one sequence at a time).  With
// Bluestein tables the length-n DFT is a length-M cyclic convolution (Bluestein 1970):
//   X[k] = h_k sum_j (x_j h_j) conj(h_{k-j}),  h_j = exp(sign i pi j^2 / n),
// computed as a decimation-in-frequency FFT (natural in, bit-reversed out), a product with the
// kernel's precomputed spectrum, and a decimation-in-time inverse FFT (bit-reversed in).
template <typename T, typename T2>
__device__ void block_dft(T* re, T* im, Len L, int cnt, int stride, const T2* __restrict__ tw, T sign,
                          T* tmp) {
    const int n = L.n;
    if (L.pow2()) {
        const int hn = n >> 1;
        const int total = cnt * hn;
        const int lhn = L.logn - 1;
        for (int s = 1; s <= L.logn; ++s) {
            const int half = 1 << (s - 1);
            const int tshift = L.logn - s;  // twiddle index = j * (n / len)
            for (int t = threadIdx.x; t < total; t += blockDim.x) {
                const int seq = t >> lhn;
                const int b = t & (hn - 1);
                const int j = b & (half - 1);
                const int a0 = ((b >> (s - 1)) << s) + j;
                const int a1 = a0 + half;
                const T2 w = tw[j << tshift];
                const T c = w.x, sn = sign * w.y;
                T* r = re + (size_t)seq * stride;
                T* i = im + (size_t)seq * stride;
                const T xr = r[a1] * c - i[a1] * sn;
                const T xi = r[a1] * sn + i[a1] * c;
                const T yr = r[a0], yi = i[a0];
                r[a1] = yr - xr;
                i[a1] = yi - xi;
                r[a0] = yr + xr;
                i[a0] = yi + xi;
            }
            __syncthreads();
        }
        return;
    }
    if (L.M > 0) {
        const int M = L.M, lM = L.logM;
        T* ar = tmp;
        T* ai = tmp + M;
        const double2* bf = sign < 0 ? L.bfwd : L.binv;
        const T hs = sign < 0 ? T(1) : T(-1);  // h = chirp (sign -1) or its conjugate
        for (int seq = 0; seq < cnt; ++seq) {
            T* r = re + (size_t)seq * stride;
            T* i = im + (size_t)seq * stride;
            for (int k = threadIdx.x; k < M; k += blockDim.x) {
                T xr = 0, xi = 0;
                if (k < n) {
                    const double2 h = L.chirp[k];
                    const T hr = (T)h.x, hi = hs * (T)h.y, a = r[k], b = i[k];
                    xr = a * hr - b * hi;
                    xi = a * hi + b * hr;
                }
                ar[k] = xr;
                ai[k] = xi;
            }
            __syncthreads();
            for (int s = lM; s >= 1; --s) {  // decimation in frequency, sign -1
                const int half = 1 << (s - 1);
                for (int t = threadIdx.x; t < M / 2; t += blockDim.x) {
                    const int j = t & (half - 1);
                    const int a0 = ((t >> (s - 1)) << s) + j, a1 = a0 + half;
                    const double2 w = L.twM[j << (lM - s)];
                    const T c = (T)w.x, sn = -(T)w.y;
                    const T ur = ar[a0], ui = ai[a0], vr = ar[a1], vi = ai[a1];
                    ar[a0] = ur + vr;
                    ai[a0] = ui + vi;
                    const T dr = ur - vr, di = ui - vi;
                    ar[a1] = dr * c - di * sn;
                    ai[a1] = dr * sn + di * c;
                }
                __syncthreads();
            }
            for (int k = threadIdx.x; k < M; k += blockDim.x) {  // times the kernel's spectrum
                const double2 b = bf[k];
                const T xr = ar[k], xi = ai[k];
                ar[k] = xr * (T)b.x - xi * (T)b.y;
                ai[k] = xr * (T)b.y + xi * (T)b.x;
            }
            __syncthreads();
            for (int s = 1; s <= lM; ++s) {  // decimation in time, sign +1
                const int half = 1 << (s - 1);
                for (int t = threadIdx.x; t < M / 2; t += blockDim.x) {
                    const int j = t & (half - 1);
                    const int a0 = ((t >> (s - 1)) << s) + j, a1 = a0 + half;
                    const double2 w = L.twM[j << (lM - s)];
                    const T c = (T)w.x, sn = (T)w.y;
                    const T xr = ar[a1] * c - ai[a1] * sn, xi = ar[a1] * sn + ai[a1] * c;
                    const T yr = ar[a0], yi = ai[a0];
                    ar[a1] = yr - xr;
                    ai[a1] = yi - xi;
                    ar[a0] = yr + xr;
                    ai[a0] = yi + xi;
                }
                __syncthreads();
            }
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const double2 h = L.chirp[k];
                const T hr = (T)h.x, hi = hs * (T)h.y, cr = ar[k], ci = ai[k];
                r[k] = cr * hr - ci * hi;
                i[k] = cr * hi + ci * hr;
            }
            __syncthreads();
        }
        return;
    }
    for (int seq = 0; seq < cnt; ++seq) {
        T* r = re + (size_t)seq * stride;
        T* i = im + (size_t)seq * stride;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            T sr = 0, si = 0;
            int idx = 0;
            for (int j = 0; j < n; ++j) {
                const T2 w = tw[idx];
                const T c = w.x, sn = sign * w.y;
                sr += r[j] * c - i[j] * sn;
                si += r[j] * sn + i[j] * c;
                idx += k;
                if (idx >= n) idx -= n;
            }
            tmp[k] = sr;
            tmp[n + k] = si;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            r[k] = tmp[k];
            i[k] = tmp[n + k];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------
// Block-wide exclusive prefix sum of v[0..n) (int), in place; `warp_tot` needs 32 ints.
// Ends with __syncthreads().
__device__ inline void block_exclusive_scan(int* v, int n, int* warp_tot) {
    // serial chunks per thread, then a scan over thread totals via warps
    const int nt = blockDim.x;
    const int per = (n + nt - 1) / nt;
    const int lo = threadIdx.x * per;
    const int hi = min(n, lo + per);
    int s = 0;
    for (int k = lo; k < hi; ++k) s += v[k];
    // inclusive warp scan of s
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = s;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int nw = (nt + 31) >> 5;
        int t = lane < nw ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    int base = (wid ? warp_tot[wid - 1] : 0) + x - s;  // exclusive prefix of this thread's chunk
    for (int k = lo; k < hi; ++k) {
        int t = v[k];
        v[k] = base;
        base += t;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------------
// Index helpers (device copies of the reference's integer formulas).

// L2-normalised three-term recurrence P(m,l+1) = an(m,l) x P(m,l) + cn(m,l) P(m,l-1) and its seed
// P(m,m)(cos theta) = pmm_const(m) sin(theta)^m.
__device__ __forceinline__ double l2_an(int m, int l) {  // l2_norms.c:16-22
    return sqrt(((2.0 * l + 3.0) / (2.0 * l + 1.0)) * ((l - m + 1.0) / (l + m + 1.0))) *
           ((2.0 * l + 1.0) / (l - m + 1.0));
}

__device__ __forceinline__ double l2_cn(int m, int l) {  // l2_norms.c:28-38
    if (l == 0) return 0.0;
    return -sqrt(((2.0 * l + 3.0) / (2.0 * l - 1.0)) * ((l - m + 1.0) / (l + m + 1.0)) *
                 (((double)l - m) / ((double)l + m))) *
           ((l + m) / (l - m + 1.0));
}

// pmm.c:21-34 normalising constant (with the Condon-Shortley sign for odd m)
__device__ inline double pmm_const(int m) {
    double c = sqrt(m + 0.5);
    for (int i = 0; i < m; ++i) c *= sqrt((m - (i / 2.0)) / ((double)m - i));
    if (m) c *= exp2(-m / 2.0);
    if (m % 2) c = -c;
    return c;
}

// util.c:42-49
__host__ __device__ __forceinline__ int index_of_harmonic_coeff(int m, int l, int bw) {
    const int L = bw - 1;
    if (m >= 0) return m * bw - (m * (m - 1)) / 2 + (l - m);
    const int am = -m;
    return (L * (L + 3)) / 2 + 1 + ((L - am) * (L - am + 1)) / 2 + (l - am);
}

// cospml.c:250-258
__host__ __device__ __forceinline__ int row_size(int m, int l) {
    if (l < m) return 0;
    return (m % 2 == 0) ? (l / 2) + 1 : ((l - 1) / 2) + 1;
}

__host__ __device__ __forceinline__ int64_t prefix_even(int64_t n) {
    if (n <= 0) return 0;
    const int64_t q = n / 2, r = n % 2;
    return q * (q - 1) + r * q + n;
}

// cospml.c:123-134 (offset of row l inside the order-m table)
__host__ __device__ __forceinline__ int64_t table_offset(int m, int l) {
    if (m % 2 == 0) return prefix_even(l) - prefix_even(m);
    return prefix_even(l - 1) - prefix_even(m - 1);
}

// cospml.c:39-59
__host__ __device__ __forceinline__ int64_t table_size(int m, int bw) { return table_offset(m, bw); }

// First degree l whose cosine series contains frequency `row` (transposed table row).
__host__ __device__ __forceinline__ int trans_first_l(int row, int m) {
    return (row > m) ? row + (m % 2) : m + (row % 2);
}

// cospml.c:270-288 (true count; equals the reference for even bandwidths)
__host__ __device__ __forceinline__ int transpose_row_size(int row, int m, int bw) {
    if (row >= bw) return 0;
    const int l0 = trans_first_l(row, m);
    if (l0 >= bw) return 0;
    return (bw - l0 + 1) / 2;
}

}  // namespace s2g
