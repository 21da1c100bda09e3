// rows.cuh -- DFTs along longitude for the whole latitude grid (FP64 and FP32 paths).
//
// k_rows_fwd: forward DFT of each latitude row (FST_semi_memo.c:81, FFTW split DFT sign -1),
//             scaled, stored transposed X[f][m][theta] (orders m < rows_out).
// k_rows_inv: DFT with sign +1 over the orders for each latitude (the reference's re/im
//             swapped forward DFT, FST_semi_memo.c:350), rows m > bw from COMPLEX data or
//             by Hermitian symmetry (REAL, FST_semi_memo.c:334-340), row bw zero.
// Both pack two real latitudes into one complex DFT when the data are real.
#pragma once
#include "s2g_common.cuh"

namespace s2g {

// ------------------------------------------------------------------------------------
// Row DFTs along phi.  One CTA: R complex sequences of length S.
//   complex mode (idata != null): sequence r = latitude j0 + r
//   real mode    (idata == null): sequence r = latitudes j0 + 2r (real part), j0 + 2r + 1 (imag part)
// Output X[f][m][theta] for m < rows_out, scaled.
template <typename T, typename T2>
__global__ void k_rows_fwd(const T* __restrict__ rdata, const T* __restrict__ idata,
                           T* __restrict__ Xr, T* __restrict__ Xi, int S, const Len L, int rows_out, int R,
                           T scale, const T2* __restrict__ tw) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T* sm = reinterpret_cast<T*>(sm_raw);
    const int SP = S + 1;
    T* re = sm;
    T* im = re + (size_t)R * SP;
    T* tmp = im + (size_t)R * SP;
    const int f = blockIdx.y;
    const bool real_mode = (idata == nullptr);
    const int lat_per_cta = real_mode ? 2 * R : R;
    const int j0 = blockIdx.x * lat_per_cta;
    const int nlat = min(lat_per_cta, S - j0);
    const int nseq = real_mode ? (nlat + 1) / 2 : nlat;
    const size_t gbase = (size_t)f * S * S;

    for (int t = threadIdx.x; t < nseq * S; t += blockDim.x) {
        const int r = t / S, k = t - r * S;
        T a, b;
        if (real_mode) {
            const int la = j0 + 2 * r, lb = la + 1;
            a = rdata[gbase + (size_t)la * S + k];
            b = (lb < j0 + nlat) ? rdata[gbase + (size_t)lb * S + k] : T(0.0);
        } else {
            a = rdata[gbase + (size_t)(j0 + r) * S + k];
            b = idata[gbase + (size_t)(j0 + r) * S + k];
        }
        re[r * SP + L.pos(k)] = a;
        im[r * SP + L.pos(k)] = b;
    }
    __syncthreads();
    block_dft<T, T2>(re, im, L, nseq, SP, tw, T(-1.0), tmp);

    const size_t xbase = (size_t)f * rows_out * S;
    for (int t = threadIdx.x; t < rows_out * nlat; t += blockDim.x) {
        const int m = t / nlat, q = t - m * nlat;
        T vr, vi;
        if (real_mode) {
            const int r = q >> 1;
            const T zr = re[r * SP + m], zi = im[r * SP + m];
            const int mm = (m == 0) ? 0 : S - m;
            const T wr = re[r * SP + mm], wi = im[r * SP + mm];
            if ((q & 1) == 0) {
                vr = T(0.5) * (zr + wr);
                vi = T(0.5) * (zi - wi);
            } else {
                vr = T(0.5) * (zi + wi);
                vi = T(-0.5) * (zr - wr);
            }
        } else {
            vr = re[q * SP + m];
            vi = im[q * SP + m];
        }
        Xr[xbase + (size_t)m * S + j0 + q] = vr * scale;
        Xi[xbase + (size_t)m * S + j0 + q] = vi * scale;
    }
}

// ------------------------------------------------------------------------------------
// Inverse DFT along m for each latitude (sign +1), R sequences per CTA.
//   fmt_complex : rows 0..S-1 from F (row B = 0)
//   REAL        : rows m > B are conj(F[S-m])
//   real output (rdata only, idata == null): two latitudes per complex DFT
template <typename T, typename T2>
__global__ void k_rows_inv(const T* __restrict__ Fr, const T* __restrict__ Fi, int frows, int fmt_complex,
                           T* __restrict__ rdata, T* __restrict__ idata, int S, const Len L, int R,
                           const T2* __restrict__ tw) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T* sm = reinterpret_cast<T*>(sm_raw);
    const int B = S / 2;
    const int SP = S + 1;
    T* re = sm;
    T* im = re + (size_t)R * SP;
    T* tmp = im + (size_t)R * SP;
    const int f = blockIdx.y;
    const bool real_out = (idata == nullptr);
    const int lat_per_cta = real_out ? 2 * R : R;
    const int j0 = blockIdx.x * lat_per_cta;
    const int nlat = min(lat_per_cta, S - j0);
    const int nseq = real_out ? (nlat + 1) / 2 : nlat;
    const size_t fb = (size_t)f * frows * S;

    // gather: consecutive threads take consecutive latitudes of one row (coalesced reads)
    for (int t = threadIdx.x; t < S * nlat; t += blockDim.x) {
        const int mrow = t / nlat, q = t - mrow * nlat;
        const int lat = j0 + q;
        T vr = T(0.0), vi = T(0.0);
        if (mrow != B) {
            if (fmt_complex) {
                vr = Fr[fb + (size_t)mrow * S + lat];
                vi = Fi[fb + (size_t)mrow * S + lat];
            } else if (mrow < B) {
                vr = Fr[fb + (size_t)mrow * S + lat];
                vi = Fi[fb + (size_t)mrow * S + lat];
            } else {
                vr = Fr[fb + (size_t)(S - mrow) * S + lat];
                vi = -Fi[fb + (size_t)(S - mrow) * S + lat];
            }
        }
        if (real_out) {
            if (mrow == 0) vi = T(0.0);  // Hermitian: the m = 0 term is real
            const int r = q >> 1;
            // Z = F_a + i F_b
            if ((q & 1) == 0) {
                re[r * SP + L.pos(mrow)] = vr;
                im[r * SP + L.pos(mrow)] = vi;
            }
        } else {
            re[q * SP + L.pos(mrow)] = vr;
            im[q * SP + L.pos(mrow)] = vi;
        }
    }
    if (real_out) {
        // second pass: add i * F_b for the odd latitudes (avoids a write race on the same slot)
        __syncthreads();
        for (int t = threadIdx.x; t < S * nlat; t += blockDim.x) {
            const int mrow = t / nlat, q = t - mrow * nlat;
            if ((q & 1) == 0) continue;
            const int lat = j0 + q;
            T vr = T(0.0), vi = T(0.0);
            if (mrow != B) {
                if (mrow < B) {
                    vr = Fr[fb + (size_t)mrow * S + lat];
                    vi = Fi[fb + (size_t)mrow * S + lat];
                } else {
                    vr = Fr[fb + (size_t)(S - mrow) * S + lat];
                    vi = -Fi[fb + (size_t)(S - mrow) * S + lat];
                }
            }
            if (mrow == 0) vi = T(0.0);
            const int r = q >> 1;
            re[r * SP + L.pos(mrow)] -= vi;
            im[r * SP + L.pos(mrow)] += vr;
        }
    }
    __syncthreads();
    block_dft<T, T2>(re, im, L, nseq, SP, tw, T(1.0), tmp);
    const size_t gb = (size_t)f * S * S;
    for (int t = threadIdx.x; t < nlat * S; t += blockDim.x) {
        const int q = t / S, k = t - q * S;
        if (real_out) {
            const int r = q >> 1;
            rdata[gb + (size_t)(j0 + q) * S + k] = (q & 1) ? im[r * SP + k] : re[r * SP + k];
        } else {
            rdata[gb + (size_t)(j0 + q) * S + k] = re[q * SP + k];
            idata[gb + (size_t)(j0 + q) * S + k] = im[q * SP + k];
        }
    }
}

}  // namespace s2g
