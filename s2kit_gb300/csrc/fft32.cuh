// fft32.cuh -- warp-level FP32 complex FFT of length n = 32 R (R = 1 .. 32, and R = 3 .. 15 that are
// not powers of two), used by the split-precision pipeline for the longitude DFTs and the
// latitude DCTs.
//
// Decomposition n = R x 32 with input index q = lane + 32 i (lane < 32, i < R):
//   X[k1 + R k2] = sum_lane w32^(lane k2) [ w_n^(lane k1) sum_i x[lane + 32 i] w_R^(i k1) ]
//   (a) R-point DFT over the registers of each lane (radix-2, fully unrolled; its twiddles
//       are compile-time constants, bit reversal is register renaming; for R not a power of
//       two a direct R-point DFT with compile-time twiddles)
//   (b) twiddle by w_n^(lane k1)
//   (c) 32-point decimation-in-frequency DFT across the lanes with __shfl_xor_sync
// On return register k1 of lane l holds X[k1 + R * brev5(l)].
// Twiddles of (c) come from a shared-memory table tw[padtw(k)] = (cos, sin)(2 pi k / n), padded
// by one entry every 16 so that the power-of-two strided reads hit distinct banks; those of (b)
// from a copy laid out by (register, lane), twb[32 k1 + lane] = tw[(lane k1) mod n], which every
// lane reads at consecutive addresses (no bank conflicts).
// Shared-memory staging of data uses pad32(p) = p + p/32, which keeps both the lane-strided
// (p = k1 + R brev(lane)) and lane-contiguous (p = lane + 32 t) patterns conflict-free.
#pragma once

#include <cuda_runtime.h>

namespace s2g {

__host__ __device__ __forceinline__ constexpr int pad32(int p) { return p + (p >> 5); }
__host__ __device__ __forceinline__ constexpr int padtw(int k) { return k + (k >> 4); }
__host__ __device__ __forceinline__ constexpr int twtab_len(int n) { return n + n / 16 + 1; }

// cos and sin of 2 pi j / n at compile time: octant reduction with exact integer arithmetic
// and Taylor series on [0, pi/4] (error far below double rounding).
namespace ct {
constexpr double kTwoPi = 6.283185307179586476925286766559;
__host__ __device__ constexpr double taylor_sin(double x) {
    double t = x, s = x;
    for (int k = 1; k < 14; ++k) {
        t *= -x * x / ((2 * k) * (2 * k + 1));
        s += t;
    }
    return s;
}
__host__ __device__ constexpr double taylor_cos(double x) {
    double t = 1.0, s = 1.0;
    for (int k = 1; k < 14; ++k) {
        t *= -x * x / ((2 * k - 1) * (2 * k));
        s += t;
    }
    return s;
}
// returns (cos, sin) of 2 pi j / n in c, s
__host__ __device__ constexpr void cossin(int j, int n, double& c, double& s) {
    j %= n;
    if (j < 0) j += n;
    // quadrant q and remainder r: angle = q * pi/2 + 2 pi r / n, 0 <= r < n/4 (n % 4 == 0)
    const int q4 = n / 4;
    int q = 0, r = j;
    if (n % 4 == 0) {
        q = j / q4;
        r = j % q4;
    }
    double a = kTwoPi * r / n;
    double cc = 0, ss = 0;
    if (n % 4 == 0 && 8 * r > n) {  // reflect into [0, pi/4]
        const double b = kTwoPi * (q4 - r) / n;
        cc = taylor_sin(b);
        ss = taylor_cos(b);
    } else {
        cc = taylor_cos(a);
        ss = taylor_sin(a);
    }
    switch (q) {
        case 0: c = cc; s = ss; break;
        case 1: c = -ss; s = cc; break;
        case 2: c = -cc; s = -ss; break;
        default: c = ss; s = -cc; break;
    }
}
__host__ __device__ constexpr float cosf_(int j, int n) {
    double c = 0, s = 0;
    cossin(j, n, c, s);
    return (float)c;
}
__host__ __device__ constexpr float sinf_(int j, int n) {
    double c = 0, s = 0;
    cossin(j, n, c, s);
    return (float)s;
}
}  // namespace ct

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One radix-2 butterfly layer of the in-register DFT: pairs (b + J, b + J + LEN/2).
template <int R, int LEN, int J>
struct RegBfly {
    __device__ __forceinline__ static void run(float2* u, float sign) {
        constexpr float c = ct::cosf_(J, LEN);
        constexpr float s = ct::sinf_(J, LEN);
        const float2 w = make_float2(c, sign * s);
#pragma unroll
        for (int b = 0; b < R; b += LEN) {
            const float2 a = u[b + J];
            const float2 d = (J == 0) ? u[b + J + LEN / 2] : cmulf(u[b + J + LEN / 2], w);
            u[b + J] = make_float2(a.x + d.x, a.y + d.y);
            u[b + J + LEN / 2] = make_float2(a.x - d.x, a.y - d.y);
        }
        RegBfly<R, LEN, J + 1>::run(u, sign);
    }
};
template <int R, int LEN>
struct RegBfly<R, LEN, LEN / 2> {
    __device__ __forceinline__ static void run(float2*, float) {}
};

template <int R, int LEN>
struct RegStages {
    __device__ __forceinline__ static void run(float2* u, float sign) {
        RegBfly<R, LEN, 0>::run(u, sign);
        RegStages<R, LEN * 2>::run(u, sign);
    }
};
template <int R>
struct RegStages<R, 2 * R> {
    __device__ __forceinline__ static void run(float2*, float) {}
};

// Direct R-point DFT in registers for R that is not a power of two: y[K] = sum_J x[J] w_R^(J K),
// w_R = exp(sign 2 pi i / R), with compile-time twiddles (angles 2 pi e / R evaluated as
// 2 pi (4 e) / (4 R), whose quadrant reduction keeps the series on [0, pi/4]).
template <int R, int K, int J>
struct DftTerm {
    __device__ __forceinline__ static void run(const float2* x, float2& acc, float sign) {
        constexpr int e = (J * K) % R;
        constexpr float c = ct::cosf_(4 * e, 4 * R);
        constexpr float s = ct::sinf_(4 * e, 4 * R);
        const float ss = sign * s;
        acc.x += x[J].x * c - x[J].y * ss;
        acc.y += x[J].x * ss + x[J].y * c;
        DftTerm<R, K, J + 1>::run(x, acc, sign);
    }
};
template <int R, int K>
struct DftTerm<R, K, R> {
    __device__ __forceinline__ static void run(const float2*, float2&, float) {}
};
template <int R, int K>
struct DftOut {
    __device__ __forceinline__ static void run(const float2* x, float2* y, float sign) {
        float2 acc = x[0];
        DftTerm<R, K, 1>::run(x, acc, sign);
        y[K] = acc;
        DftOut<R, K + 1>::run(x, y, sign);
    }
};
template <int R>
struct DftOut<R, R> {
    __device__ __forceinline__ static void run(const float2*, float2*, float) {}
};

template <int R>
struct WarpFFT {
    static constexpr bool kPow2 = (R & (R - 1)) == 0;
    __host__ __device__ static constexpr int brev(int i) {
        if (!kPow2) return i;
        int r = 0;
        for (int b = 1, c = R >> 1; b < R; b <<= 1, c >>= 1)
            if (i & b) r |= c;
        return r;
    }

    // tw: padded shared table of length twtab_len(32 R); twb: the (b) twiddles, 32 R entries
    __device__ static void run(float2 (&v)[R], const float2* __restrict__ tw, const float2* __restrict__ twb,
                               float sign) {
        constexpr int n = 32 * R;
        const int lane = threadIdx.x & 31;
        // (a) in-register DIT over i (radix 2; a direct DFT when R is not a power of two)
        float2 u[R];
        if constexpr (kPow2) {
#pragma unroll
            for (int i = 0; i < R; ++i) u[brev(i)] = v[i];
            RegStages<R, 2>::run(u, sign);
        } else {
            DftOut<R, 0>::run(v, u, sign);
        }
        // (b) w_n^(lane k1)
#pragma unroll
        for (int k1 = 1; k1 < R; ++k1) {
            float2 w = twb[32 * k1 + lane];
            w.y *= sign;
            u[k1] = cmulf(u[k1], w);
        }
        // (c) 32-point DIF across lanes
#pragma unroll
        for (int h = 16; h >= 1; h >>= 1) {
            const bool upper = (lane & h) != 0;
            float2 w = tw[padtw((lane & (h - 1)) * (n / (2 * h)))];
            w.y *= sign;
#pragma unroll
            for (int k1 = 0; k1 < R; ++k1) {
                float2 p;
                p.x = __shfl_xor_sync(0xffffffffu, u[k1].x, h);
                p.y = __shfl_xor_sync(0xffffffffu, u[k1].y, h);
                if (!upper)
                    u[k1] = make_float2(u[k1].x + p.x, u[k1].y + p.y);
                else
                    u[k1] = cmulf(make_float2(p.x - u[k1].x, p.y - u[k1].y), w);
            }
        }
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = u[i];
    }

    // natural-order index of register k1 of this lane after run()
    __device__ __forceinline__ static int out_index(int k1) {
        return k1 + R * (int)(__brev((unsigned)(threadIdx.x & 31)) >> 27);
    }
};

// Four-step form of the same transform for R in {8, 16, 32}: stages (a) and (b) as above, then the
// 32-point DFTs across the lanes go through shared memory instead of lane butterflies.
//   (c1) lane l writes u_l[k1] to row k1, column l of the warp's exchange rows: (re, im) pairs,
//        row stride 32 + P pairs (P = 32 / R), rows k1 < R/2 in the first plane and the others
//        in the second (conflict-free 8-byte accesses in both directions);
//   (c2) lane L = P c + h reads column c at lanes P j + h (j < R): y_j = u_{P j + h}[c], and
//        takes their R-point DFT in registers, Y_h[k] = sum_j y_j w_R^(j k);
//   (c3) Z_c[k + R q] = sum_h T_h[k] w_P^(h q) with T_h[k] = w_32^(h k) Y_h[k]: a P-point DFT
//        across the P lanes of column c, as log2(P) decimation-in-frequency stages.  In stage s
//        the partner lanes (h differing in bit e = log2(P) - 1 - s) split the k values they
//        hold by bit e of k (each keeps those whose bit e equals its own bit e of h), swap the
//        other half once (R shuffles per stage) and finish the butterfly, the difference twiddled
//        by w_M^(h mod 2^e), M = P >> s.  At the end lane (c, h) holds k = P k_hi + h, k_hi < R/P,
//        for every q.
// Then X[c + R k2] = Z_c[k2].  Register s of lane L holds X[out_index(s)], and for a fixed s the
// 32 lanes hold 32 consecutive indices, so spectrum stores through pad32 are conflict-free.
// Shared-memory traffic per transform: R 8-byte exchange writes and R reads, and log2(P) R
// shuffles, against 10 R shuffles of the lane-butterfly form.
// u[K] *= w_32^(h K), K = K0 .. R-1, for a runtime h in 1 .. P-1 (P <= 4): the P-1 candidate
// factors of each K are compile-time constants and h selects one.
template <int R, int P, int K>
struct C3Const {
    __device__ __forceinline__ static void run(float2* u, int h, float sign) {
        constexpr float c1 = ct::cosf_(K % 32, 32), s1 = ct::sinf_(K % 32, 32);
        constexpr float c2 = ct::cosf_((2 * K) % 32, 32), s2 = ct::sinf_((2 * K) % 32, 32);
        constexpr float c3 = ct::cosf_((3 * K) % 32, 32), s3 = ct::sinf_((3 * K) % 32, 32);
        float c = c1, s = s1;
        if (P > 2) {
            c = h == 1 ? c1 : (h == 2 ? c2 : c3);
            s = h == 1 ? s1 : (h == 2 ? s2 : s3);
        }
        u[K] = cmulf(u[K], make_float2(c, sign * s));
        C3Const<R, P, K + 1>::run(u, h, sign);
    }
};
template <int R, int P>
struct C3Const<R, P, R> {
    __device__ __forceinline__ static void run(float2*, int, float) {}
};

template <int R>
struct WarpFFT4 {
    static_assert(R == 8 || R == 16 || R == 32, "four-step warp FFT: R = 8, 16 or 32");
    static constexpr int P = 32 / R;
    static constexpr int LP = P == 1 ? 0 : P == 2 ? 1 : 2;  // log2 P
    static constexpr int XS = 32 + P;                       // exchange row stride (floats)
    static constexpr int kExchangeFloats = R * XS;          // per plane

    template <int STG>
    __device__ __forceinline__ static void stage(float2 (&u)[R], const float2* __restrict__ tw, int h, float sign) {
        constexpr int e = LP - 1 - STG;       // bit of h (and of k) this stage splits
        constexpr int ncur = R >> STG;        // k values per q-combination before the stage
        constexpr int nf = 1 << (LP - STG);   // free low bits of k, as a count
        constexpr int hf = nf / 2;
        constexpr int nq = 1 << STG;          // q-bit combinations so far
        constexpr int nnew = ncur / 2;
        constexpr int M = P >> STG;           // size of the sub-DFTs over h
        const int b = (h >> e) & 1;
        float2 w = tw[padtw((h & ((1 << e) - 1)) * (32 * R / M))];  // w_M^(h mod 2^e)
        w.y *= sign;
        float2 nv[R];
#pragma unroll
        for (int qb = 0; qb < nq; ++qb)
#pragma unroll
            for (int kh = 0; kh < R / P; ++kh)
#pragma unroll
                for (int f = 0; f < hf; ++f) {
                    const int i0 = qb * ncur + kh * nf + f, i1 = i0 + hf;  // k bit e = 0 / 1
                    const float2 own = b ? u[i1] : u[i0];
                    const float2 snd = b ? u[i0] : u[i1];
                    float2 rcv;
                    rcv.x = __shfl_xor_sync(0xffffffffu, snd.x, 1 << e);
                    rcv.y = __shfl_xor_sync(0xffffffffu, snd.y, 1 << e);
                    const float2 lo = b ? rcv : own, hi = b ? own : rcv;
                    const int kk = kh * hf + f;
                    nv[qb * nnew + kk] = make_float2(lo.x + hi.x, lo.y + hi.y);
                    nv[(qb + nq) * nnew + kk] = cmulf(make_float2(lo.x - hi.x, lo.y - hi.y), w);
                }
#pragma unroll
        for (int i = 0; i < R; ++i) u[i] = nv[i];
    }

    __device__ static void run(float2 (&v)[R], const float2* __restrict__ tw, const float2* __restrict__ twb,
                               float* __restrict__ xr, float* __restrict__ xi, float sign) {
        const int lane = threadIdx.x & 31;
        // (a) in-register DIT over i
        float2 u[R];
#pragma unroll
        for (int i = 0; i < R; ++i) u[WarpFFT<R>::brev(i)] = v[i];
        RegStages<R, 2>::run(u, sign);
        // (b) w_n^(lane k1)
#pragma unroll
        for (int k1 = 1; k1 < R; ++k1) {
            float2 w = twb[32 * k1 + lane];
            w.y *= sign;
            u[k1] = cmulf(u[k1], w);
        }
        // (c1) exchange: (re, im) pairs, row k1 < R/2 in xr and row k1 >= R/2 in xi, each row XS
        // pairs long (R XS floats per plane, as two planes of single floats would take); one
        // 8-byte store per value, conflict-free
        __syncwarp();
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1)
            *reinterpret_cast<float2*>((k1 < R / 2 ? xr : xi) + 2 * ((k1 % (R / 2)) * XS + lane)) = u[k1];
        __syncwarp();
        // (c2) column c, lanes P j + h, R-point DFT in registers; one 8-byte load per value, the
        // half-warp's 16 lanes on 16 distinct 8-byte bank pairs (XS = 32 + P)
        const int c = lane / P, h = lane % P;
        const float* xrow = (c < R / 2 ? xr + 2 * c * XS : xi + 2 * (c - R / 2) * XS) + 2 * h;
#pragma unroll
        for (int j = 0; j < R; ++j) u[WarpFFT<R>::brev(j)] = *reinterpret_cast<const float2*>(xrow + 2 * P * j);
        __syncwarp();  // the exchange planes are free again (callers reuse them)
        RegStages<R, 2>::run(u, sign);
        if constexpr (P > 1) {
            // (c3) T_h[k] = w_32^(h k) Y_h[k], then the P-point DFT across the column's lanes.  For
            // P <= 4 the factors are compile-time constants (h = 1..P-1 picks one per k); no
            // shared-memory table read.
            if (h) {
                if constexpr (P <= 4) {
                    C3Const<R, P, 1>::run(u, h, sign);
                } else {
#pragma unroll
                    for (int k = 1; k < R; ++k) {
                        float2 w = tw[padtw(((h * k) & 31) * R)];
                        w.y *= sign;
                        u[k] = cmulf(u[k], w);
                    }
                }
            }
            stage<0>(u, tw, h, sign);
            if constexpr (LP >= 2) stage<1>(u, tw, h, sign);
        }
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = u[k];
    }

    // natural-order index of register s of this lane after run()
    __device__ __forceinline__ static int out_index(int s) {
        const int lane = threadIdx.x & 31;
        const int c = lane / P, h = lane % P;
        const int qb = s / (R / P), kh = s % (R / P);
        return c + R * (P * kh + h + R * qb);
    }
};

// The warp FFT a kernel of a given R uses: the four-step form where it exists.  Both forms take
// the warp's exchange planes (the lane-butterfly form ignores them).
template <int R>
struct WarpFFTSel {
    __device__ __forceinline__ static void run(float2 (&v)[R], const float2* tw, const float2* twb, float* xr,
                                               float* xi, float sign) {
        (void)xr;
        (void)xi;
        WarpFFT<R>::run(v, tw, twb, sign);
    }
    __device__ __forceinline__ static int out_index(int s) { return WarpFFT<R>::out_index(s); }
};
template <>
struct WarpFFTSel<8> : WarpFFT4<8> {};
template <>
struct WarpFFTSel<16> : WarpFFT4<16> {};
template <>
struct WarpFFTSel<32> : WarpFFT4<32> {};

// Length 2048 (R = 64) in one warp as two four-step FFTs of length 1024 (the even and the odd
// samples, 32 values per lane each, so the lane's registers hold half of what a 64-value
// transform needs) and one radix-2 decimation-in-time step:
//   X[k] = E[k] + w^k O[k],  X[k + 1024] = E[k] - w^k O[k],  w = exp(sign 2 pi i / 2048), k < 1024.
// The spectrum is left in the warp's padded buffer zr/zi[pad32(k)], k < 2048 (at least pad32(2048)
// floats per plane).  The even pass exchanges in [0, 1056) and leaves E there; the odd pass
// exchanges in [1056, 2112); each (lane, register) then reads back the E value it stored itself.
// Tables: tw and twb of the length-1024 transform (see WarpFFT4), twc[k] = exp(2 pi i k / 2048).
struct WarpFFT2048 {
    static constexpr int H = 1024, OFF = 1056;
    __device__ __forceinline__ static void store_even(const float2 (&v)[32], float* zr, float* zi) {
#pragma unroll
        for (int k1 = 0; k1 < 32; ++k1) {
            const int o = pad32(WarpFFT4<32>::out_index(k1));
            zr[o] = v[k1].x;
            zi[o] = v[k1].y;
        }
    }
    __device__ __forceinline__ static void combine(const float2 (&v)[32], const float2* __restrict__ twc, float* zr,
                                                   float* zi, float sign) {
#pragma unroll
        for (int k1 = 0; k1 < 32; ++k1) {
            const int k = WarpFFT4<32>::out_index(k1);
            float2 w = twc[k];
            w.y *= sign;
            const float2 o = cmulf(v[k1], w);
            const int p0 = pad32(k), p1 = pad32(k + H);
            const float er = zr[p0], ei = zi[p0];
            zr[p0] = er + o.x;
            zi[p0] = ei + o.y;
            zr[p1] = er - o.x;
            zi[p1] = ei - o.y;
        }
    }
    // in(j): the complex input sample j < 2048 (read twice per call: even j, then odd j)
    template <class In>
    __device__ __forceinline__ static void to_spectrum(In in, const float2* __restrict__ tw,
                                                       const float2* __restrict__ twb, const float2* __restrict__ twc,
                                                       float* zr, float* zi, float sign) {
        const int lane = threadIdx.x & 31;
        float2 v[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = in(2 * (lane + 32 * i));
        WarpFFT4<32>::run(v, tw, twb, zr, zi, sign);
        store_even(v, zr, zi);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = in(2 * (lane + 32 * i) + 1);
        WarpFFT4<32>::run(v, tw, twb, zr + OFF, zi + OFF, sign);
        combine(v, twc, zr, zi, sign);
    }
    // the same with both halves' inputs already in registers (ve: even samples, vo: odd samples,
    // lane + 32 i each); vo is overwritten
    __device__ __forceinline__ static void to_spectrum_regs(float2 (&ve)[32], float2 (&vo)[32],
                                                            const float2* __restrict__ tw,
                                                            const float2* __restrict__ twb,
                                                            const float2* __restrict__ twc, float* zr, float* zi,
                                                            float sign) {
        WarpFFT4<32>::run(ve, tw, twb, zr, zi, sign);
        store_even(ve, zr, zi);
        WarpFFT4<32>::run(vo, tw, twb, zr + OFF, zi + OFF, sign);
        combine(vo, twc, zr, zi, sign);
    }
};

}  // namespace s2g
