// fft32.cuh -- warp-level FP32 complex FFT of length n = 32 R (R = 1 .. 32), used by the
// split-precision pipeline for the longitude DFTs and the latitude DCTs.
//
// Decomposition n = R x 32 with input index q = lane + 32 i (lane < 32, i < R):
//   X[k1 + R k2] = sum_lane w32^(lane k2) [ w_n^(lane k1) sum_i x[lane + 32 i] w_R^(i k1) ]
//   (a) R-point DFT over the registers of each lane (radix-2, fully unrolled; its twiddles
//       are compile-time constants, bit reversal is register renaming)
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

template <int R>
struct WarpFFT {
    __host__ __device__ static constexpr int brev(int i) {
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
        // (a) in-register DIT over i
        float2 u[R];
#pragma unroll
        for (int i = 0; i < R; ++i) u[brev(i)] = v[i];
        RegStages<R, 2>::run(u, sign);
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

// Four-step form of the same transform for R in {16, 32}: stages (a) and (b) as above, then the
// 32-point DFTs across the lanes go through shared memory instead of shuffles.
//   (c1) lane l writes u_l[k1] to row k1, column l of the warp's exchange planes (row stride
//        32 + P floats, P = 32 / R);
//   (c2) lane L = P c + h reads column c at lanes P j + h (j < R): y_j = u_{P j + h}[c], and
//        takes their R-point DFT in registers, Y_h[k] = sum_j y_j w_R^(j k);
//   (c3) Z_c[k + R q] = sum_h w_32^(h k) Y_h[k] w_P^(h q): nothing more for P = 1; for P = 2 the
//        two lanes of a column swap half of their values once (lane h keeps k = 2 i + h) and
//        finish with one butterfly.
// Then X[c + R k2] = Z_c[k2].  Shared-memory traffic per transform: R exchange writes and reads
// per plane (conflict-free: row stride 32 + P) and R shuffles, against 10 R shuffles of the
// lane-butterfly form.  Register s of lane L holds X[out_index(s)]; for a fixed s the 32 lanes
// hold 32 consecutive indices.
template <int R>
struct WarpFFT4 {
    static_assert(R == 16 || R == 32, "four-step warp FFT: R = 16 or 32");
    static constexpr int P = 32 / R;
    static constexpr int XS = 32 + P;   // exchange row stride (floats)
    static constexpr int kExchangeFloats = R * XS;  // per plane

    __device__ static void run(float2 (&v)[R], const float2* __restrict__ tw, const float2* __restrict__ twb,
                               float* __restrict__ xr, float* __restrict__ xi, float sign) {
        (void)tw;
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
        // (c1) exchange
        __syncwarp();
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            xr[k1 * XS + lane] = u[k1].x;
            xi[k1 * XS + lane] = u[k1].y;
        }
        __syncwarp();
        // (c2) column c, lanes P j + h, R-point DFT in registers
        const int c = lane / P, h = lane % P;
#pragma unroll
        for (int j = 0; j < R; ++j)
            u[WarpFFT<R>::brev(j)] = make_float2(xr[c * XS + P * j + h], xi[c * XS + P * j + h]);
        __syncwarp();  // the exchange planes are free again (callers reuse them)
        RegStages<R, 2>::run(u, sign);
        if (P == 1) {
#pragma unroll
            for (int k = 0; k < R; ++k) v[k] = u[k];
            return;
        }
        // (c3), P = 2: T_1[k] = w_32^k Y_1[k]; lane h keeps k = 2 i + h and gets T_{1-h}[k] from its partner
        if (h) {
#pragma unroll
            for (int k = 1; k < R; ++k) {
                const float2 w = make_float2(ct::cosf_(k, 32), sign * ct::sinf_(k, 32));
                u[k] = cmulf(u[k], w);
            }
        }
#pragma unroll
        for (int i = 0; i < R / 2; ++i) {
            const float2 own = h ? u[2 * i + 1] : u[2 * i];
            const float2 snd = h ? u[2 * i] : u[2 * i + 1];
            float2 rcv;
            rcv.x = __shfl_xor_sync(0xffffffffu, snd.x, 1);
            rcv.y = __shfl_xor_sync(0xffffffffu, snd.y, 1);
            const float2 lo = h ? rcv : own, hi = h ? own : rcv;
            v[i] = make_float2(lo.x + hi.x, lo.y + hi.y);
            v[i + R / 2] = make_float2(lo.x - hi.x, lo.y - hi.y);
        }
    }

    __device__ __forceinline__ static int out_index(int s) {
        const int lane = threadIdx.x & 31;
        if (P == 1) return lane + R * s;
        const int c = lane >> 1, h = lane & 1;
        return c + R * (2 * (s & (R / 2 - 1)) + h + 16 * (s / (R / 2)));
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
struct WarpFFTSel<16> : WarpFFT4<16> {};
template <>
struct WarpFFTSel<32> : WarpFFT4<32> {};

}  // namespace s2g
