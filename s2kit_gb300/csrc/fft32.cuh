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
// Twiddles of (b) and (c) come from a shared-memory table tw[padtw(k)] = (cos, sin)(2 pi k / n),
// padded by one entry every 16 so that the power-of-two strided reads hit distinct banks.
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

    // tw: padded shared table of length twtab_len(32 R)
    __device__ static void run(float2 (&v)[R], const float2* __restrict__ tw, float sign) {
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
            float2 w = tw[padtw((lane * k1) & (n - 1))];
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

}  // namespace s2g
