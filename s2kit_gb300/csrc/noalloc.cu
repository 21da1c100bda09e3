// noalloc.cu -- forward FP64 spherical harmonic transform of one function that allocates no
// device memory: its intermediate spectrum buffer and twiddle factors live in a file-scope
// __device__ array, and the caller passes every input (samples, tables, offsets, weights) and
// output as device pointers.
//
// Why: some callers cannot call cudaMalloc / cudaFree.  Examples are code running inside a
// host framework that has already reserved the device memory it is allowed to use (a fixed
// budget handed out at start-up), and latency-critical code for which the implicit device
// synchronisation of cudaMalloc / cudaFree is not acceptable.  This entry point gives them
// the transform with a fixed, preallocated scratch area instead.
//
// Limits: one function per call, bw <= S2G_NOALLOC_MAX_BW (256).  The scratch array takes
// S2G_NOALLOC_SCRATCH_DOUBLES doubles (about 4 MiB) on every GPU that loads the library, for
// the life of the process.  All calls share that one array: calls that overlap on the GPU
// (different streams, or several host threads) race on it and must be serialised by the caller.
//
// When 2 bw is not a power of two the length-2bw DFTs are Bluestein convolutions, whose chirp,
// kernel spectra and twiddles the other entry points build once per length with cudaMalloc.
// Here a kernel writes them into the same scratch array on every call instead.
#include <mutex>

#include "s2g_common.cuh"
#include "s2g_internal.h"

#define S2G_NOALLOC_MAX_BW 256
// Bluestein convolution length for the largest non-power-of-two 2 bw (510): the power of two
// >= 2 * 510 - 1
#define S2G_NOALLOC_MAX_M 1024
// spectrum buffer: 2 planes x (2 bw) rows x (2 bw) latitudes; twiddles: 2 tables of 2 bw double2;
// Bluestein tables: chirp (2 bw), two kernel spectra (M each) and M/2 twiddles, double2
#define S2G_NOALLOC_SCRATCH_DOUBLES                                                           \
    (2 * (2 * S2G_NOALLOC_MAX_BW) * (2 * S2G_NOALLOC_MAX_BW) + 4 * (2 * S2G_NOALLOC_MAX_BW) + \
     2 * (2 * S2G_NOALLOC_MAX_BW + 2 * S2G_NOALLOC_MAX_M + S2G_NOALLOC_MAX_M / 2))

namespace s2g {

static __device__ __align__(256) double g_noalloc_scratch[S2G_NOALLOC_SCRATCH_DOUBLES];

// Device address of g_noalloc_scratch per device.  In host code the symbol's name is only a
// host-side stand-in, so the address is looked up once per device with that device current.
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[64];

static int noalloc_scratch(int dev, double** out) {
    if (dev < 0 || dev >= 64) return fail(S2G_ERR_UNSUPPORTED, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[dev] = (double*)p;
    }
    *out = g_noalloc_ptr[dev];
    return S2G_OK;
}

// Bluestein tables of DFT length n (not a power of two), convolution length M = 2^lM >= 2n - 1,
// in the layout block_dft reads (Len): tab[0, n) chirp h_j = exp(-i pi j^2 / n); tab[n, n + M)
// and tab[n + M, n + 2M) the DFT (sign -1) of the kernel b_s[j] = conj(h^s_|j|) placed at j and
// M - j (|j| < n), for h^s = h (first) and conj(h) (second), divided by M and stored at the
// bit-reversed index; tab[n + 2M, n + 2M + M/2) twiddles exp(2 pi i k / M).  Angles are formed
// from exact integer residues (j^2 mod 2n, j k mod M) and evaluated with sincospi; the kernel
// spectra are direct sums of 2n - 1 terms in FP64 (one thread per output), which is ample for
// n <= 510.
__global__ void k_bluestein_tables(int n, int M, int lM, double2* __restrict__ tab) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        double s, c;
        sincospi((double)(((long long)i * i) % (2LL * n)) / n, &s, &c);
        tab[i] = make_double2(c, -s);
    } else if (i < n + 2 * M) {
        const int sg = (i - n) / M, k = (i - n) % M;
        // sg 0: kernel conj(h), h = exp(-i pi j^2/n) -> imaginary part +sin; sg 1: its conjugate
        const double bsign = sg == 0 ? 1.0 : -1.0;
        double sr = 0.0, si = 0.0;
        for (int j = -(n - 1); j <= n - 1; ++j) {
            const int aj = j < 0 ? -j : j, pj = j < 0 ? M + j : j;
            double hs, hc;
            sincospi((double)(((long long)aj * aj) % (2LL * n)) / n, &hs, &hc);
            const double br = hc, bi = bsign * hs;
            double ws, wc;  // exp(-2 pi i pj k / M)
            sincospi(2.0 * (double)(((long long)pj * k) % M) / M, &ws, &wc);
            sr += br * wc + bi * ws;
            si += bi * wc - br * ws;
        }
        const int rk = (int)(__brev((unsigned)k) >> (32 - lM));
        tab[n + sg * M + rk] = make_double2(sr / M, si / M);
    } else if (i < n + 2 * M + M / 2) {
        const int k = i - n - 2 * M;
        double s, c;
        sincospi(2.0 * k / M, &s, &c);
        tab[i] = make_double2(c, s);
    }
}

}  // namespace s2g

using namespace s2g;

extern "C" int s2g_fst_noalloc(const double* rdata, const double* idata, double* rcoeffs, double* icoeffs, int bw,
                               const double* table, const int64_t* table_offsets, const double* weights,
                               DataFormat data_format, int cutoff, void* stream) {
    if (bw < 2 || bw > S2G_NOALLOC_MAX_BW)
        return fail(S2G_ERR_ARG, "s2g_fst_noalloc: bandwidth %d outside [2, %d] (fixed scratch of %d doubles)", bw,
                    S2G_NOALLOC_MAX_BW, (int)S2G_NOALLOC_SCRATCH_DOUBLES);
    if (cutoff < 1 || cutoff > bw) return fail(S2G_ERR_ARG, "cutoff %d outside [1, bw=%d]", cutoff, bw);
    if (!rdata || !rcoeffs || !icoeffs || !table || !table_offsets || !weights ||
        (data_format == COMPLEX && !idata))
        return fail(S2G_ERR_ARG, "s2g_fst_noalloc: NULL argument");
    int dev;
    S2G_CUDA(cudaGetDevice(&dev));
    double* scratch = nullptr;
    S2G_TRY(noalloc_scratch(dev, &scratch));
    cudaStream_t st = (cudaStream_t)stream;
    const int S = 2 * bw;
    // layout inside the scratch array: spectrum buffer, then the two twiddle tables
    double* work = scratch;
    double2* tw_S = (double2*)(scratch + 2 * (size_t)(2 * S2G_NOALLOC_MAX_BW) * (2 * S2G_NOALLOC_MAX_BW));
    double2* tw_D = tw_S + 2 * S2G_NOALLOC_MAX_BW;
    // Nothing in the array has to start at zero: the twiddles (and Bluestein tables) are
    // rewritten for this bw and every spectrum row the transform reads is written by it first.
    S2G_TRY(twiddles_device(S, tw_S, tw_D, st));
    Len len = make_len(S);
    if (!len.pow2()) {
        int M = 1, lM = 0;
        while (M < 2 * S - 1) M <<= 1, ++lM;
        double2* blue = tw_D + 2 * S2G_NOALLOC_MAX_BW;
        const int cnt = S + 2 * M + M / 2;
        {
            ProfScope ps_("bluestein_tables", st);
            k_bluestein_tables<<<(cnt + 127) / 128, 128, 0, st>>>(S, M, lM, blue);
        }
        S2G_CUDA(cudaGetLastError());
        len.M = M;
        len.logM = lM;
        len.chirp = blue;
        len.bfwd = blue + S;
        len.binv = blue + S + M;
        len.twM = blue + S + 2 * M;
    }
    Tables view;
    view.bw = bw;
    view.cutoff = cutoff;
    view.device = dev;
    view.fwd = const_cast<double*>(table);
    view.off = const_cast<int64_t*>(table_offsets);
    view.weights = const_cast<double*>(weights);
    view.tw_S = tw_S;
    view.tw_D = tw_D;
    return fst_f64_len(&view, &len, rdata, idata, rcoeffs, icoeffs, 1, (int)data_format, cutoff, work, st);
}
