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
#include <mutex>

#include "s2g_common.cuh"
#include "s2g_internal.h"

#define S2G_NOALLOC_MAX_BW 256
// spectrum buffer: 2 planes x (2 bw) rows x (2 bw) latitudes; twiddles: 2 tables of 2 bw double2
#define S2G_NOALLOC_SCRATCH_DOUBLES \
    (2 * (2 * S2G_NOALLOC_MAX_BW) * (2 * S2G_NOALLOC_MAX_BW) + 4 * (2 * S2G_NOALLOC_MAX_BW))

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
    // Nothing in the array has to start at zero: the twiddles are rewritten for this bw and
    // every spectrum row the transform reads is written by it first.
    S2G_TRY(twiddles_device(S, tw_S, tw_D, st));
    Tables view;
    view.bw = bw;
    view.cutoff = cutoff;
    view.device = dev;
    view.fwd = const_cast<double*>(table);
    view.off = const_cast<int64_t*>(table_offsets);
    view.weights = const_cast<double*>(weights);
    view.tw_S = tw_S;
    view.tw_D = tw_D;
    return fst_f64(&view, rdata, idata, rcoeffs, icoeffs, 1, (int)data_format, cutoff, work, st);
}
