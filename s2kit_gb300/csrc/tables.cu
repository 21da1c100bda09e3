// tables.cu -- FP64 generation of the seminaive memo tables on the GPU.
//
//   k_gen_cos   : GenerateCosPmlTable (cospml.c:161-242): L2-normalised three-term recurrence
//                 (l2_norms.c:16-38) from P(m,m) (pmm.c:21-34) at bw Chebyshev nodes, divided by
//                 sin(theta) for odd m, REDFT10 of length bw per degree, scaled 1/sqrt(bw) with
//                 sqrt(1/2) on k=0, only the parity-matching (non-zero) entries kept
//   k_transpose : TransposeCosPmlTable (cospml.c:301-362) -- row i of the transposed table holds
//                 T(l, i) for the degrees l whose series contains frequency i, ascending
//   k_gen_pml   : GeneratePmlTable (pml.c:41-79) -- P(m,l) sampled at the 2bw nodes (naive orders)
//   k_weights   : GenerateWeightsForDLT (weights.c:32-47)
// One CTA per order; the degree recurrence is sequential inside the CTA, the nodes and the
// DCT butterflies are spread over the threads.
#include <math.h>

#include <vector>

#include "s2g_common.cuh"
#include "s2g_internal.h"

namespace s2g {

static constexpr double kSqrtHalf = 0.70710678118654752440;

struct GenCos {
    int B;
    int m0;
    double* fwd;
    const int64_t* off;
    const double2* twB;   // exp(2 pi i k / B), k < B
    const double2* twQ;   // (cos, sin)(pi k / 2B), k < B
    const double2* tw4;   // exp(2 pi i r / 4B), r < 4B (direct DCT for odd B)
    int logB;
};

// DCT of `cur` (length B) into cs[k], normalised as the table expects (cospml.c:203-208).
__device__ void table_dct(const GenCos& p, const double* cur, double* zr, double* zi, double* tmp, double* cs) {
    const int B = p.B;
    const Len L{B, p.logB};
    const double nrm = 1.0 / sqrt((double)B);
    if (B % 2 == 0) {
        for (int q = threadIdx.x; q < B; q += blockDim.x) {
            const int d = (q & 1) ? B - 1 - (q >> 1) : (q >> 1);
            zr[L.pos(d)] = cur[q];
            zi[L.pos(d)] = 0.0;
        }
        __syncthreads();
        block_dft<double, double2>(zr, zi, L, 1, B, p.twB, -1.0, tmp);
        for (int k = threadIdx.x; k < B; k += blockDim.x) {
            const double v = 2.0 * (zr[k] * p.twQ[k].x + zi[k] * p.twQ[k].y);
            cs[k] = v * ((k == 0) ? kSqrtHalf * nrm : nrm);
        }
    } else {
        for (int k = threadIdx.x; k < B; k += blockDim.x) {
            double s = 0.0;
            int r = k, step = 2 * k;  // (2j+1) k mod 4B
            const int n4 = 4 * B;
            for (int j = 0; j < B; ++j) {
                s += cur[j] * p.tw4[r].x;
                r += step;
                while (r >= n4) r -= n4;
            }
            cs[k] = 2.0 * s * ((k == 0) ? kSqrtHalf * nrm : nrm);
        }
    }
    __syncthreads();
}

__global__ void k_gen_cos(GenCos p) {
    extern __shared__ double sm[];
    const int B = p.B;
    const int m = p.m0 + blockIdx.x;
    double* pp = sm;
    double* pv = pp + B;
    double* cur = pv + B;
    double* x = cur + B;
    double* cs = x + B;
    double* zr = cs + B;
    double* zi = zr + B;
    double* tmp = zi + B;  // 2B (non power of two)
    __shared__ double cpmm;
    if (threadIdx.x == 0) cpmm = (m == 0) ? 0.0 : pmm_const(m);
    __syncthreads();
    for (int i = threadIdx.x; i < B; i += blockDim.x) {
        double s, c;
        sincospi((2.0 * i + 1.0) / (2.0 * B), &s, &c);  // theta_i = (2i+1) pi / 2B
        x[i] = c;
        pp[i] = 0.0;
        double v = (m == 0) ? kSqrtHalf : cpmm * pow(s, (double)m);
        if (m % 2) v /= s;
        pv[i] = v;
    }
    __syncthreads();
    double* tab = p.fwd + p.off[m];
    int deg = (m % 2 == 0) ? m : m - 1;
    table_dct(p, pv, zr, zi, tmp, cs);
    for (int f = 2 * threadIdx.x; f <= deg; f += 2 * blockDim.x) tab[f / 2] = cs[f];
    __syncthreads();
    for (int i = 0; i < B - m - 1; ++i) {
        const int l = m + i + 1;
        const double an = l2_an(m, m + i), cn = l2_cn(m, m + i);
        for (int q = threadIdx.x; q < B; q += blockDim.x) cur[q] = an * (pv[q] * x[q]) + cn * pp[q];
        __syncthreads();
        table_dct(p, cur, zr, zi, tmp, cs);
        ++deg;
        const int f0 = (i % 2) ? 0 : 1;
        double* row = tab + table_offset(m, l);
        for (int f = f0 + 2 * threadIdx.x; f <= deg; f += 2 * blockDim.x) row[f / 2] = cs[f];
        double* t = pp;
        pp = pv;
        pv = cur;
        cur = t;
        __syncthreads();
    }
}

__global__ void k_transpose(int B, int m0, const double* fwd, double* inv, const int64_t* off) {
    extern __shared__ int ism[];
    int* toff = ism;          // B + 1
    int* wtot = toff + B + 1; // 32
    const int m = m0 + blockIdx.x;
    for (int i = threadIdx.x; i < B; i += blockDim.x) toff[i] = transpose_row_size(i, m, B);
    __syncthreads();
    block_exclusive_scan(toff, B, wtot);
    const double* src = fwd + off[m];
    double* dst = inv + off[m];
    for (int l = m; l < B; ++l) {
        const int t = (l - m) & 1;
        const int rs = row_size(m, l);
        const double* row = src + table_offset(m, l);
        for (int idx = threadIdx.x; idx < rs; idx += blockDim.x) {
            const int i = 2 * idx + t;                 // frequency
            const int j = (l - trans_first_l(i, m)) / 2;
            dst[toff[i] + j] = row[idx];
        }
    }
}

__global__ void k_gen_pml(int B, int m0, double* fwd, const int64_t* off) {
    extern __shared__ double sm[];
    const int S = 2 * B;
    const int m = m0 + blockIdx.x;
    double* pp = sm;
    double* pv = pp + S;
    double* x = pv + S;
    __shared__ double cpmm;
    if (threadIdx.x == 0) cpmm = (m == 0) ? 0.0 : pmm_const(m);
    __syncthreads();
    double* tab = fwd + off[m];
    for (int q = threadIdx.x; q < S; q += blockDim.x) {
        double s, c;
        sincospi((2.0 * q + 1.0) / (2.0 * S), &s, &c);
        x[q] = c;
        pp[q] = 0.0;
        pv[q] = (m == 0) ? kSqrtHalf : cpmm * pow(s, (double)m);
        tab[q] = pv[q];
    }
    __syncthreads();
    for (int i = 0; i < B - m - 1; ++i) {
        const double an = l2_an(m, m + i), cn = l2_cn(m, m + i);
        double* row = tab + (size_t)(i + 1) * S;
        // each thread owns its nodes: no cross-thread dependence inside the recurrence
        for (int q = threadIdx.x; q < S; q += blockDim.x) {
            const double v = an * (pv[q] * x[q]) + cn * pp[q];
            pp[q] = pv[q];
            pv[q] = v;
            row[q] = v;
        }
    }
}

// weights.c:32-47 ; the angle (2j+1)(2k+1) pi / 4B is reduced exactly (integer mod 8B).
__global__ void k_weights(int B, double* w) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * B) return;
    const long long kk = 2 * j + 1;
    double s = 0.0;
    for (int q = 0; q < B; ++q) {
        const long long r = (kk * (2 * q + 1)) % (8LL * B);
        s += 1.0 / (2.0 * q + 1.0) * sinpi((double)r / (4.0 * B));
    }
    const double sk = sinpi((double)kk / (4.0 * B));
    s *= 2.0 * sk / B;
    w[j] = s;
    w[j + 2 * B] = s * sk;
}

// chebyshev_nodes.c:15-34 (acos_only: angles; else cosines) and sin of the angles
__global__ void k_nodes(int n, double* out, int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = (2.0 * i + 1.0) / (2.0 * n);
    if (mode == 0) out[i] = a * 3.14159265358979323846;
    else if (mode == 1) out[i] = cospi(a);
    else out[i] = sinpi(a);
}

__global__ void k_pmm(int m, const double* eval, int n, double* out) {
    __shared__ double c;
    if (threadIdx.x == 0) c = pmm_const(m);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = c * pow(sin(eval[i]), (double)m);
}

// ------------------------------------------------------------------------------------
int generate_weights_device(int bw, double* d_w, cudaStream_t st) {
    {
        ProfScope ps_("weights", st);
        k_weights<<<(2 * bw + 127) / 128, 128, 0, st>>>(bw, d_w);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

int nodes_device(int n, double* d_out, int mode, cudaStream_t st) {
    {
        ProfScope ps_("nodes", st);
        k_nodes<<<(n + 255) / 256, 256, 0, st>>>(n, d_out, mode);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

int pmm_device(int m, const double* d_eval, int n, double* d_out, cudaStream_t st) {
    {
        ProfScope ps_("pmm", st);
        k_pmm<<<(n + 255) / 256, 256, 0, st>>>(m, d_eval, n, d_out);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

struct TableTw {
    double2* twB = nullptr;
    double2* twQ = nullptr;
    double2* tw4 = nullptr;
    ~TableTw() {
        cudaFree(twB);
        cudaFree(twQ);
        cudaFree(tw4);
    }
};

int generate_cos_pml_device(int bw, int m_begin, int m_end, double* d_fwd, const int64_t* d_off, cudaStream_t st) {
    if (m_end <= m_begin) return S2G_OK;
    TableTw tw;
    S2G_CUDA(cudaMalloc(&tw.twB, sizeof(double2) * bw));
    S2G_CUDA(cudaMalloc(&tw.twQ, sizeof(double2) * bw));
    S2G_CUDA(cudaMalloc(&tw.tw4, sizeof(double2) * 4 * bw));
    S2G_TRY(twiddles_device(bw, tw.twB, tw.twQ, st));
    S2G_TRY(twiddles_device(4 * bw, tw.tw4, nullptr, st));
    const Len L = make_len(bw);
    GenCos p{bw, m_begin, d_fwd, d_off, tw.twB, tw.twQ, tw.tw4, L.logn};
    const size_t smem = (size_t)(7 * bw + 2 * bw) * sizeof(double);
    if (smem > 0)  // the 48 KiB default covers static plus dynamic shared memory
        S2G_CUDA(cudaFuncSetAttribute((const void*)k_gen_cos, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    {
        ProfScope ps_("gen_cos_pml", st);
        k_gen_cos<<<m_end - m_begin, 256, smem, st>>>(p);
    }
    S2G_CUDA(cudaGetLastError());
    S2G_CUDA(cudaStreamSynchronize(st));  // twiddle buffers are freed on return
    return S2G_OK;
}

int transpose_cos_pml_device(int bw, int m_begin, int m_end, const double* d_fwd, double* d_inv,
                             const int64_t* d_off, cudaStream_t st) {
    if (m_end <= m_begin) return S2G_OK;
    const size_t smem = (size_t)(bw + 1 + 32) * sizeof(int);
    {
        ProfScope ps_("transpose_cos_pml", st);
        k_transpose<<<m_end - m_begin, 256, smem, st>>>(bw, m_begin, d_fwd, d_inv, d_off);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

int generate_pml_device(int bw, int m_begin, int m_end, double* d_fwd, const int64_t* d_off, cudaStream_t st) {
    if (m_end <= m_begin) return S2G_OK;
    const size_t smem = (size_t)3 * 2 * bw * sizeof(double);
    if (smem > 0)  // the 48 KiB default covers static plus dynamic shared memory
        S2G_CUDA(cudaFuncSetAttribute((const void*)k_gen_pml, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    {
        ProfScope ps_("gen_pml", st);
        k_gen_pml<<<m_end - m_begin, 256, smem, st>>>(bw, m_begin, d_fwd, d_off);
    }
    S2G_CUDA(cudaGetLastError());
    return S2G_OK;
}

// Offsets of SemiNaive_Naive_Pml_Table (cospml.c:451-475), 64-bit.
static void host_offsets(int bw, int cutoff, std::vector<int64_t>& off, int64_t* total) {
    off.resize(bw);
    int64_t o = 0;
    for (int m = 0; m < bw; ++m) {
        off[m] = o;
        o += (m < cutoff) ? table_size(m, bw) : 2 * (int64_t)bw * (bw - m);
    }
    *total = o;
}

int build_tables(Tables* t, cudaStream_t st, const double* h_fwd, const double* h_inv) {
    const int B = t->bw, S = 2 * B;
    S2G_CUDA(cudaMalloc(&t->weights, sizeof(double) * 4 * B));
    S2G_CUDA(cudaMalloc(&t->sinv, sizeof(double) * S));
    S2G_CUDA(cudaMalloc(&t->tw_S, sizeof(double2) * S));
    S2G_CUDA(cudaMalloc(&t->tw_D, sizeof(double2) * S));
    S2G_TRY(generate_weights_device(B, t->weights, st));
    S2G_TRY(nodes_device(S, t->sinv, 2, st));
    S2G_TRY(twiddles_device(S, t->tw_S, t->tw_D, st));
    if (t->cutoff == 0) {  // on-the-fly family: no Legendre table
        t->total = 0;
        S2G_CUDA(cudaStreamSynchronize(st));
        return S2G_OK;
    }
    std::vector<int64_t> off;
    host_offsets(B, t->cutoff, off, &t->total);
    t->h_off = new int64_t[B];
    for (int m = 0; m < B; ++m) t->h_off[m] = off[m];
    S2G_CUDA(cudaMalloc(&t->fwd, sizeof(double) * (size_t)(t->total > 0 ? t->total : 1)));
    S2G_CUDA(cudaMalloc(&t->inv, sizeof(double) * (size_t)(t->total > 0 ? t->total : 1)));
    S2G_CUDA(cudaMalloc(&t->off, sizeof(int64_t) * B));
    S2G_CUDA(cudaMemcpyAsync(t->off, off.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, st));
    const int cut = t->cutoff;
    if (h_fwd && h_inv) {
        S2G_CUDA(cudaMemcpyAsync(t->fwd, h_fwd, sizeof(double) * (size_t)t->total, cudaMemcpyHostToDevice, st));
        S2G_CUDA(cudaMemcpyAsync(t->inv, h_inv, sizeof(double) * (size_t)t->total, cudaMemcpyHostToDevice, st));
        S2G_CUDA(cudaStreamSynchronize(st));
        return S2G_OK;
    }
    S2G_TRY(generate_cos_pml_device(B, 0, cut, t->fwd, t->off, st));
    S2G_TRY(transpose_cos_pml_device(B, 0, cut, t->fwd, t->inv, t->off, st));
    if (cut < B) {
        S2G_TRY(generate_pml_device(B, cut, B, t->fwd, t->off, st));
        const int64_t n0 = off[cut];
        S2G_CUDA(cudaMemcpyAsync(t->inv + n0, t->fwd + n0, sizeof(double) * (size_t)(t->total - n0),
                                 cudaMemcpyDeviceToDevice, st));
    }
    S2G_CUDA(cudaStreamSynchronize(st));
    return S2G_OK;
}

}  // namespace s2g
