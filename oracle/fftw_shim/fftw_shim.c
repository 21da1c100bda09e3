/*
 * fftw_shim.c -- FFTW3 subset restated from FFTW's documented transform definitions
 * (manual section "What FFTW Really Computes"), on top of the oracle's transforms.
 *
 * TEST INFRASTRUCTURE ONLY (reference build under oracle/_ref).
 *   split DFT  : out[k] = sum_j in[j] exp(-2 pi i j k / n), strides from the guru dims
 *   REDFT10    : out[k] = 2 sum_j in[j] cos(pi (j+1/2) k / n)
 *   REDFT01    : out[k] = in[0] + 2 sum_{j>=1} in[j] cos(pi j (k+1/2) / n)
 */
#include "fftw3.h"

#include <stdlib.h>
#include <string.h>

#include "../s2oracle.h"

struct fftw_plan_s {
    int is_r2r;
    fftw_r2r_kind kind;
    int n, is, os;           /* transform length and strides */
    int hn, his, hos;        /* howmany loop */
    double *ri, *ii, *ro, *io;
};

fftw_plan fftw_plan_r2r_1d(int n, double* in, double* out, fftw_r2r_kind kind, unsigned flags) {
    (void)flags;
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->is_r2r = 1;
    p->kind = kind;
    p->n = n;
    p->ri = in;
    p->ro = out;
    return p;
}

fftw_plan fftw_plan_guru_split_dft(int rank, const fftw_iodim* dims, int howmany_rank,
                                   const fftw_iodim* howmany_dims, double* ri, double* ii, double* ro,
                                   double* io, unsigned flags) {
    (void)flags;
    if (rank != 1 || howmany_rank > 1) return NULL;
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->n = dims[0].n;
    p->is = dims[0].is;
    p->os = dims[0].os;
    if (howmany_rank == 1) {
        p->hn = howmany_dims[0].n;
        p->his = howmany_dims[0].is;
        p->hos = howmany_dims[0].os;
    } else {
        p->hn = 1;
    }
    p->ri = ri; p->ii = ii; p->ro = ro; p->io = io;
    return p;
}

void fftw_execute_r2r(const fftw_plan p, double* in, double* out) {
    double* tmp = (double*)malloc(sizeof(double) * p->n);
    if (p->kind == FFTW_REDFT10)
        orc_redft10(p->n, in, tmp);
    else if (p->kind == FFTW_REDFT01)
        orc_redft01(p->n, in, tmp);
    else
        abort();
    memcpy(out, tmp, sizeof(double) * p->n);
    free(tmp);
}

void fftw_execute_split_dft(const fftw_plan p, double* ri, double* ii, double* ro, double* io) {
    int n = p->n;
    double* br = (double*)malloc(sizeof(double) * 2 * n);
    double* bi = br + n;
    for (int h = 0; h < p->hn; ++h) {
        for (int j = 0; j < n; ++j) {
            br[j] = ri[(long)h * p->his + (long)j * p->is];
            bi[j] = ii[(long)h * p->his + (long)j * p->is];
        }
        orc_dft(n, br, bi, -1);
        for (int k = 0; k < n; ++k) {
            ro[(long)h * p->hos + (long)k * p->os] = br[k];
            io[(long)h * p->hos + (long)k * p->os] = bi[k];
        }
    }
    free(br);
}

void fftw_execute(const fftw_plan p) {
    if (p->is_r2r)
        fftw_execute_r2r(p, p->ri, p->ro);
    else
        fftw_execute_split_dft(p, p->ri, p->ii, p->ro, p->io);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
