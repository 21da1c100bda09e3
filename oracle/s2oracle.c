/*
 * s2oracle.c -- CPU restatement of S2kit 1.1's seminaive memo SHT path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg as the checker / CPU baseline.  Never part of the product.
 *
 * Reference citations are file:line within the S2kit repository.  FFTW3 (an external,
 * unvendored dependency of the reference, linked as -lfftw3 at Makefile:3-5, no pinned
 * version) is restated from its documented transform definitions:
 *   forward split DFT  : X[k] = sum_j x[j] exp(-2 pi i j k / n)   (unnormalised)
 *   FFTW_REDFT10       : Y[k] = 2 sum_j x[j] cos(pi (j + 1/2) k / n)
 *   FFTW_REDFT01       : Y[k] = x[0] + 2 sum_{j>=1} x[j] cos(pi j (k + 1/2) / n)
 */
#include "s2oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORC_PI 3.14159265358979323846264338327950288
#define ORC_SQRT1_2 0.70710678118654752440084436210484904

/* ===================================================================== */
/* Index and size helpers                                                */
/* ===================================================================== */

/* util.c:42-49 -- position of f(m,l) in the linearised coefficient array:
 * m = 0..bw-1 (each order a run l = m..bw-1), then m = -(bw-1)..-1. */
int orc_index_of_harmonic_coeff(int m, int l, int bw) {
    int L = bw - 1;
    if (m >= 0) return m * bw - (m * (m - 1)) / 2 + (l - m);
    int am = -m;
    return (L * (L + 3)) / 2 + 1 + ((L - am) * (L - am + 1)) / 2 + (l - am);
}

/* cospml.c:250-258 -- stored (non-zero, parity-matching) cosine coefficients of
 * P(m,l) (m even: frequencies l%2..l) or G(m,l)=P(m,l)/sin (m odd: ..l-1). */
int orc_row_size(int m, int l) {
    if (l < m) return 0;
    return (m % 2 == 0) ? (l / 2) + 1 : ((l - 1) / 2) + 1;
}

/* sum_{l'=0}^{n-1} (l'/2 + 1) */
static int64_t prefix_even(int64_t n) {
    if (n <= 0) return 0;
    int64_t q = n / 2, r = n % 2;
    return q * (q - 1) + r * q + n;
}

/* cospml.c:123-134 -- offset of row l inside the order-m table = sum of row sizes m..l-1. */
int64_t orc_table_offset(int m, int l) {
    if (m % 2 == 0) return prefix_even(l) - prefix_even(m);
    return prefix_even(l - 1) - prefix_even(m - 1);
}

/* cospml.c:39-59 -- entries in the order-m table = sum_{l=m}^{bw-1} RowSize(m,l). */
int64_t orc_table_size(int m, int bw) { return orc_table_offset(m, bw); }

/* first degree l whose cosine series contains frequency `row` (see inverse below) */
static int trans_first_l(int row, int m) {
    return (row > m) ? row + (m % 2) : m + (row % 2);
}

/* cospml.c:270-288 -- number of degrees l < bw whose series holds frequency `row`
 * (l = l0, l0+2, ...).  Equal to the reference for even bw; for odd bw the reference
 * undercounts even rows (S2kit 1.1 odd-bandwidth defect) and this returns the true count. */
int orc_transpose_row_size(int row, int m, int bw) {
    if (row >= bw) return 0;
    int l0 = trans_first_l(row, m);
    if (l0 >= bw) return 0;
    return (bw - l0 + 1) / 2;
}

/* cospml.c:107-115 */
int64_t orc_reduced_spharmonic_table_size(int bw, int cutoff) {
    int64_t s = 0;
    for (int m = 0; m < cutoff; ++m) s += orc_table_size(m, bw);
    return s;
}

/* cospml.c:434-440 */
int64_t orc_reduced_naive_table_size(int bw, int cutoff) {
    int64_t s = 0;
    for (int m = cutoff; m < bw; ++m) s += bw - m;
    return 2 * (int64_t)bw * s;
}

/* ===================================================================== */
/* FFT (radix-2 for powers of two, direct DFT otherwise)                  */
/* ===================================================================== */

typedef struct fft_plan {
    int n, pow2, logn;
    double* c;   /* cos(2 pi k / n), k < n */
    double* s;   /* sin(2 pi k / n) */
    int* rev;    /* bit reversal (pow2 only) */
    struct fft_plan* next;
} fft_plan;

static pthread_mutex_t plan_lock = PTHREAD_MUTEX_INITIALIZER;
static fft_plan* plan_list = NULL;

static const fft_plan* get_plan(int n) {
    pthread_mutex_lock(&plan_lock);
    for (fft_plan* p = plan_list; p; p = p->next)
        if (p->n == n) {
            pthread_mutex_unlock(&plan_lock);
            return p;
        }
    fft_plan* p = (fft_plan*)calloc(1, sizeof(fft_plan));
    p->n = n;
    p->pow2 = (n & (n - 1)) == 0;
    p->c = (double*)malloc(sizeof(double) * n);
    p->s = (double*)malloc(sizeof(double) * n);
    for (int k = 0; k < n; ++k) {
        double a = 2.0 * ORC_PI * (double)k / (double)n;
        p->c[k] = cos(a);
        p->s[k] = sin(a);
    }
    if (p->pow2) {
        int lg = 0;
        while ((1 << lg) < n) ++lg;
        p->logn = lg;
        p->rev = (int*)malloc(sizeof(int) * n);
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < lg; ++b)
                if (i & (1 << b)) r |= 1 << (lg - 1 - b);
            p->rev[i] = r;
        }
    }
    p->next = plan_list;
    plan_list = p;
    pthread_mutex_unlock(&plan_lock);
    return p;
}

/* In-place unnormalised DFT: X[k] = sum_j x[j] exp(sign * 2 pi i j k / n). */
void orc_dft(int n, double* re, double* im, int sign) {
    if (n <= 1) return;
    const fft_plan* p = get_plan(n);
    double sg = (sign < 0) ? -1.0 : 1.0;
    if (!p->pow2) {
        double* tr = (double*)malloc(sizeof(double) * 2 * n);
        double* ti = tr + n;
        for (int k = 0; k < n; ++k) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < n; ++j) {
                int idx = (int)(((int64_t)j * k) % n);
                double c = p->c[idx], s = sg * p->s[idx];
                sr += re[j] * c - im[j] * s;
                si += re[j] * s + im[j] * c;
            }
            tr[k] = sr;
            ti[k] = si;
        }
        memcpy(re, tr, sizeof(double) * n);
        memcpy(im, ti, sizeof(double) * n);
        free(tr);
        return;
    }
    for (int i = 0; i < n; ++i) {
        int r = p->rev[i];
        if (r > i) {
            double t = re[i]; re[i] = re[r]; re[r] = t;
            t = im[i]; im[i] = im[r]; im[r] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int b = 0; b < n; b += len) {
            for (int j = 0; j < half; ++j) {
                double c = p->c[j * step], s = sg * p->s[j * step];
                int a0 = b + j, a1 = a0 + half;
                double xr = re[a1] * c - im[a1] * s;
                double xi = re[a1] * s + im[a1] * c;
                re[a1] = re[a0] - xr;
                im[a1] = im[a0] - xi;
                re[a0] += xr;
                im[a0] += xi;
            }
        }
    }
}

/* ---- DCTs ---- */

/* Direct definitions; the angle pi (2j+1) k / (2n) is reduced exactly modulo 2 pi
 * (integer (2j+1) k mod 4n) so the O(n^2) sums stay accurate for large n. */
void orc_redft10_direct(int n, const double* in, double* out) {
    const fft_plan* q = get_plan(4 * n); /* cos(2 pi r / 4n) = cos(pi r / 2n) */
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s += in[j] * q->c[(int)(((int64_t)(2 * j + 1) * k) % (4 * n))];
        out[k] = 2.0 * s;
    }
}

void orc_redft01_direct(int n, const double* in, double* out) {
    const fft_plan* q = get_plan(4 * n);
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int j = 1; j < n; ++j) s += in[j] * q->c[(int)(((int64_t)j * (2 * k + 1)) % (4 * n))];
        out[k] = in[0] + 2.0 * s;
    }
}

/* DCT-II through one length-n complex DFT of the even/odd-reordered input
 * (v[j] = x[2j], v[n-1-j] = x[2j+1]); Y[k] = 2 Re(exp(-i pi k / 2n) V[k]). */
void orc_redft10(int n, const double* in, double* out) {
    if (n % 2 || (n & (n - 1))) {
        orc_redft10_direct(n, in, out);
        return;
    }
    double* vr = (double*)malloc(sizeof(double) * 2 * n);
    double* vi = vr + n;
    for (int j = 0; j < n / 2; ++j) {
        vr[j] = in[2 * j];
        vr[n - 1 - j] = in[2 * j + 1];
    }
    memset(vi, 0, sizeof(double) * n);
    orc_dft(n, vr, vi, -1);
    const fft_plan* q = get_plan(4 * n); /* exp(-i pi k / 2n) = exp(-2 pi i k / 4n) */
    for (int k = 0; k < n; ++k) out[k] = 2.0 * (vr[k] * q->c[k] + vi[k] * q->s[k]);
    free(vr);
}

/* DCT-III: Z[k] = exp(i pi k / 2n) (X[k] - i X[n-k]) (X[n] = 0); z = sum_k Z[k] exp(+2 pi i jk/n);
 * out[2j] = Re z[j], out[2j+1] = Re z[n-1-j]. */
void orc_redft01(int n, const double* in, double* out) {
    if (n % 2 || (n & (n - 1))) {
        orc_redft01_direct(n, in, out);
        return;
    }
    double* zr = (double*)malloc(sizeof(double) * 2 * n);
    double* zi = zr + n;
    const fft_plan* q = get_plan(4 * n);
    for (int k = 0; k < n; ++k) {
        double a = in[k], b = (k == 0) ? 0.0 : -in[n - k];
        double c = q->c[k], s = q->s[k];
        zr[k] = a * c - b * s;
        zi[k] = a * s + b * c;
    }
    orc_dft(n, zr, zi, +1);
    for (int j = 0; j < n / 2; ++j) {
        out[2 * j] = zr[j];
        out[2 * j + 1] = zr[n - 1 - j];
    }
    free(zr);
}

/* ===================================================================== */
/* Table generation                                                      */
/* ===================================================================== */

/* pmm.c:21-34 -- L2-normalised P(m,m)(cos theta), Condon-Shortley sign for odd m. */
void orc_pmm_l2(int m, const double* eval_points, int n, double* result) {
    double c = sqrt(m + 0.5);
    for (int i = 0; i < m; ++i) c *= sqrt((m - (i / 2.0)) / ((double)m - i));
    if (m) c *= pow(2.0, -m / 2.0);
    if (m % 2) c = -c;
    for (int i = 0; i < n; ++i) result[i] = c * pow(sin(eval_points[i]), m);
}

/* l2_norms.c:16-22 */
double orc_l2_an(int m, int l) {
    return sqrt(((2.0 * l + 3.0) / (2.0 * l + 1.0)) * ((l - m + 1.0) / (l + m + 1.0))) *
           ((2.0 * l + 1.0) / (l - m + 1.0));
}

/* l2_norms.c:28-38 */
double orc_l2_cn(int m, int l) {
    if (l == 0) return 0.0;
    return -sqrt(((2.0 * l + 3.0) / (2.0 * l - 1.0)) * ((l - m + 1.0) / (l + m + 1.0)) *
                 (((double)l - m) / ((double)l + m))) *
           ((l + m) / (l - m + 1.0));
}

/* weights.c:32-47 -- Driscoll-Healy quadrature weights; [0,2bw) even orders,
 * [2bw,4bw) odd orders (extra sin(theta_j) factor). */
void orc_generate_weights(int bw, double* weights) {
    double h = ORC_PI / (4.0 * bw);
    for (int j = 0; j < 2 * bw; ++j) {
        double k = 2.0 * j + 1.0;
        double s = 0.0;
        for (int q = 0; q < bw; ++q) s += 1.0 / (2.0 * q + 1.0) * sin(k * (2.0 * q + 1.0) * h);
        s *= 2.0 * sin(k * h) / bw;
        weights[j] = s;
        weights[j + 2 * bw] = s * sin(k * h);
    }
}

/* DCT of length bw with the table normalisation of cospml.c:203-208:
 * out = REDFT10(in); out[0] *= sqrt(1/2); out *= 1/sqrt(bw). */
static void table_dct(int bw, const double* in, double* out) {
    orc_redft10(bw, in, out);
    out[0] *= ORC_SQRT1_2;
    double f = 1.0 / sqrt((double)bw);
    for (int i = 0; i < bw; ++i) out[i] *= f;
}

/* cospml.c:161-242 -- cosine series of P(m,l) (m even) or G(m,l) = P(m,l)/sin (m odd),
 * l = m..bw-1, sampled at bw Chebyshev nodes, zero-striped entries dropped. */
void orc_generate_cos_pml_table(int bw, int m, double* table) {
    double* buf = (double*)calloc((size_t)6 * bw, sizeof(double));
    double *pp = buf, *p = buf + bw, *cur = buf + 2 * bw, *x = buf + 3 * bw, *th = buf + 4 * bw,
           *cs = buf + 5 * bw;
    for (int i = 0; i < bw; ++i) {
        th[i] = (2.0 * i + 1.0) * ORC_PI / (2.0 * bw);
        x[i] = cos(th[i]);
        pp[i] = 0.0;
    }
    if (m == 0)
        for (int i = 0; i < bw; ++i) p[i] = ORC_SQRT1_2;
    else
        orc_pmm_l2(m, th, bw, p);
    if (m % 2)
        for (int i = 0; i < bw; ++i) p[i] /= sin(th[i]);

    int deg = (m % 2 == 0) ? m : m - 1; /* polynomial degree of the current function */
    table_dct(bw, p, cs);
    double* out = table;
    for (int f = 0; f <= deg; f += 2) *out++ = cs[f];

    for (int i = 0; i < bw - m - 1; ++i) {
        double an = orc_l2_an(m, m + i), cn = orc_l2_cn(m, m + i);
        for (int q = 0; q < bw; ++q) cur[q] = an * (p[q] * x[q]) + cn * pp[q];
        table_dct(bw, cur, cs);
        ++deg;
        for (int f = (i % 2) ? 0 : 1; f <= deg; f += 2) *out++ = cs[f];
        double* t = pp;
        pp = p;
        p = cur;
        cur = t;
    }
    free(buf);
}

/* cospml.c:301-362 -- transposed table: row i lists T(l, frequency i) for the degrees
 * l = l0(i), l0+2, ... < bw whose series contain frequency i (l0 from trans_first_l). */
void orc_transpose_cos_pml_table(int bw, int m, const double* table, double* result) {
    double* out = result;
    for (int i = 0; i < bw; ++i) {
        int rs = orc_transpose_row_size(i, m, bw);
        int l = trans_first_l(i, m);
        for (int j = 0; j < rs; ++j, l += 2) {
            int t = (l - m) % 2; /* frequency i = 2 * idx + t inside row l */
            int idx = (i - t) / 2;
            *out++ = table[orc_table_offset(m, l) + idx];
        }
    }
}

/* pml.c:41-79 -- P(m,l) sampled at the 2bw Chebyshev nodes, rows l = m..bw-1. */
void orc_generate_pml_table(int bw, int m, double* table) {
    int n = 2 * bw;
    double* buf = (double*)malloc(sizeof(double) * 5 * n);
    double *pp = buf, *p = buf + n, *cur = buf + 2 * n, *x = buf + 3 * n, *th = buf + 4 * n;
    for (int i = 0; i < n; ++i) {
        th[i] = (2.0 * i + 1.0) * ORC_PI / (2.0 * n);
        x[i] = cos(th[i]);
        pp[i] = 0.0;
    }
    if (m == 0)
        for (int i = 0; i < n; ++i) p[i] = ORC_SQRT1_2;
    else
        orc_pmm_l2(m, th, n, p);
    memcpy(table, p, sizeof(double) * n);
    for (int i = 0; i < bw - m - 1; ++i) {
        double an = orc_l2_an(m, m + i), cn = orc_l2_cn(m, m + i);
        for (int q = 0; q < n; ++q) cur[q] = an * (p[q] * x[q]) + cn * pp[q];
        memcpy(table + (int64_t)(i + 1) * n, cur, sizeof(double) * n);
        double* t = pp;
        pp = p;
        p = cur;
        cur = t;
    }
    free(buf);
}

/* One order of the packed tables: cosine table and its transpose (m < cutoff) or sampled
 * P(m,l) in both buffers (m >= cutoff). */
static void tables_order(orc_tables* t, int m) {
    int bw = t->bw;
    double* f = t->fwd + t->offsets[m];
    double* v = t->inv + t->offsets[m];
    if (m < t->cutoff) {
        orc_generate_cos_pml_table(bw, m, f);
        orc_transpose_cos_pml_table(bw, m, f, v);
    } else {
        orc_generate_pml_table(bw, m, f);
        memcpy(v, f, sizeof(double) * 2 * (int64_t)bw * (bw - m));
    }
}

typedef struct {
    orc_tables* t;
    int tid, nthreads;
} tables_arg;

static void* tables_worker(void* vp) {
    tables_arg* a = (tables_arg*)vp;
    for (int m = a->tid; m < a->t->bw; m += a->nthreads) tables_order(a->t, m);
    return NULL;
}

/* cospml.c:451-518 -- seminaive orders m < cutoff (cosine tables), naive orders
 * m >= cutoff (sampled P(m,l)), packed back to back; inverse buffer transposed.  Orders are
 * independent, so `nthreads` threads may generate them (same values as one thread). */
orc_tables* orc_tables_new_mt(int bw, int cutoff, int nthreads) {
    orc_tables* t = (orc_tables*)calloc(1, sizeof(orc_tables));
    t->bw = bw;
    t->cutoff = cutoff;
    t->offsets = (int64_t*)malloc(sizeof(int64_t) * bw);
    int64_t off = 0;
    for (int m = 0; m < bw; ++m) {
        t->offsets[m] = off;
        off += (m < cutoff) ? orc_table_size(m, bw) : 2 * (int64_t)bw * (bw - m);
    }
    t->total = off;
    t->fwd = (double*)malloc(sizeof(double) * (off ? off : 1));
    t->inv = (double*)malloc(sizeof(double) * (off ? off : 1));
    get_plan(bw);
    get_plan(4 * bw);
    if (nthreads <= 1) {
        for (int m = 0; m < bw; ++m) tables_order(t, m);
        return t;
    }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    tables_arg* args = (tables_arg*)malloc(sizeof(tables_arg) * nthreads);
    for (int i = 0; i < nthreads; ++i) {
        args[i].t = t;
        args[i].tid = i;
        args[i].nthreads = nthreads;
        pthread_create(&th[i], NULL, tables_worker, &args[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(th);
    free(args);
    return t;
}

orc_tables* orc_tables_new(int bw, int cutoff) { return orc_tables_new_mt(bw, cutoff, 1); }

void orc_tables_free(orc_tables* t) {
    if (!t) return;
    free(t->offsets);
    free(t->fwd);
    free(t->inv);
    free(t);
}

int64_t orc_tables_total(const orc_tables* t) { return t->total; }
const double* orc_tables_fwd(const orc_tables* t) { return t->fwd; }
const double* orc_tables_inv(const orc_tables* t) { return t->inv; }
const int64_t* orc_tables_offsets(const orc_tables* t) { return t->offsets; }

/* ===================================================================== */
/* Legendre transforms                                                   */
/* ===================================================================== */

/* seminaive.c:153-198 -- weights (even/odd by order), REDFT10 of length 2bw,
 * c[0] *= sqrt(1/2), c *= 1/sqrt(4bw), then result[l-m] = sum_j c[2j+t] T(m,l)[j]. */
void orc_dlt_semi(const double* data, int bw, int m, double* result, const double* cos_pml_table,
                  const double* weights) {
    int n = 2 * bw;
    double* wd = (double*)malloc(sizeof(double) * 2 * n);
    double* c = wd + n;
    const double* w = weights + ((m % 2) ? n : 0);
    for (int i = 0; i < n; ++i) wd[i] = data[i] * w[i];
    orc_redft10(n, wd, c);
    c[0] *= ORC_SQRT1_2;
    double f = 1.0 / sqrt(2.0 * n);
    for (int i = 0; i < n; ++i) c[i] *= f;
    for (int l = m; l < bw; ++l) {
        const double* row = cos_pml_table + orc_table_offset(m, l);
        int t = (l - m) % 2, rs = orc_row_size(m, l);
        double s = 0.0;
        for (int j = 0; j < rs; ++j) s += c[2 * j + t] * row[j];
        result[l - m] = s;
    }
    free(wd);
}

/* seminaive.c:56-115 -- fcos[i] = 0.5/sqrt(bw) sum_j a(l0(i)+2j) Tt(i,j) (fcos[0] = sum/sqrt(2bw)),
 * REDFT01 of length 2bw, times sin(theta) for odd m. */
void orc_inv_dlt_semi(const double* coeffs, int bw, int m, double* result, const double* trans_cos_pml_table,
                      const double* sin_values) {
    int n = 2 * bw;
    double* fc = (double*)calloc((size_t)n, sizeof(double));
    const double* row = trans_cos_pml_table;
    double scale = 0.5 / sqrt((double)bw);
    for (int i = 0; i < bw; ++i) {
        int rs = orc_transpose_row_size(i, m, bw);
        if (rs == 0) continue;
        const double* a = coeffs + (trans_first_l(i, m) - m);
        double s = 0.0;
        for (int j = 0; j < rs; ++j) s += a[2 * j] * row[j];
        fc[i] = (i == 0) ? s / sqrt((double)n) : s * scale;
        row += rs;
    }
    orc_redft01(n, fc, result);
    if (m % 2)
        for (int i = 0; i < n; ++i) result[i] *= sin_values[i];
    free(fc);
}

/* naive.c:34-59 -- plain (even) weights for every order. */
void orc_dlt_naive(const double* data, int bw, int m, const double* weights, double* result,
                   const double* pml_table) {
    int n = 2 * bw;
    for (int l = 0; l < bw - m; ++l) {
        const double* row = pml_table + (int64_t)l * n;
        double s = 0.0;
        for (int j = 0; j < n; ++j) s += (data[j] * weights[j]) * row[j];
        result[l] = s;
    }
}

/* naive.c:78-96 */
void orc_inv_dlt_naive(const double* coeffs, int bw, int m, double* result, const double* pml_table) {
    int n = 2 * bw;
    memset(result, 0, sizeof(double) * n);
    for (int l = 0; l < bw - m; ++l) {
        double a = coeffs[l];
        if (a == 0.0) continue;
        const double* row = pml_table + (int64_t)l * n;
        for (int j = 0; j < n; ++j) result[j] += a * row[j];
    }
}

/* ===================================================================== */
/* Sphere transforms                                                     */
/* ===================================================================== */

/* One order's forward DLT (seminaive below cutoff, naive above). */
static void order_dlt(const double* data, int bw, int m, double* out, const orc_tables* t, const double* weights,
                      int cutoff) {
    const double* tab = t->fwd + t->offsets[m];
    if (m < cutoff)
        orc_dlt_semi(data, bw, m, out, tab, weights);
    else
        orc_dlt_naive(data, bw, m, weights, out, tab);
}

/* FST_semi_memo.c:68-202 */
void orc_fst(const double* rdata, const double* idata, double* rcoeffs, double* icoeffs, int bw,
             const orc_tables* t, const double* weights, int data_format, int cutoff) {
    int n = 2 * bw;
    double* rres = (double*)malloc(sizeof(double) * ((int64_t)2 * n * n + 4 * n));
    double* ires = rres + (int64_t)n * n;
    double* rowr = ires + (int64_t)n * n;
    double* rowi = rowr + n;
    double* fr = rowi + n;
    double* fi = fr + n;
    /* split DFT along phi; output transposed so that row m holds all latitudes (FST_semi_memo.c:81) */
    double nc = sqrt(2.0 * ORC_PI) / n; /* FST_semi_memo.c:86 */
    for (int j = 0; j < n; ++j) {
        memcpy(rowr, rdata + (int64_t)j * n, sizeof(double) * n);
        memcpy(rowi, idata + (int64_t)j * n, sizeof(double) * n);
        orc_dft(n, rowr, rowi, -1);
        for (int m = 0; m < n; ++m) {
            rres[(int64_t)m * n + j] = rowr[m] * nc;
            ires[(int64_t)m * n + j] = rowi[m] * nc;
        }
    }
    double* rp = rcoeffs;
    double* ip = icoeffs;
    for (int m = 0; m < bw; ++m) {
        order_dlt(rres + (int64_t)m * n, bw, m, fr, t, weights, cutoff);
        order_dlt(ires + (int64_t)m * n, bw, m, fi, t, weights, cutoff);
        memcpy(rp, fr, sizeof(double) * (bw - m));
        memcpy(ip, fi, sizeof(double) * (bw - m));
        rp += bw - m;
        ip += bw - m;
    }
    if (data_format == ORC_REAL) {
        /* f(l,-m) = (-1)^m conj(f(l,m)), FST_semi_memo.c:131-145 */
        for (int m = 1; m < bw; ++m) {
            double sg = (m % 2) ? -1.0 : 1.0;
            for (int l = m; l < bw; ++l) {
                int a = orc_index_of_harmonic_coeff(m, l, bw), b = orc_index_of_harmonic_coeff(-m, l, bw);
                rcoeffs[b] = sg * rcoeffs[a];
                icoeffs[b] = -sg * icoeffs[a];
            }
        }
    } else {
        /* negative orders from rows m' = n - |m|, FST_semi_memo.c:153-201 */
        for (int row = bw + 1; row < n; ++row) {
            int om = n - row;
            order_dlt(rres + (int64_t)row * n, bw, om, fr, t, weights, cutoff);
            order_dlt(ires + (int64_t)row * n, bw, om, fi, t, weights, cutoff);
            double sg = (row % 2) ? -1.0 : 1.0;
            for (int i = 0; i < bw - om; ++i) {
                rp[i] = sg * fr[i];
                ip[i] = sg * fi[i];
            }
            rp += bw - om;
            ip += bw - om;
        }
    }
    free(rres);
}

/* One order's inverse DLT into a length-2bw latitude vector. */
static void order_inv_dlt(const double* coeffs, int bw, int m, double* out, const orc_tables* t,
                          const double* sinv, int cutoff) {
    const double* tab = t->inv + t->offsets[m];
    if (m < cutoff)
        orc_inv_dlt_semi(coeffs, bw, m, out, tab, sinv);
    else
        orc_inv_dlt_naive(coeffs, bw, m, out, tab);
}

/* FST_semi_memo.c:228-351 */
void orc_inv_fst(const double* rcoeffs, const double* icoeffs, double* rdata, double* idata, int bw,
                 const orc_tables* t, int data_format, int cutoff) {
    int n = 2 * bw;
    double* rf = (double*)calloc((size_t)((int64_t)2 * n * n + 3 * n), sizeof(double));
    double* imf = rf + (int64_t)n * n;
    double* sinv = imf + (int64_t)n * n;
    double* rowr = sinv + n;
    double* rowi = rowr + n;
    for (int i = 0; i < n; ++i) sinv[i] = sin((2.0 * i + 1.0) * ORC_PI / (2.0 * n));
    const double* rp = rcoeffs;
    const double* ip = icoeffs;
    for (int m = 0; m < bw; ++m) {
        order_inv_dlt(rp, bw, m, rf + (int64_t)m * n, t, sinv, cutoff);
        order_inv_dlt(ip, bw, m, imf + (int64_t)m * n, t, sinv, cutoff);
        rp += bw - m;
        ip += bw - m;
    }
    /* row m = bw stays zero (FST_semi_memo.c:283-284) */
    if (data_format == ORC_COMPLEX) {
        for (int row = bw + 1; row < n; ++row) {
            int om = n - row;
            order_inv_dlt(rp, bw, om, rf + (int64_t)row * n, t, sinv, cutoff);
            order_inv_dlt(ip, bw, om, imf + (int64_t)row * n, t, sinv, cutoff);
            if (row % 2)
                for (int i = 0; i < n; ++i) {
                    rf[(int64_t)row * n + i] = -rf[(int64_t)row * n + i];
                    imf[(int64_t)row * n + i] = -imf[(int64_t)row * n + i];
                }
            rp += bw - om;
            ip += bw - om;
        }
    } else {
        for (int row = bw + 1; row < n; ++row) {
            memcpy(rf + (int64_t)row * n, rf + (int64_t)(n - row) * n, sizeof(double) * n);
            for (int i = 0; i < n; ++i) imf[(int64_t)row * n + i] = -imf[(int64_t)(n - row) * n + i];
        }
    }
    double nc = 1.0 / sqrt(2.0 * ORC_PI); /* FST_semi_memo.c:344 */
    /* inverse DFT along m per latitude: the reference runs the forward split DFT on
     * (imag, real) swapped arrays (FST_semi_memo.c:350), i.e. an unnormalised +i DFT. */
    for (int k = 0; k < n; ++k) {
        for (int m = 0; m < n; ++m) {
            rowr[m] = rf[(int64_t)m * n + k] * nc;
            rowi[m] = imf[(int64_t)m * n + k] * nc;
        }
        orc_dft(n, rowr, rowi, +1);
        memcpy(rdata + (int64_t)k * n, rowr, sizeof(double) * n);
        memcpy(idata + (int64_t)k * n, rowi, sizeof(double) * n);
    }
    free(rf);
}

/* FST_semi_memo.c:374-407 -- ires receives 2*bw zeros for REAL data, as in the reference. */
void orc_fzt(const double* rdata, const double* idata, double* rres, double* ires, int bw,
             const double* cos_pml_table_m0, const double* weights, int data_format) {
    int n = 2 * bw;
    double* r0 = (double*)malloc(sizeof(double) * 2 * n);
    double* i0 = r0 + n;
    double d = sqrt(2.0 * ORC_PI) / n;
    for (int i = 0; i < n; ++i) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < n; ++j) {
            sr += rdata[(int64_t)i * n + j];
            si += idata[(int64_t)i * n + j];
        }
        r0[i] = sr * d;
        i0[i] = si * d;
    }
    orc_dlt_semi(r0, bw, 0, rres, cos_pml_table_m0, weights);
    if (data_format == ORC_COMPLEX)
        orc_dlt_semi(i0, bw, 0, ires, cos_pml_table_m0, weights);
    else
        memset(ires, 0, sizeof(double) * n);
    free(r0);
}

/* util.c:68-103 with ComplexMult util.c:23-27 (imaginary part x*v - y*u as in the reference). */
void orc_transmult(const double* rdatacoeffs, const double* idatacoeffs, const double* rfiltercoeffs,
                   const double* ifiltercoeffs, double* rres, double* ires, int bw) {
    for (int m = -(bw - 1); m < bw; ++m) {
        int am = m < 0 ? -m : m;
        for (int l = am; l < bw; ++l) {
            int idx = orc_index_of_harmonic_coeff(m, l, bw);
            double x = rfiltercoeffs[l], y = ifiltercoeffs[l];
            double u = rdatacoeffs[idx], v = idatacoeffs[idx];
            double s = sqrt(4.0 * ORC_PI / (2.0 * l + 1.0));
            rres[idx] = (x * u - y * v) * s;
            ires[idx] = (x * v - y * u) * s;
        }
    }
}

/* FST_semi_memo.c:439-518 -- always REAL, seminaive at every order (cutoff = bw). */
void orc_conv(const double* rdata, const double* idata, const double* rfilter, const double* ifilter,
              double* rres, double* ires, int bw) {
    orc_tables* t = orc_tables_new(bw, bw);
    orc_conv_tables(rdata, idata, rfilter, ifilter, rres, ires, bw, t);
    orc_tables_free(t);
}

/* The convolution of orc_conv on tables the caller built (the reference regenerates them in
 * every call, FST_semi_memo.c:498-500; the values are the same). */
void orc_conv_tables(const double* rdata, const double* idata, const double* rfilter, const double* ifilter,
                     double* rres, double* ires, int bw, const orc_tables* t) {
    int nc = bw * bw;
    double* w = (double*)malloc(sizeof(double) * 4 * bw);
    orc_generate_weights(bw, w);
    double* fr = (double*)malloc(sizeof(double) * (4 * (int64_t)nc + 4 * bw));
    double* fi = fr + nc;
    double* tr = fi + nc;
    double* ti = tr + nc;
    double* hr = ti + nc;
    double* hi = hr + 2 * bw;
    orc_fst(rdata, idata, fr, fi, bw, t, w, ORC_REAL, bw);
    orc_fzt(rfilter, ifilter, hr, hi, bw, t->fwd, w, ORC_REAL);
    orc_transmult(fr, fi, hr, hi, tr, ti, bw);
    orc_inv_fst(tr, ti, rres, ires, bw, t, ORC_REAL, bw);
    free(fr);
    free(w);
}

/* ===================================================================== */
/* Multi-threaded CPU baseline                                           */
/* ===================================================================== */

typedef struct {
    int bw, nfunc, nthreads, tid;
    const orc_tables* t;
    const double* w;
    const double* in;
    double* out;
} bench_arg;

static void* bench_worker(void* vp) {
    bench_arg* a = (bench_arg*)vp;
    int bw = a->bw, n = 2 * bw, nc = bw * bw;
    double* grid = (double*)malloc(sizeof(double) * 2 * (int64_t)n * n);
    for (int f = a->tid; f < a->nfunc; f += a->nthreads) {
        const double* ci = a->in + (int64_t)f * 2 * nc;
        double* co = a->out + (int64_t)f * 2 * nc;
        orc_inv_fst(ci, ci + nc, grid, grid + (int64_t)n * n, bw, a->t, ORC_REAL, bw);
        orc_fst(grid, grid + (int64_t)n * n, co, co + nc, bw, a->t, a->w, ORC_REAL, bw);
    }
    free(grid);
    return NULL;
}

double orc_bench_roundtrip(int bw, int nfunc, int nthreads, const double* coeffs_in, double* coeffs_out) {
    orc_tables* t = orc_tables_new(bw, bw);
    double* w = (double*)malloc(sizeof(double) * 4 * bw);
    orc_generate_weights(bw, w);
    get_plan(2 * bw);
    get_plan(8 * bw);
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    bench_arg* args = (bench_arg*)malloc(sizeof(bench_arg) * nthreads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int i = 0; i < nthreads; ++i) {
        bench_arg b = {bw, nfunc, nthreads, i, t, w, coeffs_in, coeffs_out};
        args[i] = b;
        pthread_create(&th[i], NULL, bench_worker, &args[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    free(args);
    free(w);
    orc_tables_free(t);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
