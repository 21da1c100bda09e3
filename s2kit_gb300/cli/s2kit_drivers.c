/*
 * s2kit_drivers.c -- the reference's command-line test programs, on the GPU.
 *
 * One executable; the program is chosen by the name it is run under (the build links
 * bin/<name> to it) or by a first argument naming it.  Each keeps the arguments, input parsing
 * and output formats of the reference program it replaces:
 *
 *   test_s2_semi_memo_fwd sample_file output_file bw [output_format]  test/test_s2_semi_memo_fwd.c
 *   test_s2_semi_memo_inv coeffs_file output_file bw                  test/test_s2_semi_memo_inv.c
 *   test_s2_semi_memo bw loops [error_file]                           test/test_s2_semi_memo.c
 *   test_s2_semi_fly bw loops [error_file]                            test/test_s2_semi_fly.c
 *   test_conv_semi_memo signal_file filter_file output_file bw        test/test_conv_semi_memo.c
 *   test_conv_semi_fly signal_file filter_file output_file bw         test/test_conv_semi_fly.c
 *   test_DLT_semi m bw loops                                          test/test_DLT_semi.c
 *   test_DLT_naive m bw loops                                         test/test_DLT_naive.c
 *
 * Sample files hold 4 bw^2 (re, im) pairs latitude-major, coefficient files bw^2 (re, im)
 * pairs in IndexOfHarmonicCoeff order, convolution files 4 bw^2 real values; values are read
 * with "%lf" and written with the reference's printf formats.  Times are wall clock around
 * the library call (the reference's WALLCLOCK build).  Where the reference reads past a short
 * or missing file without noticing, these programs stop with an error message.
 */
#define _DEFAULT_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "s2kit_gb300.h"

static double wall(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static double* alloc(size_t n) {
    double* p = (double*)calloc(n ? n : 1, sizeof(double));
    if (!p) {
        fprintf(stderr, "out of memory (%zu doubles)\n", n);
        exit(1);
    }
    return p;
}

static void read_values(const char* path, double* a, double* b, size_t n) {
    FILE* fp = fopen(path, "r");
    if (!fp) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(1);
    }
    for (size_t i = 0; i < n; ++i) {
        if (fscanf(fp, "%lf", a + i) != 1 || (b && fscanf(fp, "%lf", b + i) != 1)) {
            fprintf(stderr, "%s: expected %zu values%s, found fewer\n", path, n, b ? " pairs" : "");
            exit(1);
        }
    }
    fclose(fp);
}

static FILE* open_out(const char* path) {
    FILE* fp = fopen(path, "w");
    if (!fp) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(1);
    }
    return fp;
}

static int check_error(const char* what) {
    const char* e = s2g_last_error();
    if (e && e[0]) {
        fprintf(stderr, "%s: %s\n", what, e);
        return 1;
    }
    return 0;
}

/* ---- forward transform of a sample file (COMPLEX data, cutoff = bw) ---- */
static int fst_file(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stdout, "Usage: test_s2_semi_memo_fwd sample_file output_file bw [output_format]\n");
        return 0;
    }
    const int bw = atoi(argv[3]), size = 2 * bw, cutoff = bw;
    if (bw < 1) return fprintf(stderr, "bw must be positive\n"), 1;
    double *rdata = alloc((size_t)size * size), *idata = alloc((size_t)size * size);
    read_values(argv[1], rdata, idata, (size_t)size * size);
    double* tablespace = alloc((size_t)Reduced_Naive_TableSize(bw, cutoff) + Reduced_SpharmonicTableSize(bw, cutoff) +
                               4 * (size_t)bw);
    fprintf(stdout, "Generating seminaive_naive tables...\n");
    double** table = SemiNaive_Naive_Pml_Table(bw, cutoff, tablespace, NULL);
    double* weights = alloc(4 * (size_t)bw);
    GenerateWeightsForDLT(bw, weights);
    double *rc = alloc((size_t)bw * bw), *ic = alloc((size_t)bw * bw);
    const double t0 = wall();
    FSTSemiMemo(rdata, idata, rc, ic, bw, table, NULL, COMPLEX, cutoff, NULL, NULL, weights);
    fprintf(stdout, "forward time \t = %.4e\n", wall() - t0);
    if (check_error("FSTSemiMemo")) return 1;
    fprintf(stdout, "about to write out coefficients\n");
    const int order = argc == 5 ? atoi(argv[4]) : 0;
    FILE* fp = open_out(argv[2]);
    if (order == 0) {
        for (int i = 0; i < bw * bw; ++i) fprintf(fp, "%.15f\n%.15f\n", rc[i], ic[i]);
    } else {
        for (int l = 0; l < bw; ++l)
            for (int m = -l; m < l + 1; ++m) {
                const int k = IndexOfHarmonicCoeff(m, l, bw);
                fprintf(fp, "l = %d\t m = %d\t %.15f + %.15f I\n", l, m, rc[k], ic[k]);
            }
    }
    fclose(fp);
    fprintf(stdout, "finished writing coefficients\n");
    free(table), free(tablespace), free(weights), free(rc), free(ic), free(rdata), free(idata);
    return 0;
}

/* ---- inverse transform of a coefficient file ---- */
static int inv_file(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stdout, "Usage: test_s2_semi_memo_inv coeffs_file output_file bw\n");
        return 0;
    }
    const int bw = atoi(argv[3]), size = 2 * bw, cutoff = bw;
    if (bw < 1) return fprintf(stderr, "bw must be positive\n"), 1;
    double *rc = alloc((size_t)bw * bw), *ic = alloc((size_t)bw * bw);
    read_values(argv[1], rc, ic, (size_t)bw * bw);
    const size_t tsize = (size_t)Reduced_Naive_TableSize(bw, cutoff) + Reduced_SpharmonicTableSize(bw, cutoff);
    double *fwdspace = alloc(tsize + 4 * (size_t)bw), *invspace = alloc(tsize + 4 * (size_t)bw);
    fprintf(stdout, "Generating seminaive_naive tables...\n");
    double** table = SemiNaive_Naive_Pml_Table(bw, cutoff, fwdspace, NULL);
    fprintf(stdout, "Generating trans_seminaive_naive tables...\n");
    double** ttable = Transpose_SemiNaive_Naive_Pml_Table(table, bw, cutoff, invspace, NULL);
    double *rdata = alloc((size_t)size * size), *idata = alloc((size_t)size * size);
    const double t0 = wall();
    InvFSTSemiMemo(rc, ic, rdata, idata, bw, ttable, NULL, COMPLEX, cutoff, NULL, NULL);
    fprintf(stderr, "inv time \t = %.4e\n", wall() - t0);
    if (check_error("InvFSTSemiMemo")) return 1;
    fprintf(stdout, "about to write out samples\n");
    FILE* fp = open_out(argv[2]);
    for (int i = 0; i < size * size; ++i) fprintf(fp, "%.15f\n%.15f\n", rdata[i], idata[i]);
    fclose(fp);
    fprintf(stdout, "finished writing samples\n");
    free(ttable), free(table), free(fwdspace), free(invspace), free(rc), free(ic), free(rdata), free(idata);
    return 0;
}

/* ---- convolution of a signal with a filter (real data) ---- */
static int conv_file(int argc, char** argv, int fly) {
    const char* name = fly ? "test_conv_semi_fly" : "test_conv_semi_memo";
    if (argc < 5) {
        fprintf(stdout, "Usage: %s signal_file filter_file output_file bw\n", name);
        return 0;
    }
    const int bw = atoi(argv[4]), size = 2 * bw;
    if (bw < 1) return fprintf(stderr, "bw must be positive\n"), 1;
    const size_t n = (size_t)size * size;
    double *rs = alloc(n), *rf = alloc(n), *is = alloc(n), *iff = alloc(n), *rr = alloc(n), *ir = alloc(n);
    fprintf(stdout, "Reading signal file...\n");
    read_values(argv[1], rs, NULL, n);
    fprintf(stdout, "Reading filter file...\n");
    read_values(argv[2], rf, NULL, n);
    fprintf(stdout, "Calling %s()\n", fly ? "ConvOn2SphereSemiFly" : "ConvOn2SphereSemiMemo");
    if (fly)
        ConvOn2SphereSemiFly(rs, is, rf, iff, rr, ir, bw, NULL);
    else
        ConvOn2SphereSemiMemo(rs, is, rf, iff, rr, ir, bw, NULL);
    if (check_error(name)) return 1;
    fprintf(stdout, "Writing output file...\n");
    FILE* fp = open_out(argv[3]);
    for (size_t i = 0; i < n; ++i) fprintf(fp, "%.16f\n", rr[i]);
    fclose(fp);
    free(rs), free(rf), free(is), free(iff), free(rr), free(ir);
    return 0;
}

static void stats(const double* v, int loops, double* avg, double* sd) {
    double s = 0.0, q = 0.0;
    for (int i = 0; i < loops; ++i) s += v[i];
    *avg = s / loops;
    for (int i = 0; i < loops; ++i) q += (*avg - v[i]) * (*avg - v[i]);
    *sd = loops != 1 ? sqrt(q / (loops - 1)) : 0.0;
}

/* ---- round trips of random coefficients (COMPLEX data holding a real field) ---- */
static int roundtrip(int argc, char** argv, int fly) {
    const char* name = fly ? "test_s2_semi_fly" : "test_s2_semi_memo";
    if (argc < 3) {
        fprintf(stdout, "Usage: %s bw loops [error_file]\n", name);
        return 0;
    }
    const int bw = atoi(argv[1]), loops = atoi(argv[2]), size = 2 * bw, cutoff = bw;
    if (bw < 1 || loops < 1) return fprintf(stderr, "bw and loops must be positive\n"), 1;
    double** table = NULL;
    double** ttable = NULL;
    double *fwdspace = NULL, *invspace = NULL;
    if (!fly) {
        const size_t tsize = (size_t)Reduced_Naive_TableSize(bw, cutoff) + Reduced_SpharmonicTableSize(bw, cutoff);
        fwdspace = alloc(tsize + 4 * (size_t)bw);
        invspace = alloc(tsize + 4 * (size_t)bw);
        fprintf(stdout, "Generating seminaive_naive tables...\n");
        table = SemiNaive_Naive_Pml_Table(bw, cutoff, fwdspace, NULL);
        fprintf(stdout, "Generating trans_seminaive_naive tables...\n");
        ttable = Transpose_SemiNaive_Naive_Pml_Table(table, bw, cutoff, invspace, NULL);
    }
    double* weights = alloc(4 * (size_t)bw);
    GenerateWeightsForDLT(bw, weights);
    const size_t nc = (size_t)bw * bw, ng = (size_t)size * size;
    double *rc = alloc(nc), *ic = alloc(nc), *rr = alloc(nc), *ir = alloc(nc), *rd = alloc(ng), *id = alloc(ng);
    double *relerror = alloc(loops), *curmax = alloc(loops);
    double fwd_time = 0.0, inv_time = 0.0;
    srand48((long)time(NULL));
    fprintf(stdout, "about to enter loop\n\n");
    for (int i = 0; i < loops; ++i) {
        for (int m = 0; m < bw; ++m)
            for (int l = m; l < bw; ++l) {
                const double x = 2.0 * (drand48() - 0.5), y = 2.0 * (drand48() - 0.5);
                int k = IndexOfHarmonicCoeff(m, l, bw);
                rc[k] = x, ic[k] = y;
                k = IndexOfHarmonicCoeff(-m, l, bw);
                rc[k] = (m & 1 ? -1.0 : 1.0) * x, ic[k] = (m & 1 ? 1.0 : -1.0) * y;
            }
        for (int m = 0; m < bw; ++m) ic[m] = 0.0;  // the m = 0 coefficients of a real field are real
        double t0 = wall();
        if (fly)
            InvFSTSemiFly(rc, ic, rd, id, bw, NULL, COMPLEX, cutoff, NULL, NULL);
        else
            InvFSTSemiMemo(rc, ic, rd, id, bw, ttable, NULL, COMPLEX, cutoff, NULL, NULL);
        double dt = wall() - t0;
        inv_time += dt;
        fprintf(stdout, "inv time \t = %.4e\n", dt);
        t0 = wall();
        if (fly)
            FSTSemiFly(rd, id, rr, ir, bw, NULL, COMPLEX, cutoff, NULL, NULL, weights);
        else
            FSTSemiMemo(rd, id, rr, ir, bw, table, NULL, COMPLEX, cutoff, NULL, NULL, weights);
        dt = wall() - t0;
        fwd_time += dt;
        fprintf(stdout, "forward time \t = %.4e\n", dt);
        if (check_error(name)) return 1;
        relerror[i] = curmax[i] = 0.0;
        for (size_t j = 0; j < nc; ++j) {
            const double dr = rr[j] - rc[j], di = ir[j] - ic[j];
            const double om = sqrt(rc[j] * rc[j] + ic[j] * ic[j]), em = sqrt(dr * dr + di * di);
            relerror[i] = fmax(relerror[i], em / (om + 1e-50));
            curmax[i] = fmax(curmax[i], em);
        }
        fprintf(stdout, "r-o error\t = %.12f\n", curmax[i]);
        fprintf(stdout, "(r-o)/o error\t = %.12f\n\n", relerror[i]);
    }
    double ae, se, ar, sr;
    stats(curmax, loops, &ae, &se);
    stats(relerror, loops, &ar, &sr);
    fprintf(stdout, "Program: %s\n", name);
    fprintf(stdout, "Bandwidth = %d\n", bw);
    fprintf(stdout, "Total elapsed wall time :\t\t %.4e seconds.\n", inv_time + fwd_time);
    fprintf(stdout, "Average wall forward per iteration:\t %.4e seconds.\n", fwd_time / loops);
    fprintf(stdout, "Average wall inverse per iteration:\t %.4e seconds.\n", inv_time / loops);
    fprintf(stdout, "Average r-o error:\t\t %.4e\t", ae);
    fprintf(stdout, "std dev: %.4e\n", se);
    fprintf(stdout, "Average (r-o)/o error:\t\t %.4e\t", ar);
    fprintf(stdout, "std dev: %.4e\n\n", sr);
    if (argc == 4) {
        FILE* fp = open_out(argv[3]);
        for (int m = 0; m < bw; ++m)
            for (int l = m; l < bw; ++l) {
                int k = IndexOfHarmonicCoeff(m, l, bw);
                fprintf(fp, "index = %d\t m = %d\tl = %d\t%.10f  %.10f\n", k, m, l, fabs(rc[k] - rr[k]),
                        fabs(ic[k] - ir[k]));
                k = IndexOfHarmonicCoeff(-m, l, bw);
                fprintf(fp, "index = %d\t m = %d\tl = %d\t%.10f  %.10f\n", k, -m, l, fabs(rc[k] - rr[k]),
                        fabs(ic[k] - ir[k]));
            }
        fclose(fp);
    }
    free(table), free(ttable), free(fwdspace), free(invspace), free(weights);
    free(rc), free(ic), free(rr), free(ir), free(rd), free(id), free(relerror), free(curmax);
    return 0;
}

/* ---- 1-D Legendre transforms of one order: inverse then forward, errors and times ---- */
static int dlt(int argc, char** argv, int naive) {
    const char* name = naive ? "test_DLT_naive" : "test_DLT_semi";
    if (argc < 4) {
        fprintf(stdout, "Usage: %s m bw loops\n", name);
        return 0;
    }
    const int m = atoi(argv[1]), bw = atoi(argv[2]), loops = atoi(argv[3]), n = 2 * bw;
    if (bw < 1 || m < 0 || m >= bw || loops < 1) return fprintf(stderr, "need 0 <= m < bw and loops > 0\n"), 1;
    double *samples = alloc(n), *coeffs = alloc(bw - m), *out = alloc(bw - m);
    double *relerror = alloc(loops), *curmax = alloc(loops), *weights = alloc(4 * (size_t)bw);
    GenerateWeightsForDLT(bw, weights);
    double *table = NULL, *ttable = NULL, *sinv = NULL;
    if (naive) {
        table = alloc((size_t)n * (bw - m));
        GeneratePmlTable(bw, m, table, NULL);
    } else {
        table = alloc(TableSize(m, bw));
        ttable = alloc(TableSize(m, bw));
        GenerateCosPmlTable(bw, m, table, NULL);
        TransposeCosPmlTable(bw, m, table, ttable);
        double* args = alloc(n);
        sinv = alloc(n);
        AcosOfChebyshevNodes(n, args);
        for (int i = 0; i < n; ++i) sinv[i] = sin(args[i]);
        free(args);
    }
    double tf = 0.0, ti = 0.0;
    srand48((long)time(NULL));
    for (int k = 0; k < loops; ++k) {
        for (int i = 0; i < bw - m; ++i) coeffs[i] = 2.0 * (drand48() - 0.5);
        double t0 = wall();
        if (naive)
            InvDLTNaive(coeffs, bw, m, samples, table);
        else
            InvDLTSemi(coeffs, bw, m, samples, ttable, sinv, NULL, NULL);
        ti += wall() - t0;
        t0 = wall();
        if (naive)
            DLTNaive(samples, bw, m, weights, out, table, NULL);
        else
            DLTSemi(samples, bw, m, out, NULL, table, weights, NULL);
        tf += wall() - t0;
        if (check_error(name)) return 1;
        relerror[k] = curmax[k] = 0.0;
        for (int j = 0; j < bw - m; ++j) {
            const double e = fabs(coeffs[j] - out[j]);
            curmax[k] = fmax(curmax[k], e);
            relerror[k] = fmax(relerror[k], e / (fabs(coeffs[j]) + 1e-50));
        }
    }
    double ae, se, ar, sr;
    stats(curmax, loops, &ae, &se);
    stats(relerror, loops, &ar, &sr);
    fprintf(stdout, "bw = %d\tm = %d\n", bw, m);
    fprintf(stdout, "loops = %d\n", loops);
    fprintf(stdout, "Average r-o error:\t\t %.4e\t", ae);
    fprintf(stdout, "std dev: %.4e\n", se);
    fprintf(stdout, "Average (r-o)/o error:\t\t %.4e\t", ar);
    fprintf(stdout, "std dev: %.4e\n\n", sr);
    fprintf(stdout, "average forward time = %.4e\n", tf / loops);
    fprintf(stdout, "average inverse time = %.4e\n", ti / loops);
    free(samples), free(coeffs), free(out), free(relerror), free(curmax), free(weights), free(table);
    free(ttable), free(sinv);
    return 0;
}

int main(int argc, char** argv) {
    const char* prog = strrchr(argv[0], '/') ? strrchr(argv[0], '/') + 1 : argv[0];
    if (!strncmp(prog, "s2kit", 5) && argc > 1) {  // s2kit <program> args...
        prog = argv[1];
        ++argv;
        --argc;
    }
    if (!strcmp(prog, "test_s2_semi_memo_fwd")) return fst_file(argc, argv);
    if (!strcmp(prog, "test_s2_semi_memo_inv")) return inv_file(argc, argv);
    if (!strcmp(prog, "test_s2_semi_memo")) return roundtrip(argc, argv, 0);
    if (!strcmp(prog, "test_s2_semi_fly")) return roundtrip(argc, argv, 1);
    if (!strcmp(prog, "test_conv_semi_memo")) return conv_file(argc, argv, 0);
    if (!strcmp(prog, "test_conv_semi_fly")) return conv_file(argc, argv, 1);
    if (!strcmp(prog, "test_DLT_semi")) return dlt(argc, argv, 0);
    if (!strcmp(prog, "test_DLT_naive")) return dlt(argc, argv, 1);
    fprintf(stdout,
            "Usage: s2kit <program> args...\n  programs: test_s2_semi_memo_fwd, test_s2_semi_memo_inv, "
            "test_s2_semi_memo, test_s2_semi_fly, test_conv_semi_memo, test_conv_semi_fly, test_DLT_semi, "
            "test_DLT_naive\n");
    return 2;
}
