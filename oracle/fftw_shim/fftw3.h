/*
 * fftw3.h -- minimal FFTW3 API subset used by S2kit 1.1, implemented by fftw_shim.c.
 *
 * TEST INFRASTRUCTURE ONLY: lets oracle/Makefile compile the unmodified reference C sources
 * (FFTW3 is not installed in this image).  Only the six entry points the reference calls
 * exist: fftw_plan_r2r_1d, fftw_plan_guru_split_dft, fftw_execute, fftw_execute_r2r,
 * fftw_execute_split_dft, fftw_destroy_plan (call sites FST_semi_memo.c:81,350,461-495,514-517,
 * seminaive.c:107,170, cospml.c:203-204,224,241).  Enum values follow FFTW 3.3's public header.
 */
#ifndef S2_FFTW_SHIM_H
#define S2_FFTW_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fftw_plan_s* fftw_plan;

typedef struct {
    int n, is, os;
} fftw_iodim;

typedef enum {
    FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2,
    FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6,
    FFTW_RODFT00 = 7, FFTW_RODFT01 = 8, FFTW_RODFT10 = 9, FFTW_RODFT11 = 10
} fftw_r2r_kind;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_r2r_1d(int n, double* in, double* out, fftw_r2r_kind kind, unsigned flags);
fftw_plan fftw_plan_guru_split_dft(int rank, const fftw_iodim* dims, int howmany_rank,
                                   const fftw_iodim* howmany_dims, double* ri, double* ii, double* ro,
                                   double* io, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_r2r(const fftw_plan p, double* in, double* out);
void fftw_execute_split_dft(const fftw_plan p, double* ri, double* ii, double* ro, double* io);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
