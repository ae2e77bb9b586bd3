/* Stand-in for the part of FFTW 3 (fftw3.h, single precision) that the reference's
 * gridFFT.cpp, gridFFT_CoilThreaded.cpp and ArrayTemplates.cpp call, so that they compile unmodified into
 * oracle/_ref (test infrastructure).  FFTW is not installed here.  Semantics follow FFTW's
 * documentation: unnormalised transforms, FFTW_FORWARD = -1 (exp(-2 pi i jk/n)),
 * FFTW_BACKWARD = +1, multi-dimensional arrays in row-major order (the last dimension
 * contiguous), a plan executable on other arrays with fftwf_execute_dft and from several
 * threads at once.  The transforms are computed in double precision and rounded to float
 * (refshim/fftw_shim.cpp); planner flags and wisdom are accepted and ignored;
 * fftwf_malloc / fftwf_free allocate and release like malloc / free, 16-byte aligned. */
#ifndef ORACLE_REFSHIM_FFTW3_H
#define ORACLE_REFSHIM_FFTW3_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef struct fftwf_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_3d(int n0, int n1, int n2, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft(int rank, const int *n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_destroy_plan(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
int fftwf_import_wisdom_from_file(FILE *f);
void fftwf_export_wisdom_to_file(FILE *f);
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int n);

#ifdef __cplusplus
}
#endif

#endif
