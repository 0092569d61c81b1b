/* Declarations of the part of FFTW's single-precision interface that emsim's FFTW
 * extension calls (fftw_ext/src/WavePropagator.cpp, SliceBuilder.cpp), so that those
 * sources compile unchanged against fftw_stub.cpp, the oracle's own transforms.  Test
 * infrastructure only: nothing in the product links it.  The transforms follow FFTW's
 * documented conventions (unnormalised; FFTW_FORWARD = exp(-2 pi i jk / n); r2c keeps
 * the n/2 + 1 non-negative frequencies of the last dimension; c2r returns the real
 * inverse of the Hermitian array that the stored half defines). */
#ifndef EMSIM_ORACLE_FFTW3_H
#define EMSIM_ORACLE_FFTW3_H

#include <stddef.h>
/* FFTW's interface declares its plan printers with FILE *, so code written against it
 * gets the stdio declarations with it (the reference's WavePropagator.cpp relies on that) */
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef struct fftwf_plan_s* fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int nthreads);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int* n, int howmany, float* in, const int* inembed, int istride,
                                   int idist, fftwf_complex* out, const int* onembed, int ostride, int odist,
                                   unsigned flags);
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                                   int istride, int idist, float* out, const int* onembed, int ostride, int odist,
                                   unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
void* fftwf_malloc(size_t n);
void fftwf_free(void* p);

#ifdef __cplusplus
}
#endif

#endif
