/*
 * fftw3.h -- minimal FFTW3 single-precision API adaptor.
 *
 * TEST INFRASTRUCTURE (oracle only).  The reference hot path (Fourier.cpp,
 * Reco.cpp, Trajectory.cpp, IO.cpp of expRad/4d_lung CGSense) is compiled
 * unmodified against this header so that it can run here as the parity
 * reference.  FFTW itself is not installed; the calls below are served by the
 * oracle's own double-precision mixed-radix FFT (oracle_fft.h), rounding to
 * float only on store.  Declares exactly the FFTW entry points the reference
 * uses: Fourier.cpp:6-15,22,29 (plans, execute, wisdom), Reco.cpp alloc/free,
 * Fourier.h:23-24 (destroy), CGSense.cpp:101-106 (threads).
 */
#ifndef CGS_FFTW_ADAPTOR_H
#define CGS_FFTW_ADAPTOR_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef struct fftwf_plan_s* fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftwf_complex* fftwf_alloc_complex(size_t n);
void fftwf_free(void* p);
fftwf_plan fftwf_plan_dft_3d(int n0, int n1, int n2, fftwf_complex* in, fftwf_complex* out,
                             int sign, unsigned flags);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
int fftwf_import_wisdom_from_filename(const char* filename);
int fftwf_export_wisdom_to_filename(const char* filename);
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
