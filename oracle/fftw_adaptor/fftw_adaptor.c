/*
 * fftw_adaptor.c -- implementation of the FFTW-API adaptor (fftw3.h).
 *
 * TEST INFRASTRUCTURE (oracle only): lets the reference's own FFT wrapper
 * (Fourier.cpp:4-72) run unmodified.  Transforms are computed in double
 * precision by oracle_fft.h and stored back as float.  Plans are thread-safe
 * to execute concurrently (each call allocates its own scratch), which the
 * reference relies on when nufftFWD/nufftBWD run one coil per OpenMP thread
 * (Reco.cpp:470,523).
 */
#define ORACLE_REAL double
#include "../oracle_fft.h"
#include "fftw3.h"

struct fftwf_plan_s {
    int n0, n1, n2, sign;
    offt_plan* p0;
    offt_plan* p1;
    offt_plan* p2;
};

fftwf_complex* fftwf_alloc_complex(size_t n)
{
    void* p = NULL;
    if (posix_memalign(&p, 64, n * sizeof(fftwf_complex) + 64) != 0) return NULL;
    return (fftwf_complex*)p;
}

void fftwf_free(void* p) { free(p); }

fftwf_plan fftwf_plan_dft_3d(int n0, int n1, int n2, fftwf_complex* in, fftwf_complex* out,
                             int sign, unsigned flags)
{
    (void)in; (void)out; (void)flags;
    struct fftwf_plan_s* p = (struct fftwf_plan_s*)calloc(1, sizeof(*p));
    p->n0 = n0; p->n1 = n1; p->n2 = n2; p->sign = sign;
    p->p0 = offt_plan_create(n0);
    p->p1 = offt_plan_create(n1);
    p->p2 = offt_plan_create(n2);
    return p;
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out)
{
    const size_t n = (size_t)p->n0 * p->n1 * p->n2;
    ofc_t* a = (ofc_t*)malloc(sizeof(ofc_t) * n);
    for (size_t i = 0; i < n; ++i) { a[i].re = in[i][0]; a[i].im = in[i][1]; }
    offt_exec_3d(p->p0, p->p1, p->p2, a, p->sign);
    for (size_t i = 0; i < n; ++i) { out[i][0] = (float)a[i].re; out[i][1] = (float)a[i].im; }
    free(a);
}

void fftwf_destroy_plan(fftwf_plan p)
{
    if (!p) return;
    offt_plan_destroy(p->p0);
    offt_plan_destroy(p->p1);
    offt_plan_destroy(p->p2);
    free(p);
}

int fftwf_import_wisdom_from_filename(const char* f) { (void)f; return 0; }
int fftwf_export_wisdom_to_filename(const char* f) { (void)f; return 1; }
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int n) { (void)n; }
