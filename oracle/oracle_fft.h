/*
 * oracle_fft.h -- CPU mixed-radix FFT used by the test oracle only.
 *
 * TEST INFRASTRUCTURE.  Nothing in the product library links this file.  It is
 * included by
 *   - cgs_oracle.c        (the CPU restatement of the CG-SENSE path), and
 *   - fftw_adaptor.c      (an FFTW-API adaptor that lets the reference's own
 *                          Fourier.cpp / Reco.cpp compile without FFTW).
 *
 * Algorithm: iterative Stockham autosort FFT with mixed radices (4, 2, odd
 * primes; a plain O(p^2) DFT for each odd prime radix p).  Twiddles are
 * computed in double precision once per plan.  The arithmetic type is the
 * macro ORACLE_REAL (float or double), so the same code serves as an FP64
 * oracle and as an FP32 restatement of FFTW's single-precision transform
 * (Fourier.cpp:11-15, fftwf_plan_dft_3d + fftwf_execute_dft).
 *
 * Sign convention is FFTW's: sign = -1 forward, +1 backward, unnormalised:
 *   X[k] = sum_n x[n] exp(sign * 2*pi*i * n*k / N).
 */
#ifndef ORACLE_FFT_H
#define ORACLE_FFT_H

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif

typedef ORACLE_REAL ofr_t;
typedef struct { ofr_t re, im; } ofc_t;

#define OFFT_MAX_STAGES 40

typedef struct {
    int n;
    int nstages;
    int radix[OFFT_MAX_STAGES];
    int ns_before[OFFT_MAX_STAGES];   /* product of the radices before stage s */
    /* twiddles per stage: tw[s][ (j % Ns) * R + r ] = exp(sign*2*pi*i*r*(j%Ns)/(Ns*R)), stored for sign=-1 */
    double* tw_re[OFFT_MAX_STAGES];
    double* tw_im[OFFT_MAX_STAGES];
    /* roots of unity for the O(p^2) prime DFT, sign=-1: root[s][m] = exp(-2*pi*i*m/R) */
    double* rt_re[OFFT_MAX_STAGES];
    double* rt_im[OFFT_MAX_STAGES];
} offt_plan;

static const double OFFT_TWO_PI = 6.283185307179586476925286766559;

static int offt_factor(int n, int* radix)
{
    int ns = 0;
    while (n % 4 == 0) { radix[ns++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[ns++] = 2; n /= 2; }
    for (int p = 3; p * p <= n; p += 2)
        while (n % p == 0) { radix[ns++] = p; n /= p; }
    if (n > 1) radix[ns++] = n;
    return ns;
}

static offt_plan* offt_plan_create(int n)
{
    offt_plan* p = (offt_plan*)calloc(1, sizeof(offt_plan));
    p->n = n;
    p->nstages = (n > 1) ? offt_factor(n, p->radix) : 0;
    int Ns = 1;
    for (int s = 0; s < p->nstages; ++s) {
        int R = p->radix[s];
        p->ns_before[s] = Ns;
        p->tw_re[s] = (double*)malloc(sizeof(double) * (size_t)Ns * R);
        p->tw_im[s] = (double*)malloc(sizeof(double) * (size_t)Ns * R);
        for (int k = 0; k < Ns; ++k)
            for (int r = 0; r < R; ++r) {
                double a = -OFFT_TWO_PI * (double)r * (double)k / ((double)Ns * R);
                p->tw_re[s][k * R + r] = cos(a);
                p->tw_im[s][k * R + r] = sin(a);
            }
        p->rt_re[s] = (double*)malloc(sizeof(double) * R);
        p->rt_im[s] = (double*)malloc(sizeof(double) * R);
        for (int m = 0; m < R; ++m) {
            double a = -OFFT_TWO_PI * (double)m / (double)R;
            p->rt_re[s][m] = cos(a);
            p->rt_im[s][m] = sin(a);
        }
        Ns *= R;
    }
    return p;
}

static void offt_plan_destroy(offt_plan* p)
{
    if (!p) return;
    for (int s = 0; s < p->nstages; ++s) {
        free(p->tw_re[s]); free(p->tw_im[s]);
        free(p->rt_re[s]); free(p->rt_im[s]);
    }
    free(p);
}

/* In-place 1-D transform of x (length p->n); tmp must hold n elements. */
static void offt_exec(const offt_plan* p, ofc_t* x, ofc_t* tmp, int sign)
{
    const int n = p->n;
    ofc_t* src = x;
    ofc_t* dst = tmp;
    ofc_t v[64];
    ofc_t* vbig = NULL;
    for (int s = 0; s < p->nstages; ++s) {
        const int R = p->radix[s];
        const int Ns = p->ns_before[s];
        const int nR = n / R;
        ofc_t* vv = v;
        if (R > 32) {
            vbig = (ofc_t*)realloc(vbig, sizeof(ofc_t) * 2 * (size_t)R);
            vv = vbig;
        }
        ofc_t* out = vv + R;
        const double* twr = p->tw_re[s];
        const double* twi = p->tw_im[s];
        for (int j = 0; j < nR; ++j) {
            const int k = j % Ns;
            for (int r = 0; r < R; ++r) {
                ofc_t a = src[j + r * nR];
                double wr = twr[k * R + r];
                double wi = (sign < 0) ? twi[k * R + r] : -twi[k * R + r];
                vv[r].re = (ofr_t)((double)a.re * wr - (double)a.im * wi);
                vv[r].im = (ofr_t)((double)a.re * wi + (double)a.im * wr);
            }
            if (R == 2) {
                out[0].re = vv[0].re + vv[1].re; out[0].im = vv[0].im + vv[1].im;
                out[1].re = vv[0].re - vv[1].re; out[1].im = vv[0].im - vv[1].im;
            } else if (R == 4) {
                ofc_t a0 = vv[0], a1 = vv[1], a2 = vv[2], a3 = vv[3];
                ofc_t t0 = { a0.re + a2.re, a0.im + a2.im };
                ofc_t t1 = { a0.re - a2.re, a0.im - a2.im };
                ofc_t t2 = { a1.re + a3.re, a1.im + a3.im };
                ofc_t t3 = { a1.re - a3.re, a1.im - a3.im };
                /* multiply t3 by sign*i */
                ofc_t t3r = { -sign * t3.im, sign * t3.re };
                out[0].re = t0.re + t2.re;  out[0].im = t0.im + t2.im;
                out[2].re = t0.re - t2.re;  out[2].im = t0.im - t2.im;
                out[1].re = t1.re + t3r.re; out[1].im = t1.im + t3r.im;
                out[3].re = t1.re - t3r.re; out[3].im = t1.im - t3r.im;
            } else {
                const double* rr = p->rt_re[s];
                const double* ri = p->rt_im[s];
                for (int q = 0; q < R; ++q) {
                    double sr = 0.0, si = 0.0;
                    for (int r = 0; r < R; ++r) {
                        int m = (int)(((long long)r * q) % R);
                        double wr = rr[m], wi = (sign < 0) ? ri[m] : -ri[m];
                        sr += (double)vv[r].re * wr - (double)vv[r].im * wi;
                        si += (double)vv[r].re * wi + (double)vv[r].im * wr;
                    }
                    out[q].re = (ofr_t)sr;
                    out[q].im = (ofr_t)si;
                }
            }
            const int idxD = (j / Ns) * Ns * R + k;
            for (int r = 0; r < R; ++r) dst[idxD + r * Ns] = out[r];
        }
        ofc_t* t = src; src = dst; dst = t;
    }
    if (src != x) memcpy(x, src, sizeof(ofc_t) * (size_t)n);
    free(vbig);
}

/*
 * In-place 3-D transform of a row-major [n0][n1][n2] array (n2 fastest), the
 * layout of fftwf_plan_dft_3d(n0, n1, n2, ...).  Lines are copied to a
 * contiguous buffer, transformed, and copied back.
 */
static void offt_exec_3d(const offt_plan* p0, const offt_plan* p1, const offt_plan* p2,
                         ofc_t* a, int sign)
{
    const int n0 = p0->n, n1 = p1->n, n2 = p2->n;
    int nmax = n0 > n1 ? n0 : n1;
    if (n2 > nmax) nmax = n2;
    ofc_t* line = (ofc_t*)malloc(sizeof(ofc_t) * (size_t)nmax);
    ofc_t* tmp = (ofc_t*)malloc(sizeof(ofc_t) * (size_t)nmax);
    /* axis 2 (contiguous) */
    for (long long r = 0; r < (long long)n0 * n1; ++r)
        offt_exec(p2, a + r * n2, tmp, sign);
    /* axis 1 */
    for (int i = 0; i < n0; ++i)
        for (int k = 0; k < n2; ++k) {
            ofc_t* base = a + (size_t)i * n1 * n2 + k;
            for (int j = 0; j < n1; ++j) line[j] = base[(size_t)j * n2];
            offt_exec(p1, line, tmp, sign);
            for (int j = 0; j < n1; ++j) base[(size_t)j * n2] = line[j];
        }
    /* axis 0 */
    for (long long jk = 0; jk < (long long)n1 * n2; ++jk) {
        ofc_t* base = a + jk;
        for (int i = 0; i < n0; ++i) line[i] = base[(size_t)i * n1 * n2];
        offt_exec(p0, line, tmp, sign);
        for (int i = 0; i < n0; ++i) base[(size_t)i * n1 * n2] = line[i];
    }
    free(line);
    free(tmp);
}

#endif /* ORACLE_FFT_H */
