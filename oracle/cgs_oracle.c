/*
 * cgs_oracle.c -- CPU restatement of the expRad/4d_lung CG-SENSE hot path.
 *
 * TEST INFRASTRUCTURE (the oracle).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it, as the checker.  Every function cites
 * the reference file:line it restates.  Arithmetic keeps the reference's
 * float/double mix where the reference states it; the build flag ORACLE_REAL
 * selects float (a faithful FP32 port) or double (the FP64 oracle, where
 * every "float" of the reference becomes double except the stored tap
 * weights).
 *
 * Extension beyond the reference (documented in the header): the image may
 * be smaller than the grid.  The forward operator then zero-pads the image
 * into the centre of the grid and the adjoint crops it back; with
 * img == grid this is exactly the reference operator.
 */
#include "cgs_oracle.h"
#include "oracle_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef cgso_real R;

/* ---------------------------------------------------------------------- */
/* Kaiser-Bessel kernel                                                    */
/* ---------------------------------------------------------------------- */

double cgso_bessel_i0(double x)
{
    /* I0(x) = sum_k ((x/2)^(2k)) / (k!)^2, all terms positive. */
    const double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; ++k) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < sum * 1e-17) break;
    }
    return sum;
}

static inline float dk_of(int n) { return (float)(1.0 / (double)(float)(n - 1)); }

/* Reco.h:218-242.  dist is in k-space units (grid spacing dk = 1/(N-1)). */
float cgso_conv_function(const cgso_params* p, const double dist[3])
{
    const float w = p->kb_w;
    const float b = p->kb_b;
    const float wHalf = (float)(w / 2.0);
    double val = 1.0;
    for (int a = 0; a < 3; ++a) {
        const float dk = dk_of(p->grid[a]);
        const float d = (float)dist[a];
        if (d > wHalf * dk) return 0.0f;
    }
    for (int a = 0; a < 3; ++a) {
        const float dk = dk_of(p->grid[a]);
        const float d = (float)dist[a];
        const float qf = (float)(2 * d) / (float)(w * dk);
        const double q = (double)qf;
        const double arg = (double)b * sqrt(1.0 - q * q);
        val *= cgso_bessel_i0(arg) / (double)(float)(100.0f * w * dk);
    }
    return (float)val;
}

/* Reco.cpp:698-806: taps of one sample in the reference's scan order
 * (x offset outermost, z innermost), thresholded at kb_thresh * peak. */
static int sample_taps(const cgso_params* p, const double* kk, double thresh,
                       int32_t* idx_out, float* w_out)
{
    const int sx = p->grid[0], sy = p->grid[1], sz = p->grid[2];
    const float dkx = dk_of(sx), dky = dk_of(sy), dkz = dk_of(sz);
    const int order = p->kb_order;
    const int nearest[3] = {
        (int)((sx - 1) * kk[0] + 0.5),
        (int)((sy - 1) * kk[1] + 0.5),
        (int)((sz - 1) * kk[2] + 0.5),
    };
    int n = 0;
    for (int i1 = -order; i1 <= order; ++i1)
        for (int i2 = -order; i2 <= order; ++i2)
            for (int i3 = -order; i3 <= order; ++i3) {
                const int a = nearest[0] + i1, b = nearest[1] + i2, c = nearest[2] + i3;
                if (a < 0 || a > sx - 1 || b < 0 || b > sy - 1 || c < 0 || c > sz - 1) continue;
                /* distances: double k minus float (index * dk) (Reco.cpp:767-771) */
                const double dx = kk[0] - (double)((float)a * dkx);
                const double dy = kk[1] - (double)((float)b * dky);
                const double dz = kk[2] - (double)((float)c * dkz);
                const double dist[3] = { sqrt(dx * dx), sqrt(dy * dy), sqrt(dz * dz) };
                const double kv = (double)cgso_conv_function(p, dist);
                if (kv > thresh) {
                    if (idx_out) {
                        idx_out[n] = c + sz * b + sy * sz * a;
                        w_out[n] = (float)kv;
                    }
                    ++n;
                }
            }
    return n;
}

static double tap_threshold(const cgso_params* p)
{
    const double zero[3] = { 0.0, 0.0, 0.0 };
    return (double)cgso_conv_function(p, zero) * p->kb_thresh;   /* Reco.cpp:716-717 */
}

int64_t cgso_tap_counts(const cgso_params* p, const double* k, int64_t ns,
                        const uint8_t* mask, int32_t* counts)
{
    const double thresh = tap_threshold(p);
    int64_t total = 0;
#pragma omp parallel for schedule(static) reduction(+ : total)
    for (int64_t i = 0; i < ns; ++i) {
        int n = 0;
        if (!mask || mask[i]) n = sample_taps(p, k + 3 * i, thresh, NULL, NULL);
        counts[i] = n;
        total += n;
    }
    return total;
}

void cgso_taps_fill(const cgso_params* p, const double* k, int64_t ns, const uint8_t* mask,
                    const int64_t* ptr, int32_t* idx, float* w)
{
    const double thresh = tap_threshold(p);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < ns; ++i) {
        if (mask && !mask[i]) continue;
        sample_taps(p, k + 3 * i, thresh, idx + ptr[i], w + ptr[i]);
    }
}

/* ---------------------------------------------------------------------- */
/* Centred FFT (Fourier.cpp)                                               */
/* ---------------------------------------------------------------------- */

/* Fourier.cpp:45-72: negate every element whose i+j+k is even. */
static void sign_alternate_3d(const int* g, ofc_t* a)
{
    for (int i = 0; i < g[0]; ++i)
        for (int j = 0; j < g[1]; ++j)
            for (int k = 0; k < g[2]; ++k)
                if (((i + j + k) & 1) == 0) {
                    ofc_t* e = a + ((size_t)i * g[1] + j) * g[2] + k;
                    e->re = -e->re;
                    e->im = -e->im;
                }
}

static void centred_fft_plans(const int* g, ofc_t* a, int sign, int rescale,
                              offt_plan* p0, offt_plan* p1, offt_plan* p2)
{
    sign_alternate_3d(g, a);
    offt_exec_3d(p0, p1, p2, a, sign);
    sign_alternate_3d(g, a);
    if (rescale) {
        const size_t n = (size_t)g[0] * g[1] * g[2];
        const double s = 1.0 / sqrt((double)(g[0] * g[1] * g[2]));   /* Fourier.cpp:34 */
        for (size_t i = 0; i < n; ++i) {
            a[i].re = (R)((double)a[i].re * s);
            a[i].im = (R)((double)a[i].im * s);
        }
    }
}

void cgso_centred_fft(const cgso_params* p, R* a, int sign, int rescale)
{
    offt_plan* p0 = offt_plan_create(p->grid[0]);
    offt_plan* p1 = offt_plan_create(p->grid[1]);
    offt_plan* p2 = offt_plan_create(p->grid[2]);
    centred_fft_plans(p->grid, (ofc_t*)a, sign, rescale, p0, p1, p2);
    offt_plan_destroy(p0);
    offt_plan_destroy(p1);
    offt_plan_destroy(p2);
}

/* Reco.cpp:560-601: KB sampled at |i - N/2| * dk, centred backward FFT
 * without rescale, then 1/Re. */
void cgso_kernel_ft(const cgso_params* p, R* kft)
{
    const int sx = p->grid[0], sy = p->grid[1], sz = p->grid[2];
    const double dkx = 1.0 / (double)(sx - 1), dky = 1.0 / (double)(sy - 1), dkz = 1.0 / (double)(sz - 1);
    const int c[3] = { sx / 2, sy / 2, sz / 2 };
    ofc_t* a = (ofc_t*)kft;
    for (int i = 0; i < sx; ++i)
        for (int j = 0; j < sy; ++j)
            for (int k = 0; k < sz; ++k) {
                const double dist[3] = {
                    sqrt(dkx * dkx * (i - c[0]) * (i - c[0])),
                    sqrt(dky * dky * (j - c[1]) * (j - c[1])),
                    sqrt(dkz * dkz * (k - c[2]) * (k - c[2])),
                };
                ofc_t* e = a + ((size_t)i * sy + j) * sz + k;
                e->re = (R)cgso_conv_function(p, dist);
                e->im = 0;
            }
    cgso_centred_fft(p, kft, +1, 0);
    const size_t n = (size_t)sx * sy * sz;
    for (size_t i = 0; i < n; ++i) {
        const double re = (double)a[i].re;
        a[i].re = (R)(re / (re * re));
        a[i].im = 0;
    }
}

/* ---------------------------------------------------------------------- */
/* NUFFT forward / adjoint (Reco.cpp:468-553)                              */
/* ---------------------------------------------------------------------- */

static void image_box(const cgso_params* p, int* lo)
{
    for (int a = 0; a < 3; ++a) lo[a] = (p->grid[a] - p->img[a]) / 2 + p->offcenter[a];
}

static size_t n_img(const cgso_params* p) { return (size_t)p->img[0] * p->img[1] * p->img[2]; }
static size_t n_grid(const cgso_params* p) { return (size_t)p->grid[0] * p->grid[1] * p->grid[2]; }

/* zero-pad one coil image into the grid and multiply by kernelFT (Reco.cpp:529-535) */
static void pad_apod(const cgso_params* p, const ofc_t* kft, const ofc_t* img, ofc_t* grid)
{
    int lo[3];
    image_box(p, lo);
    memset(grid, 0, sizeof(ofc_t) * n_grid(p));
    for (int i = 0; i < p->img[0]; ++i)
        for (int j = 0; j < p->img[1]; ++j)
            for (int k = 0; k < p->img[2]; ++k) {
                const size_t gi = ((size_t)(i + lo[0]) * p->grid[1] + (j + lo[1])) * p->grid[2] + (k + lo[2]);
                const ofc_t v = img[((size_t)i * p->img[1] + j) * p->img[2] + k];
                const double gr = (double)v.re, gim = (double)v.im;
                grid[gi].re = (R)(gr * (double)kft[gi].re - gim * (double)kft[gi].im);
                grid[gi].im = (R)(gim * (double)kft[gi].re + gr * (double)kft[gi].im);
            }
}

/* multiply by kernelFT * rescale and crop to the image box (Reco.cpp:509-517) */
static void crop_apod(const cgso_params* p, const ofc_t* kft, const ofc_t* grid, ofc_t* img)
{
    int lo[3];
    image_box(p, lo);
    const double rescale = p->adj_scale;
    for (int i = 0; i < p->img[0]; ++i)
        for (int j = 0; j < p->img[1]; ++j)
            for (int k = 0; k < p->img[2]; ++k) {
                const size_t gi = ((size_t)(i + lo[0]) * p->grid[1] + (j + lo[1])) * p->grid[2] + (k + lo[2]);
                const double gr = (double)grid[gi].re, gim = (double)grid[gi].im;
                ofc_t* o = img + ((size_t)i * p->img[1] + j) * p->img[2] + k;
                o->re = (R)((gr * (double)kft[gi].re - gim * (double)kft[gi].im) * rescale);
                o->im = (R)((gim * (double)kft[gi].re + gr * (double)kft[gi].im) * rescale);
            }
}

typedef struct {
    offt_plan* p[3];
} plans3;

static plans3 make_plans(const cgso_params* p)
{
    plans3 pl;
    for (int a = 0; a < 3; ++a) pl.p[a] = offt_plan_create(p->grid[a]);
    return pl;
}
static void free_plans(plans3* pl)
{
    for (int a = 0; a < 3; ++a) offt_plan_destroy(pl->p[a]);
}

static void fwd_one(const cgso_params* p, const plans3* pl, const int64_t* ptr, const int32_t* idx,
                    const float* w, int64_t ns, const ofc_t* kft, const ofc_t* img, ofc_t* grid,
                    ofc_t* data)
{
    pad_apod(p, kft, img, grid);
    centred_fft_plans(p->grid, grid, -1, 0, pl->p[0], pl->p[1], pl->p[2]);
    for (int64_t i = 0; i < ns; ++i) {
        R re = 0, im = 0;
        for (int64_t t = ptr[i]; t < ptr[i + 1]; ++t) {
            const double kv = (double)w[t];   /* Reco.cpp:546: double kernelVal */
            re = (R)((double)re + (double)grid[idx[t]].re * kv);
            im = (R)((double)im + (double)grid[idx[t]].im * kv);
        }
        data[i].re = re;
        data[i].im = im;
    }
}

static void adj_one(const cgso_params* p, const plans3* pl, const int64_t* ptr, const int32_t* idx,
                    const float* w, int64_t ns, const ofc_t* kft, const ofc_t* data, ofc_t* grid,
                    ofc_t* img)
{
    memset(grid, 0, sizeof(ofc_t) * n_grid(p));
    for (int64_t i = 0; i < ns; ++i) {
        const ofc_t d = data[i];
        for (int64_t t = ptr[i]; t < ptr[i + 1]; ++t) {
            const R kv = (R)w[t];             /* Reco.cpp:491: float kernelVal */
            grid[idx[t]].re += d.re * kv;
            grid[idx[t]].im += d.im * kv;
        }
    }
    centred_fft_plans(p->grid, grid, +1, 1, pl->p[0], pl->p[1], pl->p[2]);
    crop_apod(p, kft, grid, img);
}

void cgso_nufft_fwd(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                    int64_t ns, const R* kft, const R* img, R* data)
{
    plans3 pl = make_plans(p);
#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < p->n_ch; ++c) {
        ofc_t* grid = (ofc_t*)malloc(sizeof(ofc_t) * n_grid(p));
        fwd_one(p, &pl, ptr, idx, w, ns, (const ofc_t*)kft, (const ofc_t*)img + (size_t)c * n_img(p),
                grid, (ofc_t*)data + (size_t)c * ns);
        free(grid);
    }
    free_plans(&pl);
}

void cgso_nufft_adj(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                    int64_t ns, const R* kft, const R* data, R* img)
{
    plans3 pl = make_plans(p);
#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < p->n_ch; ++c) {
        ofc_t* grid = (ofc_t*)malloc(sizeof(ofc_t) * n_grid(p));
        adj_one(p, &pl, ptr, idx, w, ns, (const ofc_t*)kft, (const ofc_t*)data + (size_t)c * ns,
                grid, (ofc_t*)img + (size_t)c * n_img(p));
        free(grid);
    }
    free_plans(&pl);
}

/* ---------------------------------------------------------------------- */
/* E^H D E and CG-SENSE (Reco.cpp:74-321)                                  */
/* ---------------------------------------------------------------------- */

/* q = sum_c conj(S_c) E_c^H D E_c (S_c x), Reco.cpp:232-262.  Coils are summed
 * in order 0..n_ch-1 (the reference sums them with omp atomics). */
static void apply_ehde_plans(const cgso_params* p, const plans3* pl, const int64_t* ptr,
                             const int32_t* idx, const float* w, int64_t ns, const ofc_t* kft,
                             const ofc_t* smaps, const float* dcf, const ofc_t* x, ofc_t* q)
{
    const size_t ni = n_img(p);
    const int nch = p->n_ch;
    ofc_t* imgs = (ofc_t*)malloc(sizeof(ofc_t) * ni * nch);
#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < nch; ++c) {
        const ofc_t* S = smaps + (size_t)c * ni;
        ofc_t* ic = imgs + (size_t)c * ni;
        ofc_t* grid = (ofc_t*)malloc(sizeof(ofc_t) * n_grid(p));
        ofc_t* data = (ofc_t*)malloc(sizeof(ofc_t) * (size_t)ns);
        /* elementProduct (Reco.cpp:85-93) */
        for (size_t i = 0; i < ni; ++i) {
            ic[i].re = x[i].re * S[i].re - x[i].im * S[i].im;
            ic[i].im = x[i].re * S[i].im + x[i].im * S[i].re;
        }
        fwd_one(p, pl, ptr, idx, w, ns, kft, ic, grid, data);
        if (dcf) /* Reco.cpp:243-254 */
            for (int64_t i = 0; i < ns; ++i) {
                data[i].re *= (R)dcf[i];
                data[i].im *= (R)dcf[i];
            }
        adj_one(p, pl, ptr, idx, w, ns, kft, data, grid, ic);
        /* mutliplyByConjSenseMap (Reco.cpp:107-117) */
        for (size_t i = 0; i < ni; ++i) {
            const double re = (double)ic[i].re, im = (double)ic[i].im;
            ic[i].re = (R)(re * (double)S[i].re + im * (double)S[i].im);
            ic[i].im = (R)(-re * (double)S[i].im + im * (double)S[i].re);
        }
        free(grid);
        free(data);
    }
    /* clearFFTWComplex + addToSumOfImages (Reco.cpp:74-82,120-129) */
    memset(q, 0, sizeof(ofc_t) * ni);
    for (int c = 0; c < nch; ++c)
        for (size_t i = 0; i < ni; ++i) {
            q[i].re += imgs[(size_t)c * ni + i].re;
            q[i].im += imgs[(size_t)c * ni + i].im;
        }
    free(imgs);
}

void cgso_apply_ehde(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                     int64_t ns, const R* kft, const R* smaps, const float* dcf, const R* x, R* q)
{
    plans3 pl = make_plans(p);
    apply_ehde_plans(p, &pl, ptr, idx, w, ns, (const ofc_t*)kft, (const ofc_t*)smaps, dcf,
                     (const ofc_t*)x, (ofc_t*)q);
    free_plans(&pl);
}

/* conjScalarProduct (Reco.cpp:131-143): sum conj(x) y with double accumulators */
static void conj_dot(const ofc_t* x, const ofc_t* y, size_t n, double* out)
{
    double r0 = 0.0, r1 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        r0 += (double)(x[i].re * y[i].re + x[i].im * y[i].im);
        r1 += (double)(x[i].re * y[i].im - x[i].im * y[i].re);
    }
    out[0] = r0;
    out[1] = r1;
}

/* complexDivision (Reco.cpp:145-151) */
static void cdiv(const double* x, const double* y, double* out)
{
    const double d = y[0] * y[0] + y[1] * y[1];
    const double a = (x[0] * y[0] + x[1] * y[1]) / d;
    const double b = (x[1] * y[0] - x[0] * y[1]) / d;
    out[0] = a;
    out[1] = b;
}

int cgso_cg_sense(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                  int64_t ns, const R* kft_, const R* smaps_, const float* dcf, const R* data_,
                  double threshold, int max_iter, R* x_out, double* residuals, int32_t* iters_out)
{
    const size_t ni = n_img(p);
    const int nch = p->n_ch;
    const ofc_t* kft = (const ofc_t*)kft_;
    const ofc_t* smaps = (const ofc_t*)smaps_;
    plans3 pl = make_plans(p);
    int status = 0;

    /* performDensityCorrection (functions.h:319-335) then nufftBWD (CGSense.cpp:226,235) */
    ofc_t* dat = (ofc_t*)malloc(sizeof(ofc_t) * (size_t)ns * nch);
    memcpy(dat, data_, sizeof(ofc_t) * (size_t)ns * nch);
    if (dcf)
        for (int c = 0; c < nch; ++c)
            for (int64_t i = 0; i < ns; ++i) {
                dat[(size_t)c * ns + i].re *= (R)dcf[i];
                dat[(size_t)c * ns + i].im *= (R)dcf[i];
            }
    ofc_t* imgs = (ofc_t*)malloc(sizeof(ofc_t) * ni * nch);
    cgso_nufft_adj(p, ptr, idx, w, ns, kft_, (const R*)dat, (R*)imgs);

    /* a = sum_c conj(S_c) img_c (Reco.cpp:182-190) */
    ofc_t* r = (ofc_t*)calloc(ni, sizeof(ofc_t));
    for (size_t i = 0; i < ni; ++i)
        for (int c = 0; c < nch; ++c) {
            const ofc_t S = smaps[(size_t)c * ni + i];
            const ofc_t g = imgs[(size_t)c * ni + i];
            r[i].re += S.re * g.re + S.im * g.im;
            r[i].im += S.re * g.im - S.im * g.re;
        }
    free(imgs);
    free(dat);

    ofc_t* x = (ofc_t*)x_out;
    ofc_t* pp = (ofc_t*)malloc(sizeof(ofc_t) * ni);
    ofc_t* q = (ofc_t*)malloc(sizeof(ofc_t) * ni);
    memcpy(pp, r, sizeof(ofc_t) * ni);
    memset(x, 0, sizeof(ofc_t) * ni);

    int iteration = 0;
    double current = 1000.0;                       /* Reco.cpp:229 */
    while (current > threshold) {
        apply_ehde_plans(p, &pl, ptr, idx, w, ns, kft, smaps, dcf, pp, q);
        if (!isfinite((double)q[0].re) || !isfinite((double)q[0].im)) {   /* Reco.cpp:264-268 */
            status = -1;
            break;
        }
        double rr[2], pq[2], alpha[2];
        conj_dot(r, r, ni, rr);
        conj_dot(pp, q, ni, pq);
        cdiv(rr, pq, alpha);
        /* x += alpha p ; r -= alpha q  (addToArrayScaled, Reco.cpp:153-161,285-290) */
        for (size_t i = 0; i < ni; ++i) {
            x[i].re = (R)((double)x[i].re + (alpha[0] * (double)pp[i].re - alpha[1] * (double)pp[i].im));
            x[i].im = (R)((double)x[i].im + (alpha[0] * (double)pp[i].im + alpha[1] * (double)pp[i].re));
        }
        const double na[2] = { -alpha[0], -alpha[1] };
        for (size_t i = 0; i < ni; ++i) {
            r[i].re = (R)((double)r[i].re + (na[0] * (double)q[i].re - na[1] * (double)q[i].im));
            r[i].im = (R)((double)r[i].im + (na[0] * (double)q[i].im + na[1] * (double)q[i].re));
        }
        /* residual norm (Reco.cpp:292-299) */
        current = 0.0;
        for (size_t i = 0; i < ni; ++i) current += (double)(r[i].re * r[i].re + r[i].im * r[i].im);
        current = sqrt(current);
        if (residuals) residuals[iteration] = current;
        /* beta = <r,r>_new / <r,r>_old ; p = r + beta p (Reco.cpp:303-306,163-173) */
        double rrn[2], beta[2];
        conj_dot(r, r, ni, rrn);
        cdiv(rrn, rr, beta);
        for (size_t i = 0; i < ni; ++i) {
            const double pr = (double)pp[i].re, pim = (double)pp[i].im;
            pp[i].re = (R)((double)r[i].re + beta[0] * pr - beta[1] * pim);
            pp[i].im = (R)((double)r[i].im + beta[0] * pim + beta[1] * pr);
        }
        ++iteration;
        if (iteration >= max_iter) break;           /* Reco.cpp:308-309 with nMaxIter = max_iter - 1 */
    }
    if (iters_out) *iters_out = iteration;
    free(pp);
    free(q);
    free(r);
    free_plans(&pl);
    return status;
}

/* ---------------------------------------------------------------------- */
/* Wave-CAIPI trajectory (Trajectory.cpp:9-184, globalVars.h:3-4)          */
/* ---------------------------------------------------------------------- */

void cgso_wave_caipi(const cgso_wave* wv, double* k_out)
{
    const double PI_REF = 3.14159265359;                       /* globalVars.h:3 */
    const double gammaBar = 4.257748059639612 * pow(10, 7);     /* globalVars.h:4 */
    const int sX = wv->sx, sY = wv->sy, sZ = wv->sz, nOsc = wv->n_osc;
    /* calculateKMax (Trajectory.cpp:9-16) */
    const double kmax[3][2] = {
        { 0.0, 1.0 },
        { sY / (double)(wv->fov_y * 2.0 * gammaBar), -sY / (double)(wv->fov_y * 2.0 * gammaBar) },
        { sZ / (double)(wv->fov_z * 2.0 * gammaBar), -sZ / (double)(wv->fov_z * 2.0 * gammaBar) },
    };
    const double tADC = wv->dwell * sX;
    const double gradRasterTime = 10 * pow(10, -6);
    const int os = 10000;
    const double gradRasterTimeOs = gradRasterTime / (double)os;
    const int gradSamples = (int)(tADC / gradRasterTime);
    const int gradSamplesZ = (int)((tADC + 0.5 * tADC / (double)nOsc) / gradRasterTime);
    const long nSamples = (long)sX * sY * sZ;
    const double sinTerm = pow(sin(nOsc * PI_REF / (double)(2 * nOsc)), 2);
    const double kSpaceOscAmpY = wv->grad_amp * wv->amp_corr_y * tADC * sinTerm / (double)(nOsc * PI_REF);
    const double kSpaceOscAmpZ = wv->grad_amp * wv->amp_corr_z * tADC * sinTerm / (double)(nOsc * PI_REF);

    /* trapezoid integration of the oversampled gradients (Trajectory.cpp:55-86) */
    const size_t nY = (size_t)gradSamples * os, nZ = (size_t)gradSamplesZ * os;
    double* kWaveY = (double*)malloc(sizeof(double) * (nY ? nY : 1));
    double* kWaveZ = (double*)malloc(sizeof(double) * (nZ ? nZ : 1));
    if (nY) kWaveY[0] = 0;
    if (nZ) kWaveZ[0] = 0;
    double* gY = (double*)malloc(sizeof(double) * (gradSamples > 0 ? gradSamples : 1));
    double* gZ = (double*)malloc(sizeof(double) * (gradSamplesZ > 0 ? gradSamplesZ : 1));
    for (int i = 0; i < gradSamples; ++i)
        gY[i] = -wv->grad_amp * wv->amp_corr_y * sin(2.0 * PI_REF * nOsc * (double)i / (double)gradSamples);
    for (int i = 0; i < gradSamplesZ; ++i)
        gZ[i] = wv->grad_amp * wv->amp_corr_z * sin(2.0 * PI_REF * (nOsc + 0.5) * (double)i / (double)gradSamplesZ);
    for (size_t i = 1; i < nY; ++i)
        kWaveY[i] = kWaveY[i - 1] + gradRasterTimeOs * 0.5 * (gY[(i - 1) / os] + gY[i / os]);
    for (size_t i = 1; i < nZ; ++i)
        kWaveZ[i] = kWaveZ[i - 1] + gradRasterTimeOs * 0.5 * (gZ[(i - 1) / os] + gZ[i / os]);
    free(gY);
    free(gZ);

    /* helix sampled at the ADC times with the delays (Trajectory.cpp:88-105) */
    double* helix = (double*)malloc(sizeof(double) * 3 * (size_t)sX);
    for (int i = 0; i < sX; ++i) {
        const double tY = (i + 1) * wv->dwell - wv->shift_y;
        const double tZ = tADC / (4.0 * nOsc) + (i + 1) * wv->dwell - wv->shift_z;
        long elY = lround(tY / tADC * (double)nY);
        long elZ = lround(tZ / (tADC + 0.5 * tADC / (double)nOsc) * (double)nZ);
        /* int vs size_t comparison: negative indices wrap to huge and clamp (Trajectory.cpp:96-97) */
        if (elY < 0 || (size_t)elY > nY - 1) elY = (long)nY - 1;
        if (elZ < 0 || (size_t)elZ > nZ - 1) elZ = (long)nZ - 1;
        helix[3 * i + 0] = i / (double)(sX - 1.0);
        helix[3 * i + 1] = (tY < 0) ? 0.0 : kWaveY[elY];
        helix[3 * i + 2] = kWaveZ[elZ];
    }
    free(kWaveY);
    free(kWaveZ);

    /* base lines and helix placement (Trajectory.cpp:113-127) */
    double* traj = (double*)malloc(sizeof(double) * 3 * (size_t)nSamples);
    for (long i = 0; i < nSamples; ++i) {
        const int ix = (int)(i % sX);
        const int iy = (int)((i / sX) % sY);
        const int iz = (int)(i / ((long)sX * sY));
        const double by = kmax[1][0] - iy / (double)(sY - 1.0) * (kmax[1][0] - kmax[1][1]);
        const double bz = kmax[2][1] - iz / (double)(sZ - 1.0) * (kmax[2][1] - kmax[2][0]);
        traj[3 * i + 0] = helix[3 * ix + 0];
        traj[3 * i + 1] = by + helix[3 * ix + 1];
        traj[3 * i + 2] = bz + helix[3 * ix + 2];
    }
    free(helix);

    /* normalisation to [0,1] with a 42-cell border (Trajectory.cpp:129-164) */
    double maxY = 0, minY = 0, maxZ = 0, minZ = 0;
    for (long i = 0; i < nSamples; ++i) {
        if (traj[3 * i + 1] > maxY) maxY = traj[3 * i + 1];
        if (traj[3 * i + 1] < minY) minY = traj[3 * i + 1];
        if (traj[3 * i + 2] > maxZ) maxZ = traj[3 * i + 2];
        if (traj[3 * i + 2] < minZ) minZ = traj[3 * i + 2];
    }
    const double nBorderPts = 42.0;
    const double fX = (1.0 * nBorderPts) / (double)wv->gx;
    const double fY = (1.0 * nBorderPts - 0.405 * kSpaceOscAmpY / (double)(fabs(kmax[1][0]) + fabs(kmax[1][1])) * wv->gy) / (double)wv->gy;
    const double fZ = (1.0 * nBorderPts - 0.405 * kSpaceOscAmpZ / (double)(fabs(kmax[2][0]) + fabs(kmax[2][1])) * wv->gz) / (double)wv->gz;
    for (long i = 0; i < nSamples; ++i) {
        double* t = traj + 3 * i;
        t[1] -= minY;
        t[2] -= minZ;
        t[1] = t[1] / (double)(maxY - minY);
        t[2] = t[2] / (double)(maxZ - minZ);
        t[0] *= (1.0 - 2 * fX);
        t[1] *= (1.0 - 2 * fY);
        t[2] *= (1.0 - 2 * fZ);
        t[0] += fX;
        t[1] += fY;
        t[2] += fZ;
    }

    /* z-fastest permutation (Trajectory.cpp:167-175) */
    for (long k = 0; k < nSamples; ++k) {
        const long i3 = k / ((long)sX * sY);
        const long i2 = (k - (long)sX * sY * i3) / sX;
        const long i1 = k - (long)sX * i2 - (long)sX * sY * i3;
        const long dst = i3 + (long)sZ * i2 + (long)sY * sZ * i1;
        for (int a = 0; a < 3; ++a) k_out[3 * dst + a] = traj[3 * k + a];
    }
    free(traj);
}

/* ---------------------------------------------------------------------- */
/* Data-consistency loss and gradients (extension; no reference code)      */
/* ---------------------------------------------------------------------- */

double cgso_bessel_i1(double x)
{
    /* I1(x) = sum_m (x/2)^(2m+1) / (m! (m+1)!) */
    const double h = 0.5 * x, q = h * h;
    double term = h, sum = h;
    for (int m = 1; m < 500; ++m) {
        term *= q / ((double)m * (double)(m + 1));
        sum += term;
        if (fabs(term) < fabs(sum) * 1e-17) break;
    }
    return sum;
}

/* KB factor of one axis and its derivative with respect to the sample
 * coordinate ka, for grid index g: f = I0(b s) / (100 w dk), s = sqrt(1 - t^2),
 * t = 2 (ka - g dk) / (w dk) (Reco.h:218-242 in double).
 * df/dka = -(I1(b s) / s) b t (2 / (w dk)) / (100 w dk); I1(b s)/s -> b/2 at s = 0. */
static void kb_axis(double ka, int g, double dk, double w, double b, double* f, double* df)
{
    const double d = ka - (double)g * dk;
    if (fabs(d) > 0.5 * w * dk) {
        *f = 0.0;
        *df = 0.0;
        return;
    }
    const double t = 2.0 * d / (w * dk);
    const double s2 = 1.0 - t * t;
    const double s = s2 > 0.0 ? sqrt(s2) : 0.0;
    const double C = 100.0 * w * dk;
    *f = cgso_bessel_i0(b * s) / C;
    const double i1s = s > 1e-12 ? cgso_bessel_i1(b * s) / s : 0.5 * b;
    *df = -i1s * b * t * (2.0 / (w * dk)) / C;
}

double cgso_loss_grad(const cgso_params* p, const double* k, int64_t ns, const R* kft, const R* smaps,
                      const float* dcf, const R* x, const R* y, R* grad_x, double* grad_k)
{
    const int nch = p->n_ch;
    const int* G = p->grid;
    const size_t ni = n_img(p), ng = n_grid(p);
    const int order = p->kb_order;
    const double w = p->kb_w, b = p->kb_b;
    double dk[3], peak = 1.0;
    for (int a = 0; a < 3; ++a) {
        dk[a] = 1.0 / (double)(G[a] - 1);
        peak *= cgso_bessel_i0(b) / (100.0 * w * dk[a]);
    }
    const double thresh = peak * p->kb_thresh;
    plans3 pl = make_plans(p);
    double* lossc = (double*)calloc((size_t)nch, sizeof(double));
    double* gk = grad_k ? (double*)calloc((size_t)nch * ns * 3, sizeof(double)) : NULL;
    ofc_t* gx = grad_x ? (ofc_t*)calloc((size_t)nch * ni, sizeof(ofc_t)) : NULL;
#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < nch; ++c) {
        const ofc_t* S = (const ofc_t*)smaps + (size_t)c * ni;
        const ofc_t* xx = (const ofc_t*)x;
        const ofc_t* yc = (const ofc_t*)y + (size_t)c * ns;
        ofc_t* img = (ofc_t*)malloc(sizeof(ofc_t) * ni);
        ofc_t* grid = (ofc_t*)malloc(sizeof(ofc_t) * ng);
        for (size_t i = 0; i < ni; ++i) {
            img[i].re = xx[i].re * S[i].re - xx[i].im * S[i].im;
            img[i].im = xx[i].re * S[i].im + xx[i].im * S[i].re;
        }
        pad_apod(p, (const ofc_t*)kft, img, grid);
        centred_fft_plans(G, grid, -1, 0, pl.p[0], pl.p[1], pl.p[2]);
        ofc_t* acc = gx ? (ofc_t*)calloc(ng, sizeof(ofc_t)) : NULL;
        double lc = 0.0;
        for (int64_t i = 0; i < ns; ++i) {
            const double* kk = k + 3 * i;
            int nr[3];
            double f[3][16], df[3][16];
            for (int a = 0; a < 3; ++a) {
                nr[a] = (int)((G[a] - 1) * kk[a] + 0.5);
                for (int j = -order; j <= order; ++j) {
                    const int g = nr[a] + j;
                    if (g < 0 || g > G[a] - 1) {
                        f[a][j + order] = df[a][j + order] = 0.0;
                        continue;
                    }
                    kb_axis(kk[a], g, dk[a], w, b, &f[a][j + order], &df[a][j + order]);
                }
            }
            double yr = 0, yi = 0, dr[3] = {0, 0, 0}, di[3] = {0, 0, 0};
            for (int i1 = 0; i1 <= 2 * order; ++i1)
                for (int i2 = 0; i2 <= 2 * order; ++i2)
                    for (int i3 = 0; i3 <= 2 * order; ++i3) {
                        const double wt = f[0][i1] * f[1][i2] * f[2][i3];
                        if (!(wt > thresh)) continue;
                        const size_t gi = ((size_t)(nr[0] - order + i1) * G[1] + (nr[1] - order + i2)) * G[2] +
                                          (nr[2] - order + i3);
                        const double gr = grid[gi].re, gim = grid[gi].im;
                        yr += wt * gr;
                        yi += wt * gim;
                        const double dw[3] = {df[0][i1] * f[1][i2] * f[2][i3], f[0][i1] * df[1][i2] * f[2][i3],
                                              f[0][i1] * f[1][i2] * df[2][i3]};
                        for (int a = 0; a < 3; ++a) {
                            dr[a] += dw[a] * gr;
                            di[a] += dw[a] * gim;
                        }
                    }
            const double D = dcf ? (double)dcf[i] : 1.0;
            const double rr = yr - (double)yc[i].re, ri = yi - (double)yc[i].im;
            lc += 0.5 * D * (rr * rr + ri * ri);
            if (gk)
                for (int a = 0; a < 3; ++a) gk[((size_t)c * ns + i) * 3 + a] = D * (rr * dr[a] + ri * di[a]);
            if (acc) {
                /* spread D r with the same taps (the transpose of the interpolation) */
                for (int i1 = 0; i1 <= 2 * order; ++i1)
                    for (int i2 = 0; i2 <= 2 * order; ++i2)
                        for (int i3 = 0; i3 <= 2 * order; ++i3) {
                            const double wt = f[0][i1] * f[1][i2] * f[2][i3];
                            if (!(wt > thresh)) continue;
                            const size_t gi = ((size_t)(nr[0] - order + i1) * G[1] + (nr[1] - order + i2)) * G[2] +
                                              (nr[2] - order + i3);
                            acc[gi].re += (R)(wt * D * rr);
                            acc[gi].im += (R)(wt * D * ri);
                        }
            }
        }
        lossc[c] = lc;
        if (acc) {
            /* exact adjoint of the unscaled centred forward FFT, then of pad_apod */
            centred_fft_plans(G, acc, +1, 0, pl.p[0], pl.p[1], pl.p[2]);
            int lo[3];
            image_box(p, lo);
            ofc_t* gc = gx + (size_t)c * ni;
            const ofc_t* K = (const ofc_t*)kft;
            for (int i = 0; i < p->img[0]; ++i)
                for (int j = 0; j < p->img[1]; ++j)
                    for (int kz = 0; kz < p->img[2]; ++kz) {
                        const size_t gi = ((size_t)(i + lo[0]) * G[1] + (j + lo[1])) * G[2] + (kz + lo[2]);
                        const size_t ii = ((size_t)i * p->img[1] + j) * p->img[2] + kz;
                        /* conj(kft) * acc, then conj(S_c) * (...) */
                        const double ar = acc[gi].re * K[gi].re + acc[gi].im * K[gi].im;
                        const double ai = acc[gi].im * K[gi].re - acc[gi].re * K[gi].im;
                        gc[ii].re = (R)(ar * S[ii].re + ai * S[ii].im);
                        gc[ii].im = (R)(ai * S[ii].re - ar * S[ii].im);
                    }
            free(acc);
        }
        free(img);
        free(grid);
    }
    double L = 0.0;
    for (int c = 0; c < nch; ++c) L += lossc[c];
    if (gk) {
        for (int64_t i = 0; i < 3 * ns; ++i) {
            double s = 0.0;
            for (int c = 0; c < nch; ++c) s += gk[(size_t)c * ns * 3 + i];
            grad_k[i] = s;
        }
        free(gk);
    }
    if (gx) {
        ofc_t* o = (ofc_t*)grad_x;
        for (size_t i = 0; i < ni; ++i) {
            double sr = 0, si = 0;
            for (int c = 0; c < nch; ++c) {
                sr += gx[(size_t)c * ni + i].re;
                si += gx[(size_t)c * ni + i].im;
            }
            o[i].re = (R)sr;
            o[i].im = (R)si;
        }
        free(gx);
    }
    free(lossc);
    free_plans(&pl);
    return L;
}
