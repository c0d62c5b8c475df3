/*
 * cgs_oracle.h -- CPU restatement of the expRad/4d_lung CG-SENSE hot path.
 *
 * TEST INFRASTRUCTURE.  This is the oracle: tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg are the only callers.  The product library
 * (4d_lung_gb300/csrc) never links or calls it.
 *
 * Built twice from one source (see Makefile):
 *   liboracle64.so  ORACLE_REAL=double   -- the FP64 oracle
 *   liboracle32.so  ORACLE_REAL=float    -- an FP32 restatement that keeps the
 *                                           reference's float/double mix, used
 *                                           as the timed CPU port
 * "real" arrays below are double in the first and float in the second;
 * complex arrays are interleaved (re, im) pairs of that type.
 *
 * Pinned against the reference itself: oracle/ref_driver.cpp compiles the
 * reference's unmodified Reco.cpp / Fourier.cpp / Trajectory.cpp / IO.cpp
 * and tests/golden/ holds fixtures generated from it.
 */
#ifndef CGS_ORACLE_H
#define CGS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL cgso_real;

typedef struct {
    int32_t img[3];     /* image size; the reference reconstructs on the grid itself (img == grid) */
    int32_t grid[3];    /* Cartesian grid size, row-major x,y,z with z fastest (Reco.cpp:603-606) */
    int32_t n_ch;       /* coils (Reco.h:165 nCh) */
    int32_t kb_order;   /* half-width of the neighbour scan, 5 (Reco.cpp:380) */
    float kb_w;         /* KB width in cells, 4.25 (Reco.cpp:379) */
    float kb_b;         /* KB shape, 14.9086 (Reco.cpp:378) */
    double kb_thresh;   /* relative tap threshold, 1e-7 (Reco.cpp:717) */
    double adj_scale;   /* adjoint rescale, 1e-3 (Reco.cpp:482) */
    int32_t offcenter[3];/* image offset inside the grid beyond centring (Reco.cpp:645-650) */
} cgso_params;

typedef struct {
    int32_t sx, sy, sz;          /* readout samples, phase-encode lines y, z (Reco.h setSampling) */
    int32_t gx, gy, gz;          /* grid size (used for the border normalisation) */
    double fov_y, fov_z;         /* m */
    int32_t n_osc;               /* wave cycles along the readout */
    double grad_amp;             /* T/m */
    double amp_corr_y, amp_corr_z;
    double shift_y, shift_z;     /* s */
    double dwell;                /* s */
} cgso_wave;

/* Modified Bessel function I0 by its power series, double precision. */
double cgso_bessel_i0(double x);

/* Reco::ConvKernel::convFunction (Reco.h:218-242): separable KB value for
 * per-axis distances in k-space units. */
float cgso_conv_function(const cgso_params* p, const double dist[3]);

/* ConvKernel::calculateWeights + excludeMissingData (Reco.cpp:681-806).
 * counts[i] = number of taps of sample i (0 where mask[i] == 0).
 * Returns the total tap count. */
int64_t cgso_tap_counts(const cgso_params* p, const double* k, int64_t ns,
                        const uint8_t* mask, int32_t* counts);
/* Fills CSR tap lists; ptr has ns+1 entries (prefix sum of counts). */
void cgso_taps_fill(const cgso_params* p, const double* k, int64_t ns, const uint8_t* mask,
                    const int64_t* ptr, int32_t* idx, float* w);

/* ConvKernel::calculateKernelFT (Reco.cpp:560-601): kft[Ng] complex. */
void cgso_kernel_ft(const cgso_params* p, cgso_real* kft);

/* Fourier::transformFWD / transformBWD (Fourier.cpp:19-42), in place on a grid. */
void cgso_centred_fft(const cgso_params* p, cgso_real* a, int sign, int rescale);

/* Reco::nufftFWD (Reco.cpp:521-553), all coils.
 * img: [n_ch][img voxels] complex; data: [n_ch][ns] complex (overwritten). */
void cgso_nufft_fwd(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                    int64_t ns, const cgso_real* kft, const cgso_real* img, cgso_real* data);

/* Reco::nufftBWD (Reco.cpp:468-519), all coils.
 * data: [n_ch][ns]; img: [n_ch][img voxels] (cropped to the image box). */
void cgso_nufft_adj(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                    int64_t ns, const cgso_real* kft, const cgso_real* data, cgso_real* img);

/* One application of A = sum_c conj(S_c) E_c^H D E_c S_c (Reco.cpp:232-262).
 * dcf may be NULL (no density correction). */
void cgso_apply_ehde(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                     int64_t ns, const cgso_real* kft, const cgso_real* smaps, const float* dcf,
                     const cgso_real* x, cgso_real* q);

/* Reco::cgSenseDynamic (Reco.cpp:175-321) including the preceding density
 * correction of the measured samples (functions.h:319-335, CGSense.cpp:226)
 * and the coil-image step nufftBWD (CGSense.cpp:235).
 * data: [n_ch][ns] measured samples (not modified).
 * Returns 0, or -1 when the NaN/Inf check fires (Reco.cpp:264-268).
 * max_iter: the reference runs at most 16 bodies (Reco.cpp:228,308-309). */
int cgso_cg_sense(const cgso_params* p, const int64_t* ptr, const int32_t* idx, const float* w,
                  int64_t ns, const cgso_real* kft, const cgso_real* smaps, const float* dcf,
                  const cgso_real* data, double threshold, int max_iter,
                  cgso_real* x_out, double* residuals, int32_t* iters_out);

/* Data-consistency loss and its gradients -- an extension: the reference has
 * no derivatives.  E_c is the forward operator of cgso_nufft_fwd applied to
 * S_c x (zero-pad, kernelFT, centred FFT, KB interpolation; Reco.cpp:521-553):
 *   L         = 1/2 sum_c sum_i D_i |(E_c S_c x)_i - y_ci|^2
 *   grad_x    = dL/dRe(x) + i dL/dIm(x) = sum_c conj(S_c) E_c^* (D r_c),
 *               E^* the exact adjoint (no 1e-3 / sqrt(Ng) rescale)
 *   grad_k    = dL/dk[i][a], k in the reference's [0,1] units
 * The KB weights and their derivatives are evaluated in double from the
 * double coordinates (the reference rounds the distance to float), so L is
 * smooth in k between changes of the tap set.  dcf NULL: D = 1.  grad_x and
 * grad_k may be NULL.  Returns L. */
double cgso_loss_grad(const cgso_params* p, const double* k, int64_t ns, const cgso_real* kft,
                      const cgso_real* smaps, const float* dcf, const cgso_real* x, const cgso_real* y,
                      cgso_real* grad_x, double* grad_k);

/* Modified Bessel function I1 by its power series, double precision. */
double cgso_bessel_i1(double x);

/* WaveCaipi::calculateTraj with Trajectory::calculateKMax (Trajectory.cpp:9-184).
 * k_out: [sx*sy*sz][3] in the reference's z-fastest sample order. */
void cgso_wave_caipi(const cgso_wave* w, double* k_out);

#ifdef __cplusplus
}
#endif
#endif
