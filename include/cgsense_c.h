/*
 * cgsense_c.h -- C ABI of the GB300 CG-SENSE library (libcgsense.so).
 *
 * The library implements the CG-SENSE encoding operator E^H D E of
 * expRad/4d_lung (CGSense/Reco.cpp) and the conjugate-gradient solve around
 * it on one NVIDIA GB300 GPU (sm_103a kernels).  It is the drop-in boundary
 * for the reference's reconstruction object: every entry point below names
 * the reference member function it replaces.  Plain pointers and sizes only.
 *
 * Conventions (all kept from the reference):
 *   - complex data are interleaved float pairs (re, im), bit-compatible with
 *     fftwf_complex;
 *   - grids and images are row-major [x][y][z], z fastest (Reco.cpp:603-606);
 *   - samples are in the reference's memory order, z-fastest
 *     (IO.cpp:109-125, Trajectory.cpp:167-175); per-coil sample arrays are
 *     [coil][sample] (Reco.cpp:478-479);
 *   - the trajectory is k in [0,1]^3 per sample, grid coordinate k*(N-1)
 *     (Reco.cpp:751-755);
 *   - the forward NUFFT is unscaled; the adjoint is scaled by
 *     adj_scale / sqrt(N_grid) (Reco.cpp:482, Fourier.cpp:31-41).
 *
 * Errors: every function returns CGS_OK (0) or a CGS_ERR_* code and stores a
 * message retrievable with cgs_last_error().  The reference instead prints
 * and calls exit(EXIT_FAILURE); the C++ drop-in shim (cgsense/Reco.h) maps a
 * non-zero status to that behaviour.
 *
 * Threading: one context per host thread.  Each context owns (or borrows,
 * cgs_set_stream) one CUDA stream.  Host-pointer calls are synchronous;
 * "_d" calls take device pointers and are asynchronous on the context's
 * stream.
 */
#ifndef CGSENSE_C_H
#define CGSENSE_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGS_OK 0
#define CGS_ERR_ARG 1          /* invalid argument or size */
#define CGS_ERR_CUDA 2         /* CUDA runtime error */
#define CGS_ERR_NONFINITE 3    /* NaN/Inf in the CG iterate (Reco.cpp:264-268) */
#define CGS_ERR_STATE 4        /* call order: e.g. no trajectory or coil maps set */
#define CGS_ERR_NOMEM 5        /* device allocation failed */
#define CGS_ERR_UNSUPPORTED 6  /* grid size without an FFT kernel */
#define CGS_ERR_NO_THRESHOLD 7 /* cg threshold == -1 (Reco.cpp:192-196) */
#define CGS_ERR_TIMEOUT 8      /* a kernel's bounded wait for its asynchronous copies ran out */
#define CGS_ERR_IO 9           /* a file could not be opened, read or written (IO.cpp) */

typedef struct cgs_ctx cgs_ctx;

/* Reconstruction parameters.  Replaces Reco::setGridSize / setNCh /
 * setOffcenter (Reco.h:112-121) and ConvKernel::setB / setW /
 * setKernelOrder (Reco.h:53-55, values set in Reco::init, Reco.cpp:377-380). */
typedef struct cgs_params {
    int32_t img[3];       /* image size; the reference uses img == grid */
    int32_t grid[3];      /* Cartesian grid size (even, from the supported FFT list) */
    int32_t n_ch;         /* coils */
    int32_t kb_order;     /* neighbour scan half-width (5) */
    float kb_w;           /* KB width in grid cells (4.25); must be < 5 */
    float kb_b;           /* KB shape (14.9086) */
    double kb_thresh;     /* relative tap threshold (1e-7) */
    double adj_scale;     /* adjoint rescale (1e-3) */
    int32_t offcenter[3]; /* image offset inside the grid beyond centring */
    int32_t device;       /* CUDA device ordinal */
    int64_t workspace_bytes; /* device workspace budget for batched bins (0: default) */
} cgs_params;

/* Wave-CAIPI parameters.  Replaces the WaveCaipi setters
 * (Trajectory.h:52-60) together with Reco::setSampling / setGridSize /
 * setFovY / setFovZ (Reco.h:108,112,122-123). */
typedef struct cgs_wave {
    int32_t sx, sy, sz;
    int32_t gx, gy, gz;
    double fov_y, fov_z;
    int32_t n_osc;
    double grad_amp;
    double amp_corr_y, amp_corr_z;
    double shift_y, shift_z;
    double dwell;
} cgs_wave;

/* Reference defaults: b = 14.9086, w = 4.25, order 5 (Reco.cpp:377-380),
 * threshold 1e-7 (Reco.cpp:717), adjoint scale 1e-3 (Reco.cpp:482). */
void cgs_default_params(cgs_params* p);

/* Reco::init + Reco::ConvKernel::calculateKernelFT + Fourier::initFT
 * (Reco.cpp:374-400, 560-601; Fourier.cpp:4-17). */
int cgs_create(const cgs_params* p, cgs_ctx** out);
/* Reco::~Reco (Reco.cpp:29-61). */
void cgs_destroy(cgs_ctx* ctx);
const char* cgs_last_error(const cgs_ctx* ctx);
/* Use an external CUDA stream (cudaStream_t); NULL returns to the context's own stream. */
int cgs_set_stream(cgs_ctx* ctx, void* stream);
/* Block until the context's stream is idle. */
/* The CUDA stream the context's work is issued on (its own or the one set
 * by cgs_set_stream). */
void* cgs_get_stream(const cgs_ctx* ctx);
int cgs_sync(cgs_ctx* ctx);

/* WaveCaipi::calculateTraj with Trajectory::calculateKMax (Trajectory.cpp:9-184):
 * k_out[(sx*sy*sz)][3], z-fastest sample order. Host only. */
int cgs_wave_caipi(const cgs_wave* w, double* k_out);

/* Reco::setTrajectory (Reco.cpp:324-336) followed by
 * ConvKernel::calculateWeights (Reco.cpp:698-806): the KB taps are evaluated
 * on the GPU.  k[ns][3] on the host.  Resets bins to one bin of all samples. */
int cgs_set_trajectory(cgs_ctx* ctx, const double* k, int64_t ns);

/* ConvKernel::excludeMissingData (Reco.cpp:681-696): samples with
 * mask[i] == 0 get no taps.  One bin of the unmasked samples.  NULL clears. */
int cgs_set_mask(cgs_ctx* ctx, const uint8_t* mask);
/* Same, with the mask taken where coil 0's sample is exactly 0+0i, as the
 * reference does.  data: host [n_ch][ns] complex. */
int cgs_mask_from_data(cgs_ctx* ctx, const float* data);

/* Respiratory bins (the reference reconstructs one state file at a time,
 * CGSense.cpp:200-282): bin b holds samples sample_idx[offsets[b] ..
 * offsets[b+1]).  Bins may differ in size. */
int cgs_set_bins(cgs_ctx* ctx, int32_t nbins, const int64_t* offsets, const int32_t* sample_idx);
int cgs_num_bins(const cgs_ctx* ctx);

/* estimateDensityV3D (functions.h:161-258, Density::VORONOI3D): the Voronoi
 * cell volume of every sample of k[n][3], 0 for samples on the convex hull,
 * divided by the largest volume.  Host computation (OpenMP); usable per bin
 * by passing that bin's coordinates. */
int cgs_voronoi_dcf(const double* k, int64_t n, float* dcf);

/* estimateDensityV3D(traj, sX, sY, sZ, average, cutoff) (functions.h:161-258)
 * with its readout averaging: average != 0 replaces every volume by the sum
 * over all readouts of the volumes at its readout position i % sX (the
 * position clamped to (sX - 1) * cutoff), divided by the total, before the
 * division by the maximum.  n must be a multiple of sX when averaging;
 * average == 0 is cgs_voronoi_dcf. */
int cgs_estimate_density_v3d(const double* k, int64_t n, int32_t sX, int32_t average, double cutoff, float* dcf);

/* Iterative density weights on the GPU (Pipe and Menon 1999), the
 * documented alternative to the Voronoi volumes: `iters` rounds of
 * w <- w / (C * w) per bin, C * w the interpolation of the spread weights
 * on the bin's grid (the KB gridding of Reco.cpp:492-550 without the FFT),
 * then normalised by each bin's maximum.  dcf float [ns] in the reference's
 * sample order (device pointer when on_device != 0); samples in no bin get
 * 0.  Needs the trajectory and bins, not the coil maps. */
int cgs_pipe_menon_dcf(cgs_ctx* ctx, int32_t iters, float* dcf, int32_t on_device);

/* Reco::denCorr with Density::IMPORT (IO.cpp:129-156, functions.h:319-335):
 * per-sample real weights D[ns].  NULL clears (Density::NONE). */
int cgs_set_dcf(cgs_ctx* ctx, const float* dcf);

/* IO::importSensitivityMaps result (IO.cpp:25-51), Reco::sMaps: host
 * [n_ch][image voxels] complex. */
int cgs_set_smaps(cgs_ctx* ctx, const float* maps);
int cgs_set_smaps_d(cgs_ctx* ctx, const float* maps_dev);

/* ConvKernel::kernelFT (Reco.cpp:560-601) as the grid volume the reference
 * stores (1/Re of the centred backward FFT of the sampled KB kernel):
 * host [grid voxels] complex. */
int cgs_kernel_ft(cgs_ctx* ctx, float* kft);

/* Fourier::transformFWD (sign -1) / transformBWD (sign +1, rescale 0|1)
 * (Fourier.cpp:19-42), in place on a host grid [grid voxels] complex. */
int cgs_fft3(cgs_ctx* ctx, float* grid, int32_t sign, int32_t rescale);
int cgs_fft3_d(cgs_ctx* ctx, float* grid_dev, int32_t sign, int32_t rescale);

/* Reco::nufftFWD (Reco.cpp:521-553): img[n_ch][image voxels] ->
 * data[n_ch][ns].  Samples outside every bin are set to 0. */
int cgs_nufft_fwd(cgs_ctx* ctx, const float* img, float* data);
int cgs_nufft_fwd_d(cgs_ctx* ctx, const float* img_dev, float* data_dev);
/* Reco::nufftBWD (Reco.cpp:468-519): data[n_ch][ns] -> img[n_ch][image voxels].
 * D is not applied (the reference applies it to `data` beforehand). */
int cgs_nufft_adj(cgs_ctx* ctx, const float* data, float* img);
int cgs_nufft_adj_d(cgs_ctx* ctx, const float* data_dev, float* img_dev);

/* One operator application of the CG loop (Reco.cpp:232-262):
 * q = sum_c conj(S_c) E_c^H D E_c (S_c x) for the samples of bin `bin`.
 * x, q: [image voxels] complex. */
int cgs_apply_ehde(cgs_ctx* ctx, int32_t bin, const float* x, float* q);
/* Bins [bin0, bin0+nb): x, q are [nb][image voxels] device arrays. */
int cgs_apply_ehde_d(cgs_ctx* ctx, int32_t bin0, int32_t nb, const float* x_dev, float* q_dev);

/* Reco::cgSenseDynamic (Reco.cpp:175-321), preceded by the density
 * correction of the measured samples and the coil-image step nufftBWD
 * (CGSense.cpp:226-235).  Bin 0 only (the single-state reconstruction).
 * data: [n_ch][ns] measured samples; x: [image voxels] result (cgSenseImg);
 * residuals: max_iter entries (cgResiduals); iters: performed iterations
 * (numPerformedCGIterations).  threshold == -1 fails like the reference.
 * The reference's cap is 16 iterations (max_iter = 16). */
int cgs_cg_solve(cgs_ctx* ctx, const float* data, float* x, double threshold, int32_t max_iter,
                 double* residuals, int32_t* iters);

/* Reco::cgSenseDynamic exactly as the reference calls it: its inputs are the
 * coil images `img` already produced by nufftBWD from density-corrected
 * samples (CGSense.cpp:226-235) and the coil maps; the loop applies D from
 * cgs_set_dcf.  coil_imgs: host [n_ch][image voxels]; bin 0 only. */
int cgs_cg_solve_images(cgs_ctx* ctx, const float* coil_imgs, float* x, double threshold, int32_t max_iter,
                        double* residuals, int32_t* iters);

/* All bins in one graph-captured launch sequence (the 4D reconstruction of
 * CGSense.cpp:200-282 without its file IO): x[nbins][image voxels],
 * residuals[nbins][max_iter], iters[nbins]. */
int cgs_cg_solve_batched(cgs_ctx* ctx, const float* data, float* x, double threshold, int32_t max_iter,
                         double* residuals, int32_t* iters);
/* Device-pointer variant; residuals/iters stay host pointers (filled after
 * the solve completes). */
int cgs_cg_solve_batched_d(cgs_ctx* ctx, const float* data_dev, float* x_dev, double threshold,
                           int32_t max_iter, double* residuals, int32_t* iters);

/* fftwf_alloc_complex / fftwf_free counterparts for host buffers handed to
 * the library (Reco.cpp:441,447,454): page-locked memory when a GPU is
 * present, so that transfers run at full speed. */
void* cgs_alloc_host(size_t bytes);
void cgs_free_host(void* p);

/* The plain per-bin GPU form of cgs_cg_solve_batched_d, kept as the
 * comparison point: bins one after another, coils one after another,
 * unfused kernels, full-grid cuFFT transforms, global-atomic spreading, a
 * host round trip per iteration (the reference's loop structure,
 * Reco.cpp:175-321, 468-553).  Same arguments and results. */
int cgs_cg_solve_plain_d(cgs_ctx* ctx, const float* data_dev, float* x_dev, double threshold, int32_t max_iter,
                         double* residuals, int32_t* iters);

/* cgs_cg_solve_batched_d that also stores x after every iteration:
 * x_trace [max_iter][nbins][image voxels] complex64 (device).  Used to state
 * the error of every iteration against the FP64 form. */
int cgs_cg_solve_trace_d(cgs_ctx* ctx, const float* data_dev, float* x_dev, double threshold, int32_t max_iter,
                         double* residuals, int32_t* iters, float* x_trace_dev);

/* The same solve entirely in FP64 on the GPU (double-complex images, grids,
 * samples, cuFFT Z2Z, FP64 CG), the precision reference of the complex64
 * path: x [nbins][image voxels] complex128 (device); x_trace (optional)
 * [max_iter][nbins][image voxels] complex128. */
int cgs_cg_solve_fp64_d(cgs_ctx* ctx, const float* data_dev, double* x_dev, double threshold, int32_t max_iter,
                        double* residuals, int32_t* iters, double* x_trace_dev);

/* Number of kernel launches issued by the last compute call (for a graph
 * replay: the kernels in the graph). */
int64_t cgs_last_launch_count(const cgs_ctx* ctx);

/* Per-stage timing of one E^H D E application (the reference prints
 * wall-clock times only, CGSense.cpp:122-135,257-261): runs
 * cgs_apply_ehde_d on device arrays with a CUDA event after every kernel and
 * returns the kernel durations in launch order (forward z, y, x passes,
 * interpolation, spreading, adjoint x, y, z passes; repeated per group of
 * bins).  stage_ms holds max_stages floats; n_stages receives the count. */
int cgs_profile_apply(cgs_ctx* ctx, int32_t bin0, int32_t nb, const float* x_dev, float* q_dev,
                      float* stage_ms, int32_t max_stages, int32_t* n_stages);

/* --- Differentiation (an extension: the reference has no derivatives) ---
 * Data-consistency loss of bin `bin`, with E_c the forward operator of
 * nufftFWD (Reco.cpp:521-553) applied to S_c x and D the density weights:
 *   L      = 1/2 sum_c sum_i D_i |(E_c S_c x)_i - y_ci|^2
 *   grad_x = dL/dRe(x) + i dL/dIm(x) = sum_c conj(S_c) E_c^* (D r_c)
 *            (E^* the exact adjoint: no 1e-3 / sqrt(Ng) rescale)
 *   grad_k = dL/dk[i][a], k in the reference's [0,1] units; 0 for samples
 *            outside the bin.
 * Device pointers: x complex64 [Ni]; y complex64 [n_ch][ns] in the
 * reference's sample order; grad_x complex64 [Ni] or NULL; grad_k float
 * [ns][3] or NULL.  FP32 gridding and FFT (the product path); *loss is the
 * FP64 sum of per-sample FP32 terms. */
int cgs_loss_grad_d(cgs_ctx* ctx, int32_t bin, const void* x_dev, const void* y_dev, double* loss,
                    void* grad_x_dev, void* grad_k_dev);

/* The same loss and gradients in FP64 (the gradient reference): x and
 * grad_x complex128, grad_k double [ns][3]; KB weights and their
 * derivatives in double from the double coordinates, cuFFT Z2Z. */
int cgs_loss_grad_fp64_d(cgs_ctx* ctx, int32_t bin, const void* x_dev, const void* y_dev, double* loss,
                         void* grad_x_dev, void* grad_k_dev);

/* New coordinates for the same samples (device pointer, double [ns][3]),
 * e.g. one step of trajectory self-calibration: the tap records are
 * recomputed on the device; the spreading lists are rebuilt lazily by the
 * next call that spreads. */
int cgs_update_trajectory_d(cgs_ctx* ctx, const double* k_dev);

/* Right-hand side of the CG solve for bins [bin0, bin0 + nb):
 * b[bin] = sum_c conj(S_c) E_c^H (D y_c)  (CGSense.cpp:226-235, Reco.cpp:182-190),
 * with the reference's rescale.  y complex64 [n_ch][ns]; b complex64 [nb][Ni]. */
int cgs_rhs_d(cgs_ctx* ctx, int32_t bin0, int32_t nb, const void* y_dev, void* b_dev);

/* Trajectory vector-Jacobian products of the solve's building blocks, for
 * backpropagation through an unrolled CG (all device pointers; grad_k is
 * float [ns][3] and ACCUMULATED, +=):
 *   cgs_apply_vjp_k_d: grad_k += d/dk Re<v, A(k) p>, A = E^H D E of
 *                      cgs_apply_ehde_d, p and v complex64 [nb][Ni];
 *   cgs_rhs_vjp_k_d:   grad_k += d/dk Re<v, b(k)>, b of cgs_rhs_d. */
/* Serial number of the context's coordinates: changes whenever
 * cgs_set_trajectory or cgs_update_trajectory_d sets new ones (callers that
 * cache an uploaded trajectory compare it). */
uint64_t cgs_trajectory_serial(const cgs_ctx* ctx);

int cgs_apply_vjp_k_d(cgs_ctx* ctx, int32_t bin0, int32_t nb, const void* p_dev, const void* v_dev, void* grad_k_dev);
int cgs_rhs_vjp_k_d(cgs_ctx* ctx, int32_t bin0, int32_t nb, const void* y_dev, const void* v_dev, void* grad_k_dev);

/* Accumulation mode of the spreading (the adjoint gridding, Reco.cpp:492-504):
 * CGS_PREC_FP32 (default) plain FP32 sums in a fixed order; CGS_PREC_COMPENSATED
 * Kahan-compensated FP32 sums (the precision form).  FFT passes are FP32 and
 * the CG scalars FP64 in both. */
#define CGS_PREC_FP32 0
#define CGS_PREC_COMPENSATED 1
int cgs_set_precision(cgs_ctx* ctx, int32_t mode);

/* Fixed summation order (default on): every result is bitwise reproducible.
 * Off, the autotuner may also pick spreading with shared-memory atomics
 * (results then vary in the last bits from run to run, as the reference's
 * OpenMP atomics do). */
int cgs_set_deterministic(cgs_ctx* ctx, int32_t on);

/* Launch shape set by hand (what cgs_autotune picks): coils per spreading
 * block (0: as many as fit), spreading variant (1 / 2: one / two warps per x
 * plane of a tile; 3: shared-memory atomics, only with determinism off;
 * 4 / 5: persistent and software-pipelined with one / two warps per plane;
 * 6: a gather over the transposed tap matrix, built with the bins when
 * sample-support pruning is on -- without it variant 2 runs -- whose row
 * offsets and taps are staged in shared memory by bulk copies; 7: the same
 * gather reading the matrix from global memory; for 6 and 7 spread_cc is the
 * coils per thread, 2, 4, 6 or 8, 0 by the coil count; 8 (default): the
 * staged gather fused with the adjoint x pass, one block per listed
 * 8-column tile and chunk of spread_cc coils (2, 4 or 6, 0 by the coil
 * count), the grid kept in shared memory -- where the grid is not twice the
 * image along x, or the coil count has no such chunk, variant 6 runs),
 * coils per interpolation thread (1, 2, 4, 6, 8).  Variants 1, 2, 4, 5, 6,
 * 7, 8 and every interpolation shape give bitwise-identical results. */
int cgs_set_launch_shape(cgs_ctx* ctx, int32_t spread_cc, int32_t spread_variant, int32_t interp_cc);

/* Sample-support pruning of the oversampled FFT (default on): the x passes
 * transform only the tiles of grid columns that some sample's kernel support
 * reaches, the forward y pass stores only those columns and the adjoint y
 * pass reads the others as zero.  Results are unchanged (a column no sample
 * reaches is never read by the interpolation, and is all zero after the
 * spreading); off, every column is transformed (the reference's full FFT,
 * Fourier.cpp:19-42). */
int cgs_set_support_pruning(cgs_ctx* ctx, int32_t on);

/* Toeplitz embedding of E^H D E (fixed trajectory): mode 1 replaces the
 * gridded normal operator inside cgs_apply_ehde* and the CG solvers by
 *   q = s sum_c conj(S_c) crop F_c^H (P_b . F_c pad(S_c x)),
 * P_b the real spectrum of bin b's point-spread function
 *   h(d) = sum_i D_i exp(2 pi i nu_i . d),  nu_ia = (k_ia (G_a - 1) - G_a / 2) / G_a,
 * on the oversampled grid (needs G_a >= 2 I_a - 1), s the adjoint scale:
 * the exact non-uniform DFT's normal operator, with no gridding inside the
 * CG loop.  It differs from the gridded operator by the gridding error
 * (about 1e-3 relative at kernel width 4 and 2x oversampling).  The
 * right-hand side stays the gridded adjoint of the data; the trajectory
 * derivatives keep the gridded operator.  The spectra (4 bytes per grid
 * point and bin) are built from the current coordinates, bins and density
 * weights (cgs_set_toeplitz_spectrum says how) and rebuilt after any of
 * them changes.  Mode 2: the same
 * operator with the x stage unfused (forward x pass, multiply, adjoint x
 * pass; for comparison).  Mode 0 (default): the gridded operator; the
 * spectra are released.  cgs_apply_vjp_k_d (the derivative of the gridded
 * operator) fails with CGS_ERR_STATE while the embedding is on. */
int cgs_set_toeplitz(cgs_ctx* ctx, int32_t mode);
/* Time of the last spectrum build (ms) and the bytes the spectra hold (0
 * while not built). */
int cgs_toeplitz_stats(cgs_ctx* ctx, double* build_ms, int64_t* bytes);

/* How the Toeplitz spectra are built (an extension; the reference has no
 * Toeplitz embedding, and its normal operator is the gridded one of
 * Reco.cpp:175-321).  method 0 (default): through each bin's point-spread
 * function h(d) = sum_i D_i exp(2 pi i nu_i . d), computed by an adjoint
 * NUFFT of the density weights -- Kaiser-Bessel window of width 7 on a
 * fine grid of at least 4 I points per axis, FP64 accumulation, the
 * library's FFT passes -- then the grid's transform; O(M w^3 + N log N) per
 * bin, window error ~5e-7 relative.  Used when every fine-grid axis has an
 * FFT line length (4 I <= 512), else the Dirichlet product.  method 1: the
 * Dirichlet-kernel product of every sample with every grid point (exact to
 * FP32 rounding, 2 Ng M flops per bin, cuBLAS).  Changing the method
 * rebuilds the spectra. */
int cgs_set_toeplitz_spectrum(cgs_ctx* ctx, int32_t method);
/* Method of the last spectrum build: 1 point-spread function, 2 Dirichlet
 * product, 0 while no spectra are built. */
int cgs_toeplitz_spectrum_method(const cgs_ctx* ctx);

/* Set-up cost of the current bins (host clock, milliseconds; the part of
 * ConvKernel::calculateWeights, Reco.cpp:698-806, that the reference repeats
 * per state, CGSense.cpp:218-222, plus this library's own set-up): ms[0]
 * sorting the samples by home tile, ms[1] the tap records on the device,
 * ms[2] the tile and support lists, ms[3] the transposed tap matrix, ms[4]
 * the remaining uploads and the grid workspaces -- all from the last
 * rebuild of the bins -- and ms[5] the capture and instantiation of the
 * last CUDA graph of a batched solve.  n: entries wanted (at most 6). */
int cgs_setup_stats(cgs_ctx* ctx, double* ms, int32_t n);

/* Device time of the parts of the last cgs_cg_solve_batched call (CUDA
 * events on the context's stream, ms): ms[0] the upload of the samples,
 * ms[1] the solve's graph, ms[2] the download of the images.
 * pinned (optional, 2 entries): 1 where the call's data / image buffer was
 * page-locked memory as the library's CUDA runtime sees it (cgs_alloc_host
 * gives such memory); copies from other memory are staged and slower.  A
 * diagnostic of the host-buffer path of CGSense.cpp:226-266 (import, solve,
 * export) with no counterpart call in the reference. */
int cgs_e2e_stats(cgs_ctx* ctx, double* ms, int32_t* pinned);

/* Coil sensitivity maps from the measured data of a single-bin context
 * (device pointers; data [n_ch][ns] in the reference's order, maps
 * [n_ch][img]): the adjoint NUFFT of each coil's samples weighted by a Hann
 * window of `radius` grid cells around the k-space centre (times the
 * density weights when set), divided by the coils' root-sum-of-squares
 * where that exceeds eps times its maximum, 0 elsewhere.  A low-resolution
 * estimate for the SENSE solve when no map files exist (the reference reads
 * maps, IO.cpp:25-51, and exports the root-sum-of-squares,
 * functions.h:290-316, for external estimation). */
int cgs_estimate_smaps_d(cgs_ctx* ctx, const void* data, double radius, double eps, void* maps);

/* Per bin (arrays of cgs_num_bins entries, either may be NULL): the (y, z)
 * grid columns the x passes transform (whole column tiles of the pass) and
 * the spreading tiles stored, as the current pruning setting uses them
 * (without pruning: every column, every tile). */
int cgs_support_stats(cgs_ctx* ctx, int64_t* listed_cols, int64_t* live_tiles);

/* 1 when the forward y pass stores only the rows of the x pass's listed
 * tiles (sample-support pruning on and the passes' column tiles coincide),
 * else 0. */
int cgs_forward_y_listed_rows(cgs_ctx* ctx, int32_t* listed);

/* The transposed tap matrix of spreading variants 6 to 8 (all bins): its taps
 * (entries) and grid points (rows); both 0 when it is not built. */
int cgs_spread_matrix_stats(cgs_ctx* ctx, int64_t* taps, int64_t* points);

/* *fused = 1 when the last operator application ran the spreading fused
 * with the adjoint x pass (variant 8 where it applies; one launch in place
 * of two), else 0. */
int cgs_spread_fused(cgs_ctx* ctx, int32_t* fused);

/* Autotuner: times one batched E^H D E application of every bin for each
 * candidate launch shape -- the spreading variants of cgs_set_launch_shape
 * (tiled kernels with coils per block all that fit, then 1/2, 1/3, 1/4 of
 * them; the transposed-matrix gather with 4, 6 or 8 coils per thread; the
 * gather fused with the adjoint x pass with 2, 4 or 6 coils per block), then
 * coils per interpolation thread (1, 2, 4, 6, 8) -- and keeps the fastest for
 * this context.  times_ms (may be NULL) receives the median time of each
 * candidate in that order; the chosen shape is returned in *spread_cc,
 * *spread_wpp (the spreading variant) and *interp_cc (each may be NULL). */
int cgs_autotune(cgs_ctx* ctx, float* times_ms, int32_t max_times, int32_t* n_times, int32_t* spread_cc,
                 int32_t* spread_wpp, int32_t* interp_cc);

/* Centred 3-D FFT (sign -1 forward, +1 backward, unscaled) that allocates no
 * device memory, for callers that cannot let a library allocate: code
 * running under a host application that owns all device memory through its
 * own allocator, or a latency-critical loop that must not pay for
 * cudaMalloc/cudaFree.  No counterpart in the reference.  in and out are
 * device arrays of grid[0]*grid[1]*grid[2] complex values (they may be the
 * same array), each 8-byte aligned (a misaligned pointer is CGS_ERR_ARG,
 * checked before any launch); no context is needed.  The intermediate grid
 * lives in a fixed file-scope device array of 2^19 complex values (4 MiB,
 * held by every GPU that loads the library); larger grids are rejected with
 * CGS_ERR_ARG, sizes without an FFT kernel with CGS_ERR_UNSUPPORTED
 * (messages go to stderr).  The first call in each CUDA context looks up
 * that array's device address there (cached per device and context), so
 * make that first call before any stream capture; cudaDeviceReset between
 * calls is not supported (the driver may hand the new context the old
 * handle, and the cached address would be stale).  All calls share the
 * array: calls that overlap on the GPU race and must be serialised.  stream
 * is a cudaStream_t (NULL: the default stream); the call is asynchronous. */
int cgs_fft3_noalloc(const float* in_dev, float* out_dev, const int32_t* grid, int32_t sign, void* stream);

/* --- File IO of the reconstruction (IO.cpp), context-free --------------
 * stream: CUDA stream of the device work, NULL for the default stream. */

/* IO::importDataBin (IO.cpp:55-98): reads nch * sx*sy*sz complex64 samples
 * (interleaved float32) stored channel by channel in readout-fastest order
 * (sample i1 + sx*i2 + sx*sy*i3) and writes them to the device in the
 * reconstruction's z-fastest order (ch*ns + i3 + sz*i2 + sy*sz*i1).  The
 * file is read in chunks through two pinned host buffers (the next chunk is
 * read while the previous one is copied) and permuted by a kernel.  A
 * missing or short file is CGS_ERR_IO. */
int cgs_import_data_bin(const char* path, int32_t sx, int32_t sy, int32_t sz, int32_t nch, void* data_dev,
                        void* stream);

/* The permutation of cgs_import_data_bin alone, device to device. */
int cgs_permute_samples_d(const void* file_order_dev, void* data_dev, int32_t sx, int32_t sy, int32_t sz,
                          int32_t nch, void* stream);

/* IO::exportFFTWComplexBin (IO.cpp:158-186): n complex64 values as
 * interleaved float32; a path that cannot be opened is retried as
 * path + "_1.bin".  src is a device pointer when src_on_device != 0. */
int cgs_export_complex_bin(const char* path, const void* src, int64_t n, int32_t src_on_device, void* stream);

/* IO::exportVectorBin (IO.cpp:12-22): n float32 values. */
int cgs_export_float_bin(const char* path, const void* src, int64_t n, int32_t src_on_device, void* stream);

/* IO::importSensitivityMaps (IO.cpp:25-51): dir + "map<c>.bin", n complex64
 * values each, into maps_host [nch][n]. */
int cgs_import_smaps_bin(const char* dir, int64_t n, int32_t nch, float* maps_host);

/* IO::importDensityCorr (IO.cpp:129-156): n float32 weights. */
int cgs_import_density_bin(const char* path, int64_t n, float* d_host);

/* rssq2DVecImg (functions.h:290-316) on the device: out[i] =
 * sqrt(sum_c |img_c[i]|^2), coils summed in order in float.  imgs: complex64
 * [nch][n]; out float32 [n]. */
int cgs_rss_d(const void* imgs_dev, int32_t nch, int64_t n, float* out_dev, void* stream);

/* The state loop of CGSense.cpp:200-282 on the GPU: for every state file,
 * IO::importDataBin (the next file is read on a host thread while the
 * current state is reconstructed), excludeMissingData, density correction
 * with the context's weights, the coil images and their root-sum-of-squares
 * exported as out_dir/resultRssq.bin (float32, img voxels) when
 * write_rss != 0, cgSenseDynamic, and the image exported as
 * out_dir/results/b_state<k>.bin (complex64).  iters (may be NULL) receives
 * the iteration count of every state.  Coil maps and trajectory must be set
 * (one bin). */
int cgs_reconstruct_states(cgs_ctx* ctx, const char* const* files, int32_t n_files, int32_t sx, int32_t sy,
                           int32_t sz, const char* out_dir, double thresh, int32_t max_iter, int32_t write_rss,
                           int32_t* iters);

#ifdef __cplusplus
}
#endif
#endif /* CGSENSE_C_H */
