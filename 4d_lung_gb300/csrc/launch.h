// launch.h -- host-side launch interface of the CG-SENSE kernels.
#pragma once
#include <cuda_runtime.h>
#include "cgs_types.h"
#include <cufft.h>
#include <cuda.h>
#include <string>

namespace cgs {

// Supported line lengths of the 3-D FFT (each a product R1*R2 of two
// register codelets).  Grid sizes must be taken from this list.
bool fft_supported(int L);
// per-device kernel attributes of the FFT passes (dynamic shared memory)
cudaError_t fft_init_all();
// 4-D tensor map [batch][A][Lin][B] of a strided pass's input with a
// TB x box_rows box; false when the buffer or strides are not 16-byte aligned.
// promo: L2 promotion of the box's rows in bytes (64, 128 or 256)
bool encode_strided_map(CUtensorMap* map, const StridedPassArgs& a, int A, int batch, int TB, int* box_rows,
                        int promo = 256);
// 3-D tensor map [nbins][L][B] of 4-byte spectrum values with a TB x
// box_rows box; false when the buffer or pitch is not 16-byte aligned
bool encode_spectrum_map(CUtensorMap* map, const float* P, long long B, int L, int nbins, int TB, int* box_rows);
const int* fft_supported_list(int* n);
// columns per tile of the strided passes of line length L (0: unsupported)
int fft_strided_cols(int L);
// columns per listed tile of the x passes over the sample support of a grid
// of L points along x holding an image of I points from row lo: the narrow
// tiles when both x passes run half-pruned (4 lo == L, 2 I == L), else the
// strided passes' width (0: unsupported)
int fft_listed_cols(int L, int lo, int I);

// One launch per pass; `batch` items along blockIdx.y.
cudaError_t launch_strided(int L, int sign, const StridedPassArgs& a, int A, int batch, cudaStream_t s);
cudaError_t launch_contig(int L, int sign, const ContigPassArgs& a, int batch, cudaStream_t s);
cudaError_t launch_fwd_z(int L, const FwdZArgs& a, int batch, cudaStream_t s);

// grid.x of the adjoint z pass (number of partial sums per batch item)
int adj_z_blocks(int L, long long nl);
cudaError_t launch_adj_z(int L, const AdjZArgs& a, int batch, cudaStream_t s);

// Gridding and element-wise kernels (kernels_misc.cu).
cudaError_t launch_tap_records(const double* k, const int* sample_idx, long long n, const KbParams& kb,
                               TapRecord* out, cudaStream_t s);
cudaError_t launch_interp(const InterpArgs& a, long long max_bin_samples, int nbins, int cc, cudaStream_t s);
cudaError_t launch_spread(const SpreadArgs& a, int ntiles, int nbins, bool kahan, int wpp, cudaStream_t s);
// packed nearest grid point of each tap record
cudaError_t launch_record_nearest(const TapRecord* rec, long long n, unsigned* out, cudaStream_t s);
size_t spread_smem_bytes(int cc, bool kahan);
// one-time kernel attributes (dynamic shared memory limits); call per device
cudaError_t kernels_init();
int spread_max_coils(bool kahan);

// Transposed tap matrix (spread_csr.cu).  csr_build runs the count pass,
// the scan, the fill pass and the per-row ordering; ent must hold
// *entries pairs (csr_count_and_scan returns that number).
cudaError_t csr_count_and_scan(const CsrBuildArgs& a, long long npts, unsigned* ptr, unsigned* scan_tmp,
                               size_t scan_tmp_elems, unsigned long long* entries, cudaStream_t s);
cudaError_t csr_fill_and_order(const CsrBuildArgs& a, long long npts, cudaStream_t s);
size_t csr_scan_tmp_elems(long long n);
cudaError_t launch_spread_csr(const CsrSpreadArgs& a, bool kahan, bool staged, cudaStream_t s);

// samples: reference order [nch][ns] <-> sorted, coil-interleaved [total][nch]
cudaError_t launch_gather_samples(const float2* data, long long ns, const int* sorted, long long total, int nch,
                                  const float* dcf_sorted, float2* yv, cudaStream_t s);
cudaError_t launch_scatter_samples(const float2* yv, const int* sorted, long long total, int nch, long long ns,
                                   float2* data, cudaStream_t s);
cudaError_t launch_zero(void* p, size_t bytes, cudaStream_t s);
cudaError_t launch_coil_combine(const float2* imgs, const float2* smaps, int nch, long long n, float2* b,
                                cudaStream_t s);

// CG
int cg_blocks(long long n, int nbins);
cudaError_t launch_cg_init(const float2* b, float2* r, float2* p, float2* x, long long n, long long bs,
                           double* partials, const CgState* st, int nbins, cudaStream_t s);
cudaError_t launch_cg_arm(CgState* st, const double* partials, int nblk, int nbins, double thresh, int max_iter,
                          cudaStream_t s);
cudaError_t launch_cg_alpha(CgState* st, const double* partials, int nblk, int nbins, const float2* q0,
                            long long bs, cudaStream_t s);
cudaError_t launch_cg_update_xr(float2* x, float2* r, const float2* p, const float2* q, long long n, long long bs,
                                const CgState* st, double* partials, int nbins, cudaStream_t s);
cudaError_t launch_cg_beta(CgState* st, const double* partials, int nblk, int nbins, double* residuals,
                           int res_stride, cudaStream_t s);
cudaError_t launch_cg_update_p(float2* p, const float2* r, long long n, long long bs, const CgState* st, int nbins,
                               cudaStream_t s);
cudaError_t launch_cg_loop_test(CgState* st, int nbins, cudaStream_t s);
// fused solve: r update (after launch_cg_alpha), beta + loop test, the final pending x update
cudaError_t launch_cg_update_r(float2* r, const float2* q, long long n, long long bs, CgState* st,
                               double* partials, int nbins, cudaStream_t s);
cudaError_t launch_cg_beta_test(CgState* st, const double* partials, int nblk, int nbins, double* residuals,
                                int res_stride, cudaStream_t s);
cudaError_t launch_cg_finish_x(float2* x, const float2* p, long long n, long long bs, const CgState* st, int nbins,
                               cudaStream_t s);

// Plain per-bin form (plain.cu): unfused kernels + cuFFT, comparison only.
struct PlainGeom {
    int I[3], G[3], lo[3];
    long long Ni, Ng;
};

struct PlainArgs {
    PlainGeom g;
    int nch;
    const float2* smaps;
    const float* ap[3];
    float scale;
    float thresh;
    cufftHandle plan;
    cudaStream_t s;
    float2* grid;   // [Ng]
    float2* y;      // [max bin samples]
};

cudaError_t plain_apply(const PlainArgs& P, const TapRecord* rec, const float* dcf, long long n, const float2* x,
                        float2* q, long long* launches);
cudaError_t plain_rhs(const PlainArgs& P, const TapRecord* rec, const float* dcf, const int* sorted, long long n,
                      const float2* data, long long ns, float2* b, long long* launches);
cudaError_t plain_dot(const float2* p, const float2* q, long long n, double* partials, int nblocks, cudaStream_t s);

// Loss gradients (grad.cu)
cudaError_t launch_tap_grad_records(const double* k, const int* sample_idx, long long n, const KbParams& kb,
                                    TapRecord* out, cudaStream_t s);
int interp_grad_blocks(long long n);
cudaError_t launch_interp_grad(const InterpGradArgs& a, cudaStream_t s);
cudaError_t launch_check_finite(const double* v, long long n, int* bad, cudaStream_t s);
cudaError_t launch_pair_grad(const PairGradArgs& a, cudaStream_t s);
cudaError_t launch_pm_init(float* w, float2* v, long long n, cudaStream_t s);
cudaError_t launch_pm_update(float* w, float2* v, const float2* u, long long n, cudaStream_t s);

// Coil maps from low-resolution coil images (smaps.cu)
cudaError_t launch_lowpass_weights(const double* k, const int* sorted, long long n, const int* G, double radius,
                                   const float* dcf_sorted, float* w, cudaStream_t s);
// imgs [nch][n] coil images -> maps in place; rss_tmp [n], max_tmp one word
cudaError_t launch_smaps_from_images(float2* imgs, int nch, long long n, float eps, float* rss_tmp,
                                     unsigned* max_tmp, cudaStream_t s);

// Toeplitz embedding of E^H D E (toeplitz.cu, fft_inst.cu).  toeplitz_build
// accumulates one bin's P with cuBLAS over chunks of toeplitz_chunk samples
// (work: work_elems floats; *handle: the caller's cuBLAS handle, created at
// the first call, released with toeplitz_release); returns 0 on success,
// else sets *err.
long long toeplitz_chunk(const int G[3], long long work_elems);
int toeplitz_build(const ToepBuildArgs& a, float* work, long long work_elems, void** handle, cudaStream_t s,
                   std::string* err);
void toeplitz_release(void* handle);
// Spectrum through the point-spread function (toeplitz.cu): FP64 window
// spreading of one bin's density weights onto the fine grid, conversion to
// complex, placement of the deapodised central box into the grid, and the
// real spectrum of the grid's transform.
cudaError_t launch_psf_spread(const PsfSpreadArgs& a, cudaStream_t s);
cudaError_t launch_psf_convert(const double* in, float2* out, long long n, cudaStream_t s);
cudaError_t launch_psf_place(const float2* R, const float* rx, const float* ry, const float* rz, const int G[3],
                             const int I[3], float sgn, float2* grid, cudaStream_t s);
cudaError_t launch_psf_spectrum(const float2* grid, float scale, long long n, float* P, cudaStream_t s);
// grid[item][j] *= P[item / nch][j] over items grids of Ng points
cudaError_t launch_toep_mul(float2* grid, const float* P, long long Ng, int nch, int items, cudaStream_t s);
// Fused x stage in place: forward x transform of the Lin = L/2 stored rows,
// multiply by P (bin of item = item / nsub, bin stride p_bs), adjoint x
// transform, the L/2 kept rows stored over the input.  cudaErrorNotSupported
// when the pass does not apply (line length, pruning, alignment).
cudaError_t launch_toep_x(int L, const StridedPassArgs& a, const float* P, long long p_bs, int nsub, int batch,
                          cudaStream_t s);
// Spreading fused with the adjoint x pass of a grid of L points along x
// (spread_adjx.cuh).  cudaErrorNotSupported when it does not apply (line
// length without narrow tiles, coil count, alignment, shared memory).
cudaError_t launch_spread_adjx(int L, const SpreadAdjxArgs& a, bool kahan, cudaStream_t s);

// File IO (io.cu)
cudaError_t launch_scale_samples(float2* data, const float* d, long long ns, int nch, cudaStream_t s);

// Full-FP64 form (fp64.cu): the precision reference on the GPU.
struct Fp64Args {
    PlainGeom g;
    int nch;
    const float2* smaps;
    const float* ap[3];
    double scale;
    float thresh;
    cufftHandle plan;
    cudaStream_t s;
    double2* grid;
    double2* y;
};
cudaError_t fp64_solve_bin(const Fp64Args& P, const TapRecord* rec, const float* dcf, const int* sorted, long long n,
                           const float2* data, long long ns, double2* x, double2* r, double2* p, double2* q,
                           double* partials, double thresh, int max_iter, double* residuals, int* iters,
                           double2* x_trace, long long trace_stride);
// FP64 loss and gradients of one bin: KB weights and derivatives in double
// from the double coordinates; grad_k (double [ns][3], global index) is
// accumulated over coils; grad_x (double complex [Ni]) written when non-null.
cudaError_t fp64_loss_grad(const Fp64Args& P, const double* k, const int* sorted, long long n, const float* dcf,
                           double kb_w, double kb_b, double thresh, const float2* y, long long ns,
                           const double2* x, double* loss, double2* grad_x, double* grad_k, double* partials,
                           int nblk);

}  // namespace cgs
