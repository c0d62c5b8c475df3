// kernels_misc.cu -- launch wrappers of the gridding, sample-reordering and
// CG kernels.
#include "launch.h"
#include "cg_kernels.cuh"
#include "gridding.cuh"

namespace cgs {

// ---------------------------------------------------------------------------
// sample reordering
// ---------------------------------------------------------------------------

// yv[j][c] = D[j] * data[c][sorted[j]]   (performDensityCorrection, functions.h:319-335)
__global__ void k_gather_samples(const float2* __restrict__ data, long long ns, const int* __restrict__ sorted,
                                 long long total, int nch, const float* __restrict__ dcf, float2* __restrict__ yv)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total * nch) return;
    const long long j = e / nch;
    const int c = (int)(e - j * nch);
    float2 v = data[(long long)c * ns + sorted[j]];
    if (dcf) v = cscale(v, dcf[j]);
    yv[e] = v;
}

// data[c][sorted[j]] = yv[j][c]
__global__ void k_scatter_samples(const float2* __restrict__ yv, const int* __restrict__ sorted, long long total,
                                  int nch, long long ns, float2* __restrict__ data)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total * nch) return;
    const long long j = e / nch;
    const int c = (int)(e - j * nch);
    data[(long long)c * ns + sorted[j]] = yv[e];
}

cudaError_t launch_gather_samples(const float2* data, long long ns, const int* sorted, long long total, int nch,
                                  const float* dcf_sorted, float2* yv, cudaStream_t s)
{
    const long long n = total * nch;
    if (n == 0) return cudaSuccess;
    k_gather_samples<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data, ns, sorted, total, nch, dcf_sorted, yv);
    return cudaGetLastError();
}

cudaError_t launch_scatter_samples(const float2* yv, const int* sorted, long long total, int nch, long long ns,
                                   float2* data, cudaStream_t s)
{
    const long long n = total * nch;
    if (n == 0) return cudaSuccess;
    k_scatter_samples<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(yv, sorted, total, nch, ns, data);
    return cudaGetLastError();
}

cudaError_t launch_zero(void* p, size_t bytes, cudaStream_t s) { return cudaMemsetAsync(p, 0, bytes, s); }

// b = sum_c conj(S_c) img_c, coils summed in order (Reco.cpp:182-190)
__global__ void k_coil_combine(const float2* __restrict__ imgs, const float2* __restrict__ smaps, int nch,
                               long long n, float2* __restrict__ b)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 acc = make_float2(0.f, 0.f);
    for (int c = 0; c < nch; ++c) {
        const float2 s = smaps[(long long)c * n + i], g = imgs[(long long)c * n + i];
        acc.x += s.x * g.x + s.y * g.y;
        acc.y += s.x * g.y - s.y * g.x;
    }
    b[i] = acc;
}

cudaError_t launch_coil_combine(const float2* imgs, const float2* smaps, int nch, long long n, float2* b,
                                cudaStream_t s)
{
    k_coil_combine<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(imgs, smaps, nch, n, b);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// gridding
// ---------------------------------------------------------------------------

cudaError_t launch_tap_records(const double* k, const int* sample_idx, long long n, const KbParams& kb,
                               TapRecord* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_tap_records<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, sample_idx, n, kb, out);
    return cudaGetLastError();
}

// coils per interpolation thread: one of 2, 4, 6, 8 (autotuned per context)
cudaError_t launch_interp(const InterpArgs& a, long long max_bin_samples, int nbins, int cc, cudaStream_t s)
{
    if (max_bin_samples == 0 || nbins == 0) return cudaSuccess;
    const long long nblk = ((max_bin_samples + 127) / 128) * ((a.nch + cc - 1) / cc);
    if (nblk > 0x7fffffffLL) return cudaErrorInvalidValue;
    dim3 grid((unsigned)nblk, 1u, (unsigned)nbins);
    switch (cc) {
    case 1: k_interp<1><<<grid, 128, 0, s>>>(a); break;
    case 2: k_interp<2><<<grid, 128, 0, s>>>(a); break;
    case 4: k_interp<4><<<grid, 128, 0, s>>>(a); break;
    case 6: k_interp<6><<<grid, 128, 0, s>>>(a); break;
    case 8: k_interp<8><<<grid, 128, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

__global__ void k_record_nearest(const TapRecord* __restrict__ rec, long long n, unsigned* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float_as_uint(rec[i].q[3].w);
}

cudaError_t launch_record_nearest(const TapRecord* rec, long long n, unsigned* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_record_nearest<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rec, n, out);
    return cudaGetLastError();
}

// coils per spreading block: staged values use a row of SPREAD_CC_MAX
constexpr int SPREAD_CC_MAX = 12;

size_t spread_smem_bytes(int cc, bool kahan)
{
    return (size_t)(kahan ? 2 : 1) * cc * ACC_PTS * sizeof(float2) + SPREAD_BATCH * sizeof(TapRecord) +
           (size_t)SPREAD_BATCH * SPREAD_VAL_STRIDE * sizeof(float2);
}

int spread_max_coils(bool kahan) { return kahan ? SPREAD_CC_MAX / 2 : SPREAD_CC_MAX; }

// the pipelined variant stages two batches
size_t spread_pipe_smem_bytes(int cc)
{
    return (size_t)cc * ACC_PTS * sizeof(float2) +
           2 * ((size_t)SPREAD_BATCH * sizeof(TapRecord) + (size_t)SPREAD_BATCH * SPREAD_VAL_STRIDE * sizeof(float2));
}

static int sm_count_misc()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int CCW, int WPP>
static cudaError_t spread_pipe_run(const SpreadArgs& a, int ntiles, int nbins, cudaStream_t s)
{
    const size_t smem = spread_pipe_smem_bytes(a.cc);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spread_pipe<CCW, WPP>, 32 * TILE_X * WPP,
                                                                  smem);
    if (e != cudaSuccess) return e;
    const int nchunk = (a.nch + a.cc - 1) / a.cc;
    const long long nitems = (long long)ntiles * nchunk * nbins;
    long long nblk = (long long)sm_count_misc() * (per_sm > 0 ? per_sm : 1);
    if (nblk > nitems) nblk = nitems;
    k_spread_pipe<CCW, WPP><<<(unsigned)nblk, 32 * TILE_X * WPP, smem, s>>>(a, nitems, nchunk);
    return cudaGetLastError();
}

template <int CCW, int WPP>
static cudaError_t spread_attr_one(int smax_plain, int smax_kahan)
{
    cudaError_t e = cudaFuncSetAttribute(k_spread<CCW, WPP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smax_plain);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_spread<CCW, WPP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax_kahan);
    return e;
}

cudaError_t kernels_init()
{
    const int sp = (int)spread_smem_bytes(SPREAD_CC_MAX, false), sk = (int)spread_smem_bytes(SPREAD_CC_MAX / 2, true);
    cudaError_t e = spread_attr_one<4, 1>(sp, sk);
    if (e == cudaSuccess) e = spread_attr_one<8, 1>(sp, sk);
    if (e == cudaSuccess) e = spread_attr_one<12, 1>(sp, sk);
    if (e == cudaSuccess) e = spread_attr_one<2, 2>(sp, sk);
    if (e == cudaSuccess) e = spread_attr_one<4, 2>(sp, sk);
    if (e == cudaSuccess) e = spread_attr_one<6, 2>(sp, sk);
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
        const void* f = i == 0 ? (const void*)k_spread_atomic<4> : i == 1 ? (const void*)k_spread_atomic<8>
                                                                           : (const void*)k_spread_atomic<12>;
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, sp);
    }
    const int spp = (int)spread_pipe_smem_bytes(SPREAD_CC_MAX);
    const void* pipes[6] = {(const void*)k_spread_pipe<4, 1>, (const void*)k_spread_pipe<8, 1>,
                            (const void*)k_spread_pipe<12, 1>, (const void*)k_spread_pipe<2, 2>,
                            (const void*)k_spread_pipe<4, 2>, (const void*)k_spread_pipe<6, 2>};
    for (int i = 0; i < 6 && e == cudaSuccess; ++i)
        e = cudaFuncSetAttribute(pipes[i], cudaFuncAttributeMaxDynamicSharedMemorySize, spp);
    if (e == cudaSuccess) e = fft_init_all();
    return e;
}

template <bool K>
static void spread_launch(const SpreadArgs& a, dim3 grid, size_t smem, int wpp, cudaStream_t s)
{
    if (wpp == 3 && !K) {   // shared-memory atomics (no fixed order)
        if (a.cc <= 4) k_spread_atomic<4><<<grid, SPREAD_ATOMIC_THREADS, smem, s>>>(a);
        else if (a.cc <= 8) k_spread_atomic<8><<<grid, SPREAD_ATOMIC_THREADS, smem, s>>>(a);
        else k_spread_atomic<12><<<grid, SPREAD_ATOMIC_THREADS, smem, s>>>(a);
        return;
    }
    if (wpp == 2) {
        const int ccw = (a.cc + 1) / 2;
        if (ccw <= 2) k_spread<2, 2, K><<<grid, 32 * TILE_X * 2, smem, s>>>(a);
        else if (ccw <= 4) k_spread<4, 2, K><<<grid, 32 * TILE_X * 2, smem, s>>>(a);
        else k_spread<6, 2, K><<<grid, 32 * TILE_X * 2, smem, s>>>(a);
        return;
    }
    if (a.cc <= 4) k_spread<4, 1, K><<<grid, 32 * TILE_X, smem, s>>>(a);
    else if (a.cc <= 8) k_spread<8, 1, K><<<grid, 32 * TILE_X, smem, s>>>(a);
    else k_spread<12, 1, K><<<grid, 32 * TILE_X, smem, s>>>(a);
}

cudaError_t launch_spread(const SpreadArgs& a, int ntiles, int nbins, bool kahan, int wpp, cudaStream_t s)
{
    if (ntiles == 0 || nbins == 0) return cudaSuccess;
    // wpp: 1 or 2 warps per x plane (fixed order), 3 = shared-memory atomics,
    // 4 / 5 = persistent and pipelined with 1 / 2 warps per x plane (fixed order)
    if (a.cc < 1 || a.cc > spread_max_coils(kahan) || wpp < 1 || wpp > 5 || (wpp >= 3 && kahan))
        return cudaErrorInvalidValue;
    if (wpp >= 4 && a.live) {   // the persistent variants store every tile
        SpreadArgs b = a;
        b.live = nullptr;
        b.live_off = nullptr;
        return launch_spread(b, ntiles, nbins, kahan, wpp, s);
    }
    if (wpp == 4) {
        if (a.cc <= 4) return spread_pipe_run<4, 1>(a, ntiles, nbins, s);
        if (a.cc <= 8) return spread_pipe_run<8, 1>(a, ntiles, nbins, s);
        return spread_pipe_run<12, 1>(a, ntiles, nbins, s);
    }
    if (wpp == 5) {
        const int ccw = (a.cc + 1) / 2;
        if (ccw <= 2) return spread_pipe_run<2, 2>(a, ntiles, nbins, s);
        if (ccw <= 4) return spread_pipe_run<4, 2>(a, ntiles, nbins, s);
        return spread_pipe_run<6, 2>(a, ntiles, nbins, s);
    }
    const size_t smem = spread_smem_bytes(a.cc, kahan);
    const int nx = a.live ? a.live_max : ntiles;
    if (nx <= 0) return cudaSuccess;
    dim3 grid((unsigned)nx, (unsigned)((a.nch + a.cc - 1) / a.cc), (unsigned)nbins);
    if (kahan) spread_launch<true>(a, grid, smem, wpp, s);
    else spread_launch<false>(a, grid, smem, wpp, s);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// CG
// ---------------------------------------------------------------------------

// Blocks per bin of the CG vector kernels (grid-stride loops; 4 per SM and
// bin at most).  The bin count is part of the signature so that a
// different split could depend on it; measured on 16 bins, 152 blocks per
// bin ran the fused solve 0.24 ms per iteration slower than 608.
int cg_blocks(long long n, int nbins)
{
    (void)nbins;
    long long b = (n + RED_THREADS - 1) / RED_THREADS;
    if (b > 4 * 152) b = 4 * 152;
    if (b < 1) b = 1;
    return (int)b;
}

cudaError_t launch_cg_init(const float2* b, float2* r, float2* p, float2* x, long long n, long long bs,
                           double* partials, const CgState* st, int nbins, cudaStream_t s)
{
    dim3 grid((unsigned)cg_blocks(n, nbins), (unsigned)nbins);
    k_cg_init<<<grid, RED_THREADS, 0, s>>>(b, r, p, x, n, bs, partials, st);
    return cudaGetLastError();
}

cudaError_t launch_cg_arm(CgState* st, const double* partials, int nblk, int nbins, double thresh, int max_iter,
                          cudaStream_t s)
{
    k_cg_arm<<<nbins, 32, 0, s>>>(st, partials, nblk, nbins, thresh, max_iter);
    return cudaGetLastError();
}

cudaError_t launch_cg_alpha(CgState* st, const double* partials, int nblk, int nbins, const float2* q0,
                            long long bs, cudaStream_t s)
{
    k_cg_alpha<<<nbins, 32, 0, s>>>(st, partials, nblk, nbins, q0, bs);
    return cudaGetLastError();
}

cudaError_t launch_cg_update_xr(float2* x, float2* r, const float2* p, const float2* q, long long n, long long bs,
                                const CgState* st, double* partials, int nbins, cudaStream_t s)
{
    dim3 grid((unsigned)cg_blocks(n, nbins), (unsigned)nbins);
    k_cg_update_xr<<<grid, RED_THREADS, 0, s>>>(x, r, p, q, n, bs, st, partials);
    return cudaGetLastError();
}

cudaError_t launch_cg_beta(CgState* st, const double* partials, int nblk, int nbins, double* residuals,
                           int res_stride, cudaStream_t s)
{
    k_cg_beta<<<nbins, 32, 0, s>>>(st, partials, nblk, nbins, residuals, res_stride);
    return cudaGetLastError();
}

cudaError_t launch_cg_update_p(float2* p, const float2* r, long long n, long long bs, const CgState* st, int nbins,
                               cudaStream_t s)
{
    dim3 grid((unsigned)cg_blocks(n, nbins), (unsigned)nbins);
    k_cg_update_p<<<grid, RED_THREADS, 0, s>>>(p, r, n, bs, st);
    return cudaGetLastError();
}

cudaError_t launch_cg_loop_test(CgState* st, int nbins, cudaStream_t s)
{
    k_cg_loop_test<<<(nbins + 63) / 64, 64, 0, s>>>(st, nbins);
    return cudaGetLastError();
}

cudaError_t launch_cg_update_r(float2* r, const float2* q, long long n, long long bs, CgState* st,
                               double* partials, int nbins, cudaStream_t s)
{
    dim3 grid((unsigned)cg_blocks(n, nbins), (unsigned)nbins);
    k_cg_update_r<<<grid, RED_THREADS, 0, s>>>(r, q, n, bs, st, partials);
    return cudaGetLastError();
}

cudaError_t launch_cg_beta_test(CgState* st, const double* partials, int nblk, int nbins, double* residuals,
                                int res_stride, cudaStream_t s)
{
    k_cg_beta_test<<<nbins, 32, 0, s>>>(st, partials, nblk, nbins, residuals, res_stride);
    return cudaGetLastError();
}

cudaError_t launch_cg_finish_x(float2* x, const float2* p, long long n, long long bs, const CgState* st, int nbins,
                               cudaStream_t s)
{
    dim3 grid((unsigned)cg_blocks(n, nbins), (unsigned)nbins);
    k_cg_finish_x<<<grid, RED_THREADS, 0, s>>>(x, p, n, bs, st);
    return cudaGetLastError();
}

}  // namespace cgs
