// cg_kernels.cuh -- vector updates and FP64 reductions of the CG-SENSE loop
// (Reco.cpp:175-321), batched over respiratory bins (blockIdx.y).
//
// All control stays on the device so that a whole solve can be captured in
// one CUDA graph: every kernel of an iteration first reads its bin's
// CgState and returns at once when the bin has stopped (residual below the
// threshold or the iteration cap reached), which reproduces the reference's
// `while (currentResidual > cgThreshold)` loop with its 16-iteration cap.
// Dot products follow conjScalarProduct (Reco.cpp:131-143): the products of
// an element are formed in FP32 and accumulated in FP64 -- here a thread
// adds CG_FCHUNK elements' FP32 terms before each FP64 addition, which keeps
// the FP64 pipe (a small fraction of GB300's FP32 rate) off the critical
// path.  Per-block partial sums are then added in a fixed order in one
// thread, so results do not depend on scheduling.  The vector updates use
// the FP64 step sizes rounded to FP32 (relative change ~1e-7 per update).
#pragma once
#include "cgs_common.cuh"
#include "cgs_types.h"

namespace cgs {

constexpr int CG_FCHUNK = 4;   // elements per FP32 partial of a dot product

// |v|^2 with a fixed rounding (one fused multiply-add), the same in every kernel
CGS_D float cg_abs2(float2 v) { return __fmaf_rn(v.x, v.x, __fmul_rn(v.y, v.y)); }

CGS_D void block_reduce2(double& a, double& b, double* s_red /* [2][RED_THREADS/32] */)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_red[w] = a;
        s_red[RED_THREADS / 32 + w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ra = 0.0, rb = 0.0;
        for (int i = 0; i < RED_THREADS / 32; ++i) {
            ra += s_red[i];
            rb += s_red[RED_THREADS / 32 + i];
        }
        a = ra;
        b = rb;
    }
}

// r = b, p = b, x = 0; partial sums of <b, b>.  grid: (nblk, nbins)
__global__ void __launch_bounds__(RED_THREADS)
k_cg_init(const float2* __restrict__ b, float2* r, float2* p, float2* x, long long n, long long bs,
          double* partials, const CgState* st)
{
    __shared__ double s_red[2 * RED_THREADS / 32];
    const int bin = blockIdx.y;
    const long long off = (long long)bin * bs;
    double acc = 0.0, dummy = 0.0;
    float fa = 0.f;
    int cnt = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = b[off + i];
        r[off + i] = v;
        p[off + i] = v;
        x[off + i] = make_float2(0.f, 0.f);
        fa = __fadd_rn(fa, cg_abs2(v));
        if (++cnt == CG_FCHUNK) {
            acc += (double)fa;
            fa = 0.f;
            cnt = 0;
        }
    }
    acc += (double)fa;
    block_reduce2(acc, dummy, s_red);
    if (threadIdx.x == 0) {
        double* o = partials + 2 * ((long long)bin * gridDim.x + blockIdx.x);
        o[0] = acc;
        o[1] = 0.0;
    }
}

// alpha = rr / pq (complexDivision, Reco.cpp:145-151), every product and
// sum rounded on its own, so that the separate alpha kernel and the fused
// residual update compute the same bits.
CGS_D void cg_alpha(const double* rr, double pr, double pim, double* alpha)
{
    const double d = __dadd_rn(__dmul_rn(pr, pr), __dmul_rn(pim, pim));
    alpha[0] = __ddiv_rn(__dadd_rn(__dmul_rn(rr[0], pr), __dmul_rn(rr[1], pim)), d);
    alpha[1] = __ddiv_rn(__dsub_rn(__dmul_rn(rr[1], pr), __dmul_rn(rr[0], pim)), d);
}

// Sum of a bin's nblk (re, im) partials by one warp: lane l adds the
// partials l, l + 32, ... in order, then a butterfly of shuffles (a fixed
// order; every lane ends with the same sums).
CGS_D void warp_partials(const double* partials, long long base, int nblk, double& re, double& im)
{
    const int lane = threadIdx.x & 31;
    double a = 0.0, b = 0.0;
    for (int i = lane; i < nblk; i += 32) {
        a += partials[2 * (base + i)];
        b += partials[2 * (base + i) + 1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    re = a;
    im = b;
}

// Sum the partials of <b, b> and arm the state: rr, active.  One warp per bin.
__global__ void k_cg_arm(CgState* st, const double* partials, int nblk, int nbins, double thresh, int max_iter)
{
    const int bin = blockIdx.x;
    if (bin >= nbins) return;
    double s, unused;
    warp_partials(partials, (long long)bin * nblk, nblk, s, unused);
    if (threadIdx.x != 0) return;
    CgState& S = st[bin];
    S.rr[0] = s;
    S.rr[1] = 0.0;
    S.pq[0] = S.pq[1] = 0.0;
    S.alpha[0] = S.alpha[1] = 0.0;
    S.beta[0] = S.beta[1] = 0.0;
    S.res = 1000.0;          // Reco.cpp:229
    S.thresh = thresh;
    S.iter = 0;
    S.max_iter = max_iter;
    S.error = 0;
    S.xpend = 0;
    // A zero right-hand side (empty bin, all-zero data) would make the
    // reference divide 0/0 and return NaN; here the solve stops at x = 0.
    S.active = (S.res > thresh && max_iter > 0 && s > 0.0) ? 1 : 0;
}

// alpha = rr / pq from the <p, q> partials (complexDivision, Reco.cpp:145-151).
__global__ void k_cg_alpha(CgState* st, const double* partials, int nblk, int nbins, const float2* q0,
                           long long bs)
{
    const int bin = blockIdx.x;   // one warp per bin
    if (bin >= nbins) return;
    CgState& S = st[bin];
    if (!S.active) return;
    double pr, pim;
    warp_partials(partials, (long long)bin * nblk, nblk, pr, pim);
    if (threadIdx.x != 0) return;
    S.pq[0] = pr;
    S.pq[1] = pim;
    const float2 qv = q0[(long long)bin * bs];
    if (!isfinite(qv.x) || !isfinite(qv.y) || !isfinite(pr) || !isfinite(pim)) {
        S.error = 1;
        S.active = 0;
        S.xpend = 0;   // fused solve: x already holds the last applied update
        return;
    }
    cg_alpha(S.rr, pr, pim, S.alpha);
}

// x += alpha p ; r -= alpha q ; partial sums of |r|^2  (Reco.cpp:285-298)
__global__ void __launch_bounds__(RED_THREADS)
k_cg_update_xr(float2* x, float2* r, const float2* __restrict__ p, const float2* __restrict__ q, long long n,
               long long bs, const CgState* st, double* partials)
{
    __shared__ double s_red[2 * RED_THREADS / 32];
    const int bin = blockIdx.y;
    const CgState& S = st[bin];
    if (!S.active) return;
    const float ar = (float)S.alpha[0], ai = (float)S.alpha[1];
    const long long off = (long long)bin * bs;
    double acc = 0.0, dummy = 0.0;
    float fa = 0.f;
    int cnt = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 pv = p[off + i], qv = q[off + i];
        float2 xv = x[off + i], rv = r[off + i];
        xv = cg_axpy(xv, ar, ai, pv);
        rv = cg_axmy(rv, ar, ai, qv);
        x[off + i] = xv;
        r[off + i] = rv;
        fa = __fadd_rn(fa, cg_abs2(rv));
        if (++cnt == CG_FCHUNK) {
            acc += (double)fa;
            fa = 0.f;
            cnt = 0;
        }
    }
    acc += (double)fa;
    block_reduce2(acc, dummy, s_red);
    if (threadIdx.x == 0) {
        double* o = partials + 2 * ((long long)bin * gridDim.x + blockIdx.x);
        o[0] = acc;
        o[1] = 0.0;
    }
}

// residual, beta = rr_new / rr_old (rr_new real), iteration count
// (Reco.cpp:292-309); residuals: the bin's row of the residual record
CGS_D void cg_residual_beta(CgState& S, double s, double* residuals)
{
    S.res = sqrt(s);
    if (residuals) residuals[S.iter] = S.res;
    const double d = __dadd_rn(__dmul_rn(S.rr[0], S.rr[0]), __dmul_rn(S.rr[1], S.rr[1]));
    S.beta[0] = __ddiv_rn(__dmul_rn(s, S.rr[0]), d);
    S.beta[1] = __ddiv_rn(__dmul_rn(-s, S.rr[1]), d);
    S.rr[0] = s;
    S.rr[1] = 0.0;
    S.iter += 1;
}

// residual, beta = rr_new / rr, loop control (Reco.cpp:292-309)
__global__ void k_cg_beta(CgState* st, const double* partials, int nblk, int nbins, double* residuals,
                          int res_stride)
{
    const int bin = blockIdx.x;   // one warp per bin
    if (bin >= nbins) return;
    CgState& S = st[bin];
    if (!S.active) return;
    double s, unused;
    warp_partials(partials, (long long)bin * nblk, nblk, s, unused);
    if (threadIdx.x != 0) return;
    cg_residual_beta(S, s, residuals ? residuals + (long long)bin * res_stride : nullptr);
    // p is updated in this same iteration before the loop test
}

// p = r + beta p ; then the loop test  (Reco.cpp:306-309)
__global__ void k_cg_update_p(float2* p, const float2* __restrict__ r, long long n, long long bs, const CgState* st)
{
    const int bin = blockIdx.y;
    const CgState& S = st[bin];
    if (!S.active) return;
    const float br = (float)S.beta[0], bi = (float)S.beta[1];
    const long long off = (long long)bin * bs;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        p[off + i] = cg_axpy(r[off + i], br, bi, p[off + i]);
    }
}

__global__ void k_cg_loop_test(CgState* st, int nbins)
{
    const int bin = blockIdx.x * blockDim.x + threadIdx.x;
    if (bin >= nbins) return;
    CgState& S = st[bin];
    if (!S.active) return;
    S.active = (S.res > S.thresh && S.iter < S.max_iter) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Fused solve.  Per iteration: the forward z pass forms p = r + beta p and
// x = x + alpha p of the previous iteration while it reads p (FwdZArgs::cg);
// the adjoint z pass sums <p, q>; k_cg_alpha computes alpha from those
// partial sums; k_cg_update_r updates r with the partial sums of <r, r>;
// k_cg_beta_test computes the residual, beta and the loop test.  After the loop k_cg_finish_x applies the last
// pending x update.  Same arithmetic as the separate kernels above, hence
// the same bits; three graph nodes per iteration besides the operator instead
// of five, and x and p are read and written in the pass that reads p anyway.
// ---------------------------------------------------------------------------

// r -= alpha q with the alpha that k_cg_alpha recorded; partial sums of
// |r|^2.  grid: (nblk, nbins).  Block 0 of a bin marks the x / p updates
// pending (k_cg_alpha has already stopped a bin with non-finite values).
__global__ void __launch_bounds__(RED_THREADS)
k_cg_update_r(float2* r, const float2* __restrict__ q, long long n, long long bs, CgState* st, double* partials)
{
    __shared__ double s_red[2 * RED_THREADS / 32];
    const int bin = blockIdx.y;
    CgState& S = st[bin];
    if (!S.active) return;   // not written by this kernel
    if (blockIdx.x == 0 && threadIdx.x == 0) S.xpend = 1;
    const float ar = (float)S.alpha[0], ai = (float)S.alpha[1];
    const long long off = (long long)bin * bs;
    double acc = 0.0, dummy = 0.0;
    float fa = 0.f;
    int cnt = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // CG_FCHUNK consecutive elements of the thread at a time: their loads in
    // flight together; the same elements, order and partial sums as the
    // one-at-a-time loop below (and k_cg_update_xr)
    for (; i + (CG_FCHUNK - 1) * stride < n; i += CG_FCHUNK * stride) {
        float2 rv[CG_FCHUNK], qv[CG_FCHUNK];
#pragma unroll
        for (int j = 0; j < CG_FCHUNK; ++j) {
            rv[j] = r[off + i + j * stride];
            qv[j] = q[off + i + j * stride];
        }
#pragma unroll
        for (int j = 0; j < CG_FCHUNK; ++j) {
            rv[j] = cg_axmy(rv[j], ar, ai, qv[j]);
            r[off + i + j * stride] = rv[j];
            fa = __fadd_rn(fa, cg_abs2(rv[j]));
        }
        acc += (double)fa;
        fa = 0.f;
    }
    for (; i < n; i += stride) {
        float2 rv = r[off + i];
        rv = cg_axmy(rv, ar, ai, q[off + i]);
        r[off + i] = rv;
        fa = __fadd_rn(fa, cg_abs2(rv));
        if (++cnt == CG_FCHUNK) {
            acc += (double)fa;
            fa = 0.f;
            cnt = 0;
        }
    }
    acc += (double)fa;
    block_reduce2(acc, dummy, s_red);
    if (threadIdx.x == 0) {
        double* o = partials + 2 * ((long long)bin * gridDim.x + blockIdx.x);
        o[0] = acc;
        o[1] = 0.0;
    }
}

// residual, beta and the loop test in one step.  One warp per bin.
__global__ void k_cg_beta_test(CgState* st, const double* partials, int nblk, int nbins, double* residuals,
                               int res_stride)
{
    const int bin = blockIdx.x;
    if (bin >= nbins) return;
    CgState& S = st[bin];
    if (!S.active) return;
    double s, unused;
    warp_partials(partials, (long long)bin * nblk, nblk, s, unused);
    if (threadIdx.x != 0) return;
    cg_residual_beta(S, s, residuals ? residuals + (long long)bin * res_stride : nullptr);
    S.active = (S.res > S.thresh && S.iter < S.max_iter) ? 1 : 0;
}

// x += alpha p for the bins whose last update is still pending.  grid: (nblk, nbins)
__global__ void k_cg_finish_x(float2* x, const float2* __restrict__ p, long long n, long long bs, const CgState* st)
{
    const int bin = blockIdx.y;
    const CgState& S = st[bin];
    if (!S.xpend) return;
    const float ar = (float)S.alpha[0], ai = (float)S.alpha[1];
    const long long off = (long long)bin * bs;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[off + i] = cg_axpy(x[off + i], ar, ai, p[off + i]);
}

}  // namespace cgs
