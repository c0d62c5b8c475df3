// plain.cu -- the plain per-bin GPU form of the CG-SENSE solve, kept frozen
// as the comparison point of the batched form.
//
// It is the direct GPU transcription of the reference's loop structure
// (Reco.cpp:175-321 with nufftFWD / nufftBWD, Reco.cpp:468-553): one bin
// after the other, one coil after the other, every step its own kernel:
// zero-fill + coil multiply + deapodise, sign alternation, cuFFT 3-D c2c on
// the full grid, sign alternation, per-sample gather, density multiply,
// zero-fill + per-sample scatter with global float atomics, sign
// alternation, inverse cuFFT, sign alternation, crop + deapodise + conj(S)
// accumulate, then the CG updates with a host round trip for the residual
// test every iteration.  No graph, no pruning, no fusion.
#include "cgsense_c.h"
#include "launch.h"
#include "gridding_common.cuh"

#include <cufft.h>

namespace cgs {

// grid = 0 outside the image box, x * S_c * apod inside (Reco.cpp:236-240, 529-535)
__global__ void k_plain_pad(const float2* __restrict__ x, const float2* __restrict__ S, const float* apx,
                            const float* apy, const float* apz, PlainGeom g, float2* __restrict__ grid)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Ng) return;
    const int k = (int)(e % g.G[2]);
    const int j = (int)((e / g.G[2]) % g.G[1]);
    const int i = (int)(e / ((long long)g.G[1] * g.G[2]));
    const int a = i - g.lo[0], b = j - g.lo[1], c = k - g.lo[2];
    float2 v = make_float2(0.f, 0.f);
    if (a >= 0 && a < g.I[0] && b >= 0 && b < g.I[1] && c >= 0 && c < g.I[2]) {
        const long long ii = ((long long)a * g.I[1] + b) * g.I[2] + c;
        v = cscale(cmul(x[ii], S[ii]), apx[a] * apy[b] * apz[c]);
    }
    grid[e] = v;
}

// Fourier.cpp:45-72: negate where i+j+k is even
__global__ void k_plain_sign(float2* grid, PlainGeom g)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Ng) return;
    const int k = (int)(e % g.G[2]);
    const int j = (int)((e / g.G[2]) % g.G[1]);
    const int i = (int)(e / ((long long)g.G[1] * g.G[2]));
    if (((i + j + k) & 1) == 0) grid[e] = cneg(grid[e]);
}

// y[m] = sum_taps w grid[idx] (Reco.cpp:539-550), one coil
__global__ void k_plain_interp(const float2* __restrict__ grid, const TapRecord* __restrict__ rec, long long n,
                               int Gy, int Gz, float thresh, float2* __restrict__ y)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float w[15];
    int nx, ny, nz;
    load_record(rec, i, w, nx, ny, nz);
    float2 acc = make_float2(0.f, 0.f);
    for (int jx = 0; jx < 5; ++jx)
        for (int jy = 0; jy < 5; ++jy)
            for (int jz = 0; jz < 5; ++jz) {
                const float wt = w[jx] * w[5 + jy] * w[10 + jz];
                if (w[jx] != 0.f && w[5 + jy] != 0.f && w[10 + jz] != 0.f && wt > thresh) {
                    const long long idx = ((long long)(nx - 2 + jx) * Gy + (ny - 2 + jy)) * Gz + (nz - 2 + jz);
                    acc.x += grid[idx].x * wt;
                    acc.y += grid[idx].y * wt;
                }
            }
    y[i] = acc;
}

// y[m] *= D[m] (Reco.cpp:243-254)
__global__ void k_plain_dcf(float2* y, const float* d, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = cscale(y[i], d[i]);
}

// grid[idx] += y[m] w with global atomics (Reco.cpp:492-504)
__global__ void k_plain_spread(const float2* __restrict__ y, const TapRecord* __restrict__ rec, long long n, int Gy,
                               int Gz, float thresh, float2* grid)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float w[15];
    int nx, ny, nz;
    load_record(rec, i, w, nx, ny, nz);
    const float2 v = y[i];
    for (int jx = 0; jx < 5; ++jx)
        for (int jy = 0; jy < 5; ++jy)
            for (int jz = 0; jz < 5; ++jz) {
                const float wt = w[jx] * w[5 + jy] * w[10 + jz];
                if (w[jx] != 0.f && w[5 + jy] != 0.f && w[10 + jz] != 0.f && wt > thresh) {
                    const long long idx = ((long long)(nx - 2 + jx) * Gy + (ny - 2 + jy)) * Gz + (nz - 2 + jz);
                    atomicAdd(&grid[idx].x, v.x * wt);
                    atomicAdd(&grid[idx].y, v.y * wt);
                }
            }
}

// q (+)= scale * apod * conj(S_c) * crop(grid) (Reco.cpp:509-517, 257-262)
__global__ void k_plain_crop(const float2* __restrict__ grid, const float2* __restrict__ S, const float* apx,
                             const float* apy, const float* apz, float scale, PlainGeom g, int first,
                             float2* __restrict__ q)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Ni) return;
    const int c = (int)(e % g.I[2]);
    const int b = (int)((e / g.I[2]) % g.I[1]);
    const int a = (int)(e / ((long long)g.I[1] * g.I[2]));
    const long long gi = ((long long)(a + g.lo[0]) * g.G[1] + (b + g.lo[1])) * g.G[2] + (c + g.lo[2]);
    const float2 v = cmulc(cscale(grid[gi], scale * apx[a] * apy[b] * apz[c]), S[e]);
    q[e] = first ? v : cadd(q[e], v);
}

__global__ void k_plain_gather(const float2* __restrict__ data, long long ns, const int* __restrict__ sorted,
                               long long n, const float* dcf, float2* __restrict__ y)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 v = data[sorted[i]];
    if (dcf) v = cscale(v, dcf[i]);
    y[i] = v;
}

static inline unsigned nblk(long long n) { return (unsigned)((n + 255) / 256); }

// <p, q> = sum conj(p) q: per-block FP64 partials (the fused form computes
// this inside its adjoint z pass)
__global__ void __launch_bounds__(256) k_plain_dot(const float2* __restrict__ p, const float2* __restrict__ q,
                                                   long long n, double* partials)
{
    __shared__ double s_re[8], s_im[8];
    double re = 0.0, im = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 a = p[i], b = q[i];
        re += (double)a.x * b.x + (double)a.y * b.y;
        im += (double)a.x * b.y - (double)a.y * b.x;
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_re[threadIdx.x >> 5] = re;
        s_im[threadIdx.x >> 5] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; ++w) {
            a += s_re[w];
            b += s_im[w];
        }
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
    }
}

cudaError_t plain_dot(const float2* p, const float2* q, long long n, double* partials, int nblocks, cudaStream_t s)
{
    k_plain_dot<<<nblocks, 256, 0, s>>>(p, q, n, partials);
    return cudaGetLastError();
}

// q = sum_c conj(S_c) E_c^H D E_c S_c x for one bin (samples rec[0..n))
cudaError_t plain_apply(const PlainArgs& P, const TapRecord* rec, const float* dcf, long long n, const float2* x,
                        float2* q, long long* launches)
{
    const PlainGeom& g = P.g;
    for (int c = 0; c < P.nch; ++c) {
        const float2* S = P.smaps + (long long)c * g.Ni;
        k_plain_pad<<<nblk(g.Ng), 256, 0, P.s>>>(x, S, P.ap[0], P.ap[1], P.ap[2], g, P.grid);
        k_plain_sign<<<nblk(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecC2C(P.plan, (cufftComplex*)P.grid, (cufftComplex*)P.grid, CUFFT_FORWARD) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k_plain_sign<<<nblk(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (n > 0) {
            k_plain_interp<<<nblk(n), 256, 0, P.s>>>(P.grid, rec, n, g.G[1], g.G[2], P.thresh, P.y);
            if (dcf) k_plain_dcf<<<nblk(n), 256, 0, P.s>>>(P.y, dcf, n);
        }
        cudaMemsetAsync(P.grid, 0, g.Ng * sizeof(float2), P.s);
        if (n > 0) k_plain_spread<<<nblk(n), 256, 0, P.s>>>(P.y, rec, n, g.G[1], g.G[2], P.thresh, P.grid);
        k_plain_sign<<<nblk(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecC2C(P.plan, (cufftComplex*)P.grid, (cufftComplex*)P.grid, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k_plain_sign<<<nblk(g.Ng), 256, 0, P.s>>>(P.grid, g);
        k_plain_crop<<<nblk(g.Ni), 256, 0, P.s>>>(P.grid, S, P.ap[0], P.ap[1], P.ap[2], P.scale, g, c == 0, q);
        *launches += 9 + (n > 0 ? (dcf ? 3 : 2) : 0);
    }
    return cudaGetLastError();
}

// right-hand side b = sum_c conj(S_c) E_c^H (D y_c) for one bin
cudaError_t plain_rhs(const PlainArgs& P, const TapRecord* rec, const float* dcf, const int* sorted, long long n,
                      const float2* data, long long ns, float2* b, long long* launches)
{
    const PlainGeom& g = P.g;
    for (int c = 0; c < P.nch; ++c) {
        const float2* S = P.smaps + (long long)c * g.Ni;
        cudaMemsetAsync(P.grid, 0, g.Ng * sizeof(float2), P.s);
        if (n > 0) {
            k_plain_gather<<<nblk(n), 256, 0, P.s>>>(data + (long long)c * ns, ns, sorted, n, dcf, P.y);
            k_plain_spread<<<nblk(n), 256, 0, P.s>>>(P.y, rec, n, g.G[1], g.G[2], P.thresh, P.grid);
        }
        k_plain_sign<<<nblk(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecC2C(P.plan, (cufftComplex*)P.grid, (cufftComplex*)P.grid, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k_plain_sign<<<nblk(g.Ng), 256, 0, P.s>>>(P.grid, g);
        k_plain_crop<<<nblk(g.Ni), 256, 0, P.s>>>(P.grid, S, P.ap[0], P.ap[1], P.ap[2], P.scale, g, c == 0, b);
        *launches += 5 + (n > 0 ? 2 : 0);
    }
    return cudaGetLastError();
}

}  // namespace cgs
