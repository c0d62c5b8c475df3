// fp64.cu -- the full-FP64 GPU form of the CG-SENSE solve: the precision
// reference that the FP32 (complex64) path is measured against.
//
// Same operator and loop as the plain per-bin form (plain.cu), every value in
// double precision: double-complex images, grids and samples, cuFFT Z2Z
// transforms, double atomics in the spreading, double CG vectors and scalars.
// The KB tap weights are the float weights of the tap records, as in the
// reference, where ConvKernel::weights is float (Reco.h:58).
#include "cgsense_c.h"
#include "launch.h"
#include "gridding_common.cuh"

#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace cgs {

namespace {

CGS_HD double2 zmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
CGS_HD double2 zmulc(double2 a, double2 b) { return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }

inline unsigned nb64(long long n) { return (unsigned)((n + 255) / 256); }

__global__ void k64_pad(const double2* __restrict__ x, const float2* __restrict__ S, const float* apx,
                        const float* apy, const float* apz, PlainGeom g, double2* __restrict__ grid)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Ng) return;
    const int k = (int)(e % g.G[2]);
    const int j = (int)((e / g.G[2]) % g.G[1]);
    const int i = (int)(e / ((long long)g.G[1] * g.G[2]));
    const int a = i - g.lo[0], b = j - g.lo[1], c = k - g.lo[2];
    double2 v = make_double2(0.0, 0.0);
    if (a >= 0 && a < g.I[0] && b >= 0 && b < g.I[1] && c >= 0 && c < g.I[2]) {
        const long long ii = ((long long)a * g.I[1] + b) * g.I[2] + c;
        const double ap = (double)apx[a] * (double)apy[b] * (double)apz[c];
        const double2 s = make_double2(S[ii].x, S[ii].y);
        const double2 t = zmul(x[ii], s);
        v = make_double2(t.x * ap, t.y * ap);
    }
    grid[e] = v;
}

__global__ void k64_sign(double2* grid, PlainGeom g)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Ng) return;
    const int k = (int)(e % g.G[2]);
    const int j = (int)((e / g.G[2]) % g.G[1]);
    const int i = (int)(e / ((long long)g.G[1] * g.G[2]));
    if (((i + j + k) & 1) == 0) grid[e] = make_double2(-grid[e].x, -grid[e].y);
}

__global__ void k64_interp(const double2* __restrict__ grid, const TapRecord* __restrict__ rec, const float* dcf,
                           long long n, int Gy, int Gz, float thresh, double2* __restrict__ y)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float w[15];
    int nx, ny, nz;
    load_record(rec, i, w, nx, ny, nz);
    double2 acc = make_double2(0.0, 0.0);
    for (int jx = 0; jx < 5; ++jx)
        for (int jy = 0; jy < 5; ++jy)
            for (int jz = 0; jz < 5; ++jz) {
                const float wt = w[jx] * w[5 + jy] * w[10 + jz];
                if (w[jx] != 0.f && w[5 + jy] != 0.f && w[10 + jz] != 0.f && wt > thresh) {
                    const long long idx = ((long long)(nx - 2 + jx) * Gy + (ny - 2 + jy)) * Gz + (nz - 2 + jz);
                    acc.x += grid[idx].x * (double)wt;
                    acc.y += grid[idx].y * (double)wt;
                }
            }
    const double d = dcf ? (double)dcf[i] : 1.0;
    y[i] = make_double2(acc.x * d, acc.y * d);
}

__global__ void k64_spread(const double2* __restrict__ y, const TapRecord* __restrict__ rec, long long n, int Gy,
                           int Gz, float thresh, double2* grid)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float w[15];
    int nx, ny, nz;
    load_record(rec, i, w, nx, ny, nz);
    const double2 v = y[i];
    for (int jx = 0; jx < 5; ++jx)
        for (int jy = 0; jy < 5; ++jy)
            for (int jz = 0; jz < 5; ++jz) {
                const float wt = w[jx] * w[5 + jy] * w[10 + jz];
                if (w[jx] != 0.f && w[5 + jy] != 0.f && w[10 + jz] != 0.f && wt > thresh) {
                    const long long idx = ((long long)(nx - 2 + jx) * Gy + (ny - 2 + jy)) * Gz + (nz - 2 + jz);
                    atomicAdd(&grid[idx].x, v.x * (double)wt);
                    atomicAdd(&grid[idx].y, v.y * (double)wt);
                }
            }
}

__global__ void k64_crop(const double2* __restrict__ grid, const float2* __restrict__ S, const float* apx,
                         const float* apy, const float* apz, double scale, PlainGeom g, int first,
                         double2* __restrict__ q)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.Ni) return;
    const int c = (int)(e % g.I[2]);
    const int b = (int)((e / g.I[2]) % g.I[1]);
    const int a = (int)(e / ((long long)g.I[1] * g.I[2]));
    const long long gi = ((long long)(a + g.lo[0]) * g.G[1] + (b + g.lo[1])) * g.G[2] + (c + g.lo[2]);
    const double f = scale * (double)apx[a] * (double)apy[b] * (double)apz[c];
    const double2 v0 = make_double2(grid[gi].x * f, grid[gi].y * f);
    const double2 v = zmulc(v0, make_double2(S[e].x, S[e].y));
    q[e] = first ? v : make_double2(q[e].x + v.x, q[e].y + v.y);
}

__global__ void k64_gather(const float2* __restrict__ data, const int* __restrict__ sorted, long long n,
                           const float* dcf, double2* __restrict__ y)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 v = data[sorted[i]];
    const double d = dcf ? (double)dcf[i] : 1.0;
    y[i] = make_double2(v.x * d, v.y * d);
}

// sums of conj(a) b over blocks -> partials[blockIdx][2]
__global__ void __launch_bounds__(256) k64_dot(const double2* __restrict__ a, const double2* __restrict__ b,
                                               long long n, double* partials)
{
    __shared__ double s_re[8], s_im[8];
    double re = 0.0, im = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        re += a[i].x * b[i].x + a[i].y * b[i].y;
        im += a[i].x * b[i].y - a[i].y * b[i].x;
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
        double x = 0.0, y = 0.0;
        for (int w = 0; w < 8; ++w) {
            x += s_re[w];
            y += s_im[w];
        }
        partials[2 * blockIdx.x] = x;
        partials[2 * blockIdx.x + 1] = y;
    }
}

// v1 += s * v2 (complex s)
__global__ void k64_axpy(double2* v1, const double2* __restrict__ v2, double sr, double si, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 b = v2[i];
    v1[i] = make_double2(v1[i].x + sr * b.x - si * b.y, v1[i].y + sr * b.y + si * b.x);
}

// p = r + s p
__global__ void k64_xpay(double2* p, const double2* __restrict__ r, double sr, double si, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 a = p[i];
    p[i] = make_double2(r[i].x + sr * a.x - si * a.y, r[i].y + sr * a.y + si * a.x);
}


// KB factor and its derivative in double from a double coordinate (the
// extension used by the gradient reference; cf. Reco.h:218-242).
__device__ void kb64(double ka, int gi, double dk, double w, double b, double& f, double& df)
{
    const double d = ka - (double)gi * dk;
    if (fabs(d) > 0.5 * w * dk) {
        f = df = 0.0;
        return;
    }
    const double t = 2.0 * d / (w * dk);
    const double s2 = 1.0 - t * t;
    const double s = s2 > 0.0 ? sqrt(s2) : 0.0;
    const double C = 100.0 * w * dk;
    f = cyl_bessel_i0(b * s) / C;
    const double i1s = s > 1e-12 ? cyl_bessel_i1(b * s) / s : 0.5 * b;
    df = -i1s * b * t * (2.0 / (w * dk)) / C;
}

struct Taps64 {
    double f[3][5], df[3][5];
    int nr[3];
};

__device__ void taps64(const double* kk, const PlainGeom& g, double w, double b, Taps64& t)
{
    for (int a = 0; a < 3; ++a) {
        const int N = g.G[a];
        const double dk = 1.0 / (double)(N - 1);
        int nr = (int)__dadd_rn(__dmul_rn((double)(N - 1), kk[a]), 0.5);
        nr = nr < 0 ? 0 : (nr > N - 1 ? N - 1 : nr);
        t.nr[a] = nr;
        for (int j = 0; j < 5; ++j) {
            const int gi = nr - 2 + j;
            if (gi < 0 || gi > N - 1) {
                t.f[a][j] = t.df[a][j] = 0.0;
                continue;
            }
            kb64(kk[a], gi, dk, w, b, t.f[a][j], t.df[a][j]);
        }
    }
}

// One coil: loss partials, grad_k += per-coil term, rv = D r (sorted order).
__global__ void __launch_bounds__(256) k64_loss_grad(const double2* __restrict__ grid, const double* __restrict__ k,
                                                     const int* __restrict__ sorted, long long n, PlainGeom g,
                                                     double w, double b, double thresh,
                                                     const float2* __restrict__ yc, const float* dcf,
                                                     double* grad_k, double2* rv, double* partials)
{
    __shared__ double s_red[8];
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double loss = 0.0;
    if (j < n) {
        const long long gi = sorted[j];
        Taps64 t;
        taps64(k + 3 * gi, g, w, b, t);
        double yr = 0, yi = 0, dr[3] = {0, 0, 0}, di[3] = {0, 0, 0};
        for (int jx = 0; jx < 5; ++jx)
            for (int jy = 0; jy < 5; ++jy)
                for (int jz = 0; jz < 5; ++jz) {
                    const double wt = t.f[0][jx] * t.f[1][jy] * t.f[2][jz];
                    if (!(wt > thresh)) continue;
                    const long long idx =
                        ((long long)(t.nr[0] - 2 + jx) * g.G[1] + (t.nr[1] - 2 + jy)) * g.G[2] + (t.nr[2] - 2 + jz);
                    const double2 v = grid[idx];
                    yr += wt * v.x;
                    yi += wt * v.y;
                    const double e[3] = {t.df[0][jx] * t.f[1][jy] * t.f[2][jz], t.f[0][jx] * t.df[1][jy] * t.f[2][jz],
                                         t.f[0][jx] * t.f[1][jy] * t.df[2][jz]};
                    for (int a = 0; a < 3; ++a) {
                        dr[a] += e[a] * v.x;
                        di[a] += e[a] * v.y;
                    }
                }
        const double D = dcf ? (double)dcf[j] : 1.0;
        const double rr = yr - (double)yc[gi].x, ri = yi - (double)yc[gi].y;
        loss = 0.5 * D * (rr * rr + ri * ri);
        if (grad_k)
            for (int a = 0; a < 3; ++a) grad_k[3 * gi + a] += D * (rr * dr[a] + ri * di[a]);
        if (rv) rv[j] = make_double2(D * rr, D * ri);
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int i = 0; i < 8; ++i) sum += s_red[i];
        partials[blockIdx.x] = sum;
    }
}

// transpose of the interpolation with the double taps (double atomics)
__global__ void k64_spread_taps(const double2* __restrict__ v, const double* __restrict__ k,
                                const int* __restrict__ sorted, long long n, PlainGeom g, double w, double b,
                                double thresh, double2* grid)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    Taps64 t;
    taps64(k + 3 * (long long)sorted[j], g, w, b, t);
    const double2 d = v[j];
    for (int jx = 0; jx < 5; ++jx)
        for (int jy = 0; jy < 5; ++jy)
            for (int jz = 0; jz < 5; ++jz) {
                const double wt = t.f[0][jx] * t.f[1][jy] * t.f[2][jz];
                if (!(wt > thresh)) continue;
                const long long idx =
                    ((long long)(t.nr[0] - 2 + jx) * g.G[1] + (t.nr[1] - 2 + jy)) * g.G[2] + (t.nr[2] - 2 + jz);
                atomicAdd(&grid[idx].x, wt * d.x);
                atomicAdd(&grid[idx].y, wt * d.y);
            }
}

}  // namespace


static cudaError_t fp64_apply(const Fp64Args& P, const TapRecord* rec, const float* dcf, long long n,
                              const double2* x, double2* q)
{
    const PlainGeom& g = P.g;
    for (int c = 0; c < P.nch; ++c) {
        const float2* S = P.smaps + (long long)c * g.Ni;
        k64_pad<<<nb64(g.Ng), 256, 0, P.s>>>(x, S, P.ap[0], P.ap[1], P.ap[2], g, P.grid);
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecZ2Z(P.plan, (cufftDoubleComplex*)P.grid, (cufftDoubleComplex*)P.grid, CUFFT_FORWARD) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (n > 0) k64_interp<<<nb64(n), 256, 0, P.s>>>(P.grid, rec, dcf, n, g.G[1], g.G[2], P.thresh, P.y);
        cudaMemsetAsync(P.grid, 0, g.Ng * sizeof(double2), P.s);
        if (n > 0) k64_spread<<<nb64(n), 256, 0, P.s>>>(P.y, rec, n, g.G[1], g.G[2], P.thresh, P.grid);
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecZ2Z(P.plan, (cufftDoubleComplex*)P.grid, (cufftDoubleComplex*)P.grid, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        k64_crop<<<nb64(g.Ni), 256, 0, P.s>>>(P.grid, S, P.ap[0], P.ap[1], P.ap[2], P.scale, g, c == 0, q);
    }
    return cudaGetLastError();
}

static cudaError_t fp64_rhs(const Fp64Args& P, const TapRecord* rec, const float* dcf, const int* sorted, long long n,
                            const float2* data, long long ns, double2* b)
{
    const PlainGeom& g = P.g;
    for (int c = 0; c < P.nch; ++c) {
        const float2* S = P.smaps + (long long)c * g.Ni;
        cudaMemsetAsync(P.grid, 0, g.Ng * sizeof(double2), P.s);
        if (n > 0) {
            k64_gather<<<nb64(n), 256, 0, P.s>>>(data + (long long)c * ns, sorted, n, dcf, P.y);
            k64_spread<<<nb64(n), 256, 0, P.s>>>(P.y, rec, n, g.G[1], g.G[2], P.thresh, P.grid);
        }
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecZ2Z(P.plan, (cufftDoubleComplex*)P.grid, (cufftDoubleComplex*)P.grid, CUFFT_INVERSE) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        k64_crop<<<nb64(g.Ni), 256, 0, P.s>>>(P.grid, S, P.ap[0], P.ap[1], P.ap[2], P.scale, g, c == 0, b);
    }
    return cudaGetLastError();
}

static cudaError_t fp64_dot(const double2* a, const double2* b, long long n, double* partials, int nblk,
                            cudaStream_t s, double* out)
{
    k64_dot<<<nblk, 256, 0, s>>>(a, b, n, partials);
    std::vector<double> h(2 * (size_t)nblk);
    cudaError_t e = cudaMemcpyAsync(h.data(), partials, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    out[0] = out[1] = 0.0;
    for (int i = 0; i < nblk; ++i) {
        out[0] += h[2 * i];
        out[1] += h[2 * i + 1];
    }
    return e;
}

// The whole solve for one bin, host-driven (the reference's loop,
// Reco.cpp:175-321), everything in FP64.  x_trace (optional) receives x
// after every iteration.
cudaError_t fp64_solve_bin(const Fp64Args& P, const TapRecord* rec, const float* dcf, const int* sorted, long long n,
                           const float2* data, long long ns, double2* x, double2* r, double2* p, double2* q,
                           double* partials, double thresh, int max_iter, double* residuals, int* iters,
                           double2* x_trace, long long trace_stride)
{
    const long long Ni = P.g.Ni;
    const int nblk = (int)std::min<long long>((Ni + 255) / 256, 1024);
    cudaError_t e = fp64_rhs(P, rec, dcf, sorted, n, data, ns, r);
    if (e != cudaSuccess) return e;
    cudaMemcpyAsync(p, r, Ni * sizeof(double2), cudaMemcpyDeviceToDevice, P.s);
    cudaMemsetAsync(x, 0, Ni * sizeof(double2), P.s);
    double rr[2];
    e = fp64_dot(r, r, Ni, partials, nblk, P.s, rr);
    if (e != cudaSuccess) return e;
    int it = 0;
    double current = 1000.0;
    if (!(rr[0] > 0.0)) current = 0.0;   // zero right-hand side: x = 0
    while (current > thresh && it < max_iter) {
        e = fp64_apply(P, rec, dcf, n, p, q);
        if (e != cudaSuccess) return e;
        double pq[2];
        e = fp64_dot(p, q, Ni, partials, nblk, P.s, pq);
        if (e != cudaSuccess) return e;
        const double d = pq[0] * pq[0] + pq[1] * pq[1];
        const double ar = (rr[0] * pq[0] + rr[1] * pq[1]) / d, ai = (rr[1] * pq[0] - rr[0] * pq[1]) / d;
        k64_axpy<<<nb64(Ni), 256, 0, P.s>>>(x, p, ar, ai, Ni);
        k64_axpy<<<nb64(Ni), 256, 0, P.s>>>(r, q, -ar, -ai, Ni);
        double rn[2];
        e = fp64_dot(r, r, Ni, partials, nblk, P.s, rn);
        if (e != cudaSuccess) return e;
        current = std::sqrt(rn[0]);
        if (residuals) residuals[it] = current;
        const double dd = rr[0] * rr[0] + rr[1] * rr[1];
        const double br = (rn[0] * rr[0]) / dd, bi = (-rn[0] * rr[1]) / dd;
        k64_xpay<<<nb64(Ni), 256, 0, P.s>>>(p, r, br, bi, Ni);
        rr[0] = rn[0];
        rr[1] = 0.0;
        if (x_trace) cudaMemcpyAsync(x_trace + (long long)it * trace_stride, x, Ni * sizeof(double2),
                                     cudaMemcpyDeviceToDevice, P.s);
        ++it;
    }
    *iters = it;
    return cudaGetLastError();
}

cudaError_t fp64_loss_grad(const Fp64Args& P, const double* k, const int* sorted, long long n, const float* dcf,
                           double kb_w, double kb_b, double thresh, const float2* y, long long ns,
                           const double2* x, double* loss, double2* grad_x, double* grad_k, double* partials,
                           int /*nblk*/)
{
    const PlainGeom& g = P.g;
    const unsigned nblk = nb64(std::max<long long>(n, 1));
    std::vector<double> h(nblk);
    double total = 0.0;
    cudaError_t e = cudaSuccess;
    if (grad_k) e = cudaMemsetAsync(grad_k, 0, (size_t)ns * 3 * sizeof(double), P.s);
    for (int c = 0; c < P.nch && e == cudaSuccess; ++c) {
        const float2* S = P.smaps + (long long)c * g.Ni;
        k64_pad<<<nb64(g.Ng), 256, 0, P.s>>>(x, S, P.ap[0], P.ap[1], P.ap[2], g, P.grid);
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        if (cufftExecZ2Z(P.plan, (cufftDoubleComplex*)P.grid, (cufftDoubleComplex*)P.grid, CUFFT_FORWARD) != CUFFT_SUCCESS)
            return cudaErrorUnknown;
        k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
        k64_loss_grad<<<nblk, 256, 0, P.s>>>(P.grid, k, sorted, n, g, kb_w, kb_b, thresh, y + (long long)c * ns, dcf,
                                            grad_k, grad_x ? P.y : nullptr, partials);
        e = cudaMemcpyAsync(h.data(), partials, nblk * sizeof(double), cudaMemcpyDeviceToHost, P.s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(P.s);
        for (unsigned i = 0; i < nblk; ++i) total += h[i];
        if (grad_x) {
            cudaMemsetAsync(P.grid, 0, g.Ng * sizeof(double2), P.s);
            if (n > 0) k64_spread_taps<<<nb64(n), 256, 0, P.s>>>(P.y, k, sorted, n, g, kb_w, kb_b, thresh, P.grid);
            k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
            if (cufftExecZ2Z(P.plan, (cufftDoubleComplex*)P.grid, (cufftDoubleComplex*)P.grid, CUFFT_INVERSE) !=
                CUFFT_SUCCESS)
                return cudaErrorUnknown;
            k64_sign<<<nb64(g.Ng), 256, 0, P.s>>>(P.grid, g);
            k64_crop<<<nb64(g.Ni), 256, 0, P.s>>>(P.grid, S, P.ap[0], P.ap[1], P.ap[2], 1.0, g, c == 0, grad_x);
        }
    }
    *loss = total;
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

}  // namespace cgs
