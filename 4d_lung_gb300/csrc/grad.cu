// grad.cu -- gradients of the data-consistency loss
//   L = 1/2 sum_c sum_i D_i |(E_c S_c x)_i - y_ci|^2
// with respect to the sample coordinates (and, through the adjoint chain,
// the image).  E_c is the forward operator of nufftFWD (Reco.cpp:521-553);
// the reference has no derivatives, this is the extension that trajectory
// self-calibration needs.
//
// The interpolation weight of a tap is the product of three per-axis KB
// factors, w = fx(kx) fy(ky) fz(kz), so dw/dkx = fx'(kx) fy fz and so on.
// The per-axis derivatives are stored per sample like the tap records
// (15 floats + the packed nearest point), and one gather pass computes the
// predicted samples, their three coordinate derivatives, the residual, the
// loss partials and dL/dk.
#include "launch.h"
#include "gridding_common.cuh"

#include <algorithm>

namespace cgs {

// Derivative records: df/dk of the 5 candidate factors per axis, with the
// distance arithmetic of k_tap_records (Reco.cpp:763-771: double k minus
// float index * float dk, distance rounded to float).  For
// f = I0(b s) / C, s = sqrt(1 - q^2), q = 2 |d| / (w dk):
//   df/dk = -(I1(b s) / s) * b * q * sign(d) * 2 / (w dk) / C,
// with I1(b s) / s -> b / 2 as s -> 0.
__global__ void k_tap_grad_records(const double* __restrict__ k, const int* __restrict__ sample_idx, long long n,
                                   KbParams kb, TapRecord* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long g = sample_idx ? sample_idx[i] : i;
    TapRecord r;
    float* f = reinterpret_cast<float*>(&r);
    const float wHalf = (float)(kb.w / 2.0);
    int nearest[3];
    for (int a = 0; a < 3; ++a) {
        const int N = kb.G[a];
        const double ka = k[3 * g + a];
        const float dk = (float)(1.0 / (double)(float)(N - 1));
        int nr = (int)__dadd_rn(__dmul_rn((double)(N - 1), ka), 0.5);
        nr = nr < 0 ? 0 : (nr > N - 1 ? N - 1 : nr);
        nearest[a] = nr;
        for (int j = 0; j < TAPS_1D; ++j) {
            const int gi = nr - 2 + j;
            float val = 0.f;
            if (gi >= 0 && gi <= N - 1) {
                const double dd = ka - (double)__fmul_rn((float)gi, dk);
                const float d = (float)fabs(dd);
                if (!(d > wHalf * dk)) {
                    const float q = (float)(2.f * d) / (float)(kb.w * dk);
                    const double s2 = __dadd_rn(1.0, -__dmul_rn((double)q, (double)q));
                    const double s = s2 > 0.0 ? sqrt(s2) : 0.0;
                    const double b = (double)kb.b;
                    const double i1s = s > 1e-12 ? cyl_bessel_i1(b * s) / s : 0.5 * b;
                    const double C = (double)(float)(100.0f * kb.w * dk);
                    const double dv = -i1s * b * (double)q * (2.0 / ((double)kb.w * (double)dk)) / C;
                    val = (float)(dd >= 0.0 ? dv : -dv);
                }
            }
            f[a * TAPS_1D + j] = val;
        }
    }
    f[15] = __uint_as_float(pack_nearest(nearest[0], nearest[1], nearest[2]));
    out[i] = r;
}

cudaError_t launch_tap_grad_records(const double* k, const int* sample_idx, long long n, const KbParams& kb,
                                    TapRecord* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_tap_grad_records<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, sample_idx, n, kb, out);
    return cudaGetLastError();
}

// One thread per sample of one bin; coils in chunks of CC.  Writes
//   rv[i][c]     = D_i r_ci          (the adjoint chain's samples), if rv
//   grad_k[g][a] = sum_c D_i Re(conj(r_ci) dy_ci/dk_a), g the global index
//   partials[b]  = sum over the block of 1/2 D_i |r_ci|^2
template <int CC>
__global__ void __launch_bounds__(128) k_interp_grad(InterpGradArgs a)
{
    __shared__ double s_red[4];
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double loss = 0.0;
    if (j < a.n) {
        const long long i = a.s0 + j;
        float w[15], dw[15];
        int nx, ny, nz, t0, t1, t2;
        load_record(a.rec, i, w, nx, ny, nz);
        load_record(a.drec, i, dw, t0, t1, t2);
        const float D = a.dcf ? a.dcf[i] : 1.f;
        const int Gy = a.G[1], Gz = a.G[2];
        float gk0 = 0.f, gk1 = 0.f, gk2 = 0.f;
        for (int c0 = 0; c0 < a.nch; c0 += CC) {
            const int ncc = min(CC, a.nch - c0);
            const float2* grid = a.grid + (long long)c0 * a.coil_stride;
            float2 y[CC], d0[CC], d1[CC], d2[CC];
#pragma unroll
            for (int c = 0; c < CC; ++c) y[c] = d0[c] = d1[c] = d2[c] = make_float2(0.f, 0.f);
#pragma unroll
            for (int jx = 0; jx < 5; ++jx) {
                const float wx = w[jx], dwx = dw[jx];
                if (wx == 0.f) continue;
                const int gx = nx - 2 + jx;
#pragma unroll
                for (int jy = 0; jy < 5; ++jy) {
                    const float wy = w[5 + jy], dwy = dw[5 + jy];
                    if (wy == 0.f) continue;
                    const long long row = ((long long)gx * Gy + (ny - 2 + jy)) * Gz + (nz - 2);
#pragma unroll
                    for (int jz = 0; jz < 5; ++jz) {
                        const float wz = w[10 + jz], dwz = dw[10 + jz];
                        const float wt = (wx * wy) * wz;
                        if (wz != 0.f && wt > a.thresh) {
                            const float ex = (dwx * wy) * wz, ey = (wx * dwy) * wz, ez = (wx * wy) * dwz;
#pragma unroll
                            for (int c = 0; c < CC; ++c)
                                if (c < ncc) {
                                    const float2 g = __ldg(grid + (long long)c * a.coil_stride + row + jz);
                                    y[c].x = fmaf(g.x, wt, y[c].x);
                                    y[c].y = fmaf(g.y, wt, y[c].y);
                                    d0[c].x = fmaf(g.x, ex, d0[c].x);
                                    d0[c].y = fmaf(g.y, ex, d0[c].y);
                                    d1[c].x = fmaf(g.x, ey, d1[c].x);
                                    d1[c].y = fmaf(g.y, ey, d1[c].y);
                                    d2[c].x = fmaf(g.x, ez, d2[c].x);
                                    d2[c].y = fmaf(g.y, ez, d2[c].y);
                                }
                        }
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < CC; ++c)
                if (c < ncc) {
                    const float2 m = a.ymeas[i * a.nch + c0 + c];
                    const float rx = y[c].x - m.x, ry = y[c].y - m.y;
                    loss += 0.5 * (double)D * ((double)rx * rx + (double)ry * ry);
                    gk0 += D * (rx * d0[c].x + ry * d0[c].y);
                    gk1 += D * (rx * d1[c].x + ry * d1[c].y);
                    gk2 += D * (rx * d2[c].x + ry * d2[c].y);
                    if (a.rv) a.rv[i * a.nch + c0 + c] = make_float2(D * rx, D * ry);
                }
        }
        if (a.grad_k) {
            const long long g = a.sorted[i];
            a.grad_k[3 * g + 0] = gk0;
            a.grad_k[3 * g + 1] = gk1;
            a.grad_k[3 * g + 2] = gk2;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = loss;
    __syncthreads();
    if (threadIdx.x == 0) a.partials[blockIdx.x] = s_red[0] + s_red[1] + s_red[2] + s_red[3];
}

int interp_grad_blocks(long long n) { return (int)std::max<long long>((n + 127) / 128, 1); }

cudaError_t launch_interp_grad(const InterpGradArgs& a, cudaStream_t s)
{
    k_interp_grad<4><<<(unsigned)interp_grad_blocks(a.n), 128, 0, s>>>(a);
    return cudaGetLastError();
}

// Finiteness of device coordinates: *bad = 1 when any is NaN or Inf.
__global__ void k_check_finite(const double* __restrict__ v, long long n, int* bad)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !isfinite(v[i])) atomicExch(bad, 1);
}

cudaError_t launch_check_finite(const double* v, long long n, int* bad, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_check_finite<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(v, n, bad);
    return cudaGetLastError();
}

// Values and coordinate derivatives of E S u at one bin's samples, then
// either stored (outA) or contracted with a stored pair (A, dA).  One thread
// per sample; coils in chunks of CC.
template <int CC>
__global__ void __launch_bounds__(128) k_pair_grad(PairGradArgs a)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    const long long i = a.s0 + j;
    float w[15], dw[15];
    int nx, ny, nz, t0, t1, t2;
    load_record(a.rec, i, w, nx, ny, nz);
    load_record(a.drec, i, dw, t0, t1, t2);
    const float D = a.dcf ? a.dcf[i] : 1.f;
    const int Gy = a.G[1], Gz = a.G[2];
    float gk0 = 0.f, gk1 = 0.f, gk2 = 0.f;
    for (int c0 = 0; c0 < a.nch; c0 += CC) {
        const int ncc = min(CC, a.nch - c0);
        const float2* grid = a.grid + (long long)c0 * a.coil_stride;
        float2 y[CC], d0[CC], d1[CC], d2[CC];
#pragma unroll
        for (int c = 0; c < CC; ++c) y[c] = d0[c] = d1[c] = d2[c] = make_float2(0.f, 0.f);
#pragma unroll
        for (int jx = 0; jx < 5; ++jx) {
            const float wx = w[jx], dwx = dw[jx];
            if (wx == 0.f) continue;
            const int gx = nx - 2 + jx;
#pragma unroll
            for (int jy = 0; jy < 5; ++jy) {
                const float wy = w[5 + jy], dwy = dw[5 + jy];
                if (wy == 0.f) continue;
                const long long row = ((long long)gx * Gy + (ny - 2 + jy)) * Gz + (nz - 2);
#pragma unroll
                for (int jz = 0; jz < 5; ++jz) {
                    const float wz = w[10 + jz], dwz = dw[10 + jz];
                    const float wt = (wx * wy) * wz;
                    if (wz != 0.f && wt > a.thresh) {
                        const float ex = (dwx * wy) * wz, ey = (wx * dwy) * wz, ez = (wx * wy) * dwz;
#pragma unroll
                        for (int c = 0; c < CC; ++c)
                            if (c < ncc) {
                                const float2 g = __ldg(grid + (long long)c * a.coil_stride + row + jz);
                                y[c].x = fmaf(g.x, wt, y[c].x);
                                y[c].y = fmaf(g.y, wt, y[c].y);
                                d0[c].x = fmaf(g.x, ex, d0[c].x);
                                d0[c].y = fmaf(g.y, ex, d0[c].y);
                                d1[c].x = fmaf(g.x, ey, d1[c].x);
                                d1[c].y = fmaf(g.y, ey, d1[c].y);
                                d2[c].x = fmaf(g.x, ez, d2[c].x);
                                d2[c].y = fmaf(g.y, ez, d2[c].y);
                            }
                    }
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CC; ++c)
            if (c < ncc) {
                const long long e = i * a.nch + c0 + c;
                if (a.outA) {
                    a.outA[e] = y[c];
                    a.outdA[3 * e + 0] = d0[c];
                    a.outdA[3 * e + 1] = d1[c];
                    a.outdA[3 * e + 2] = d2[c];
                } else {
                    // Re(conj(B) dA + conj(dB) A), B = y, dB = d*
                    const float2 A = a.A[e];
                    gk0 += A.x * d0[c].x + A.y * d0[c].y;
                    gk1 += A.x * d1[c].x + A.y * d1[c].y;
                    gk2 += A.x * d2[c].x + A.y * d2[c].y;
                    if (a.dA) {
                        const float2 e0 = a.dA[3 * e + 0], e1 = a.dA[3 * e + 1], e2 = a.dA[3 * e + 2];
                        gk0 += y[c].x * e0.x + y[c].y * e0.y;
                        gk1 += y[c].x * e1.x + y[c].y * e1.y;
                        gk2 += y[c].x * e2.x + y[c].y * e2.y;
                    }
                }
            }
    }
    if (!a.outA) {
        const long long g = a.sorted[i];
        const float f = a.scale * D;
        a.grad_k[3 * g + 0] += f * gk0;
        a.grad_k[3 * g + 1] += f * gk1;
        a.grad_k[3 * g + 2] += f * gk2;
    }
}

cudaError_t launch_pair_grad(const PairGradArgs& a, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    k_pair_grad<2><<<(unsigned)((a.n + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

// Iterative density weights (Pipe and Menon, Magn. Reson. Med. 41:179-186,
// 1999): w <- w / (C * w) at the samples, C * w the interpolation of the
// spread weights.  v is the spread input (w, 0) and u the interpolated sum.
// A sample without any tap in the grid (C * w = 0) gets weight 0, as a hull
// sample's Voronoi cell does.
__global__ void k_pm_update(float* __restrict__ w, float2* __restrict__ v, const float2* __restrict__ u, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c = u[i].x;
    const float nw = c > 0.f ? w[i] / c : 0.f;
    w[i] = nw;
    v[i] = make_float2(nw, 0.f);
}

cudaError_t launch_pm_update(float* w, float2* v, const float2* u, long long n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_pm_update<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, v, u, n);
    return cudaGetLastError();
}

__global__ void k_pm_init(float* __restrict__ w, float2* __restrict__ v, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    w[i] = 1.f;
    v[i] = make_float2(1.f, 0.f);
}

cudaError_t launch_pm_init(float* w, float2* v, long long n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_pm_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, v, n);
    return cudaGetLastError();
}

}  // namespace cgs
