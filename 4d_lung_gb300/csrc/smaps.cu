// smaps.cu -- coil sensitivity maps from low-resolution coil images, the
// optional on-GPU companion of the root-sum-of-squares pre-step
// (Reco.cpp:468-519 on measured data, rssq2DVecImg functions.h:290-316):
//   S_c = I_c / sqrt(sum_c |I_c|^2)  where the root-sum-of-squares exceeds
//   eps * its maximum, 0 elsewhere,
// I_c the adjoint NUFFT of the measured samples weighted by a Hann window of
// radius r grid cells around the k-space centre (and D when set).  No
// eigen-decomposition (ESPIRiT) is involved.
#include "launch.h"

namespace cgs {

// w[j] = (D[j] or 1) * cos^2(pi d / (2 r)) for d < r, else 0, with d the
// distance of sorted sample j from the k-space centre in grid cells
// (grid coordinate k (N - 1), centre (N - 1) / 2)
__global__ void k_lowpass_weights(const double* __restrict__ k, const int* __restrict__ sorted, long long n,
                                  int Gx, int Gy, int Gz, double radius, const float* __restrict__ dcf,
                                  float* __restrict__ w)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long long g = sorted[j];
    const double dx = (k[3 * g] - 0.5) * (Gx - 1), dy = (k[3 * g + 1] - 0.5) * (Gy - 1),
                 dz = (k[3 * g + 2] - 0.5) * (Gz - 1);
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    double v = 0.0;
    if (d < radius) {
        const double cs = cospi(d / (2.0 * radius));
        v = cs * cs;
    }
    w[j] = (float)v * (dcf ? dcf[j] : 1.f);
}

__global__ void k_rss_max(const float2* __restrict__ imgs, int nch, long long n, float* __restrict__ rss,
                          unsigned* __restrict__ max_bits)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float r = 0.f;
    if (i < n) {
        float acc = 0.f;
        for (int c = 0; c < nch; ++c) {
            const float2 v = imgs[(long long)c * n + i];
            acc += v.x * v.x + v.y * v.y;
        }
        r = sqrtf(acc);
        rss[i] = r;
    }
    // non-negative floats order like their bit patterns: the maximum is exact
    // and independent of the order of the updates
    for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_bits, __float_as_uint(r));
}

__global__ void k_smaps_divide(float2* __restrict__ imgs, int nch, long long n, const float* __restrict__ rss,
                               const unsigned* __restrict__ max_bits, float eps)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nch * n) return;
    const long long i = e % n;
    const float r = rss[i];
    const float lim = eps * __uint_as_float(*max_bits);
    float2 v = imgs[e];
    if (r > lim && r > 0.f) v = make_float2(v.x / r, v.y / r);
    else v = make_float2(0.f, 0.f);
    imgs[e] = v;
}

cudaError_t launch_lowpass_weights(const double* k, const int* sorted, long long n, const int* G, double radius,
                                   const float* dcf_sorted, float* w, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_lowpass_weights<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(k, sorted, n, G[0], G[1], G[2], radius, dcf_sorted,
                                                                   w);
    return cudaGetLastError();
}

cudaError_t launch_smaps_from_images(float2* imgs, int nch, long long n, float eps, float* rss_tmp,
                                     unsigned* max_tmp, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(max_tmp, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    k_rss_max<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(imgs, nch, n, rss_tmp, max_tmp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const long long m = n * nch;
    k_smaps_divide<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(imgs, nch, n, rss_tmp, max_tmp, eps);
    return cudaGetLastError();
}

}  // namespace cgs
