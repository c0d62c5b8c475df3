// toeplitz.cu -- Toeplitz embedding of the normal operator E^H D E for a
// fixed trajectory: the per-bin spectrum of its point-spread function on the
// oversampled grid, built once, and the element-wise multiply of the
// unfused form.
//
// With E the exact non-uniform DFT of the sample positions
//   (E x)_i = sum_r x[r] exp(-2 pi i nu_i . (r + lo - G/2)),
//   nu_ia = (k_ia (G_a - 1) - G_a / 2) / G_a   (cycles per grid cell),
// the normal operator is a convolution over the image box,
//   (E^H D E x)[r'] = sum_r x[r] h(r' - r),  h(d) = sum_i D_i exp(2 pi i nu_i . d),
// which the grid holds without wrap-around once G_a >= 2 I_a - 1.  Between
// the library's centred forward and adjoint transforms F_c, F_c^H it is the
// diagonal
//   P[k] = s / Ng * sum_{|d_a| < I_a} (-1)^(dx+dy+dz) h(d) exp(-2 pi i k . d / G)
//        = s / Ng * sum_i D_i Kx_i(kx) Ky_i(ky) Kz_i(kz),
//   K_ia(k) = sum_{|d| < I_a} exp(2 pi i psi d) = sin((2 I_a - 1) pi psi) / sin(pi psi),
//   psi = nu_ia - k / G_a + 1/2,
// a real array (s: the adjoint scale of the gridded operator).  The sum over
// samples is a rank-M product of per-axis Dirichlet kernels; it is formed as
// one FP32 matrix product per chunk of samples,
//   P[kx][ky, kz] += sum_i Kx[kx][i] * W[i][ky, kz],  W[i] = s/Ng D_i Ky_i (x) Kz_i,
// through cuBLAS (opened at run time; no link-time dependency).
#include "launch.h"
#include <cublas_v2.h>
#include <dlfcn.h>
#include <algorithm>
#include <string>

namespace cgs {

namespace {

// Dirichlet kernel sum_{|d| <= m2} exp(2 pi i psi d), m = 2 m2 + 1 terms;
// psi reduced to [-1/2, 1/2) (the kernel has period 1 for odd m)
__device__ double dirichlet(double psi, int m)
{
    double e = psi - floor(psi + 0.5);
    if (e == 0.0) return (double)m;
    return sinpi((double)m * e) / sinpi(e);
}

// Per chunk of n sorted samples [s0, s0 + n):
//   kx[kx * n + i]            = Kx_i(kx)
//   ky[i * Gy + ky]           = s/Ng * D_i * Ky_i(ky)
//   kz[i * Gz + kz]           = Kz_i(kz)
__global__ void k_toep_tables(ToepBuildArgs a, long long n, float* __restrict__ kx, float* __restrict__ ky,
                              float* __restrict__ kz)
{
    const long long i = blockIdx.y;
    if (i >= n) return;
    const long long g = a.sorted[a.s0 + i];
    const int Gs = a.G[0] + a.G[1] + a.G[2];
    for (int t = threadIdx.x + blockIdx.x * blockDim.x; t < Gs; t += blockDim.x * gridDim.x) {
        int ax = 0, kk = t;
        if (kk >= a.G[0]) {
            kk -= a.G[0];
            ax = 1;
            if (kk >= a.G[1]) {
                kk -= a.G[1];
                ax = 2;
            }
        }
        const int G = a.G[ax];
        const double nu = (a.k[3 * g + ax] * (double)(G - 1) - 0.5 * (double)G) / (double)G;
        const double v = dirichlet(nu - (double)kk / (double)G + 0.5, 2 * a.I[ax] - 1);
        if (ax == 0) {
            kx[(long long)kk * n + i] = (float)v;
        } else if (ax == 1) {
            const double d = a.dcf ? (double)a.dcf[a.s0 + i] : 1.0;
            ky[i * a.G[1] + kk] = (float)(v * d * a.scale);
        } else {
            kz[i * a.G[2] + kk] = (float)v;
        }
    }
}

// w[i][ky * Gz + kz] = ky[i][ky] * kz[i][kz]
__global__ void k_toep_outer(const float* __restrict__ ky, const float* __restrict__ kz, long long n, int Gy, int Gz,
                             float* __restrict__ w)
{
    const long long yz = (long long)Gy * Gz;
    const long long total = n * yz;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long i = e / yz;
        const long long r = e - i * yz;
        const int y = (int)(r / Gz), z = (int)(r - (long long)y * Gz);
        w[e] = ky[i * Gy + y] * kz[i * Gz + z];
    }
}

// grid[item][j] *= P[item / nch][j]  (unfused form)
__global__ void k_toep_mul(float2* __restrict__ grid, const float* __restrict__ P, long long Ng, int nch,
                           long long total)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long item = e / Ng;
        const long long j = e - item * Ng;
        const float p = P[(item / nch) * Ng + j];
        float2 v = grid[e];
        v.x *= p;
        v.y *= p;
        grid[e] = v;
    }
}

// cuBLAS entry points, resolved once (thread-safe: a function-local static
// is initialised by exactly one thread, the others wait for it)
struct Blas {
    void* lib = nullptr;
    cublasStatus_t (*create)(cublasHandle_t*) = nullptr;
    cublasStatus_t (*destroy)(cublasHandle_t) = nullptr;
    cublasStatus_t (*set_stream)(cublasHandle_t, cudaStream_t) = nullptr;
    cublasStatus_t (*sgemm)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int, int, int, const float*,
                            const float*, int, const float*, int, const float*, float*, int) = nullptr;
};

Blas open_blas()
{
    Blas b;
    for (const char* name : {"libcublas.so.13", "libcublas.so"}) {
        b.lib = dlopen(name, RTLD_NOW | RTLD_LOCAL);
        if (b.lib) break;
    }
    if (b.lib) {
        b.create = reinterpret_cast<decltype(b.create)>(dlsym(b.lib, "cublasCreate_v2"));
        b.destroy = reinterpret_cast<decltype(b.destroy)>(dlsym(b.lib, "cublasDestroy_v2"));
        b.set_stream = reinterpret_cast<decltype(b.set_stream)>(dlsym(b.lib, "cublasSetStream_v2"));
        b.sgemm = reinterpret_cast<decltype(b.sgemm)>(dlsym(b.lib, "cublasSgemm_v2"));
    }
    return b;
}

const Blas& blas()
{
    static const Blas b = open_blas();
    return b;
}

}  // namespace

long long toeplitz_chunk(const int G[3], long long work_elems)
{
    const long long yz = (long long)G[1] * G[2];
    const long long per = yz + G[0] + G[1] + G[2];   // W row + the three table entries of a sample
    long long n = work_elems / per;
    // W within 2^30 elements (32-bit GEMM extents), one sample per grid row of the table kernel
    n = std::min(n, (1LL << 30) / std::max<long long>(yz, 1));
    return std::min(n, 65535LL);
}

void toeplitz_release(void* handle)
{
    const Blas& b = blas();
    if (handle && b.destroy) b.destroy(static_cast<cublasHandle_t>(handle));
}

int toeplitz_build(const ToepBuildArgs& a, float* work, long long work_elems, void** handle, cudaStream_t s,
                   std::string* err)
{
    const Blas& b = blas();
    if (!b.lib || !b.create || !b.destroy || !b.set_stream || !b.sgemm) {
        if (err) *err = "cuBLAS could not be opened (libcublas.so.13)";
        return 1;
    }
    const long long Ng = (long long)a.G[0] * a.G[1] * a.G[2];
    const long long yz = (long long)a.G[1] * a.G[2];
    if (a.n == 0) {
        cudaError_t e = cudaMemsetAsync(a.P, 0, (size_t)Ng * sizeof(float), s);
        if (e != cudaSuccess && err) *err = cudaGetErrorString(e);
        return e == cudaSuccess ? 0 : 1;
    }
    const long long chunk = toeplitz_chunk(a.G, work_elems);
    if (chunk < 1) {
        if (err) *err = "Toeplitz work buffer too small";
        return 1;
    }
    // one handle per context, created at its first build
    if (!*handle) {
        cublasHandle_t hn = nullptr;
        if (b.create(&hn) != CUBLAS_STATUS_SUCCESS) {
            if (err) *err = "cublasCreate failed";
            return 1;
        }
        *handle = hn;
    }
    cublasHandle_t h = static_cast<cublasHandle_t>(*handle);
    int rc = 0;
    if (b.set_stream(h, s) != CUBLAS_STATUS_SUCCESS) rc = 1;
    for (long long c0 = 0; rc == 0 && c0 < a.n; c0 += chunk) {
        const long long n = std::min(chunk, a.n - c0);
        float* w = work;
        float* kx = w + n * yz;
        float* ky = kx + n * a.G[0];
        float* kz = ky + n * a.G[1];
        ToepBuildArgs ca = a;
        ca.s0 = a.s0 + c0;
        const int gs = a.G[0] + a.G[1] + a.G[2];
        k_toep_tables<<<dim3((unsigned)((gs + 255) / 256), (unsigned)n), 256, 0, s>>>(ca, n, kx, ky, kz);
        k_toep_outer<<<2048, 256, 0, s>>>(ky, kz, n, a.G[1], a.G[2], w);
        if (cudaGetLastError() != cudaSuccess) {
            rc = 2;
            break;
        }
        // column-major view: P^T (yz x Gx) = W^T (yz x n) * Kx^T (n x Gx)
        const float one = 1.f, beta = c0 == 0 ? 0.f : 1.f;
        if (b.sgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)yz, a.G[0], (int)n, &one, w, (int)yz, kx, (int)n, &beta, a.P,
                    (int)yz) != CUBLAS_STATUS_SUCCESS)
            rc = 1;
    }
    if (rc && err) *err = rc == 2 ? "Toeplitz table kernels failed to launch" : "cublasSgemm failed";
    return rc;
}

// ---------------------------------------------------------------------------
// Spectrum through the point-spread function (the default where the fine
// grid's line lengths have FFT kernels).  h(d) = sum_i D_i exp(2 pi i nu_i.d)
// on |d_a| < I_a is an adjoint (type-1) NUFFT of the density weights:
//   1. k_psf_spread: D_i times a Kaiser-Bessel window of width w <= 7 on the
//      fine grid nf (nf_a >= 4 I_a, two-fold oversampling of the 2 I_a
//      modes), sample at nf nu + nf/2, periodic; FP64 accumulation;
//   2. k_psf_convert: to complex float;
//   3. the library's centred FFT passes (sign +1) keeping the 2 I_a central
//      output positions per axis (d in [-I_a, I_a));
//   4. k_psf_place: divide by the window's Fourier transform, times
//      (-1)^(sum nf_a / 2), into the grid at d + G/2 (zero outside |d_a| < I_a);
//   5. the centred FFT of the grid (sign -1);
//   6. k_psf_spectrum: P = s/Ng (-1)^(sum G_a / 2) Re(.).
// Cost O(M w^3 + N_fine log N_fine) per bin instead of the Dirichlet
// product's 2 Ng M flops; the window error at w = 7 is ~5e-7 relative.
// ---------------------------------------------------------------------------

// One warp per sample: lanes 0..23 evaluate the 3 x PSF_TAPS window factors
// (FP64 I0), then the warp adds the PSF_TAPS^3 products (z fastest, so
// consecutive lanes hit consecutive addresses) with FP64 atomics.
__global__ void __launch_bounds__(256) k_psf_spread(PsfSpreadArgs a)
{
    __shared__ double s_f[8][3 * PSF_TAPS];
    __shared__ int s_g[8][3 * PSF_TAPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long i = (long long)blockIdx.x * 8 + warp;
    if (i >= a.n) return;                       // whole warp
    const long long g = a.sorted[a.s0 + i];
    const double d = a.dcf ? (double)a.dcf[a.s0 + i] : 1.0;
    if (lane < 3 * PSF_TAPS) {
        const int ax = lane / PSF_TAPS, t = lane % PSF_TAPS;
        const double G = (double)a.G[ax], nf = (double)a.nf[ax];
        const double nu = (a.k[3 * g + ax] * (G - 1.0) - 0.5 * G) / G;
        const double u = nf * nu + 0.5 * nf;
        const double g0 = ceil(u - 0.5 * a.w);
        const double x = g0 + (double)t - u;
        const double q = 1.0 - (2.0 * x / a.w) * (2.0 * x / a.w);
        double f = q >= 0.0 ? cyl_bessel_i0(a.beta * sqrt(q)) : 0.0;
        if (ax == 0) f *= d;
        int gi = (int)g0 + t;
        gi %= a.nf[ax];
        if (gi < 0) gi += a.nf[ax];
        s_f[warp][lane] = f;
        s_g[warp][lane] = gi;
    }
    __syncwarp();
    const double* f = s_f[warp];
    const int* gg = s_g[warp];
    constexpr int T3 = PSF_TAPS * PSF_TAPS * PSF_TAPS;
    for (int c = lane; c < T3; c += 32) {
        const int tx = c / (PSF_TAPS * PSF_TAPS), ty = (c / PSF_TAPS) % PSF_TAPS, tz = c % PSF_TAPS;
        const double v = f[tx] * f[PSF_TAPS + ty] * f[2 * PSF_TAPS + tz];
        if (v == 0.0) continue;
        const long long e = ((long long)gg[tx] * a.nf[1] + gg[PSF_TAPS + ty]) * a.nf[2] + gg[2 * PSF_TAPS + tz];
        atomicAdd(a.out + e, v);
    }
}

__global__ void k_psf_convert(const double* __restrict__ in, float2* __restrict__ out, long long n)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        out[e] = make_float2((float)in[e], 0.f);
}

// grid[k] = sgn * R[d + I] * rx[dx + I] ry[..] rz[..] for |d_a| < I_a, d = k - G/2; else 0.
// R: [2Ix][2Iy][2Iz]; r*: reciprocal window transforms at d / nf, d in [-I, I).
__global__ void k_psf_place(const float2* __restrict__ R, const float* __restrict__ rx, const float* __restrict__ ry,
                            const float* __restrict__ rz, int Gx, int Gy, int Gz, int Ix, int Iy, int Iz, float sgn,
                            float2* __restrict__ grid)
{
    const long long n = (long long)Gx * Gy * Gz;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(e % Gz);
        const long long t = e / Gz;
        const int ky = (int)(t % Gy), kx = (int)(t / Gy);
        const int dx = kx - Gx / 2, dy = ky - Gy / 2, dz = kz - Gz / 2;
        float2 v = make_float2(0.f, 0.f);
        if (dx > -Ix && dx < Ix && dy > -Iy && dy < Iy && dz > -Iz && dz < Iz) {
            const int jx = dx + Ix, jy = dy + Iy, jz = dz + Iz;
            const float2 r = R[((long long)jx * (2 * Iy) + jy) * (2 * Iz) + jz];
            const float m = sgn * rx[jx] * ry[jy] * rz[jz];
            v = make_float2(r.x * m, r.y * m);
        }
        grid[e] = v;
    }
}

// P[k] = scale * Re(grid[k])
__global__ void k_psf_spectrum(const float2* __restrict__ grid, float scale, long long n, float* __restrict__ P)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        P[e] = scale * grid[e].x;
}

namespace {
unsigned grid_stride_blocks(long long n)
{
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16));
}
}  // namespace

cudaError_t launch_psf_spread(const PsfSpreadArgs& a, cudaStream_t s)
{
    if (a.n <= 0) return cudaSuccess;
    k_psf_spread<<<(unsigned)((a.n + 7) / 8), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_psf_convert(const double* in, float2* out, long long n, cudaStream_t s)
{
    k_psf_convert<<<grid_stride_blocks(n), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_psf_place(const float2* R, const float* rx, const float* ry, const float* rz, const int G[3],
                             const int I[3], float sgn, float2* grid, cudaStream_t s)
{
    const long long n = (long long)G[0] * G[1] * G[2];
    k_psf_place<<<grid_stride_blocks(n), 256, 0, s>>>(R, rx, ry, rz, G[0], G[1], G[2], I[0], I[1], I[2], sgn, grid);
    return cudaGetLastError();
}

cudaError_t launch_psf_spectrum(const float2* grid, float scale, long long n, float* P, cudaStream_t s)
{
    k_psf_spectrum<<<grid_stride_blocks(n), 256, 0, s>>>(grid, scale, n, P);
    return cudaGetLastError();
}

cudaError_t launch_toep_mul(float2* grid, const float* P, long long Ng, int nch, int items, cudaStream_t s)
{
    const long long total = Ng * items;
    const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 16);
    k_toep_mul<<<(unsigned)blocks, 256, 0, s>>>(grid, P, Ng, nch, total);
    return cudaGetLastError();
}

}  // namespace cgs
