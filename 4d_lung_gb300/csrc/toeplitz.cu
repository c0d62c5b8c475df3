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

cudaError_t launch_toep_mul(float2* grid, const float* P, long long Ng, int nch, int items, cudaStream_t s)
{
    const long long total = Ng * items;
    const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 16);
    k_toep_mul<<<(unsigned)blocks, 256, 0, s>>>(grid, P, Ng, nch, total);
    return cudaGetLastError();
}

}  // namespace cgs
