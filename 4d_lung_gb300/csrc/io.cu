// io.cu -- file IO of the reconstruction (IO.cpp of the reference) with the
// sample permutation and the coil-image root-sum-of-squares on the GPU.
//
// File formats are the reference's: raw samples are interleaved float32
// complex values, channel by channel, readout-fastest within a channel
// (IO.cpp:55-98); coil maps are <dir>/map<c>.bin (IO.cpp:25-51); images and
// weights are plain float32 arrays (IO.cpp:12-22, 129-186).
#include "cgsense_c.h"
#include "cgs_common.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <thread>
#include <vector>

namespace cgs {

// file order (ch, i1 + sx*i2 + sx*sy*i3) -> memory order (ch, i3 + sz*i2 + sy*sz*i1)
__global__ void k_permute_samples(const float2* __restrict__ src, float2* __restrict__ dst, int sx, int sy, int sz,
                                  long long total)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= total) return;
    const long long ns = (long long)sx * sy * sz;
    const long long ch = k / ns;
    const long long s = k - ch * ns;
    const long long sxsy = (long long)sx * sy;
    const long long i3 = s / sxsy;
    const long long r = s - i3 * sxsy;
    const long long i2 = r / sx;
    const long long i1 = r - i2 * sx;
    dst[ch * ns + i3 + (long long)sz * i2 + (long long)sy * sz * i1] = src[k];
}

// out[i] = sqrt(sum_c |img_c[i]|^2), coils in order, float arithmetic as
// rssq2DVecImg (functions.h:290-316)
__global__ void k_rss(const float2* __restrict__ imgs, int nch, long long n, float* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float acc = 0.f;
    for (int c = 0; c < nch; ++c) {
        const float2 v = imgs[(long long)c * n + i];
        acc += v.x * v.x + v.y * v.y;
    }
    out[i] = sqrtf(acc);
}

// data[ch][i] *= d[i] (performDensityCorrection, functions.h:319-335)
__global__ void k_scale_samples(float2* data, const float* __restrict__ d, long long ns, int nch)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns * nch) return;
    const float w = d[k % ns];
    data[k] = make_float2(data[k].x * w, data[k].y * w);
}

cudaError_t launch_scale_samples(float2* data, const float* d, long long ns, int nch, cudaStream_t s)
{
    if (ns * nch == 0) return cudaSuccess;
    k_scale_samples<<<(unsigned)((ns * nch + 255) / 256), 256, 0, s>>>(data, d, ns, nch);
    return cudaGetLastError();
}

namespace {

struct PinnedBuf {
    void* p = nullptr;
    size_t n = 0;
    ~PinnedBuf()
    {
        if (p) cudaFreeHost(p);
    }
    bool ensure(size_t bytes)
    {
        if (bytes <= n) return true;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) return false;
        n = bytes;
        return true;
    }
};

// writes `bytes` from a host pointer; the reference retries path + "_1.bin"
// when the path cannot be opened (IO.cpp:170-183)
int write_file(const std::string& path, const void* h, size_t bytes, bool retry)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f && retry) f = std::fopen((path + "_1.bin").c_str(), "wb");
    if (!f) return CGS_ERR_IO;
    const size_t w = bytes ? std::fwrite(h, 1, bytes, f) : 0;
    std::fclose(f);
    return w == bytes ? CGS_OK : CGS_ERR_IO;
}

int export_bin(const char* path, const void* src, size_t bytes, int on_device, void* stream, bool retry)
{
    if (!path || (!src && bytes)) return CGS_ERR_ARG;
    if (!on_device) return write_file(path, src, bytes, retry);
    PinnedBuf hb;
    if (!hb.ensure(bytes ? bytes : 1)) return CGS_ERR_NOMEM;
    cudaStream_t s = (cudaStream_t)stream;
    if (bytes && cudaMemcpyAsync(hb.p, src, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return CGS_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return CGS_ERR_CUDA;
    return write_file(path, hb.p, bytes, retry);
}

}  // namespace

}  // namespace cgs

using namespace cgs;

extern "C" {

int cgs_permute_samples_d(const void* src, void* dst, int32_t sx, int32_t sy, int32_t sz, int32_t nch, void* stream)
{
    if (!src || !dst || sx < 1 || sy < 1 || sz < 1 || nch < 1 || src == dst) return CGS_ERR_ARG;
    const long long total = (long long)sx * sy * sz * nch;
    k_permute_samples<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float2*>(src), reinterpret_cast<float2*>(dst), sx, sy, sz, total);
    return cudaGetLastError() == cudaSuccess ? CGS_OK : CGS_ERR_CUDA;
}

int cgs_import_data_bin(const char* path, int32_t sx, int32_t sy, int32_t sz, int32_t nch, void* data_dev,
                        void* stream)
{
    if (!path || !data_dev || sx < 1 || sy < 1 || sz < 1 || nch < 1) return CGS_ERR_ARG;
    const size_t total = (size_t)sx * sy * sz * nch;
    const size_t bytes = total * sizeof(float2);
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return CGS_ERR_IO;
    cudaStream_t s = (cudaStream_t)stream;
    void* staging = nullptr;
    if (cudaMalloc(&staging, bytes) != cudaSuccess) {
        std::fclose(f);
        return CGS_ERR_NOMEM;
    }
    // two pinned chunks: the file is read into one while the other is copied
    const size_t chunk = std::min<size_t>(bytes, (size_t)32 << 20);
    PinnedBuf hb[2];
    cudaEvent_t done[2] = {nullptr, nullptr};
    int st = CGS_OK;
    if (!hb[0].ensure(chunk) || !hb[1].ensure(chunk)) st = CGS_ERR_NOMEM;
    for (int i = 0; i < 2 && st == CGS_OK; ++i)
        if (cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess) st = CGS_ERR_CUDA;
    size_t off = 0;
    int b = 0;
    while (st == CGS_OK && off < bytes) {
        const size_t n = std::min(chunk, bytes - off);
        if (cudaEventSynchronize(done[b]) != cudaSuccess) {   // the copy out of this buffer has finished
            st = CGS_ERR_CUDA;
            break;
        }
        if (std::fread(hb[b].p, 1, n, f) != n) {
            st = CGS_ERR_IO;   // short file (IO.cpp:68-74)
            break;
        }
        if (cudaMemcpyAsync(static_cast<char*>(staging) + off, hb[b].p, n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaEventRecord(done[b], s) != cudaSuccess) {
            st = CGS_ERR_CUDA;
            break;
        }
        off += n;
        b ^= 1;
    }
    std::fclose(f);
    if (st == CGS_OK) st = cgs_permute_samples_d(staging, data_dev, sx, sy, sz, nch, stream);
    if (cudaStreamSynchronize(s) != cudaSuccess && st == CGS_OK) st = CGS_ERR_CUDA;
    for (int i = 0; i < 2; ++i)
        if (done[i]) cudaEventDestroy(done[i]);
    cudaFree(staging);
    return st;
}

int cgs_export_complex_bin(const char* path, const void* src, int64_t n, int32_t on_device, void* stream)
{
    if (n < 0) return CGS_ERR_ARG;
    return export_bin(path, src, (size_t)n * sizeof(float2), on_device, stream, true);
}

int cgs_export_float_bin(const char* path, const void* src, int64_t n, int32_t on_device, void* stream)
{
    if (n < 0) return CGS_ERR_ARG;
    return export_bin(path, src, (size_t)n * sizeof(float), on_device, stream, false);
}

int cgs_import_smaps_bin(const char* dir, int64_t n, int32_t nch, float* maps)
{
    if (!dir || !maps || n < 0 || nch < 1) return CGS_ERR_ARG;
    for (int c = 0; c < nch; ++c) {
        const std::string name = std::string(dir) + "map" + std::to_string(c) + ".bin";
        std::FILE* f = std::fopen(name.c_str(), "rb");
        if (!f) return CGS_ERR_IO;
        const size_t want = (size_t)2 * n;
        const size_t got = std::fread(maps + (size_t)c * want, sizeof(float), want, f);
        std::fclose(f);
        if (got != want) return CGS_ERR_IO;
    }
    return CGS_OK;
}

int cgs_import_density_bin(const char* path, int64_t n, float* d)
{
    if (!path || !d || n < 0) return CGS_ERR_ARG;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return CGS_ERR_IO;
    const size_t got = std::fread(d, sizeof(float), (size_t)n, f);
    std::fclose(f);
    return got == (size_t)n ? CGS_OK : CGS_ERR_IO;
}

int cgs_rss_d(const void* imgs, int32_t nch, int64_t n, float* out, void* stream)
{
    if (!imgs || !out || nch < 1 || n < 0) return CGS_ERR_ARG;
    if (n == 0) return CGS_OK;
    k_rss<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2*>(imgs), nch,
                                                                         n, out);
    return cudaGetLastError() == cudaSuccess ? CGS_OK : CGS_ERR_CUDA;
}

}  // extern "C"
