// fft_noalloc.cu -- centred 3-D FFT for callers that cannot allocate device
// memory.
//
// Some callers run inside a host application that owns every byte of device
// memory through its own allocator (a fixed per-process budget, a pooled
// allocator that must see all allocations), or inside a latency-critical
// loop where a cudaMalloc/cudaFree and the device synchronisation they imply
// are not acceptable.  They can pass device buffers for the input and the
// output, but they cannot let the library allocate its temporary memory.
//
// cgs_fft3_noalloc therefore keeps the intermediate grid of the three
// one-axis passes (z pass: input -> scratch; y pass: scratch in place;
// x pass: scratch -> output) and the twiddle tables in file-scope device
// arrays of fixed size.  Those arrays are part of the library image: every
// GPU that loads the library holds them (4 MiB + 12 KiB) until the process
// exits.  Device code could name the arrays directly; host code only has a
// host-side stand-in for each symbol, so their device addresses are looked
// up with cudaGetSymbolAddress on the first call in each CUDA context (the
// device current, the module loaded there) and passed to the kernels.  The
// addresses are cached per device and context: a caller that switches
// between several contexts of one device gets each context's own copy of
// the arrays.
//
// in and out are read and written as float2, so both must be 8-byte
// aligned; a misaligned pointer is rejected before anything is launched (a
// misaligned access would end the caller's CUDA context).
//
// All calls share the same arrays and the arrays keep the last call's
// contents.  Nothing here relies on them starting at zero: the z pass writes
// every scratch element the later passes read, and each call rewrites the
// twiddles it uses.  Calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the arrays and corrupt each
// other's results; serialise them.
#include "cgsense_c.h"
#include "launch.h"

#include <cstdio>
#include <mutex>
#include <string>

using namespace cgs;

// Largest grid (points) this entry point accepts: 2^19 complex values, e.g.
// 64 x 64 x 128 or 80 x 80 x 80.
#define CGS_FFT_NOALLOC_MAX_POINTS (1 << 19)
#define CGS_FFT_NOALLOC_MAX_LINE 512

static __device__ __align__(256) float2 g_noalloc_scratch[CGS_FFT_NOALLOC_MAX_POINTS];
static __device__ __align__(256) float2 g_noalloc_twiddles[3 * CGS_FFT_NOALLOC_MAX_LINE];

namespace {

struct NoallocSymbols {
    void* ctx = nullptr;        // the CUDA context the addresses belong to
    float2* scratch = nullptr;
    float2* twiddles = nullptr;
};

constexpr int kMaxDevices = 64;
std::mutex g_symbols_mutex;
NoallocSymbols g_symbols[kMaxDevices];

// cuCtxGetCurrent from the driver (no link-time dependency on libcuda)
typedef int (*CtxGetCurrentFn)(void**);

void* current_context()
{
    static CtxGetCurrentFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    void* ctx = nullptr;
    if (fn && fn(&ctx) != 0) ctx = nullptr;
    return ctx;
}
// There is no context to hold a message: errors go to stderr with the code.
int noalloc_fail(int code, const std::string& msg)
{
    std::fprintf(stderr, "cgs_fft3_noalloc: %s\n", msg.c_str());
    return code;
}

// tw[m] = exp(-2 pi i m / L), computed in double and rounded to float
__global__ void k_noalloc_twiddles(float2* tw, int L)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= L) return;
    double s, c;
    sincospi(-2.0 * (double)m / (double)L, &s, &c);
    tw[m] = make_float2((float)c, (float)s);
}

}  // namespace

extern "C" int cgs_fft3_noalloc(const float* in, float* out, const int32_t* grid, int32_t sign, void* stream)
{
    if (!in || !out || !grid) return noalloc_fail(CGS_ERR_ARG, "null pointer");
    if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 7)
        return noalloc_fail(CGS_ERR_ARG, "in and out must be 8-byte aligned (complex float values)");
    if (sign != -1 && sign != 1) return noalloc_fail(CGS_ERR_ARG, "sign must be -1 or +1");
    long long n = 1;
    for (int a = 0; a < 3; ++a) {
        if (grid[a] < 2 || (grid[a] & 1)) return noalloc_fail(CGS_ERR_ARG, "grid sizes must be even");
        if (!fft_supported(grid[a]))
            return noalloc_fail(CGS_ERR_UNSUPPORTED, "grid size " + std::to_string(grid[a]) + " has no FFT kernel");
        n *= grid[a];
    }
    if (n > CGS_FFT_NOALLOC_MAX_POINTS)
        return noalloc_fail(CGS_ERR_ARG, "grid of " + std::to_string(n) + " points exceeds the fixed scratch of " +
                                             std::to_string(CGS_FFT_NOALLOC_MAX_POINTS) + " points");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(CGS_ERR_CUDA, "no current CUDA device");
    void* ctx = current_context();   // null before the runtime has made a context current
    NoallocSymbols sym;
    {
        std::lock_guard<std::mutex> lock(g_symbols_mutex);
        if (!g_symbols[dev].scratch || g_symbols[dev].ctx != ctx) {
            // once per device and context, with that device current: device
            // addresses of the file-scope arrays (the host names are only
            // stand-ins)
            void* s = nullptr;
            void* t = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&s, g_noalloc_scratch);
            if (e != cudaSuccess) return noalloc_fail(CGS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            e = cudaGetSymbolAddress(&t, g_noalloc_twiddles);
            if (e != cudaSuccess) return noalloc_fail(CGS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_symbols[dev].ctx = current_context();   // the lookup made the primary context current
            g_symbols[dev].scratch = reinterpret_cast<float2*>(s);
            g_symbols[dev].twiddles = reinterpret_cast<float2*>(t);
        }
        sym = g_symbols[dev];
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int Gx = grid[0], Gy = grid[1], Gz = grid[2];
    for (int a = 0; a < 3; ++a) {
        k_noalloc_twiddles<<<(grid[a] + 127) / 128, 128, 0, st>>>(sym.twiddles + a * CGS_FFT_NOALLOC_MAX_LINE, grid[a]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return noalloc_fail(CGS_ERR_CUDA, cudaGetErrorString(e));
    }
    // z pass: input -> scratch
    ContigPassArgs cz{};
    cz.in = reinterpret_cast<const float2*>(in);
    cz.out = sym.scratch;
    cz.nl = (long long)Gx * Gy;
    cz.Lin = cz.Lout = Gz;
    cz.tw = sym.twiddles + 2 * CGS_FFT_NOALLOC_MAX_LINE;
    cudaError_t e = launch_contig(Gz, sign, cz, 1, st);
    // y pass: scratch in place
    StridedPassArgs sy{};
    sy.in = sym.scratch;
    sy.out = sym.scratch;
    sy.in_as = sy.out_as = (long long)Gy * Gz;
    sy.B = Gz;
    sy.Lin = sy.Lout = Gy;
    sy.tw = sym.twiddles + CGS_FFT_NOALLOC_MAX_LINE;
    if (e == cudaSuccess) e = launch_strided(Gy, sign, sy, Gx, 1, st);
    // x pass: scratch -> output
    StridedPassArgs sx{};
    sx.in = sym.scratch;
    sx.out = reinterpret_cast<float2*>(out);
    sx.B = Gy * Gz;
    sx.Lin = sx.Lout = Gx;
    sx.tw = sym.twiddles;
    if (e == cudaSuccess) e = launch_strided(Gx, sign, sx, 1, 1, st);
    if (e != cudaSuccess) return noalloc_fail(CGS_ERR_CUDA, cudaGetErrorString(e));
    return CGS_OK;
}
