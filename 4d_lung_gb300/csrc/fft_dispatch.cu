// fft_dispatch.cu -- runtime dispatch from a line length to its instantiated
// pass kernels.
#include "fft_sizes.h"
#include "launch.h"

namespace cgs {

#define CGS_DECLARE(L_, R1_, R2_, G_)                                                               \
    cudaError_t fft_strided_##L_(int sign, const StridedPassArgs& a, int A, int batch, cudaStream_t s); \
    cudaError_t fft_contig_##L_(int sign, const ContigPassArgs& a, int batch, cudaStream_t s);        \
    cudaError_t fft_fwd_z_##L_(const FwdZArgs& a, int batch, cudaStream_t s);                          \
    cudaError_t fft_adj_z_##L_(const AdjZArgs& a, int batch, cudaStream_t s);                          \
    int fft_adj_blocks_##L_(long long nl);                                                             \
    cudaError_t fft_init_##L_();                                                                       \
    cudaError_t fft_toep_x_##L_(const StridedPassArgs& a, const float* P, long long p_bs, int nsub, int batch, \
                                cudaStream_t s);                                                       \
    cudaError_t fft_spread_adjx_##L_(const SpreadAdjxArgs& a, bool kahan, cudaStream_t s);
CGS_FFT_SIZES(CGS_DECLARE)

static const int kSizes[] = {
#define CGS_LIST(L_, R1_, R2_, G_) L_,
    CGS_FFT_SIZES(CGS_LIST)
};

cudaError_t fft_init_all()
{
    cudaError_t e = cudaSuccess;
#define CGS_INIT(L_, R1_, R2_, G_) if (e == cudaSuccess) e = fft_init_##L_();
    CGS_FFT_SIZES(CGS_INIT)
#undef CGS_INIT
    return e;
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

bool encode_strided_map(CUtensorMap* map, const StridedPassArgs& a, int A, int batch, int TB, int* box_rows,
                        int promo)
{
    // TMA rows start on 16-byte boundaries: base pointer, row pitch and
    // strides must be multiples of 16 bytes (even element counts)
    if ((reinterpret_cast<uintptr_t>(a.in) & 15) || (a.B & 1) || a.Lin < 1) return false;
    const long long as = A > 1 ? a.in_as : (long long)a.Lin * a.B;
    const long long bs = batch > 1 ? a.in_bs : (long long)A * as;
    if ((as & 1) || (bs & 1)) return false;
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    int br = a.Lin;
    if (br > 256)
        for (br = 256; br > 1 && a.Lin % br != 0; --br) {
        }
    // each box of a stage lands on a 128-byte boundary
    if (br < a.Lin && ((long long)br * TB * 8) % 128 != 0) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)a.B, (cuuint64_t)a.Lin, (cuuint64_t)A, (cuuint64_t)batch};
    const cuuint64_t strides[3] = {(cuuint64_t)a.B * 8, (cuuint64_t)as * 8, (cuuint64_t)bs * 8};
    const cuuint32_t box[4] = {(cuuint32_t)TB, (cuuint32_t)br, 1, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUtensorMapL2promotion pr = promo <= 64    ? CU_TENSOR_MAP_L2_PROMOTION_L2_64B
                                      : promo <= 128 ? CU_TENSOR_MAP_L2_PROMOTION_L2_128B
                                                     : CU_TENSOR_MAP_L2_PROMOTION_L2_256B;
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<float2*>(a.in), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, pr, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    *box_rows = br;
    return true;
}

bool encode_spectrum_map(CUtensorMap* map, const float* P, long long B, int L, int nbins, int TB, int* box_rows)
{
    // rows of 4-byte elements: base and row pitch on 16-byte boundaries
    if ((reinterpret_cast<uintptr_t>(P) & 15) || (B & 3) || nbins < 1) return false;
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    int br = L;
    if (br > 256)
        for (br = 256; br > 1 && L % br != 0; --br) {
        }
    const cuuint64_t dims[3] = {(cuuint64_t)B, (cuuint64_t)L, (cuuint64_t)nbins};
    const cuuint64_t strides[2] = {(cuuint64_t)B * 4, (cuuint64_t)B * L * 4};
    const cuuint32_t box[3] = {(cuuint32_t)TB, (cuuint32_t)br, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(P), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    *box_rows = br;
    return true;
}

bool fft_supported(int L)
{
    for (int s : kSizes)
        if (s == L) return true;
    return false;
}

int fft_strided_cols(int L)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_strided_tile_cols(R1_, R2_);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return 0;
}

int fft_listed_cols(int L, int lo, int I)
{
    const bool half = 4 * lo == L && 2 * I == L;
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) \
    case L_: return half ? fft_listed_tile_cols(R1_, R2_) : fft_strided_tile_cols(R1_, R2_);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return 0;
}

const int* fft_supported_list(int* n)
{
    *n = (int)(sizeof(kSizes) / sizeof(kSizes[0]));
    return kSizes;
}

cudaError_t launch_strided(int L, int sign, const StridedPassArgs& a, int A, int batch, cudaStream_t s)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_strided_##L_(sign, a, A, batch, s);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_contig(int L, int sign, const ContigPassArgs& a, int batch, cudaStream_t s)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_contig_##L_(sign, a, batch, s);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_fwd_z(int L, const FwdZArgs& a, int batch, cudaStream_t s)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_fwd_z_##L_(a, batch, s);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return cudaErrorInvalidValue;
}

int adj_z_blocks(int L, long long nl)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_adj_blocks_##L_(nl);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return 0;
}

cudaError_t launch_adj_z(int L, const AdjZArgs& a, int batch, cudaStream_t s)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_adj_z_##L_(a, batch, s);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_toep_x(int L, const StridedPassArgs& a, const float* P, long long p_bs, int nsub, int batch,
                          cudaStream_t s)
{
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_toep_x_##L_(a, P, p_bs, nsub, batch, s);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return cudaErrorNotSupported;
}

cudaError_t launch_spread_adjx(int L, const SpreadAdjxArgs& a, bool kahan, cudaStream_t s)
{
    if (a.nj <= 0) return cudaSuccess;
    switch (L) {
#define CGS_CASE(L_, R1_, R2_, G_) case L_: return fft_spread_adjx_##L_(a, kahan, s);
        CGS_FFT_SIZES(CGS_CASE)
#undef CGS_CASE
    }
    return cudaErrorNotSupported;
}

}  // namespace cgs
