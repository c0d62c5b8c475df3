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
    cudaError_t fft_init_##L_();
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

bool fft_supported(int L)
{
    for (int s : kSizes)
        if (s == L) return true;
    return false;
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

}  // namespace cgs
