// fft_sizes.h -- supported FFT line lengths and their two-stage split
// L = R1 * R2 (both register codelets).  X(L, R1, R2, GROUP): GROUP picks
// the translation unit that instantiates the size (parallel builds).
#pragma once
#define CGS_FFT_SIZES(X)                                                              \
    X(16, 4, 4, 0) X(20, 4, 5, 1) X(24, 4, 6, 2) X(32, 4, 8, 3) X(40, 8, 5, 4)        \
    X(48, 8, 6, 5) X(64, 8, 8, 0) X(80, 8, 10, 1) X(96, 8, 12, 2) X(128, 8, 16, 3)    \
    X(160, 16, 10, 4) X(176, 16, 11, 5) X(192, 16, 12, 0) X(224, 16, 14, 1)           \
    X(256, 16, 16, 2) X(320, 16, 20, 3) X(352, 32, 11, 4) X(384, 16, 24, 5)           \
    X(448, 16, 28, 0) X(512, 16, 32, 1)
#define CGS_FFT_NGROUPS 6

// columns per tile of the strided passes of a line length L = R1 * R2
constexpr int fft_strided_tile_cols(int r1, int r2) { return (r1 > r2 ? r1 : r2) > 16 ? 8 : 16; }
// columns per listed tile of the sample-support-pruned x passes (input-pruned
// forward, output-pruned adjoint; both need R1 and R2 multiples of 4): 8
// columns (64-byte rows), so that a listed tile carries fewer columns no
// sample reaches than a 16-column one
constexpr bool fft_has_narrow_tiles(int r1, int r2) { return r1 % 4 == 0 && r2 % 4 == 0; }
constexpr int fft_listed_tile_cols(int r1, int r2)
{
    return fft_has_narrow_tiles(r1, r2) ? 8 : fft_strided_tile_cols(r1, r2);
}

// spreading fused with the adjoint x pass (spread_adjx.cuh): threads per
// block, columns per tile (the x passes' narrow tiles)
constexpr int SAX_NT = 1024, SAX_TB = 8;
