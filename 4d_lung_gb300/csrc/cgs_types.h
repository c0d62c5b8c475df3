// cgs_types.h -- argument records and layout constants shared by the
// kernels (device side) and their launchers (host side).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgs {

// KB taps: 5 candidate grid points per axis (w < 5)
constexpr int TAPS_1D = 5;
// spreading tile (grid points) owned by one block
constexpr int TILE_X = 4, TILE_Y = 8, TILE_Z = 16;
constexpr int TILE_PTS = TILE_X * TILE_Y * TILE_Z;
// shared accumulator pitch along z: 16 + 5, so that the 5x5 (y, z) lanes of a
// sample fall on distinct 8-byte bank pairs (two wavefronts, no conflicts)
constexpr int TILE_ZP = TILE_Z + 5;
constexpr int ACC_PTS = TILE_X * TILE_Y * TILE_ZP;
constexpr int SPREAD_THREADS = 32 * TILE_X;
constexpr int RED_THREADS = 256;

struct CgState {
    double rr[2];      // <r, r> of the current residual
    double pq[2];      // <p, q>
    double alpha[2];
    double beta[2];
    double res;        // ||r||_2 after the last update
    double thresh;     // absolute residual threshold (Reco.cpp:230)
    int iter;          // completed iterations
    int max_iter;
    int active;        // 1 while the loop runs
    int error;         // 1: non-finite value detected (Reco.cpp:264-268)
    int xpend;         // fused solve: x += alpha p and p = r + beta p of the last
                       // iteration still to be applied (by the next forward z
                       // pass, or by the final x update once the loop stopped)
    int pad_;
};

struct StridedPassArgs {
    const float2* in;
    float2* out;
    long long in_bs, out_bs;   // batch strides (blockIdx.y)
    long long in_as, out_as;   // strides of the outer index a
    int B;                     // columns (contiguous extent)
    int ntb;                   // column tiles per outer index
    int Lin, in_off, Lout, out_off;
    const float2* tw;          // L twiddles
    int* err;                  // error flag of the pipelined pass (null: plain loads)
    // Sample-support pruning (pipelined pass only; the plain pass ignores it
    // and computes every tile, which is also correct): the pass visits only
    // the listed tiles {bin, first column} (outer index 0), each for every
    // sub-item (coil), sup_ntiles * sup_nsub tiles (tile t: sub-item
    // t / sup_ntiles, list entry t % sup_ntiles); batch item
    // (bin - sup_bin0) * sup_nsub + sub.
    const int2* sup_tiles;
    long long sup_ntiles;
    int sup_tb;                // columns per listed tile
    int sup_bin0, sup_nsub;
    // Forward y pass: only the rows that the x pass reads are stored.  Per
    // bin and x-pass tile of the row's column (column / sup_rowmask_tb),
    // L / 32 words of row bits; bin of item = item / sup_nsub, words per bin
    // sup_rowmask_bs.
    const unsigned* sup_rowmask;
    long long sup_rowmask_bs;
    int sup_rowmask_tb;
};

struct ContigPassArgs {
    const float2* in;
    float2* out;
    long long in_bs, out_bs;
    long long nl;              // lines per batch item
    int Lin, in_off, Lout, out_off;
    const float2* tw;
};

struct FwdZArgs {
    const float2* x;        // [nl][Iz]   image (one bin), or one image per coil
    long long x_cs;         // coil stride of x (0: one image shared by all coils)
    const float2* smaps;    // [nch][nl][Iz], or null (no coil multiply)
    const float* apx;       // [Ix]
    const float* apy;       // [Iy]
    const float* apz;       // [Iz]
    float2* out;            // [nch][nl][L]
    long long nl;
    int Iy, Iz, lo_z, nch;
    long long x_bs, out_bs; // batch strides (blockIdx.y: bins)
    long long coil_in, coil_out;  // coil strides of smaps and out
    const float2* tw;
    int* err;               // timeout flag of the pipelined variant (null: plain kernel)
    // Fused CG step: with cg set, the image read is the search direction p of
    // bin cg[blockIdx.y]; when that bin's xpend is set the pass first forms
    // p = r + beta p and x = x + alpha p (the previous iteration's updates,
    // Reco.cpp:285-290,306-307) and stores both.
    const CgState* cg;
    float2* cg_p;           // == x (stored back)
    const float2* cg_r;     // residual, same layout as x
    float2* cg_x;           // the solution, same layout as x
    int nbatch;             // batch items of the launch (set by the launcher; see zp_item)
};

struct AdjZArgs {
    const float2* in;       // [nch][nl][L]
    const float2* smaps;    // [nch][nl][Iz]; null: one output image per coil, no coil sum
    const float* apx;
    const float* apy;
    const float* apz;
    float scale;            // adj_scale / sqrt(Ng)
    float2* q;              // [nl][Iz]
    const float2* p;        // optional [nl][Iz]
    double* partials;       // [gridDim.y][gridDim.x][2]
    long long nl;
    int Iy, Iz, lo_z, nch;
    long long in_bs, q_bs;  // batch strides (bins)
    long long coil_in, coil_s;
    long long q_cs;         // coil stride of q when smaps is null
    const float2* tw;
    int* err;               // timeout flag of the pipelined variant (null: plain kernel)
    int nbatch;             // batch items of the launch (set by the launcher; see zp_item)
};

struct TapRecord {
    float4 q[4];   // w[0..14] = x(5) y(5) z(5); q[3].w holds the packed nearest point
};

struct KbParams {
    int G[3];          // grid size
    float w;           // KB width (cells)
    float b;           // KB shape
    float thresh;      // absolute tap threshold
};

struct InterpArgs {
    const float2* grid;        // coil c at grid + c*coil_stride (+ bin stride)
    long long coil_stride;
    long long grid_bs;         // bin stride of the grids (blockIdx.z)
    const TapRecord* rec;      // sorted tap records (all bins concatenated)
    const float* dcf;          // sorted density weights, or null
    const long long* bin_off;  // [nbins+1] sample offsets
    int bin0;                  // first bin of this launch
    float2* yv;                // [total samples][nch]
    int nch;
    int G[3];
    float thresh;
};

struct SpreadArgs {
    float2* grid;              // coil c at grid + c*coil_stride (+ bin stride)
    long long coil_stride;
    long long grid_bs;
    const TapRecord* rec;
    const float2* yv;          // [total samples][nch]
    const long long* bin_off;  // [nbins+1]
    const int* tile_ptr;       // per bin: [ntiles+1] offsets into tile_idx (relative to bin)
    const long long* tile_ptr_off;  // [nbins] start of each bin's tile_ptr array
    const long long* tile_idx_off;  // [nbins] start of each bin's tile_idx array
    const int* tile_idx;       // sample positions relative to the bin start, sorted by nearest x
    const int2* plane_rng;     // [nbins][ntiles][TILE_X]: entries of the tile's list whose
                               // x support covers plane x0 + p (relative to the list start)
    int bin0;
    int nch;
    int cc;                    // coils per block (chunk)
    int G[3];
    int ntx, nty, ntz;         // tiles per axis
    float thresh;
    // tiles to store (null: all): per bin the ascending tile indices
    // live[live_off[bin] ..< live_off[bin + 1]]; live_max = the longest list
    const int* live;
    const long long* live_off;
    int live_max;
};

// Spreading as a gather over the transposed tap matrix (spread_csr.cu).
// Grid points of the listed x-pass column tiles are numbered
//   p = (J * Gx + x) * tb + k,
// J the global index of a listed tile {bin, first column b0} (all bins'
// lists concatenated), x the grid row, k < tb the column within the tile
// (flattened (y, z) column b0 + k).  Row p of the matrix lists the
// (sorted sample, weight) pairs of the taps landing on point p.
struct CsrBuildArgs {
    const TapRecord* rec;      // sorted tap records (all bins)
    long long total;           // sorted samples
    const long long* bin_off;  // [nbins + 1]
    int nbins;
    const int* col_tile;       // [nbins][Gy * Gz]: listed tile J of a column, -1 if unlisted
    int G[3];
    int tb;                    // columns per listed tile
    float thresh;
    unsigned* cnt;             // [P] tap counts, then fill cursors
    const unsigned* ptr;       // [P + 1] row offsets (fill pass)
    int2* ent;                 // {sorted sample, weight bits} (fill pass)
    int* err;                  // set when a tap lands outside the listed columns
};

struct CsrSpreadArgs {
    float2* grid;              // coil c of bin slot s at grid + s * grid_bs + c * coil_stride
    long long coil_stride, grid_bs;
    const unsigned* ptr;       // [P + 1]
    const int2* ent;
    const float2* yv;          // [total samples][nch]
    const int2* tiles;         // listed tiles {bin, first column}, global index
    long long j0, nj;          // the tiles of this launch: [j0, j0 + nj)
    int bin0;                  // bin of workspace slot 0
    int nch;
    int Gx;
    long long B;               // Gy * Gz
    int tb;
    int cc;                    // coils per thread (2, 4, 6, 8; 0: by the coil count)
    int* err;                  // error flag (a bounded wait of the staged form ran out)
};

// Spreading fused with the adjoint x pass (spread_adjx.cuh): the gather of
// CsrSpreadArgs over listed tiles of 8 columns and Gx = L rows (grid and
// coil_stride unused), then the output-pruned x transform into the adjoint
// y pass's input: coil c of bin slot s at out + (s * nch + c) * out_bs, row
// l - L/4 of column b at (l - L/4) * B + b.
struct SpreadAdjxArgs {
    const unsigned* ptr;       // [P + 1] (+ 16-byte padding)
    const int2* ent;
    const float2* yv;          // [total samples][nch]
    const int2* tiles;         // listed tiles {bin, first column}, global index
    long long j0, nj;          // the tiles of this launch: [j0, j0 + nj)
    int bin0;                  // bin of workspace slot 0
    int nch;
    long long B;               // Gy * Gz
    int cc;                    // coils per block (2, 4, 6; 0: by the coil count)
    float2* out;
    long long out_bs;
    const float2* tw;          // L twiddles
    int* err;
};

// Toeplitz embedding (toeplitz.cu): the spectrum P of one bin's point-spread
// function, from sorted samples [s0, s0 + n).
struct ToepBuildArgs {
    const double* k;           // coordinates [ns][3] (global index)
    const int* sorted;         // sorted position -> global sample index
    const float* dcf;          // sorted density weights, or null
    long long s0, n;
    int G[3], I[3];
    double scale;              // adjoint scale / Ng
    float* P;                  // out: [Gx][Gy * Gz]
};

// Point-spread function of one bin by an adjoint NUFFT (toeplitz.cu): the
// density weights spread with a Kaiser-Bessel window of width w onto a fine
// grid nf (periodic, sample at nf nu + nf/2), accumulated in FP64.
constexpr int PSF_TAPS = 8;        // candidate points per axis (window width <= 7)
struct PsfSpreadArgs {
    const double* k;           // coordinates [ns][3] (global index)
    const int* sorted;         // sorted position -> global sample index
    const float* dcf;          // sorted density weights, or null
    long long s0, n;
    int G[3];                  // grid of the operator (defines nu)
    int nf[3];                 // fine grid
    double w, beta;            // window width and shape
    double* out;               // [nf0][nf1][nf2]
};

// Loss gradient pass (grad.cu): one bin's samples [s0, s0 + n) in sorted order.
struct InterpGradArgs {
    const float2* grid;        // coil c at grid + c * coil_stride (one bin)
    long long coil_stride;
    const TapRecord* rec;      // tap records (sorted order)
    const TapRecord* drec;     // derivative records (sorted order)
    const float2* ymeas;       // measured samples [sorted][nch]
    const float* dcf;          // sorted density weights, or null
    const int* sorted;         // sorted position -> global sample index
    long long s0, n;
    int nch;
    int G[3];
    float thresh;
    float2* rv;                // out: D r [sorted][nch], or null
    float* grad_k;             // out: [ns][3] by global index, or null
    double* partials;          // out: [blocks] loss partial sums
};

// Trajectory vector-Jacobian products of the operator (grad.cu): one bin's
// samples [s0, s0 + n) in sorted order; B = E S u and dB = dB/dk come from
// the grid of the current image u.
//   store mode (outA != null): outA = B, outdA = dB   [sorted][nch] / [sorted][nch][3]
//   contract mode: grad_k[g] += scale D_i Re sum_c (conj(B) dA + conj(dB) A)
//                  (dA may be null: a fixed first factor such as measured data)
struct PairGradArgs {
    const float2* grid;
    long long coil_stride;
    const TapRecord* rec;
    const TapRecord* drec;
    const float2* A;           // [sorted][nch]
    const float2* dA;          // [sorted][nch][3], or null
    float2* outA;              // store mode
    float2* outdA;
    const float* dcf;
    const int* sorted;
    long long s0, n;
    int nch;
    int G[3];
    float thresh;
    float scale;
    float* grad_k;             // [ns][3] by global index, accumulated
};

}  // namespace cgs
