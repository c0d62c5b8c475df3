// gridding.cuh -- Kaiser-Bessel interpolation (gather) and spreading
// (scatter) between the non-Cartesian samples and the Cartesian grid.
//
// Kernel and tap set follow Reco::ConvKernel (Reco.h:218-242,
// Reco.cpp:698-806):
//   * sample k in [0,1]^3 sits at grid coordinate k*(N-1), dk = 1/(N-1);
//   * per axis the KB factor is I0(b*sqrt(1-(2d/(w dk))^2)) / (100 w dk) for
//     |d| <= w/2 dk, else 0; the 3-D weight is the product of the factors;
//   * a tap is kept when its weight exceeds thresh = KB(0,0,0) * 1e-7;
//   * taps outside [0, N-1] are dropped (no wrap-around).
// With w <= 5 every tap lies within +-2 cells of the nearest grid point
// (int)(k*(N-1) + 0.5), so each sample has 5 candidate factors per axis.
//
// The per-axis factors are computed once per trajectory into a 64-byte tap
// record per sample: 15 weights (0 for candidates outside the support or the
// grid) and the packed nearest grid point.
#pragma once
#include "cgs_common.cuh"
#include "cgs_types.h"
#include "gridding_common.cuh"

namespace cgs {



// ---------------------------------------------------------------------------
// Tap records.  sample_idx maps sorted position -> global sample index.
// The distance arithmetic follows Reco.cpp:763-771: double k minus the
// float product (index * float dk), then a float distance.
// ---------------------------------------------------------------------------
__global__ void k_tap_records(const double* __restrict__ k, const int* __restrict__ sample_idx,
                              long long n, KbParams kb, TapRecord* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long g = sample_idx ? sample_idx[i] : i;
    float wv[3][TAPS_1D];
    int nearest[3];
    const float wHalf = (float)(kb.w / 2.0);
    for (int a = 0; a < 3; ++a) {
        const int N = kb.G[a];
        const double ka = k[3 * g + a];
        const float dk = (float)(1.0 / (double)(float)(N - 1));
        int nr = (int)__dadd_rn(__dmul_rn((double)(N - 1), ka), 0.5);   // no FMA: matches the host
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
                    const double arg = (double)kb.b * sqrt(__dadd_rn(1.0, -__dmul_rn((double)q, (double)q)));
                    val = (float)(cyl_bessel_i0(arg) / (double)(float)(100.0f * kb.w * dk));
                }
            }
            wv[a][j] = val;
        }
    }
    TapRecord r;
    float* f = reinterpret_cast<float*>(&r);
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < TAPS_1D; ++j) f[a * TAPS_1D + j] = wv[a][j];
    f[15] = __uint_as_float(pack_nearest(nearest[0], nearest[1], nearest[2]));
    out[i] = r;
}

// ---------------------------------------------------------------------------
// Interpolation (Reco.cpp:539-550) fused with the density weights
// (Reco.cpp:243-254):  yv[i][c] = D[i] * sum_taps w * grid_c[idx]
// One thread per (sample, chunk of CC coils).  Grids are [coil][Ng]; the
// sample values are written coil-interleaved, yv[i][c].
// ---------------------------------------------------------------------------

template <int CC>
__global__ void __launch_bounds__(128) k_interp(InterpArgs a)
{
    const int bin = a.bin0 + blockIdx.z;
    const long long s0 = a.bin_off[bin], s1 = a.bin_off[bin + 1];
    // blockIdx.x = sample block * chunks + coil chunk: the chunks of a sample
    // block run side by side, so the blocks in flight cover a short run of
    // samples (a compact region of the grid) for all coils, which L2 holds
    const int nchunk = (a.nch + CC - 1) / CC;
    const int chunk = (int)(blockIdx.x % (unsigned)nchunk);
    const long long i = s0 + (long long)(blockIdx.x / (unsigned)nchunk) * blockDim.x + threadIdx.x;
    if (i >= s1) return;
    const int c0 = chunk * CC;
    const float2* grid = a.grid + (long long)blockIdx.z * a.grid_bs + (long long)c0 * a.coil_stride;
    float w[15];
    int nx, ny, nz;
    load_record(a.rec, i, w, nx, ny, nz);
    float2 acc[CC];
#pragma unroll
    for (int c = 0; c < CC; ++c) acc[c] = make_float2(0.f, 0.f);
    const int Gy = a.G[1], Gz = a.G[2];
    const int ncc = min(CC, a.nch - c0);
    // Rows of 5 z taps away from the z edges are read as three aligned
    // 16-byte loads (6 points from the even index at or below the row's
    // first); grids and coil planes start on 16-byte boundaries (Ng even).
    const bool vec = nz >= 3 && nz + 3 <= Gz - 1 && (a.coil_stride & 1) == 0 &&
                     (reinterpret_cast<uintptr_t>(a.grid) & 15) == 0 && (a.grid_bs & 1) == 0;
    // Interior samples whose x and y supports hold exactly four candidates
    // each (a kernel of width 4 away from the grid points and the grid's
    // faces): a 4 x 4 loop over the rows without a branch per row, so that
    // the loads of several rows can be in flight at once.  The rows, the
    // products wx * wy, the z taps and their order are those of the general
    // loop below, so the sums are bitwise the same.
    int x0 = 5, nxt = 0, y0 = 5, nyt = 0;
#pragma unroll
    for (int q = 4; q >= 0; --q) {
        if (w[q] != 0.f) x0 = q;
        if (w[5 + q] != 0.f) y0 = q;
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        nxt += w[q] != 0.f ? 1 : 0;
        nyt += w[5 + q] != 0.f ? 1 : 0;
    }
    if (vec && nxt == 4 && nyt == 4 && x0 <= 1 && y0 <= 1) {
        float wxs[4], wys[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            wxs[q] = x0 ? w[q + 1] : w[q];
            wys[q] = y0 ? w[6 + q] : w[5 + q];
        }
        const long long base = ((long long)(nx - 2 + x0) * Gy + (ny - 2 + y0)) * Gz + (nz - 2);
        const int odd = (int)(base & 1);   // Gz even: every row of the sample has this parity
        const float4* b4 = reinterpret_cast<const float4*>(grid + (base - odd));
        const long long gz4 = Gz / 2, gyz4 = (long long)Gy * Gz / 2;
#pragma unroll
        for (int ix = 0; ix < 4; ++ix)
#pragma unroll
            for (int iy = 0; iy < 4; ++iy) {
                const float wxy = wxs[ix] * wys[iy];
                const float4* r4 = b4 + ix * gyz4 + iy * gz4;
#pragma unroll
                for (int c = 0; c < CC; ++c)
                    if (c < ncc) {
                        const float4* p = r4 + (long long)c * (a.coil_stride / 2);
                        const float4 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2);
                        const float2 e[6] = {make_float2(q0.x, q0.y), make_float2(q0.z, q0.w), make_float2(q1.x, q1.y),
                                             make_float2(q1.z, q1.w), make_float2(q2.x, q2.y), make_float2(q2.z, q2.w)};
#pragma unroll
                        for (int jz = 0; jz < 5; ++jz) {
                            const float wz = w[10 + jz];
                            const float wt = wxy * wz;
                            if (wz != 0.f && wt > a.thresh) {
                                const float2 g = odd ? e[jz + 1] : e[jz];
                                acc[c].x = fmaf(g.x, wt, acc[c].x);
                                acc[c].y = fmaf(g.y, wt, acc[c].y);
                            }
                        }
                    }
            }
    } else {
#pragma unroll
    for (int jx = 0; jx < 5; ++jx) {
        const float wx = w[jx];
        if (wx == 0.f) continue;
        const int gx = nx - 2 + jx;
#pragma unroll
        for (int jy = 0; jy < 5; ++jy) {
            const float wxy = wx * w[5 + jy];
            if (wxy == 0.f) continue;
            const long long row = ((long long)gx * Gy + (ny - 2 + jy)) * Gz + (nz - 2);
            if (vec) {
                const int odd = (int)(row & 1);
                const float4* r4 = reinterpret_cast<const float4*>(grid + (row - odd));
#pragma unroll
                for (int c = 0; c < CC; ++c)
                    if (c < ncc) {
                        const float4* p = r4 + (long long)c * (a.coil_stride / 2);
                        const float4 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2);
                        const float2 e[6] = {make_float2(q0.x, q0.y), make_float2(q0.z, q0.w), make_float2(q1.x, q1.y),
                                             make_float2(q1.z, q1.w), make_float2(q2.x, q2.y), make_float2(q2.z, q2.w)};
#pragma unroll
                        for (int jz = 0; jz < 5; ++jz) {
                            const float wz = w[10 + jz];
                            const float wt = wxy * wz;
                            if (wz != 0.f && wt > a.thresh) {
                                const float2 g = odd ? e[jz + 1] : e[jz];
                                acc[c].x = fmaf(g.x, wt, acc[c].x);
                                acc[c].y = fmaf(g.y, wt, acc[c].y);
                            }
                        }
                    }
                continue;
            }
#pragma unroll
            for (int jz = 0; jz < 5; ++jz) {
                const float wz = w[10 + jz];
                const float wt = wxy * wz;
                if (wz != 0.f && wt > a.thresh) {   // wz != 0: the tap lies inside the grid
                    const long long idx = row + jz;
#pragma unroll
                    for (int c = 0; c < CC; ++c)
                        if (c < ncc) {
                            const float2 g = __ldg(grid + (long long)c * a.coil_stride + idx);
                            acc[c].x = fmaf(g.x, wt, acc[c].x);
                            acc[c].y = fmaf(g.y, wt, acc[c].y);
                        }
                }
            }
        }
    }
    }
    const float d = a.dcf ? a.dcf[i] : 1.f;
    float2* out = a.yv + i * a.nch + c0;
#pragma unroll
    for (int c = 0; c < CC; ++c)
        if (c < ncc) out[c] = cscale(acc[c], d);
}

// ---------------------------------------------------------------------------
// Spreading (Reco.cpp:492-504) without atomics.  One block owns one
// TILE_X x TILE_Y x TILE_Z tile of the grid for a chunk of coils.  The
// tile's list holds every sample whose support touches the tile, ordered by
// nearest x; the block stages it in batches.  Warp w owns the grid plane
// x = tile_x0 + w and walks only its run of the list (the samples whose x
// support covers the plane); lane l owns (y, z) offset (l / 5, l % 5) of the
// current sample.  Every grid value is therefore updated by one lane at a
// time in a fixed sample order: the result is deterministic.  The whole tile
// (zeros included) is then stored, so the grid needs no separate clearing.
// ---------------------------------------------------------------------------

constexpr int SPREAD_BATCH = 32;   // samples staged per round

// WPP warps share an x plane, each owning an equal part of the block's coils
// (so every grid value still has a single owning lane).  CCW: compile-time
// upper bound of the coils of one warp; the coil loop is unrolled so that the
// shared-memory loads, FMAs and stores of all its coils of one grid point
// issue back to back.
// KAHAN: compensated summation (the precision form): every accumulator has
// a compensation term (the low-order part lost by its last addition), and
// the stored value is sum - compensation.
constexpr int SPREAD_VAL_STRIDE = 12;   // staged values per sample (max coils per block)

template <int CCW, int WPP, bool KAHAN>
__global__ void __launch_bounds__(32 * TILE_X * WPP) k_spread(SpreadArgs a)
{
    constexpr int NT = 32 * TILE_X * WPP;
    static_assert(CCW * WPP <= SPREAD_VAL_STRIDE, "staged value row");
    extern __shared__ float4 s_dyn[];
    const int bin = a.bin0 + blockIdx.z;
    int tile = blockIdx.x;
    if (a.live) {   // only the listed tiles are stored; the rest of the grid is never read
        const long long o = a.live_off[bin];
        if ((long long)blockIdx.x >= a.live_off[bin + 1] - o) return;
        tile = a.live[o + blockIdx.x];
    }
    const int c0 = blockIdx.y * a.cc;
    const int ncc = min(a.cc, a.nch - c0);
    const int tz = tile % a.ntz;
    const int ty = (tile / a.ntz) % a.nty;
    const int tx = tile / (a.ntz * a.nty);
    const int x0 = tx * TILE_X, y0 = ty * TILE_Y, z0 = tz * TILE_Z;

    // shared: accumulators [cc][ACC_PTS] float2, then staged records and values
    float2* acc = reinterpret_cast<float2*>(s_dyn);
    float2* cmp = acc + (size_t)a.cc * ACC_PTS;   // compensation terms (KAHAN only)
    TapRecord* s_rec = reinterpret_cast<TapRecord*>(acc + (size_t)(KAHAN ? 2 : 1) * a.cc * ACC_PTS);
    float2* s_val = reinterpret_cast<float2*>(s_rec + SPREAD_BATCH);

    const int tid = threadIdx.x;
    {
        // ACC_PTS is even and both regions start 16-byte aligned: zero two points per store
        float4* a4 = reinterpret_cast<float4*>(acc);
        float4* c4 = reinterpret_cast<float4*>(cmp);
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int e = tid; e < ncc * (ACC_PTS / 2); e += NT) {
            a4[e] = z4;
            if (KAHAN) c4[e] = z4;
        }
    }

    const long long tp = a.tile_ptr_off[bin];
    const int beg = a.tile_ptr[tp + tile], end = a.tile_ptr[tp + tile + 1];
    const int* idx = a.tile_idx + a.tile_idx_off[bin];
    const long long sbase = a.bin_off[bin];
    const int warp = tid >> 5, lane = tid & 31;
    const int plane = warp % TILE_X, part = warp / TILE_X;
    const int per = (ncc + WPP - 1) / WPP;
    const int cb = part * per, nmy = min(per, ncc - cb);   // this warp's coils [cb, cb + nmy)
    const int gx = x0 + plane;
    const int jy = lane / 5, jz = lane - 5 * (lane / 5);
    const long long ntiles = (long long)a.ntx * a.nty * a.ntz;
    const int2 run = a.plane_rng[((long long)bin * ntiles + tile) * TILE_X + plane];

    for (int s = beg; s < end; s += SPREAD_BATCH) {
        const int nbat = min(SPREAD_BATCH, end - s);
        __syncthreads();
        for (int e = tid; e < nbat * 4; e += NT) {
            const long long si = sbase + idx[s + e / 4];
            reinterpret_cast<float4*>(s_rec)[e] = __ldg(reinterpret_cast<const float4*>(a.rec + si) + (e & 3));
        }
        for (int e = tid; e < nbat * ncc; e += NT) {
            const int j = e / ncc, c = e - j * ncc;
            const long long si = sbase + idx[s + j];
            s_val[j * SPREAD_VAL_STRIDE + c] = a.yv[si * a.nch + c0 + c];
        }
        __syncthreads();
        const int j0 = max(run.x - (s - beg), 0), j1 = min(run.y - (s - beg), nbat);
        if (lane < 25 && nmy > 0) {
            for (int j = j0; j < j1; ++j) {
                const float* w = reinterpret_cast<const float*>(&s_rec[j]);
                int nx, ny, nz;
                unpack_nearest(__float_as_uint(w[15]), nx, ny, nz);
                const int jx = gx - (nx - 2);
                if (jx < 0 || jx > 4) continue;
                const int gy = ny - 2 + jy, gz = nz - 2 + jz;
                if (gy < y0 || gy >= y0 + TILE_Y || gz < z0 || gz >= z0 + TILE_Z) continue;
                const float wxv = w[jx], wyv = w[5 + jy], wzv = w[10 + jz];
                const float wt = (wxv * wyv) * wzv;
                if (wxv == 0.f || wyv == 0.f || wzv == 0.f || !(wt > a.thresh)) continue;
                float2* pt = acc + (size_t)cb * ACC_PTS + (plane * TILE_Y + (gy - y0)) * TILE_ZP + (gz - z0);
                const float2* v = s_val + j * SPREAD_VAL_STRIDE + cb;
                float2 t[CCW], vv[CCW], e[CCW];
#pragma unroll
                for (int c = 0; c < CCW; ++c)
                    if (c < nmy) {
                        t[c] = pt[c * ACC_PTS];
                        vv[c] = v[c];
                        if (KAHAN) e[c] = pt[(size_t)a.cc * ACC_PTS + c * ACC_PTS];
                    }
#pragma unroll
                for (int c = 0; c < CCW; ++c)
                    if (c < nmy) {
                        if (KAHAN) {
                            // y = v w - e;  s = t + y;  e = (s - t) - y;  t = s
                            const float yx = fmaf(vv[c].x, wt, -e[c].x), yy = fmaf(vv[c].y, wt, -e[c].y);
                            const float sx = __fadd_rn(t[c].x, yx), sy = __fadd_rn(t[c].y, yy);
                            e[c].x = __fsub_rn(__fsub_rn(sx, t[c].x), yx);
                            e[c].y = __fsub_rn(__fsub_rn(sy, t[c].y), yy);
                            t[c] = make_float2(sx, sy);
                            pt[(size_t)a.cc * ACC_PTS + c * ACC_PTS] = e[c];
                        } else {
                            t[c].x = fmaf(vv[c].x, wt, t[c].x);
                            t[c].y = fmaf(vv[c].y, wt, t[c].y);
                        }
                        pt[c * ACC_PTS] = t[c];
                    }
            }
        }
    }
    __syncthreads();
    // store the tile: every thread keeps one (y, two-point z) position and
    // walks the coils and every other x plane; two points per 16-byte store
    // (a whole pair is in the grid when Gz is even)
    static_assert(TILE_Z % 2 == 0 && (TILE_Z & (TILE_Z - 1)) == 0 && (TILE_Y & (TILE_Y - 1)) == 0,
                  "tile sides must be powers of two");
    constexpr int ZH = TILE_Z / 2;
    constexpr int XSTEP = NT / (ZH * TILE_Y);
    static_assert(NT % (ZH * TILE_Y) == 0 && TILE_X % XSTEP == 0, "store mapping");
    float2* grid = a.grid + (long long)blockIdx.z * a.grid_bs + (long long)c0 * a.coil_stride;
    const int Gx = a.G[0], Gy = a.G[1], Gz = a.G[2];
    const bool pairs = (Gz % 2 == 0) && (reinterpret_cast<uintptr_t>(a.grid) & 15) == 0 && (a.coil_stride % 2 == 0) &&
                       (a.grid_bs % 2 == 0);
    const int zh = tid % ZH, ly = (tid / ZH) % TILE_Y, lx0 = tid / (ZH * TILE_Y);
    const int Y = y0 + ly, Z = z0 + 2 * zh;
    if (Y < Gy && Z < Gz) {
        for (int c = 0; c < ncc; ++c) {
            for (int lx = lx0; lx < TILE_X; lx += XSTEP) {
                const int X = x0 + lx;
                if (X >= Gx) break;
                const int q = c * ACC_PTS + (lx * TILE_Y + ly) * TILE_ZP + 2 * zh;
                float2 v0 = acc[q], v1 = acc[q + 1];
                if (KAHAN) {
                    v0 = make_float2(__fsub_rn(v0.x, cmp[q].x), __fsub_rn(v0.y, cmp[q].y));
                    v1 = make_float2(__fsub_rn(v1.x, cmp[q + 1].x), __fsub_rn(v1.y, cmp[q + 1].y));
                }
                float2* dst = grid + (long long)c * a.coil_stride + ((long long)X * Gy + Y) * Gz + Z;
                if (pairs) {
                    *reinterpret_cast<float4*>(dst) = make_float4(v0.x, v0.y, v1.x, v1.y);
                } else {
                    dst[0] = v0;
                    if (Z + 1 < Gz) dst[1] = v1;
                }
            }
        }
    }
}

// Spreading with shared-memory atomics (no fixed summation order, so not
// bitwise reproducible; chosen only for contexts that allow it): the warps
// of the block take the staged samples round-robin, and the lanes of a warp
// split the taps of one sample that fall inside the tile, so the sample's
// set-up is paid once per tile instead of once per x plane.
constexpr int SPREAD_ATOMIC_THREADS = 256;

template <int CC>
__global__ void __launch_bounds__(SPREAD_ATOMIC_THREADS) k_spread_atomic(SpreadArgs a)
{
    constexpr int NT = SPREAD_ATOMIC_THREADS, NW = NT / 32;
    static_assert(CC <= SPREAD_VAL_STRIDE, "staged value row");
    extern __shared__ float4 s_dyn[];
    const int bin = a.bin0 + blockIdx.z;
    int tile = blockIdx.x;
    if (a.live) {   // only the listed tiles are stored; the rest of the grid is never read
        const long long o = a.live_off[bin];
        if ((long long)blockIdx.x >= a.live_off[bin + 1] - o) return;
        tile = a.live[o + blockIdx.x];
    }
    const int c0 = blockIdx.y * a.cc;
    const int ncc = min(a.cc, a.nch - c0);
    const int tz = tile % a.ntz;
    const int ty = (tile / a.ntz) % a.nty;
    const int tx = tile / (a.ntz * a.nty);
    const int x0 = tx * TILE_X, y0 = ty * TILE_Y, z0 = tz * TILE_Z;
    float2* acc = reinterpret_cast<float2*>(s_dyn);
    TapRecord* s_rec = reinterpret_cast<TapRecord*>(acc + (size_t)a.cc * ACC_PTS);
    float2* s_val = reinterpret_cast<float2*>(s_rec + SPREAD_BATCH);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    {
        float4* a4 = reinterpret_cast<float4*>(acc);
        for (int e = tid; e < ncc * (ACC_PTS / 2); e += NT) a4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const long long tp = a.tile_ptr_off[bin];
    const int beg = a.tile_ptr[tp + tile], end = a.tile_ptr[tp + tile + 1];
    const int* idx = a.tile_idx + a.tile_idx_off[bin];
    const long long sbase = a.bin_off[bin];
    for (int s = beg; s < end; s += SPREAD_BATCH) {
        const int nbat = min(SPREAD_BATCH, end - s);
        __syncthreads();
        for (int e = tid; e < nbat * 4; e += NT) {
            const long long si = sbase + idx[s + e / 4];
            reinterpret_cast<float4*>(s_rec)[e] = __ldg(reinterpret_cast<const float4*>(a.rec + si) + (e & 3));
        }
        for (int e = tid; e < nbat * ncc; e += NT) {
            const int j = e / ncc, c = e - j * ncc;
            const long long si = sbase + idx[s + j];
            s_val[j * SPREAD_VAL_STRIDE + c] = a.yv[si * a.nch + c0 + c];
        }
        __syncthreads();
        for (int j = warp; j < nbat; j += NW) {
            const float* w = reinterpret_cast<const float*>(&s_rec[j]);
            int nx, ny, nz;
            unpack_nearest(__float_as_uint(w[15]), nx, ny, nz);
            const int xl = max(nx - 2, x0), xh = min(nx + 2, x0 + TILE_X - 1);
            const int yl = max(ny - 2, y0), yh = min(ny + 2, y0 + TILE_Y - 1);
            const int zl = max(nz - 2, z0), zh = min(nz + 2, z0 + TILE_Z - 1);
            if (xl > xh || yl > yh || zl > zh) continue;
            const int cy = yh - yl + 1, cz = zh - zl + 1;
            const int ntap = (xh - xl + 1) * cy * cz;
            const float2* v = s_val + j * SPREAD_VAL_STRIDE;
            for (int t = lane; t < ntap; t += 32) {
                const int ix = t / (cy * cz), r = t - ix * (cy * cz);
                const int iy = r / cz, iz = r - iy * cz;
                const int gx = xl + ix, gy = yl + iy, gz = zl + iz;
                const float wxv = w[gx - (nx - 2)], wyv = w[5 + gy - (ny - 2)], wzv = w[10 + gz - (nz - 2)];
                const float wt = (wxv * wyv) * wzv;
                if (wxv == 0.f || wyv == 0.f || wzv == 0.f || !(wt > a.thresh)) continue;
                float2* pt = acc + ((gx - x0) * TILE_Y + (gy - y0)) * TILE_ZP + (gz - z0);
#pragma unroll
                for (int c = 0; c < CC; ++c)
                    if (c < ncc) {
                        const float2 vv = v[c];
                        atomicAdd(&pt[c * ACC_PTS].x, vv.x * wt);
                        atomicAdd(&pt[c * ACC_PTS].y, vv.y * wt);
                    }
            }
        }
    }
    __syncthreads();
    constexpr int ZH = TILE_Z / 2;
    constexpr int XSTEP = NT / (ZH * TILE_Y);
    static_assert(NT % (ZH * TILE_Y) == 0 && TILE_X % XSTEP == 0, "store mapping");
    float2* grid = a.grid + (long long)blockIdx.z * a.grid_bs + (long long)c0 * a.coil_stride;
    const int Gx = a.G[0], Gy = a.G[1], Gz = a.G[2];
    const bool pairs = (Gz % 2 == 0) && (reinterpret_cast<uintptr_t>(a.grid) & 15) == 0 && (a.coil_stride % 2 == 0) &&
                       (a.grid_bs % 2 == 0);
    const int zq = tid % ZH, ly = (tid / ZH) % TILE_Y, lx0 = tid / (ZH * TILE_Y);
    const int Y = y0 + ly, Z = z0 + 2 * zq;
    if (Y < Gy && Z < Gz) {
        for (int c = 0; c < ncc; ++c) {
            for (int lx = lx0; lx < TILE_X; lx += XSTEP) {
                const int X = x0 + lx;
                if (X >= Gx) break;
                const int q = c * ACC_PTS + (lx * TILE_Y + ly) * TILE_ZP + 2 * zq;
                const float2 v0 = acc[q], v1 = acc[q + 1];
                float2* dst = grid + (long long)c * a.coil_stride + ((long long)X * Gy + Y) * Gz + Z;
                if (pairs) {
                    *reinterpret_cast<float4*>(dst) = make_float4(v0.x, v0.y, v1.x, v1.y);
                } else {
                    dst[0] = v0;
                    if (Z + 1 < Gz) dst[1] = v1;
                }
            }
        }
    }
}

// Persistent, software-pipelined spreading: every block walks work items
// (bin, coil chunk, tile) with stride gridDim.x; the loads of the next batch
// of samples (tile list entries, tap records, values -- the same or the next
// item) are issued into registers before the current batch is processed and
// written to the second shared-memory buffer after it, so their latency
// hides behind the work.  Ownership, summation order and results are those
// of k_spread<CCW, WPP, false>.
template <int CCW, int WPP>
__global__ void __launch_bounds__(32 * TILE_X * WPP) k_spread_pipe(SpreadArgs a, long long nitems, int nchunk)
{
    constexpr int NT = 32 * TILE_X * WPP;
    constexpr int SB = SPREAD_BATCH;
    constexpr int NREC = (SB * 4 + NT - 1) / NT;                       // float4 record pieces per thread
    constexpr int NVAL = (SB * SPREAD_VAL_STRIDE + NT - 1) / NT;      // values per thread
    static_assert(CCW * WPP <= SPREAD_VAL_STRIDE, "staged value row");
    extern __shared__ float4 s_dyn[];
    float2* acc = reinterpret_cast<float2*>(s_dyn);
    TapRecord* s_rec[2];
    float2* s_val[2];
    s_rec[0] = reinterpret_cast<TapRecord*>(acc + (size_t)a.cc * ACC_PTS);
    s_val[0] = reinterpret_cast<float2*>(s_rec[0] + SB);
    s_rec[1] = reinterpret_cast<TapRecord*>(s_val[0] + SB * SPREAD_VAL_STRIDE);
    s_val[1] = reinterpret_cast<float2*>(s_rec[1] + SB);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int plane = warp % TILE_X, part = warp / TILE_X;
    const int jy = lane / 5, jz = lane - 5 * (lane / 5);
    const int ntiles = a.ntx * a.nty * a.ntz;

    struct Item {
        int bin, c0, ncc, tile, beg, end, x0, y0, z0;
        long long sbase;
        const int* idx;
    };
    auto item_of = [&](long long it) {
        Item m;
        const int tile = (int)(it % ntiles);
        const long long r = it / ntiles;
        const int ch = (int)(r % nchunk);
        m.bin = a.bin0 + (int)(r / nchunk);
        m.tile = tile;
        m.c0 = ch * a.cc;
        m.ncc = min(a.cc, a.nch - m.c0);
        const long long tp = a.tile_ptr_off[m.bin];
        m.beg = a.tile_ptr[tp + tile];
        m.end = a.tile_ptr[tp + tile + 1];
        m.idx = a.tile_idx + a.tile_idx_off[m.bin];
        m.sbase = a.bin_off[m.bin];
        const int tz = tile % a.ntz, ty = (tile / a.ntz) % a.nty, tx = tile / (a.ntz * a.nty);
        m.x0 = tx * TILE_X;
        m.y0 = ty * TILE_Y;
        m.z0 = tz * TILE_Z;
        return m;
    };
    // registers of one prefetched batch
    float4 pr[NREC];
    float2 pv[NVAL];
    auto prefetch = [&](const Item& m, int s) {
        const int nbat = min(SB, m.end - s);
#pragma unroll
        for (int q = 0; q < NREC; ++q) {
            const int e = tid + q * NT;
            if (e < nbat * 4) {
                const long long si = m.sbase + m.idx[s + e / 4];
                pr[q] = __ldg(reinterpret_cast<const float4*>(a.rec + si) + (e & 3));
            }
        }
#pragma unroll
        for (int q = 0; q < NVAL; ++q) {
            const int e = tid + q * NT;
            if (e < nbat * m.ncc) {
                const int j = e / m.ncc, c = e - j * m.ncc;
                const long long si = m.sbase + m.idx[s + j];
                pv[q] = a.yv[si * a.nch + m.c0 + c];
            }
        }
    };
    auto commit = [&](const Item& m, int s, int buf) {
        const int nbat = min(SB, m.end - s);
#pragma unroll
        for (int q = 0; q < NREC; ++q) {
            const int e = tid + q * NT;
            if (e < nbat * 4) reinterpret_cast<float4*>(s_rec[buf])[e] = pr[q];
        }
#pragma unroll
        for (int q = 0; q < NVAL; ++q) {
            const int e = tid + q * NT;
            if (e < nbat * m.ncc) {
                const int j = e / m.ncc, c = e - j * m.ncc;
                s_val[buf][j * SPREAD_VAL_STRIDE + c] = pv[q];
            }
        }
    };
    auto zero_acc = [&](int ncc) {
        float4* a4 = reinterpret_cast<float4*>(acc);
        for (int e = tid; e < ncc * (ACC_PTS / 2); e += NT) a4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    };

    long long it = blockIdx.x;
    if (it >= nitems) return;
    Item cur = item_of(it);
    int s = cur.beg;       // first sample of the current batch
    int buf = 0;
    if (s < cur.end) {
        prefetch(cur, s);
        commit(cur, s, buf);
    }
    zero_acc(cur.ncc);
    __syncthreads();
    while (true) {
        // the batch after this one: the same item's next, or the next item's
        // first (an item without samples is stored as zeros when reached)
        long long it_n = it;
        Item nxt = cur;
        int s_n = s + SB;
        bool have_next = true;
        if (s_n >= cur.end) {
            it_n = it + gridDim.x;
            if (it_n >= nitems) {
                have_next = false;
            } else {
                nxt = item_of(it_n);
                s_n = nxt.beg;
            }
        }
        const bool next_in_item = have_next && it_n == it;
        const bool fetch = have_next && s_n < nxt.end;
        if (fetch) prefetch(nxt, s_n);
        // process the current batch
        if (s < cur.end) {
            const int nbat = min(SB, cur.end - s);
            const int per = (cur.ncc + WPP - 1) / WPP;
            const int cb = part * per, nmy = min(per, cur.ncc - cb);
            const int2 run = a.plane_rng[((long long)cur.bin * ntiles + cur.tile) * TILE_X + plane];
            const int j0 = max(run.x - (s - cur.beg), 0), j1 = min(run.y - (s - cur.beg), nbat);
            const int gx = cur.x0 + plane;
            if (lane < 25 && nmy > 0) {
                for (int j = j0; j < j1; ++j) {
                    const float* w = reinterpret_cast<const float*>(&s_rec[buf][j]);
                    int nx, ny, nz;
                    unpack_nearest(__float_as_uint(w[15]), nx, ny, nz);
                    const int jx = gx - (nx - 2);
                    if (jx < 0 || jx > 4) continue;
                    const int gy = ny - 2 + jy, gz = nz - 2 + jz;
                    if (gy < cur.y0 || gy >= cur.y0 + TILE_Y || gz < cur.z0 || gz >= cur.z0 + TILE_Z) continue;
                    const float wxv = w[jx], wyv = w[5 + jy], wzv = w[10 + jz];
                    const float wt = (wxv * wyv) * wzv;
                    if (wxv == 0.f || wyv == 0.f || wzv == 0.f || !(wt > a.thresh)) continue;
                    float2* pt = acc + (size_t)cb * ACC_PTS + (plane * TILE_Y + (gy - cur.y0)) * TILE_ZP + (gz - cur.z0);
                    const float2* v = s_val[buf] + j * SPREAD_VAL_STRIDE + cb;
                    float2 t[CCW], vv[CCW];
#pragma unroll
                    for (int c = 0; c < CCW; ++c)
                        if (c < nmy) {
                            t[c] = pt[c * ACC_PTS];
                            vv[c] = v[c];
                        }
#pragma unroll
                    for (int c = 0; c < CCW; ++c)
                        if (c < nmy) {
                            t[c].x = fmaf(vv[c].x, wt, t[c].x);
                            t[c].y = fmaf(vv[c].y, wt, t[c].y);
                            pt[c * ACC_PTS] = t[c];
                        }
                }
            }
        }
        __syncthreads();   // the batch is consumed; buffer buf ^ 1 is free
        if (fetch) commit(nxt, s_n, buf ^ 1);
        if (!next_in_item) {
            // store the finished tile (zeros included)
            constexpr int ZH = TILE_Z / 2;
            constexpr int XSTEP = NT / (ZH * TILE_Y);
            static_assert(NT % (ZH * TILE_Y) == 0 && TILE_X % XSTEP == 0, "store mapping");
            float2* grid = a.grid + (long long)(cur.bin - a.bin0) * a.grid_bs + (long long)cur.c0 * a.coil_stride;
            const int Gx = a.G[0], Gy = a.G[1], Gz = a.G[2];
            const bool pairs = (Gz % 2 == 0) && (reinterpret_cast<uintptr_t>(a.grid) & 15) == 0 &&
                               (a.coil_stride % 2 == 0) && (a.grid_bs % 2 == 0);
            const int zq = tid % ZH, ly = (tid / ZH) % TILE_Y, lx0 = tid / (ZH * TILE_Y);
            const int Y = cur.y0 + ly, Z = cur.z0 + 2 * zq;
            if (Y < Gy && Z < Gz) {
                for (int c = 0; c < cur.ncc; ++c) {
                    for (int lx = lx0; lx < TILE_X; lx += XSTEP) {
                        const int X = cur.x0 + lx;
                        if (X >= Gx) break;
                        const int q = c * ACC_PTS + (lx * TILE_Y + ly) * TILE_ZP + 2 * zq;
                        const float2 v0 = acc[q], v1 = acc[q + 1];
                        float2* dst = grid + (long long)c * a.coil_stride + ((long long)X * Gy + Y) * Gz + Z;
                        if (pairs) {
                            *reinterpret_cast<float4*>(dst) = make_float4(v0.x, v0.y, v1.x, v1.y);
                        } else {
                            dst[0] = v0;
                            if (Z + 1 < Gz) dst[1] = v1;
                        }
                    }
                }
            }
            if (!have_next) break;
            __syncthreads();   // the tile is read out before it is cleared
            zero_acc(nxt.ncc);
        }
        __syncthreads();
        cur = nxt;
        it = it_n;
        s = s_n;
        buf ^= 1;
    }
}

}  // namespace cgs
