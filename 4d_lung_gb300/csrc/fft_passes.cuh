// fft_passes.cuh -- one-axis passes of the centred 3-D FFT, with the
// coil / deapodisation / crop work of the NUFFT fused into the passes that
// touch the image.
//
// The reference's centred transform (Fourier.cpp:19-42) multiplies by
// (-1)^(i+j+k) before and after an unnormalised FFTW c2c transform.  The
// sign factor separates per axis, so every pass below multiplies its input
// by (-1)^l and its output by (-1)^l, l being the grid position along the
// pass axis.
//
// A line of length L = R1 * R2 is transformed in two register stages with
// one exchange through shared memory:
//   stage 1: thread n2 loads x[R2*n1 + n2] (n1 < R1), runs an R1-point DFT,
//            multiplies by W_L^(n2*k1) and stores Y[k1][n2];
//   stage 2: thread k1 loads Y[k1][n2] (n2 < R2), runs an R2-point DFT and
//            writes X[k1 + R1*k2].
// Global loads of stage 1 and stores of stage 2 are coalesced in both
// layouts: along the line for z passes, across the tile's columns otherwise.
//
// Pruning (zero-padded oversampled grid): a pass reads only the Lin stored
// input positions [in_off, in_off+Lin) of each line (the rest are zero) and
// writes only the Lout kept output positions [out_off, out_off+Lout).
#pragma once
#include "fft_codelets.cuh"
#include "cgs_types.h"
#include "ptx_async.cuh"
#include <cuda.h>

namespace cgs {

// Twiddle table tw[m] = exp(-2*pi*i*m/L), m < L; SIGN=+1 uses the conjugate.
template <int SIGN>
CGS_D float2 table_twiddle(float2 v, float2 w)
{
    if (SIGN < 0) return cmul(v, w);
    return cmulc(v, w);
}

CGS_D float2 parity(float2 v, int l) { return (l & 1) ? cneg(v) : v; }

// Block order of the z passes: block b of a launch over nbatch items (bins)
// is line block b / nbatch of item b % nbatch.  The blocks of one line block
// run side by side for every bin, so its coil-map tiles, which all bins
// share, come from DRAM once and from L2 for the other bins.
CGS_D int zp_item(int nbatch) { return (int)(blockIdx.x % (unsigned)nbatch); }
CGS_D long long zp_lblk(int nbatch) { return (long long)(blockIdx.x / (unsigned)nbatch); }

// Image value read by a forward z pass.  In a fused CG solve (a.cg set) the
// pass reads the search direction p and, while its bin has updates pending,
// first applies them: x = x + alpha p, p = r + beta p (Reco.cpp:285-290,
// 306-307); both are stored back.  Each image element is read by one thread
// of one block, so each update is applied once.
struct FwdZCg {
    bool upd;
    float ar, ai, br, bi;
};
CGS_D FwdZCg fwd_z_cg(const FwdZArgs& a, int item)
{
    FwdZCg u{false, 0.f, 0.f, 0.f, 0.f};
    if (a.cg) {
        const CgState& S = a.cg[item];
        if (S.active && S.xpend) {
            u.upd = true;
            u.ar = (float)S.alpha[0];
            u.ai = (float)S.alpha[1];
            u.br = (float)S.beta[0];
            u.bi = (float)S.beta[1];
        }
    }
    return u;
}

// Fused form of a thread's image reads: for each of its line positions the
// pending updates are applied and stored, and p * apod * parity is handed to
// `put`.  The loads of a group of positions are issued together before any
// of the group's stores (restrict-qualified pointers), so that the loads'
// latency is paid once per group.
// eb: element index of the line start within the batch.
constexpr int fwd_z_group(int r1) { return r1 % 8 == 0 ? 8 : (r1 % 4 == 0 ? 4 : (r1 % 2 == 0 ? 2 : 1)); }

template <int R1, int R2, class Put>
CGS_D void fwd_z_fused_line(const FwdZArgs& a, const FwdZCg& u, long long eb, int n2, float axy, Put put)
{
    constexpr int GRP = fwd_z_group(R1);
    float2* __restrict__ P = a.cg_p + eb;
    const float2* __restrict__ Rr = a.cg_r + eb;
    float2* __restrict__ X = a.cg_x + eb;
#pragma unroll
    for (int g0 = 0; g0 < R1; g0 += GRP) {
        float2 pv[GRP], rv[GRP], xv[GRP];
#pragma unroll
        for (int j = 0; j < GRP; ++j) {
            const int zi = R2 * (g0 + j) + n2 - a.lo_z;
            if (zi >= 0 && zi < a.Iz) {
                pv[j] = P[zi];
                rv[j] = Rr[zi];
                xv[j] = X[zi];
            }
        }
#pragma unroll
        for (int j = 0; j < GRP; ++j) {
            const int n1 = g0 + j;
            const int l = R2 * n1 + n2;
            const int zi = l - a.lo_z;
            if (zi >= 0 && zi < a.Iz) {
                X[zi] = cg_axpy(xv[j], u.ar, u.ai, pv[j]);
                const float2 p1 = cg_axpy(rv[j], u.br, u.bi, pv[j]);
                P[zi] = p1;
                put(n1, zi, parity(cscale(p1, axy * a.apz[zi]), l));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Strided pass: lines along a non-contiguous axis of an [A][Lrows][B] array.
// One block handles TB consecutive columns b of one outer index a.
// ---------------------------------------------------------------------------

template <int R1, int R2, int SIGN, int TB>
__global__ void __launch_bounds__(TB * (R1 > R2 ? R1 : R2))
k_fft_strided(StridedPassArgs a)
{
    constexpr int L = R1 * R2;
    __shared__ float2 s_tw[L];
    __shared__ float2 s_y[L * TB];
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += blockDim.x) s_tw[m] = a.tw[m];

    const int tile = blockIdx.x;
    const int ai = tile / a.ntb;
    const int b0 = (tile - ai * a.ntb) * TB;
    const int bi = tid % TB;
    const int b = b0 + bi;
    const bool bok = b < a.B;
    const float2* in = a.in + (long long)blockIdx.y * a.in_bs + (long long)ai * a.in_as + b;
    float2* out = a.out + (long long)blockIdx.y * a.out_bs + (long long)ai * a.out_as + b;

    __syncthreads();
    {
        const int n2 = tid / TB;
        if (n2 < R2) {
            float2 v[R1];
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) {
                const int l = R2 * n1 + n2;
                const int li = l - a.in_off;
                float2 x = make_float2(0.f, 0.f);
                if (bok && li >= 0 && li < a.Lin) x = parity(in[(long long)li * a.B], l);
                v[n1] = x;
            }
            Dft<R1, SIGN>::run(v);
#pragma unroll
            for (int k1 = 0; k1 < R1; ++k1) {
                float2 t = v[k1];
                if (k1 > 0) t = table_twiddle<SIGN>(t, s_tw[n2 * k1]);
                s_y[(k1 * R2 + n2) * TB + bi] = t;
            }
        }
    }
    __syncthreads();
    {
        const int k1 = tid / TB;
        if (k1 < R1) {
            float2 u[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2) u[n2] = s_y[(k1 * R2 + n2) * TB + bi];
            Dft<R2, SIGN>::run(u);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) {
                const int l = k1 + R1 * k2;
                const int lo = l - a.out_off;
                if (bok && lo >= 0 && lo < a.Lout) out[(long long)lo * a.B] = parity(u[k2], l);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// TMA-pipelined strided pass.  Persistent blocks walk the tiles (batch item,
// outer index, TB-column strip) round-robin.  A tile's Lin stored rows are
// one 4-D tensor-map box (or a few, each at most 256 rows) fetched by the TMA
// unit into shared memory, NSTAGE tiles ahead of the FFT, completion counted
// on an mbarrier.  The two register stages are those of k_fft_strided.
// Every wait is bounded (2 s); on a timeout the block sets *err, lets its
// issued copies land and exits.
// The tensor map views the input as [items][A][Lin][B] (B innermost) with a
// box of TB x box_rows x 1 x 1 elements of 8 bytes.
// ---------------------------------------------------------------------------
constexpr unsigned long long PIPE_WAIT_NS = 2000000000ull;

// Pruning modes of the strided pass, for a 2x oversampled axis with the
// image centred in the line (rows L/4 .. 3L/4):
//   PRUNE_NONE  any Lin / in_off / Lout / out_off (predicated rows);
//   PRUNE_IN    Lin = L/2 rows at in_off = L/4: stage 1 loads only the
//               n1 in [R1/4, 3R1/4) that hold them (compile-time range);
//   PRUNE_OUT   Lout = L/2 rows at out_off = L/4: stage 2 stores only the
//               k2 in [R2/4, 3R2/4) that land there.
constexpr int PRUNE_NONE = 0, PRUNE_IN = 1, PRUNE_OUT = 2;

template <int R1, int R2, int TB, int NSTAGE>
struct PipeLayout {
    static constexpr int L = R1 * R2;
    static constexpr int NT = TB * (R1 > R2 ? R1 : R2);
    // the stage exchange: rows of TB values; with 8-column tiles 8 float2 of
    // padding after every R2 rows, so that the 4 row groups k1 a warp reads
    // in stage 2 fall in different halves of the banks
    static constexpr int YP = TB == 8 ? 8 : 0;
    static constexpr int SY = L * TB + R1 * YP;
    // a pipeline stage: Lin rows of TB values, rounded up to 128 bytes so
    // that every stage starts on the 128-byte boundary a TMA destination needs
    __host__ __device__ static int stage_elems(int Lin) { return (Lin * TB + 15) & ~15; }
    // 128 bytes of slack to align the first stage (the tiles are not
    // swizzled); the twiddle table (R2 rows of R1 + 1 when signed)
    static size_t smem_bytes(int Lin)
    {
        return 128 + ((size_t)NSTAGE * stage_elems(Lin) + (size_t)SY + L + R2) * sizeof(float2) + NSTAGE * sizeof(uint64_t);
    }
};

// The centring signs (-1)^l of input row l = R2 n1 + n2 and output row
// l = k1 + R1 k2 are (-1)^n2 and (-1)^k1 when R1 and R2 are even: constant
// per stage-1 thread and per stage-2 row.  Both then fold into the stage-1
// twiddle W^(n2 k1) of thread n2 and row k1 (the passes are linear), and no
// element is negated on its own.
template <int R1, int R2>
struct SignFold {
    static constexpr bool value = (R1 % 2 == 0) && (R2 % 2 == 0);
};

// resident blocks the compiler must allow: 3 (input-pruned, L <= 320) or 2
// blocks of 256 threads, twice as many of 128 threads
template <int R1, int R2, int TB, int NSTAGE, int MODE>
constexpr int strided_tma_min_blocks()
{
    constexpr int NT = PipeLayout<R1, R2, TB, NSTAGE>::NT;
    return ((MODE == PRUNE_IN && R1 * R2 <= 320) ? 3 : 2) * (256 / NT > 1 ? 256 / NT : 1);
}

template <int R1, int R2, int SIGN, int TB, int NSTAGE, int MODE>
__global__ void __launch_bounds__(PipeLayout<R1, R2, TB, NSTAGE>::NT, strided_tma_min_blocks<R1, R2, TB, NSTAGE, MODE>())
k_fft_strided_tma(StridedPassArgs a, const __grid_constant__ CUtensorMap tmap, long long ntiles,
                  int tiles_per_item, int box_rows)
{
    constexpr int L = R1 * R2;
    constexpr int NT = PipeLayout<R1, R2, TB, NSTAGE>::NT;
    constexpr int YP = PipeLayout<R1, R2, TB, NSTAGE>::YP;
    constexpr bool FOLD = SignFold<R1, R2>::value;
    static_assert(MODE != PRUNE_IN || R1 % 4 == 0, "input pruning needs R1 % 4 == 0");
    static_assert(MODE != PRUNE_OUT || R2 % 4 == 0, "output pruning needs R2 % 4 == 0");
    extern __shared__ float4 s_pipe[];
    // 128-byte-aligned start, derived from the shared array itself so that
    // the compiler keeps shared-memory (not generic) loads and stores
    const uint32_t pad = (128u - (smem_addr(s_pipe) & 127u)) & 127u;
    const int stage_elems = PipeLayout<R1, R2, TB, NSTAGE>::stage_elems(a.Lin);
    float2* s_in = reinterpret_cast<float2*>(reinterpret_cast<char*>(s_pipe) + pad);
    float2* s_y = s_in + (size_t)NSTAGE * stage_elems;
    float2* s_tw = s_y + PipeLayout<R1, R2, TB, NSTAGE>::SY;   // W^m, or the signed table [n2][k1] when FOLD
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_tw + L + R2);
    __shared__ long long s_item[NSTAGE];   // per stage: the tile's batch item,
    __shared__ int2 s_ab[NSTAGE];          // outer index and first column,
    __shared__ long long s_rmb[NSTAGE];    // first row-mask word of its bin
    const int tid = threadIdx.x;
    // columns per row-mask tile: a power of two (8 or 16)
    const int rm_shift = a.sup_rowmask ? __ffs(a.sup_rowmask_tb) - 1 : 0;
    if (FOLD) {
        for (int m = tid; m < L; m += NT) {
            const int n2 = m / R1, k1 = m - n2 * R1;
            const float2 w = a.tw[n2 * k1];
            s_tw[n2 * (R1 + 1) + k1] = ((n2 + k1) & 1) ? cneg(w) : w;   // rows padded by one: no bank conflicts
        }
    } else {
        for (int m = tid; m < L; m += NT) s_tw[m] = a.tw[m];
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&s_bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long my_n = ntiles > (long long)blockIdx.x ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

    // tile t -> (batch item, outer index, first column)
    auto decode = [&](long long t, long long& item, int& ai, int& b0) {
        if (a.sup_tiles) {   // sub-item outer: blocks in flight share a coil plane
            const int sub = (int)(t / a.sup_ntiles);
            const long long j = t - (long long)sub * a.sup_ntiles;
            const int2 e = a.sup_tiles[j];
            item = (long long)(e.x - a.sup_bin0) * a.sup_nsub + sub;
            ai = 0;
            b0 = e.y;
        } else {
            item = t / tiles_per_item;
            const int rem = (int)(t - item * tiles_per_item);
            ai = rem / a.ntb;
            b0 = (rem - ai * a.ntb) * TB;
        }
    };

    auto issue = [&](long long k) {   // thread 0 only
        const long long t = blockIdx.x + k * gridDim.x;
        long long item;
        int ai, b0;
        decode(t, item, ai, b0);
        const int s = (int)(k % NSTAGE);
        // the tile's coordinates for the threads that transform it (read
        // after the barriers that follow the copy's completion)
        s_item[s] = item;
        s_ab[s] = make_int2(ai, b0);
        if (a.sup_rowmask) s_rmb[s] = (item / a.sup_nsub) * a.sup_rowmask_bs;
        mbar_arrive_expect_tx(&s_bar[s], (uint32_t)((size_t)a.Lin * TB * sizeof(float2)));   // the rows copied
        float2* dst = s_in + (size_t)s * stage_elems;
        for (int r0 = 0; r0 < a.Lin; r0 += box_rows)
            tma_load_4d(dst + (size_t)r0 * TB, &tmap, b0, r0, ai, (int)item, &s_bar[s]);
    };


    if (tid == 0)
        for (long long k = 0; k < NSTAGE - 1 && k < my_n; ++k) issue(k);
    for (long long k = 0; k < my_n; ++k) {
        const int s = (int)(k % NSTAGE);
        if (tid == 0 && k + NSTAGE - 1 < my_n) issue(k + NSTAGE - 1);
        const bool ok = mbar_wait_bounded(&s_bar[s], (uint32_t)((k / NSTAGE) & 1), PIPE_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            // timeout: report, let the copies already issued land, leave
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (long long j = k; j < my_n && j < k + NSTAGE; ++j)
                    mbar_wait_bounded(&s_bar[j % NSTAGE], (uint32_t)((j / NSTAGE) & 1), PIPE_WAIT_NS);
            }
            return;
        }
        // the tile's coordinates: from the issuing thread's arithmetic, or
        // read from the list (listed tiles; measured faster than the slots)
        long long item;
        int ai, b0;
        if (a.sup_tiles) {
            decode(blockIdx.x + k * gridDim.x, item, ai, b0);
        } else {
            item = s_item[s];
            ai = s_ab[s].x;
            b0 = s_ab[s].y;
        }
        const int bi = tid % TB;
        const int b = b0 + bi;
        const bool bok = b < a.B;
        const float2* sin_s = s_in + (size_t)s * stage_elems;
        {
            const int n2 = tid / TB;
            if (n2 < R2) {
                float2 v[R1];
                if constexpr (MODE == PRUNE_IN) {
                    // rows L/4 + R2 m + n2 (m = n1 - R1/4) of the line are the tile's rows
                    const float2* src = sin_s + n2 * TB + bi;
#pragma unroll
                    for (int n1 = 0; n1 < R1; ++n1) {
                        if (n1 >= R1 / 4 && n1 < 3 * R1 / 4) {
                            const float2 x = src[(R2 * (n1 - R1 / 4)) * TB];
                            v[n1] = FOLD ? x : parity(x, R2 * n1 + n2);
                        } else {
                            v[n1] = make_float2(0.f, 0.f);
                        }
                    }
                    DftMid<R1, SIGN>::run(v);
                } else {
#pragma unroll
                    for (int n1 = 0; n1 < R1; ++n1) {
                        const int l = R2 * n1 + n2;
                        const int li = l - a.in_off;
                        float2 x = make_float2(0.f, 0.f);
                        if (li >= 0 && li < a.Lin) x = sin_s[li * TB + bi];
                        v[n1] = FOLD ? x : parity(x, l);
                    }
                    Dft<R1, SIGN>::run(v);
                }
#pragma unroll
                for (int k1 = 0; k1 < R1; ++k1) {
                    float2 tv = v[k1];
                    if (FOLD) tv = table_twiddle<SIGN>(tv, s_tw[n2 * (R1 + 1) + k1]);
                    else if (k1 > 0) tv = table_twiddle<SIGN>(tv, s_tw[n2 * k1]);
                    s_y[(k1 * R2 + n2) * TB + bi + k1 * YP] = tv;
                }
            }
        }
        __syncthreads();
        {
            const int k1 = tid / TB;
            if (k1 < R1) {
                float2 u[R2];
#pragma unroll
                for (int n2 = 0; n2 < R2; ++n2) u[n2] = s_y[(k1 * R2 + n2) * TB + bi + k1 * YP];
                Dft<R2, SIGN>::run(u);
                float2* out = a.out + item * a.out_bs + (long long)ai * a.out_as + b;
                if constexpr (MODE == PRUNE_OUT) {
                    // output rows L/4 .. 3L/4: k2 in [R2/4, 3R2/4), row k1 + R1 (k2 - R2/4)
                    if (bok) {
                        float2* o = out + (long long)k1 * a.B;
                        const long long step = (long long)R1 * a.B;
#pragma unroll
                        for (int k2 = R2 / 4; k2 < 3 * R2 / 4; ++k2)
                            o[(k2 - R2 / 4) * step] = FOLD ? u[k2] : parity(u[k2], k1 + R1 * k2);
                    }
                } else {
                    // with a row mask (forward y pass): only the rows the x pass reads.  Row
                    // l = k1 + R1 k2 is bit (R1 k2 + k1) & 31 of word (R1 k2) / 32 when R1 is a
                    // power of two up to 32 (k1 < R1): compile-time words in registers
                    constexpr bool RM = (R1 & (R1 - 1)) == 0 && R1 <= 32 && L % 32 == 0;
                    bool done = false;
                    if constexpr (RM) {
                        if (a.sup_rowmask && a.out_off == 0 && a.Lout == L) {
                            // the x-pass tile of this thread's column (in range: b0 < B)
                            const unsigned* mw = a.sup_rowmask + s_rmb[s] +
                                                 (long long)((bok ? b : b0) >> rm_shift) * (L / 32);
                            unsigned rm[L / 32];
                            if constexpr ((L / 32) % 4 == 0) {
                                // 16-byte words: a bin's words and a tile's are multiples of 4
                                const uint4* mw4 = reinterpret_cast<const uint4*>(mw);
#pragma unroll
                                for (int q = 0; q < L / 128; ++q) {
                                    const uint4 v4 = __ldg(mw4 + q);
                                    rm[4 * q] = v4.x;
                                    rm[4 * q + 1] = v4.y;
                                    rm[4 * q + 2] = v4.z;
                                    rm[4 * q + 3] = v4.w;
                                }
                            } else {
#pragma unroll
                                for (int q = 0; q < L / 32; ++q) rm[q] = __ldg(mw + q);
                            }
#pragma unroll
                            for (int k2 = 0; k2 < R2; ++k2) {
                                const int l = k1 + R1 * k2;
                                if (bok && ((rm[(R1 * k2) / 32] >> (((R1 * k2) & 31) + k1)) & 1u))
                                    out[(long long)l * a.B] = FOLD ? u[k2] : parity(u[k2], l);
                            }
                            done = true;
                        }
                    }
                    if (!done) {
#pragma unroll
                        for (int k2 = 0; k2 < R2; ++k2) {
                            const int l = k1 + R1 * k2;
                            const int lo = l - a.out_off;
                            if (bok && lo >= 0 && lo < a.Lout) out[(long long)lo * a.B] = FOLD ? u[k2] : parity(u[k2], l);
                        }
                    }
                }
            }
        }
        // (the __syncthreads_or of the next wait would order the next stage 1
        // after this stage 2 as well; without this barrier the forward passes
        // measured 4-6 % slower)
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Toeplitz x stage, in place on the [items][Lin][B] buffer of the forward y
// pass: the forward x transform of a tile's L/2 stored rows (rows L/4 ..
// 3L/4 of the line), the product with the real spectrum P of the tile's bin,
// and the adjoint x transform of which the same L/2 rows are stored back.
//   stage 1: thread n2: R1-point DFT over n1 (rows R2 n1 + n2), W^(-n2 k1)
//            -> Y[k1][n2]
//   stage 2: thread k1: R2-point DFT over n2 -> X[k1 + R1 k2]; X *= P; the
//            R2-point inverse DFT over k2 -> Z[n2]; W^(+n2 k1) -> Y[k1][n2]
//            (the row it read)
//   stage 3: thread n2: R1-point inverse DFT over k1 -> row n2 + R2 n1
// The centring sign (-1)^k of the forward output and that of the adjoint
// input cancel; the rows keep theirs.  A pipeline stage holds the tile's
// rows (4-D map over the buffer) and its strip of P (3-D map [bins][L][B],
// 4-byte elements), both fetched by the TMA unit NSTAGE - 1 tiles ahead on
// one mbarrier.  Tiles t -> (sub-item t % nsub, column strip, bin): the nsub
// tiles of one strip run back to back, so that the strip of P they share
// comes from DRAM once.  Bounded waits and the timeout exit are those of
// k_fft_strided_tma.
// ---------------------------------------------------------------------------
template <int R1, int R2, int TB, int NSTAGE>
struct ToepLayout {
    static constexpr int L = R1 * R2;
    static constexpr int NT = TB * (R1 > R2 ? R1 : R2);
    static size_t smem_bytes(int Lin)
    {
        return 1024 + (size_t)NSTAGE * Lin * TB * sizeof(float2) + (size_t)NSTAGE * L * TB * sizeof(float) +
               (size_t)L * TB * sizeof(float2) + (size_t)L * sizeof(float2) + NSTAGE * sizeof(uint64_t);
    }
};

template <int R1, int R2, int TB, int NSTAGE>
__global__ void __launch_bounds__(ToepLayout<R1, R2, TB, NSTAGE>::NT, ToepLayout<R1, R2, TB, NSTAGE>::NT <= 128 ? 4 : 2)
k_toep_x_tma(StridedPassArgs a, int nsub, const __grid_constant__ CUtensorMap tmap,
             const __grid_constant__ CUtensorMap pmap, long long ntiles, int box_rows, int pbox_rows)
{
    constexpr int L = R1 * R2;
    constexpr int NT = ToepLayout<R1, R2, TB, NSTAGE>::NT;
    static_assert(R1 % 4 == 0, "the stored rows L/4 .. 3L/4 need R1 % 4 == 0");
    extern __shared__ float4 s_pipe[];
    const uint32_t pad = (1024u - (smem_addr(s_pipe) & 1023u)) & 1023u;   // as in k_fft_strided_tma
    const int stage_elems = a.Lin * TB;
    float2* s_in = reinterpret_cast<float2*>(reinterpret_cast<char*>(s_pipe) + pad);
    float* s_p = reinterpret_cast<float*>(s_in + (size_t)NSTAGE * stage_elems);
    float2* s_y = reinterpret_cast<float2*>(s_p + (size_t)NSTAGE * L * TB);
    float2* s_tw = s_y + L * TB;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_tw + L);
    __shared__ long long s_item[NSTAGE];   // per stage: the tile's batch item
    __shared__ int s_b0[NSTAGE];           // and first column (left by the issuing thread)
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += NT) s_tw[m] = a.tw[m];
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&s_bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long my_n = ntiles > (long long)blockIdx.x ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

    auto decode = [&](long long t, long long& item, long long& bin, int& b0) {
        const long long strip = t / nsub;
        const int sub = (int)(t - strip * nsub);
        bin = strip / a.ntb;
        b0 = (int)(strip - bin * a.ntb) * TB;
        item = bin * nsub + sub;
    };
    auto issue = [&](long long k) {   // thread 0 only
        const long long t = blockIdx.x + k * gridDim.x;
        long long item, bin;
        int b0;
        decode(t, item, bin, b0);
        const int s = (int)(k % NSTAGE);
        s_item[s] = item;
        s_b0[s] = b0;
        mbar_arrive_expect_tx(&s_bar[s], (uint32_t)(stage_elems * sizeof(float2) + L * TB * sizeof(float)));
        float2* dst = s_in + (size_t)s * stage_elems;
        for (int r0 = 0; r0 < a.Lin; r0 += box_rows)
            tma_load_4d(dst + (size_t)r0 * TB, &tmap, b0, r0, 0, (int)item, &s_bar[s]);
        float* pdst = s_p + (size_t)s * L * TB;
        for (int r0 = 0; r0 < L; r0 += pbox_rows) tma_load_3d(pdst + (size_t)r0 * TB, &pmap, b0, r0, (int)bin, &s_bar[s]);
    };

    if (tid == 0)
        for (long long k = 0; k < NSTAGE - 1 && k < my_n; ++k) issue(k);
    for (long long k = 0; k < my_n; ++k) {
        const int s = (int)(k % NSTAGE);
        if (tid == 0 && k + NSTAGE - 1 < my_n) issue(k + NSTAGE - 1);
        const bool ok = mbar_wait_bounded(&s_bar[s], (uint32_t)((k / NSTAGE) & 1), PIPE_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (long long j = k; j < my_n && j < k + NSTAGE; ++j)
                    mbar_wait_bounded(&s_bar[j % NSTAGE], (uint32_t)((j / NSTAGE) & 1), PIPE_WAIT_NS);
            }
            return;
        }
        // the tile's coordinates, as the issuing thread decoded them (no
        // per-thread 64-bit divisions)
        const long long item = s_item[s];
        const int b0 = s_b0[s];
        const int bi = tid % TB;
        const int b = b0 + bi;
        const bool bok = b < a.B;
        const float2* sin_s = s_in + (size_t)s * stage_elems;
        const float* sp = s_p + (size_t)s * L * TB;
        {
            const int n2 = tid / TB;
            if (n2 < R2) {
                float2 v[R1];
                const float2* src = sin_s + n2 * TB + bi;
#pragma unroll
                for (int n1 = 0; n1 < R1; ++n1) {
                    if (n1 >= R1 / 4 && n1 < 3 * R1 / 4)
                        v[n1] = parity(src[(R2 * (n1 - R1 / 4)) * TB], R2 * n1 + n2);
                    else
                        v[n1] = make_float2(0.f, 0.f);
                }
                DftMid<R1, -1>::run(v);
#pragma unroll
                for (int q = 0; q < R1; ++q) {
                    float2 tv = v[q];
                    if (q > 0) tv = table_twiddle<-1>(tv, s_tw[n2 * q]);
                    s_y[(q * R2 + n2) * TB + bi] = tv;
                }
            }
        }
        __syncthreads();
        const int k1 = tid / TB;
        float2 u[R2];
        if (k1 < R1) {
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2) u[n2] = s_y[(k1 * R2 + n2) * TB + bi];
            Dft<R2, -1>::run(u);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) {
                const float pv = sp[(k1 + R1 * k2) * TB + bi];
                u[k2].x *= pv;
                u[k2].y *= pv;
            }
            Dft<R2, +1>::run(u);
            // back into the positions this thread read (row k1): no other
            // thread touches them before the barrier
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2)
                s_y[(k1 * R2 + n2) * TB + bi] = n2 > 0 ? table_twiddle<+1>(u[n2], s_tw[n2 * k1]) : u[n2];
        }
        __syncthreads();
        {
            const int n2 = tid / TB;
            if (n2 < R2) {
                float2 w[R1];
#pragma unroll
                for (int q = 0; q < R1; ++q) w[q] = s_y[(q * R2 + n2) * TB + bi];
                Dft<R1, +1>::run(w);
                if (bok) {
                    float2* out = a.out + item * a.out_bs + b;
#pragma unroll
                    for (int n1 = R1 / 4; n1 < 3 * R1 / 4; ++n1)
                        out[(long long)(n2 + R2 * (n1 - R1 / 4)) * a.B] = parity(w[n1], n2 + R2 * n1);
                }
            }
        }
        // no barrier here: stage 3 of thread (n2, bi) read exactly the s_y
        // positions that its own stage 1 of the next tile writes, and the
        // stage refilled next was last read before the barrier above
    }
}

// ---------------------------------------------------------------------------
// Contiguous passes (z axis): LPB whole lines per block.
// Shared layout per line: Y[n2][k1] with an odd row pitch (conflict-free).
// ---------------------------------------------------------------------------
template <int R1, int R2>
struct ContigLayout {
    static constexpr int L = R1 * R2;
    static constexpr int R1P = R1 | 1;
    static constexpr int LINE = R2 * R1P;
    static constexpr int RMAX = R1 > R2 ? R1 : R2;
};

// Plain centred pass on contiguous lines: out[line][l] = F(in[line][.])

template <int R1, int R2, int SIGN, int LPB>
__global__ void __launch_bounds__(LPB * ContigLayout<R1, R2>::RMAX)
k_fft_contig(ContigPassArgs a)
{
    using Lay = ContigLayout<R1, R2>;
    constexpr int L = Lay::L;
    __shared__ float2 s_tw[L];
    __shared__ float2 s_y[LPB * Lay::LINE];
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += blockDim.x) s_tw[m] = a.tw[m];
    const long long line0 = (long long)blockIdx.x * LPB;
    const float2* in = a.in + (long long)blockIdx.y * a.in_bs;
    float2* out = a.out + (long long)blockIdx.y * a.out_bs;
    __syncthreads();
    {
        const int ln = tid / R2, n2 = tid % R2;
        const long long line = line0 + ln;
        if (ln < LPB && line < a.nl) {
            float2 v[R1];
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) {
                const int l = R2 * n1 + n2;
                const int li = l - a.in_off;
                float2 x = make_float2(0.f, 0.f);
                if (li >= 0 && li < a.Lin) x = parity(in[line * a.Lin + li], l);
                v[n1] = x;
            }
            Dft<R1, SIGN>::run(v);
#pragma unroll
            for (int k1 = 0; k1 < R1; ++k1) {
                float2 t = v[k1];
                if (k1 > 0) t = table_twiddle<SIGN>(t, s_tw[n2 * k1]);
                s_y[ln * Lay::LINE + n2 * Lay::R1P + k1] = t;
            }
        }
    }
    __syncthreads();
    {
        const int ln = tid / R1, k1 = tid % R1;
        const long long line = line0 + ln;
        if (ln < LPB && line < a.nl) {
            float2 u[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2) u[n2] = s_y[ln * Lay::LINE + n2 * Lay::R1P + k1];
            Dft<R2, SIGN>::run(u);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) {
                const int l = k1 + R1 * k2;
                const int lo = l - a.out_off;
                if (lo >= 0 && lo < a.Lout) out[line * a.Lout + lo] = parity(u[k2], l);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Forward z pass fused with the coil multiply, deapodisation and zero-pad
// (Reco.cpp:236-240 elementProduct, Reco.cpp:529-535 kernelFT multiply):
//   zbuf[c][line][l] = F_z( pad( x * S_c * apod ) ),  for all coils c.
// Lines are the Ix*Iy image (x, y) positions; their x/y apodisation factors
// and the x/y parities are applied here and in the later passes respectively.
// ---------------------------------------------------------------------------

template <int R1, int R2, int LPB, bool CGF>
__global__ void __launch_bounds__(LPB * ContigLayout<R1, R2>::RMAX)
k_fwd_z(FwdZArgs a)
{
    using Lay = ContigLayout<R1, R2>;
    constexpr int L = Lay::L;
    constexpr int SIGN = -1;
    __shared__ float2 s_tw[L];
    __shared__ float2 s_y[LPB * Lay::LINE];
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += blockDim.x) s_tw[m] = a.tw[m];
    const int item = zp_item(a.nbatch);
    const long long line0 = zp_lblk(a.nbatch) * LPB;
    float2* outb = a.out + (long long)item * a.out_bs;

    // stage-1 role
    const int ln1 = tid / R2, n2 = tid % R2;
    const long long line1 = line0 + ln1;
    const bool act1 = ln1 < LPB && line1 < a.nl;
    // image values times apodisation (reloaded per coil only for per-coil images)
    float2 xa[R1];
    float axy = 0.f;
    if (act1) {
        const int ix = (int)(line1 / a.Iy), iy = (int)(line1 - (long long)ix * a.Iy);
        axy = a.apx[ix] * a.apy[iy];
    }
    const int ln2 = tid / R1, k1 = tid % R1;
    const long long line2 = line0 + ln2;
    const bool act2 = ln2 < LPB && line2 < a.nl;
    const FwdZCg cg = CGF ? fwd_z_cg(a, item) : FwdZCg{false, 0.f, 0.f, 0.f, 0.f};

    for (int c = 0; c < a.nch; ++c) {
        __syncthreads();   // s_tw ready / previous coil's stage 2 finished
        if (act1) {
            if (c == 0 || a.x_cs != 0) {
                // a.cg is only set with x_cs == 0: each element is read once
                const long long eb = (long long)item * a.x_bs + (long long)c * a.x_cs + line1 * a.Iz;
                if (CGF && cg.upd) {
#pragma unroll
                    for (int n1 = 0; n1 < R1; ++n1) xa[n1] = make_float2(0.f, 0.f);
                    fwd_z_fused_line<R1, R2>(a, cg, eb, n2, axy, [&](int n1, int, float2 v) { xa[n1] = v; });
                } else {
                    const float2* xl = a.x + eb;
#pragma unroll
                    for (int n1 = 0; n1 < R1; ++n1) {
                        const int l = R2 * n1 + n2;
                        const int zi = l - a.lo_z;
                        float2 v = make_float2(0.f, 0.f);
                        if (zi >= 0 && zi < a.Iz) v = parity(cscale(xl[zi], axy * a.apz[zi]), l);
                        xa[n1] = v;
                    }
                }
            }
            float2 v[R1];
            if (a.smaps) {
                const float2* S = a.smaps + (long long)c * a.coil_in + line1 * a.Iz;
#pragma unroll
                for (int n1 = 0; n1 < R1; ++n1) {
                    const int zi = R2 * n1 + n2 - a.lo_z;
                    v[n1] = (zi >= 0 && zi < a.Iz) ? cmul(xa[n1], S[zi]) : make_float2(0.f, 0.f);
                }
            } else {
#pragma unroll
                for (int n1 = 0; n1 < R1; ++n1) v[n1] = xa[n1];
            }
            Dft<R1, SIGN>::run(v);
#pragma unroll
            for (int kk = 0; kk < R1; ++kk) {
                float2 t = v[kk];
                if (kk > 0) t = table_twiddle<SIGN>(t, s_tw[n2 * kk]);
                s_y[ln1 * Lay::LINE + n2 * Lay::R1P + kk] = t;
            }
        }
        __syncthreads();
        if (act2) {
            float2 u[R2];
#pragma unroll
            for (int m = 0; m < R2; ++m) u[m] = s_y[ln2 * Lay::LINE + m * Lay::R1P + k1];
            Dft<R2, SIGN>::run(u);
            float2* o = outb + (long long)c * a.coil_out + line2 * L;
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) {
                const int l = k1 + R1 * k2;
                o[l] = parity(u[k2], l);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint z pass fused with crop, deapodisation, rescale, conjugate coil
// multiply and the coil sum (Reco.cpp:509-517, 257-262; Fourier.cpp:31-41):
//   q[line][z] = scale * apod * sum_c conj(S_c) * F^H_z(zbuf[c][line])[z + lo_z]
// The coil sum is accumulated in registers in coil order (no atomics).
// When p != nullptr, the block also accumulates <p, q> = sum conj(p) q in
// double precision and writes it to partials[item][line block] (re, im).
// ---------------------------------------------------------------------------

template <int R1, int R2, int LPB>
__global__ void __launch_bounds__(LPB * ContigLayout<R1, R2>::RMAX)
k_adj_z(AdjZArgs a)
{
    using Lay = ContigLayout<R1, R2>;
    constexpr int L = Lay::L;
    constexpr int SIGN = +1;
    constexpr int NT = LPB * Lay::RMAX;
    __shared__ float2 s_tw[L];
    __shared__ float2 s_y[LPB * Lay::LINE];
    __shared__ double s_red[2][NT / 32];
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += blockDim.x) s_tw[m] = a.tw[m];
    const int item = zp_item(a.nbatch);
    const long long lblk = zp_lblk(a.nbatch);
    const long long line0 = lblk * LPB;
    const float2* inb = a.in + (long long)item * a.in_bs;
    float2* qb = a.q + (long long)item * a.q_bs;

    const int ln1 = tid / R2, n2 = tid % R2;
    const long long line1 = line0 + ln1;
    const bool act1 = ln1 < LPB && line1 < a.nl;
    const int ln2 = tid / R1, k1 = tid % R1;
    const long long line2 = line0 + ln2;
    const bool act2 = ln2 < LPB && line2 < a.nl;

    float2 acc[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) acc[k2] = make_float2(0.f, 0.f);

    for (int c = 0; c < a.nch; ++c) {
        __syncthreads();
        if (act1) {
            const float2* src = inb + (long long)c * a.coil_in + line1 * L;
            float2 v[R1];
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) {
                const int l = R2 * n1 + n2;
                v[n1] = parity(src[l], l);
            }
            Dft<R1, SIGN>::run(v);
#pragma unroll
            for (int kk = 0; kk < R1; ++kk) {
                float2 t = v[kk];
                if (kk > 0) t = table_twiddle<SIGN>(t, s_tw[n2 * kk]);
                s_y[ln1 * Lay::LINE + n2 * Lay::R1P + kk] = t;
            }
        }
        __syncthreads();
        if (act2) {
            float2 u[R2];
#pragma unroll
            for (int m = 0; m < R2; ++m) u[m] = s_y[ln2 * Lay::LINE + m * Lay::R1P + k1];
            Dft<R2, SIGN>::run(u);
            if (a.smaps) {
                const float2* S = a.smaps + (long long)c * a.coil_s + line2 * a.Iz;
#pragma unroll
                for (int k2 = 0; k2 < R2; ++k2) {
                    const int l = k1 + R1 * k2;
                    const int zi = l - a.lo_z;
                    if (zi >= 0 && zi < a.Iz) acc[k2] = cadd(acc[k2], cmulc(parity(u[k2], l), S[zi]));
                }
            } else {
                const int ix = (int)(line2 / a.Iy), iy = (int)(line2 - (long long)ix * a.Iy);
                const float sxy = a.scale * a.apx[ix] * a.apy[iy];
                float2* qc = qb + (long long)c * a.q_cs + line2 * a.Iz;
#pragma unroll
                for (int k2 = 0; k2 < R2; ++k2) {
                    const int l = k1 + R1 * k2;
                    const int zi = l - a.lo_z;
                    if (zi >= 0 && zi < a.Iz) qc[zi] = cscale(parity(u[k2], l), sxy * a.apz[zi]);
                }
            }
        }
    }
    if (!a.smaps) return;
    // <p, q>: FP32 products of the thread's R2 elements (as conjScalarProduct,
    // Reco.cpp:139-140, forms them), accumulated from here on in FP64
    double dre = 0.0, dim = 0.0;
    if (act2) {
        const int ix = (int)(line2 / a.Iy), iy = (int)(line2 - (long long)ix * a.Iy);
        const float sxy = a.scale * a.apx[ix] * a.apy[iy];
        float fre = 0.f, fim = 0.f;
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
            const int zi = k1 + R1 * k2 - a.lo_z;
            if (zi >= 0 && zi < a.Iz) {
                const float2 qv = cscale(acc[k2], sxy * a.apz[zi]);
                qb[line2 * a.Iz + zi] = qv;
                if (a.p) {
                    const float2 pv = a.p[(long long)item * a.q_bs + line2 * a.Iz + zi];
                    fre += pv.x * qv.x + pv.y * qv.y;
                    fim += pv.x * qv.y - pv.y * qv.x;
                }
            }
        }
        dre = (double)fre;
        dim = (double)fim;
    }
    if (a.p) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dre += __shfl_xor_sync(0xffffffffu, dre, o);
            dim += __shfl_xor_sync(0xffffffffu, dim, o);
        }
        if ((tid & 31) == 0) {
            s_red[0][tid >> 5] = dre;
            s_red[1][tid >> 5] = dim;
        }
        __syncthreads();
        if (tid == 0) {
            double r0 = 0.0, r1 = 0.0;
            for (int w = 0; w < NT / 32; ++w) {
                r0 += s_red[0][w];
                r1 += s_red[1][w];
            }
            double* out = a.partials + 2 * ((long long)item * (gridDim.x / a.nbatch) + lblk);
            out[0] = r0;
            out[1] = r1;
        }
    }
}

// ---------------------------------------------------------------------------
// Pipelined z passes.  The per-coil inputs of a block -- its LPB lines of the
// coil map S_c (forward and adjoint) and of the z-pass buffer (adjoint) --
// are contiguous, so each is one cp.async.bulk copy into a ring of NST
// shared-memory stages, NST - 1 coils ahead of the FFT.  Arithmetic and
// results are those of k_fwd_z / k_adj_z.  Every wait is bounded (2 s); on a
// timeout the block sets *err, lets its issued copies land and exits.
// Shared layout: [NST stages][bars][twiddles][exchange rows].
// ---------------------------------------------------------------------------
template <int R1, int R2, int LPB, int NST>
struct ZPipeLayout {
    using Lay = ContigLayout<R1, R2>;
    static constexpr int L = Lay::L;
    static constexpr int NT = LPB * Lay::RMAX;
    // elements of one stage: S tile (+ z-buffer tile for the adjoint)
    __host__ __device__ static size_t stage_elems(int Iz, bool adj) { return (size_t)LPB * Iz + (adj ? (size_t)LPB * L : 0); }
    // forward: the block's x * apod lines stay in shared memory across the coils
    // twiddles W^(n2 k1) as R2 rows of R1 + 1 (padded: a warp's rows in
    // different banks)
    static constexpr int TW = R2 * (R1 + 1);
    static size_t smem_bytes(int Iz, bool adj)
    {
        return (NST * stage_elems(Iz, adj) + TW + (size_t)LPB * Lay::LINE + (adj ? 0 : (size_t)LPB * Iz)) *
                   sizeof(float2) +
               16 * NST;
    }
};

// CGF: the fused CG form (a.cg set); a separate instantiation, so that the
// plain pass compiles without the update path.
template <int R1, int R2, int LPB, int NST, bool CGF>
__global__ void __launch_bounds__(LPB * ContigLayout<R1, R2>::RMAX, (R1 > 16 || R2 > 16) ? 2 : 3)
k_fwd_z_pipe(FwdZArgs a)
{
    using Lay = ContigLayout<R1, R2>;
    using ZL = ZPipeLayout<R1, R2, LPB, NST>;
    constexpr int L = Lay::L;
    constexpr int SIGN = -1;
    extern __shared__ float4 s_dyn[];
    const size_t se = ZL::stage_elems(a.Iz, false);
    float2* s_stage = reinterpret_cast<float2*>(s_dyn);
    float2* s_tw = s_stage + NST * se;      // [R2][R1 + 1]: W^(n2 k1)
    float2* s_y = s_tw + ZL::TW;
    float2* s_xa = s_y + LPB * Lay::LINE;   // x * apod * parity of the block's lines, [LPB][Iz]
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_xa + (size_t)LPB * a.Iz);
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += ZL::NT) {
        const int r = m / R1, q = m - r * R1;
        s_tw[r * (R1 + 1) + q] = a.tw[r * q];
    }
    const int item = zp_item(a.nbatch);
    const long long line0 = zp_lblk(a.nbatch) * LPB;
    const int rows = (int)min((long long)LPB, a.nl - line0);
    const uint32_t tile_bytes = (uint32_t)rows * (uint32_t)a.Iz * (uint32_t)sizeof(float2);
    const float2* Sb = a.smaps + line0 * a.Iz;
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) mbar_init(&s_bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int c) {   // thread 0 only
        const int st = c % NST;
        mbar_arrive_expect_tx(&s_bar[st], tile_bytes);
        bulk_load(s_stage + (size_t)st * se, Sb + (long long)c * a.coil_in, tile_bytes, &s_bar[st]);
    };
    if (tid == 0)
        for (int c = 0; c < NST - 1 && c < a.nch; ++c) issue(c);

    float2* outb = a.out + (long long)item * a.out_bs;
    const int ln1 = tid / R2, n2 = tid % R2;
    const long long line1 = line0 + ln1;
    const bool act1 = ln1 < LPB && line1 < a.nl;
    float2* xa = s_xa + (size_t)ln1 * a.Iz;   // written and read by this thread only
    if (act1) {
        const int ix = (int)(line1 / a.Iy), iy = (int)(line1 - (long long)ix * a.Iy);
        const float axy = a.apx[ix] * a.apy[iy];
        const FwdZCg cg = CGF ? fwd_z_cg(a, item) : FwdZCg{false, 0.f, 0.f, 0.f, 0.f};
        const long long eb = (long long)item * a.x_bs + line1 * a.Iz;
        if (CGF && cg.upd) {
            fwd_z_fused_line<R1, R2>(a, cg, eb, n2, axy, [&](int, int zi, float2 v) { xa[zi] = v; });
        } else {
            const float2* xl = a.x + eb;
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) {
                const int l = R2 * n1 + n2;
                const int zi = l - a.lo_z;
                if (zi >= 0 && zi < a.Iz) xa[zi] = parity(cscale(xl[zi], axy * a.apz[zi]), l);
            }
        }
    }
    const int ln2 = tid / R1, k1 = tid % R1;
    const long long line2 = line0 + ln2;
    const bool act2 = ln2 < LPB && line2 < a.nl;

    for (int c = 0; c < a.nch; ++c) {
        const int st = c % NST;
        // stage (c - 1) % NST was last read in stage 1 of coil c - 1, before
        // the barrier that followed it: it can be refilled now
        if (tid == 0 && c + NST - 1 < a.nch) issue(c + NST - 1);
        const bool ok = mbar_wait_bounded(&s_bar[st], (uint32_t)((c / NST) & 1), PIPE_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (int j = c; j < a.nch && j < c + NST; ++j)
                    mbar_wait_bounded(&s_bar[j % NST], (uint32_t)((j / NST) & 1), PIPE_WAIT_NS);
            }
            return;
        }
        if (act1) {
            const float2* S = s_stage + (size_t)st * se + ln1 * a.Iz;
            float2 v[R1];
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) {
                const int zi = R2 * n1 + n2 - a.lo_z;
                v[n1] = (zi >= 0 && zi < a.Iz) ? cmul(xa[zi], S[zi]) : make_float2(0.f, 0.f);
            }
            Dft<R1, SIGN>::run(v);
#pragma unroll
            for (int kk = 0; kk < R1; ++kk) {
                float2 t = v[kk];
                if (kk > 0) t = table_twiddle<SIGN>(t, s_tw[n2 * (R1 + 1) + kk]);
                s_y[ln1 * Lay::LINE + n2 * Lay::R1P + kk] = t;
            }
        }
        __syncthreads();
        if (act2) {
            float2 u[R2];
#pragma unroll
            for (int m = 0; m < R2; ++m) u[m] = s_y[ln2 * Lay::LINE + m * Lay::R1P + k1];
            Dft<R2, SIGN>::run(u);
            float2* o = outb + (long long)c * a.coil_out + line2 * L;
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) {
                const int l = k1 + R1 * k2;
                o[l] = parity(u[k2], l);
            }
        }
    }
}

template <int R1, int R2, int LPB, int NST>
__global__ void __launch_bounds__(LPB * ContigLayout<R1, R2>::RMAX)
k_adj_z_pipe(AdjZArgs a)
{
    using Lay = ContigLayout<R1, R2>;
    using ZL = ZPipeLayout<R1, R2, LPB, NST>;
    constexpr int L = Lay::L;
    constexpr int SIGN = +1;
    constexpr int NT = ZL::NT;
    extern __shared__ float4 s_dyn[];
    __shared__ double s_red[2][NT / 32];
    const size_t se = ZL::stage_elems(a.Iz, true);
    const size_t s_off = (size_t)LPB * L;   // S tile after the z-buffer tile
    float2* s_stage = reinterpret_cast<float2*>(s_dyn);
    float2* s_tw = s_stage + NST * se;      // [R2][R1 + 1]: W^(n2 k1)
    float2* s_y = s_tw + ZL::TW;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_y + LPB * Lay::LINE);
    const int tid = threadIdx.x;
    for (int m = tid; m < L; m += NT) {
        const int r = m / R1, q = m - r * R1;
        s_tw[r * (R1 + 1) + q] = a.tw[r * q];
    }
    const int item = zp_item(a.nbatch);
    const long long lblk = zp_lblk(a.nbatch);
    const long long line0 = lblk * LPB;
    const int rows = (int)min((long long)LPB, a.nl - line0);
    const uint32_t in_bytes = (uint32_t)rows * (uint32_t)L * (uint32_t)sizeof(float2);
    const uint32_t s_bytes = (uint32_t)rows * (uint32_t)a.Iz * (uint32_t)sizeof(float2);
    const float2* inb = a.in + (long long)item * a.in_bs + line0 * L;
    const float2* Sb = a.smaps + line0 * a.Iz;
    float2* qb = a.q + (long long)item * a.q_bs;
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) mbar_init(&s_bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int c) {   // thread 0 only
        const int st = c % NST;
        float2* dst = s_stage + (size_t)st * se;
        mbar_arrive_expect_tx(&s_bar[st], in_bytes + s_bytes);
        bulk_load(dst, inb + (long long)c * a.coil_in, in_bytes, &s_bar[st]);
        bulk_load(dst + s_off, Sb + (long long)c * a.coil_s, s_bytes, &s_bar[st]);
    };
    if (tid == 0)
        for (int c = 0; c < NST - 1 && c < a.nch; ++c) issue(c);

    const int ln1 = tid / R2, n2 = tid % R2;
    const long long line1 = line0 + ln1;
    const bool act1 = ln1 < LPB && line1 < a.nl;
    const int ln2 = tid / R1, k1 = tid % R1;
    const long long line2 = line0 + ln2;
    const bool act2 = ln2 < LPB && line2 < a.nl;

    float2 acc[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) acc[k2] = make_float2(0.f, 0.f);

    for (int c = 0; c < a.nch; ++c) {
        const int st = c % NST;
        // stage (c - 1) % NST is read up to stage 2 of coil c - 1
        __syncthreads();
        if (tid == 0 && c + NST - 1 < a.nch) issue(c + NST - 1);
        const bool ok = mbar_wait_bounded(&s_bar[st], (uint32_t)((c / NST) & 1), PIPE_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (int j = c; j < a.nch && j < c + NST; ++j)
                    mbar_wait_bounded(&s_bar[j % NST], (uint32_t)((j / NST) & 1), PIPE_WAIT_NS);
            }
            return;
        }
        const float2* tin = s_stage + (size_t)st * se;
        if (act1) {
            const float2* src = tin + ln1 * L;
            float2 v[R1];
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) {
                const int l = R2 * n1 + n2;
                v[n1] = parity(src[l], l);
            }
            Dft<R1, SIGN>::run(v);
#pragma unroll
            for (int kk = 0; kk < R1; ++kk) {
                float2 t = v[kk];
                if (kk > 0) t = table_twiddle<SIGN>(t, s_tw[n2 * (R1 + 1) + kk]);
                s_y[ln1 * Lay::LINE + n2 * Lay::R1P + kk] = t;
            }
        }
        __syncthreads();
        if (act2) {
            float2 u[R2];
#pragma unroll
            for (int m = 0; m < R2; ++m) u[m] = s_y[ln2 * Lay::LINE + m * Lay::R1P + k1];
            Dft<R2, SIGN>::run(u);
            const float2* S = tin + s_off + ln2 * a.Iz;
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) {
                const int l = k1 + R1 * k2;
                const int zi = l - a.lo_z;
                if (zi >= 0 && zi < a.Iz) acc[k2] = cadd(acc[k2], cmulc(parity(u[k2], l), S[zi]));
            }
        }
    }
    // <p, q>: FP32 products of the thread's R2 elements, accumulated in FP64
    double dre = 0.0, dim = 0.0;
    if (act2) {
        const int ix = (int)(line2 / a.Iy), iy = (int)(line2 - (long long)ix * a.Iy);
        const float sxy = a.scale * a.apx[ix] * a.apy[iy];
        float fre = 0.f, fim = 0.f;
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
            const int zi = k1 + R1 * k2 - a.lo_z;
            if (zi >= 0 && zi < a.Iz) {
                const float2 qv = cscale(acc[k2], sxy * a.apz[zi]);
                qb[line2 * a.Iz + zi] = qv;
                if (a.p) {
                    const float2 pv = a.p[(long long)item * a.q_bs + line2 * a.Iz + zi];
                    fre += pv.x * qv.x + pv.y * qv.y;
                    fim += pv.x * qv.y - pv.y * qv.x;
                }
            }
        }
        dre = (double)fre;
        dim = (double)fim;
    }
    if (a.p) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dre += __shfl_xor_sync(0xffffffffu, dre, o);
            dim += __shfl_xor_sync(0xffffffffu, dim, o);
        }
        if ((tid & 31) == 0) {
            s_red[0][tid >> 5] = dre;
            s_red[1][tid >> 5] = dim;
        }
        __syncthreads();
        if (tid == 0) {
            double r0 = 0.0, r1 = 0.0;
            for (int w = 0; w < NT / 32; ++w) {
                r0 += s_red[0][w];
                r1 += s_red[1][w];
            }
            double* out = a.partials + 2 * ((long long)item * (gridDim.x / a.nbatch) + lblk);
            out[0] = r0;
            out[1] = r1;
        }
    }
}

}  // namespace cgs
