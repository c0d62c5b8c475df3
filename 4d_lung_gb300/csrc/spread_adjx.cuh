// spread_adjx.cuh -- spreading (Reco.cpp:492-504) fused with the adjoint x
// pass of the centred FFT (Fourier.cpp:19-42, sign +1): the grid never goes
// to memory.
//
// Work unit: one listed x-pass tile (8 consecutive (y, z) columns, all Gx
// x rows) of one bin, for one chunk of CC coils.  The block
//   1. gathers every point of the tile over the transposed tap matrix, as
//      k_spread_csr_staged does (the unit's row offsets, and its taps when
//      they fit, staged in shared memory by bulk copies a unit ahead, the
//      sample values read from L2; the same sums in the same order), into
//      shared memory;
//   2. runs the x transform of the tile's 8 x CC lines in place there: the
//      stage-1 R1-point codelets with their twiddles (each thread's rows are
//      read and written by that thread alone), one barrier, the stage-2
//      R2-point codelets, of which only the output rows L/4 .. 3L/4 that
//      the crop keeps are stored -- k_fft_strided_tma's output-pruned form,
//      the same operations on the same values.
// So the adjoint y pass's input equals that of the unfused spreading + x
// pass bit for bit, and the grid's store and reload (16 bytes per point and
// coil) are gone.  One block of SAX_NT threads per SM (the unit's lines take
// most of its shared memory): 32 warps for the gather's dependent loads,
// three barriers per unit.  Every wait is bounded: on a timeout the block
// sets the error flag, lets its issued copies land and leaves.
#pragma once
#include "fft_sizes.h"
#include "fft_passes.cuh"

namespace cgs {

constexpr int SAX_NST = 2;        // pipeline stages of the matrix copies
constexpr unsigned long long SAX_WAIT_NS = 2000000000ull;

template <int R1, int R2, int CC>
struct SaxLayout {
    static constexpr int L = R1 * R2;
    static constexpr int PTS = L * SAX_TB;              // points of a unit
    static constexpr int PS = ((PTS + 1) + 3) & ~3;     // staged row offsets per stage
    // a coil's lines in shared memory: 8 float2 of padding after every 16
    // rows of the 8 columns, so that the 4 row groups a warp reads in the
    // transform's stage 2 fall in different halves of the banks
    static constexpr int GS = PTS + PTS / 16;
    static constexpr long long fixed = (long long)SAX_NST * PS * sizeof(unsigned) +
                                       (long long)CC * GS * sizeof(float2) + (long long)(L + R2) * sizeof(float2) +
                                       SAX_NST * sizeof(uint64_t);
    // staged taps per stage: what the 227 KiB of a block's shared memory
    // leave (at most 8192, an even count; 0: never staged)
    static constexpr long long room = (232448 - fixed) / (long long)(SAX_NST * sizeof(int2));
    static constexpr int CAP = room >= 8192 ? 8192 : room >= 2 ? (int)(room & ~1LL) : 0;
    static constexpr size_t bytes = (size_t)SAX_NST * CAP * sizeof(int2) + (size_t)fixed;
};

template <int R1, int R2, int CC, bool KAHAN>
__global__ void __launch_bounds__(SAX_NT, 1) k_spread_adjx(SpreadAdjxArgs a, int nunits)
{
    constexpr int L = R1 * R2, TB = SAX_TB;
    using Lay = SaxLayout<R1, R2, CC>;
    constexpr int PTS = Lay::PTS, PS = Lay::PS, CAP = Lay::CAP, GS = Lay::GS;
    // shared-memory position of row l, column bi of a coil's lines
    auto gi = [](int l, int bi) { return l * TB + bi + (l >> 4) * TB; };
    constexpr bool FOLD = SignFold<R1, R2>::value;
    constexpr int MR = R1 > R2 ? R1 : R2;
    constexpr int TPC = TB * MR;                               // transform threads per coil
    constexpr int CPP = SAX_NT / TPC;                          // coils per transform pass
    static_assert(CPP >= 1, "one coil's lines fit a block");
    static_assert(R2 % 4 == 0, "output pruning needs R2 % 4 == 0");
    static_assert(CC % 2 == 0, "sample values are read as coil pairs");
    extern __shared__ float4 s_sax[];
    int2* s_ent = reinterpret_cast<int2*>(s_sax);                             // [SAX_NST][CAP]
    unsigned* s_ptr = reinterpret_cast<unsigned*>(s_ent + SAX_NST * CAP);     // [SAX_NST][PS]
    float2* s_g = reinterpret_cast<float2*>(s_ptr + SAX_NST * PS);           // [CC][L][TB]
    float2* s_tw = s_g + CC * GS;                                             // W^m, or [n2][k1] signed (FOLD)
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_tw + L + R2);
    const int tid = threadIdx.x;
    if (FOLD) {
        for (int m = tid; m < L; m += SAX_NT) {
            const int n2 = m / R1, k1 = m - n2 * R1;
            const float2 w = a.tw[n2 * k1];
            s_tw[n2 * (R1 + 1) + k1] = ((n2 + k1) & 1) ? cneg(w) : w;   // rows padded by one: no bank conflicts
        }
    } else {
        for (int m = tid; m < L; m += SAX_NT) s_tw[m] = a.tw[m];
    }
    if (tid == 0) {
        for (int s = 0; s < SAX_NST; ++s) mbar_init(&s_bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    const int nchunk = a.nch / CC;   // the launcher guarantees nch % CC == 0
    const int yv4_stride = a.nch / 2;
    float2 acc[CC], cmp[CC];
    auto add = [&](const float4 (&v)[CC / 2], float w) {
#pragma unroll
        for (int c = 0; c < CC; ++c) {
            const float vx = (c & 1) ? v[c / 2].z : v[c / 2].x;
            const float vy = (c & 1) ? v[c / 2].w : v[c / 2].y;
            if (KAHAN) {
                const float yx = fmaf(vx, w, -cmp[c].x), yy = fmaf(vy, w, -cmp[c].y);
                const float sx = __fadd_rn(acc[c].x, yx), sy = __fadd_rn(acc[c].y, yy);
                cmp[c].x = __fsub_rn(__fsub_rn(sx, acc[c].x), yx);
                cmp[c].y = __fsub_rn(__fsub_rn(sy, acc[c].y), yy);
                acc[c] = make_float2(sx, sy);
            } else {
                acc[c].x = fmaf(vx, w, acc[c].x);
                acc[c].y = fmaf(vy, w, acc[c].y);
            }
        }
    };
    auto issue = [&](int kk) {   // thread 0 only
        const unsigned u = blockIdx.x + (unsigned)kk * gridDim.x;
        const long long p0 = (a.j0 + u / (unsigned)nchunk) * (long long)PTS;
        const unsigned e0a = __ldg(a.ptr + p0) & ~1u, e1 = __ldg(a.ptr + p0 + PTS);
        const unsigned ne = e1 - e0a;
        const uint32_t pb = ((uint32_t)(PTS + 1) * 4u + 15u) & ~15u;
        const uint32_t eb = ne <= (unsigned)CAP ? ((ne * 8u + 15u) & ~15u) : 0u;
        const int st = kk % SAX_NST;
        mbar_arrive_expect_tx(&s_bar[st], pb + eb);
        bulk_load(s_ptr + st * PS, a.ptr + p0, pb, &s_bar[st]);
        if (eb) bulk_load(s_ent + st * CAP, a.ent + e0a, eb, &s_bar[st]);
    };

    const int my_n = nunits > (int)blockIdx.x ? (nunits - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    if (tid == 0)
        for (int kk = 0; kk < SAX_NST - 1 && kk < my_n; ++kk) issue(kk);
    for (int kk = 0; kk < my_n; ++kk) {
        const int st = kk % SAX_NST;
        const bool ok = mbar_wait_bounded(&s_bar[st], (uint32_t)((kk / SAX_NST) & 1), SAX_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            // timeout: report, let the copies already issued land, leave
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (int j = kk; j < my_n && j < kk + SAX_NST - 1; ++j)
                    mbar_wait_bounded(&s_bar[j % SAX_NST], (uint32_t)((j / SAX_NST) & 1), SAX_WAIT_NS);
            }
            return;
        }
        // every thread is past the previous unit (its transform's reads of
        // the lines, its gather's reads of stage (kk - 1) % SAX_NST): fetch
        // unit kk + SAX_NST - 1 into that stage
        if (tid == 0 && kk + SAX_NST - 1 < my_n) {
            fence_proxy_async_smem();
            issue(kk + SAX_NST - 1);
        }
        const unsigned u = blockIdx.x + (unsigned)kk * gridDim.x;
        const unsigned jt = u / (unsigned)nchunk;
        const int ch = (int)(u - jt * (unsigned)nchunk);
        const int2 t = a.tiles[a.j0 + jt];
        const unsigned* sp = s_ptr + st * PS;
        const int2* se = s_ent + st * CAP;
        const unsigned e0a = sp[0] & ~1u;
        const bool staged = sp[PTS] - e0a <= (unsigned)CAP;
        const float4* yv4 = reinterpret_cast<const float4*>(a.yv) + ch * (CC / 2);
        auto ent = [&](unsigned q) { return staged ? se[q - e0a] : __ldg(a.ent + q); };
        auto load_v = [&](int i, float4 (&v)[CC / 2]) {
            const float4* p = yv4 + (long long)i * yv4_stride;
#pragma unroll
            for (int c = 0; c < CC / 2; ++c) v[c] = __ldg(p + c);
        };

        // 1. the gather: point i = x * TB + column
        for (int i = tid; i < PTS; i += SAX_NT) {
            const unsigned e0 = sp[i], e1 = sp[i + 1];
#pragma unroll
            for (int c = 0; c < CC; ++c) acc[c] = cmp[c] = make_float2(0.f, 0.f);
            unsigned q = e0;
            for (; q + 1 < e1; q += 2) {
                const int2 p = ent(q), r = ent(q + 1);
                float4 vp[CC / 2], vr[CC / 2];
                load_v(p.x, vp);
                load_v(r.x, vr);
                add(vp, __int_as_float(p.y));
                add(vr, __int_as_float(r.y));
            }
            if (q < e1) {
                const int2 p = ent(q);
                float4 vp[CC / 2];
                load_v(p.x, vp);
                add(vp, __int_as_float(p.y));
            }
#pragma unroll
            for (int c = 0; c < CC; ++c) {
                float2 o = acc[c];
                if (KAHAN) o = make_float2(__fsub_rn(o.x, cmp[c].x), __fsub_rn(o.y, cmp[c].y));
                s_g[c * GS + gi(i / TB, i % TB)] = o;
            }
        }
        __syncthreads();

        // 2. the x transform of the unit's lines, CPP coils at a time
        const int lc = tid / TPC, r = tid - lc * TPC;
        const int bi = r % TB, rq = r / TB;
        const long long b = (long long)t.y + bi;
        const bool bok = b < a.B;
        for (int c0 = 0; c0 < CC; c0 += CPP) {
            const int c = c0 + lc;
            const bool act = lc < CPP && c < CC;
            float2* g = s_g + c * GS;
            if (act && rq < R2) {
                const int n2 = rq;
                float2 v[R1];
#pragma unroll
                for (int n1 = 0; n1 < R1; ++n1) {
                    const float2 x = g[gi(R2 * n1 + n2, bi)];
                    v[n1] = FOLD ? x : parity(x, R2 * n1 + n2);
                }
                Dft<R1, +1>::run(v);
#pragma unroll
                for (int k1 = 0; k1 < R1; ++k1) {
                    float2 tv = v[k1];
                    if (FOLD) tv = table_twiddle<+1>(tv, s_tw[n2 * (R1 + 1) + k1]);
                    else if (k1 > 0) tv = table_twiddle<+1>(tv, s_tw[n2 * k1]);
                    g[gi(k1 * R2 + n2, bi)] = tv;
                }
            }
            __syncthreads();
            if (act && rq < R1 && bok) {
                const int k1 = rq;
                float2 w[R2];
#pragma unroll
                for (int n2 = 0; n2 < R2; ++n2) w[n2] = g[gi(k1 * R2 + n2, bi)];
                Dft<R2, +1>::run(w);
                const long long item = (long long)(t.x - a.bin0) * a.nch + ch * CC + c;
                float2* o = a.out + item * a.out_bs + (long long)k1 * a.B + b;
                const long long step = (long long)R1 * a.B;
#pragma unroll
                for (int k2 = R2 / 4; k2 < 3 * R2 / 4; ++k2)
                    o[(k2 - R2 / 4) * step] = FOLD ? w[k2] : parity(w[k2], k1 + R1 * k2);
            }
        }
        // the next wait's barrier orders this unit's reads of the lines and
        // of its stage before the next unit's writes
    }
}

}  // namespace cgs
