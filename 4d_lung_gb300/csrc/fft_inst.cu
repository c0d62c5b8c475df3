// fft_inst.cu -- instantiation of the FFT pass kernels for one group of line
// lengths (compiled once per group with -DCGS_FFT_GROUP=g).
#include "fft_sizes.h"
#include "launch.h"
#include "fft_passes.cuh"
#include "spread_adjx.cuh"

#ifndef CGS_FFT_GROUP
#define CGS_FFT_GROUP 0
#endif

namespace cgs {

static int sm_count()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

constexpr int rmax2(int a, int b) { return a > b ? a : b; }
constexpr int strided_tb(int r1, int r2) { return fft_strided_tile_cols(r1, r2); }
constexpr int contig_lpb(int r1, int r2) { return rmax2(r1, r2) > 16 ? 8 : (rmax2(r1, r2) > 8 ? 16 : 32); }

template <int R1, int R2>
struct SizeImpl {
    static constexpr int L = R1 * R2;
    static constexpr int TB = strided_tb(R1, R2);
    static constexpr int LPB = contig_lpb(R1, R2);
    static constexpr int NT_S = TB * rmax2(R1, R2);
    static constexpr int NT_C = LPB * rmax2(R1, R2);
    static_assert(NT_C % 32 == 0, "contiguous pass block must be whole warps");

    static constexpr int NSTAGE = 2;
    using Pipe = PipeLayout<R1, R2, TB, NSTAGE>;
    // Toeplitz x stage: the strided passes' tile width (8-column tiles, four
    // 128-thread blocks per SM, measured 2 % slower at L = 256)
    static constexpr int TBT = TB;

    // pipelined z passes: coil tiles in flight ahead of the FFT
    static constexpr int ZNST_F = 2, ZNST_A = 2;
    using ZF = ZPipeLayout<R1, R2, LPB, ZNST_F>;
    using ZA = ZPipeLayout<R1, R2, LPB, ZNST_A>;

    // the TMA strided variants instantiated: forward (input-pruned or not),
    // adjoint (output-pruned or not)
    static constexpr bool HAS_IN = R1 % 4 == 0, HAS_OUT = R2 % 4 == 0;
    // x passes over listed tiles of the sample support: narrower tiles
    // (fft_listed_tile_cols) when both pruned forms exist
    static constexpr int TBN = fft_listed_tile_cols(R1, R2);
    static constexpr bool NARROW = HAS_IN && HAS_OUT && TBN != TB;
    static_assert(!(HAS_IN && HAS_OUT) || fft_has_narrow_tiles(R1, R2), "listed width and pruned forms agree");

    // pipeline stages of the narrow forward pass: its stages hold half as
    // many bytes (Ix rows of 64 bytes), so one more keeps as many in flight
    static constexpr int NSTAGE_NI = 3;

    template <int SIGN, int MODE, int TBK = TB, int NS = NSTAGE>
    static cudaError_t tma_attr(int smem)
    {
        return cudaFuncSetAttribute(k_fft_strided_tma<R1, R2, SIGN, TBK, NS, MODE>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    }

    static cudaError_t init()
    {
        const int smem = (int)Pipe::smem_bytes(L);
        cudaError_t e = tma_attr<-1, PRUNE_NONE>(smem);
        if (e == cudaSuccess) e = tma_attr<+1, PRUNE_NONE>(smem);
        if constexpr (HAS_IN)
            if (e == cudaSuccess) e = tma_attr<-1, PRUNE_IN>(smem);
        if constexpr (HAS_OUT)
            if (e == cudaSuccess) e = tma_attr<+1, PRUNE_OUT>(smem);
        if constexpr (NARROW) {
            if (e == cudaSuccess)
                e = tma_attr<-1, PRUNE_IN, TBN, NSTAGE_NI>((int)PipeLayout<R1, R2, TBN, NSTAGE_NI>::smem_bytes(L));
            if (e == cudaSuccess)
                e = tma_attr<+1, PRUNE_OUT, TBN>((int)PipeLayout<R1, R2, TBN, NSTAGE>::smem_bytes(L));
        }
        if constexpr (HAS_IN)
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_toep_x_tma<R1, R2, TBT, NSTAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)ToepLayout<R1, R2, TBT, NSTAGE>::smem_bytes(L / 2));
        // the z extent of an image never exceeds the grid's: size for Iz = L
        if constexpr (HAS_IN && HAS_OUT) {
            if (e == cudaSuccess) e = sax_attr<2, false>();
            if (e == cudaSuccess) e = sax_attr<2, true>();
            if (e == cudaSuccess) e = sax_attr<4, false>();
            if (e == cudaSuccess) e = sax_attr<4, true>();
            if (e == cudaSuccess) e = sax_attr<6, false>();
            if (e == cudaSuccess) e = sax_attr<6, true>();
        }
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_fwd_z_pipe<R1, R2, LPB, ZNST_F, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ZF::smem_bytes(L, false));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_fwd_z_pipe<R1, R2, LPB, ZNST_F, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ZF::smem_bytes(L, false));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_adj_z_pipe<R1, R2, LPB, ZNST_A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)ZA::smem_bytes(L, true));
        return e;
    }

    static bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

    // persistent launch: as many blocks as fit, at most one per tile
    template <int SIGN, int MODE, int TBK = TB, int NS = NSTAGE, int MAXB = 0>
    static cudaError_t tma_run(const StridedPassArgs& a, const CUtensorMap& map, int A, int batch, int box_rows,
                               cudaStream_t s)
    {
        using P = PipeLayout<R1, R2, TBK, NS>;
        const size_t smem = P::smem_bytes(a.Lin);
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_fft_strided_tma<R1, R2, SIGN, TBK, NS, MODE>, P::NT, smem);
        if (e != cudaSuccess) return e;
        const long long tiles_per_item = (long long)A * a.ntb;
        const long long ntiles = a.sup_tiles ? a.sup_ntiles * a.sup_nsub : tiles_per_item * batch;
        if (ntiles <= 0) return cudaSuccess;   // no listed tile: nothing to transform
        if (MAXB > 0 && per_sm > MAXB) per_sm = MAXB;
        long long nblk = (long long)sm_count() * (per_sm > 0 ? per_sm : 1);
        if (nblk > ntiles) nblk = ntiles;
        k_fft_strided_tma<R1, R2, SIGN, TBK, NS, MODE><<<(unsigned)nblk, P::NT, smem, s>>>(
            a, map, ntiles, (int)tiles_per_item, box_rows);
        return cudaGetLastError();
    }

    static cudaError_t strided(int sign, StridedPassArgs a, int A, int batch, cudaStream_t s)
    {
        const bool half_in = 4 * a.in_off == L && 2 * a.Lin == L;
        const bool half_out = 4 * a.out_off == L && 2 * a.Lout == L;
        CUtensorMap map;
        int box_rows = 0;
        // listed tiles are visited at the width they were listed with
        if (a.sup_tiles && a.sup_tb != TB && !(NARROW && a.sup_tb == TBN)) return cudaErrorInvalidValue;
        if constexpr (NARROW) {
            // tiles of fft_listed_cols' width: 64-byte rows, promoted to L2
            // as 64-byte requests
            if (a.sup_tiles && a.sup_tb == TBN) {
                if (!a.err || !(sign < 0 ? half_in : half_out)) return cudaErrorInvalidValue;
                a.ntb = (a.B + TBN - 1) / TBN;
                if (!encode_strided_map(&map, a, A, batch, TBN, &box_rows, TBN * 8)) return cudaErrorInvalidValue;
                // four blocks per SM: five (what shared memory allows) measured 7 % slower
                if (sign < 0) return tma_run<-1, PRUNE_IN, TBN, NSTAGE_NI, 4>(a, map, A, batch, box_rows, s);
                return tma_run<+1, PRUNE_OUT, TBN>(a, map, A, batch, box_rows, s);
            }
        }
        a.ntb = (a.B + TB - 1) / TB;
        if (a.err && encode_strided_map(&map, a, A, batch, TB, &box_rows)) {
            if (sign < 0) {
                if constexpr (HAS_IN)
                    if (half_in) return tma_run<-1, PRUNE_IN>(a, map, A, batch, box_rows, s);
                return tma_run<-1, PRUNE_NONE>(a, map, A, batch, box_rows, s);
            }
            if constexpr (HAS_OUT)
                if (half_out) return tma_run<+1, PRUNE_OUT>(a, map, A, batch, box_rows, s);
            return tma_run<+1, PRUNE_NONE>(a, map, A, batch, box_rows, s);
        }
        dim3 grid((unsigned)(A * a.ntb), (unsigned)batch);
        if (sign < 0) k_fft_strided<R1, R2, -1, TB><<<grid, NT_S, 0, s>>>(a);
        else k_fft_strided<R1, R2, +1, TB><<<grid, NT_S, 0, s>>>(a);
        return cudaGetLastError();
    }
    // Toeplitz x stage (in place, rows L/4 .. 3L/4 in and out)
    static cudaError_t toep_x(StridedPassArgs a, const float* P, long long p_bs, int nsub, int batch, cudaStream_t s)
    {
        if constexpr (!HAS_IN) {
            return cudaErrorNotSupported;
        } else {
            using Lay = ToepLayout<R1, R2, TBT, NSTAGE>;
            a.ntb = (a.B + TBT - 1) / TBT;
            if (4 * a.in_off != L || 2 * a.Lin != L || 4 * a.out_off != L || 2 * a.Lout != L || !a.err || nsub < 1 ||
                batch % nsub != 0 || p_bs != (long long)L * a.B)
                return cudaErrorNotSupported;
            CUtensorMap map, pmap;
            int box_rows = 0, pbox_rows = 0;
            if (!encode_strided_map(&map, a, 1, batch, TBT, &box_rows)) return cudaErrorNotSupported;
            if (!encode_spectrum_map(&pmap, P, a.B, L, batch / nsub, TBT, &pbox_rows)) return cudaErrorNotSupported;
            const size_t smem = Lay::smem_bytes(a.Lin);
            int per_sm = 0;
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_toep_x_tma<R1, R2, TBT, NSTAGE>,
                                                                          Lay::NT, smem);
            if (e != cudaSuccess) return e;
            const long long ntiles = (long long)a.ntb * batch;
            if (ntiles <= 0) return cudaSuccess;
            long long nblk = (long long)sm_count() * (per_sm > 0 ? per_sm : 1);
            if (nblk > ntiles) nblk = ntiles;
            k_toep_x_tma<R1, R2, TBT, NSTAGE><<<(unsigned)nblk, Lay::NT, smem, s>>>(a, nsub, map, pmap, ntiles,
                                                                                   box_rows, pbox_rows);
            return cudaGetLastError();
        }
    }
    // spreading fused with the adjoint x pass (tiles of 8 columns, output
    // pruned); layouts above the opt-in shared-memory limit are not launched
    static constexpr size_t SAX_SMEM_MAX = 227 * 1024;
    template <int CC, bool K>
    static cudaError_t sax_attr()
    {
        if (SaxLayout<R1, R2, CC>::bytes > SAX_SMEM_MAX) return cudaSuccess;   // not launched
        return cudaFuncSetAttribute(k_spread_adjx<R1, R2, CC, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)SaxLayout<R1, R2, CC>::bytes);
    }
    template <int CC, bool K>
    static cudaError_t sax_run(const SpreadAdjxArgs& a, cudaStream_t s)
    {
        constexpr size_t smem = SaxLayout<R1, R2, CC>::bytes;
        if (smem > SAX_SMEM_MAX || a.nch % CC != 0) return cudaErrorNotSupported;
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spread_adjx<R1, R2, CC, K>, SAX_NT,
                                                                      smem);
        if (e != cudaSuccess) return e;
        const long long nunits = a.nj * (a.nch / CC);
        if (nunits <= 0) return cudaSuccess;
        if (nunits >= 0x7fffffffLL) return cudaErrorInvalidValue;
        const long long nblk = std::min<long long>(nunits, (long long)sm_count() * std::max(per_sm, 1));
        k_spread_adjx<R1, R2, CC, K><<<(unsigned)nblk, SAX_NT, smem, s>>>(a, (int)nunits);
        return cudaGetLastError();
    }
    static cudaError_t spread_adjx(const SpreadAdjxArgs& a, bool kahan, cudaStream_t s)
    {
        if constexpr (!(HAS_IN && HAS_OUT)) {
            return cudaErrorNotSupported;
        } else {
            // 16-byte aligned row offsets and taps (bulk copies), coil pairs
            if (!a.err || (reinterpret_cast<uintptr_t>(a.ptr) & 15) || (reinterpret_cast<uintptr_t>(a.ent) & 15) ||
                (reinterpret_cast<uintptr_t>(a.yv) & 15) || a.nch < 2)
                return cudaErrorNotSupported;
            int cc = a.cc;
            if (cc == 0) cc = a.nch % 6 == 0 ? 6 : a.nch % 4 == 0 ? 4 : 2;
            switch (cc) {
            case 2: return kahan ? sax_run<2, true>(a, s) : sax_run<2, false>(a, s);
            case 4: return kahan ? sax_run<4, true>(a, s) : sax_run<4, false>(a, s);
            case 6: return kahan ? sax_run<6, true>(a, s) : sax_run<6, false>(a, s);
            }
            return cudaErrorNotSupported;
        }
    }
    static cudaError_t contig(int sign, const ContigPassArgs& a, int batch, cudaStream_t s)
    {
        dim3 grid((unsigned)((a.nl + LPB - 1) / LPB), (unsigned)batch);
        if (sign < 0) k_fft_contig<R1, R2, -1, LPB><<<grid, NT_C, 0, s>>>(a);
        else k_fft_contig<R1, R2, +1, LPB><<<grid, NT_C, 0, s>>>(a);
        return cudaGetLastError();
    }
    // z passes: one block per (line block, batch item), items fastest (zp_item)
    static cudaError_t fwd_z(const FwdZArgs& a0, int batch, cudaStream_t s)
    {
        FwdZArgs a = a0;
        a.nbatch = batch;
        dim3 grid((unsigned)(((a.nl + LPB - 1) / LPB) * batch));
        // bulk copies need 16-byte aligned tiles: even Iz and coil strides
        if (a.err && a.smaps && a.x_cs == 0 && a.Iz <= L && (a.Iz & 1) == 0 && (a.coil_in & 1) == 0 &&
            al16(a.smaps)) {
            if (a.cg) k_fwd_z_pipe<R1, R2, LPB, ZNST_F, true><<<grid, NT_C, ZF::smem_bytes(a.Iz, false), s>>>(a);
            else k_fwd_z_pipe<R1, R2, LPB, ZNST_F, false><<<grid, NT_C, ZF::smem_bytes(a.Iz, false), s>>>(a);
            return cudaGetLastError();
        }
        if (a.cg) k_fwd_z<R1, R2, LPB, true><<<grid, NT_C, 0, s>>>(a);
        else k_fwd_z<R1, R2, LPB, false><<<grid, NT_C, 0, s>>>(a);
        return cudaGetLastError();
    }
    static int adj_blocks(long long nl) { return (int)((nl + LPB - 1) / LPB); }
    static cudaError_t adj_z(const AdjZArgs& a0, int batch, cudaStream_t s)
    {
        AdjZArgs a = a0;
        a.nbatch = batch;
        dim3 grid((unsigned)((long long)adj_blocks(a.nl) * batch));
        if (a.err && a.smaps && a.Iz <= L && (a.Iz & 1) == 0 && (a.coil_s & 1) == 0 && (a.coil_in & 1) == 0 &&
            (a.in_bs & 1) == 0 && al16(a.smaps) && al16(a.in)) {
            k_adj_z_pipe<R1, R2, LPB, ZNST_A><<<grid, NT_C, ZA::smem_bytes(a.Iz, true), s>>>(a);
            return cudaGetLastError();
        }
        k_adj_z<R1, R2, LPB><<<grid, NT_C, 0, s>>>(a);
        return cudaGetLastError();
    }
};

#define CGS_DEFINE(L_, R1_, R2_, G_)                                                                \
    cudaError_t fft_strided_##L_(int sign, const StridedPassArgs& a, int A, int batch, cudaStream_t s); \
    cudaError_t fft_contig_##L_(int sign, const ContigPassArgs& a, int batch, cudaStream_t s);        \
    cudaError_t fft_fwd_z_##L_(const FwdZArgs& a, int batch, cudaStream_t s);                          \
    cudaError_t fft_adj_z_##L_(const AdjZArgs& a, int batch, cudaStream_t s);                          \
    int fft_adj_blocks_##L_(long long nl);                                                             \
    cudaError_t fft_init_##L_();                                                                       \
    cudaError_t fft_toep_x_##L_(const StridedPassArgs& a, const float* P, long long p_bs, int nsub, int batch, \
                                cudaStream_t s);                                                       \
    cudaError_t fft_spread_adjx_##L_(const SpreadAdjxArgs& a, bool kahan, cudaStream_t s);             \
    CGS_DEFINE_IF_##G_(L_, R1_, R2_)

#define CGS_BODY(L_, R1_, R2_)                                                                      \
    cudaError_t fft_strided_##L_(int sign, const StridedPassArgs& a, int A, int batch, cudaStream_t s) \
    { return SizeImpl<R1_, R2_>::strided(sign, a, A, batch, s); }                                   \
    cudaError_t fft_contig_##L_(int sign, const ContigPassArgs& a, int batch, cudaStream_t s)         \
    { return SizeImpl<R1_, R2_>::contig(sign, a, batch, s); }                                       \
    cudaError_t fft_fwd_z_##L_(const FwdZArgs& a, int batch, cudaStream_t s)                           \
    { return SizeImpl<R1_, R2_>::fwd_z(a, batch, s); }                                              \
    cudaError_t fft_adj_z_##L_(const AdjZArgs& a, int batch, cudaStream_t s)                           \
    { return SizeImpl<R1_, R2_>::adj_z(a, batch, s); }                                              \
    int fft_adj_blocks_##L_(long long nl) { return SizeImpl<R1_, R2_>::adj_blocks(nl); }               \
    cudaError_t fft_init_##L_() { return SizeImpl<R1_, R2_>::init(); }                                 \
    cudaError_t fft_toep_x_##L_(const StridedPassArgs& a, const float* P, long long p_bs, int nsub, int batch, \
                                cudaStream_t s)                                                        \
    { return SizeImpl<R1_, R2_>::toep_x(a, P, p_bs, nsub, batch, s); }                                \
    cudaError_t fft_spread_adjx_##L_(const SpreadAdjxArgs& a, bool kahan, cudaStream_t s)              \
    { return SizeImpl<R1_, R2_>::spread_adjx(a, kahan, s); }

#if CGS_FFT_GROUP == 0
#define CGS_DEFINE_IF_0(L, R1, R2) CGS_BODY(L, R1, R2)
#else
#define CGS_DEFINE_IF_0(L, R1, R2)
#endif
#if CGS_FFT_GROUP == 1
#define CGS_DEFINE_IF_1(L, R1, R2) CGS_BODY(L, R1, R2)
#else
#define CGS_DEFINE_IF_1(L, R1, R2)
#endif
#if CGS_FFT_GROUP == 2
#define CGS_DEFINE_IF_2(L, R1, R2) CGS_BODY(L, R1, R2)
#else
#define CGS_DEFINE_IF_2(L, R1, R2)
#endif
#if CGS_FFT_GROUP == 3
#define CGS_DEFINE_IF_3(L, R1, R2) CGS_BODY(L, R1, R2)
#else
#define CGS_DEFINE_IF_3(L, R1, R2)
#endif
#if CGS_FFT_GROUP == 4
#define CGS_DEFINE_IF_4(L, R1, R2) CGS_BODY(L, R1, R2)
#else
#define CGS_DEFINE_IF_4(L, R1, R2)
#endif
#if CGS_FFT_GROUP == 5
#define CGS_DEFINE_IF_5(L, R1, R2) CGS_BODY(L, R1, R2)
#else
#define CGS_DEFINE_IF_5(L, R1, R2)
#endif

CGS_FFT_SIZES(CGS_DEFINE)

}  // namespace cgs
