// cgs_api.cu -- C ABI of the GB300 CG-SENSE library: context, trajectory
// and bin set-up, NUFFT / E^H D E chains, and the graph-captured CG solve.
//
// Replaces the reference's Reco object (Reco.h:13-214, Reco.cpp) for the
// reconstruction hot path; see include/cgsense_c.h for the entry points and
// the reference functions each one stands for.
#include "cgsense_c.h"
#include "launch.h"
#include "fft_sizes.h"

#include <algorithm>
#include <chrono>
#include <sys/stat.h>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

using namespace cgs;

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n)
    {
        if (n <= bytes && p) return cudaSuccess;
        release();
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
    template <class T>
    T* as() const { return reinterpret_cast<T*>(p); }
};

struct GraphKey {
    const void* data;
    void* x;
    double thresh;
    int max_iter;
    int rhs_from_images;
    void* trace;
    bool operator<(const GraphKey& o) const
    {
        return std::tie(data, x, thresh, max_iter, rhs_from_images, trace) <
               std::tie(o.data, o.x, o.thresh, o.max_iter, o.rhs_from_images, o.trace);
    }
};

}  // namespace

struct cgs_ctx {
    cgs_params p{};
    int I[3]{}, G[3]{}, lo[3]{};
    long long Ni = 0, Ng = 0, Nl = 0;
    int nch = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    float thresh = 0.f;          // absolute tap threshold
    double adj_scale_total = 0;  // adj_scale / sqrt(Ng)
    std::vector<double> apod_full[3];   // 1/R_a(g) over the whole grid axis

    DevBuf tw[3], ap[3];
    DevBuf d_err;                // set by a kernel whose bounded wait timed out
    // trajectory
    long long ns = 0;
    std::vector<double> h_k;
    DevBuf d_k;
    std::vector<float> h_dcf;
    bool has_dcf = false;
    // bins
    std::vector<std::vector<int>> bins;   // global sample indices per bin (user order)
    bool bins_dirty = true;
    int nbins = 0;
    long long total = 0;
    long long max_bin = 0;
    std::vector<long long> h_bin_off;
    DevBuf d_sorted, d_rec, d_dcf_sorted, d_bin_off, d_tile_ptr, d_tile_ptr_off, d_tile_idx, d_tile_idx_off;
    DevBuf d_plane_rng;
    // loss gradients: derivative records, gathered measured samples, partials
    DevBuf d_drec, d_gy, d_gpart, d_flag;
    DevBuf d_pa, d_pda;          // stored values / derivatives of E S p (operator VJPs)
    bool drec_valid = false;
    bool kahan = false;          // compensated spreading (cgs_set_precision)
    // launch shapes (cgs_autotune): coils per spreading block (0: as many as
    // fit), coils per interpolation thread
    int spread_cc = 0;
    int spread_wpp = 8;          // spreading variant: warps per x plane 1 / 2, 3 atomics, 4 / 5 pipelined,
                                 // 6 / 7 gather over the transposed tap matrix, staged in shared memory /
                                 // read from global memory (2 when it is not built), 8 the staged gather
                                 // fused with the adjoint x pass (6 where that does not apply)
    bool deterministic = true;   // fixed summation order everywhere (cgs_set_deterministic)
    bool spread_fused = false;   // the last adjoint half ran the fused spreading + x pass
    int interp_cc = 4;
    bool k_host_stale = false;   // d_k updated on the device (cgs_update_trajectory_d)
    uint64_t traj_serial = 0;    // incremented whenever the coordinates change
    bool tiles_stale = false;    // spreading lists built from older coordinates
    int ntx = 0, nty = 0, ntz = 0, ntiles = 0;
    // sample-support pruning of the x FFT passes and the spreading
    // (cgs_set_support_pruning)
    bool sup_prune = true;
    bool sup_built = false;
    std::vector<long long> h_sup_off;        // per bin: first entry in d_sup_tiles
    std::vector<int2> h_sup_tiles;           // listed tiles {bin, first column}, all bins
    // rows of each forward-y-pass tile that the x pass reads (per bin, z tile, Gy / 32 words);
    // built when the x and y passes' column tiles coincide
    DevBuf d_sup_rowmask;
    long long sup_rowmask_bs = 0;            // words per bin (0: not built)
    int sup_tb = 0;                          // columns per listed x-pass tile (fft_listed_cols)
    // the spreading gather's listing (variants 6, 7): tiles of the strided
    // passes' width, each a union of x-pass tiles, so that it stores every
    // column the adjoint x pass reads, in 128-byte rows
    int spr_tb = 0;
    std::vector<long long> h_spr_off;
    std::vector<int2> h_spr_tiles;
    DevBuf d_spr_tiles;
    int csr_list = -1;                       // listing of the transposed tap matrix: 0 the spreading's,
                                             // 1 the x passes' (fused variant 8); -1 not built
    // transposed tap matrix of the listed tiles' points (spreading variant 6)
    bool csr_valid = false;
    long long csr_pts = 0;
    unsigned long long csr_entries = 0;
    DevBuf d_col_tile, d_csr_cnt, d_csr_ptr, d_csr_ent, d_csr_tmp;
    std::vector<long long> h_live_off;       // per bin: first entry in d_live (spreading tiles)
    DevBuf d_sup_tiles, d_live, d_live_off;
    // The adjoint x pass writes its own y buffer (d_ybuf_adj), and with
    // pruning only the supported columns of the slot's bin; the rest of the
    // slot must hold zeros.  adj_slot[j]: the bin whose supported columns
    // bound the non-zeros of workspace slot j, -1 when unknown.
    DevBuf d_ybuf_adj;
    std::vector<int> adj_slot;
    // Toeplitz embedding of E^H D E (cgs_set_toeplitz): 0 off, 1 on (fused x
    // stage where it applies), 2 on with the unfused x stage; per bin the real
    // spectrum P [Gx][Gy * Gz] of the point-spread function
    int toep_mode = 0;
    bool toep_valid = false;
    uint64_t toep_serial = 0;    // traj_serial the spectra were built from
    double toep_build_ms = 0.0;
    int toep_method = 0;         // spectrum build: 0 through the PSF where possible, 1 Dirichlet product
    int toep_used = 0;           // method of the last build: 1 PSF (adjoint NUFFT), 2 Dirichlet product
    // set-up cost of the last rebuild of the bins and of the last graph
    // capture (host clock, ms): sort, tap records, tile and support lists,
    // transposed tap matrix, workspaces, graph capture + instantiation
    double setup_ms[6] = {0, 0, 0, 0, 0, 0};
    DevBuf d_toep, d_ones;
    void* blas = nullptr;        // cuBLAS handle of the spectrum builds
    // coil maps
    DevBuf d_smaps;
    bool smaps_set = false;
    // workspace
    int ws_bins = 0;
    DevBuf d_zbuf, d_ybuf, d_grid, d_yv, d_img, d_data;
    // CG
    DevBuf d_b, d_x, d_r, d_pv, d_q, d_state, d_partials, d_partials2, d_res;
    // while a fused solve is recorded: the vectors whose pending updates the
    // forward z pass applies (FwdZArgs::cg); all null otherwise
    struct {
        CgState* st = nullptr;
        float2 *p = nullptr, *x = nullptr;
        const float2* r = nullptr;
    } cgf;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::map<GraphKey, long long> graph_launches;
    // adjoint y-buffer slot records at the start and at the end of each graph
    std::map<GraphKey, std::pair<std::vector<int>, std::vector<int>>> graph_slots;
    long long launches = 0;
    // plain per-bin form (cgs_cg_solve_plain_d)
    cufftHandle plain_plan = 0;
    bool plain_plan_ok = false;
    DevBuf d_plain_grid, d_plain_y, d_plain_dot;
    // full-FP64 form (cgs_cg_solve_fp64_d)
    cufftHandle z_plan = 0;
    bool z_plan_ok = false;
    DevBuf d64_grid, d64_y, d64_r, d64_p, d64_q, d64_part;
    // per-stage timing (cgs_profile_apply): events recorded after each pass
    cudaEvent_t* prof_ev = nullptr;
    int prof_n = 0;
    // parts of the last host-buffer solve (cgs_e2e_stats): events before the
    // upload, after it, after the graph launch and after the download
    cudaEvent_t e2e_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool e2e_mark = false;       // solve_d records e2e_ev[2] after its graph launch
    void* h_stage = nullptr;     // page-locked staging of the solve's iteration record
    size_t h_stage_bytes = 0;
    int e2e_pinned[2] = {0, 0};  // host buffers of the last call page-locked (as this runtime sees them)
    std::string err;
};

namespace {

int fail(cgs_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

#define CGS_CUDA(ctx, call)                                                                     \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? CGS_ERR_NOMEM : CGS_ERR_CUDA,    \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

#define CGS_LAUNCH(ctx, call)                                                       \
    do {                                                                            \
        CGS_CUDA(ctx, call);                                                        \
        ++(ctx)->launches;                                                          \
        if ((ctx)->prof_ev) CGS_CUDA(ctx, cudaEventRecord((ctx)->prof_ev[(ctx)->prof_n++], (ctx)->stream)); \
    } while (0)

#define CGS_TRY(call)              \
    do {                           \
        int s_ = (call);           \
        if (s_ != CGS_OK) return s_; \
    } while (0)

// Per-axis KB factor of Reco::ConvKernel::convFunction (Reco.h:218-242) at a
// k-space distance `dist` on an axis of n grid points.
double kb_factor(const cgs_params& p, int n, double dist)
{
    const float w = p.kb_w, b = p.kb_b;
    const float dk = (float)(1.0 / (double)(float)(n - 1));
    const float wHalf = (float)(w / 2.0);
    const float d = (float)dist;
    if (d > wHalf * dk) return 0.0;
    const float q = (float)(2.f * d) / (float)(w * dk);
    const double arg = (double)b * std::sqrt(1.0 - (double)q * (double)q);
    return std::cyl_bessel_i(0.0, arg) / (double)(float)(100.0f * w * dk);
}

// ConvKernel::calculateKernelFT (Reco.cpp:560-601) is separable: the 3-D
// sampled kernel is the product of per-axis factors, so its centred
// backward transform is the product of per-axis transforms
//   R_a(g) = (-1)^g sum_n (-1)^n f_a(n) exp(+2 pi i n g / N),
// which are real (f_a is symmetric about N/2).  kernelFT = 1/(Rx Ry Rz).
std::vector<double> deapod_axis(const cgs_params& p, int n)
{
    const double dk = 1.0 / (double)(n - 1);
    std::vector<double> f(n);
    for (int i = 0; i < n; ++i) f[i] = kb_factor(p, n, std::sqrt(dk * dk * (double)(i - n / 2) * (double)(i - n / 2)));
    std::vector<double> out(n);
    for (int g = 0; g < n; ++g) {
        double re = 0.0;
        for (int i = 0; i < n; ++i) {
            if (f[i] == 0.0) continue;
            const long long m = ((long long)i * g) % n;
            const double s = (((i + g) & 1) ? -1.0 : 1.0);
            re += s * f[i] * std::cos(kTwoPi * (double)m / (double)n);
        }
        out[g] = 1.0 / re;
    }
    return out;
}

// Host-side bin preparation.  Samples are sorted by their home spreading
// tile (the tile of the nearest grid point).  Each tile then gets the list of
// the samples whose 5-point support touches it, ordered by nearest x (stable
// in sorted position), and per x plane of the tile the range of that list
// whose support covers the plane.  The lists use the nearest points of the
// device's tap records, so that list membership and the taps agree exactly.
struct BinPrep {
    std::vector<int> sorted;
    std::vector<int> tile_ptr;
    std::vector<int> tile_idx;
    std::vector<int> plane_rng;   // [ntiles][TILE_X][2]
    std::vector<int> sup_cols;        // first column of each x-pass tile the samples touch
    std::vector<int> spr_cols;        // the same for the spreading gather's wider tiles
    std::vector<int> live;            // spreading tiles holding a supported column
};

void nearest_point(const double* kk, const int* G, int* nr)
{
    for (int a = 0; a < 3; ++a) {
        int v = (int)((G[a] - 1) * kk[a] + 0.5);
        nr[a] = std::min(std::max(v, 0), G[a] - 1);
    }
}

void sort_bin(const cgs_ctx* c, const std::vector<int>& samples, BinPrep& out)
{
    const int* G = c->G;
    const long long n = (long long)samples.size();
    std::vector<int> key(n);
    std::vector<int> count(c->ntiles + 1, 0);
    for (long long i = 0; i < n; ++i) {
        int nr[3];
        nearest_point(&c->h_k[3 * (size_t)samples[i]], G, nr);
        const int k = ((nr[0] / TILE_X) * c->nty + nr[1] / TILE_Y) * c->ntz + nr[2] / TILE_Z;
        key[i] = k;
        count[k + 1]++;
    }
    for (int t = 0; t < c->ntiles; ++t) count[t + 1] += count[t];
    out.sorted.assign(n, 0);
    std::vector<int> pos(count.begin(), count.end() - 1);
    for (long long i = 0; i < n; ++i) out.sorted[pos[key[i]]++] = samples[i];
}

// nearest: packed nearest points of the bin's sorted samples (device records)
void tile_lists(const cgs_ctx* c, const unsigned* nearest, long long n, BinPrep& out)
{
    const int* G = c->G;
    auto unpack = [](unsigned u, int* nr) {
        nr[0] = (int)(u & 2047u);
        nr[1] = (int)((u >> 11) & 2047u);
        nr[2] = (int)(u >> 22);
    };
    // visit the samples in order of nearest x (counting sort, stable)
    std::vector<int> xcount(G[0] + 1, 0);
    for (long long j = 0; j < n; ++j) xcount[(nearest[j] & 2047u) + 1]++;
    for (int x = 0; x < G[0]; ++x) xcount[x + 1] += xcount[x];
    std::vector<int> byx(n);
    {
        std::vector<int> p(xcount.begin(), xcount.end() - 1);
        for (long long j = 0; j < n; ++j) byx[p[nearest[j] & 2047u]++] = (int)j;
    }
    auto range = [&](int nr, int a, int T, int nt, int& t0, int& t1) {
        const int lo = std::max(nr - 2, 0), hi = std::min(nr + 2, G[a] - 1);
        t0 = lo / T;
        t1 = std::min(hi / T, nt - 1);
    };
    out.tile_ptr.assign(c->ntiles + 1, 0);
    std::vector<int> fill;
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            for (int t = 0; t < c->ntiles; ++t) out.tile_ptr[t + 1] += out.tile_ptr[t];
            out.tile_idx.assign(out.tile_ptr[c->ntiles], 0);
            fill.assign(out.tile_ptr.begin(), out.tile_ptr.end() - 1);
        }
        for (long long m = 0; m < n; ++m) {
            const int j = byx[m];
            int nr[3];
            unpack(nearest[j], nr);
            int x0, x1, y0, y1, z0, z1;
            range(nr[0], 0, TILE_X, c->ntx, x0, x1);
            range(nr[1], 1, TILE_Y, c->nty, y0, y1);
            range(nr[2], 2, TILE_Z, c->ntz, z0, z1);
            for (int tx = x0; tx <= x1; ++tx)
                for (int ty = y0; ty <= y1; ++ty)
                    for (int tz = z0; tz <= z1; ++tz) {
                        const int t = (tx * c->nty + ty) * c->ntz + tz;
                        if (pass == 0) out.tile_ptr[t + 1]++;
                        else out.tile_idx[fill[t]++] = j;
                    }
        }
    }
    // plane ranges: the list is sorted by nearest x, so the samples whose
    // support [nx - 2, nx + 2] covers plane x form one run
    out.plane_rng.assign((size_t)c->ntiles * TILE_X * 2, 0);
    for (int t = 0; t < c->ntiles; ++t) {
        const int b = out.tile_ptr[t], e = out.tile_ptr[t + 1];
        const int xt0 = (t / (c->nty * c->ntz)) * TILE_X;
        int lo = b, hi = b;
        for (int p = 0; p < TILE_X; ++p) {
            const int x = xt0 + p;
            while (lo < e && (int)(nearest[out.tile_idx[lo]] & 2047u) < x - 2) ++lo;
            if (hi < lo) hi = lo;
            while (hi < e && (int)(nearest[out.tile_idx[hi]] & 2047u) <= x + 2) ++hi;
            out.plane_rng[((size_t)t * TILE_X + p) * 2] = lo - b;
            out.plane_rng[((size_t)t * TILE_X + p) * 2 + 1] = (x < G[0] ? hi : lo) - b;
        }
    }
}

// Sample-support lists of one bin.  The interpolation reads, and the
// spreading writes, grid points within +-2 cells of each sample's nearest
// point (clipped to the grid).  A (y, z) column of the grid that no sample's
// support reaches is never read after the forward x pass, and the adjoint x
// pass transforms zeros there.  The x passes work on tiles of tb consecutive
// columns of the flattened [Gy][Gz] plane: the tiles holding a supported
// column are listed (sup_cols); the spreading stores the grid tiles whose
// (y, z) extent meets a listed column (live).
void support_lists(const cgs_ctx* c, const unsigned* nearest, long long n, int tb, int tbs, BinPrep& out)
{
    const int Gy = c->G[1], Gz = c->G[2];
    const long long ncol = (long long)Gy * Gz;
    std::vector<unsigned char> col(ncol, 0);
    for (long long j = 0; j < n; ++j) {
        const int ny = (int)((nearest[j] >> 11) & 2047u), nz = (int)(nearest[j] >> 22);
        const int y0 = std::max(ny - 2, 0), y1 = std::min(ny + 2, Gy - 1);
        const int z0 = std::max(nz - 2, 0), z1 = std::min(nz + 2, Gz - 1);
        for (int y = y0; y <= y1; ++y)
            for (int z = z0; z <= z1; ++z) col[(long long)y * Gz + z] = 1;
    }
    std::vector<unsigned char> listed(ncol, 0);   // column lies in a listed tile
    out.sup_cols.clear();
    for (long long b0 = 0; b0 < ncol; b0 += tb) {
        const long long b1 = std::min(ncol, b0 + tb);
        bool any = false;
        for (long long b = b0; b < b1 && !any; ++b) any = col[b] != 0;
        if (!any) continue;
        out.sup_cols.push_back((int)b0);
        for (long long b = b0; b < b1; ++b) listed[b] = 1;
    }
    // the spreading gather's tiles (tb divides tbs)
    out.spr_cols.clear();
    for (long long b0 = 0; b0 < ncol; b0 += tbs) {
        const long long b1 = std::min(ncol, b0 + tbs);
        bool any = false;
        for (long long b = b0; b < b1 && !any; ++b) any = col[b] != 0;
        if (any) out.spr_cols.push_back((int)b0);
    }
    // spreading tiles whose (y, z) extent holds a masked column: the adjoint
    // x pass reads those columns at every x, so these tiles are stored (with
    // zeros where no sample reaches); no other grid point is ever read
    std::vector<unsigned char> tcol((size_t)c->nty * c->ntz, 0);
    for (int ty = 0; ty < c->nty; ++ty)
        for (int tz = 0; tz < c->ntz; ++tz) {
            bool any = false;
            for (int y = ty * TILE_Y; y < std::min((ty + 1) * TILE_Y, Gy) && !any; ++y)
                for (int z = tz * TILE_Z; z < std::min((tz + 1) * TILE_Z, Gz) && !any; ++z) {
                    any = listed[(long long)y * Gz + z] != 0;
                }
            tcol[(size_t)ty * c->ntz + tz] = any;
        }
    out.live.clear();
    for (int tx = 0; tx < c->ntx; ++tx)
        for (int j = 0; j < c->nty * c->ntz; ++j)
            if (tcol[j]) out.live.push_back(tx * c->nty * c->ntz + j);
}

int upload(cgs_ctx* c, DevBuf& b, const void* h, size_t bytes)
{
    CGS_CUDA(c, b.ensure(bytes));
    if (bytes) CGS_CUDA(c, cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, c->stream));
    return CGS_OK;
}

// The transposed tap matrix over the points of the listed tiles of the
// spreading gather (list 0, variants 6 and 7) or of the x passes (list 1,
// the gather fused with the adjoint x pass), from the current tap records
// and support lists.  Skipped (the gather variants then fall back to the
// tiled kernel) when the counts could overflow 32-bit offsets.
int build_csr(cgs_ctx* c, int list)
{
    c->csr_valid = false;
    c->csr_list = -1;
    c->csr_entries = 0;
    if (!c->sup_built || c->total == 0) return CGS_OK;
    const int tbx = list == 1 ? c->sup_tb : c->spr_tb;
    const std::vector<long long>& off = list == 1 ? c->h_sup_off : c->h_spr_off;
    const std::vector<int2>& tl = list == 1 ? c->h_sup_tiles : c->h_spr_tiles;
    const long long ncol = (long long)c->G[1] * c->G[2];
    const long long ntl = off[c->nbins];
    const long long npts = ntl * c->G[0] * tbx;
    if (npts <= 0 || (unsigned long long)c->total * 125ull >= 0xffffffffull || npts + 1 >= 0x7fffffffLL) return CGS_OK;
    std::vector<int> ct((size_t)c->nbins * ncol, -1);
    for (int b = 0; b < c->nbins; ++b)
        for (long long J = off[b]; J < off[b + 1]; ++J)
            for (int k = 0; k < tbx && tl[J].y + k < ncol; ++k) ct[(size_t)b * ncol + tl[J].y + k] = (int)J;
    CGS_TRY(upload(c, c->d_col_tile, ct.data(), ct.size() * sizeof(int)));
    const size_t tmp = csr_scan_tmp_elems(npts + 1);
    CGS_CUDA(c, c->d_csr_cnt.ensure((size_t)(npts + 1) * sizeof(unsigned)));
    // padding: the staged gather copies whole 16-byte words past a slab's last offset and tap
    CGS_CUDA(c, c->d_csr_ptr.ensure((size_t)(npts + 8) * sizeof(unsigned)));
    CGS_CUDA(c, c->d_csr_tmp.ensure(tmp * sizeof(unsigned)));
    CGS_CUDA(c, c->d_flag.ensure(sizeof(int)));
    CGS_CUDA(c, cudaMemsetAsync(c->d_flag.p, 0, sizeof(int), c->stream));
    CsrBuildArgs a{};
    a.rec = c->d_rec.as<TapRecord>();
    a.total = c->total;
    a.bin_off = c->d_bin_off.as<long long>();
    a.nbins = c->nbins;
    a.col_tile = c->d_col_tile.as<int>();
    for (int i = 0; i < 3; ++i) a.G[i] = c->G[i];
    a.tb = tbx;
    a.thresh = c->thresh;
    a.cnt = c->d_csr_cnt.as<unsigned>();
    a.ptr = c->d_csr_ptr.as<unsigned>();
    a.err = c->d_flag.as<int>();
    unsigned long long ne = 0;
    CGS_CUDA(c, csr_count_and_scan(a, npts, c->d_csr_ptr.as<unsigned>(), c->d_csr_tmp.as<unsigned>(), tmp, &ne,
                                   c->stream));
    CGS_CUDA(c, c->d_csr_ent.ensure((ne + 2) * sizeof(int2)));
    a.ent = c->d_csr_ent.as<int2>();
    CGS_CUDA(c, csr_fill_and_order(a, npts, c->stream));
    int bad = 0;
    CGS_CUDA(c, cudaMemcpyAsync(&bad, c->d_flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->d_csr_cnt.release();   // the counts / fill cursors are not needed after the build
    if (bad) return CGS_OK;   // a tap outside the lists: keep the tiled kernel
    c->csr_pts = npts;
    c->csr_entries = ne;
    c->csr_valid = true;
    c->csr_list = list;
    return CGS_OK;
}

void drop_graphs(cgs_ctx* c);

// The fused spreading + adjoint x pass (variant 8) applies: listed x-pass
// tiles of 8 columns, both x passes half-pruned, a coil chunk (2, 4, 6) that
// divides the coil count
bool fused_spread_applies(const cgs_ctx* c)
{
    if (c->sup_tb != SAX_TB || 4 * c->lo[0] != c->G[0] || 2 * c->I[0] != c->G[0] || c->nch % 2 != 0) return false;
    const int cc = c->spread_cc;
    return !(cc == 2 || cc == 4 || cc == 6) || c->nch % cc == 0;
}

// The transposed tap matrix over the listing the current spreading variant
// reads (rebuilt, and the captured graphs dropped, when it changes)
int ensure_csr(cgs_ctx* c)
{
    if (!c->sup_built) return CGS_OK;
    const int want = (c->spread_wpp == 8 && fused_spread_applies(c)) ? 1 : 0;
    if (c->csr_list == want && c->csr_valid) return CGS_OK;
    drop_graphs(c);
    return build_csr(c, want);
}

void drop_graphs(cgs_ctx* c)
{
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    c->graph_launches.clear();
    c->graph_slots.clear();
}

KbParams kb_params(const cgs_ctx* c)
{
    KbParams kb;
    for (int a = 0; a < 3; ++a) kb.G[a] = c->G[a];
    kb.w = c->p.kb_w;
    kb.b = c->p.kb_b;
    kb.thresh = c->thresh;
    return kb;
}

int rebuild_bins(cgs_ctx* c)
{
    if (!c->bins_dirty) return CGS_OK;
    if (c->k_host_stale) {
        CGS_CUDA(c, cudaMemcpyAsync(c->h_k.data(), c->d_k.p, c->h_k.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream));
        CGS_CUDA(c, cudaStreamSynchronize(c->stream));
        c->k_host_stale = false;
    }
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set");
    drop_graphs(c);
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t0) { return std::chrono::duration<double, std::milli>(clk::now() - t0).count(); };
    auto t0 = clk::now();
    c->nbins = (int)c->bins.size();
    std::vector<BinPrep> prep(c->nbins);
    c->h_bin_off.assign(c->nbins + 1, 0);
    for (int b = 0; b < c->nbins; ++b) {
        sort_bin(c, c->bins[b], prep[b]);
        c->h_bin_off[b + 1] = c->h_bin_off[b] + (long long)c->bins[b].size();
    }
    c->total = c->h_bin_off[c->nbins];
    c->max_bin = 0;
    for (int b = 0; b < c->nbins; ++b) c->max_bin = std::max(c->max_bin, (long long)c->bins[b].size());
    std::vector<int> sorted;
    sorted.reserve(c->total);
    for (int b = 0; b < c->nbins; ++b) sorted.insert(sorted.end(), prep[b].sorted.begin(), prep[b].sorted.end());
    CGS_TRY(upload(c, c->d_sorted, sorted.data(), std::max<size_t>(sorted.size(), 1) * sizeof(int)));
    CGS_TRY(upload(c, c->d_bin_off, c->h_bin_off.data(), c->h_bin_off.size() * sizeof(long long)));
    c->setup_ms[0] = ms_since(t0);
    t0 = clk::now();
    // tap records (the device's nearest points decide the tile lists)
    CGS_CUDA(c, c->d_rec.ensure(std::max<long long>(c->total, 1) * sizeof(TapRecord)));
    const KbParams kb = kb_params(c);
    CGS_CUDA(c, launch_tap_records(c->d_k.as<double>(), c->d_sorted.as<int>(), c->total, kb, c->d_rec.as<TapRecord>(),
                                   c->stream));
    c->drec_valid = false;
    c->tiles_stale = false;
    std::vector<unsigned> nearest(std::max<long long>(c->total, 1));
    {
        DevBuf d_near;
        CGS_CUDA(c, d_near.ensure(nearest.size() * sizeof(unsigned)));
        CGS_CUDA(c, launch_record_nearest(c->d_rec.as<TapRecord>(), c->total, d_near.as<unsigned>(), c->stream));
        CGS_CUDA(c, cudaMemcpyAsync(nearest.data(), d_near.p, nearest.size() * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                    c->stream));
        CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    c->setup_ms[1] = ms_since(t0);
    t0 = clk::now();
    // the x passes' tiles: 8 columns (64-byte rows) where both passes run
    // half-pruned, else the strided passes' width
    const int tbx = fft_listed_cols(c->G[0], c->lo[0], c->I[0]);
    int tbs = fft_strided_cols(c->G[0]);
    if (tbx <= 0 || tbs % tbx != 0) tbs = tbx;
    c->sup_tb = tbx;
    c->spr_tb = tbs;
#pragma omp parallel for schedule(dynamic, 1)
    for (int b = 0; b < c->nbins; ++b) {
        tile_lists(c, nearest.data() + c->h_bin_off[b], c->h_bin_off[b + 1] - c->h_bin_off[b], prep[b]);
        if (tbx > 0)
            support_lists(c, nearest.data() + c->h_bin_off[b], c->h_bin_off[b + 1] - c->h_bin_off[b], tbx, tbs,
                          prep[b]);
    }
    c->sup_built = false;
    c->h_sup_off.assign(c->nbins + 1, 0);
    c->h_spr_off.assign(c->nbins + 1, 0);
    if (tbx > 0) {
        std::vector<int2> tiles, spr;
        std::vector<int> live;
        c->h_live_off.assign(c->nbins + 1, 0);
        for (int b = 0; b < c->nbins; ++b) {
            for (int b0 : prep[b].sup_cols) tiles.push_back(make_int2(b, b0));
            c->h_sup_off[b + 1] = (long long)tiles.size();
            for (int b0 : prep[b].spr_cols) spr.push_back(make_int2(b, b0));
            c->h_spr_off[b + 1] = (long long)spr.size();
            live.insert(live.end(), prep[b].live.begin(), prep[b].live.end());
            c->h_live_off[b + 1] = (long long)live.size();
        }
        CGS_TRY(upload(c, c->d_sup_tiles, tiles.data(), std::max<size_t>(tiles.size(), 1) * sizeof(int2)));
        c->h_sup_tiles = tiles;
        CGS_TRY(upload(c, c->d_spr_tiles, spr.data(), std::max<size_t>(spr.size(), 1) * sizeof(int2)));
        c->h_spr_tiles = spr;
        CGS_TRY(upload(c, c->d_live, live.data(), std::max<size_t>(live.size(), 1) * sizeof(int)));
        CGS_TRY(upload(c, c->d_live_off, c->h_live_off.data(), c->h_live_off.size() * sizeof(long long)));
        c->sup_built = true;
        // row masks of the forward y pass: it stores row y of column z only
        // when the x pass lists the column tile starting at y * Gz + zs * tb,
        // zs = z / tb (the x-pass tiles never straddle two rows: Gz % tb == 0)
        c->sup_rowmask_bs = 0;
        if (c->G[2] % tbx == 0 && c->G[1] % 32 == 0) {
            const int nzs = c->G[2] / tbx, wpr = c->G[1] / 32;
            const long long bs = (long long)nzs * wpr;
            std::vector<unsigned> rm((size_t)c->nbins * bs, 0u);
            for (int b = 0; b < c->nbins; ++b)
                for (long long J = c->h_sup_off[b]; J < c->h_sup_off[b + 1]; ++J) {
                    const int f = tiles[J].y, y = f / c->G[2], zs = (f % c->G[2]) / tbx;
                    rm[(size_t)b * bs + (size_t)zs * wpr + y / 32] |= 1u << (y % 32);
                }
            CGS_TRY(upload(c, c->d_sup_rowmask, rm.data(), rm.size() * sizeof(unsigned)));
            c->sup_rowmask_bs = bs;
        }
    }
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->setup_ms[2] = ms_since(t0);
    t0 = clk::now();
    c->csr_list = -1;
    CGS_TRY(ensure_csr(c));
    c->setup_ms[3] = ms_since(t0);
    t0 = clk::now();
    std::vector<int> tile_ptr;
    std::vector<int> tile_idx;
    std::vector<int> plane_rng;
    std::vector<long long> tp_off(c->nbins), ti_off(c->nbins);
    for (int b = 0; b < c->nbins; ++b) {
        tp_off[b] = (long long)tile_ptr.size();
        tile_ptr.insert(tile_ptr.end(), prep[b].tile_ptr.begin(), prep[b].tile_ptr.end());
        ti_off[b] = (long long)tile_idx.size();
        tile_idx.insert(tile_idx.end(), prep[b].tile_idx.begin(), prep[b].tile_idx.end());
        plane_rng.insert(plane_rng.end(), prep[b].plane_rng.begin(), prep[b].plane_rng.end());
    }
    CGS_TRY(upload(c, c->d_tile_ptr, tile_ptr.data(), tile_ptr.size() * sizeof(int)));
    CGS_TRY(upload(c, c->d_tile_idx, tile_idx.data(), std::max<size_t>(tile_idx.size(), 1) * sizeof(int)));
    CGS_TRY(upload(c, c->d_tile_ptr_off, tp_off.data(), tp_off.size() * sizeof(long long)));
    CGS_TRY(upload(c, c->d_tile_idx_off, ti_off.data(), ti_off.size() * sizeof(long long)));
    CGS_TRY(upload(c, c->d_plane_rng, plane_rng.data(), std::max<size_t>(plane_rng.size(), 2) * sizeof(int)));
    if (c->has_dcf) {
        std::vector<float> ds(c->total);
        for (long long j = 0; j < c->total; ++j) ds[j] = c->h_dcf[sorted[j]];
        CGS_TRY(upload(c, c->d_dcf_sorted, ds.data(), ds.size() * sizeof(float)));
    }
    CGS_CUDA(c, c->d_yv.ensure(std::max<long long>(c->total, 1) * c->nch * sizeof(float2)));
    // workspace for a group of bins
    const long long per_bin = (long long)c->nch * (c->Nl * c->G[2] + 2LL * c->I[0] * c->G[1] * c->G[2] + c->Ng) *
                              (long long)sizeof(float2);
    long long budget = c->p.workspace_bytes > 0 ? c->p.workspace_bytes : (64LL << 30);
    int wsb = (int)std::max<long long>(1, std::min<long long>(c->nbins, budget / std::max<long long>(per_bin, 1)));
    c->ws_bins = std::max(wsb, 1);
    const long long wsn = (long long)c->ws_bins * c->nch;
    CGS_CUDA(c, c->d_zbuf.ensure(wsn * c->Nl * c->G[2] * sizeof(float2)));
    CGS_CUDA(c, c->d_ybuf.ensure(wsn * (long long)c->I[0] * c->G[1] * c->G[2] * sizeof(float2)));
    CGS_CUDA(c, c->d_ybuf_adj.ensure(wsn * (long long)c->I[0] * c->G[1] * c->G[2] * sizeof(float2)));
    c->adj_slot.assign(c->ws_bins, -1);
    CGS_CUDA(c, c->d_grid.ensure(wsn * c->Ng * sizeof(float2)));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->setup_ms[4] = ms_since(t0);   // the remaining lists' uploads and the workspaces
    c->toep_valid = false;
    c->bins_dirty = false;
    return CGS_OK;
}

// ---------------------------------------------------------------------------
// chains
// ---------------------------------------------------------------------------

// The support lists describe the current tap records (not after
// cgs_update_trajectory_d until the lists are rebuilt).
bool support_pruned(const cgs_ctx* c) { return c->sup_prune && !c->tiles_stale && c->sup_built; }

// Zero the adjoint y-buffer slots [0, nb) that held other bins' columns
// before bins [b0, b0 + nb) are written there with pruning (the adjoint y
// pass reads whole planes).  During graph capture the clears become graph
// nodes; the host's slot record then describes the state after the graph.
int prepare_adj_slots(cgs_ctx* c, int b0, int nb, bool pruned)
{
    const long long slot = (long long)c->nch * c->I[0] * c->G[1] * c->G[2];
    for (int j = 0; j < nb; ++j) {
        if (!pruned) {
            c->adj_slot[j] = -1;   // every column written
        } else if (c->adj_slot[j] != b0 + j) {
            CGS_CUDA(c, cudaMemsetAsync(c->d_ybuf_adj.as<float2>() + j * slot, 0, (size_t)slot * sizeof(float2),
                                        c->stream));
            c->adj_slot[j] = b0 + j;
        }
    }
    return CGS_OK;
}

// x pass over bins [b0, b0 + nb): only the listed tiles
void set_support_tiles(const cgs_ctx* c, StridedPassArgs& a, int b0, int nb)
{
    a.sup_tiles = c->d_sup_tiles.as<int2>() + c->h_sup_off[b0];
    a.sup_ntiles = c->h_sup_off[b0 + nb] - c->h_sup_off[b0];
    a.sup_tb = c->sup_tb;
    a.sup_bin0 = b0;
    a.sup_nsub = c->nch;
}

// In a fused solve the forward z pass of bins [b0, ...) applies their pending
// CG updates while it reads the search direction x (== cgf.p + offset).
void set_cg_fusion(const cgs_ctx* c, FwdZArgs& fz, int b0, const float2* x)
{
    if (!c->cgf.st) return;
    const long long off = x - c->cgf.p;
    fz.cg = c->cgf.st + b0;
    fz.cg_p = c->cgf.p + off;
    fz.cg_r = c->cgf.r + off;
    fz.cg_x = c->cgf.x + off;
}

// Forward half for bins [b0, b0+nb) (nb <= ws_bins): image(s) -> grid -> samples (yv).
// x: per bin [Ni] (x_bs) shared by the coils, or per coil (x_cs) without coil maps.
int fwd_chain(cgs_ctx* c, int b0, int nb, const float2* x, long long x_bs, long long x_cs, bool use_smaps,
              bool use_dcf)
{
    const int Ix = c->I[0], Iy = c->I[1], Iz = c->I[2];
    const int Gx = c->G[0], Gy = c->G[1], Gz = c->G[2];
    const long long zb = c->Nl * Gz, yb = (long long)Ix * Gy * Gz;
    FwdZArgs fz{};
    fz.x = x;
    fz.x_cs = x_cs;
    fz.smaps = use_smaps ? c->d_smaps.as<float2>() : nullptr;
    fz.apx = c->ap[0].as<float>();
    fz.apy = c->ap[1].as<float>();
    fz.apz = c->ap[2].as<float>();
    fz.out = c->d_zbuf.as<float2>();
    fz.nl = c->Nl;
    fz.Iy = Iy;
    fz.Iz = Iz;
    fz.lo_z = c->lo[2];
    fz.nch = c->nch;
    fz.x_bs = x_bs;
    fz.out_bs = (long long)c->nch * zb;
    fz.err = c->d_err.as<int>();
    fz.coil_in = c->Ni;
    fz.coil_out = zb;
    fz.tw = c->tw[2].as<float2>();
    if (x_cs == 0) set_cg_fusion(c, fz, b0, x);
    CGS_LAUNCH(c, launch_fwd_z(Gz, fz, nb, c->stream));

    StridedPassArgs fy{};
    fy.in = c->d_zbuf.as<float2>();
    fy.out = c->d_ybuf.as<float2>();
    fy.in_bs = zb;
    fy.out_bs = yb;
    fy.in_as = (long long)Iy * Gz;
    fy.out_as = (long long)Gy * Gz;
    fy.B = Gz;
    fy.Lin = Iy;
    fy.in_off = c->lo[1];
    fy.Lout = Gy;
    fy.out_off = 0;
    fy.err = c->d_err.as<int>();
    fy.tw = c->tw[1].as<float2>();
    // only the rows of the tiles the forward x pass lists are stored
    const bool sup = support_pruned(c);
    if (sup && c->sup_rowmask_bs > 0) {
        fy.sup_rowmask = c->d_sup_rowmask.as<unsigned>() + (long long)b0 * c->sup_rowmask_bs;
        fy.sup_rowmask_bs = c->sup_rowmask_bs;
        fy.sup_rowmask_tb = c->sup_tb;
        fy.sup_nsub = c->nch;
    }
    CGS_LAUNCH(c, launch_strided(Gy, -1, fy, Ix, nb * c->nch, c->stream));

    StridedPassArgs fx{};
    fx.in = c->d_ybuf.as<float2>();
    fx.out = c->d_grid.as<float2>();
    fx.in_bs = yb;
    fx.out_bs = c->Ng;
    fx.in_as = 0;
    fx.out_as = 0;
    fx.B = Gy * Gz;
    fx.Lin = Ix;
    fx.in_off = c->lo[0];
    fx.Lout = Gx;
    fx.out_off = 0;
    fx.err = c->d_err.as<int>();
    fx.tw = c->tw[0].as<float2>();
    if (sup) set_support_tiles(c, fx, b0, nb);
    CGS_LAUNCH(c, launch_strided(Gx, -1, fx, 1, nb * c->nch, c->stream));

    InterpArgs ia{};
    ia.grid = c->d_grid.as<float2>();
    ia.coil_stride = c->Ng;
    ia.grid_bs = (long long)c->nch * c->Ng;
    ia.rec = c->d_rec.as<TapRecord>();
    ia.dcf = (use_dcf && c->has_dcf) ? c->d_dcf_sorted.as<float>() : nullptr;
    ia.bin_off = c->d_bin_off.as<long long>();
    ia.bin0 = b0;
    ia.yv = c->d_yv.as<float2>();
    ia.nch = c->nch;
    for (int a = 0; a < 3; ++a) ia.G[a] = c->G[a];
    ia.thresh = c->thresh;
    long long mx = 0;
    for (int b = b0; b < b0 + nb; ++b) mx = std::max(mx, c->h_bin_off[b + 1] - c->h_bin_off[b]);
    CGS_LAUNCH(c, launch_interp(ia, mx, nb, c->interp_cc, c->stream));
    return CGS_OK;
}

// Adjoint half for bins [b0, b0+nb): samples (yv) -> grid -> image.
// use_smaps: q[bin] = sum_c conj(S_c) (...) ; else q[coil] per coil (nb == 1).
// scale < 0: the reference's rescale adj_scale / sqrt(Ng) (Reco.cpp:482,
// Fourier.cpp:34); scale = 1: the exact adjoint of the forward chain.
int adj_chain(cgs_ctx* c, int b0, int nb, float2* q, long long q_bs, bool use_smaps, const float2* pdot,
              double* partials, double scale = -1.0)
{
    const int Ix = c->I[0], Iy = c->I[1], Iz = c->I[2];
    const int Gx = c->G[0], Gy = c->G[1], Gz = c->G[2];
    const long long zb = c->Nl * Gz, yb = (long long)Ix * Gy * Gz;
    const bool sup = support_pruned(c);
    {
        SpreadArgs sa{};
        sa.grid = c->d_grid.as<float2>();
        sa.coil_stride = c->Ng;
        sa.grid_bs = (long long)c->nch * c->Ng;
        sa.rec = c->d_rec.as<TapRecord>();
        sa.yv = c->d_yv.as<float2>();
        sa.bin_off = c->d_bin_off.as<long long>();
        sa.tile_ptr = c->d_tile_ptr.as<int>();
        sa.tile_ptr_off = c->d_tile_ptr_off.as<long long>();
        sa.tile_idx_off = c->d_tile_idx_off.as<long long>();
        sa.tile_idx = c->d_tile_idx.as<int>();
        sa.plane_rng = c->d_plane_rng.as<int2>();
        sa.bin0 = b0;
        sa.nch = c->nch;
        const int mc = c->spread_cc > 0 ? std::min(c->spread_cc, spread_max_coils(c->kahan)) : spread_max_coils(c->kahan);
        const int nchunk = (c->nch + mc - 1) / mc;
        sa.cc = (c->nch + nchunk - 1) / nchunk;
        for (int a = 0; a < 3; ++a) sa.G[a] = c->G[a];
        sa.ntx = c->ntx;
        sa.nty = c->nty;
        sa.ntz = c->ntz;
        sa.thresh = c->thresh;
        if (sup) {
            sa.live = c->d_live.as<int>();
            sa.live_off = c->d_live_off.as<long long>();
            for (int b = b0; b < b0 + nb; ++b)
                sa.live_max = (int)std::max<long long>(sa.live_max, c->h_live_off[b + 1] - c->h_live_off[b]);
        }
        // variant 8: the gather fused with the adjoint x pass (the listed
        // tiles of 8 columns of a half-pruned x pass); where it does not
        // apply, the staged gather and the x pass run as variant 6
        bool fused = false;
        if (sup && c->spread_wpp == 8 && c->csr_valid && c->csr_list == 1 && fused_spread_applies(c)) {
            CGS_TRY(prepare_adj_slots(c, b0, nb, sup));
            SpreadAdjxArgs fa{};
            fa.ptr = c->d_csr_ptr.as<unsigned>();
            fa.ent = c->d_csr_ent.as<int2>();
            fa.yv = c->d_yv.as<float2>();
            fa.tiles = c->d_sup_tiles.as<int2>();
            fa.j0 = c->h_sup_off[b0];
            fa.nj = c->h_sup_off[b0 + nb] - c->h_sup_off[b0];
            fa.bin0 = b0;
            fa.nch = c->nch;
            fa.B = (long long)Gy * Gz;
            fa.cc = (c->spread_cc == 2 || c->spread_cc == 4 || c->spread_cc == 6) ? c->spread_cc : 0;
            fa.out = c->d_ybuf_adj.as<float2>();
            fa.out_bs = yb;
            fa.tw = c->tw[0].as<float2>();
            fa.err = c->d_err.as<int>();
            const cudaError_t e = launch_spread_adjx(Gx, fa, c->kahan, c->stream);
            if (e == cudaSuccess) {
                ++c->launches;
                if (c->prof_ev) CGS_CUDA(c, cudaEventRecord(c->prof_ev[c->prof_n++], c->stream));
                fused = true;
            } else if (e == cudaErrorNotSupported) {
                cudaGetLastError();
            } else {
                CGS_CUDA(c, e);
            }
        }
        c->spread_fused = fused;
        if (fused) {
            // the adjoint y pass reads what the fused kernel stored
        } else if (sup && c->spread_wpp >= 6 && c->csr_valid) {
            // gather over the transposed tap matrix: stores the listed tiles' points
            CsrSpreadArgs ca{};
            ca.grid = c->d_grid.as<float2>();
            ca.coil_stride = c->Ng;
            ca.grid_bs = (long long)c->nch * c->Ng;
            ca.ptr = c->d_csr_ptr.as<unsigned>();
            ca.ent = c->d_csr_ent.as<int2>();
            ca.yv = c->d_yv.as<float2>();
            // the listing the matrix was built on
            const bool xl = c->csr_list == 1;
            const std::vector<long long>& off = xl ? c->h_sup_off : c->h_spr_off;
            ca.tiles = (xl ? c->d_sup_tiles : c->d_spr_tiles).as<int2>();
            ca.j0 = off[b0];
            ca.nj = off[b0 + nb] - off[b0];
            ca.bin0 = b0;
            ca.nch = c->nch;
            ca.Gx = Gx;
            ca.B = (long long)Gy * Gz;
            ca.tb = xl ? c->sup_tb : c->spr_tb;
            ca.cc = c->spread_cc;   // coils per thread of the gather (0: by the coil count)
            if (ca.cc != 2 && ca.cc != 4 && ca.cc != 6 && ca.cc != 8) ca.cc = 0;
            ca.err = c->d_err.as<int>();
            // variants 6 (and 8): the matrix staged in shared memory; 7: read from global memory
            CGS_LAUNCH(c, launch_spread_csr(ca, c->kahan, c->spread_wpp != 7, c->stream));
        } else {
            // variants 6 / 7 without their matrix: the two-warps-per-plane tiled kernel
            const int wpp = c->spread_wpp >= 6 ? 2 : c->spread_wpp;
            if (wpp == 2 && sa.cc < 2) sa.cc = std::min(2, c->nch);
            CGS_LAUNCH(c, launch_spread(sa, c->ntiles, nb, c->kahan, wpp, c->stream));
        }

        if (!fused) {
            CGS_TRY(prepare_adj_slots(c, b0, nb, sup));
            StridedPassArgs ax{};
            ax.in = c->d_grid.as<float2>();
            ax.out = c->d_ybuf_adj.as<float2>();
            ax.in_bs = c->Ng;
            ax.out_bs = yb;
            ax.B = Gy * Gz;
            ax.Lin = Gx;
            ax.in_off = 0;
            ax.Lout = Ix;
            ax.out_off = c->lo[0];
            ax.err = c->d_err.as<int>();
            ax.tw = c->tw[0].as<float2>();
            if (sup) set_support_tiles(c, ax, b0, nb);
            CGS_LAUNCH(c, launch_strided(Gx, +1, ax, 1, nb * c->nch, c->stream));
        }
    }

    StridedPassArgs ay{};
    ay.in = c->d_ybuf_adj.as<float2>();
    ay.out = c->d_zbuf.as<float2>();
    ay.in_bs = yb;
    ay.out_bs = zb;
    ay.in_as = (long long)Gy * Gz;
    ay.out_as = (long long)Iy * Gz;
    ay.B = Gz;
    ay.Lin = Gy;
    ay.in_off = 0;
    ay.Lout = Iy;
    ay.out_off = c->lo[1];
    ay.err = c->d_err.as<int>();
    ay.tw = c->tw[1].as<float2>();
    CGS_LAUNCH(c, launch_strided(Gy, +1, ay, Ix, nb * c->nch, c->stream));

    AdjZArgs az{};
    az.in = c->d_zbuf.as<float2>();
    az.smaps = use_smaps ? c->d_smaps.as<float2>() : nullptr;
    az.apx = c->ap[0].as<float>();
    az.apy = c->ap[1].as<float>();
    az.apz = c->ap[2].as<float>();
    az.scale = (float)(scale < 0 ? c->adj_scale_total : scale);
    az.q = q;
    az.p = pdot;
    az.partials = partials;
    az.nl = c->Nl;
    az.Iy = Iy;
    az.Iz = Iz;
    az.lo_z = c->lo[2];
    az.nch = c->nch;
    az.in_bs = (long long)c->nch * zb;
    az.q_bs = q_bs;
    az.coil_in = zb;
    az.coil_s = c->Ni;
    az.q_cs = c->Ni;
    az.tw = c->tw[2].as<float2>();
    az.err = c->d_err.as<int>();
    CGS_LAUNCH(c, launch_adj_z(Gz, az, nb, c->stream));
    return CGS_OK;
}

int centred_fft_dev(cgs_ctx* c, float2* a, int sign, int rescale);
int check_timeout(cgs_ctx* c);

// Fine grid of the PSF build: per axis the shortest line length with FFT
// kernels that is at least 4 I_a (two-fold oversampling of the 2 I_a modes
// of the point-spread function); false when an axis has none.
bool psf_fine_grid(const cgs_ctx* c, int nf[3])
{
    int n = 0;
    const int* list = fft_supported_list(&n);
    for (int a = 0; a < 3; ++a) {
        nf[a] = 0;
        for (int i = 0; i < n; ++i)
            if (list[i] >= 4 * c->I[a] && (nf[a] == 0 || list[i] < nf[a])) nf[a] = list[i];
        if (nf[a] == 0) return false;
    }
    return true;
}

// Spectra through the point-spread function of each bin (toeplitz.cu,
// k_psf_*): FP64 Kaiser-Bessel spreading of D onto the fine grid, the
// centred transform (sign +1) keeping the 2 I_a central positions per axis,
// deapodisation into the grid, the grid's centred transform (sign -1).
int build_toeplitz_psf(cgs_ctx* c, const int nf[3])
{
    constexpr double kW = 7.0;   // window width (window error ~5e-7 relative)
    const double beta = 0.5 * kTwoPi * std::sqrt(kW * kW / 4.0 * 1.5 * 1.5 - 0.8);
    const int* I = c->I;
    const long long nft = (long long)nf[0] * nf[1] * nf[2];
    const long long Ng = c->Ng;
    DevBuf bufA, bufB, bufG, tw[3], rcp[3];
    // A: FP64 fine grid, then the z pass's output, then the box R; B: the
    // complex fine grid, then the y pass's output, then the grid (when it fits)
    CGS_CUDA(c, bufA.ensure((size_t)nft * sizeof(double)));
    CGS_CUDA(c, bufB.ensure((size_t)nft * sizeof(float2)));
    float2* gbuf = bufB.as<float2>();
    if (Ng > nft) {
        CGS_CUDA(c, bufG.ensure((size_t)Ng * sizeof(float2)));
        gbuf = bufG.as<float2>();
    }
    for (int a = 0; a < 3; ++a) {
        std::vector<float2> t(nf[a]);
        for (int m = 0; m < nf[a]; ++m) {
            const double ang = -kTwoPi * (double)m / (double)nf[a];
            t[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
        }
        CGS_TRY(upload(c, tw[a], t.data(), t.size() * sizeof(float2)));
        // 1 / window transform at d / nf, d in [-I, I)
        std::vector<float> r(2 * I[a]);
        for (int j = 0; j < 2 * I[a]; ++j) {
            const double xi = (double)(j - I[a]) / (double)nf[a];
            const double z = beta * beta - (0.5 * kTwoPi * kW * xi) * (0.5 * kTwoPi * kW * xi);
            const double rt = std::sqrt(std::fabs(z));
            const double ft = rt == 0.0 ? kW : kW * (z > 0 ? std::sinh(rt) / rt : std::sin(rt) / rt);
            r[j] = (float)(1.0 / ft);
        }
        CGS_TRY(upload(c, rcp[a], r.data(), r.size() * sizeof(float)));
    }
    int sf = 0, sg = 0;
    for (int a = 0; a < 3; ++a) {
        sf += nf[a] / 2;
        sg += c->G[a] / 2;
    }
    const float sgn_f = (sf & 1) ? -1.f : 1.f;
    const float scale = (float)(c->adj_scale_total / (double)Ng) * ((sg & 1) ? -1.f : 1.f);
    for (int b = 0; b < c->nbins; ++b) {
        PsfSpreadArgs ps{};
        ps.k = c->d_k.as<double>();
        ps.sorted = c->d_sorted.as<int>();
        ps.dcf = c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr;
        ps.s0 = c->h_bin_off[b];
        ps.n = c->h_bin_off[b + 1] - c->h_bin_off[b];
        for (int a = 0; a < 3; ++a) {
            ps.G[a] = c->G[a];
            ps.nf[a] = nf[a];
        }
        ps.w = kW;
        ps.beta = beta;
        ps.out = bufA.as<double>();
        CGS_CUDA(c, cudaMemsetAsync(bufA.p, 0, (size_t)nft * sizeof(double), c->stream));
        CGS_LAUNCH(c, launch_psf_spread(ps, c->stream));
        CGS_LAUNCH(c, launch_psf_convert(bufA.as<double>(), bufB.as<float2>(), nft, c->stream));
        ContigPassArgs cz{};
        cz.in = bufB.as<float2>();
        cz.out = bufA.as<float2>();
        cz.nl = (long long)nf[0] * nf[1];
        cz.Lin = nf[2];
        cz.in_off = 0;
        cz.Lout = 2 * I[2];
        cz.out_off = nf[2] / 2 - I[2];
        cz.tw = tw[2].as<float2>();
        CGS_LAUNCH(c, launch_contig(nf[2], +1, cz, 1, c->stream));
        StridedPassArgs sy{};
        sy.in = bufA.as<float2>();
        sy.out = bufB.as<float2>();
        sy.in_as = (long long)nf[1] * 2 * I[2];
        sy.out_as = (long long)2 * I[1] * 2 * I[2];
        sy.B = 2 * I[2];
        sy.Lin = nf[1];
        sy.in_off = 0;
        sy.Lout = 2 * I[1];
        sy.out_off = nf[1] / 2 - I[1];
        sy.tw = tw[1].as<float2>();
        sy.err = c->d_err.as<int>();
        CGS_LAUNCH(c, launch_strided(nf[1], +1, sy, nf[0], 1, c->stream));
        StridedPassArgs sx{};
        sx.in = bufB.as<float2>();
        sx.out = bufA.as<float2>();
        sx.B = 2 * I[1] * 2 * I[2];
        sx.Lin = nf[0];
        sx.in_off = 0;
        sx.Lout = 2 * I[0];
        sx.out_off = nf[0] / 2 - I[0];
        sx.tw = tw[0].as<float2>();
        sx.err = c->d_err.as<int>();
        CGS_LAUNCH(c, launch_strided(nf[0], +1, sx, 1, 1, c->stream));
        CGS_LAUNCH(c, launch_psf_place(bufA.as<float2>(), rcp[0].as<float>(), rcp[1].as<float>(), rcp[2].as<float>(),
                                       c->G, I, sgn_f, gbuf, c->stream));
        CGS_TRY(centred_fft_dev(c, gbuf, -1, 0));
        CGS_LAUNCH(c, launch_psf_spectrum(gbuf, scale, Ng, c->d_toep.as<float>() + (long long)b * Ng, c->stream));
    }
    return CGS_OK;
}

// Toeplitz embedding: per bin the spectrum P of the point-spread function
// of its samples (current coordinates and density weights), scaled so that
// F_c^H P F_c between the unscaled passes is the gridded operator's
// adjoint scale times the exact E^H D E.
int build_toeplitz(cgs_ctx* c)
{
    for (int a = 0; a < 3; ++a)
        if (c->G[a] < 2 * c->I[a] - 1)
            return fail(c, CGS_ERR_ARG, "the Toeplitz embedding needs grid >= 2 x image - 1 on every axis");
    const long long Ng = c->Ng;
    CGS_CUDA(c, c->d_toep.ensure((size_t)std::max(c->nbins, 1) * Ng * sizeof(float)));
    // unit deapodisation vectors of the operator's z passes (either method)
    const int gmax = std::max(c->G[0], std::max(c->G[1], c->G[2]));
    if (c->d_ones.bytes < (size_t)gmax * sizeof(float)) {
        std::vector<float> one(gmax, 1.f);
        CGS_TRY(upload(c, c->d_ones, one.data(), one.size() * sizeof(float)));
    }
    int nf[3];
    if (c->toep_method == 0 && psf_fine_grid(c, nf)) {
        cudaEvent_t e0, e1;
        CGS_CUDA(c, cudaEventCreate(&e0));
        CGS_CUDA(c, cudaEventCreate(&e1));
        cudaEventRecord(e0, c->stream);
        int st = build_toeplitz_psf(c, nf);
        cudaEventRecord(e1, c->stream);
        const cudaError_t es = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (es == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st != CGS_OK) return st;
        CGS_CUDA(c, es);
        CGS_TRY(check_timeout(c));
        c->toep_build_ms = ms;
        c->toep_used = 1;
        c->toep_valid = true;
        c->toep_serial = c->traj_serial;
        return CGS_OK;
    }
    // work: a chunk of samples' Dirichlet tables and their (y, z) products (W
    // of at most 2^28 floats, the whole bin when it fits)
    const long long yz = (long long)c->G[1] * c->G[2];
    const long long per = yz + c->G[0] + c->G[1] + c->G[2];
    const long long chunk = std::max<long long>(1, std::min<long long>(std::max<long long>(c->max_bin, 1),
                                                                     std::max<long long>(64, (1LL << 28) / yz)));
    DevBuf work;
    CGS_CUDA(c, work.ensure((size_t)(chunk * per) * sizeof(float)));
    cudaEvent_t e0, e1;
    CGS_CUDA(c, cudaEventCreate(&e0));
    CGS_CUDA(c, cudaEventCreate(&e1));
    CGS_CUDA(c, cudaEventRecord(e0, c->stream));
    int st = CGS_OK;
    for (int b = 0; b < c->nbins && st == CGS_OK; ++b) {
        ToepBuildArgs a{};
        a.k = c->d_k.as<double>();
        a.sorted = c->d_sorted.as<int>();
        a.dcf = c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr;
        a.s0 = c->h_bin_off[b];
        a.n = c->h_bin_off[b + 1] - c->h_bin_off[b];
        for (int ax = 0; ax < 3; ++ax) {
            a.G[ax] = c->G[ax];
            a.I[ax] = c->I[ax];
        }
        a.scale = c->adj_scale_total / (double)Ng;
        a.P = c->d_toep.as<float>() + (long long)b * Ng;
        std::string e;
        if (toeplitz_build(a, work.as<float>(), chunk * per, &c->blas, c->stream, &e) != 0)
            st = fail(c, CGS_ERR_CUDA, "Toeplitz spectrum of bin " + std::to_string(b) + ": " + e);
    }
    cudaEventRecord(e1, c->stream);
    const cudaError_t es = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (es == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != CGS_OK) return st;
    CGS_CUDA(c, es);
    c->toep_build_ms = ms;
    c->toep_used = 2;
    c->toep_valid = true;
    c->toep_serial = c->traj_serial;
    return CGS_OK;
}

// q = c sum_c conj(S_c) crop F_c^H P F_c pad (S_c x) for bins [b0, b0 + nb)
// (nb <= ws_bins): the forward z and y passes without deapodisation, the x
// stage (forward x transform, P, adjoint x transform) in place on the y
// buffer, the adjoint y and z passes.
int toep_chain(cgs_ctx* c, int b0, int nb, const float2* x, float2* q, const float2* pdot, double* partials)
{
    const int Ix = c->I[0], Iy = c->I[1], Iz = c->I[2];
    const int Gx = c->G[0], Gy = c->G[1], Gz = c->G[2];
    const long long zb = c->Nl * Gz, yb = (long long)Ix * Gy * Gz;
    const float* one = c->d_ones.as<float>();
    FwdZArgs fz{};
    fz.x = x;
    fz.x_cs = 0;
    fz.smaps = c->d_smaps.as<float2>();
    fz.apx = one;
    fz.apy = one;
    fz.apz = one;
    fz.out = c->d_zbuf.as<float2>();
    fz.nl = c->Nl;
    fz.Iy = Iy;
    fz.Iz = Iz;
    fz.lo_z = c->lo[2];
    fz.nch = c->nch;
    fz.x_bs = c->Ni;
    fz.out_bs = (long long)c->nch * zb;
    fz.err = c->d_err.as<int>();
    fz.coil_in = c->Ni;
    fz.coil_out = zb;
    fz.tw = c->tw[2].as<float2>();
    set_cg_fusion(c, fz, b0, x);
    CGS_LAUNCH(c, launch_fwd_z(Gz, fz, nb, c->stream));

    StridedPassArgs fy{};
    fy.in = c->d_zbuf.as<float2>();
    fy.out = c->d_ybuf.as<float2>();
    fy.in_bs = zb;
    fy.out_bs = yb;
    fy.in_as = (long long)Iy * Gz;
    fy.out_as = (long long)Gy * Gz;
    fy.B = Gz;
    fy.Lin = Iy;
    fy.in_off = c->lo[1];
    fy.Lout = Gy;
    fy.out_off = 0;
    fy.err = c->d_err.as<int>();
    fy.tw = c->tw[1].as<float2>();
    CGS_LAUNCH(c, launch_strided(Gy, -1, fy, Ix, nb * c->nch, c->stream));

    const float* P = c->d_toep.as<float>() + (long long)b0 * c->Ng;
    StridedPassArgs tx{};
    tx.in = c->d_ybuf.as<float2>();
    tx.out = c->d_ybuf.as<float2>();
    tx.in_bs = yb;
    tx.out_bs = yb;
    tx.B = Gy * Gz;
    tx.Lin = Ix;
    tx.in_off = c->lo[0];
    tx.Lout = Ix;
    tx.out_off = c->lo[0];
    tx.err = c->d_err.as<int>();
    tx.tw = c->tw[0].as<float2>();
    cudaError_t ex = cudaErrorNotSupported;
    if (c->toep_mode == 1) ex = launch_toep_x(Gx, tx, P, c->Ng, c->nch, nb * c->nch, c->stream);
    if (ex == cudaSuccess) {
        ++c->launches;
        if (c->prof_ev) CGS_CUDA(c, cudaEventRecord(c->prof_ev[c->prof_n++], c->stream));
    } else if (ex == cudaErrorNotSupported) {
        cudaGetLastError();
        // unfused: forward x pass onto the grid, P, adjoint x pass back
        StridedPassArgs fx = tx;
        fx.out = c->d_grid.as<float2>();
        fx.out_bs = c->Ng;
        fx.Lout = Gx;
        fx.out_off = 0;
        CGS_LAUNCH(c, launch_strided(Gx, -1, fx, 1, nb * c->nch, c->stream));
        CGS_LAUNCH(c, launch_toep_mul(c->d_grid.as<float2>(), P, c->Ng, c->nch, nb * c->nch, c->stream));
        StridedPassArgs ax = tx;
        ax.in = c->d_grid.as<float2>();
        ax.in_bs = c->Ng;
        ax.Lin = Gx;
        ax.in_off = 0;
        CGS_LAUNCH(c, launch_strided(Gx, +1, ax, 1, nb * c->nch, c->stream));
    } else {
        CGS_CUDA(c, ex);
    }

    StridedPassArgs ay{};
    ay.in = c->d_ybuf.as<float2>();
    ay.out = c->d_zbuf.as<float2>();
    ay.in_bs = yb;
    ay.out_bs = zb;
    ay.in_as = (long long)Gy * Gz;
    ay.out_as = (long long)Iy * Gz;
    ay.B = Gz;
    ay.Lin = Gy;
    ay.in_off = 0;
    ay.Lout = Iy;
    ay.out_off = c->lo[1];
    ay.err = c->d_err.as<int>();
    ay.tw = c->tw[1].as<float2>();
    CGS_LAUNCH(c, launch_strided(Gy, +1, ay, Ix, nb * c->nch, c->stream));

    AdjZArgs az{};
    az.in = c->d_zbuf.as<float2>();
    az.smaps = c->d_smaps.as<float2>();
    az.apx = one;
    az.apy = one;
    az.apz = one;
    az.scale = 1.f;
    az.q = q;
    az.p = pdot;
    az.partials = partials;
    az.nl = c->Nl;
    az.Iy = Iy;
    az.Iz = Iz;
    az.lo_z = c->lo[2];
    az.nch = c->nch;
    az.in_bs = (long long)c->nch * zb;
    az.q_bs = c->Ni;
    az.coil_in = zb;
    az.coil_s = c->Ni;
    az.q_cs = c->Ni;
    az.tw = c->tw[2].as<float2>();
    az.err = c->d_err.as<int>();
    CGS_LAUNCH(c, launch_adj_z(Gz, az, nb, c->stream));
    return CGS_OK;
}

// q = A x for bins [b0, b0+nb) (all groups).  pdot/partials: fused <p, q>.
int apply_bins(cgs_ctx* c, int b0, int nb, const float2* x, float2* q, const float2* pdot, double* partials,
               int nblk)
{
    for (int g = b0; g < b0 + nb; g += c->ws_bins) {
        const int n = std::min(c->ws_bins, b0 + nb - g);
        const long long off = (long long)(g - b0) * c->Ni;
        if (c->toep_mode) {
            CGS_TRY(toep_chain(c, g, n, x + off, q + off, pdot ? pdot + off : nullptr,
                               partials ? partials + 2LL * (g - b0) * nblk : nullptr));
            continue;
        }
        CGS_TRY(fwd_chain(c, g, n, x + off, c->Ni, 0, true, true));
        CGS_TRY(adj_chain(c, g, n, q + off, c->Ni, true, pdot ? pdot + off : nullptr,
                          partials ? partials + 2LL * (g - b0) * nblk : nullptr));
    }
    return CGS_OK;
}

// A pipelined pass whose bounded wait ran out sets the context's flag; read
// it at the host synchronisation points.
int check_timeout(cgs_ctx* c)
{
    int h = 0;
    CGS_CUDA(c, cudaMemcpyAsync(&h, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (h) {
        CGS_CUDA(c, cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->stream));
        return fail(c, CGS_ERR_TIMEOUT, "a pipelined FFT pass timed out waiting for its copies");
    }
    return CGS_OK;
}

// need_tiles: the call spreads, so the tile lists must match the current
// coordinates (after cgs_update_trajectory_d they are rebuilt here).
int check_ready(cgs_ctx* c, bool need_smaps, bool need_tiles = true)
{
    if (!c) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set (cgs_set_trajectory)");
    if (need_smaps && !c->smaps_set) return fail(c, CGS_ERR_STATE, "no coil maps set (cgs_set_smaps)");
    if (need_tiles && c->tiles_stale) c->bins_dirty = true;
    CGS_TRY(rebuild_bins(c));
    if (c->toep_mode && (!c->toep_valid || c->toep_serial != c->traj_serial)) CGS_TRY(build_toeplitz(c));
    return CGS_OK;
}

int centred_fft_dev(cgs_ctx* c, float2* a, int sign, int rescale)
{
    const int Gx = c->G[0], Gy = c->G[1], Gz = c->G[2];
    ContigPassArgs cz{};
    cz.in = a;
    cz.out = a;
    cz.nl = (long long)Gx * Gy;
    cz.Lin = Gz;
    cz.in_off = 0;
    cz.Lout = Gz;
    cz.out_off = 0;
    cz.tw = c->tw[2].as<float2>();
    CGS_LAUNCH(c, launch_contig(Gz, sign, cz, 1, c->stream));
    StridedPassArgs sy{};
    sy.in = a;
    sy.out = a;
    sy.in_as = sy.out_as = (long long)Gy * Gz;
    sy.B = Gz;
    sy.Lin = sy.Lout = Gy;
    sy.tw = c->tw[1].as<float2>();
    sy.err = c->d_err.as<int>();
    CGS_LAUNCH(c, launch_strided(Gy, sign, sy, Gx, 1, c->stream));
    StridedPassArgs sx{};
    sx.in = a;
    sx.out = a;
    sx.B = Gy * Gz;
    sx.Lin = sx.Lout = Gx;
    sx.tw = c->tw[0].as<float2>();
    sx.err = c->d_err.as<int>();
    CGS_LAUNCH(c, launch_strided(Gx, sign, sx, 1, 1, c->stream));
    if (rescale) {
        // Fourier.cpp:31-41 rescales by 1/sqrt(N) after the backward transform;
        // the host API applies it here, the operator chains fold it into the
        // adjoint epilogue.
        return fail(c, CGS_ERR_ARG, "internal: rescale handled by caller");
    }
    return CGS_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

// derivative records for the current coordinates
int ensure_grad_records(cgs_ctx* c)
{
    if (c->drec_valid) return CGS_OK;
    CGS_CUDA(c, c->d_drec.ensure(std::max<long long>(c->total, 1) * sizeof(TapRecord)));
    CGS_CUDA(c, launch_tap_grad_records(c->d_k.as<double>(), c->d_sorted.as<int>(), c->total, kb_params(c),
                                        c->d_drec.as<TapRecord>(), c->stream));
    c->drec_valid = true;
    return CGS_OK;
}

PairGradArgs pair_args(const cgs_ctx* c, int b, int slot)
{
    PairGradArgs pa{};
    pa.grid = c->d_grid.as<float2>() + (long long)slot * c->nch * c->Ng;
    pa.coil_stride = c->Ng;
    pa.rec = c->d_rec.as<TapRecord>();
    pa.drec = c->d_drec.as<TapRecord>();
    pa.dcf = c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr;
    pa.sorted = c->d_sorted.as<int>();
    pa.s0 = c->h_bin_off[b];
    pa.n = c->h_bin_off[b + 1] - pa.s0;
    pa.nch = c->nch;
    for (int a = 0; a < 3; ++a) pa.G[a] = c->G[a];
    pa.thresh = c->thresh;
    pa.scale = (float)c->adj_scale_total;
    return pa;
}

extern "C" {

void cgs_default_params(cgs_params* p)
{
    std::memset(p, 0, sizeof(*p));
    p->n_ch = 1;
    p->kb_order = 5;
    p->kb_w = 4.25f;
    p->kb_b = 14.9086f;
    p->kb_thresh = 1e-7;
    p->adj_scale = 1e-3;
}

const char* cgs_last_error(const cgs_ctx* c) { return c ? c->err.c_str() : "null context"; }

int cgs_create(const cgs_params* p, cgs_ctx** out)
{
    if (!p || !out) return CGS_ERR_ARG;
    *out = nullptr;
    cgs_ctx* c = new cgs_ctx();
    c->p = *p;
    auto bad = [&](int code, const std::string& m) {
        static thread_local std::string last;
        last = m;
        std::fprintf(stderr, "cgs_create: %s\n", m.c_str());
        delete c;
        return code;
    };
    if (p->n_ch < 1) return bad(CGS_ERR_ARG, "n_ch must be >= 1");
    if (!(p->kb_w > 0.f && p->kb_w < 5.f)) return bad(CGS_ERR_ARG, "kb_w must be in (0, 5)");
    if (!(p->kb_b >= 0.f) || !(p->kb_thresh >= 0.0) || !std::isfinite(p->adj_scale))
        return bad(CGS_ERR_ARG, "kb_b and kb_thresh must be >= 0, adj_scale finite");
    for (int a = 0; a < 3; ++a) {
        const int g = p->grid[a], i = p->img[a];
        if (g < 2 || (g & 1)) return bad(CGS_ERR_ARG, "grid sizes must be even (Fourier.cpp:54,64)");
        if (!fft_supported(g)) return bad(CGS_ERR_UNSUPPORTED, "grid size " + std::to_string(g) + " has no FFT kernel");
        if (i < 1 || i > g) return bad(CGS_ERR_ARG, "image size must be in [1, grid]");
        const int lo = (g - i) / 2 + p->offcenter[a];
        if (lo < 0 || lo + i > g) return bad(CGS_ERR_ARG, "image box (offcenter) outside the grid");
        c->I[a] = i;
        c->G[a] = g;
        c->lo[a] = lo;
    }
    if (p->grid[0] > 2048 || p->grid[1] > 2048 || p->grid[2] > 1024) return bad(CGS_ERR_ARG, "grid too large");
    c->nch = p->n_ch;
    c->Ni = (long long)c->I[0] * c->I[1] * c->I[2];
    c->Ng = (long long)c->G[0] * c->G[1] * c->G[2];
    c->Nl = (long long)c->I[0] * c->I[1];
    c->device = p->device;
    if (cudaSetDevice(c->device) != cudaSuccess) return bad(CGS_ERR_CUDA, "cudaSetDevice failed");
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        return bad(CGS_ERR_CUDA, "cudaStreamCreate failed");
    c->stream = c->own_stream;
    if (kernels_init() != cudaSuccess) return bad(CGS_ERR_CUDA, "kernel attribute setup failed");
    // tap threshold: convFunction(0) * kb_thresh (Reco.cpp:716-717)
    double kb0 = 1.0;
    for (int a = 0; a < 3; ++a) kb0 *= kb_factor(*p, c->G[a], 0.0);
    c->thresh = (float)((double)(float)kb0 * p->kb_thresh);
    c->adj_scale_total = p->adj_scale / std::sqrt((double)c->Ng);
    for (int a = 0; a < 3; ++a) {
        const int L = c->G[a];
        std::vector<float2> tw(L);
        for (int m = 0; m < L; ++m) {
            const double ang = -kTwoPi * (double)m / (double)L;
            tw[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
        }
        if (upload(c, c->tw[a], tw.data(), L * sizeof(float2)) != CGS_OK) return bad(CGS_ERR_CUDA, c->err);
        c->apod_full[a] = deapod_axis(*p, L);
        std::vector<float> ap(c->I[a]);
        for (int i = 0; i < c->I[a]; ++i) ap[i] = (float)c->apod_full[a][i + c->lo[a]];
        if (upload(c, c->ap[a], ap.data(), ap.size() * sizeof(float)) != CGS_OK) return bad(CGS_ERR_CUDA, c->err);
    }
    c->ntx = (c->G[0] + TILE_X - 1) / TILE_X;
    c->nty = (c->G[1] + TILE_Y - 1) / TILE_Y;
    c->ntz = (c->G[2] + TILE_Z - 1) / TILE_Z;
    c->ntiles = c->ntx * c->nty * c->ntz;
    if (c->d_err.ensure(sizeof(int)) != cudaSuccess || cudaMemset(c->d_err.p, 0, sizeof(int)) != cudaSuccess)
        return bad(CGS_ERR_NOMEM, "error flag allocation failed");
    if (cudaMalloc(&c->d_smaps.p, (size_t)c->nch * c->Ni * sizeof(float2)) != cudaSuccess)
        return bad(CGS_ERR_NOMEM, "coil map allocation failed");
    c->d_smaps.bytes = (size_t)c->nch * c->Ni * sizeof(float2);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bad(CGS_ERR_CUDA, "set-up failed");
    *out = c;
    return CGS_OK;
}

void cgs_destroy(cgs_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    if (c->plain_plan_ok) cufftDestroy(c->plain_plan);
    if (c->z_plan_ok) cufftDestroy(c->z_plan);
    if (c->blas) toeplitz_release(c->blas);
    for (cudaEvent_t& e : c->e2e_ev)
        if (e) cudaEventDestroy(e);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

int cgs_set_stream(cgs_ctx* c, void* stream)
{
    if (!c) return CGS_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : c->own_stream;
    if (s != c->stream) drop_graphs(c);
    c->stream = s;
    return CGS_OK;
}

void* cgs_get_stream(const cgs_ctx* c) { return c ? (void*)c->stream : nullptr; }

int cgs_sync(cgs_ctx* c)
{
    if (!c) return CGS_ERR_ARG;
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_timeout(c);
}

int cgs_set_trajectory(cgs_ctx* c, const double* k, int64_t ns)
{
    if (!c || (!k && ns > 0) || ns < 0) return CGS_ERR_ARG;
    if (ns > (int64_t)0x7fffffff) return fail(c, CGS_ERR_ARG, "too many samples");
    for (int64_t i = 0; i < 3 * ns; ++i)
        if (!std::isfinite(k[i])) return fail(c, CGS_ERR_NONFINITE, "non-finite trajectory coordinate");
    c->h_k.assign(k, k + 3 * ns);
    c->ns = ns;
    c->k_host_stale = false;
    c->tiles_stale = false;
    ++c->traj_serial;
    CGS_TRY(upload(c, c->d_k, k, (size_t)(3 * std::max<int64_t>(ns, 1)) * sizeof(double)));
    c->bins.assign(1, std::vector<int>());
    c->bins[0].resize(ns);
    for (int64_t i = 0; i < ns; ++i) c->bins[0][i] = (int)i;
    c->has_dcf = false;
    c->h_dcf.clear();
    c->bins_dirty = true;
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return CGS_OK;
}

int cgs_set_mask(cgs_ctx* c, const uint8_t* mask)
{
    if (!c) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set");
    c->bins.assign(1, std::vector<int>());
    for (long long i = 0; i < c->ns; ++i)
        if (!mask || mask[i]) c->bins[0].push_back((int)i);
    c->bins_dirty = true;
    return CGS_OK;
}

int cgs_mask_from_data(cgs_ctx* c, const float* data)
{
    if (!c || !data) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set");
    std::vector<uint8_t> m(c->ns);
    for (long long i = 0; i < c->ns; ++i) m[i] = (data[2 * i] == 0.f && data[2 * i + 1] == 0.f) ? 0 : 1;
    return cgs_set_mask(c, m.data());
}

int cgs_set_bins(cgs_ctx* c, int32_t nbins, const int64_t* offsets, const int32_t* idx)
{
    if (!c || nbins < 1 || !offsets || nbins > 65535) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set");
    if (offsets[0] != 0) return fail(c, CGS_ERR_ARG, "offsets[0] must be 0");
    std::vector<std::vector<int>> bins(nbins);
    for (int b = 0; b < nbins; ++b) {
        if (offsets[b + 1] < offsets[b]) return fail(c, CGS_ERR_ARG, "offsets must be non-decreasing");
        for (int64_t j = offsets[b]; j < offsets[b + 1]; ++j) {
            if (idx[j] < 0 || idx[j] >= c->ns) return fail(c, CGS_ERR_ARG, "sample index out of range");
            bins[b].push_back(idx[j]);
        }
    }
    c->bins.swap(bins);
    c->bins_dirty = true;
    return CGS_OK;
}

int cgs_num_bins(const cgs_ctx* c) { return c ? (int)c->bins.size() : 0; }

int cgs_set_dcf(cgs_ctx* c, const float* dcf)
{
    if (!c) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set");
    if (!dcf) {
        c->has_dcf = false;
        c->h_dcf.clear();
    } else {
        for (long long i = 0; i < c->ns; ++i)
            if (!std::isfinite(dcf[i])) return fail(c, CGS_ERR_NONFINITE, "non-finite density weight");
        c->h_dcf.assign(dcf, dcf + c->ns);
        c->has_dcf = true;
    }
    c->bins_dirty = true;
    return CGS_OK;
}

int cgs_set_smaps(cgs_ctx* c, const float* maps)
{
    if (!c || !maps) return CGS_ERR_ARG;
    const size_t n = (size_t)c->nch * c->Ni * 2;
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(maps[i])) return fail(c, CGS_ERR_NONFINITE, "non-finite coil map value");
    CGS_CUDA(c, cudaMemcpyAsync(c->d_smaps.p, maps, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->smaps_set = true;
    return CGS_OK;
}

int cgs_set_smaps_d(cgs_ctx* c, const float* maps)
{
    if (!c || !maps) return CGS_ERR_ARG;
    CGS_CUDA(c, cudaMemcpyAsync(c->d_smaps.p, maps, (size_t)c->nch * c->Ni * sizeof(float2),
                                cudaMemcpyDeviceToDevice, c->stream));
    c->smaps_set = true;
    return CGS_OK;
}

int cgs_kernel_ft(cgs_ctx* c, float* kft)
{
    if (!c || !kft) return CGS_ERR_ARG;
    const int Gx = c->G[0], Gy = c->G[1], Gz = c->G[2];
    for (int i = 0; i < Gx; ++i)
        for (int j = 0; j < Gy; ++j)
            for (int k = 0; k < Gz; ++k) {
                const size_t e = ((size_t)i * Gy + j) * Gz + k;
                kft[2 * e] = (float)(c->apod_full[0][i] * c->apod_full[1][j] * c->apod_full[2][k]);
                kft[2 * e + 1] = 0.f;
            }
    return CGS_OK;
}

int cgs_fft3_d(cgs_ctx* c, float* grid, int32_t sign, int32_t rescale)
{
    if (!c || !grid || (sign != -1 && sign != 1)) return CGS_ERR_ARG;
    c->launches = 0;
    CGS_TRY(centred_fft_dev(c, reinterpret_cast<float2*>(grid), sign, 0));
    (void)rescale;
    return CGS_OK;
}

int cgs_fft3(cgs_ctx* c, float* grid, int32_t sign, int32_t rescale)
{
    if (!c || !grid || (sign != -1 && sign != 1)) return CGS_ERR_ARG;
    const size_t bytes = (size_t)c->Ng * sizeof(float2);
    CGS_CUDA(c, c->d_img.ensure(bytes));
    CGS_CUDA(c, cudaMemcpyAsync(c->d_img.p, grid, bytes, cudaMemcpyHostToDevice, c->stream));
    c->launches = 0;
    CGS_TRY(centred_fft_dev(c, c->d_img.as<float2>(), sign, 0));
    CGS_CUDA(c, cudaMemcpyAsync(grid, c->d_img.p, bytes, cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    CGS_TRY(check_timeout(c));
    if (rescale) {
        const double s = 1.0 / std::sqrt((double)c->Ng);
        for (size_t i = 0; i < 2 * (size_t)c->Ng; ++i) grid[i] = (float)((double)grid[i] * s);
    }
    return CGS_OK;
}

int cgs_nufft_fwd_d(cgs_ctx* c, const float* img, float* data)
{
    CGS_TRY(check_ready(c, false));
    if (!img || !data) return fail(c, CGS_ERR_ARG, "null pointer");
    if (c->nbins != 1) return fail(c, CGS_ERR_STATE, "cgs_nufft_fwd works on a single bin (mask)");
    c->launches = 0;
    CGS_CUDA(c, cudaMemsetAsync(data, 0, (size_t)c->nch * c->ns * sizeof(float2), c->stream));
    CGS_TRY(fwd_chain(c, 0, 1, reinterpret_cast<const float2*>(img), 0, c->Ni, false, false));
    CGS_LAUNCH(c, launch_scatter_samples(c->d_yv.as<float2>(), c->d_sorted.as<int>(), c->total, c->nch, c->ns,
                                         reinterpret_cast<float2*>(data), c->stream));
    return CGS_OK;
}

int cgs_nufft_adj_d(cgs_ctx* c, const float* data, float* img)
{
    CGS_TRY(check_ready(c, false));
    if (!img || !data) return fail(c, CGS_ERR_ARG, "null pointer");
    if (c->nbins != 1) return fail(c, CGS_ERR_STATE, "cgs_nufft_adj works on a single bin (mask)");
    c->launches = 0;
    CGS_LAUNCH(c, launch_gather_samples(reinterpret_cast<const float2*>(data), c->ns, c->d_sorted.as<int>(), c->total,
                                        c->nch, nullptr, c->d_yv.as<float2>(), c->stream));
    CGS_TRY(adj_chain(c, 0, 1, reinterpret_cast<float2*>(img), 0, false, nullptr, nullptr));
    return CGS_OK;
}

int cgs_estimate_smaps_d(cgs_ctx* c, const void* data, double radius, double eps, void* maps)
{
    CGS_TRY(check_ready(c, false));
    if (!data || !maps) return fail(c, CGS_ERR_ARG, "null pointer");
    if (c->nbins != 1) return fail(c, CGS_ERR_STATE, "coil maps are estimated from a single bin (mask)");
    if (!(radius > 0.0) || !(eps >= 0.0) || !(eps < 1.0)) return fail(c, CGS_ERR_ARG, "radius > 0, 0 <= eps < 1");
    c->launches = 0;
    DevBuf w, rss, mx;
    CGS_CUDA(c, w.ensure(std::max<long long>(c->total, 1) * sizeof(float)));
    CGS_CUDA(c, rss.ensure((size_t)c->Ni * sizeof(float)));
    CGS_CUDA(c, mx.ensure(sizeof(unsigned)));
    CGS_LAUNCH(c, launch_lowpass_weights(c->d_k.as<double>(), c->d_sorted.as<int>(), c->total, c->G, radius,
                                         c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr, w.as<float>(), c->stream));
    CGS_LAUNCH(c, launch_gather_samples(reinterpret_cast<const float2*>(data), c->ns, c->d_sorted.as<int>(), c->total,
                                        c->nch, w.as<float>(), c->d_yv.as<float2>(), c->stream));
    // per-coil images (no coil maps): the adjoint chain of bin 0
    CGS_TRY(adj_chain(c, 0, 1, reinterpret_cast<float2*>(maps), 0, false, nullptr, nullptr));
    CGS_LAUNCH(c, launch_smaps_from_images(reinterpret_cast<float2*>(maps), c->nch, c->Ni, (float)eps, rss.as<float>(),
                                           mx.as<unsigned>(), c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_timeout(c);
}

int cgs_nufft_fwd(cgs_ctx* c, const float* img, float* data)
{
    CGS_TRY(check_ready(c, false));
    if (!img || !data) return fail(c, CGS_ERR_ARG, "null pointer");
    const size_t bi = (size_t)c->nch * c->Ni * sizeof(float2), bd = (size_t)c->nch * c->ns * sizeof(float2);
    CGS_CUDA(c, c->d_img.ensure(bi));
    CGS_CUDA(c, c->d_data.ensure(bd));
    CGS_CUDA(c, cudaMemcpyAsync(c->d_img.p, img, bi, cudaMemcpyHostToDevice, c->stream));
    CGS_TRY(cgs_nufft_fwd_d(c, c->d_img.as<float>(), c->d_data.as<float>()));
    CGS_CUDA(c, cudaMemcpyAsync(data, c->d_data.p, bd, cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_timeout(c);
}

int cgs_nufft_adj(cgs_ctx* c, const float* data, float* img)
{
    CGS_TRY(check_ready(c, false));
    if (!img || !data) return fail(c, CGS_ERR_ARG, "null pointer");
    const size_t bi = (size_t)c->nch * c->Ni * sizeof(float2), bd = (size_t)c->nch * c->ns * sizeof(float2);
    CGS_CUDA(c, c->d_img.ensure(bi));
    CGS_CUDA(c, c->d_data.ensure(bd));
    CGS_CUDA(c, cudaMemcpyAsync(c->d_data.p, data, bd, cudaMemcpyHostToDevice, c->stream));
    CGS_TRY(cgs_nufft_adj_d(c, c->d_data.as<float>(), c->d_img.as<float>()));
    CGS_CUDA(c, cudaMemcpyAsync(img, c->d_img.p, bi, cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_timeout(c);
}

int cgs_apply_ehde_d(cgs_ctx* c, int32_t bin0, int32_t nb, const float* x, float* q)
{
    CGS_TRY(check_ready(c, true));
    if (!x || !q) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin0 < 0 || nb < 1 || bin0 + nb > c->nbins) return fail(c, CGS_ERR_ARG, "bin range out of bounds");
    c->launches = 0;
    return apply_bins(c, bin0, nb, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(q), nullptr, nullptr,
                      0);
}

int cgs_apply_ehde(cgs_ctx* c, int32_t bin, const float* x, float* q)
{
    CGS_TRY(check_ready(c, true));
    if (!x || !q) return fail(c, CGS_ERR_ARG, "null pointer");
    const size_t b = (size_t)c->Ni * sizeof(float2);
    CGS_CUDA(c, c->d_img.ensure(2 * b));
    CGS_CUDA(c, cudaMemcpyAsync(c->d_img.p, x, b, cudaMemcpyHostToDevice, c->stream));
    float2* dq = c->d_img.as<float2>() + c->Ni;
    CGS_TRY(cgs_apply_ehde_d(c, bin, 1, c->d_img.as<float>(), reinterpret_cast<float*>(dq)));
    CGS_CUDA(c, cudaMemcpyAsync(q, dq, b, cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_timeout(c);
}

// The whole batched solve is recorded once into a CUDA graph (per data/x
// pointers, threshold and iteration cap) and replayed.
static int record_solve(cgs_ctx* c, const float2* data, float2* x, double thresh, int max_iter,
                        bool rhs_from_images, float2* x_trace)
{
    const int nb = c->nbins;
    const long long Ni = c->Ni;
    const int nblk_adj = adj_z_blocks(c->G[2], c->Nl);
    const int nblk_cg = cg_blocks(Ni, nb);
    if (rhs_from_images) {
        // b = sum_c conj(S_c) img_c from given coil images (Reco.cpp:182-190)
        CGS_LAUNCH(c, launch_coil_combine(data, c->d_smaps.as<float2>(), c->nch, Ni, c->d_b.as<float2>(), c->stream));
    } else {
        // RHS: b = sum_c conj(S_c) E_c^H (D y_c)   (CGSense.cpp:226-235, Reco.cpp:182-190)
        CGS_LAUNCH(c, launch_gather_samples(data, c->ns, c->d_sorted.as<int>(), c->total, c->nch,
                                            c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr,
                                            c->d_yv.as<float2>(), c->stream));
        for (int g = 0; g < nb; g += c->ws_bins) {
            const int n = std::min(c->ws_bins, nb - g);
            CGS_TRY(adj_chain(c, g, n, c->d_b.as<float2>() + (long long)g * Ni, Ni, true, nullptr, nullptr));
        }
    }
    CgState* st = c->d_state.as<CgState>();
    CGS_LAUNCH(c, launch_cg_init(c->d_b.as<float2>(), c->d_r.as<float2>(), c->d_pv.as<float2>(), x, Ni, Ni,
                                 c->d_partials2.as<double>(), st, nb, c->stream));
    CGS_LAUNCH(c, launch_cg_arm(st, c->d_partials2.as<double>(), nblk_cg, nb, thresh, max_iter, c->stream));
    if (!x_trace) {
        // fused iteration: operator (its forward z pass applies the previous
        // iteration's x and p updates), alpha, r update, beta + loop test
        struct Scope {   // the fusion pointers never outlive the recording
            cgs_ctx* c;
            ~Scope() { c->cgf = {}; }
        } scope{c};
        c->cgf.st = st;
        c->cgf.p = c->d_pv.as<float2>();
        c->cgf.r = c->d_r.as<float2>();
        c->cgf.x = x;
        for (int it = 0; it < max_iter; ++it) {
            CGS_TRY(apply_bins(c, 0, nb, c->d_pv.as<float2>(), c->d_q.as<float2>(), c->d_pv.as<float2>(),
                               c->d_partials.as<double>(), nblk_adj));
            CGS_LAUNCH(c, launch_cg_alpha(st, c->d_partials.as<double>(), nblk_adj, nb, c->d_q.as<float2>(), Ni,
                                          c->stream));
            CGS_LAUNCH(c, launch_cg_update_r(c->d_r.as<float2>(), c->d_q.as<float2>(), Ni, Ni, st,
                                             c->d_partials2.as<double>(), nb, c->stream));
            CGS_LAUNCH(c, launch_cg_beta_test(st, c->d_partials2.as<double>(), nblk_cg, nb, c->d_res.as<double>(),
                                              max_iter, c->stream));
        }
        c->cgf = {};
        CGS_LAUNCH(c, launch_cg_finish_x(x, c->d_pv.as<float2>(), Ni, Ni, st, nb, c->stream));
        return CGS_OK;
    }
    for (int it = 0; it < max_iter; ++it) {
        CGS_TRY(apply_bins(c, 0, nb, c->d_pv.as<float2>(), c->d_q.as<float2>(), c->d_pv.as<float2>(),
                           c->d_partials.as<double>(), nblk_adj));
        CGS_LAUNCH(c, launch_cg_alpha(st, c->d_partials.as<double>(), nblk_adj, nb, c->d_q.as<float2>(), Ni, c->stream));
        CGS_LAUNCH(c, launch_cg_update_xr(x, c->d_r.as<float2>(), c->d_pv.as<float2>(), c->d_q.as<float2>(), Ni, Ni, st,
                                          c->d_partials2.as<double>(), nb, c->stream));
        CGS_LAUNCH(c, launch_cg_beta(st, c->d_partials2.as<double>(), nblk_cg, nb, c->d_res.as<double>(), max_iter,
                                     c->stream));
        CGS_LAUNCH(c, launch_cg_update_p(c->d_pv.as<float2>(), c->d_r.as<float2>(), Ni, Ni, st, nb, c->stream));
        CGS_LAUNCH(c, launch_cg_loop_test(st, nb, c->stream));
        if (x_trace)
            CGS_CUDA(c, cudaMemcpyAsync(x_trace + (long long)it * nb * Ni, x, (size_t)nb * Ni * sizeof(float2),
                                        cudaMemcpyDeviceToDevice, c->stream));
    }
    return CGS_OK;
}

// x_host / x_bytes: the host-buffer call's download of x, enqueued right
// after the graph, ahead of the iteration record's read-back, so that one
// synchronisation covers both.
static int solve_d(cgs_ctx* c, const float* data, float* x, double thresh, int32_t max_iter, double* residuals,
                   int32_t* iters, bool rhs_from_images, float* x_trace = nullptr, void* x_host = nullptr,
                   size_t x_bytes = 0)
{
    CGS_TRY(check_ready(c, true));
    if (!data || !x) return fail(c, CGS_ERR_ARG, "null pointer");
    if (thresh == -1.0) return fail(c, CGS_ERR_NO_THRESHOLD, "no threshold set for CG SENSE (Reco.cpp:192-196)");
    if (max_iter < 0 || max_iter > 10000) return fail(c, CGS_ERR_ARG, "max_iter out of range");
    const int nb = c->nbins;
    const long long Ni = c->Ni;
    const size_t vb = (size_t)nb * Ni * sizeof(float2);
    const int nblk_adj = adj_z_blocks(c->G[2], c->Nl);
    const int nblk_cg = cg_blocks(Ni, nb);
    CGS_CUDA(c, c->d_b.ensure(vb));
    CGS_CUDA(c, c->d_r.ensure(vb));
    CGS_CUDA(c, c->d_pv.ensure(vb));
    CGS_CUDA(c, c->d_q.ensure(vb));
    CGS_CUDA(c, c->d_state.ensure(nb * sizeof(CgState)));
    CGS_CUDA(c, c->d_partials.ensure((size_t)nb * nblk_adj * 2 * sizeof(double)));
    CGS_CUDA(c, c->d_partials2.ensure((size_t)nb * nblk_cg * 2 * sizeof(double)));
    CGS_CUDA(c, c->d_res.ensure((size_t)nb * std::max(max_iter, 1) * sizeof(double)));

    if (rhs_from_images && nb != 1) return fail(c, CGS_ERR_STATE, "coil-image right-hand side needs one bin");
    GraphKey key{data, x, thresh, max_iter, rhs_from_images ? 1 : 0, x_trace};
    auto it = c->graphs.find(key);
    cudaGraphExec_t exec = nullptr;
    if (it == c->graphs.end()) {
        // one group of bins: clear stale adjoint y-buffer slots now, so that the
        // graph holds no clears (with several groups the clears between them are
        // part of the graph)
        if (c->ws_bins >= nb) CGS_TRY(prepare_adj_slots(c, 0, nb, support_pruned(c)));
        c->launches = 0;
        const std::vector<int> entry = c->adj_slot;
        const auto tc0 = std::chrono::steady_clock::now();
        CGS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int st = record_solve(c, reinterpret_cast<const float2*>(data), reinterpret_cast<float2*>(x), thresh, max_iter,
                              rhs_from_images, reinterpret_cast<float2*>(x_trace));
        cudaGraph_t graph = nullptr;
        cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
        if (st != CGS_OK || ee != cudaSuccess) c->adj_slot = entry;   // nothing of the capture ran
        if (st != CGS_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        CGS_CUDA(c, ee);
        cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) c->adj_slot = entry;
        CGS_CUDA(c, ei);
        c->graphs[key] = exec;
        c->setup_ms[5] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tc0).count();
        c->graph_launches[key] = c->launches;
        c->graph_slots[key] = {entry, c->adj_slot};
    } else {
        exec = it->second;
        // the graph's clears assume the slot records it was captured with: a
        // slot recorded differently now is cleared (zeros suit any record)
        const auto& gs = c->graph_slots[key];
        const long long slot = (long long)c->nch * c->I[0] * c->G[1] * c->G[2];
        for (size_t j = 0; j < gs.first.size() && j < c->adj_slot.size(); ++j)
            if (c->adj_slot[j] != gs.first[j])
                CGS_CUDA(c, cudaMemsetAsync(c->d_ybuf_adj.as<float2>() + (long long)j * slot, 0,
                                            (size_t)slot * sizeof(float2), c->stream));
        c->adj_slot = gs.second;
    }
    c->launches = c->graph_launches[key];
    CGS_CUDA(c, cudaGraphLaunch(exec, c->stream));
    if (c->e2e_mark) CGS_CUDA(c, cudaEventRecord(c->e2e_ev[2], c->stream));
    if (x_host) CGS_CUDA(c, cudaMemcpyAsync(x_host, x, x_bytes, cudaMemcpyDeviceToHost, c->stream));
    if (c->e2e_mark) CGS_CUDA(c, cudaEventRecord(c->e2e_ev[3], c->stream));
    if (residuals || iters) {
        // the iteration record goes through a page-locked staging buffer of
        // the context (a copy into pageable memory would be staged by the
        // driver behind the call's other copies)
        const size_t sb = nb * sizeof(CgState), rb = (size_t)nb * std::max(max_iter, 1) * sizeof(double);
        if (c->h_stage_bytes < sb + rb) {
            if (c->h_stage) cudaFreeHost(c->h_stage);
            c->h_stage = nullptr;
            c->h_stage_bytes = 0;
            CGS_CUDA(c, cudaMallocHost(&c->h_stage, sb + rb));
            c->h_stage_bytes = sb + rb;
        }
        CgState* hs = reinterpret_cast<CgState*>(c->h_stage);
        double* hr = reinterpret_cast<double*>(static_cast<char*>(c->h_stage) + sb);
        CGS_CUDA(c, cudaMemcpyAsync(hs, c->d_state.p, sb, cudaMemcpyDeviceToHost, c->stream));
        if (residuals) CGS_CUDA(c, cudaMemcpyAsync(hr, c->d_res.p, rb, cudaMemcpyDeviceToHost, c->stream));
        CGS_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int b = 0; b < nb; ++b) {
            if (iters) iters[b] = hs[b].iter;
            if (residuals)
                for (int i = 0; i < max_iter; ++i)
                    residuals[(size_t)b * max_iter + i] = i < hs[b].iter ? hr[(size_t)b * max_iter + i] : 0.0;
        }
        CGS_TRY(check_timeout(c));
        for (int b = 0; b < nb; ++b)
            if (hs[b].error)
                return fail(c, CGS_ERR_NONFINITE, "NaN or INF value in image detected (bin " + std::to_string(b) + ")");
    }
    return CGS_OK;
}

int cgs_cg_solve_batched_d(cgs_ctx* c, const float* data, float* x, double thresh, int32_t max_iter,
                           double* residuals, int32_t* iters)
{
    return solve_d(c, data, x, thresh, max_iter, residuals, iters, false);
}

int cgs_cg_solve_trace_d(cgs_ctx* c, const float* data, float* x, double thresh, int32_t max_iter,
                         double* residuals, int32_t* iters, float* x_trace)
{
    if (!x_trace) return fail(c, CGS_ERR_ARG, "null trace pointer");
    return solve_d(c, data, x, thresh, max_iter, residuals, iters, false, x_trace);
}

int cgs_cg_solve_fp64_d(cgs_ctx* c, const float* data, double* x, double thresh, int32_t max_iter,
                        double* residuals, int32_t* iters, double* x_trace)
{
    CGS_TRY(check_ready(c, true));
    if (!data || !x) return fail(c, CGS_ERR_ARG, "null pointer");
    if (thresh == -1.0) return fail(c, CGS_ERR_NO_THRESHOLD, "no threshold set for CG SENSE (Reco.cpp:192-196)");
    if (max_iter < 0 || max_iter > 10000) return fail(c, CGS_ERR_ARG, "max_iter out of range");
    if (!c->z_plan_ok) {
        if (cufftPlan3d(&c->z_plan, c->G[0], c->G[1], c->G[2], CUFFT_Z2Z) != CUFFT_SUCCESS)
            return fail(c, CGS_ERR_CUDA, "cufftPlan3d (Z2Z) failed");
        c->z_plan_ok = true;
    }
    if (cufftSetStream(c->z_plan, c->stream) != CUFFT_SUCCESS) return fail(c, CGS_ERR_CUDA, "cufftSetStream failed");
    const long long Ni = c->Ni;
    CGS_CUDA(c, c->d64_grid.ensure(c->Ng * sizeof(double2)));
    CGS_CUDA(c, c->d64_y.ensure(std::max<long long>(c->max_bin, 1) * sizeof(double2)));
    CGS_CUDA(c, c->d64_r.ensure(Ni * sizeof(double2)));
    CGS_CUDA(c, c->d64_p.ensure(Ni * sizeof(double2)));
    CGS_CUDA(c, c->d64_q.ensure(Ni * sizeof(double2)));
    CGS_CUDA(c, c->d64_part.ensure(2048 * sizeof(double)));
    Fp64Args P{};
    for (int a2 = 0; a2 < 3; ++a2) {
        P.g.I[a2] = c->I[a2];
        P.g.G[a2] = c->G[a2];
        P.g.lo[a2] = c->lo[a2];
        P.ap[a2] = c->ap[a2].as<float>();
    }
    P.g.Ni = Ni;
    P.g.Ng = c->Ng;
    P.nch = c->nch;
    P.smaps = c->d_smaps.as<float2>();
    P.scale = c->adj_scale_total;
    P.thresh = c->thresh;
    P.plan = c->z_plan;
    P.s = c->stream;
    P.grid = c->d64_grid.as<double2>();
    P.y = c->d64_y.as<double2>();
    for (int b = 0; b < c->nbins; ++b) {
        const long long off = c->h_bin_off[b], n = c->h_bin_off[b + 1] - off;
        int it = 0;
        std::vector<double> res(std::max(max_iter, 1), 0.0);
        CGS_CUDA(c, fp64_solve_bin(P, c->d_rec.as<TapRecord>() + off, c->has_dcf ? c->d_dcf_sorted.as<float>() + off : nullptr,
                                   c->d_sorted.as<int>() + off, n, reinterpret_cast<const float2*>(data), c->ns,
                                   reinterpret_cast<double2*>(x) + (long long)b * Ni, c->d64_r.as<double2>(),
                                   c->d64_p.as<double2>(), c->d64_q.as<double2>(), c->d64_part.as<double>(), thresh,
                                   max_iter, res.data(), &it,
                                   x_trace ? reinterpret_cast<double2*>(x_trace) + (long long)b * Ni : nullptr,
                                   (long long)c->nbins * Ni));
        if (iters) iters[b] = it;
        if (residuals)
            for (int i = 0; i < max_iter; ++i) residuals[(size_t)b * max_iter + i] = res[i];
    }
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return CGS_OK;
}

int cgs_cg_solve_images(cgs_ctx* c, const float* coil_imgs, float* x, double thresh, int32_t max_iter,
                        double* residuals, int32_t* iters)
{
    CGS_TRY(check_ready(c, true));
    if (!coil_imgs || !x) return fail(c, CGS_ERR_ARG, "null pointer");
    if (c->nbins != 1) return fail(c, CGS_ERR_STATE, "cgs_cg_solve_images reconstructs one bin");
    const size_t bi = (size_t)c->nch * c->Ni * sizeof(float2), bx = (size_t)c->Ni * sizeof(float2);
    CGS_CUDA(c, c->d_img.ensure(bi));
    CGS_CUDA(c, c->d_x.ensure(bx));
    CGS_CUDA(c, cudaMemcpyAsync(c->d_img.p, coil_imgs, bi, cudaMemcpyHostToDevice, c->stream));
    int32_t it_local = 0;
    int st = solve_d(c, c->d_img.as<float>(), c->d_x.as<float>(), thresh, max_iter, residuals,
                     iters ? iters : &it_local, true);
    if (st != CGS_OK && st != CGS_ERR_NONFINITE) return st;
    CGS_CUDA(c, cudaMemcpyAsync(x, c->d_x.p, bx, cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return st;
}

int cgs_cg_solve_batched(cgs_ctx* c, const float* data, float* x, double thresh, int32_t max_iter,
                         double* residuals, int32_t* iters)
{
    CGS_TRY(check_ready(c, true));
    if (!data || !x) return fail(c, CGS_ERR_ARG, "null pointer");
    const size_t bd = (size_t)c->nch * c->ns * sizeof(float2);
    const size_t bx = (size_t)c->nbins * c->Ni * sizeof(float2);
    CGS_CUDA(c, c->d_data.ensure(bd));
    CGS_CUDA(c, c->d_x.ensure(bx));
    for (cudaEvent_t& e : c->e2e_ev)
        if (!e) CGS_CUDA(c, cudaEventCreate(&e));
    const void* hp[2] = {data, x};
    for (int j = 0; j < 2; ++j) {
        cudaPointerAttributes pa{};
        c->e2e_pinned[j] = cudaPointerGetAttributes(&pa, hp[j]) == cudaSuccess && pa.type == cudaMemoryTypeHost;
        cudaGetLastError();
    }
    CGS_CUDA(c, cudaEventRecord(c->e2e_ev[0], c->stream));
    CGS_CUDA(c, cudaMemcpyAsync(c->d_data.p, data, bd, cudaMemcpyHostToDevice, c->stream));
    CGS_CUDA(c, cudaEventRecord(c->e2e_ev[1], c->stream));
    std::vector<int32_t> it_local(c->nbins);
    c->e2e_mark = true;
    const int st = solve_d(c, c->d_data.as<float>(), c->d_x.as<float>(), thresh, max_iter, residuals,
                           iters ? iters : it_local.data(), false, nullptr, x, bx);
    c->e2e_mark = false;
    return st;
}

int cgs_cg_solve_plain_d(cgs_ctx* c, const float* data, float* x, double thresh, int32_t max_iter,
                         double* residuals, int32_t* iters)
{
    CGS_TRY(check_ready(c, true));
    if (!data || !x) return fail(c, CGS_ERR_ARG, "null pointer");
    if (thresh == -1.0) return fail(c, CGS_ERR_NO_THRESHOLD, "no threshold set for CG SENSE (Reco.cpp:192-196)");
    if (max_iter < 0 || max_iter > 10000) return fail(c, CGS_ERR_ARG, "max_iter out of range");
    const int nb = c->nbins;
    const long long Ni = c->Ni;
    const int nblk_cg = cg_blocks(Ni, 1);
    const int nblk_dot = cg_blocks(Ni, 1);
    if (!c->plain_plan_ok) {
        if (cufftPlan3d(&c->plain_plan, c->G[0], c->G[1], c->G[2], CUFFT_C2C) != CUFFT_SUCCESS)
            return fail(c, CGS_ERR_CUDA, "cufftPlan3d failed");
        c->plain_plan_ok = true;
    }
    if (cufftSetStream(c->plain_plan, c->stream) != CUFFT_SUCCESS) return fail(c, CGS_ERR_CUDA, "cufftSetStream failed");
    CGS_CUDA(c, c->d_plain_grid.ensure(c->Ng * sizeof(float2)));
    CGS_CUDA(c, c->d_plain_y.ensure(std::max<long long>(c->max_bin, 1) * sizeof(float2)));
    CGS_CUDA(c, c->d_plain_dot.ensure((size_t)nblk_dot * 2 * sizeof(double)));
    CGS_CUDA(c, c->d_b.ensure(Ni * sizeof(float2)));
    CGS_CUDA(c, c->d_r.ensure(Ni * sizeof(float2)));
    CGS_CUDA(c, c->d_pv.ensure(Ni * sizeof(float2)));
    CGS_CUDA(c, c->d_q.ensure(Ni * sizeof(float2)));
    CGS_CUDA(c, c->d_state.ensure(sizeof(CgState)));
    CGS_CUDA(c, c->d_partials2.ensure((size_t)nblk_cg * 2 * sizeof(double)));
    CGS_CUDA(c, c->d_res.ensure((size_t)nb * std::max(max_iter, 1) * sizeof(double)));
    PlainArgs P{};
    for (int a = 0; a < 3; ++a) {
        P.g.I[a] = c->I[a];
        P.g.G[a] = c->G[a];
        P.g.lo[a] = c->lo[a];
        P.ap[a] = c->ap[a].as<float>();
    }
    P.g.Ni = Ni;
    P.g.Ng = c->Ng;
    P.nch = c->nch;
    P.smaps = c->d_smaps.as<float2>();
    P.scale = (float)c->adj_scale_total;
    P.thresh = c->thresh;
    P.plan = c->plain_plan;
    P.s = c->stream;
    P.grid = c->d_plain_grid.as<float2>();
    P.y = c->d_plain_y.as<float2>();
    c->launches = 0;
    CgState* st = c->d_state.as<CgState>();
    std::vector<double> hres;
    for (int b = 0; b < nb; ++b) {
        const long long off = c->h_bin_off[b], n = c->h_bin_off[b + 1] - off;
        const TapRecord* rec = c->d_rec.as<TapRecord>() + off;
        const float* dcf = c->has_dcf ? c->d_dcf_sorted.as<float>() + off : nullptr;
        const int* sorted = c->d_sorted.as<int>() + off;
        float2* xb = reinterpret_cast<float2*>(x) + (long long)b * Ni;
        double* resb = c->d_res.as<double>() + (long long)b * std::max(max_iter, 1);
        CGS_CUDA(c, plain_rhs(P, rec, dcf, sorted, n, reinterpret_cast<const float2*>(data), c->ns, c->d_b.as<float2>(),
                              &c->launches));
        CGS_LAUNCH(c, launch_cg_init(c->d_b.as<float2>(), c->d_r.as<float2>(), c->d_pv.as<float2>(), xb, Ni, Ni,
                                     c->d_partials2.as<double>(), st, 1, c->stream));
        CGS_LAUNCH(c, launch_cg_arm(st, c->d_partials2.as<double>(), nblk_cg, 1, thresh, max_iter, c->stream));
        CgState hs{};
        for (int it = 0; it < max_iter; ++it) {
            // host-side loop test every iteration, as the reference's while loop
            CGS_CUDA(c, cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, c->stream));
            CGS_CUDA(c, cudaStreamSynchronize(c->stream));
            if (!hs.active) break;
            CGS_CUDA(c, plain_apply(P, rec, dcf, n, c->d_pv.as<float2>(), c->d_q.as<float2>(), &c->launches));
            CGS_LAUNCH(c, plain_dot(c->d_pv.as<float2>(), c->d_q.as<float2>(), Ni, c->d_plain_dot.as<double>(), nblk_dot,
                                    c->stream));
            CGS_LAUNCH(c, launch_cg_alpha(st, c->d_plain_dot.as<double>(), nblk_dot, 1, c->d_q.as<float2>(), Ni,
                                          c->stream));
            CGS_LAUNCH(c, launch_cg_update_xr(xb, c->d_r.as<float2>(), c->d_pv.as<float2>(), c->d_q.as<float2>(), Ni, Ni,
                                              st, c->d_partials2.as<double>(), 1, c->stream));
            CGS_LAUNCH(c, launch_cg_beta(st, c->d_partials2.as<double>(), nblk_cg, 1, resb, max_iter, c->stream));
            CGS_LAUNCH(c, launch_cg_update_p(c->d_pv.as<float2>(), c->d_r.as<float2>(), Ni, Ni, st, 1, c->stream));
            CGS_LAUNCH(c, launch_cg_loop_test(st, 1, c->stream));
        }
        CGS_CUDA(c, cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, c->stream));
        if (residuals) {
            hres.assign(std::max(max_iter, 1), 0.0);
            CGS_CUDA(c, cudaMemcpyAsync(hres.data(), resb, hres.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        c->stream));
        }
        CGS_CUDA(c, cudaStreamSynchronize(c->stream));
        if (iters) iters[b] = hs.iter;
        if (residuals)
            for (int i = 0; i < max_iter; ++i) residuals[(size_t)b * max_iter + i] = i < hs.iter ? hres[i] : 0.0;
        if (hs.error) return fail(c, CGS_ERR_NONFINITE, "NaN or INF value in image detected (bin " + std::to_string(b) + ")");
    }
    return CGS_OK;
}

int cgs_cg_solve(cgs_ctx* c, const float* data, float* x, double thresh, int32_t max_iter, double* residuals,
                 int32_t* iters)
{
    CGS_TRY(check_ready(c, true));
    if (c->nbins != 1) return fail(c, CGS_ERR_STATE, "cgs_cg_solve reconstructs one bin; use cgs_cg_solve_batched");
    return cgs_cg_solve_batched(c, data, x, thresh, max_iter, residuals, iters);
}

int64_t cgs_last_launch_count(const cgs_ctx* c) { return c ? c->launches : 0; }

void* cgs_alloc_host(size_t bytes)
{
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        p = std::malloc(bytes ? bytes : 1);   // no usable GPU: ordinary memory
    }
    return p;
}

void cgs_free_host(void* p)
{
    if (!p) return;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost) {
        cudaFreeHost(p);
    } else {
        cudaGetLastError();
        std::free(p);
    }
}

int cgs_profile_apply(cgs_ctx* c, int32_t bin0, int32_t nb, const float* x, float* q, float* stage_ms,
                      int32_t max_stages, int32_t* n_stages)
{
    CGS_TRY(check_ready(c, true));
    if (!x || !q || !stage_ms || max_stages < 1) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin0 < 0 || nb < 1 || bin0 + nb > c->nbins) return fail(c, CGS_ERR_ARG, "bin range out of bounds");
    const int groups = (nb + c->ws_bins - 1) / c->ws_bins;
    const int nev = 1 + 8 * groups;
    std::vector<cudaEvent_t> ev(nev);
    for (auto& e : ev) CGS_CUDA(c, cudaEventCreate(&e));
    CGS_CUDA(c, cudaEventRecord(ev[0], c->stream));
    c->prof_ev = ev.data() + 1;
    c->prof_n = 0;
    c->launches = 0;
    int st = apply_bins(c, bin0, nb, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(q), nullptr,
                        nullptr, 0);
    const int rec = c->prof_n;
    c->prof_ev = nullptr;
    c->prof_n = 0;
    if (st == CGS_OK) {
        CGS_CUDA(c, cudaStreamSynchronize(c->stream));
        const int ns = std::min(rec, (int)max_stages);
        for (int i = 0; i < ns; ++i) CGS_CUDA(c, cudaEventElapsedTime(&stage_ms[i], ev[i], ev[i + 1]));
        if (n_stages) *n_stages = ns;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return st;
}

int cgs_update_trajectory_d(cgs_ctx* c, const double* k)
{
    if (!c || !k) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set (cgs_set_trajectory)");
    CGS_CUDA(c, c->d_flag.ensure(sizeof(int)));
    CGS_CUDA(c, cudaMemsetAsync(c->d_flag.p, 0, sizeof(int), c->stream));
    CGS_CUDA(c, launch_check_finite(k, 3 * c->ns, c->d_flag.as<int>(), c->stream));
    int bad = 0;
    CGS_CUDA(c, cudaMemcpyAsync(&bad, c->d_flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (bad) return fail(c, CGS_ERR_NONFINITE, "non-finite trajectory coordinate");
    CGS_CUDA(c, cudaMemcpyAsync(c->d_k.p, k, (size_t)(3 * c->ns) * sizeof(double), cudaMemcpyDeviceToDevice,
                                c->stream));
    c->k_host_stale = true;
    c->tiles_stale = true;
    c->drec_valid = false;
    ++c->traj_serial;
    if (!c->bins_dirty)   // same samples, same sorted order: new tap records only
        CGS_CUDA(c, launch_tap_records(c->d_k.as<double>(), c->d_sorted.as<int>(), c->total, kb_params(c),
                                       c->d_rec.as<TapRecord>(), c->stream));
    return CGS_OK;
}

int cgs_loss_grad_d(cgs_ctx* c, int32_t bin, const void* x, const void* y, double* loss, void* grad_x, void* grad_k)
{
    CGS_TRY(check_ready(c, true, grad_x != nullptr));
    if (!x || !y || !loss) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin < 0 || bin >= c->nbins) return fail(c, CGS_ERR_ARG, "bin out of range");
    const long long s0 = c->h_bin_off[bin], n = c->h_bin_off[bin + 1] - s0;
    CGS_TRY(ensure_grad_records(c));
    // forward chain of the bin: every coil's grid (the interpolation it ends
    // with is recomputed below together with the derivatives)
    CGS_TRY(fwd_chain(c, bin, 1, reinterpret_cast<const float2*>(x), 0, 0, true, false));
    CGS_CUDA(c, c->d_gy.ensure(std::max<long long>(c->total, 1) * c->nch * sizeof(float2)));
    CGS_CUDA(c, launch_gather_samples(reinterpret_cast<const float2*>(y), c->ns, c->d_sorted.as<int>() + s0, n, c->nch,
                                      nullptr, c->d_gy.as<float2>() + s0 * c->nch, c->stream));
    const int nblk = interp_grad_blocks(n);
    CGS_CUDA(c, c->d_gpart.ensure((size_t)nblk * sizeof(double)));
    if (grad_k) CGS_CUDA(c, cudaMemsetAsync(grad_k, 0, (size_t)(3 * c->ns) * sizeof(float), c->stream));
    InterpGradArgs ga{};
    ga.grid = c->d_grid.as<float2>();
    ga.coil_stride = c->Ng;
    ga.rec = c->d_rec.as<TapRecord>();
    ga.drec = c->d_drec.as<TapRecord>();
    ga.ymeas = c->d_gy.as<float2>();
    ga.dcf = c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr;
    ga.sorted = c->d_sorted.as<int>();
    ga.s0 = s0;
    ga.n = n;
    ga.nch = c->nch;
    for (int a = 0; a < 3; ++a) ga.G[a] = c->G[a];
    ga.thresh = c->thresh;
    ga.rv = grad_x ? c->d_yv.as<float2>() : nullptr;
    ga.grad_k = reinterpret_cast<float*>(grad_k);
    ga.partials = c->d_gpart.as<double>();
    CGS_LAUNCH(c, launch_interp_grad(ga, c->stream));
    if (grad_x)   // sum_c conj(S_c) E_c^* (D r_c): the adjoint chain at the exact-adjoint scale
        CGS_TRY(adj_chain(c, bin, 1, reinterpret_cast<float2*>(grad_x), c->Ni, true, nullptr, nullptr, 1.0));
    std::vector<double> h(nblk);
    CGS_CUDA(c, cudaMemcpyAsync(h.data(), c->d_gpart.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    double L = 0.0;
    for (double v : h) L += v;
    *loss = L;
    return check_timeout(c);
}

int cgs_loss_grad_fp64_d(cgs_ctx* c, int32_t bin, const void* x, const void* y, double* loss, void* grad_x,
                         void* grad_k)
{
    CGS_TRY(check_ready(c, true, false));
    if (!x || !y || !loss) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin < 0 || bin >= c->nbins) return fail(c, CGS_ERR_ARG, "bin out of range");
    if (!c->z_plan_ok) {
        if (cufftPlan3d(&c->z_plan, c->G[0], c->G[1], c->G[2], CUFFT_Z2Z) != CUFFT_SUCCESS)
            return fail(c, CGS_ERR_CUDA, "cufftPlan3d (Z2Z) failed");
        c->z_plan_ok = true;
    }
    if (cufftSetStream(c->z_plan, c->stream) != CUFFT_SUCCESS) return fail(c, CGS_ERR_CUDA, "cufftSetStream failed");
    const long long s0 = c->h_bin_off[bin], n = c->h_bin_off[bin + 1] - s0;
    CGS_CUDA(c, c->d64_grid.ensure(c->Ng * sizeof(double2)));
    CGS_CUDA(c, c->d64_y.ensure(std::max<long long>(c->max_bin, 1) * sizeof(double2)));
    CGS_CUDA(c, c->d64_part.ensure(std::max<long long>((c->max_bin + 255) / 256, 2048) * sizeof(double)));
    Fp64Args P{};
    for (int a2 = 0; a2 < 3; ++a2) {
        P.g.I[a2] = c->I[a2];
        P.g.G[a2] = c->G[a2];
        P.g.lo[a2] = c->lo[a2];
        P.ap[a2] = c->ap[a2].as<float>();
    }
    P.g.Ni = c->Ni;
    P.g.Ng = c->Ng;
    P.nch = c->nch;
    P.smaps = c->d_smaps.as<float2>();
    P.scale = 1.0;
    P.thresh = c->thresh;
    P.plan = c->z_plan;
    P.s = c->stream;
    P.grid = c->d64_grid.as<double2>();
    P.y = c->d64_y.as<double2>();
    // tap threshold in double: kb_thresh times the kernel's peak (Reco.cpp:716-717)
    double peak = 1.0;
    for (int a = 0; a < 3; ++a) {
        const double dk = 1.0 / (double)(c->G[a] - 1);
        peak *= std::cyl_bessel_i(0.0, (double)c->p.kb_b) / (100.0 * c->p.kb_w * dk);
    }
    CGS_CUDA(c, fp64_loss_grad(P, c->d_k.as<double>(), c->d_sorted.as<int>() + s0, n,
                               c->has_dcf ? c->d_dcf_sorted.as<float>() + s0 : nullptr, c->p.kb_w, c->p.kb_b,
                               peak * c->p.kb_thresh, reinterpret_cast<const float2*>(y), c->ns,
                               reinterpret_cast<const double2*>(x), loss, reinterpret_cast<double2*>(grad_x),
                               reinterpret_cast<double*>(grad_k), c->d64_part.as<double>(), 0));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return CGS_OK;
}

int cgs_set_precision(cgs_ctx* c, int32_t mode)
{
    if (!c) return CGS_ERR_ARG;
    if (mode != CGS_PREC_FP32 && mode != CGS_PREC_COMPENSATED) return fail(c, CGS_ERR_ARG, "unknown precision mode");
    const bool k = mode == CGS_PREC_COMPENSATED;
    if (k != c->kahan) {
        c->kahan = k;
        if (k && c->spread_wpp >= 3 && c->spread_wpp <= 5) c->spread_wpp = 1;
        drop_graphs(c);
    }
    return CGS_OK;
}

// Project autotuner: times one batched E^H D E application of every bin for
// each candidate launch shape and keeps the fastest (first coils per
// spreading block with the interpolation fixed, then coils per
// interpolation thread).  times_ms (optional, max_times entries) receives
// the median time of every candidate in that order.
int cgs_autotune(cgs_ctx* c, float* times_ms, int32_t max_times, int32_t* n_times, int32_t* spread_cc,
                 int32_t* spread_wpp, int32_t* interp_cc)
{
    CGS_TRY(check_ready(c, true));
    // the candidates are shapes of the gridded operator's kernels: timed with
    // the Toeplitz embedding off
    struct ModeGuard {
        cgs_ctx* c;
        int mode;
        ~ModeGuard() { c->toep_mode = mode; }
    } guard{c, c->toep_mode};
    c->toep_mode = 0;
    const long long Ni = c->Ni;
    const int nb = c->nbins;
    DevBuf xb, qb;
    CGS_CUDA(c, xb.ensure((size_t)nb * Ni * sizeof(float2)));
    CGS_CUDA(c, qb.ensure((size_t)nb * Ni * sizeof(float2)));
    CGS_CUDA(c, cudaMemsetAsync(xb.p, 0, (size_t)nb * Ni * sizeof(float2), c->stream));
    cudaEvent_t e0, e1;
    CGS_CUDA(c, cudaEventCreate(&e0));
    CGS_CUDA(c, cudaEventCreate(&e1));
    std::vector<float> all;
    auto time_apply = [&](float& best) -> int {
        std::vector<float> t;
        for (int rep = 0; rep < 4; ++rep) {
            CGS_CUDA(c, cudaEventRecord(e0, c->stream));
            CGS_TRY(apply_bins(c, 0, nb, xb.as<float2>(), qb.as<float2>(), nullptr, nullptr, 0));
            CGS_CUDA(c, cudaEventRecord(e1, c->stream));
            CGS_CUDA(c, cudaEventSynchronize(e1));
            float ms = 0.f;
            CGS_CUDA(c, cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0) t.push_back(ms);   // the first run warms up
        }
        std::sort(t.begin(), t.end());
        best = t[t.size() / 2];
        all.push_back(best);
        return CGS_OK;
    };
    // coils per spreading block (the largest that fits, then halves, thirds,
    // quarters) x warps per x plane (1, 2)
    std::vector<int> sc;
    const int mc = std::min(c->nch, spread_max_coils(c->kahan));
    for (int d = 1; d <= 4; ++d) {
        const int v = (mc + d - 1) / d;
        if (std::find(sc.begin(), sc.end(), v) == sc.end()) sc.push_back(v);
    }
    float best = 1e30f;
    int best_sc = sc[0], best_wpp = 1;
    for (int wpp : {1, 2, 4, 5, 3, 7, 6, 8}) {
        if (wpp == 3 && (c->deterministic || c->kahan)) continue;
        if ((wpp == 4 || wpp == 5) && c->kahan) continue;
        if (wpp >= 6 && !support_pruned(c)) continue;
        // the gather's shape parameter is its coils per thread (per block when fused)
        const std::vector<int> cand = wpp == 8 ? std::vector<int>{2, 4, 6} : wpp >= 6 ? std::vector<int>{4, 6, 8} : sc;
        for (int v : cand) {
            if (wpp == 2 && v < 2) continue;
            if (wpp == 8 && c->nch % v != 0) continue;
            c->spread_cc = v;
            c->spread_wpp = wpp;
            CGS_TRY(ensure_csr(c));
            if (wpp >= 6 && !c->csr_valid) continue;
            float ms;
            CGS_TRY(time_apply(ms));
            if (ms < best) {
                best = ms;
                best_sc = v;
                best_wpp = wpp;
            }
        }
    }
    c->spread_wpp = best_wpp;
    c->spread_cc = best_sc;
    CGS_TRY(ensure_csr(c));
    best = 1e30f;
    int best_ic = c->interp_cc;
    for (int v : {1, 2, 4, 6, 8}) {
        c->interp_cc = v;
        float ms;
        CGS_TRY(time_apply(ms));
        if (ms < best) {
            best = ms;
            best_ic = v;
        }
    }
    c->interp_cc = best_ic;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    drop_graphs(c);
    if (times_ms)
        for (int i = 0; i < (int)all.size() && i < max_times; ++i) times_ms[i] = all[i];
    if (n_times) *n_times = (int32_t)all.size();
    if (spread_cc) *spread_cc = c->spread_cc;
    if (spread_wpp) *spread_wpp = c->spread_wpp;
    if (interp_cc) *interp_cc = c->interp_cc;
    return check_timeout(c);
}

int cgs_rhs_d(cgs_ctx* c, int32_t bin0, int32_t nb, const void* y, void* b)
{
    CGS_TRY(check_ready(c, true));
    if (!y || !b) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin0 < 0 || nb < 1 || bin0 + nb > c->nbins) return fail(c, CGS_ERR_ARG, "bin range out of bounds");
    CGS_CUDA(c, launch_gather_samples(reinterpret_cast<const float2*>(y), c->ns, c->d_sorted.as<int>(), c->total,
                                      c->nch, c->has_dcf ? c->d_dcf_sorted.as<float>() : nullptr, c->d_yv.as<float2>(),
                                      c->stream));
    for (int g = bin0; g < bin0 + nb; g += c->ws_bins) {
        const int n = std::min(c->ws_bins, bin0 + nb - g);
        CGS_TRY(adj_chain(c, g, n, reinterpret_cast<float2*>(b) + (long long)(g - bin0) * c->Ni, c->Ni, true, nullptr,
                          nullptr));
    }
    return check_timeout(c);
}

int cgs_apply_vjp_k_d(cgs_ctx* c, int32_t bin0, int32_t nb, const void* p, const void* v, void* grad_k)
{
    if (c && c->toep_mode)
        return fail(c, CGS_ERR_STATE, "the operator's trajectory derivative is that of the gridded operator: "
                                      "turn the Toeplitz embedding off (cgs_set_toeplitz 0)");
    CGS_TRY(check_ready(c, true, false));
    if (!p || !v || !grad_k) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin0 < 0 || nb < 1 || bin0 + nb > c->nbins) return fail(c, CGS_ERR_ARG, "bin range out of bounds");
    CGS_TRY(ensure_grad_records(c));
    CGS_CUDA(c, c->d_pa.ensure(std::max<long long>(c->total, 1) * c->nch * sizeof(float2)));
    CGS_CUDA(c, c->d_pda.ensure(std::max<long long>(c->total, 1) * c->nch * 3 * sizeof(float2)));
    const float2* P = reinterpret_cast<const float2*>(p);
    const float2* V = reinterpret_cast<const float2*>(v);
    for (int g = bin0; g < bin0 + nb; g += c->ws_bins) {
        const int n = std::min(c->ws_bins, bin0 + nb - g);
        const long long off = (long long)(g - bin0) * c->Ni;
        // pass 1: A = E S p and its derivatives, stored per sample
        CGS_TRY(fwd_chain(c, g, n, P + off, c->Ni, 0, true, false));
        for (int b = g; b < g + n; ++b) {
            PairGradArgs pa = pair_args(c, b, b - g);
            pa.outA = c->d_pa.as<float2>();
            pa.outdA = c->d_pda.as<float2>();
            CGS_LAUNCH(c, launch_pair_grad(pa, c->stream));
        }
        // pass 2: B = E S v, contracted with (A, dA)
        CGS_TRY(fwd_chain(c, g, n, V + off, c->Ni, 0, true, false));
        for (int b = g; b < g + n; ++b) {
            PairGradArgs pa = pair_args(c, b, b - g);
            pa.A = c->d_pa.as<float2>();
            pa.dA = c->d_pda.as<float2>();
            pa.grad_k = reinterpret_cast<float*>(grad_k);
            CGS_LAUNCH(c, launch_pair_grad(pa, c->stream));
        }
    }
    return check_timeout(c);
}

int cgs_rhs_vjp_k_d(cgs_ctx* c, int32_t bin0, int32_t nb, const void* y, const void* v, void* grad_k)
{
    CGS_TRY(check_ready(c, true, false));
    if (!y || !v || !grad_k) return fail(c, CGS_ERR_ARG, "null pointer");
    if (bin0 < 0 || nb < 1 || bin0 + nb > c->nbins) return fail(c, CGS_ERR_ARG, "bin range out of bounds");
    CGS_TRY(ensure_grad_records(c));
    CGS_CUDA(c, c->d_gy.ensure(std::max<long long>(c->total, 1) * c->nch * sizeof(float2)));
    // measured samples in sorted, coil-interleaved order (D is applied in the contraction)
    CGS_CUDA(c, launch_gather_samples(reinterpret_cast<const float2*>(y), c->ns, c->d_sorted.as<int>(), c->total,
                                      c->nch, nullptr, c->d_gy.as<float2>(), c->stream));
    const float2* V = reinterpret_cast<const float2*>(v);
    for (int g = bin0; g < bin0 + nb; g += c->ws_bins) {
        const int n = std::min(c->ws_bins, bin0 + nb - g);
        CGS_TRY(fwd_chain(c, g, n, V + (long long)(g - bin0) * c->Ni, c->Ni, 0, true, false));
        for (int b = g; b < g + n; ++b) {
            PairGradArgs pa = pair_args(c, b, b - g);
            pa.A = c->d_gy.as<float2>();
            pa.grad_k = reinterpret_cast<float*>(grad_k);
            CGS_LAUNCH(c, launch_pair_grad(pa, c->stream));
        }
    }
    return check_timeout(c);
}

uint64_t cgs_trajectory_serial(const cgs_ctx* c) { return c ? c->traj_serial : 0; }

// The state loop of CGSense.cpp:200-282: one reconstruction per state file,
// the next file read on a host thread while the current state runs.
int cgs_reconstruct_states(cgs_ctx* c, const char* const* files, int32_t n_files, int32_t sx, int32_t sy, int32_t sz,
                           const char* out_dir, double thresh, int32_t max_iter, int32_t write_rss, int32_t* iters)
{
    if (!c || !files || n_files < 1 || !out_dir) return CGS_ERR_ARG;
    if (c->ns == 0) return fail(c, CGS_ERR_STATE, "no trajectory set (cgs_set_trajectory)");
    if (!c->smaps_set) return fail(c, CGS_ERR_STATE, "no coil maps set (cgs_set_smaps)");
    if ((long long)sx * sy * sz != c->ns) return fail(c, CGS_ERR_ARG, "sx*sy*sz differs from the trajectory's samples");
    if (thresh == -1.0) return fail(c, CGS_ERR_NO_THRESHOLD, "no threshold set for CG SENSE (Reco.cpp:192-196)");
    const std::string dir = std::string(out_dir) + "/";
    mkdir(dir.c_str(), 0755);
    mkdir((dir + "results").c_str(), 0755);
    const long long ns = c->ns;
    const size_t bytes = (size_t)ns * c->nch * sizeof(float2);
    // pinned host buffers for two files, device buffers for one state
    void* hbuf[2] = {nullptr, nullptr};
    for (int i = 0; i < 2; ++i)
        if (cudaMallocHost(&hbuf[i], bytes) != cudaSuccess) {
            for (int j = 0; j < i; ++j) cudaFreeHost(hbuf[j]);
            return fail(c, CGS_ERR_NOMEM, "pinned host buffers");
        }
    auto release = [&]() {
        for (int i = 0; i < 2; ++i) cudaFreeHost(hbuf[i]);
    };
    auto read_file = [&](const char* path, void* h) -> int {
        std::FILE* f = std::fopen(path, "rb");
        if (!f) return CGS_ERR_IO;
        const size_t got = std::fread(h, 1, bytes, f);
        std::fclose(f);
        return got == bytes ? CGS_OK : CGS_ERR_IO;
    };
    int st = read_file(files[0], hbuf[0]);
    if (st != CGS_OK) {
        release();
        return fail(c, st, std::string("cannot read ") + files[0]);
    }
    DevBuf stage, data, img, rss, x, dglob;
    if (stage.ensure(bytes) != cudaSuccess || data.ensure(bytes) != cudaSuccess ||
        x.ensure((size_t)c->Ni * sizeof(float2)) != cudaSuccess) {
        release();
        return fail(c, CGS_ERR_NOMEM, "state buffers");
    }
    if (write_rss) {
        if (img.ensure((size_t)c->nch * c->Ni * sizeof(float2)) != cudaSuccess ||
            rss.ensure((size_t)c->Ni * sizeof(float)) != cudaSuccess) {
            release();
            return fail(c, CGS_ERR_NOMEM, "coil-image buffers");
        }
        if (c->has_dcf && (dglob.ensure((size_t)ns * sizeof(float)) != cudaSuccess ||
                           cudaMemcpyAsync(dglob.p, c->h_dcf.data(), (size_t)ns * sizeof(float),
                                           cudaMemcpyHostToDevice, c->stream) != cudaSuccess)) {
            release();
            return fail(c, CGS_ERR_CUDA, "density weights");
        }
    }
    std::vector<float2> coil0(ns);
    for (int k = 0; k < n_files && st == CGS_OK; ++k) {
        // the next file is read while this state is reconstructed (CGSense.cpp:205-215)
        int next_st = CGS_OK;
        std::thread reader;
        if (k + 1 < n_files) reader = std::thread([&, k]() { next_st = read_file(files[k + 1], hbuf[(k + 1) & 1]); });
        auto run = [&]() -> int {
            CGS_CUDA(c, cudaMemcpyAsync(stage.p, hbuf[k & 1], bytes, cudaMemcpyHostToDevice, c->stream));
            CGS_TRY(cgs_permute_samples_d(stage.p, data.p, sx, sy, sz, c->nch, c->stream));
            // excludeMissingData (Reco.cpp:681-696): samples whose channel-0 value is 0 + 0i
            CGS_CUDA(c, cudaMemcpyAsync(coil0.data(), data.p, (size_t)ns * sizeof(float2), cudaMemcpyDeviceToHost,
                                        c->stream));
            CGS_CUDA(c, cudaStreamSynchronize(c->stream));
            std::vector<int> keep;
            keep.reserve(ns);
            for (long long i = 0; i < ns; ++i)
                if (coil0[i].x != 0.f || coil0[i].y != 0.f) keep.push_back((int)i);
            c->bins.assign(1, std::move(keep));
            c->bins_dirty = true;
            if (write_rss) {
                // coil images of the density-corrected data and their root-sum-of-squares
                // (CGSense.cpp:226-244)
                CGS_CUDA(c, cudaMemcpyAsync(stage.p, data.p, bytes, cudaMemcpyDeviceToDevice, c->stream));
                if (c->has_dcf)
                    CGS_CUDA(c, launch_scale_samples(stage.as<float2>(), dglob.as<float>(), ns, c->nch, c->stream));
                CGS_TRY(cgs_nufft_adj_d(c, stage.as<float>(), img.as<float>()));
                CGS_TRY(cgs_rss_d(img.p, c->nch, c->Ni, rss.as<float>(), c->stream));
                CGS_TRY(cgs_export_float_bin((dir + "resultRssq.bin").c_str(), rss.p, c->Ni, 1, c->stream));
            }
            int it = 0;
            CGS_TRY(cgs_cg_solve_batched_d(c, data.as<float>(), x.as<float>(), thresh, max_iter, nullptr, &it));
            if (iters) iters[k] = it;
            const std::string out = dir + "results/b_state" + std::to_string(k) + ".bin";
            CGS_TRY(cgs_export_complex_bin(out.c_str(), x.p, c->Ni, 1, c->stream));
            return CGS_OK;
        };
        st = run();
        if (reader.joinable()) reader.join();
        if (st == CGS_OK && next_st != CGS_OK) st = fail(c, next_st, std::string("cannot read ") + files[k + 1]);
    }
    release();
    return st;
}

// Pipe-Menon density weights of every bin on the GPU: `iters` rounds of
// w <- w / (C * w), C * w = interpolation (Reco.cpp:539-550 without the FFT)
// of the spreading (Reco.cpp:492-504) of the weights on the bin's grid;
// then each bin's weights are divided by their maximum (as
// estimateDensityV3D normalises, functions.h:234-245).  dcf: float [ns],
// device or host (on_device), in the reference's sample order; samples in no
// bin get 0.
int cgs_pipe_menon_dcf(cgs_ctx* c, int32_t iters, float* dcf, int32_t on_device)
{
    CGS_TRY(check_ready(c, false));
    if (!dcf || iters < 1 || iters > 1000) return fail(c, CGS_ERR_ARG, "bad arguments");
    const long long n = c->total;
    DevBuf w, v, u;
    CGS_CUDA(c, w.ensure(std::max<long long>(n, 1) * sizeof(float)));
    CGS_CUDA(c, v.ensure(std::max<long long>(n, 1) * sizeof(float2)));
    CGS_CUDA(c, u.ensure(std::max<long long>(n, 1) * sizeof(float2)));
    CGS_CUDA(c, launch_pm_init(w.as<float>(), v.as<float2>(), n, c->stream));
    const long long grid_bs = c->Ng;   // one "coil" per bin
    for (int it = 0; it < iters; ++it) {
        for (int g = 0; g < c->nbins; g += c->ws_bins * c->nch) {
            // the workspace holds ws_bins * nch grids: as many single-coil bins at once
            const int nb = std::min(c->ws_bins * c->nch, c->nbins - g);
            SpreadArgs sa{};
            sa.grid = c->d_grid.as<float2>();
            sa.coil_stride = c->Ng;
            sa.grid_bs = grid_bs;
            sa.rec = c->d_rec.as<TapRecord>();
            sa.yv = v.as<float2>();
            sa.bin_off = c->d_bin_off.as<long long>();
            sa.tile_ptr = c->d_tile_ptr.as<int>();
            sa.tile_ptr_off = c->d_tile_ptr_off.as<long long>();
            sa.tile_idx_off = c->d_tile_idx_off.as<long long>();
            sa.tile_idx = c->d_tile_idx.as<int>();
            sa.plane_rng = c->d_plane_rng.as<int2>();
            sa.bin0 = g;
            sa.nch = 1;
            sa.cc = 1;
            for (int a = 0; a < 3; ++a) sa.G[a] = c->G[a];
            sa.ntx = c->ntx;
            sa.nty = c->nty;
            sa.ntz = c->ntz;
            sa.thresh = c->thresh;
            CGS_LAUNCH(c, launch_spread(sa, c->ntiles, nb, false, 1, c->stream));
            InterpArgs ia{};
            ia.grid = c->d_grid.as<float2>();
            ia.coil_stride = c->Ng;
            ia.grid_bs = grid_bs;
            ia.rec = c->d_rec.as<TapRecord>();
            ia.dcf = nullptr;
            ia.bin_off = c->d_bin_off.as<long long>();
            ia.bin0 = g;
            ia.yv = u.as<float2>();
            ia.nch = 1;
            for (int a = 0; a < 3; ++a) ia.G[a] = c->G[a];
            ia.thresh = c->thresh;
            long long mx = 0;
            for (int b = g; b < g + nb; ++b) mx = std::max(mx, c->h_bin_off[b + 1] - c->h_bin_off[b]);
            CGS_LAUNCH(c, launch_interp(ia, mx, nb, 2, c->stream));
        }
        CGS_CUDA(c, launch_pm_update(w.as<float>(), v.as<float2>(), u.as<float2>(), n, c->stream));
    }
    // per-bin normalisation by the maximum, scatter to the reference's order
    std::vector<float> hw(std::max<long long>(n, 1));
    std::vector<int> hs(std::max<long long>(n, 1));
    CGS_CUDA(c, cudaMemcpyAsync(hw.data(), w.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaMemcpyAsync(hs.data(), c->d_sorted.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<float> out(c->ns, 0.f);
    for (int b = 0; b < c->nbins; ++b) {
        float mx = 0.f;
        for (long long j = c->h_bin_off[b]; j < c->h_bin_off[b + 1]; ++j) mx = std::max(mx, hw[j]);
        const float inv = mx > 0.f ? 1.f / mx : 0.f;
        for (long long j = c->h_bin_off[b]; j < c->h_bin_off[b + 1]; ++j) out[hs[j]] = hw[j] * inv;
    }
    if (on_device)
        CGS_CUDA(c, cudaMemcpyAsync(dcf, out.data(), (size_t)c->ns * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    else
        std::copy(out.begin(), out.end(), dcf);
    CGS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_timeout(c);
}

int cgs_set_deterministic(cgs_ctx* c, int32_t on)
{
    if (!c) return CGS_ERR_ARG;
    c->deterministic = on != 0;
    if (c->deterministic && c->spread_wpp == 3) {
        c->spread_wpp = 1;
        drop_graphs(c);
    }
    return CGS_OK;
}

int cgs_set_toeplitz(cgs_ctx* c, int32_t mode)
{
    if (!c) return CGS_ERR_ARG;
    if (mode < 0 || mode > 2) return fail(c, CGS_ERR_ARG, "Toeplitz mode must be 0, 1 or 2");
    if (mode)
        for (int a = 0; a < 3; ++a)
            if (c->G[a] < 2 * c->I[a] - 1)
                return fail(c, CGS_ERR_ARG, "the Toeplitz embedding needs grid >= 2 x image - 1 on every axis");
    if (c->toep_mode != mode) drop_graphs(c);
    c->toep_mode = mode;
    if (!mode) {   // the spectra are rebuilt when the embedding is turned on again
        c->d_toep.release();
        c->toep_valid = false;
    }
    // with a trajectory and bins the spectra are built now, else at first use
    if (mode && c->ns > 0 && !c->bins.empty()) return check_ready(c, false, false);
    return CGS_OK;
}

int cgs_toeplitz_stats(cgs_ctx* c, double* build_ms, int64_t* bytes)
{
    if (!c) return CGS_ERR_ARG;
    if (build_ms) *build_ms = c->toep_valid ? c->toep_build_ms : 0.0;
    if (bytes) *bytes = c->toep_valid ? (int64_t)c->nbins * c->Ng * (int64_t)sizeof(float) : 0;
    return CGS_OK;
}

int cgs_set_toeplitz_spectrum(cgs_ctx* c, int32_t method)
{
    if (!c) return CGS_ERR_ARG;
    if (method < 0 || method > 1) return fail(c, CGS_ERR_ARG, "spectrum method must be 0 or 1");
    if (c->toep_method != method) {
        c->toep_method = method;
        c->toep_valid = false;
        drop_graphs(c);
        if (c->toep_mode && c->ns > 0 && !c->bins.empty()) return check_ready(c, false, false);
    }
    return CGS_OK;
}

int cgs_toeplitz_spectrum_method(const cgs_ctx* c) { return c && c->toep_valid ? c->toep_used : 0; }

int cgs_set_support_pruning(cgs_ctx* c, int32_t on)
{
    if (!c) return CGS_ERR_ARG;
    if (c->sup_prune != (on != 0)) drop_graphs(c);
    c->sup_prune = on != 0;
    return CGS_OK;
}

int cgs_support_stats(cgs_ctx* c, int64_t* listed_cols, int64_t* live_tiles)
{
    CGS_TRY(check_ready(c, false));
    const bool sup = support_pruned(c);
    const long long ncol = (long long)c->G[1] * c->G[2];
    const int tbx = c->sup_tb;
    for (int b = 0; b < c->nbins; ++b) {
        if (listed_cols)
            listed_cols[b] = sup ? std::min(ncol, (c->h_sup_off[b + 1] - c->h_sup_off[b]) * (long long)tbx) : ncol;
        if (live_tiles) live_tiles[b] = sup ? c->h_live_off[b + 1] - c->h_live_off[b] : c->ntiles;
    }
    return CGS_OK;
}

int cgs_forward_y_listed_rows(cgs_ctx* c, int32_t* listed)
{
    CGS_TRY(check_ready(c, false));
    if (!listed) return fail(c, CGS_ERR_ARG, "null pointer");
    *listed = (support_pruned(c) && c->sup_rowmask_bs > 0) ? 1 : 0;
    return CGS_OK;
}

int cgs_spread_fused(cgs_ctx* c, int32_t* fused)
{
    CGS_TRY(check_ready(c, false));
    if (!fused) return fail(c, CGS_ERR_ARG, "null pointer");
    *fused = c->spread_fused ? 1 : 0;
    return CGS_OK;
}

int cgs_spread_matrix_stats(cgs_ctx* c, int64_t* taps, int64_t* points)
{
    CGS_TRY(check_ready(c, false));
    if (taps) *taps = c->csr_valid ? (int64_t)c->csr_entries : 0;
    if (points) *points = c->csr_valid ? (int64_t)c->csr_pts : 0;
    return CGS_OK;
}

int cgs_setup_stats(cgs_ctx* c, double* ms, int32_t n)
{
    if (!c || (!ms && n > 0) || n < 0) return CGS_ERR_ARG;
    for (int i = 0; i < n && i < 6; ++i) ms[i] = c->setup_ms[i];
    return CGS_OK;
}

int cgs_e2e_stats(cgs_ctx* c, double* ms, int32_t* pinned)
{
    if (!c || !ms) return CGS_ERR_ARG;
    if (pinned) {
        pinned[0] = c->e2e_pinned[0];
        pinned[1] = c->e2e_pinned[1];
    }
    for (const cudaEvent_t& e : c->e2e_ev)
        if (!e) return fail(c, CGS_ERR_STATE, "no host-buffer solve has run (cgs_cg_solve_batched)");
    for (int i = 0; i < 3; ++i) {
        float t = 0.f;
        CGS_CUDA(c, cudaEventElapsedTime(&t, c->e2e_ev[i], c->e2e_ev[i + 1]));
        ms[i] = t;
    }
    return CGS_OK;
}

int cgs_set_launch_shape(cgs_ctx* c, int32_t spread_cc, int32_t spread_variant, int32_t interp_cc)
{
    if (!c) return CGS_ERR_ARG;
    if (spread_cc < 0 || spread_cc > spread_max_coils(c->kahan)) return fail(c, CGS_ERR_ARG, "spread_cc out of range");
    if (spread_variant < 1 || spread_variant > 8 || (spread_variant >= 3 && spread_variant <= 5 && c->kahan) ||
        (spread_variant == 3 && c->deterministic))
        return fail(c, CGS_ERR_ARG, "spreading variant not allowed here");
    if (interp_cc != 1 && interp_cc != 2 && interp_cc != 4 && interp_cc != 6 && interp_cc != 8)
        return fail(c, CGS_ERR_ARG, "interp_cc must be 1, 2, 4, 6 or 8");
    c->spread_cc = spread_cc;
    c->spread_wpp = spread_variant;
    c->interp_cc = interp_cc;
    drop_graphs(c);
    return ensure_csr(c);
}

}  // extern "C"
