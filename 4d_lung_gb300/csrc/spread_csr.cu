// spread_csr.cu -- spreading (Reco.cpp:492-504) as a gather over the
// transposed tap matrix.
//
// The tap set of a trajectory is fixed, so its transpose is built once per
// set of tap records: for every grid point of the listed column tiles (the
// unfused gather's 16-column tiles, or the x passes' own tiles for the gather
// fused with the adjoint x pass; either covers every point the adjoint x
// pass reads), the (sample, weight) pairs of the taps that land on it.  Rows are ordered by (nearest x, sorted sample
// position) -- the order in which the tiled spreading kernels add the
// samples to a grid point -- so the gather sums every point in the same
// order with the same fused multiply-adds and gives bitwise the same grid.
// One thread owns a grid point and a chunk of coils, sums in registers and
// stores once: no shared-memory read-modify-write chains, no barriers, and
// every point of the listed tiles is stored (zeros where no tap lands).
#include "launch.h"
#include "gridding_common.cuh"
#include "ptx_async.cuh"

namespace cgs {

// Taps of sorted sample i: the same products and tests as the tiled
// spreading (weight (wx wy) wz, every factor non-zero, above the threshold).
template <bool FILL>
__global__ void __launch_bounds__(128) k_csr_taps(CsrBuildArgs a)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.total) return;
    int lo = 0, hi = a.nbins;   // bin: bin_off[bin] <= i < bin_off[bin + 1]
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (a.bin_off[mid] <= i) lo = mid;
        else hi = mid;
    }
    const int bin = lo;
    float w[15];
    int nx, ny, nz;
    load_record(a.rec, i, w, nx, ny, nz);
    const int Gx = a.G[0], Gz = a.G[2];
    const long long ncol = (long long)a.G[1] * Gz;
    const int* ct = a.col_tile + (long long)bin * ncol;
#pragma unroll
    for (int jx = 0; jx < 5; ++jx) {
        const float wx = w[jx];
        if (wx == 0.f) continue;
        const int x = nx - 2 + jx;
#pragma unroll
        for (int jy = 0; jy < 5; ++jy) {
            const float wy = w[5 + jy];
            if (wy == 0.f) continue;
            const int y = ny - 2 + jy;
#pragma unroll
            for (int jz = 0; jz < 5; ++jz) {
                const float wz = w[10 + jz];
                const float wt = (wx * wy) * wz;
                if (wz == 0.f || !(wt > a.thresh)) continue;
                const long long f = (long long)y * Gz + (nz - 2 + jz);
                const int J = ct[f];
                if (J < 0 || x < 0 || x >= Gx) {   // cannot happen: the lists hold every support column
                    atomicExch(a.err, 1);
                    continue;
                }
                const long long p = ((long long)J * Gx + x) * a.tb + (int)(f % a.tb);
                if (FILL) {
                    const unsigned slot = atomicAdd(a.cnt + p, 1u);
                    a.ent[a.ptr[p] + slot] = make_int2((int)i, __float_as_int(wt));
                } else {
                    atomicAdd(a.cnt + p, 1u);
                }
            }
        }
    }
}

// Order each row by (nearest x, sorted position): insertion sort (rows hold
// a few to a few tens of taps).
__global__ void k_csr_order(CsrBuildArgs a, long long npts)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const unsigned e0 = a.ptr[p], e1 = a.ptr[p + 1];
    auto key = [&](int2 e) {
        const unsigned nr = __float_as_uint(__ldg(&a.rec[e.x].q[3].w));
        return ((unsigned long long)(nr & 2047u) << 32) | (unsigned)e.x;
    };
    for (unsigned q = e0 + 1; q < e1; ++q) {
        const int2 v = a.ent[q];
        const unsigned long long kv = key(v);
        unsigned r = q;
        while (r > e0 && key(a.ent[r - 1]) > kv) {
            a.ent[r] = a.ent[r - 1];
            --r;
        }
        a.ent[r] = v;
    }
}

// ---------------------------------------------------------------------------
// exclusive scan of unsigned counts (three-level block scan)
// ---------------------------------------------------------------------------
constexpr int SCAN_T = 512, SCAN_PER = 4, SCAN_CHUNK = SCAN_T * SCAN_PER;

// out[j] = sum of in[0..j) within each chunk; sums[chunk] = chunk total
__global__ void __launch_bounds__(SCAN_T) k_scan_chunk(const unsigned* __restrict__ in, long long n,
                                                       unsigned* __restrict__ out, unsigned* __restrict__ sums)
{
    __shared__ unsigned s_w[SCAN_T / 32];
    const long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_PER;
    unsigned v[SCAN_PER], t = 0;
#pragma unroll
    for (int q = 0; q < SCAN_PER; ++q) {
        v[q] = base + q < n ? in[base + q] : 0u;
        t += v[q];
    }
    // inclusive scan of the thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned inc = t;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned ws = lane < SCAN_T / 32 ? s_w[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned o = __shfl_up_sync(0xffffffffu, ws, d);
            if (lane >= d) ws += o;
        }
        if (lane < SCAN_T / 32) s_w[lane] = ws;
    }
    __syncthreads();
    unsigned run = inc - t + (warp > 0 ? s_w[warp - 1] : 0u);
#pragma unroll
    for (int q = 0; q < SCAN_PER; ++q) {
        if (base + q < n) out[base + q] = run;
        run += v[q];
    }
    if (threadIdx.x == SCAN_T - 1) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(unsigned* __restrict__ out, long long n, const unsigned* __restrict__ offs)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] += offs[j / SCAN_CHUNK];
}

size_t csr_scan_tmp_elems(long long n)
{
    size_t e = 0;
    for (long long m = (n + SCAN_CHUNK - 1) / SCAN_CHUNK; m > 1; m = (m + SCAN_CHUNK - 1) / SCAN_CHUNK) e += 2 * (size_t)m;
    return e + 2;
}

// out[j] = sum in[0..j) for j < n; tmp holds the per-level chunk sums
static cudaError_t scan_exclusive(const unsigned* in, long long n, unsigned* out, unsigned* tmp, cudaStream_t s)
{
    const long long nchunk = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    unsigned* sums = tmp;
    unsigned* sums_scan = tmp + nchunk;
    k_scan_chunk<<<(unsigned)nchunk, SCAN_T, 0, s>>>(in, n, out, sums);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || nchunk == 1) return e;
    e = scan_exclusive(sums, nchunk, sums_scan, tmp + 2 * nchunk, s);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, sums_scan);
    return cudaGetLastError();
}

cudaError_t csr_count_and_scan(const CsrBuildArgs& a, long long npts, unsigned* ptr, unsigned* scan_tmp,
                               size_t scan_tmp_elems, unsigned long long* entries, cudaStream_t s)
{
    if (scan_tmp_elems < csr_scan_tmp_elems(npts + 1)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a.cnt, 0, (size_t)(npts + 1) * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    if (a.total > 0) {
        k_csr_taps<false><<<(unsigned)((a.total + 127) / 128), 128, 0, s>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // ptr[p] = taps before point p; ptr[npts] = all taps (cnt[npts] is 0)
    if ((e = scan_exclusive(a.cnt, npts + 1, ptr, scan_tmp, s)) != cudaSuccess) return e;
    unsigned tot = 0;
    if ((e = cudaMemcpyAsync(&tot, ptr + npts, sizeof(unsigned), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    *entries = tot;
    return cudaSuccess;
}

cudaError_t csr_fill_and_order(const CsrBuildArgs& a, long long npts, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(a.cnt, 0, (size_t)npts * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    if (a.total > 0) {
        k_csr_taps<true><<<(unsigned)((a.total + 127) / 128), 128, 0, s>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (npts > 0) {
        k_csr_order<<<(unsigned)((npts + 255) / 256), 256, 0, s>>>(a, npts);
        e = cudaGetLastError();
    }
    return e;
}

// ---------------------------------------------------------------------------
// the gather: block-persistent over the listed tiles.  Thread (column k,
// coil chunk ch, row offset xo) owns points (x, k) for x = xo, xo + xs, ...
// and coils [ch CC, ch CC + CC): the coil chunks of a point run on
// neighbouring threads, the columns of a tile on consecutive threads
// (coalesced stores, one 16 x 8-byte row segment per coil).  The row
// offsets of the next point are loaded before the current point's taps,
// and the taps two at a time (their sample values in flight together); the
// sums keep the row order.
// ---------------------------------------------------------------------------
template <int CC, bool KAHAN>
__global__ void __launch_bounds__(256, (KAHAN || CC > 6) ? 3 : 4) k_spread_csr(CsrSpreadArgs a)
{
    const int nchunk = (a.nch + CC - 1) / CC;
    const int tid = threadIdx.x;
    const int k = tid % a.tb;
    const int ch = (tid / a.tb) % nchunk;
    const int xo = tid / (a.tb * nchunk), xs = blockDim.x / (a.tb * nchunk);
    const int c0 = ch * CC;
    const int ncc = min(CC, a.nch - c0);
    const bool pairs = (a.nch % 2) == 0 && (reinterpret_cast<uintptr_t>(a.yv) & 15) == 0 && ncc == CC;
    auto load_v = [&](int i, float2 (&vv)[CC]) {
        const float2* v = a.yv + (long long)i * a.nch + c0;
        if (pairs) {
#pragma unroll
            for (int c = 0; c < CC; c += 2) {
                const float4 f = __ldg(reinterpret_cast<const float4*>(v + c));
                vv[c] = make_float2(f.x, f.y);
                vv[c + 1] = make_float2(f.z, f.w);
            }
        } else {
#pragma unroll
            for (int c = 0; c < CC; ++c) vv[c] = c < ncc ? __ldg(v + c) : make_float2(0.f, 0.f);
        }
    };
    float2 acc[CC], cmp[CC];
    auto add = [&](const float2 (&vv)[CC], float w) {
#pragma unroll
        for (int c = 0; c < CC; ++c) {
            if (KAHAN) {
                // y = v w - e;  s = t + y;  e = (s - t) - y;  t = s
                const float yx = fmaf(vv[c].x, w, -cmp[c].x), yy = fmaf(vv[c].y, w, -cmp[c].y);
                const float sx = __fadd_rn(acc[c].x, yx), sy = __fadd_rn(acc[c].y, yy);
                cmp[c].x = __fsub_rn(__fsub_rn(sx, acc[c].x), yx);
                cmp[c].y = __fsub_rn(__fsub_rn(sy, acc[c].y), yy);
                acc[c] = make_float2(sx, sy);
            } else {
                acc[c].x = fmaf(vv[c].x, w, acc[c].x);
                acc[c].y = fmaf(vv[c].y, w, acc[c].y);
            }
        }
    };
    if (xo >= a.Gx || ch >= nchunk) return;
    for (long long J = a.j0 + blockIdx.x; J < a.j0 + a.nj; J += gridDim.x) {
        const int2 t = a.tiles[J];
        float2* g = a.grid + (long long)(t.x - a.bin0) * a.grid_bs + (long long)c0 * a.coil_stride;
        const bool col_ok = (long long)t.y + k < a.B;
        const long long pbase = J * a.Gx * a.tb + k;
        unsigned n0 = __ldg(a.ptr + pbase + (long long)xo * a.tb), n1 = __ldg(a.ptr + pbase + (long long)xo * a.tb + 1);
        for (int x = xo; x < a.Gx; x += xs) {
            const unsigned e0 = n0, e1 = n1;
            if (x + xs < a.Gx) {   // the next point's row
                const long long pn = pbase + (long long)(x + xs) * a.tb;
                n0 = __ldg(a.ptr + pn);
                n1 = __ldg(a.ptr + pn + 1);
            }
#pragma unroll
            for (int c = 0; c < CC; ++c) acc[c] = cmp[c] = make_float2(0.f, 0.f);
            unsigned q = e0;
            for (; q + 1 < e1; q += 2) {
                const int2 u = __ldg(a.ent + q), v = __ldg(a.ent + q + 1);
                float2 vu[CC], vv[CC];
                load_v(u.x, vu);
                load_v(v.x, vv);
                add(vu, __int_as_float(u.y));
                add(vv, __int_as_float(v.y));
            }
            if (q < e1) {
                const int2 u = __ldg(a.ent + q);
                float2 vu[CC];
                load_v(u.x, vu);
                add(vu, __int_as_float(u.y));
            }
            if (col_ok) {
                const long long go = (long long)x * a.B + t.y + k;
#pragma unroll
                for (int c = 0; c < CC; ++c)
                    if (c < ncc) {
                        float2 o = acc[c];
                        if (KAHAN) o = make_float2(__fsub_rn(o.x, cmp[c].x), __fsub_rn(o.y, cmp[c].y));
                        g[(long long)c * a.coil_stride + go] = o;
                    }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The same gather with the matrix staged in shared memory.  Work unit: a
// slab of csr_slab_rows(tb) consecutive x rows of one listed tile (CSR_PTS points,
// consecutive in the matrix, so their row offsets and their taps are two
// contiguous ranges).  One thread per block issues both ranges of the unit
// CSR_NST - 1 ahead as bulk copies (cp.async.bulk, completion on an
// mbarrier); the threads then read row offsets and taps from shared memory
// and only the sample values (L2-resident) from global memory, which takes
// the matrix's DRAM latency out of every point's dependent-load chain.  A
// slab with more than CSR_CAP taps reads its taps from global memory as
// the unstaged kernel does.  Sums, their order and the stores are those of
// k_spread_csr: the grids are bitwise equal.
// Every wait is bounded: on a timeout the block sets the error flag, lets
// its issued copies land and leaves.
// ---------------------------------------------------------------------------
constexpr int CSR_PTS = 1024;         // points per unit (64 rows of a 16-column tile)
constexpr int CSR_CAP = 2048;         // staged taps per unit
constexpr int CSR_NST = 2;            // pipeline stages
constexpr unsigned long long CSR_WAIT_NS = 2000000000ull;

// x rows per unit for tiles of tb columns (tb divides CSR_PTS: 4, 8, 16 or 32)
__host__ __device__ inline int csr_slab_rows(int tb) { return CSR_PTS / tb; }
__host__ __device__ inline int csr_ptr_stride(int tb) { return ((CSR_PTS + 1) + 3) & ~3; }

static size_t csr_staged_smem(int tb)
{
    return (size_t)CSR_NST * ((size_t)csr_ptr_stride(tb) * sizeof(unsigned) + (size_t)CSR_CAP * sizeof(int2)) +
           CSR_NST * sizeof(uint64_t);
}

template <int CC, bool KAHAN>
__global__ void __launch_bounds__(256, (KAHAN || CC > 6) ? 3 : 4) k_spread_csr_staged(CsrSpreadArgs a, int nunits)
{
    static_assert(CC % 2 == 0, "sample values are read as coil pairs");
    extern __shared__ float4 s_csr[];
    const int PS = csr_ptr_stride(a.tb);
    int2* s_ent = reinterpret_cast<int2*>(s_csr);                                // [CSR_NST][CSR_CAP]
    unsigned* s_ptr = reinterpret_cast<unsigned*>(s_ent + CSR_NST * CSR_CAP);   // [CSR_NST][PS]
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_ptr + CSR_NST * PS);
    const int tb = a.tb;
    const int nchunk = a.nch / CC;     // the launcher guarantees nch % CC == 0
    const int tid = threadIdx.x;
    const int k = tid % tb;
    const int ch = (tid / tb) % nchunk;
    const int xo = tid / (tb * nchunk), xs = blockDim.x / (tb * nchunk);
    const int sx = csr_slab_rows(tb);
    const unsigned nslab = (unsigned)((a.Gx + sx - 1) / sx);
    const float4* yv4 = reinterpret_cast<const float4*>(a.yv) + ch * (CC / 2);
    const int yv4_stride = a.nch / 2;
    const long long cs = a.coil_stride;
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
    auto load_v = [&](int i, float4 (&v)[CC / 2]) {
        const float4* p = yv4 + (long long)i * yv4_stride;
#pragma unroll
        for (int c = 0; c < CC / 2; ++c) v[c] = __ldg(p + c);
    };
    // the points of a unit: row offsets sp (local), taps from ENT(q)
    auto points = [&](const unsigned* sp, int nx, float2* gp, long long gstep, auto ent) {
        for (int x = xo; x < nx; x += xs, gp += gstep) {
            const unsigned e0 = sp[x * tb + k], e1 = sp[x * tb + k + 1];
#pragma unroll
            for (int c = 0; c < CC; ++c) acc[c] = cmp[c] = make_float2(0.f, 0.f);
            unsigned q = e0;
            for (; q + 1 < e1; q += 2) {
                const int2 u = ent(q), v = ent(q + 1);
                float4 vu[CC / 2], vv[CC / 2];
                load_v(u.x, vu);
                load_v(v.x, vv);
                add(vu, __int_as_float(u.y));
                add(vv, __int_as_float(v.y));
            }
            if (q < e1) {
                const int2 u = ent(q);
                float4 vu[CC / 2];
                load_v(u.x, vu);
                add(vu, __int_as_float(u.y));
            }
            if (gp) {
#pragma unroll
                for (int c = 0; c < CC; ++c) {
                    float2 o = acc[c];
                    if (KAHAN) o = make_float2(__fsub_rn(o.x, cmp[c].x), __fsub_rn(o.y, cmp[c].y));
                    gp[c * cs] = o;
                }
            }
        }
    };
    auto issue = [&](int kk) {   // thread 0 only
        const unsigned u = blockIdx.x + (unsigned)kk * gridDim.x;
        const unsigned jt = u / nslab;
        const int xa = (int)(u - jt * nslab) * sx;
        const int nx = min(sx, a.Gx - xa);
        const long long p0 = ((a.j0 + jt) * a.Gx + xa) * tb;
        const int np = nx * tb;
        const unsigned e0a = __ldg(a.ptr + p0) & ~1u, e1 = __ldg(a.ptr + p0 + np);
        const unsigned ne = e1 - e0a;
        const uint32_t pb = ((uint32_t)(np + 1) * 4u + 15u) & ~15u;
        const uint32_t eb = ne <= (unsigned)CSR_CAP ? ((ne * 8u + 15u) & ~15u) : 0u;
        const int st = kk % CSR_NST;
        mbar_arrive_expect_tx(&s_bar[st], pb + eb);
        bulk_load(s_ptr + st * PS, a.ptr + p0, pb, &s_bar[st]);
        if (eb) bulk_load(s_ent + st * CSR_CAP, a.ent + e0a, eb, &s_bar[st]);
    };
    if (tid == 0) {
        for (int st = 0; st < CSR_NST; ++st) mbar_init(&s_bar[st], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int my_n = nunits > (int)blockIdx.x ? (nunits - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    if (tid == 0)
        for (int kk = 0; kk < CSR_NST - 1 && kk < my_n; ++kk) issue(kk);
    for (int kk = 0; kk < my_n; ++kk) {
        const int st = kk % CSR_NST;
        if (tid == 0 && kk + CSR_NST - 1 < my_n) issue(kk + CSR_NST - 1);
        const bool ok = mbar_wait_bounded(&s_bar[st], (uint32_t)((kk / CSR_NST) & 1), CSR_WAIT_NS);
        if (__syncthreads_or(!ok)) {
            // timeout: report, let the copies already issued land, leave
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (int j = kk; j < my_n && j < kk + CSR_NST; ++j)
                    mbar_wait_bounded(&s_bar[j % CSR_NST], (uint32_t)((j / CSR_NST) & 1), CSR_WAIT_NS);
            }
            return;
        }
        const unsigned u = blockIdx.x + (unsigned)kk * gridDim.x;
        const unsigned jt = u / nslab;
        const int xa = (int)(u - jt * nslab) * sx;
        const int nx = min(sx, a.Gx - xa);
        const unsigned* sp = s_ptr + st * PS;
        const int2 t = a.tiles[a.j0 + jt];
        // store pointer of (x = xa + xo, column t.y + k, first coil of the chunk); null: no column
        float2* gp = (long long)t.y + k < a.B
                         ? a.grid + (long long)(t.x - a.bin0) * a.grid_bs + (long long)(ch * CC) * cs +
                               (long long)(xa + xo) * a.B + t.y + k
                         : nullptr;
        const long long gstep = gp ? (long long)xs * a.B : 0;
        const unsigned e0a = sp[0] & ~1u;
        if (sp[nx * tb] - e0a <= (unsigned)CSR_CAP) {
            const int2* se = s_ent + st * CSR_CAP;
            points(sp, nx, gp, gstep, [&](unsigned q) { return se[q - e0a]; });
        } else {
            points(sp, nx, gp, gstep, [&](unsigned q) { return __ldg(a.ent + q); });
        }
        __syncthreads();   // the stage is free for the copy issued next
    }
}

static int sm_count_csr()
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

template <int CC, bool KAHAN>
static cudaError_t spread_csr_run(const CsrSpreadArgs& a, cudaStream_t s)
{
    const int nchunk = (a.nch + CC - 1) / CC;
    const int per = a.tb * nchunk;
    if (per > 256) return cudaErrorInvalidValue;
    const int nt = (256 / per) * per;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spread_csr<CC, KAHAN>, nt, 0);
    if (e != cudaSuccess) return e;
    const long long nblk = std::min<long long>(a.nj, (long long)sm_count_csr() * std::max(per_sm, 1));
    k_spread_csr<CC, KAHAN><<<(unsigned)nblk, nt, 0, s>>>(a);
    return cudaGetLastError();
}

template <int CC, bool KAHAN>
static cudaError_t spread_csr_staged_run(const CsrSpreadArgs& a, cudaStream_t s)
{
    const int nchunk = a.nch / CC;
    const int per = a.tb * nchunk;
    if (per > 256) return cudaErrorInvalidValue;
    const int nt = (256 / per) * per;
    const size_t smem = csr_staged_smem(a.tb);
    static bool attr = false;   // above 48 KiB only with the opt-in (set once per template)
    if (!attr && smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_spread_csr_staged<CC, KAHAN>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spread_csr_staged<CC, KAHAN>, nt, smem);
    if (e != cudaSuccess) return e;
    const int sx = csr_slab_rows(a.tb);
    const long long nunits = a.nj * ((a.Gx + sx - 1) / sx);
    if (nunits >= 0x7fffffffLL) return cudaErrorInvalidValue;
    const long long nblk = std::min<long long>(nunits, (long long)sm_count_csr() * std::max(per_sm, 1));
    k_spread_csr_staged<CC, KAHAN><<<(unsigned)nblk, nt, smem, s>>>(a, (int)nunits);
    return cudaGetLastError();
}

// coils per thread: a.cc (2, 4, 6, 8) or, with 0, 2 / 4 for up to 2 / 4
// coils, else 6 (12 coils: two threads per point).  staged: the
// shared-memory staged form (needs the error flag and 16-byte aligned row
// offsets of every slab: tb a multiple of 4, 16-byte aligned arrays).
cudaError_t launch_spread_csr(const CsrSpreadArgs& a, bool kahan, bool staged, cudaStream_t s)
{
    if (a.nj <= 0) return cudaSuccess;
    if (a.tb < 1 || a.tb > 32 || a.nch < 1) return cudaErrorInvalidValue;
    int cc = a.cc;
    if (cc == 0) cc = a.nch <= 2 ? 2 : a.nch <= 4 ? 4 : 6;
    // the staged form: an error flag, 16-byte aligned row offsets of every
    // slab (tb a multiple of 4), whole coil chunks of 16-byte coil pairs
    staged = staged && a.err && (a.tb % 4) == 0 && (CSR_PTS % a.tb) == 0 && (reinterpret_cast<uintptr_t>(a.ptr) & 15) == 0 &&
             (reinterpret_cast<uintptr_t>(a.ent) & 15) == 0 && (reinterpret_cast<uintptr_t>(a.yv) & 15) == 0 &&
             (cc % 2) == 0 && (a.nch % cc) == 0;
    if (staged) {
        switch (cc) {
        case 2: return kahan ? spread_csr_staged_run<2, true>(a, s) : spread_csr_staged_run<2, false>(a, s);
        case 4: return kahan ? spread_csr_staged_run<4, true>(a, s) : spread_csr_staged_run<4, false>(a, s);
        case 6: return kahan ? spread_csr_staged_run<6, true>(a, s) : spread_csr_staged_run<6, false>(a, s);
        case 8: return kahan ? spread_csr_staged_run<8, true>(a, s) : spread_csr_staged_run<8, false>(a, s);
        }
        return cudaErrorInvalidValue;
    }
    switch (cc) {
    case 2: return kahan ? spread_csr_run<2, true>(a, s) : spread_csr_run<2, false>(a, s);
    case 4: return kahan ? spread_csr_run<4, true>(a, s) : spread_csr_run<4, false>(a, s);
    case 6: return kahan ? spread_csr_run<6, true>(a, s) : spread_csr_run<6, false>(a, s);
    case 8: return kahan ? spread_csr_run<8, true>(a, s) : spread_csr_run<8, false>(a, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace cgs
