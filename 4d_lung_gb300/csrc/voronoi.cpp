// voronoi.cpp -- Voronoi-cell density weights of a 3-D k-space trajectory
// (the reference's estimateDensityV3D, functions.h:161-258, which uses a
// CGAL Delaunay triangulation; CGAL is not available here).
//
// Same definition as the reference:
//   * D[i] = volume of the Voronoi cell of sample i;
//   * cells of samples on the convex hull (unbounded cells) get 0
//     (functions.h:96-106,149-150);
//   * the volumes are divided by their maximum (functions.h:234-245).
// Method: each cell is built directly as the intersection of half-spaces.
// It starts as a large box around the sample and is clipped by the bisector
// plane of every neighbour, nearest shells of a uniform cell grid first,
// until no unvisited sample can cut it (all of them lie farther than twice
// the cell's circumradius).  The start box lies 1000 data diameters out, so
// a cell that still touches it after the search is unbounded (a hull
// sample) and gets 0; bounded cells near the hull keep their (large) volume,
// as in the reference.  Volumes are summed from the
// faces (divergence theorem, pyramids from the sample point).  One cell per
// OpenMP iteration; samples are treated independently, so duplicate points
// share nothing and the result does not depend on the thread count.
#include "cgsense_c.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// Convex polyhedron as flat arrays (faces are vertex ranges); clipping
// writes into scratch arrays that keep their capacity, so a cell allocates
// only while it grows.
struct Cell {
    std::vector<V3> vtx, nvtx, cap;
    std::vector<int> fstart, nfstart;
    std::vector<char> fbox, nfbox;
    std::vector<std::pair<double, V3>> ang;

    void make_box(V3 c, double h)
    {
        const V3 p[8] = {{c.x - h, c.y - h, c.z - h}, {c.x + h, c.y - h, c.z - h}, {c.x + h, c.y + h, c.z - h},
                         {c.x - h, c.y + h, c.z - h}, {c.x - h, c.y - h, c.z + h}, {c.x + h, c.y - h, c.z + h},
                         {c.x + h, c.y + h, c.z + h}, {c.x - h, c.y + h, c.z + h}};
        const int f[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {1, 2, 6, 5}, {0, 4, 7, 3}};
        vtx.clear();
        fstart.assign(1, 0);
        fbox.clear();
        for (auto& q : f) {
            for (int i = 0; i < 4; ++i) vtx.push_back(p[q[i]]);
            fstart.push_back((int)vtx.size());
            fbox.push_back(1);
        }
    }

    int nfaces() const { return (int)fbox.size(); }

    double max_dist2(V3 c) const
    {
        double m = 0.0;
        for (const auto& v : vtx) m = std::max(m, dot(v - c, v - c));
        return m;
    }

    // axis-aligned bounds of the vertices relative to c
    void bounds(V3 c, V3& lo, V3& hi) const
    {
        lo = {1e300, 1e300, 1e300};
        hi = {-1e300, -1e300, -1e300};
        for (const auto& v : vtx) {
            const V3 r = v - c;
            lo = {std::min(lo.x, r.x), std::min(lo.y, r.y), std::min(lo.z, r.z)};
            hi = {std::max(hi.x, r.x), std::max(hi.y, r.y), std::max(hi.z, r.z)};
        }
    }

    bool touches_box() const
    {
        for (char b : fbox)
            if (b) return true;
        return false;
    }

    // keep {x : dot(x, n) <= d}; returns true when the cell changed
    bool clip(V3 n, double d, double eps)
    {
        bool any_out = false;
        for (const auto& v : vtx)
            if (dot(v, n) - d > eps) {
                any_out = true;
                break;
            }
        if (!any_out) return false;
        nvtx.clear();
        nfstart.assign(1, 0);
        nfbox.clear();
        cap.clear();
        for (int f = 0; f < nfaces(); ++f) {
            const int b0 = fstart[f], m = fstart[f + 1] - b0;
            const size_t before = nvtx.size();
            for (int i = 0; i < m; ++i) {
                const V3 a = vtx[b0 + i], b = vtx[b0 + (i + 1) % m];
                const double da = dot(a, n) - d, db = dot(b, n) - d;
                const bool ina = da <= eps, inb = db <= eps;
                if (ina) nvtx.push_back(a);
                if (ina != inb) {
                    const double t = da / (da - db);
                    const V3 q = a + (b - a) * t;
                    nvtx.push_back(q);
                    cap.push_back(q);
                }
            }
            if (nvtx.size() - before >= 3) {
                nfstart.push_back((int)nvtx.size());
                nfbox.push_back(fbox[f]);
            } else {
                nvtx.resize(before);
            }
        }
        if (cap.size() >= 3) {
            // order the cap's points around their centroid in the plane
            V3 c{0, 0, 0};
            for (const auto& q : cap) c = c + q;
            c = c * (1.0 / cap.size());
            V3 u = cap[0] - c;
            const double lu = std::sqrt(dot(u, u));
            if (lu > 0) {
                u = u * (1.0 / lu);
                const V3 w = cross(n, u);
                ang.clear();
                for (const auto& q : cap) ang.push_back({std::atan2(dot(q - c, w), dot(q - c, u)), q});
                std::sort(ang.begin(), ang.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
                const size_t before = nvtx.size();
                for (const auto& e : ang) {
                    if (nvtx.size() > before) {
                        const V3 r = e.second - nvtx.back();
                        if (dot(r, r) <= eps * eps) continue;
                    }
                    nvtx.push_back(e.second);
                }
                if (nvtx.size() - before >= 3) {
                    const V3 r = nvtx[before] - nvtx.back();
                    if (dot(r, r) <= eps * eps) nvtx.pop_back();
                }
                if (nvtx.size() - before >= 3) {
                    nfstart.push_back((int)nvtx.size());
                    nfbox.push_back(0);
                } else {
                    nvtx.resize(before);
                }
            }
        }
        vtx.swap(nvtx);
        fstart.swap(nfstart);
        fbox.swap(nfbox);
        return true;
    }

    // volume as the sum of pyramids from c over the faces
    double volume(V3 c) const
    {
        double vol = 0.0;
        for (int f = 0; f < nfaces(); ++f) {
            const int b0 = fstart[f], m = fstart[f + 1] - b0;
            V3 an{0, 0, 0};
            for (int i = 1; i + 1 < m; ++i) an = an + cross(vtx[b0 + i] - vtx[b0], vtx[b0 + i + 1] - vtx[b0]);
            vol += std::fabs(dot(vtx[b0] - c, an)) / 6.0;
        }
        return vol;
    }
};

}  // namespace

// Voronoi cell volume of every sample (0 on the convex hull).
static int voronoi_volumes(const double* k, int64_t n, std::vector<double>& volumes)
{
    V3 lo{1e300, 1e300, 1e300}, hi{-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < n; ++i) {
        const V3 p{k[3 * i], k[3 * i + 1], k[3 * i + 2]};
        if (!std::isfinite(p.x) || !std::isfinite(p.y) || !std::isfinite(p.z)) return CGS_ERR_NONFINITE;
        lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
        hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
    }
    const V3 ext = hi - lo;
    const double diam = std::sqrt(dot(ext, ext)) + 1e-12;
    // uniform cell grid with about two samples per cell
    const double vol = std::max(ext.x, diam * 1e-6) * std::max(ext.y, diam * 1e-6) * std::max(ext.z, diam * 1e-6);
    const double h = std::cbrt(vol * 2.0 / (double)n);
    int nc[3];
    const double e3[3] = {ext.x, ext.y, ext.z};
    for (int a = 0; a < 3; ++a) nc[a] = std::max(1, std::min(1024, (int)std::ceil(e3[a] / h)));
    auto cell_of = [&](const V3& p, int* c) {
        const double q[3] = {(p.x - lo.x) / h, (p.y - lo.y) / h, (p.z - lo.z) / h};
        for (int a = 0; a < 3; ++a) c[a] = std::min(nc[a] - 1, std::max(0, (int)q[a]));
    };
    const int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    std::vector<int64_t> start(ncell + 1, 0);
    std::vector<int64_t> items(n);
    for (int64_t i = 0; i < n; ++i) {
        int c[3];
        cell_of({k[3 * i], k[3 * i + 1], k[3 * i + 2]}, c);
        start[((int64_t)c[0] * nc[1] + c[1]) * nc[2] + c[2] + 1]++;
    }
    for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
    {
        std::vector<int64_t> fill(start.begin(), start.end() - 1);
        for (int64_t i = 0; i < n; ++i) {
            int c[3];
            cell_of({k[3 * i], k[3 * i + 1], k[3 * i + 2]}, c);
            items[fill[((int64_t)c[0] * nc[1] + c[1]) * nc[2] + c[2]]++] = i;
        }
    }
    const int max_shell = std::max({nc[0], nc[1], nc[2]});
    // start box far outside the data: only unbounded cells still touch it
    // after every sample that could cut them has been used
    const double box_h = 1e3 * diam;
    const double eps = diam * 1e-12;
    volumes.assign(n, 0.0);

#pragma omp parallel
    {
        Cell cell;
        std::vector<std::pair<double, int64_t>> cand;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            const V3 p{k[3 * i], k[3 * i + 1], k[3 * i + 2]};
            cell.make_box(p, box_h);
            int c[3];
            cell_of(p, c);
            double r2 = cell.max_dist2(p);
            V3 blo, bhi;
            cell.bounds(p, blo, bhi);
            // the bisector of q can cut the cell only if the cell reaches past
            // it along n = q - p: max over the cell of (v-p).n > |n|^2 / 2;
            // the bounding box bounds that maximum in O(1)
            auto may_cut = [&](const V3& nrm, double l2) {
                const double sup = std::max(nrm.x * blo.x, nrm.x * bhi.x) + std::max(nrm.y * blo.y, nrm.y * bhi.y) +
                                   std::max(nrm.z * blo.z, nrm.z * bhi.z);
                return sup > 0.5 * l2;
            };
            for (int s = 0; s <= max_shell; ++s) {
                // shell s: cells at Chebyshev distance s from the home cell,
                // nearest samples first so that the cell shrinks early
                cand.clear();
                for (int dx = -s; dx <= s; ++dx)
                    for (int dy = -s; dy <= s; ++dy)
                        for (int dz = -s; dz <= s; ++dz) {
                            if (std::max({std::abs(dx), std::abs(dy), std::abs(dz)}) != s) continue;
                            const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                            if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) continue;
                            const int64_t cid = ((int64_t)x * nc[1] + y) * nc[2] + z;
                            for (int64_t e = start[cid]; e < start[cid + 1]; ++e) {
                                const int64_t j = items[e];
                                if (j == i) continue;
                                const V3 q{k[3 * j], k[3 * j + 1], k[3 * j + 2]};
                                const double l2 = dot(q - p, q - p);
                                if (l2 > 0.0 && l2 < 4.0 * r2) cand.push_back({l2, j});
                            }
                        }
                // the first shells are sorted so that the cell shrinks early;
                // later shells only meet the O(1) tests below
                if (s <= 1) std::sort(cand.begin(), cand.end());
                for (const auto& e : cand) {
                    if (e.first >= 4.0 * r2) continue;   // too far to cut the cell
                    const int64_t j = e.second;
                    const V3 q{k[3 * j], k[3 * j + 1], k[3 * j + 2]};
                    const V3 nrm = q - p;
                    if (!may_cut(nrm, e.first)) continue;
                    if (cell.clip(nrm, dot(nrm, (p + q) * 0.5), eps)) {
                        r2 = cell.max_dist2(p);
                        cell.bounds(p, blo, bhi);
                    }
                }
                // every unvisited sample is at least s*h away; it cannot cut
                // the cell once that exceeds twice the cell's radius
                const double reach = (double)s * h;
                if (reach * reach >= 4.0 * r2) break;
                if (s >= 2 && cell.touches_box()) {
                    // Still unbounded after the local shells: either a hull
                    // sample or a long cell near the hull.  For a direction u
                    // towards a vertex on the start box, the cell is unbounded
                    // along u iff no sample lies ahead of p along u (then the
                    // ray p + t u satisfies every bisector); otherwise the
                    // sample farthest ahead cuts that far region off.
                    bool unbounded = false;
                    for (int it = 0; it < 256 && cell.touches_box(); ++it) {
                        V3 u{0, 0, 0};
                        for (int f = 0; f < cell.nfaces(); ++f)
                            if (cell.fbox[f]) {
                                u = cell.vtx[cell.fstart[f]] - p;
                                break;
                            }
                        double best = 0.0;
                        int64_t jb = -1;
                        for (int64_t j = 0; j < n; ++j) {
                            const V3 q{k[3 * j], k[3 * j + 1], k[3 * j + 2]};
                            const double t = dot(q - p, u);
                            if (t > best && dot(q - p, q - p) > 0.0) {
                                best = t;
                                jb = j;
                            }
                        }
                        if (jb < 0) {
                            unbounded = true;
                            break;
                        }
                        const V3 q{k[3 * jb], k[3 * jb + 1], k[3 * jb + 2]};
                        const V3 nrm = q - p;
                        if (!cell.clip(nrm, dot(nrm, (p + q) * 0.5), eps)) {
                            unbounded = true;   // numerically on the hull
                            break;
                        }
                        r2 = cell.max_dist2(p);
                        cell.bounds(p, blo, bhi);
                    }
                    if (unbounded) break;
                }
            }
            volumes[i] = cell.touches_box() ? 0.0 : cell.volume(p);
        }
    }
    return CGS_OK;
}

static int check_traj(const double* k, int64_t n)
{
    for (int64_t i = 0; i < 3 * n; ++i)
        if (!std::isfinite(k[i])) return CGS_ERR_NONFINITE;
    return CGS_OK;
}

// division by the largest value (functions.h:234-245)
static void normalise_max(const std::vector<double>& v, float* dcf)
{
    double mx = 0.0;
    for (double x : v) mx = std::max(mx, x);
    const double inv = mx > 0 ? 1.0 / mx : 0.0;
    for (size_t i = 0; i < v.size(); ++i) dcf[i] = (float)(v[i] * inv);
}

extern "C" int cgs_voronoi_dcf(const double* k, int64_t n, float* dcf)
{
    if (!k || !dcf || n < 0) return CGS_ERR_ARG;
    if (n == 0) return CGS_OK;
    const int st = check_traj(k, n);
    if (st != CGS_OK) return st;
    std::vector<double> vol;
    voronoi_volumes(k, n, vol);
    normalise_max(vol, dcf);
    return CGS_OK;
}

// estimateDensityV3D with its `average` option (functions.h:212-232): the
// volumes are summed per readout position i % sX over all readouts, divided
// by the total, and every sample takes the sum of its position -- positions
// beyond (sX - 1) * cutoff take the value at that position -- before the
// division by the maximum.  The reference adds into a float array from
// several threads without a reduction; here the sums are FP64 and ordered.
extern "C" int cgs_estimate_density_v3d(const double* k, int64_t n, int32_t sX, int32_t average, double cutoff,
                                        float* dcf)
{
    if (!k || !dcf || n < 0) return CGS_ERR_ARG;
    if (n == 0) return CGS_OK;
    if (average && (sX <= 0 || n % sX != 0 || !(cutoff >= 0.0 && cutoff <= 1.0))) return CGS_ERR_ARG;
    const int st = check_traj(k, n);
    if (st != CGS_OK) return st;
    std::vector<double> vol;
    voronoi_volumes(k, n, vol);
    if (average) {
        std::vector<double> avg(sX, 0.0);
        for (int64_t i = 0; i < n; ++i) avg[i % sX] += vol[i];
        double tot = 0.0;
        for (int i = 0; i < sX; ++i) tot += avg[i];
        const double inv = tot > 0 ? 1.0 / tot : 0.0;
        const int lim = (int)((sX - 1) * cutoff);
        for (int64_t i = 0; i < n; ++i) vol[i] = inv * avg[std::min((int)(i % sX), lim)];
    }
    normalise_max(vol, dcf);
    return CGS_OK;
}
