// tess_radius.cu -- fixed-radius queries on the bin grid (sm_103a).
//
// Four query kinds share one kernel body:
//   RQ_CELLS        Celery::find_cells_in_radius (celery.rs:753-796): the bins
//                   of the box [q - r, q + r] (clamped to the point bounds)
//                   whose gap distance to q's bin is within r
//                   (check_cell_in_range, celery.rs:708-748), in i, j, k order.
//   RQ_CELL_RADIUS  find_neighbors_in_cell_radius (celery.rs:802-818): every
//                   point of those bins, bin by bin.
//   RQ_REAL_RADIUS  find_neighbors_in_real_radius (celery.rs:825-855): those
//                   points whose squared distance (celery.rs:700-702) is at
//                   most r * r.
//   RQ_CLOUD        Cell::compute_neighbor_cloud (interface.rs:348-365): the
//                   expanding search from the cell's position over the search
//                   order up to the first key above r (celery.rs:1023-1075),
//                   optionally filtered by group.
//
// One warp answers one query.  The warp takes 32 candidate bins at a time
// (box cells or search-order entries), keeps the ones in range, and then
// walks the kept bins' points as one concatenated stream, 32 points per step:
// a warp prefix sum of the bins' counts maps each lane to its bin.  Results
// stay in the reference's order (bins in query order, sorted_indices order
// within a bin, which is ascending point index here) because every step
// compacts with a ballot.  Each query runs twice: a count pass, then (after a
// scan of the counts into offsets) a fill pass that writes at the offsets.
// All FP64 arithmetic is correctly rounded with no contraction, so the bins
// and points found are the reference's exactly.
#include <algorithm>
#include <cmath>

#include "tess_internal.cuh"

namespace tess {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// max_float / min_float, celery.rs:682-698: on ties and NaN the second wins.
__device__ __forceinline__ double max_float(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double min_float(double a, double b) { return a < b ? a : b; }

__device__ __forceinline__ double sq_rn(double a) { return __dmul_rn(a, a); }

struct WarpOut {
    uint64_t pos;   // fill pass: next output slot of this query
    uint32_t cnt;   // results so far
};

// The points of up to 32 kept bins (one per lane: first sorted position `beg`,
// point count `c`), as one stream in lane order.
template <int MODE, bool FILL>
__device__ __forceinline__ void emit_points(const RadiusParams& p, uint32_t beg, uint32_t c, double x, double y,
                                            double z, double r2, uint32_t pt_base, int lane, WarpOut& w) {
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t tot = __shfl_sync(kFull, incl, 31);
    if (tot == 0) return;
    const bool test = MODE == RQ_REAL_RADIUS || (MODE == RQ_CLOUD && p.group >= 0);
    if (!test && !FILL) {
        w.cnt += tot;
        return;
    }
    const uint32_t excl = incl - c;
    const unsigned lt = (1u << lane) - 1u;
    for (uint32_t o = 0; o < tot; o += 32) {
        const uint32_t t = o + lane;
        // owner lane: the first lane whose inclusive count exceeds t
        int L = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t v = __shfl_sync(kFull, incl, L + step - 1);
            if (v <= t) L += step;
        }
        const uint32_t ex = __shfl_sync(kFull, excl, L);
        const uint32_t b0 = __shfl_sync(kFull, beg, L);
        bool ok = t < tot;
        const uint32_t s = b0 + (t - ex);
        if (MODE == RQ_REAL_RADIUS && ok) {
            // distance_squared(x, y, z, point), celery.rs:700-702
            const double dx = __dsub_rn(x, p.spx[s]);
            const double dy = __dsub_rn(y, p.spy[s]);
            const double dz = __dsub_rn(z, p.spz[s]);
            const double d2 = __dadd_rn(__dadd_rn(sq_rn(dx), sq_rn(dy)), sq_rn(dz));
            ok = d2 <= r2;
        }
        if (MODE == RQ_CLOUD && ok && p.group >= 0) ok = (int64_t)(p.sgroup ? p.sgroup[s] : 0u) == p.group;
        const unsigned bal = __ballot_sync(kFull, ok);
        if (FILL && ok) p.out[w.pos + __popc(bal & lt)] = p.sorted[s] - pt_base;
        w.pos += __popc(bal);
        w.cnt += __popc(bal);
    }
}

// One batch of up to 32 candidate bins (one per lane).
template <int MODE, bool FILL>
__device__ __forceinline__ void emit_bins(const RadiusParams& p, bool keep, uint32_t bin, uint64_t bin_base,
                                          double x, double y, double z, double r2, uint32_t pt_base, int lane,
                                          WarpOut& w) {
    if (MODE == RQ_CELLS) {
        const unsigned bal = __ballot_sync(kFull, keep);
        if (FILL && keep) p.out[w.pos + __popc(bal & ((1u << lane) - 1u))] = bin;
        w.pos += __popc(bal);
        w.cnt += __popc(bal);
        return;
    }
    uint32_t beg = 0, c = 0;
    if (keep) {
        beg = p.delims[bin_base + bin];
        c = p.delims[bin_base + bin + 1] - beg;
    }
    emit_points<MODE, FILL>(p, beg, c, x, y, z, r2, pt_base, lane, w);
}

template <int MODE, bool FILL>
__global__ void __launch_bounds__(256) k_radius(RadiusParams p) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const DiagDesc& D = p.desc[0];
    const double glo0 = D.glo[0], glo1 = D.glo[1], glo2 = D.glo[2];
    const double ghi0 = D.ghi[0], ghi1 = D.ghi[1], ghi2 = D.ghi[2];
    const double inv0 = D.inv[0], inv1 = D.inv[1], inv2 = D.inv[2];
    const double sz0 = D.size[0], sz1 = D.size[1], sz2 = D.size[2];
    const int cpd = D.cpd;
    const uint64_t bin_base = D.bin_base;
    const uint32_t pt_base = D.pt_base;
    const double r = p.radius;
    const double r2 = sq_rn(r);

    for (uint32_t wq = warp; wq < p.nq; wq += nwarps) {
        uint32_t q = wq;
        double x, y, z;
        if (p.qxyz) {
            x = p.qxyz[3 * (size_t)wq];
            y = p.qxyz[3 * (size_t)wq + 1];
            z = p.qxyz[3 * (size_t)wq + 2];
        } else if (p.qcell) {
            const uint32_t c = p.qcell[wq];
            if (c >= D.n) {                     // not a cell of this diagram: no results, flagged
                if (lane == 0) {
                    if (!FILL) p.count[q] = 0;
                    atomicExch(p.err, 1);
                }
                continue;
            }
            const size_t g = (size_t)pt_base + c;
            x = p.xyz[3 * g];
            y = p.xyz[3 * g + 1];
            z = p.xyz[3 * g + 2];
        } else {
            // every cell, walked in bin order so neighbouring warps share bins
            const uint32_t s = pt_base + wq;
            q = p.sorted[s] - pt_base;
            x = p.spx[s];
            y = p.spy[s];
            z = p.spz[s];
        }
        WarpOut w{FILL ? p.offs[q] : 0, 0};

        if (MODE == RQ_CLOUD) {
            // ExpandingSearch::new, celery.rs:882-902
            const int bx = axis_index(x, glo0, ghi0, inv0, cpd);
            const int by = axis_index(y, glo1, ghi1, inv1, cpd);
            const int bz = axis_index(z, glo2, ghi2, inv2, cpd);
            for (uint32_t base = 0; base < p.rtab_len; base += 32) {
                const uint32_t t = base + lane;
                bool keep = false;
                uint32_t bin = 0;
                if (t < p.rtab_len) {
                    const short4 e = p.rtab[t];
                    const int X = bx + e.x, Y = by + e.y, Z = bz + e.z;
                    keep = X >= 0 && X < cpd && Y >= 0 && Y < cpd && Z >= 0 && Z < cpd;
                    if (keep) bin = ((uint32_t)X * (uint32_t)cpd + (uint32_t)Y) * (uint32_t)cpd + (uint32_t)Z;
                }
                emit_bins<MODE, FILL>(p, keep, bin, bin_base, x, y, z, r2, pt_base, lane, w);
            }
        } else {
            // find_cells_in_radius, celery.rs:753-796
            const int i0 = axis_index(max_float(__dsub_rn(x, r), glo0), glo0, ghi0, inv0, cpd);
            const int j0 = axis_index(max_float(__dsub_rn(y, r), glo1), glo1, ghi1, inv1, cpd);
            const int k0 = axis_index(max_float(__dsub_rn(z, r), glo2), glo2, ghi2, inv2, cpd);
            const int i1 = axis_index(min_float(__dadd_rn(x, r), ghi0), glo0, ghi0, inv0, cpd);
            const int j1 = axis_index(min_float(__dadd_rn(y, r), ghi1), glo1, ghi1, inv1, cpd);
            const int k1 = axis_index(min_float(__dadd_rn(z, r), ghi2), glo2, ghi2, inv2, cpd);
            // the query's own bin (check_cell_in_range, celery.rs:729-731)
            const int xi = axis_index(x, glo0, ghi0, inv0, cpd);
            const int yi = axis_index(y, glo1, ghi1, inv1, cpd);
            const int zi = axis_index(z, glo2, ghi2, inv2, cpd);
            // box cells, i-major; at most cpd^3 < 2^32 of them
            const int nx = i1 - i0 + 1, ny = j1 - j0 + 1, nz = k1 - k0 + 1;
            const uint32_t nyz = (uint32_t)(ny > 0 && nz > 0 ? ny * nz : 0);
            const uint32_t nbox = nx > 0 ? (uint32_t)nx * nyz : 0u;
            for (uint32_t base = 0; base < nbox; base += 32) {
                const uint32_t t = base + lane;
                bool keep = false;
                uint32_t bin = 0;
                if (t < nbox) {
                    const int i = i0 + (int)(t / nyz);
                    const uint32_t rem = t % nyz;
                    const int j = j0 + (int)(rem / (uint32_t)nz);
                    const int k = k0 + (int)(rem % (uint32_t)nz);
                    const int gx = max(abs(xi - i) - 1, 0);
                    const int gy = max(abs(yi - j) - 1, 0);
                    const int gz = max(abs(zi - k) - 1, 0);
                    const double ds = __dadd_rn(__dadd_rn(sq_rn(__dmul_rn((double)gx, sz0)),
                                                          sq_rn(__dmul_rn((double)gy, sz1))),
                                                sq_rn(__dmul_rn((double)gz, sz2)));
                    keep = ds <= r2;
                    bin = ((uint32_t)i * (uint32_t)cpd + (uint32_t)j) * (uint32_t)cpd + (uint32_t)k;
                }
                emit_bins<MODE, FILL>(p, keep, bin, bin_base, x, y, z, r2, pt_base, lane, w);
            }
        }
        if (!FILL && lane == 0) p.count[q] = w.cnt;
    }
}

template <int MODE>
cudaError_t launch_mode(const RadiusParams& p, bool fill, int blocks, cudaStream_t s) {
    if (fill)
        k_radius<MODE, true><<<blocks, 256, 0, s>>>(p);
    else
        k_radius<MODE, false><<<blocks, 256, 0, s>>>(p);
    return cudaGetLastError();
}

// Host copy of the search-order key (celery.rs:423-427 on gap counts); the
// library's host code is compiled without FMA contraction, so this is the
// same correctly rounded FP64 arithmetic as the device's gap_key.
double host_gap_key(const double size[3], int i, int j, int k) {
    if (i == 0 && j == 0 && k == 0) return -1.0;
    const int gi = i < 0 ? -i - 1 : (i > 0 ? i - 1 : 0);
    const int gj = j < 0 ? -j - 1 : (j > 0 ? j - 1 : 0);
    const int gk = k < 0 ? -k - 1 : (k > 0 ? k - 1 : 0);
    const double a = (double)gi * size[0], b = (double)gj * size[1], c = (double)gk * size[2];
    return a * a + b * b + c * c;
}

// Largest offset along an axis that can still have key <= radius: offsets
// with gap g >= G satisfy (g * s)^2 > radius, so |offset| <= G suffices.
int axis_reach(double s, int cpd, double radius) {
    if (!(s > 0.0) || std::isnan(radius) || std::isinf(radius)) return cpd - 1;
    auto beyond = [&](long g) {
        const double a = (double)g * s;
        return a * a > radius;
    };
    long g = radius > 0.0 ? (long)std::min(std::floor(std::sqrt(radius) / s), (double)cpd) : 0;
    while (g > 0 && beyond(g - 1)) --g;
    while (g < cpd && !beyond(g)) ++g;
    return (int)std::min<long>(g, cpd - 1);
}

struct RadiusEntry {
    double key;
    int i, j, k;
};

}  // namespace

cudaError_t launch_radius(const RadiusParams& p, int mode, bool fill, int blocks, cudaStream_t s) {
    if (p.nq == 0) return cudaSuccess;
    switch (mode) {
        case RQ_CELLS: return launch_mode<RQ_CELLS>(p, fill, blocks, s);
        case RQ_CELL_RADIUS: return launch_mode<RQ_CELL_RADIUS>(p, fill, blocks, s);
        case RQ_REAL_RADIUS: return launch_mode<RQ_REAL_RADIUS>(p, fill, blocks, s);
        case RQ_CLOUD: return launch_mode<RQ_CLOUD>(p, fill, blocks, s);
        default: return cudaErrorInvalidValue;
    }
}

// The prefix of the search order (celery.rs:418-679: every offset with
// |i|, |j|, |k| <= cpd - 1, sorted by key; ties broken by i, j, k) that
// expand_all_in_radius visits before its first key above the radius.
bool build_radius_table(const double size[3], int cpd, double radius, size_t max_entries,
                        std::vector<short4>& out) {
    out.clear();
    if (radius < -1.0) return true;                     // even the own bin (key -1) is beyond
    const int gx = axis_reach(size[0], cpd, radius);
    const int gy = axis_reach(size[1], cpd, radius);
    const int gz = axis_reach(size[2], cpd, radius);
    const double enumerate = (2.0 * gx + 1) * (2.0 * gy + 1) * (2.0 * gz + 1);
    if (enumerate > (double)max_entries) return false;
    std::vector<RadiusEntry> e;
    e.reserve((size_t)enumerate);
    for (int i = -gx; i <= gx; ++i)
        for (int j = -gy; j <= gy; ++j)
            for (int k = -gz; k <= gz; ++k) {
                const double key = host_gap_key(size, i, j, k);
                if (key > radius) continue;             // celery.rs:1037-1039
                e.push_back({key, i, j, k});
            }
    std::sort(e.begin(), e.end(), [](const RadiusEntry& a, const RadiusEntry& b) {
        if (a.key != b.key) return a.key < b.key;
        if (a.i != b.i) return a.i < b.i;
        if (a.j != b.j) return a.j < b.j;
        return a.k < b.k;
    });
    out.resize(e.size());
    for (size_t t = 0; t < e.size(); ++t)
        out[t] = make_short4((short)e[t].i, (short)e[t].j, (short)e[t].k, 0);
    return true;
}

}  // namespace tess
