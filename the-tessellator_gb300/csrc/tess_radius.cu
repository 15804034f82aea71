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

__device__ __forceinline__ double sq_rn(double a) { return __dmul_rn(a, a); }

struct WarpOut {
    uint64_t pos;   // fill pass: next output slot of this query
    uint32_t cnt;   // results so far
};

// One query as the point test sees it: the FP64 position and radius of the
// reference's arithmetic, and an FP32 pre-filter.  The filter decides a
// candidate when its FP32 squared distance (from the points' FP32 high
// parts) is farther than `band` from r^2, where `band` bounds the FP32
// estimate's error against the exact squared distance; inside the band the
// exact FP64 test decides.  Either way the answer is the FP64 one.
struct QueryTest {
    double x, y, z, r2;
    float fx, fy, fz;
    float lo_thr, hi_thr;   // accept below, reject above (when on)
    bool on;
};

// Kept out of line: inlined, the compiler predicates these FP64 operations
// into every candidate step, and predicated-off FP64 instructions still take
// the (slow) FP64 pipe's issue slots.
__device__ __noinline__ bool exact_within(const RadiusParams& p, const QueryTest& qt, uint32_t s) {
    // distance_squared(x, y, z, point), celery.rs:700-702
    const double dx = __dsub_rn(qt.x, p.spx[s]);
    const double dy = __dsub_rn(qt.y, p.spy[s]);
    const double dz = __dsub_rn(qt.z, p.spz[s]);
    return __dadd_rn(__dadd_rn(sq_rn(dx), sq_rn(dy)), sq_rn(dz)) <= qt.r2;
}

// Up to 32 runs (one per lane: first element `beg`, length `c`) as one
// stream in lane order.  The elements are sorted positions of points, or
// bin ids for RQ_CELLS.
template <int MODE, bool FILL>
__device__ __forceinline__ void emit_stream(const RadiusParams& p, uint32_t beg, uint32_t c, const QueryTest& qt,
                                            uint32_t pt_base, int lane, WarpOut& w) {
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
    if (MODE == RQ_CELLS) {
        const uint32_t ex = incl - c;
        for (uint32_t o = 0; o < tot; o += 32) {
            const uint32_t t = o + lane;
            int L = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const uint32_t v = __shfl_sync(kFull, incl, L + step - 1);
                if (v <= t) L += step;
            }
            const uint32_t e0 = __shfl_sync(kFull, ex, L);
            const uint32_t b0 = __shfl_sync(kFull, beg, L);
            if (t < tot) p.out[w.pos + t - o] = b0 + (t - e0);
            w.pos += min(32u, tot - o);
        }
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
        const bool valid = t < tot;
        bool ok = valid;
        const uint32_t s = b0 + (t - ex);
        if (MODE == RQ_REAL_RADIUS) {
            bool band = false;
            if (qt.on) {
                if (valid) {
                    const float* h = p.shi + 3 * (size_t)s;
                    const float dx = __fsub_rn(qt.fx, h[0]);
                    const float dy = __fsub_rn(qt.fy, h[1]);
                    const float dz = __fsub_rn(qt.fz, h[2]);
                    const float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
                    ok = d2 < qt.lo_thr;
                    band = !ok && !(d2 > qt.hi_thr);      // NaN lands in the band
                }
            } else {
                band = valid;
                ok = false;
            }
            if (__any_sync(kFull, band) && band) ok = exact_within(p, qt, s);
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
                                          const QueryTest& qt, uint32_t pt_base, int lane, WarpOut& w) {
    uint32_t beg = 0, c = 0;
    if (keep) {
        beg = p.delims[bin_base + bin];
        c = p.delims[bin_base + bin + 1] - beg;
    }
    emit_stream<MODE, FILL>(p, beg, c, qt, pt_base, lane, w);
}

// A double to float, rounded toward zero, from the bit pattern alone (no
// FP64-pipe conversion): |result| <= |v| and |v - result| < 2^-23 |v| in the
// float range; below it 0 (error under 2^-126), above it (and NaN) +-inf.
__device__ __forceinline__ float f64_to_f32_rz(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
}

__device__ __forceinline__ bool is_nan_bits(unsigned long long b) {
    return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}

// axis_index(v) (celery.rs:269-314) without FP64 arithmetic: axis_index is
// monotone in v, so it is the number of bin boundaries at or below v, found by
// binary search over the order codes of the boundaries.  NaN gives 0, as
// axis_index does.
__device__ __forceinline__ int axis_index_table(unsigned long long vbits, const unsigned long long* b, int cpd,
                                                int top) {
    if (is_nan_bits(vbits)) return 0;
    const unsigned long long e = (vbits >> 63) ? ~vbits : (vbits | 0x8000000000000000ull);
    int i = 0;
    for (int step = top; step > 0; step >>= 1)
        if (i + step < cpd && __ldg(b + i + step) <= e) i += step;
    return i;
}

// Smallest double (as an order code) whose axis_index is >= i, by binary
// search over the order codes between -inf and +inf, evaluating the exact
// FP64 axis_index.
__global__ void k_axis_bounds(const DiagDesc* desc, int cpd, unsigned long long* bnd) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * cpd) return;
    const int a = t / cpd, i = t % cpd;
    const DiagDesc& D = desc[0];
    if (i == 0) {
        bnd[t] = 0ull;
        return;
    }
    unsigned long long lo = ord_enc(-INFINITY), hi = ord_enc(INFINITY);   // axis_index(+inf) = cpd - 1 >= i
    while (lo < hi) {
        const unsigned long long mid = lo + (hi - lo) / 2;
        if (axis_index(ord_dec(mid), D.glo[a], D.ghi[a], D.inv[a], cpd) >= i)
            hi = mid;
        else
            lo = mid + 1;
    }
    bnd[t] = lo;
}

// check_cell_in_range's squared gap distance (celery.rs:708-748) in FP64;
// out of line for the same reason as exact_within.
__device__ __noinline__ double gap_ds(int gx, int gy, int gz, double sz0, double sz1, double sz2) {
    return __dadd_rn(__dadd_rn(sq_rn(__dmul_rn((double)gx, sz0)), sq_rn(__dmul_rn((double)gy, sz1))),
                     sq_rn(__dmul_rn((double)gz, sz2)));
}

template <int MODE, bool FILL>
__global__ void __launch_bounds__(256) k_radius(RadiusParams p) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const DiagDesc& D = p.desc[0];
    const int cpd = D.cpd;
    const uint64_t bin_base = D.bin_base;
    const uint32_t pt_base = D.pt_base;
    const double sz0 = D.size[0], sz1 = D.size[1], sz2 = D.size[2];
    const double r = p.radius;
    const double r2 = sq_rn(r);
    // Per-lane axis for the spread evaluation of the query's bin indices:
    // lanes 0-2 the query's own bin (x, y, z), lanes 3-5 the box's low end,
    // lanes 6-8 its high end (celery.rs:753-778); other lanes repeat lane % 3.
    const int ax = lane % 3;
    const int kind = lane < 9 ? lane / 3 : 0;
    const unsigned long long* abnd = p.bnd + ax * cpd;
    // box ends clamp to the point bounds: max_float(c - r, min), min_float(c + r, max)
    const unsigned long long clamp_bits =
        (unsigned long long)__double_as_longlong(kind == 2 ? D.ghi[ax] : D.glo[ax]);
    const unsigned long long clamp_code = (clamp_bits >> 63) ? ~clamp_bits : (clamp_bits | 0x8000000000000000ull);
    // lanes 9-11 form the query relative to the diagram's centre (the frame
    // of the points' FP32 parts) in the same FP64 add
    const double delta = kind == 1 ? -r : (kind == 2 ? r : (lane >= 9 && lane < 12 ? -D.ctr[ax] : 0.0));
    int top = 1;
    while (2 * top < cpd) top *= 2;
    // magnitude bound of the point coordinates relative to the centre, and
    // the radius, for the FP32 filter's error band
    double gm = 0.0;
    for (int a = 0; a < 3; ++a) gm = fmax(gm, fmax(fabs(D.glo[a] - D.ctr[a]), fabs(D.ghi[a] - D.ctr[a])));
    const float gmag = (float)gm;
    const float fr = (float)r;
    const float r2f = (float)r2;

    for (uint32_t wq0 = warp; wq0 < p.nq; wq0 += nwarps) {
        const uint32_t wq = p.qorder ? p.qorder[wq0] : wq0;
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
        QueryTest qt;
        qt.x = x;
        qt.y = y;
        qt.z = z;
        qt.r2 = r2;
        qt.on = false;

        // the bin indices this query needs, one per lane, with exact FP64
        // arithmetic: get_{x,y,z}_cell_index of the coordinate, of
        // max_float(c - r, min) and of min_float(c + r, max)
        const double ca = ax == 0 ? x : (ax == 1 ? y : z);
        unsigned long long vb = (unsigned long long)__double_as_longlong(ca);
        if (MODE != RQ_CLOUD) {
            // c - r (exactly c + (-r)) or c + r, one FP64 add for all lanes
            vb = (unsigned long long)__double_as_longlong(__dadd_rn(ca, delta));
            if (kind != 0) {
                // max_float / min_float: v is kept only when strictly inside
                // the bound (NaN: the bound)
                const unsigned long long ve = (vb >> 63) ? ~vb : (vb | 0x8000000000000000ull);
                const bool inside = kind == 1 ? ve > clamp_code : ve < clamp_code;
                if (is_nan_bits(vb) || !inside) vb = clamp_bits;
            }
        }
        const int idx = axis_index_table(vb, abnd, cpd, top);
        const int xi = __shfl_sync(kFull, idx, 0);
        const int yi = __shfl_sync(kFull, idx, 1);
        const int zi = __shfl_sync(kFull, idx, 2);

        if (MODE == RQ_CLOUD) {
            // ExpandingSearch::new, celery.rs:882-902
            for (uint32_t base = 0; base < p.rtab_len; base += 32) {
                const uint32_t t = base + lane;
                bool keep = false;
                uint32_t bin = 0;
                if (t < p.rtab_len) {
                    const short4 e = p.rtab[t];
                    const int X = xi + e.x, Y = yi + e.y, Z = zi + e.z;
                    keep = X >= 0 && X < cpd && Y >= 0 && Y < cpd && Z >= 0 && Z < cpd;
                    if (keep) bin = ((uint32_t)X * (uint32_t)cpd + (uint32_t)Y) * (uint32_t)cpd + (uint32_t)Z;
                }
                emit_bins<MODE, FILL>(p, keep, bin, bin_base, qt, pt_base, lane, w);
            }
        } else {
            // find_cells_in_radius, celery.rs:753-796
            const int i0 = __shfl_sync(kFull, idx, 3), j0 = __shfl_sync(kFull, idx, 4);
            const int k0 = __shfl_sync(kFull, idx, 5), i1 = __shfl_sync(kFull, idx, 6);
            const int j1 = __shfl_sync(kFull, idx, 7), k1 = __shfl_sync(kFull, idx, 8);
            if (MODE == RQ_REAL_RADIUS && p.f32_filter) {
                // error band of the FP32 squared distance, q and p relative to
                // the diagram's centre (each FP64-rounded, 2^-53 |q|): per axis
                // the query's truncation to FP32 (2^-23 |q|), the point's
                // rounding (2^-24 |p|) and the subtraction's (2^-24 |dq|), at most
                // e = 6e-8 (3 m + 2.1 r); squared and summed near r^2 that is
                // 2 sqrt(3) 1.01 r e + 3 e^2, plus 4 roundings of the sum and
                // the FP64 side, doubled
                // integer ops, the centre-relative coordinates of lanes 9-11
                const float fa = f64_to_f32_rz(__longlong_as_double((long long)vb));
                qt.fx = __shfl_sync(kFull, fa, 9);
                qt.fy = __shfl_sync(kFull, fa, 10);
                qt.fz = __shfl_sync(kFull, fa, 11);
                const float qmag = fmaxf(fmaxf(fabsf(qt.fx), fabsf(qt.fy)), fabsf(qt.fz));
                const float m = fmaxf(gmag, qmag) * 1.0001f;
                const float e = 6.0e-8f * (3.0f * m + 2.1f * fr);
                const float band = 2.0f * (3.5f * fr * e + 3.0f * e * e) + 1.0e-6f * r2f;
                qt.lo_thr = r2f - band;
                qt.hi_thr = r2f + band;
                qt.on = m < 1.0e18f;
            }
            // The box's rows (i, j), i-major, one per lane.  Within a row the
            // kept bins are those whose gap gz = max(|zi - k| - 1, 0) is at
            // most the row's limit T (the gap distance grows with gz), i.e. one
            // contiguous k range around zi; its points are one contiguous run
            // of the sorted order (bins in k order, sorted order within).
            const int nx = i1 - i0 + 1, ny = j1 - j0 + 1;
            const int nrows = (nx > 0 && ny > 0 && k1 >= k0) ? nx * ny : 0;
            for (int base = 0; base < nrows; base += 32) {
                const int t = base + lane;
                uint32_t beg = 0, c = 0;
                if (t < nrows) {
                    const int i = i0 + t / ny, j = j0 + t % ny;
                    const int gx = max(abs(xi - i) - 1, 0), gy = max(abs(yi - j) - 1, 0);
                    const int gz_need = max(max(zi - k0, k1 - zi) - 1, 0);   // largest gap in the row
                    int T = -1;
                    int from = 0;
                    if (p.gtab && gx <= p.gtab_x && gy <= p.gtab_y) {
                        T = __ldg(p.gtab + gx * (p.gtab_y + 1) + gy);
                        from = T == p.gtab_z ? p.gtab_z + 1 : gz_need + 1;    // table ends at gtab_z
                    }
                    for (int gz = from; gz <= gz_need; ++gz) {                 // FP64 rows (rare)
                        if (!(gap_ds(gx, gy, gz, sz0, sz1, sz2) <= r2)) break;
                        T = gz;
                    }
                    if (T >= 0) {
                        const int kl = max(k0, zi - T - 1), kh = min(k1, zi + T + 1);
                        if (kl <= kh) {
                            const uint32_t row = ((uint32_t)i * (uint32_t)cpd + (uint32_t)j) * (uint32_t)cpd;
                            if (MODE == RQ_CELLS) {
                                beg = row + (uint32_t)kl;
                                c = (uint32_t)(kh - kl + 1);
                            } else {
                                beg = p.delims[bin_base + row + (uint32_t)kl];
                                c = p.delims[bin_base + row + (uint32_t)kh + 1] - beg;
                            }
                        }
                    }
                }
                emit_stream<MODE, FILL>(p, beg, c, qt, pt_base, lane, w);
            }
        }
        if (!FILL && lane == 0) p.count[q] = w.cnt;
    }
}

// Position of query wq (a given position, or the position of a given cell).
__device__ __forceinline__ bool query_position(const RadiusParams& p, uint32_t wq, double& x, double& y, double& z) {
    if (p.qxyz) {
        x = p.qxyz[3 * (size_t)wq];
        y = p.qxyz[3 * (size_t)wq + 1];
        z = p.qxyz[3 * (size_t)wq + 2];
        return true;
    }
    const uint32_t c = p.qcell[wq];
    if (c >= p.desc[0].n) return false;
    const size_t g = (size_t)p.desc[0].pt_base + c;
    x = p.xyz[3 * g];
    y = p.xyz[3 * g + 1];
    z = p.xyz[3 * g + 2];
    return true;
}

__global__ void __launch_bounds__(256) k_query_bin(RadiusParams p, QueryOrder o) {
    const DiagDesc& D = p.desc[0];
    const int shift = 1;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < p.nq; q += gridDim.x * blockDim.x) {
        double x = 0.0, y = 0.0, z = 0.0;
        uint32_t c = 0;
        if (query_position(p, q, x, y, z)) {
            int top = 1;
            while (2 * top < D.cpd) top *= 2;
            const uint32_t ix =
                (uint32_t)axis_index_table((unsigned long long)__double_as_longlong(x), p.bnd, D.cpd, top) >> shift;
            const uint32_t iy = (uint32_t)axis_index_table((unsigned long long)__double_as_longlong(y),
                                                           p.bnd + D.cpd, D.cpd, top) >> shift;
            const uint32_t iz = (uint32_t)axis_index_table((unsigned long long)__double_as_longlong(z),
                                                           p.bnd + 2 * D.cpd, D.cpd, top) >> shift;
            c = (ix * (uint32_t)o.cpdc + iy) * (uint32_t)o.cpdc + iz;
        }
        o.qbin[q] = c;
        o.qrank[q] = atomicAdd(&o.cnt[c], 1u);
    }
}

__global__ void __launch_bounds__(256) k_query_scatter(uint32_t nq, QueryOrder o) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
        o.order[o.coff[o.qbin[q]] + o.qrank[q]] = q;
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

// check_cell_in_range's squared gap distance on the host (same operation
// order, no contraction).
double host_gap_ds(const double size[3], int gx, int gy, int gz) {
    const double a = (double)gx * size[0], b = (double)gy * size[1], c = (double)gz * size[2];
    return a * a + b * b + c * c;
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

cudaError_t launch_axis_bounds(const DiagDesc* desc, int cpd, unsigned long long* bnd, cudaStream_t s) {
    k_axis_bounds<<<(3 * cpd + 127) / 128, 128, 0, s>>>(desc, cpd, bnd);
    return cudaGetLastError();
}

cudaError_t launch_query_order(const RadiusParams& p, const QueryOrder& o, int blocks, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(o.cnt, 0, sizeof(uint32_t) * o.ncoarse, s);
    if (e != cudaSuccess) return e;
    k_query_bin<<<blocks, 256, 0, s>>>(p, o);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = launch_csr_offsets(o.cnt, o.ncoarse, o.coff, o.scan_tmp, s)) != cudaSuccess) return e;
    k_query_scatter<<<blocks, 256, 0, s>>>(p.nq, o);
    return cudaGetLastError();
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

bool build_gap_table(const double size[3], const double inv[3], int cpd, double radius, size_t max_entries,
                     std::vector<int16_t>& out, int* gx, int* gy, int* gz) {
    if (!(radius >= 0.0) || std::isinf(radius)) return false;
    // The box of find_cells_in_radius spans at most ceil(r * inv) + 1 bins on
    // either side of the query's bin, so gaps stay below ceil(r * inv) + 1.
    int g[3];
    for (int a = 0; a < 3; ++a) {
        const double reach = radius * inv[a];
        g[a] = (size[a] > 0.0 && reach < 1e6) ? std::min(cpd - 1, (int)std::ceil(reach) + 2) : cpd - 1;
        if (g[a] > 32767) return false;
    }
    if ((size_t)(g[0] + 1) * (size_t)(g[1] + 1) > max_entries) return false;
    const double r2 = radius * radius;
    out.assign((size_t)(g[0] + 1) * (size_t)(g[1] + 1), (int16_t)-1);
    for (int i = 0; i <= g[0]; ++i)
        for (int j = 0; j <= g[1]; ++j) {
            int best = -1;
            for (int k = 0; k <= g[2]; ++k) {           // the distance grows with k
                if (!(host_gap_ds(size, i, j, k) <= r2)) break;
                best = k;
            }
            out[(size_t)i * (size_t)(g[1] + 1) + (size_t)j] = (int16_t)best;
        }
    *gx = g[0];
    *gy = g[1];
    *gz = g[2];
    return true;
}

}  // namespace tess
