// tess_grid.cu -- the binning pass (the GPU form of Celery::reset,
// celery.rs:253-266): tight bounds, bin sizes, bin histogram, exclusive scan
// into delimiters, scatter into bin order, gather of sorted positions, and the
// per-diagram shell table.  All passes are HBM-bound streaming kernels; the
// integer outputs (bins, delimiters, sorted order) are bit-exact with the
// reference formulas.
#include <cfloat>
#include <cmath>

#include "tess_internal.cuh"

namespace tess {
namespace {

constexpr int kBoundsThreads = 256;

// The pass runs on the integer pipes: on this part an FP64 instruction costs
// dozens of issue slots' worth of pipe time, which made the FP64 forms of the
// bounds, the bin formula and the split bound the pass by the FP64 pipe.

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// CeleryBounds::new (celery.rs:81-125): per-chunk min/max of the coordinates'
// order-preserving integer codes (ord_enc: the same order as the doubles),
// merged with 64-bit atomics.  Non-finite inputs (exponent all ones) raise
// error_flag.
__global__ void __launch_bounds__(kBoundsThreads) k_bounds(GridBuffers g) {
    __shared__ unsigned long long red[6][kBoundsThreads / 32];
    for (uint32_t c = blockIdx.x; c < g.nchunks; c += gridDim.x) {
        const uint32_t d = g.chunk_diag[c];
        const uint32_t beg = g.chunk_start[c];
        const DiagDesc& D = g.diags[d];
        const uint32_t end = min(beg + kChunk, D.pt_base + D.n);
        unsigned long long mn[3] = {~0ull, ~0ull, ~0ull};
        unsigned long long mx[3] = {0ull, 0ull, 0ull};
        bool bad = false;
        for (uint32_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
            for (int a = 0; a < 3; ++a) {
                const unsigned long long b = (unsigned long long)__double_as_longlong(g.xyz[3ull * i + a]);
                bad |= ((b >> 52) & 0x7FFull) == 0x7FFull;
                const unsigned long long e = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
                mn[a] = min(mn[a], e);
                mx[a] = max(mx[a], e);
            }
        }
        if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(g.error_flag, 1);
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        for (int a = 0; a < 3; ++a) {
            const unsigned long long lo = warp_min_u64(mn[a]), hi = warp_max_u64(mx[a]);
            if (l == 0) { red[a][w] = lo; red[3 + a][w] = hi; }
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            const int a = threadIdx.x;
            unsigned long long v = red[a][0];
            for (int k = 1; k < kBoundsThreads / 32; ++k) v = a < 3 ? min(v, red[a][k]) : max(v, red[a][k]);
            if (a < 3) atomicMin(&g.bounds[6 * d + a], v);
            else atomicMax(&g.bounds[6 * d + a], v);
        }
        __syncthreads();
    }
}

// x rounded toward zero to FP32 by integer operations (within 2^-23 |x|).
// False for zeros, subnormals, non-finite values and magnitudes outside
// FP32's normal range: those take the exact FP64 formula.
__device__ __forceinline__ bool f32_trunc(double x, float& f) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7FFu);
    const int fe = e - 1023 + 127;
    if (e == 0 || e == 0x7FF || fe < 1 || fe > 254) return false;
    f = __uint_as_float((hi & 0x80000000u) | ((uint32_t)fe << 23) | (uint32_t)((b >> 29) & 0x7FFFFFull));
    return true;
}

// axis_index (celery.rs:269-314) without the FP64 pipe for nearly every point:
// x >= max is decided on the order-preserving codes (exact), and
// v = (x - min) * inv by an FP32 estimate t with a bound E on |t - v|:
//   x to FP32 by truncation (2^-23 |x|), min and inv rounded (2^-24 each),
//   the difference and the product rounded (2^-24 each), and v's own two
//   FP64 roundings (2^-52 each), so
//   |t - v| <= inv (2^-23 |x| + 2^-24 |min|) + 3.1 * 2^-24 |t|,
// which E = inv (|x| + |min|) 2^-22 + |t| 2^-21 covers twice over.  When
// [t - E, t + E] holds no integer (nor 0, nor cpd - 1) the bin is the one
// the FP64 formula gives; otherwise (a point within E of a bin boundary,
// about 2 * 10^-4 of a bin for the unit cube at cpd = 238) ok is false and
// the caller uses the FP64 formula.
__device__ __forceinline__ int axis_index_fast(double x, const DiagDesc& D, int a, int cpd, bool& ok) {
    const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
    float xf;
    if (!f32_trunc(x, xf)) {
        ok = false;
        return 0;
    }
    const unsigned long long hb = (unsigned long long)__double_as_longlong(D.ghi[a]);
    const unsigned long long xe = (xb >> 63) ? ~xb : (xb | 0x8000000000000000ull);
    const unsigned long long he = (hb >> 63) ? ~hb : (hb | 0x8000000000000000ull);
    if (xe >= he) return cpd - 1;
    const float lf = D.glo_f[a], inv = D.inv_f[a];
    const float t = (xf - lf) * inv;
    const float E = inv * (fabsf(xf) + fabsf(lf)) * 2.3841858e-7f + fabsf(t) * 4.7683716e-7f;
    const float up = t + E;
    if (up < 1.0f) return 0;                      // v < 1: 0 (v <= 0 gives 0 too)
    const float dn = t - E;
    if (dn >= (float)(cpd - 1)) return cpd - 1;   // v >= cpd - 1
    const float fl = floorf(dn);
    if (dn > 0.f && fl == floorf(up)) return (int)fl;
    ok = false;
    return 0;
}

// CeleryCellInfo::new (celery.rs:153-181) from the bounds and the host's cpd.
__global__ void k_grid_params(GridBuffers g) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.ndiag) return;
    DiagDesc& D = g.diags[d];
    const double c = (double)D.cpd;
    double m = DBL_MAX;
    for (int a = 0; a < 3; ++a) {
        const double lo = ord_dec(g.bounds[6 * d + a]);
        const double hi = ord_dec(g.bounds[6 * d + 3 + a]);
        D.glo[a] = lo;
        D.ghi[a] = hi;
        const double ctr = 0.5 * lo + 0.5 * hi;
        D.ctr[a] = isfinite(ctr) ? ctr : 0.0;
        const double ext = __dsub_rn(hi, lo);
        D.size[a] = __ddiv_rn(ext, c);
        D.inv[a] = __ddiv_rn(c, ext);
        if (D.size[a] > 0.0) m = fmin(m, D.size[a]);
        // FP32 forms for the FP32 clipping pass: offsets from the centre as
        // FP32 pairs (48 bits), the bin sides and their inverses
        const double gl = lo - D.ctr[a], bl = D.blo[a] - D.ctr[a], bh = D.bhi[a] - D.ctr[a];
        D.glo_hi[a] = __double2float_rn(gl);
        D.glo_lo[a] = __double2float_rn(gl - (double)D.glo_hi[a]);
        D.blo_hi[a] = __double2float_rn(bl);
        D.blo_lo[a] = __double2float_rn(bl - (double)D.blo_hi[a]);
        D.bhi_hi[a] = __double2float_rn(bh);
        D.bhi_lo[a] = __double2float_rn(bh - (double)D.bhi_hi[a]);
        D.inv_f[a] = __double2float_rn(D.inv[a]);
        D.glo_f[a] = __double2float_rn(lo);
        D.size_f[a] = __double2float_rn(D.size[a]);
    }
    D.rcp_cpd = 1.0f / (float)D.cpd;
    D.rcp_cpd2 = 1.0f / ((float)D.cpd * (float)D.cpd);
    // (x - glo) * inv from the FP32 pairs: one rounding of the difference, one
    // of inv, one of the product (u = 2^-24 each, relative to the result, at
    // most cpd bins), with a factor 4 in hand
    D.frac_eps = 4.0f * 5.9604645e-8f * (float)D.cpd + 1e-6f;
    // Table extent: every offset whose key is <= (gaps * m)^2 has all gap
    // counts <= gaps, hence |offset| <= gaps + 1 on every axis.
    int cheb = g.table_gaps + 1;
    if (cheb > D.cpd - 1) cheb = D.cpd - 1;
    if (cheb < 0) cheb = 0;
    D.cheb = cheb;
    // The table holds every offset of the grid when that fits; otherwise the
    // offsets with key <= kmax, and the walk continues ring by ring.
    const bool complete = cheb == D.cpd - 1 && (2 * cheb + 1) * (2 * cheb + 1) * (2 * cheb + 1) <= kMaxTable;
    D.has_extent = m != DBL_MAX;
    if (m == DBL_MAX) {          // every point identical: only the own bin holds points
        D.min_size = 0.0;
        D.tab_kmax = INFINITY;
        D.cheb = 0;
    } else {
        D.min_size = m;
        const int gaps = cheb - 1;
        D.tab_kmax = complete ? (double)INFINITY
                              : __dmul_rn(__dmul_rn((double)gaps, m), __dmul_rn((double)gaps, m));
    }
}

// get_cells (celery.rs:342-354) + histogram.  rank = arrival order in the bin.
__global__ void k_bin_count(GridBuffers g) {
    for (uint32_t c = blockIdx.x; c < g.nchunks; c += gridDim.x) {
        const uint32_t d = g.chunk_diag[c];
        const uint32_t beg = g.chunk_start[c];
        const DiagDesc& D = g.diags[d];
        const uint32_t end = min(beg + kChunk, D.pt_base + D.n);
        const int cpd = D.cpd;
        for (uint32_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
            const double x = g.xyz[3ull * i], y = g.xyz[3ull * i + 1], z = g.xyz[3ull * i + 2];
            bool okx = true, oky = true, okz = true;
            int bx = axis_index_fast(x, D, 0, cpd, okx);
            int by = axis_index_fast(y, D, 1, cpd, oky);
            int bz = axis_index_fast(z, D, 2, cpd, okz);
            // the exact FP64 formula for the few coordinates near a boundary
            if (!okx) bx = axis_index(x, D.glo[0], D.ghi[0], D.inv[0], cpd);
            if (!oky) by = axis_index(y, D.glo[1], D.ghi[1], D.inv[1], cpd);
            if (!okz) bz = axis_index(z, D.glo[2], D.ghi[2], D.inv[2], cpd);
            // get_cell_from_indices, celery.rs:317-325
            const uint64_t b = tess_chk(D.bin_base + ((uint64_t)bx * cpd + by) * cpd + bz, g.total_bins, g.check, CK_GRID);
            g.bin[i] = (uint32_t)b;
            g.rank[i] = atomicAdd(&g.delims[b], 1u);
        }
    }
}

// ---- exclusive scan of the bin counts -> delimiters (celery.rs:372-414) ----
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int l = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (l >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of kScanThreads values; returns the block total.
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* out, uint32_t* sh) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    uint32_t inc = warp_incl_scan(v);
    if (l == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t s = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0;
        uint32_t si = warp_incl_scan(s);
        sh[l] = si - s;
        if (l == 31) sh[32] = si;
    }
    __syncthreads();
    *out = inc - v + sh[w];
    uint32_t total = sh[32];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partial(uint32_t* data, uint64_t n, uint32_t* sums) {
    __shared__ uint32_t sh[33];
    const uint64_t base = (uint64_t)blockIdx.x * kScanThreads * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) s += (base + k < n) ? data[base + k] : 0u;
    uint32_t ex;
    uint32_t tot = block_excl_scan(s, &ex, sh);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* sums, uint32_t nblocks) {
    __shared__ uint32_t sh[33];
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < nblocks; b0 += kScanThreads) {
        const uint32_t b = b0 + threadIdx.x;
        uint32_t v = b < nblocks ? sums[b] : 0u;
        uint32_t ex;
        uint32_t tot = block_excl_scan(v, &ex, sh);
        if (b < nblocks) sums[b] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_final(uint32_t* data, uint64_t n, const uint32_t* sums) {
    __shared__ uint32_t sh[33];
    const uint64_t base = (uint64_t)blockIdx.x * kScanThreads * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        s += v[k];
    }
    uint32_t ex;
    block_excl_scan(s, &ex, sh);
    uint32_t run = sums[blockIdx.x] + ex;
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
}

// get_sorted_indices (celery.rs:357-369): counting-sort scatter.
__global__ void k_scatter(GridBuffers g) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.total) return;
    const uint32_t b = tess_chk(g.bin[i], g.total_bins, g.check, CK_GRID);
    g.sorted[tess_chk(g.delims[b] + g.rank[i], g.total, g.check, CK_GRID)] = i;
}

// Ascending sort of a[0, n) by one block: a bitonic network in the form whose
// comparators all point the same way (the first step of each merge compares
// mirrored positions), over n rounded up to a power of two.  Positions >= n
// stand for +inf: a comparator with one of them never swaps, so they are
// simply skipped and never stored.  a is shared or global memory; the block's
// barriers order the steps either way.
// I is the index type: 32-bit in shared memory, 64-bit for a bin that may
// approach 2^32 points.
template <typename I>
__device__ void block_bitonic_sort(uint32_t* a, I n) {
    I np = 1;
    while (np < n) np <<= 1;
    const I half = np >> 1;
    auto cmpswap = [&](I lo, I hi) {
        if (hi < n) {
            const uint32_t x = a[lo], y = a[hi];
            if (x > y) {
                a[lo] = y;
                a[hi] = x;
            }
        }
    };
    for (I k = 2; k <= np; k <<= 1) {
        const I hk = k >> 1;
        for (I i = threadIdx.x; i < half; i += blockDim.x) {
            const I base = (i / hk) * k, off = i % hk;
            cmpswap(base + off, base + k - 1 - off);
        }
        __syncthreads();
        for (I j = hk >> 1; j > 0; j >>= 1) {
            for (I i = threadIdx.x; i < half; i += blockDim.x) {
                const I lo = (i / j) * 2 * j + i % j;
                cmpswap(lo, lo + j);
            }
            __syncthreads();
        }
    }
}

// Within-bin order ascending by input index (deterministic; the reference's
// sort_unstable_by leaves it unspecified).  Bins hold ~1.25 points on
// average: a thread per bin sorts the small ones by insertion; bins of more
// than 32 points (crowded regions) are sorted afterwards by the whole block,
// in shared memory up to kSortSmem points, in place beyond.
constexpr uint32_t kSortSmem = 4096;
__global__ void __launch_bounds__(256) k_bin_order(GridBuffers g) {
    __shared__ uint32_t big[256];
    __shared__ uint32_t nbig;
    __shared__ uint32_t buf[kSortSmem];
    if (threadIdx.x == 0) nbig = 0;
    __syncthreads();
    const uint64_t b0 = (uint64_t)blockIdx.x * blockDim.x;
    const uint64_t b = b0 + threadIdx.x;
    if (b < g.total_bins) {
        const uint32_t beg = g.delims[b], end = g.delims[b + 1];
        if (end - beg > 32) {
            big[atomicAdd(&nbig, 1u)] = threadIdx.x;
        } else if (end - beg >= 2) {
            for (uint32_t s = beg + 1; s < end; ++s) {
                uint32_t v = g.sorted[s];
                uint32_t t = s;
                while (t > beg && g.sorted[t - 1] > v) {
                    g.sorted[t] = g.sorted[t - 1];
                    --t;
                }
                g.sorted[t] = v;
            }
        }
    }
    __syncthreads();
    const uint32_t nb = nbig;
    for (uint32_t q = 0; q < nb; ++q) {
        const uint64_t bb = b0 + big[q];
        const uint32_t beg = g.delims[bb], n = g.delims[bb + 1] - beg;
        if (n <= kSortSmem) {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) buf[i] = g.sorted[beg + i];
            __syncthreads();
            block_bitonic_sort<uint32_t>(buf, n);
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) g.sorted[beg + i] = buf[i];
        } else {
            block_bitonic_sort<uint64_t>(g.sorted + beg, (uint64_t)n);
        }
        __syncthreads();
    }
}

// hi = u rounded to FP32 (to nearest, ties to even) and lo = u - hi rounded to
// FP32, by integer operations on u's bits: the same values as
// __double2float_rn(u) and __double2float_rn(u - (double)hi).  u - hi is
// exact in units of 2^(E - 52) (at most 29 bits), so one integer-to-FP32
// rounding and an exact power-of-two scale give lo.  False (the FP64 form
// then runs) when lo would be subnormal or hi leaves FP32's normal range.
__device__ __forceinline__ bool split_rn_int(double u, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(u);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FFull);
    if (e == 0) {
        if ((b << 1) != 0) return false;          // subnormal
        hi = __uint_as_float(sign);               // +-0: lo = +0 as u - hi is +0
        lo = 0.f;
        return true;
    }
    if (e == 0x7FF) return false;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    unsigned long long q = m >> 29;
    const unsigned long long rem = m & ((1ull << 29) - 1);
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (q & 1ull))) q += 1;
    const long long diff = (long long)m - (long long)(q << 29);
    int ehi = e;
    if (q == (1ull << 24)) {
        q >>= 1;
        ehi += 1;
    }
    const int fe = ehi - 1023 + 127;
    const int pe = e - 1023 - 52 + 127;
    if (fe < 1 || fe > 254 || (diff != 0 && pe < 1)) return false;
    hi = __uint_as_float(sign | ((uint32_t)fe << 23) | ((uint32_t)q & 0x7FFFFFu));
    lo = diff == 0 ? 0.f : __ll2float_rn(sign ? -diff : diff) * __uint_as_float((uint32_t)pe << 23);
    return true;
}

// Positions (and groups) in sorted order, SoA for coalesced candidate loads.
// The FP32 pair (hi, lo) splits the position relative to its diagram's
// centre: the split keeps 48 bits of that offset, so its error scales with
// the diagram's extent rather than with the coordinates' distance from 0.
__global__ void k_gather(GridBuffers g) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.total) return;
    const uint32_t i = tess_chk(g.sorted[s], g.total, g.check, CK_GRID);
    if (g.inv) g.inv[i] = s;
    const double x = g.xyz[3ull * i], y = g.xyz[3ull * i + 1], z = g.xyz[3ull * i + 2];
    g.spx[s] = x;
    g.spy[s] = y;
    g.spz[s] = z;
    int lo = 0, hi = g.ndiag - 1;     // the diagram holding sorted position s
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g.diags[mid].pt_base <= s) lo = mid;
        else hi = mid - 1;
    }
    const DiagDesc& D = g.diags[lo];
    const double u[3] = {x - D.ctr[0], y - D.ctr[1], z - D.ctr[2]};
    for (int a = 0; a < 3; ++a) {
        float h, l;
        if (!split_rn_int(u[a], h, l)) {
            h = __double2float_rn(u[a]);
            l = __double2float_rn(u[a] - (double)h);
        }
        g.shi[3ull * s + a] = h;
        g.slo[3ull * s + a] = l;
    }
    if (g.sgroup) g.sgroup[s] = g.groups[i];
}

// ---- shell table (get_search_order, celery.rs:418-679) ----
// One block per diagram: every offset within Chebyshev radius `cheb` whose key
// is <= tab_kmax, sorted by (key, i, j, k) with a bitonic sort in shared memory.
constexpr int kTabThreads = 1024;

// The inverse permutation, point -> sorted position, for the queries that
// start from a point's original index (radius queries by cell, single-cell
// computes).  Built on first use after a binning pass rather than in it: its
// 4-byte scatter writes cost a partial DRAM sector per point.
__global__ void k_inverse(const uint32_t* sorted, uint32_t* inv, uint32_t n, int* check) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        inv[tess_chk(sorted[s], n, check, CK_GRID)] = s;
}

__global__ void __launch_bounds__(kTabThreads) k_table(GridBuffers g) {
    __shared__ unsigned long long skey[kMaxTable];
    __shared__ uint16_t sidx[kMaxTable];
    __shared__ unsigned int count;
    const int d = blockIdx.x;
    DiagDesc& D = g.diags[d];
    const int c = D.cheb;
    const int side = 2 * c + 1;
    const int total = side * side * side;
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int i = t / (side * side) - c;
        const int j = (t / side) % side - c;
        const int k = t % side - c;
        const double key = gap_key(D.size, i, j, k);
        if (key <= D.tab_kmax) {
            unsigned int slot = atomicAdd(&count, 1u);
            if (slot < (unsigned)kMaxTable) {
                // keys >= 0 order as their bit patterns; self (-1) sorts first
                skey[slot] = key < 0.0 ? 0ull : (unsigned long long)__double_as_longlong(key) + 1ull;
                sidx[slot] = (uint16_t)t;   // t orders (i, j, k) lexicographically
            }
        }
    }
    __syncthreads();
    const unsigned cap = min((unsigned)kMaxTable, D.tab_cap);
    if (count > cap && threadIdx.x == 0) atomicExch(g.error_flag, 2);
    const int m = (int)min(count, cap);
    int p2 = 1;
    while (p2 < m) p2 <<= 1;
    for (int t = m + threadIdx.x; t < p2; t += blockDim.x) {
        skey[t] = ~0ull;
        sidx[t] = 0xFFFF;
    }
    __syncthreads();
    for (int k2 = 2; k2 <= p2; k2 <<= 1) {
        for (int j2 = k2 >> 1; j2 > 0; j2 >>= 1) {
            for (int t = threadIdx.x; t < p2; t += blockDim.x) {
                const int u = t ^ j2;
                if (u > t) {
                    const bool up = (t & k2) == 0;
                    const unsigned long long ka = skey[t], kb = skey[u];
                    const uint16_t ia = sidx[t], ib = sidx[u];
                    const bool gt = (ka > kb) || (ka == kb && ia > ib);
                    if (gt == up) {
                        skey[t] = kb; skey[u] = ka;
                        sidx[t] = ib; sidx[u] = ia;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        const int e = sidx[t];
        const int i = e / (side * side) - c;
        const int j = (e / side) % side - c;
        const int k = e % side - c;
        const double key = gap_key(D.size, i, j, k);
        TabEntry te;
        te.key = key < 0.0 ? -1.0f : __double2float_rz(key);
        te.i = (int8_t)i;
        te.j = (int8_t)j;
        te.k = (int8_t)k;
        te.pad = 0;
        g.table[D.tab_base + t] = te;
    }
    if (threadIdx.x == 0) D.tab_len = (uint32_t)m;
}

}  // namespace

size_t scan_tmp_words(uint64_t nitems) {
    const uint64_t per = (uint64_t)kScanThreads * kScanItems;
    return (size_t)((nitems + per - 1) / per) + 1;
}

namespace {
// Bin occupancy for the autotuner: out[0] = most points in one bin, out[1] =
// points in bins of at least `crowd` points.  One atomic per warp.
__global__ void k_occupancy(const uint32_t* delims, uint64_t nbins, uint32_t crowd, unsigned long long* out) {
    unsigned long long mx = 0, crowded = 0;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = delims[b + 1] - delims[b];
        mx = c > mx ? c : mx;
        if (c >= crowd) crowded += c;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        crowded += __shfl_xor_sync(0xffffffffu, crowded, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], mx);
        atomicAdd(&out[1], crowded);
    }
}

__global__ void k_bounds_init(unsigned long long* b, int ndiag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 6 * ndiag) b[t] = (t % 6) < 3 ? ~0ull : 0ull;
}
}  // namespace

cudaError_t launch_inverse(const uint32_t* sorted, uint32_t* inv, uint32_t n, int* check, cudaStream_t s) {
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 152u * 16u);
    if (blocks) k_inverse<<<blocks, 256, 0, s>>>(sorted, inv, n, check);
    return cudaGetLastError();
}

// Bulk copy by the SMs: 16-byte loads and stores, grid-stride, then the tail
// byte by byte.  Either side may be pinned host memory (its device address):
// the SMs then move the bytes over the host link themselves.
__global__ void k_copy_bytes(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t n16 = n / 16;
    const uint4* s16 = reinterpret_cast<const uint4*>(src);
    uint4* d16 = reinterpret_cast<uint4*>(dst);
    for (size_t i = i0; i < n16; i += stride) d16[i] = s16[i];
    for (size_t i = 16 * n16 + i0; i < n; i += stride) dst[i] = src[i];
}

cudaError_t launch_copy_bytes(void* dst, const void* src, size_t n, int sms, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    // 4 blocks of 256 threads per SM keep enough 16-byte requests in flight
    // to fill the host link (≈ 192 GB/s measured either way)
    const size_t want = (n / 16 + 255) / 256;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)4 * (sms > 0 ? sms : 152)));
    k_copy_bytes<<<blocks, 256, 0, s>>>(static_cast<const uint8_t*>(src), static_cast<uint8_t*>(dst), n);
    return cudaGetLastError();
}

cudaError_t launch_occupancy(const uint32_t* delims, uint64_t nbins, uint32_t crowd, unsigned long long* out,
                             int blocks, cudaStream_t s) {
    cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), s);
    k_occupancy<<<blocks, 256, 0, s>>>(delims, nbins, crowd, out);
    return cudaGetLastError();
}

// Binning pass: bounds -> grid parameters -> shell tables -> histogram ->
// scan -> scatter -> within-bin order -> gather.  A fixed launch sequence
// (no host synchronisation), so it can be captured in a CUDA graph.
cudaError_t launch_grid_build(const GridBuffers& g, cudaStream_t s, cudaStream_t side, cudaEvent_t fork,
                              cudaEvent_t join) {
    const int ndiag = g.ndiag;
    k_bounds_init<<<(6 * ndiag + 255) / 256, 256, 0, s>>>(g.bounds, ndiag);
    cudaMemsetAsync(g.delims, 0, sizeof(uint32_t) * (g.total_bins + 1), s);
    cudaMemsetAsync(g.error_flag, 0, sizeof(int), s);
    const int cblocks = (int)(g.nchunks < 4096u ? g.nchunks : 4096u);
    k_bounds<<<cblocks, kBoundsThreads, 0, s>>>(g);
    k_grid_params<<<(ndiag + 127) / 128, 128, 0, s>>>(g);
    // the shell tables need only the grid parameters: build them beside the
    // histogram, scan and scatter when a side stream is given
    const bool forked = side && fork && join;
    if (forked) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
        k_table<<<ndiag, kTabThreads, 0, side>>>(g);
        cudaEventRecord(join, side);
    } else {
        k_table<<<ndiag, kTabThreads, 0, s>>>(g);
    }
    k_bin_count<<<cblocks, 256, 0, s>>>(g);
    const uint64_t nscan = g.total_bins + 1;
    const uint64_t per = (uint64_t)kScanThreads * kScanItems;
    const uint32_t nblk = (uint32_t)((nscan + per - 1) / per);
    k_scan_partial<<<nblk, kScanThreads, 0, s>>>(g.delims, nscan, g.scan_tmp);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(g.scan_tmp, nblk);
    k_scan_final<<<nblk, kScanThreads, 0, s>>>(g.delims, nscan, g.scan_tmp);
    k_scatter<<<(g.total + 255) / 256, 256, 0, s>>>(g);
    k_bin_order<<<(unsigned)((g.total_bins + 255) / 256), 256, 0, s>>>(g);
    k_gather<<<(g.total + 255) / 256, 256, 0, s>>>(g);
    if (forked) cudaStreamWaitEvent(s, join, 0);
    return cudaGetLastError();
}

}  // namespace tess
