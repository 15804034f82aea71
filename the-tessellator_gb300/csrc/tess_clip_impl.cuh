// tess_clip.cu -- the clipping kernel: one Voronoi cell per warp.
//
// The GPU form of Cell::compute_voronoi_cell (interface.rs:257-313) with
// Polyhedron::cut_with_plane (polyhedron.rs:438-642), ExpandingSearch
// (celery.rs:865-1075) and the cell outputs (polyhedron.rs:776-935).
//
// Cell representation (per warp).  The polyhedron starts as the container
// box translated by -site (polyhedron.rs:268-392, interface.rs:266).  Every
// vertex is the meeting point of three face planes and is stored as
//   - its position: in lane registers (slot s lives in lane s % 32, register
//     set s / 32) with a mirror in shared memory,
//   - its plane triple (a, b, c), ordered counter-clockwise seen from outside,
//   - its three neighbours: adj[i] is the vertex across the edge (t[i], t[i+1]).
// The half-edge pools of the reference (pool.rs) become these fixed-capacity
// slot arrays; a cell that outgrows them is flagged and re-run at a larger
// capacity.
//
// Cutting by a bisector (vector3.rs:223-239):
//   1. every lane classifies its vertices, sd = n.v - offset, Outside when
//      sd > 1e-12 (vector3.rs:170-193, polyhedron.rs:221); one ballot per
//      register set gives the Outside mask.  No Outside vertex: no cut.
//   2. an edge of an Outside vertex X whose neighbour Y is not Outside is a
//      boundary edge; it gets a new vertex at the reference's intersection
//      X + (Y - X) * sd_X / (sd_X - sd_Y) (vector3.rs:213-219) with the
//      triple (a, b, new plane).  An Incident Y (|sd| <= tol) yields a
//      vertex at Y's position, as the reference duplicates Incident vertices
//      (polyhedron.rs:554-565).
//   3. the new vertices link into a ring through two small maps
//      (first plane -> vertex, second plane -> vertex), Outside slots are
//      freed and reused (clean_up_vertices / clean_up_edges, polyhedron.rs:645-730).
//
// Candidates come bin by bin in shell order (get_search_order,
// celery.rs:418-679) and the walk stops once the next bin's gap distance is
// at least twice the largest vertex distance: no farther point can cut
// (the security radius; the reference walks every point instead,
// celery.rs:971-1018, with the same result).
//
// FP32 form: positions, planes and classification in FP32; a plane test
// whose |sd| lies within its rigorous rounding bound (see cut()) aborts the
// cell, which is then re-run with those tests decided in FP64 (or wholly in
// FP64).  Areas and volumes are accumulated in FP64 in both forms (weighted
// normals and volume / 6, polyhedron.rs:776-855).
//
// Crowded bins: a cell whose own bin holds many points is first cut by the
// nearest point of each lane's stride of that bin (32 seeds, nearest first),
// which shrinks it to about its final size before the shell walk.
#pragma once
#include <cfloat>
#include <cmath>
#include <mutex>

#include "tess_internal.cuh"

namespace tess {
namespace clipk {

constexpr unsigned FULL = 0xffffffffu;
// FP32 form: relative error constant of a vertex solved from its three planes
// (a few FP32 roundings of the plane data and of Cramer's rule).
constexpr float kVertexErr = 1.5e-6f;
// Load the next batch's table entries and bin ranges before cutting the
// current batch (overlaps their latency, costs registers).
constexpr bool kPrefetch = true;
// Pre-test a window's candidates against the live vertices (re-run form)
// when at least this many are within twice the cell radius.  The lean
// first-pass form leaves it out: on uniform inputs windows are small and its
// mere presence costs the hot loop registers.
constexpr int kPretestMin = 2;
// A site whose own bin holds at least ClipParams::seed_min points (12 by
// default, autotuned per input) is seeded before the shell walk: every lane
// takes the nearest point of its stride of that bin and the 32 seeds are cut
// nearest first.  In crowded bins the walk's 32-point windows otherwise meet
// the nearest points late, after many cuts by farther ones (plane capacity,
// larger radius, more guard-band tests).
// Hybrid form: a new FP32 vertex whose error bound exceeds kNumBad * guard_rel
// * R (1e-3 R at the default guard_rel) sends the cell to the FP64 form.
constexpr float kNumBad = 2500.0f;

template <typename T, int K>
struct Smem {
    static constexpr int V = 32 * K;                                 // vertex slots
    static constexpr int P = (32 * K + 32) < 254 ? (32 * K + 32) : 254;  // planes (< 0xFF)
    static constexpr int VUSE = V < 255 ? V : 255;                    // slot 255 is the map sentinel
    static constexpr int PF = sizeof(T) == 4 ? P : 1;
    static constexpr int VF = sizeof(T) == 4 ? V : 1;
    static constexpr int VD = sizeof(T) == 8 ? V : 1;
    // live through the whole cell
    T vx[V], vy[V], vz[V];            // vertex mirror
    int32_t pid[P];                   // neighbour id (local original index) or wall code
    uint32_t psrc[P];                 // sorted index of the point that made the plane
    uint32_t tri[V];                  // planes a | b << 8 | c << 16
    uint32_t adj[V];                  // neighbours n0 | n1 << 8 | n2 << 16
    // The walk's working arrays and the finalize's share storage: no array
    // of one phase is read in the other, and every walk array is set up
    // again at the start of each cell.
    union {
        struct {                      // walk
            T px[P], py[P], pz[P], pd[P];     // plane: normal, offset (n.x = offset)
            T pn[P];                          // |normal| (1 for the FP64 form and the walls)
            T vsd[V];                         // signed distances of the current cut
            float vr[V];                      // (|v| + e_v)^2 of each slot (FP32), |v|^2 rounded up (FP64)
            T cbx[32], cby[32], cbz[32], cb2[32];   // kept candidates waiting for a full window ...
            uint32_t cbj[32];                 // ... their sorted indices
            int32_t cbid[32];                 // ... and local original ids
            uint32_t nbeg[32], ncnt[32];      // crowded bins: the 27 neighbour bins' ranges ...
            float nd[32];                     // ... and the squared distance to their nearest point
            uint32_t pending;                 // crowded bins still to handle (mask over the 27)
            T sdx[32], sdy[32], sdz[32], sd2[32];   // each lane's seed: offset, squared length ...
            uint32_t sdj[32];                 // ... sorted index (~0: none)
            int32_t sdcid[32];                // ... and local original id
            int32_t cbin;                     // the crowded bin being handled
            int32_t ring;                     // Chebyshev ring being walked ...
            uint32_t r0;                      // ... and the position in it
            uint32_t pused[(P + 31) / 32];    // plane recycling: planes referenced by live vertices
            float ve[VF];                     // vertex error bounds (mirror of CellRegs::ve)
            uint16_t items[V + 32];           // boundary edges of a cut: slot | edge << 8
            uint8_t fl[V + 32];               // free-slot stack (top = lowest free slot)
            // new-vertex ring maps: gen << 8 | slot; entries with another
            // cut's tag are stale
            uint16_t mapf[P], maps[P];
            float fvx[VD], fvy[VD], fvz[VD];  // FP64 form: the vertices rounded to FP32 (window pre-test)
        };
        struct {                      // finalize
            // FP32 forms only: face planes {n, h} (n.x = h), their distance
            // from the site, and per-vertex FP32 corrections to the FP64
            // position.  The FP64-accurate finish keeps the planes in FP64;
            // the FP32 form keeps them as FP32 pairs: n = fq + ql, h = hh + hl.
            union {
                struct {
                    double qx[PF], qy[PF], qz[PF], qh[PF];
                };
                struct {
                    float qlx[PF], qly[PF], qlz[PF], qhh[PF], qhl[PF];
                };
            };
            float fqx[PF], fqy[PF], fqz[PF], qdist[PF];
            float dx[VF], dy[VF], dz[VF];
            double rx[VF], ry[VF], rz[VF];    // exact form: refined FP64 positions
            uint32_t fdeg[P];                 // live vertices per face
            int32_t flist[P];                 // compacted face ids
            uint8_t fsta[P];                  // one vertex of each face
            uint8_t rank2p[P];                // geometry output: rank -> plane
        };
    };
};

__device__ __forceinline__ unsigned warp_incl_scan_u(unsigned v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// Position of the q-th (0-based) set bit of m; requires q < popc(m).
__device__ __forceinline__ int select32(uint32_t m, int q) {
    int pos = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const uint32_t low = (1u << (pos + s)) - 1u;
        if (__popc(m & low) <= q) pos += s;
    }
    return pos;
}

template <int K>
__device__ __forceinline__ int select_k(const uint32_t (&m)[K], int q) {
    int res = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int c = __popc(m[k]);
        if (res < 0) {
            if (q < c) res = k * 32 + select32(m[k], q);
            else q -= c;
        }
    }
    return res;
}

template <int K>
__device__ __forceinline__ bool bit_k(const uint32_t (&m)[K], int s) {
    uint32_t w = m[0];
#pragma unroll
    for (int k = 1; k < K; ++k)
        if ((s >> 5) == k) w = m[k];
    return (w >> (s & 31)) & 1u;
}

template <int K>
__device__ __forceinline__ void set_k(uint32_t (&m)[K], int s) {
#pragma unroll
    for (int k = 0; k < K; ++k)
        if ((s >> 5) == k) m[k] |= 1u << (s & 31);
}

__device__ __forceinline__ int plane_of(uint32_t t, int i) { return (int)((t >> (8 * i)) & 0xFFu); }

// Error-free transforms (Knuth's TwoSum; the product's rounding error by one
// FMA): s + e == a + b and p + e == a * b exactly.  Explicit round-to-nearest
// intrinsics keep the compiler from contracting or reordering them.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

// q = b / d and r = b % d, exactly, for b < 2^32 and a quotient below 2^11
// (bin coordinates: cpd <= 1625).  The FP32 estimate b * (1/d) carries three
// roundings of 2^-24 relative, under 2e-4 on such a quotient, so its floor is
// off by at most one and one correction step settles it.
__device__ __forceinline__ void divmod_est(uint32_t b, uint32_t d, float rcp, uint32_t& q, uint32_t& r) {
    long long qq = (long long)((float)b * rcp);
    long long rr = (long long)b - qq * (long long)d;
    if (rr < 0) {
        --qq;
        rr += d;
    } else if (rr >= (long long)d) {
        ++qq;
        rr -= d;
    }
    q = (uint32_t)qq;
    r = (uint32_t)rr;
}

// Bin coordinates of local bin id b = (x * cpd + y) * cpd + z
// (get_cell_from_indices, celery.rs:317-325), without FP64.
__device__ __forceinline__ void split_bin(uint32_t b, int cpd, float rcp, float rcp2, int& x, int& y, int& z) {
    const uint32_t c = (uint32_t)cpd;
    uint32_t qx, rx, qy, ry;
    divmod_est(b, c * c, rcp2, qx, rx);
    divmod_est(rx, c, rcp, qy, ry);
    x = (int)qx;
    y = (int)qy;
    z = (int)ry;
}

// Signed distance n.v - offset.
__device__ __forceinline__ float sdist(float nx, float ny, float nz, float off, float x, float y, float z) {
    return fmaf(nx, x, fmaf(ny, y, fmaf(nz, z, -off)));
}
__device__ __forceinline__ double sdist(double nx, double ny, double nz, double off, double x, double y,
                                        double z) {
    return fma(nx, x, fma(ny, y, fma(nz, z, -off)));
}

// Upper bound of sqrt(x) for the FP32 form's bounds (cell radius, plane
// norms): rsqrt is within 2 ulp and the product adds half an ulp, so the
// 2^-20 inflation keeps it above the exact root.  0 and NaN give 0, +inf
// stays +inf.  Double inputs keep the IEEE square root.
__device__ __forceinline__ float sqrt_up(float x) {
    const float r = x * rsqrtf(x) * 1.00000095367431640625f;
    return x > 0.f ? (x < INFINITY ? r : x) : 0.f;
}
__device__ __forceinline__ double sqrt_up(double x) { return sqrt(x); }
// Reciprocal for the FP32 Cramer solves: the hardware approximation (about
// 1 ulp); its error sits well inside the vertex error bound kVertexErr.
__device__ __forceinline__ float recip(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

// Bisector of the site (origin) and r (halfway_from_origin_to, vector3.rs:223-239).
// FP32 form: the same plane unnormalised, n = r, off = r.r / 2; rn = |r|.
__device__ __forceinline__ void bisector(float rx, float ry, float rz, float r2, float& nx, float& ny,
                                         float& nz, float& off, float& rn) {
    nx = rx;
    ny = ry;
    nz = rz;
    off = 0.5f * r2;
    rn = sqrt_up(r2);     // an upper bound: it only widens the guard band
}
// FP64 form: unnormalised too, with rn = r.r = |n|^2, so that the
// reference's test of the normalised signed distance against 1e-12
// (Plane::vector_location, vector3.rs:170-185) compares with one threshold
// (tol_of): no FP64 square root and no division per candidate.  A normalised
// plane cost ~27 FP64-pipe instructions per candidate, and the plain FP64 form
// is bound by that pipe.
__device__ __forceinline__ void bisector(double rx, double ry, double rz, double r2, double& nx,
                                         double& ny, double& nz, double& off, double& rn) {
    nx = rx;
    ny = ry;
    nz = rz;
    off = 0.5 * r2;
    rn = r2;
}

// 1/d for the FP64 form's edge interpolation, by Newton-Raphson: the FP32
// reciprocal, then two steps y' = y + y (1 - d y) in FP64, each of which
// squares the relative error (2^-23 -> 2^-46 -> the FP64 rounding, about 2
// ulp in all).  Outside FP32's normal range, the FP64 division.
__device__ __forceinline__ double recip_nr(double d) {
    const float df = (float)d;
    const float a = fabsf(df);
    if (!(a > 1e-36f && a < 1e36f)) return 1.0 / d;
    double y = (double)__frcp_rn(df);
    double e = fma(-d, y, 1.0);
    y = fma(y, e, y);
    e = fma(-d, y, 1.0);
    return fma(y, e, y);
}

// The FP64 form's tolerance for a plane with |n|^2 = n2: Outside is
// sd > 1e-12 |n|, Inside sd < -1e-12 |n| (the reference's test on the
// normalised distance).  |n| comes from the FP32 square root: off by ~1e-7 of
// 1e-12 |n|, far inside the FP64 rounding of a signed distance, and each test
// is one compare.  Planes beyond FP32's range take the FP64 root.
__device__ __forceinline__ double tol_of(double n2) {
    const float n2f = (float)n2;
    return n2f < 1e37f ? (double)(1e-12f * sqrtf(n2f)) : kTolerance * sqrt(n2);
}

__device__ __forceinline__ float round_up_f(float x) { return x; }
__device__ __forceinline__ float round_up_f(double x) { return __double2float_ru(x); }

// A vertex's share of the cell radius: (|v| + e_v)^2 in the FP32 form (|v|
// from the upper-bound root), |v|^2 rounded up to FP32 in the FP64 form (the
// radius only bounds the search, and FP32 keeps its warp maximum off the FP64
// pipe).
__device__ __forceinline__ float vrad2(float x, float y, float z, float e) {
    const float r = sqrt_up(x * x + y * y + z * z) + e;
    return r * r;
}
__device__ __forceinline__ float vrad2(double x, double y, double z, double) {
    return __double2float_ru(x * x + y * y + z * z);
}

// Per-warp work counters (reported when ClipParams::work_ctr is set).  The
// lean first-pass form does not count: the registers cost it 2%.
struct Work {
    unsigned tested = 0, cuts = 0, newv = 0, windows = 0, batches = 0;
};

template <typename T, int K>
struct CellRegs {
    T vx[K], vy[K], vz[K];
    T ve[K];          // FP32 form: bound on each vertex's position error
    uint32_t lm[K];   // live masks (warp-uniform)
    int np;           // planes used (warp-uniform)
    int nfree;        // entries on the free-slot stack (warp-uniform)
    uint32_t gen;     // tag of the current cut in the ring maps, 0..255 (warp-uniform)
};

// The general form of a cut (more than 32 edges leave the Outside
// vertices): owners loop over their edges; placement runs in rounds of 32.
// The plane table is full: find a plane id (not a wall) that no live vertex
// references any more, or -1.  Faces cut away entirely leave such ids
// behind; cells cut hundreds of times (next to dense clusters) need them.
template <typename T, int K>
__device__ __noinline__ int recycle_plane(Smem<T, K>& S, const CellRegs<T, K>& C, int lane) {
    using S_t = Smem<T, K>;
    constexpr int NW = (S_t::P + 31) / 32;
    for (int w = lane; w < NW; w += 32) S.pused[w] = 0;
    __syncwarp();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if ((C.lm[k] >> lane) & 1u) {
            const uint32_t t = S.tri[k * 32 + lane];
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const int p = plane_of(t, e);
                if (p < S_t::P) atomicOr(&S.pused[p >> 5], 1u << (p & 31));
            }
        }
    }
    __syncwarp();
    int res = -1;
    for (int w = 0; w < NW && res < 0; ++w) {
        uint32_t fr = ~S.pused[w];
        if (w == 0) fr &= ~0x3Fu;                                  // the walls stay
        if (w == NW - 1 && (S_t::P & 31)) fr &= (1u << (S_t::P & 31)) - 1u;
        if (fr) res = w * 32 + __ffs(fr) - 1;
    }
    __syncwarp();
    return res;
}

template <typename T, int K>
struct Regs {
    T v[K];
};

template <typename T, int K, bool GUARD, bool RESOLVE>
__device__ __forceinline__ int cut_general(Smem<T, K>& S, CellRegs<T, K>& C, const Regs<T, K> sdv,
                                        const Regs<uint32_t, K> omv, T nx, T ny, T nz, T off, T rn, T cR,
                                        T gr, int32_t id, uint32_t src, int f, int lane, int* P_check) {
    using S_t = Smem<T, K>;
    const T(&sd)[K] = sdv.v;
    const uint32_t(&om)[K] = omv.v;

    // Signed distances of live vertices go to shared memory for the lanes
    // that place new vertices; my Outside vertices' triples and neighbours are
    // read before any slot is reused.
    uint32_t xt[K], xa[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int s = k * 32 + lane;
        if (!GUARD && ((C.lm[k] >> lane) & 1u)) S.vsd[s] = sd[k];   // read by the FP64 interpolation
        xt[k] = 0;
        xa[k] = 0;
        if ((om[k] >> lane) & 1u) {
            xt[k] = S.tri[s];
            xa[k] = S.adj[s];
        }
    }
    // Every slot and plane id read below must be in range; a violation
    // (inconsistent topology) abandons the cell before anything is written.
    bool badref = false;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if ((om[k] >> lane) & 1u) {
#pragma unroll
            for (int e = 0; e < 3; ++e)
                badref |= plane_of(xt[k], e) >= C.np || plane_of(xa[k], e) >= S_t::V;
        }
    }
    if (__any_sync(FULL, badref)) return -ST_DEGEN;
    // Boundary edges: edges of Outside vertices whose neighbour is not Outside.
    unsigned bnd = 0;
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if ((om[k] >> lane) & 1u) {
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const int nb = plane_of(xa[k], e);
                if (!bit_k<K>(om, nb)) {
                    bnd |= 1u << (3 * k + e);
                    ++cnt;
                }
            }
        }
    }
    const unsigned incl = warp_incl_scan_u((unsigned)cnt, lane);
    const int B = (int)__shfl_sync(FULL, incl, 31);
    const int q0 = (int)incl - cnt;
    int nlive = 0;
    uint32_t fm[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint32_t keep = C.lm[k] & ~om[k];
        nlive += __popc(keep);
        fm[k] = ~keep;
    }
    if (K == 8) fm[K - 1] &= 0x7FFFFFFFu;
    if (nlive + B > S_t::VUSE) return -ST_VCAP;
    const int rounds = (B + 31) >> 5;
    if (rounds > 1) {
        // More than 32 new vertices (a cut through a large cell): make sure
        // no Outside slot is reused before every round has read it.
        int nfree_clean = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) nfree_clean += __popc(fm[k] & ~om[k]);
        if (nfree_clean < B) return -ST_VCAP;
#pragma unroll
        for (int k = 0; k < K; ++k) fm[k] &= ~om[k];
    }
    // Owners list their boundary edges (slot | edge << 8) at their prefix
    // positions; lane l then places new vertex l (+ 32 per round).
    uint16_t* items = S.items;
    {
        int qq = q0;
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
            for (int e = 0; e < 3; ++e)
                if (bnd & (1u << (3 * k + e)))
                    items[tess_chk(qq++, S_t::V + 32, P_check, CK_SLOT)] = (uint16_t)((k * 32 + lane) | (e << 8));
    }
    __syncwarp();
    uint32_t newm[K];
#pragma unroll
    for (int k = 0; k < K; ++k) newm[k] = 0;
    bool bad = false;
    bool numbad = false;
    for (int r0 = 0; r0 < B; r0 += 32) {
        const int qi = r0 + lane;
        const bool act = qi < B;
        int y = 0, a = 0, b = 0, slot = 0;
        uint32_t ty = 0;
        T px = 0, py = 0, pz = 0, pe = 0;
        if (act) {
            const uint32_t it = items[qi];
            const int x = it & 0xFF, e = it >> 8;
            const uint32_t xt_ = S.tri[x], xa_ = S.adj[x];
            a = plane_of(xt_, e);
            b = plane_of(xt_, e == 2 ? 0 : e + 1);
            y = plane_of(xa_, e);
            const T xx = S.vx[x], xy = S.vy[x], xz = S.vz[x], xsd = S.vsd[x];
            const T yx = S.vx[y], yy = S.vy[y], yz = S.vz[y], ysd = S.vsd[y];
            ty = S.tri[y];
            // intersection(outside X, inside Y) (vector3.rs:213-219); an
            // Incident Y is kept as the new vertex (polyhedron.rs:554-565)
            if constexpr (GUARD) {
                // FP32 form: the vertex of planes (a, b, f) by Cramer's rule,
                // x = (h_a (n_b x n_f) + h_b (n_f x n_a) + h_f (n_a x n_b)) / det.
                // Its error depends on its own conditioning only (not on the
                // edge it came from): |dx| <~ c |x| / |det of unit normals|.
                const T ax = S.px[a], ay = S.py[a], az = S.pz[a], ah = S.pd[a];
                const T bx = S.px[b], by = S.py[b], bz = S.pz[b], bh = S.pd[b];
                const T bfx = by * nz - bz * ny, bfy = bz * nx - bx * nz, bfz = bx * ny - by * nx;
                const T fax = ny * az - nz * ay, fay = nz * ax - nx * az, faz = nx * ay - ny * ax;
                const T abx = ay * bz - az * by, aby = az * bx - ax * bz, abz = ax * by - ay * bx;
                const T det = ax * bfx + ay * bfy + az * bfz;
                const T inv = recip(det);
                px = (ah * bfx + bh * fax + off * abx) * inv;
                py = (ah * bfy + bh * fay + off * aby) * inv;
                pz = (ah * bfz + bh * faz + off * abz) * inv;
                // e = kVertexErr |x|_1 / dhat, dhat = |det| / (|n_a| |n_b| |n_f|)
                const T x1 = fabs(px) + fabs(py) + fabs(pz);
                pe = (T)kVertexErr * x1 * (S.pn[a] * S.pn[b] * rn) * fabs(inv);
                if (!(pe < (T)1e30)) pe = (T)1e30;
                // hybrid form: a cell that keeps going after FP64-decided
                // tests must not carry an ill-conditioned (or non-finite)
                // FP32 vertex; it re-runs in FP64 instead
                if (RESOLVE && !(pe <= (T)kNumBad * cR)) numbad = true;
                // plus the vertex's share of a plane test's FP32 rounding
                pe += gr * x1;
            } else {
                const T den = xsd - ysd;
                const T t = ysd >= -(T)tol_of(rn) ? (T)1 : xsd * recip_nr(den);
                px = xx + (yx - xx) * t;
                py = xy + (yy - xy) * t;
                pz = xz + (yz - xz) * t;
            }
            slot = tess_chk(select_k<K>(fm, qi), S_t::V, P_check, CK_SLOT);
        }
        if (RESOLVE && __any_sync(FULL, numbad)) return -ST_GUARD;
        __syncwarp();
        if (act) {
            S.vx[slot] = px;
            S.vy[slot] = py;
            S.vz[slot] = pz;
            if constexpr (GUARD) S.ve[slot] = pe;
            if constexpr (sizeof(T) == 8) {
                // FP64 form: the FP32 copies (rounded to nearest) serve the
                // window pre-test and the cell radius: |v|^2 from them, times
                // 1 + 5 * 2^-23 (the copies' and the sum's rounding are at
                // most 2.5 * 2^-23), is an upper bound, off the FP64 pipe
                const float fx = (float)px, fy = (float)py, fz = (float)pz;
                S.fvx[slot % S_t::VD] = fx;
                S.fvy[slot % S_t::VD] = fy;
                S.fvz[slot % S_t::VD] = fz;
                S.vr[slot] = fmaf(fx, fx, fmaf(fy, fy, fz * fz)) * 1.000000596f;
            } else {
                S.vr[slot] = vrad2(px, py, pz, pe);
            }
            S.tri[slot] = (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)f << 16);
            // Y's pointer back to X is the edge (b, a) of Y's triple.
            const int yi = (plane_of(ty, 0) == b && plane_of(ty, 1) == a)   ? 0
                           : (plane_of(ty, 1) == b && plane_of(ty, 2) == a) ? 1
                                                                            : 2;
            reinterpret_cast<uint8_t*>(S.adj)[4 * y + yi] = (uint8_t)slot;
            S.mapf[a] = (uint16_t)((C.gen << 8) | (uint32_t)slot);
            S.maps[b] = (uint16_t)((C.gen << 8) | (uint32_t)slot);
            S.adj[slot] = (uint32_t)y;
#pragma unroll
            for (int k = 0; k < K; ++k)
                if ((slot >> 5) == k) newm[k] |= 1u << (slot & 31);
        }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < K; ++k) newm[k] = __reduce_or_sync(FULL, newm[k]);
    // Link the ring of new vertices (each by its owner lane): across (b, f)
    // lies the new vertex whose first plane is b, across (f, a) the one whose
    // second plane is a.
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if ((newm[k] >> lane) & 1u) {
            const int s = k * 32 + lane;
            const uint32_t tt = S.tri[s];
            const int a = plane_of(tt, 0), b = plane_of(tt, 1);
            const uint32_t tag = C.gen << 8;
            const uint32_t mb = S.mapf[b], ma = S.maps[a];
            const int n1 = (mb & 0xFF00u) == tag ? (int)(mb & 0xFFu) : 0xFF;
            const int n2 = (ma & 0xFF00u) == tag ? (int)(ma & 0xFFu) : 0xFF;
            bad |= (S.mapf[a] != (tag | (uint32_t)s)) || (S.maps[b] != (tag | (uint32_t)s)) || n1 == 0xFF || n2 == 0xFF;
            S.adj[s] = (S.adj[s] & 0xFFu) | ((uint32_t)n1 << 8) | ((uint32_t)n2 << 16);
        }
    }
    if (__any_sync(FULL, bad)) return -ST_DEGEN;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        C.lm[k] = (C.lm[k] & ~om[k]) | newm[k];
        if ((newm[k] >> lane) & 1u) {
            const int s = k * 32 + lane;
            C.vx[k] = S.vx[s];
            C.vy[k] = S.vy[s];
            C.vz[k] = S.vz[s];
            if constexpr (GUARD) C.ve[k] = S.ve[s];
        }
    }
    if (lane == 0) {
        S.px[f] = nx;
        S.py[f] = ny;
        S.pz[f] = nz;
        S.pd[f] = off;
        S.pn[f] = GUARD ? rn : (T)1;
        S.pid[f] = id;
        S.psrc[f] = src;
    }
    if (f >= C.np) C.np = f + 1;
    // rebuild the free-slot stack from the live masks
    {
        int n = 0;
#pragma unroll
        for (int k = K - 1; k >= 0; --k) {
            uint32_t fr = ~C.lm[k];
            if (K == 8 && k == K - 1) fr &= 0x7FFFFFFFu;
            const int c = __popc(fr);
            // descending slot order, so the lowest free slot is on top
            if ((fr >> (31 - lane)) & 1u) {
                const uint32_t above = lane == 0 ? 0u : (fr >> (32 - lane));
                S.fl[n + __popc(above)] = (uint8_t)(k * 32 + 31 - lane);
            }
            n += c;
        }
        C.nfree = n;
    }
    __syncwarp();
    return B + 1;
}

// Clip the cell by the half-space {x : n.x - off <= 0}.
//   FP64 form: n is the unit normal of the bisector and off its offset; a
//     vertex is Outside when n.v - off > 1e-12 (vector3.rs:170-193,
//     polyhedron.rs:221).
//   FP32 form: n = r and off = r.r / 2 (the same plane, scaled by rn = |r|).
//     Every vertex carries a bound e_v on its position error, to which
//     guard_rel * |v|_1 is added at its creation.  A test with
//     |n.v - off| <= rn * (e_v + guard_rel * rn) + eC cannot be decided in
//     FP32: the cell goes to the FP64 form (ST_GUARD); eC covers the hi/lo
//     split of the positions (see run_cell).  The bound on the FP32 test,
//     with u = 2^-24, r~ the FP32 offset (|r~ - r| <= 2u |r|) and v~ the
//     FP32 vertex (|v~ - v| <= e_v):
//       fma chain rounding       3u (rn |v~|_1 + off)
//       plane normal, vertex     2u rn |v|  +  rn e_v
//       offset r.r / 2           3u rn^2
//     <= rn (e_v + 5u |v~|_1 + 4.5u rn), about rn (e_v + 3e-7 (|v~|_1 + rn));
//     the default guard_rel 4e-7 leaves a third in hand.
// Returns 1 when vertices were cut off, 0 when nothing was Outside, or
// -status.
// FP64 view of the site and its container, for deciding guard-band plane
// tests in FP64 (hybrid form).
struct Fp64Site {
    double sx, sy, sz;
    const double* blo;
    const double* bhi;
};

// Side of the vertex in slot s relative to the bisector of the site and the
// point at sorted position cj, decided in FP64: the vertex is recomputed from
// its three planes (walls, or bisectors of the site and the FP64 points that
// made them) by Cramer's rule, and classified with the reference's test on
// the normalised bisector (vector3.rs:170-239, tolerance 1e-12).  Returns 1
// (Outside), -1 (Inside or Incident) or 0 (the three planes are singular).
template <typename T, int K>
__device__ __noinline__ int resolve_fp64(const Smem<T, K>& S, const ClipParams& P, const Fp64Site& st, int s,
                                         uint32_t cj) {
    const uint32_t tt = S.tri[s];
    double n[3][3], h[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int p = plane_of(tt, e);
        if (p < 6) {
            const int a = p >> 1;
            const bool mx = p & 1;
            const double s_a = a == 0 ? st.sx : (a == 1 ? st.sy : st.sz);
            n[e][0] = a == 0 ? (mx ? 1.0 : -1.0) : 0.0;
            n[e][1] = a == 1 ? (mx ? 1.0 : -1.0) : 0.0;
            n[e][2] = a == 2 ? (mx ? 1.0 : -1.0) : 0.0;
            h[e] = mx ? (st.bhi[a] - s_a) : (s_a - st.blo[a]);
        } else {
            const uint32_t j = tess_chk(S.psrc[p], P.npts, P.check, CK_POINT);
            n[e][0] = P.spx[j] - st.sx;
            n[e][1] = P.spy[j] - st.sy;
            n[e][2] = P.spz[j] - st.sz;
            h[e] = 0.5 * (n[e][0] * n[e][0] + n[e][1] * n[e][1] + n[e][2] * n[e][2]);
        }
    }
    const double bc0 = n[1][1] * n[2][2] - n[1][2] * n[2][1], bc1 = n[1][2] * n[2][0] - n[1][0] * n[2][2],
                 bc2 = n[1][0] * n[2][1] - n[1][1] * n[2][0];
    const double ca0 = n[2][1] * n[0][2] - n[2][2] * n[0][1], ca1 = n[2][2] * n[0][0] - n[2][0] * n[0][2],
                 ca2 = n[2][0] * n[0][1] - n[2][1] * n[0][0];
    const double ab0 = n[0][1] * n[1][2] - n[0][2] * n[1][1], ab1 = n[0][2] * n[1][0] - n[0][0] * n[1][2],
                 ab2 = n[0][0] * n[1][1] - n[0][1] * n[1][0];
    const double det = n[0][0] * bc0 + n[0][1] * bc1 + n[0][2] * bc2;
    if (!(fabs(det) > 0.0)) return 0;
    const double x = (h[0] * bc0 + h[1] * ca0 + h[2] * ab0) / det;
    const double y = (h[0] * bc1 + h[1] * ca1 + h[2] * ab1) / det;
    const double z = (h[0] * bc2 + h[1] * ca2 + h[2] * ab2) / det;
    cj = tess_chk(cj, P.npts, P.check, CK_POINT);
    const double qx = P.spx[cj] - st.sx, qy = P.spy[cj] - st.sy, qz = P.spz[cj] - st.sz;
    const double q2 = qx * qx + qy * qy + qz * qz;
    const double sd = (qx * x + qy * y + qz * z - 0.5 * q2) / sqrt(q2);
    return sd > kTolerance ? 1 : -1;
}

template <typename T, int K, bool GUARD, bool RESOLVE = false>
__device__ int cut(Smem<T, K>& S, CellRegs<T, K>& C, T nx, T ny, T nz, T off, T rn, T cR, T eC, int32_t id,
                   uint32_t src, int lane, const ClipParams& P, const Fp64Site& site) {
    using S_t = Smem<T, K>;
    T sd[K];
    uint32_t om[K];
    bool gh = false;
    // the plane's share of the test's FP32 rounding (FP32 form)
    const T gr = GUARD ? (T)P.guard_rel : (T)0;
    const T rc = gr * rn;
    // FP64 form: the tolerance of the normalised test, rn = |n|^2 (see bisector)
    T tolr = 0;
    if constexpr (!GUARD) tolr = tol_of(rn);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        sd[k] = (T)0;
        om[k] = 0;
        // register sets without live vertices are skipped (the free-slot
        // stack hands out the lowest slots first, so the upper sets are
        // usually empty)
        if (C.lm[k] == 0) continue;
        const bool live = (C.lm[k] >> lane) & 1u;
        sd[k] = sdist(nx, ny, nz, off, C.vx[k], C.vy[k], C.vz[k]);
        bool out;
        if constexpr (GUARD) out = live && sd[k] > (T)0;
        else out = live && sd[k] > tolr;
        if constexpr (GUARD) gh |= live && fabs(sd[k]) <= fma(rn, C.ve[k] + rc, eC);
        om[k] = __ballot_sync(FULL, out);
    }
    if (GUARD && __any_sync(FULL, gh)) {
        if constexpr (!RESOLVE) {
            return -ST_GUARD;
        } else {
            // decide the guard-band vertices in FP64 (src is the candidate's
            // sorted index); the rest keep their FP32 decision
            bool fail = false;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (C.lm[k] == 0) continue;
                const bool live = (C.lm[k] >> lane) & 1u;
                const bool amb = live && fabs(sd[k]) <= fma(rn, C.ve[k] + rc, eC);
                bool out = live && sd[k] > (T)0;
                if (amb) {
                    const int r = resolve_fp64<T, K>(S, P, site, k * 32 + lane, src);
                    fail |= r == 0;
                    out = r > 0;
                }
                om[k] = __ballot_sync(FULL, out);
            }
            if (__any_sync(FULL, fail)) return -ST_GUARD;
        }
    }
    uint32_t anyo = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) anyo |= om[k];
    if (!anyo) return 0;
    int f = C.np;
    if (f >= S_t::P) {
        // Only the largest capacity recycles plane ids: a call here costs the
        // smaller instantiations' hot path registers even when never taken,
        // and their cells re-run at the next capacity instead.
        if constexpr (K == 8) {
            f = recycle_plane<T, K>(S, C, lane);
            if (f < 0) return -ST_PCAP;
        } else {
            return -ST_PCAP;
        }
    }
    // a new tag for this cut's ring-map entries; every 256 cuts the maps are
    // cleared, so a stale entry never carries the current tag
    C.gen = (C.gen + 1) & 0xFFu;
    if (C.gen == 0) {
        for (int i = lane; i < S_t::P; i += 32) {
            S.mapf[i] = 0xFFFF;
            S.maps[i] = 0xFFFF;
        }
        __syncwarp();
    }
    int R = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) R += __popc(om[k]);
    if (3 * R <= 32) {
        // Fast path: one lane per edge of an Outside vertex.  The Outside
        // slots are pushed onto the free-slot stack; the new vertices pop
        // slots from its top (reusing freed slots first).
        const int base = C.nfree;
        int before = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int s = k * 32 + lane;
            if (!GUARD && ((C.lm[k] >> lane) & 1u)) S.vsd[s] = sd[k];   // read by the FP64 interpolation
            if ((om[k] >> lane) & 1u)
                S.fl[tess_chk(base + before + __popc(om[k] & ((1u << lane) - 1u)), S_t::V + 32, P.check, CK_SLOT)] = (uint8_t)s;
            before += __popc(om[k]);
        }
        __syncwarp();
        const bool edge = lane < 3 * R;
        int x = 0, y = 0, a = 0, b = 0;
        bool bnd = false, bad = false;
        if (edge) {
            const int xi = (lane * 11) >> 5;          // lane / 3 for lane < 32
            const int e = lane - 3 * xi;
            x = tess_chk((int)S.fl[tess_chk(base + xi, S_t::V + 32, P.check, CK_SLOT)], S_t::V, P.check, CK_SLOT);
            const uint32_t xt_ = S.tri[x], xa_ = S.adj[x];
            a = plane_of(xt_, e);
            b = plane_of(xt_, e == 2 ? 0 : e + 1);
            y = plane_of(xa_, e);
            bad = a >= C.np || b >= C.np || y >= S_t::V;
            bnd = !bad && !bit_k<K>(om, y);
        }
        if (__any_sync(FULL, bad)) return -ST_DEGEN;
        const unsigned bm = __ballot_sync(FULL, bnd);
        const int B = __popc(bm);
        // capacity: the stack (with the pushed Outside slots) must hold B
        if (B > base + R) return -ST_VCAP;
        const int q = __popc(bm & ((1u << lane) - 1u));
        int slot = 0;
        uint32_t ty = 0;
        T px = 0, py = 0, pz = 0, pe = 0;
        bool numbad = false;
        if (bnd) {
            if constexpr (GUARD) {
                // the vertex of planes (a, b, f) by Cramer's rule (see above)
                const T ax = S.px[a], ay = S.py[a], az = S.pz[a], ah = S.pd[a];
                const T bx = S.px[b], by = S.py[b], bz = S.pz[b], bh = S.pd[b];
                const T bfx = by * nz - bz * ny, bfy = bz * nx - bx * nz, bfz = bx * ny - by * nx;
                const T fax = ny * az - nz * ay, fay = nz * ax - nx * az, faz = nx * ay - ny * ax;
                const T abx = ay * bz - az * by, aby = az * bx - ax * bz, abz = ax * by - ay * bx;
                const T det = ax * bfx + ay * bfy + az * bfz;
                const T inv = recip(det);
                px = (ah * bfx + bh * fax + off * abx) * inv;
                py = (ah * bfy + bh * fay + off * aby) * inv;
                pz = (ah * bfz + bh * faz + off * abz) * inv;
                // e = kVertexErr |x|_1 / dhat, dhat = |det| / (|n_a| |n_b| |n_f|)
                const T x1 = fabs(px) + fabs(py) + fabs(pz);
                pe = (T)kVertexErr * x1 * (S.pn[a] * S.pn[b] * rn) * fabs(inv);
                if (!(pe < (T)1e30)) pe = (T)1e30;
                // hybrid form: a cell that keeps going after FP64-decided
                // tests must not carry an ill-conditioned (or non-finite)
                // FP32 vertex; it re-runs in FP64 instead
                if (RESOLVE && !(pe <= (T)kNumBad * cR)) numbad = true;
                // plus the vertex's share of a plane test's FP32 rounding
                pe += gr * x1;
            } else {
                const T xx = S.vx[x], xy = S.vy[x], xz = S.vz[x], xsd = S.vsd[x];
                const T yx = S.vx[y], yy = S.vy[y], yz = S.vz[y], ysd = S.vsd[y];
                const T t = ysd >= -tolr ? (T)1 : xsd * recip_nr(xsd - ysd);
                px = xx + (yx - xx) * t;
                py = xy + (yy - xy) * t;
                pz = xz + (yz - xz) * t;
            }
            ty = S.tri[y];
            slot = tess_chk((int)S.fl[tess_chk(base + R - 1 - q, S_t::V + 32, P.check, CK_SLOT)], S_t::V, P.check, CK_SLOT);
        }
        if (RESOLVE && __any_sync(FULL, numbad)) return -ST_GUARD;
        __syncwarp();
        if (bnd) {
            S.vx[slot] = px;
            S.vy[slot] = py;
            S.vz[slot] = pz;
            if constexpr (GUARD) S.ve[slot] = pe;
            if constexpr (sizeof(T) == 8) {
                // FP64 form: the FP32 copies (rounded to nearest) serve the
                // window pre-test and the cell radius: |v|^2 from them, times
                // 1 + 5 * 2^-23 (the copies' and the sum's rounding are at
                // most 2.5 * 2^-23), is an upper bound, off the FP64 pipe
                const float fx = (float)px, fy = (float)py, fz = (float)pz;
                S.fvx[slot % S_t::VD] = fx;
                S.fvy[slot % S_t::VD] = fy;
                S.fvz[slot % S_t::VD] = fz;
                S.vr[slot] = fmaf(fx, fx, fmaf(fy, fy, fz * fz)) * 1.000000596f;
            } else {
                S.vr[slot] = vrad2(px, py, pz, pe);
            }
            S.tri[slot] = (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)f << 16);
            // Y's pointer back to X is the edge (b, a) of Y's triple.
            const int yi = (plane_of(ty, 0) == b && plane_of(ty, 1) == a)   ? 0
                           : (plane_of(ty, 1) == b && plane_of(ty, 2) == a) ? 1
                                                                            : 2;
            reinterpret_cast<uint8_t*>(S.adj)[4 * y + yi] = (uint8_t)slot;
            S.mapf[a] = (uint16_t)((C.gen << 8) | (uint32_t)slot);
            S.maps[b] = (uint16_t)((C.gen << 8) | (uint32_t)slot);
        }
        __syncwarp();
        if (bnd) {
            // across (b, f): the new vertex whose first plane is b; across
            // (f, a): the one whose second plane is a (entries of this cut only)
            const uint32_t tag = C.gen << 8;
            const uint32_t mb = S.mapf[b], ma = S.maps[a];
            const int n1 = (mb & 0xFF00u) == tag ? (int)(mb & 0xFFu) : 0xFF;
            const int n2 = (ma & 0xFF00u) == tag ? (int)(ma & 0xFFu) : 0xFF;
            bad = (S.mapf[a] != (tag | (uint32_t)slot)) || (S.maps[b] != (tag | (uint32_t)slot)) || n1 == 0xFF ||
                  n2 == 0xFF;
            S.adj[slot] = (uint32_t)y | ((uint32_t)n1 << 8) | ((uint32_t)n2 << 16);
        }
        if (__any_sync(FULL, bad)) return -ST_DEGEN;
        C.nfree = base + R - B;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const uint32_t nm = __reduce_or_sync(FULL, (bnd && (slot >> 5) == k) ? (1u << (slot & 31)) : 0u);
            C.lm[k] = (C.lm[k] & ~om[k]) | nm;
            if ((nm >> lane) & 1u) {
                const int s = k * 32 + lane;
                C.vx[k] = S.vx[s];
                C.vy[k] = S.vy[s];
                C.vz[k] = S.vz[s];
                if constexpr (GUARD) C.ve[k] = S.ve[s];
            }
        }
        // the plane (predicated stores of one lane: no divergent branches)
        if (lane == 0) {
            S.px[f] = nx;
            S.py[f] = ny;
            S.pz[f] = nz;
            S.pd[f] = off;
            S.pn[f] = GUARD ? rn : (T)1;
            S.pid[f] = id;
            S.psrc[f] = src;
        }
        if (f >= C.np) C.np = f + 1;
        __syncwarp();
        return B + 1;
    }
    Regs<T, K> sdv;
    Regs<uint32_t, K> omv;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        sdv.v[k] = sd[k];
        omv.v[k] = om[k];
    }
    return cut_general<T, K, GUARD, RESOLVE>(S, C, sdv, omv, nx, ny, nz, off, rn, cR, gr, id, src, f, lane, P.check);
}

// Squared radius of the cell about its site: max |v|^2 over live vertices,
// an upper bound (FP32 form: each |v| inflated by its error bound; FP64
// form: an FP32 upper bound of each |v|^2).  Each slot's term (vrad2) is written with
// the vertex, so a cut costs one load per register set here instead of a
// square root per vertex.
template <typename T, int K>
__device__ __forceinline__ T live_r2(const Smem<T, K>& S, const CellRegs<T, K>& C, int lane) {
    float r2 = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (C.lm[k] == 0) continue;
        if ((C.lm[k] >> lane) & 1u) r2 = fmaxf(r2, S.vr[k * 32 + lane]);
    }
    // r2 >= 0 and never NaN (fmaxf drops NaN): its bits order like its
    // value, so one warp reduction of the bits gives the maximum
    return (T)__uint_as_float(__reduce_max_sync(FULL, __float_as_uint(r2)));
}

// The same maximum as an FP32 value (the FP64 form's search bounds).
template <typename T, int K>
__device__ __forceinline__ float live_r2f(const Smem<T, K>& S, const CellRegs<T, K>& C, int lane) {
    float r2 = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (C.lm[k] == 0) continue;
        if ((C.lm[k] >> lane) & 1u) r2 = fmaxf(r2, S.vr[k * 32 + lane]);
    }
    return __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(r2)));
}

__device__ __forceinline__ void ring_offset(int s, uint32_t r, int& i, int& j, int& k) {
    const uint32_t a = 2u * s + 1u, b = 2u * s - 1u;
    const uint32_t nx = 2u * a * a, ny = 2u * b * a;
    if (r < nx) {
        const uint32_t side = r / (a * a), rem = r % (a * a);
        i = side ? s : -s;
        j = (int)(rem / a) - s;
        k = (int)(rem % a) - s;
    } else if (r < nx + ny) {
        r -= nx;
        const uint32_t side = r / (b * a), rem = r % (b * a);
        j = side ? s : -s;
        i = (int)(rem / a) - (s - 1);
        k = (int)(rem % a) - s;
    } else {
        r -= nx + ny;
        const uint32_t side = r / (b * b), rem = r % (b * b);
        k = side ? s : -s;
        i = (int)(rem / b) - (s - 1);
        j = (int)(rem % b) - (s - 1);
    }
}

template <typename T, int K, bool GEO, int FORM>
__device__ void run_cell(const ClipParams& P, Smem<T, K>& S, uint32_t gs, int lane, Work& W) {
    using S_t = Smem<T, K>;
    constexpr bool GUARD = sizeof(T) == 4;
    constexpr int BASE = FORM & 3;                                  // lean, std or hybrid
    constexpr bool EXACT = GUARD && (FORM & kFormExact) != 0;       // FP64-accurate finalize
    // the lean first pass sends crowded cells to a seeded pass instead (the
    // seeding code would cost its hot loop registers)
    constexpr bool kSeedForm = BASE != kFormLean;
    // ---- diagram of this cell ----
    int d = 0;
    if (P.ndiag > 1 && !P.at_point) {
        int lo = 0, hi = P.ndiag - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (P.diags[mid].pt_base <= gs) lo = mid;
            else hi = mid - 1;
        }
        d = lo;
    }
    const DiagDesc& D = P.diags[d];
    const uint32_t pt_base = D.pt_base;
    const uint64_t bin_base = D.bin_base;
    const uint32_t tab_len = D.tab_len;
    double sx, sy, sz;
    uint32_t self = 0xFFFFFFFFu, orig = 0;
    if (P.at_point) {
        sx = P.point[0];
        sy = P.point[1];
        sz = P.point[2];
    } else {
        sx = P.spx[gs];
        sy = P.spy[gs];
        sz = P.spz[gs];
        self = gs;
        orig = tess_chk(P.sorted[tess_chk(gs, P.npts, P.check, CK_POINT)], P.npts, P.check, CK_POINT);
    }
    // FP32 form: the site as an FP32 pair (hi + lo) relative to the diagram's
    // centre, like the points, so candidate offsets (p - site) come out of
    // FP32 arithmetic nearly as accurate as FP64's.
    float shx = 0.f, shy = 0.f, shz = 0.f, slx = 0.f, sly = 0.f, slz = 0.f;
    if constexpr (GUARD) {
        if (P.at_point) {
            const double ux = sx - D.ctr[0], uy = sy - D.ctr[1], uz = sz - D.ctr[2];
            shx = __double2float_rn(ux); slx = __double2float_rn(ux - (double)shx);
            shy = __double2float_rn(uy); sly = __double2float_rn(uy - (double)shy);
            shz = __double2float_rn(uz); slz = __double2float_rn(uz - (double)shz);
        } else {
            shx = P.shi[3ull * gs]; shy = P.shi[3ull * gs + 1]; shz = P.shi[3ull * gs + 2];
            slx = P.slo[3ull * gs]; sly = P.slo[3ull * gs + 1]; slz = P.slo[3ull * gs + 2];
        }
    }

    // ---- the container box, translated by -site (polyhedron.rs:268-392) ----
    const double* blo = P.box_override ? P.box : D.blo;
    const double* bhi = P.box_override ? P.box + 3 : D.bhi;
    const Fp64Site fsite{sx, sy, sz, blo, bhi};
    CellRegs<T, K> C;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        C.vx[k] = C.vy[k] = C.vz[k] = (T)0;
        C.ve[k] = (T)0;
        C.lm[k] = 0;
    }
    C.lm[0] = 0xFFu;
    C.np = 6;
    // The FP32 first pass sets up without the FP64 pipe (dozens of cycles per
    // warp instruction on this part): box offsets from the FP32 pairs of the
    // box and the site relative to the centre, one rounding each side of the
    // sum (<= 2^-23 relative) plus the pairs' own ~2^-47 of the extent.
    constexpr bool kF32Setup = BASE == kFormLean;
    if (lane < 6) {
        const int a = lane >> 1;
        const bool mx = lane & 1;
        T offt;
        if constexpr (kF32Setup) {
            const float sh_a = a == 0 ? shx : (a == 1 ? shy : shz);
            const float sl_a = a == 0 ? slx : (a == 1 ? sly : slz);
            offt = mx ? ((D.bhi_hi[a] - sh_a) + (D.bhi_lo[a] - sl_a)) : ((sh_a - D.blo_hi[a]) + (sl_a - D.blo_lo[a]));
        } else {
            const double s_a = a == 0 ? sx : (a == 1 ? sy : sz);
            offt = (T)(mx ? (bhi[a] - s_a) : (s_a - blo[a]));
        }
        const T sg = mx ? (T)1 : (T)-1;
        S.px[lane] = a == 0 ? sg : (T)0;
        S.py[lane] = a == 1 ? sg : (T)0;
        S.pz[lane] = a == 2 ? sg : (T)0;
        S.pd[lane] = offt;
        S.pn[lane] = (T)1;
        S.pid[lane] = -1 - lane;   // -1 x_min, -2 x_max, -3 y_min, -4 y_max, -5 z_min, -6 z_max
    }
    if (lane < 8) {
        const int bx = lane & 1, by = (lane >> 1) & 1, bz = (lane >> 2) & 1;
        if constexpr (kF32Setup) {
            C.vx[0] = bx ? ((D.bhi_hi[0] - shx) + (D.bhi_lo[0] - slx)) : ((D.blo_hi[0] - shx) + (D.blo_lo[0] - slx));
            C.vy[0] = by ? ((D.bhi_hi[1] - shy) + (D.bhi_lo[1] - sly)) : ((D.blo_hi[1] - shy) + (D.blo_lo[1] - sly));
            C.vz[0] = bz ? ((D.bhi_hi[2] - shz) + (D.bhi_lo[2] - slz)) : ((D.blo_hi[2] - shz) + (D.blo_lo[2] - slz));
        } else {
            C.vx[0] = (T)((bx ? bhi[0] : blo[0]) - sx);
            C.vy[0] = (T)((by ? bhi[1] : blo[1]) - sy);
            C.vz[0] = (T)((bz ? bhi[2] : blo[2]) - sz);
        }
        S.vx[lane] = C.vx[0];
        S.vy[lane] = C.vy[0];
        S.vz[lane] = C.vz[0];
        if constexpr (sizeof(T) == 8) {
            S.fvx[lane % S_t::VD] = (float)C.vx[0];
            S.fvy[lane % S_t::VD] = (float)C.vy[0];
            S.fvz[lane % S_t::VD] = (float)C.vz[0];
        }
        if constexpr (GUARD) {
            // the corner's rounding to FP32: 2^-24 relative per component from
            // FP64, 2^-23 from the FP32 pairs (doubled here)
            C.ve[0] = ((T)(kF32Setup ? 2.5e-7 : 1.2e-7) + (T)P.guard_rel) * (fabs(C.vx[0]) + fabs(C.vy[0]) + fabs(C.vz[0]));
            S.ve[lane] = C.ve[0];
        }
        S.vr[lane] = vrad2(C.vx[0], C.vy[0], C.vz[0], C.ve[0]);
        const int pX = bx, pY = 2 + by, pZ = 4 + bz;
        const int sgn = (bx ? 1 : -1) * (by ? 1 : -1) * (bz ? 1 : -1);
        const int t0 = pX, t1 = sgn > 0 ? pY : pZ, t2 = sgn > 0 ? pZ : pY;
        S.tri[lane] = (uint32_t)t0 | ((uint32_t)t1 << 8) | ((uint32_t)t2 << 16);
        auto flip = [](int p) { return p < 2 ? 1 : (p < 4 ? 2 : 4); };
        const int n0 = lane ^ flip(t2), n1 = lane ^ flip(t0), n2 = lane ^ flip(t1);
        S.adj[lane] = (uint32_t)n0 | ((uint32_t)n1 << 8) | ((uint32_t)n2 << 16);
    }
    C.gen = 0;
    for (int i = lane; i < S_t::P; i += 32) {
        S.mapf[i] = 0xFFFF;
        S.maps[i] = 0xFFFF;
    }
    // free-slot stack: slots 8 .. VUSE-1, lowest on top
    C.nfree = S_t::VUSE - 8;
    for (int i = lane; i < C.nfree; i += 32) S.fl[i] = (uint8_t)(S_t::VUSE - 1 - i);
    __syncwarp();
    T R2;
    // FP64 form: the same value in FP32 (R2 is an FP32 upper bound in every
    // form), for the search bounds, so that they stay off the FP64 pipe;
    // 4 R2f is then exactly the round_up_f(4 R2) of the other forms
    float R2f = 0.f;
    if constexpr (sizeof(T) == 8) {
        R2f = live_r2f(S, C, lane);
        R2 = (T)R2f;
    } else {
        R2 = live_r2(S, C, lane);
    }
    // guard_rel * cell radius: the hybrid form's limit on a vertex's error bound
    T cR = GUARD ? (T)P.guard_rel * sqrt_up(R2) : (T)0;
    // FP32 form, the hi/lo split's share of a plane test's error (u = 2^-24,
    // positions relative to the diagram's centre): per component the offset
    // r~ = (hi_p - hi_s) + (lo_p - lo_s) is off by at most 2u |r| (relative,
    // in the bound of a test) plus eta = 6.1 u^2 (|site|_inf + R) (the lo
    // parts' rounding, the hi subtraction's share of it, the FP64 centring),
    // which moves n.v - off by at most eta (|v|_1 + 1.8 rn) <= 5.4 eta R.
    // R only shrinks, so the initial radius bounds it for the whole cell.
    // Candidates nearer than 4 eta / u (plane error above u/4 relative, beyond
    // the vertex error model) send the cell to the FP64 form.
    T eC = 0, dup2 = 0;
    if constexpr (GUARD) {
        const float sa = fmaxf(fabsf(shx), fmaxf(fabsf(shy), fabsf(shz))) * 1.001f;
        const T R = sqrt_up(R2) * (T)1.001;
        eC = (T)1.3e-13 * (sa + R) * R;
        const T d = (T)1.5e-6 * (sa + R);
        dup2 = d * d;
    }
    int status = ST_OK;

    // ---- the walk over bins in shell order (celery.rs:1023-1075) ----
    const int cpd = D.cpd;
    int cbx, cby, cbz;
    if constexpr (kF32Setup) {
        // the site's bin from the binning pass (bit-exact axis_index there)
        split_bin(P.bin[orig] - (uint32_t)bin_base, cpd, D.rcp_cpd, D.rcp_cpd2, cbx, cby, cbz);
    } else {
        cbx = axis_index(sx, D.glo[0], D.ghi[0], D.inv[0], cpd);
        cby = axis_index(sy, D.glo[1], D.ghi[1], D.inv[1], cpd);
        cbz = axis_index(sz, D.glo[2], D.ghi[2], D.inv[2], cpd);
    }
    const double radius = P.search_radius;
    const bool has_radius = radius >= 0.0;
    const int64_t tgroup = P.target_group;
    const TabEntry* tab = P.table + D.tab_base;

    // The offset p - site of sorted point j and its squared length.
    auto cand = [&](uint32_t j, T& rx, T& ry, T& rz, T& r2) {
        if constexpr (GUARD) {
            rx = (T)((P.shi[3ull * j] - shx) + (P.slo[3ull * j] - slx));
            ry = (T)((P.shi[3ull * j + 1] - shy) + (P.slo[3ull * j + 1] - sly));
            rz = (T)((P.shi[3ull * j + 2] - shz) + (P.slo[3ull * j + 2] - slz));
        } else {
            rx = (T)(P.spx[j] - sx);
            ry = (T)(P.spy[j] - sy);
            rz = (T)(P.spz[j] - sz);
        }
        r2 = rx * rx + ry * ry + rz * rz;
    };
    // Sorted index of the lane's seed (none: ~0u); never a window candidate.
    uint32_t seedj = 0xFFFFFFFFu;

    // One window: up to one candidate per lane (keep), cut nearest first.
    auto run_window = [&](bool keep, T rx, T ry, T rz, T r2, uint32_t j, int32_t cid) -> int {
        unsigned km = __ballot_sync(FULL, keep);
        // Pre-test the window at once: each lane tests its own candidate's
        // bisector against every live vertex (read from the shared
        // mirror).  A bisector with no vertex Outside cuts nothing now and
        // nothing later (the cell only shrinks), so only possible cutters
        // (and guard-band cases, which the serial test reports) go on to
        // the serial nearest-first loop.  Same arithmetic as cut().
        if (BASE != kFormLean && __popc(km) >= kPretestMin) {
            bool maycut = false;
            if (keep && sizeof(T) == 8) {
                // FP64 form: the test in FP32 on the vertices' FP32 copies,
                // kept unless the FP32 distance is below minus four times
                // its error bound (inputs rounded: 2u |r_i v_i|; FMA chain
                // and offset: 3u (sum |r_i v_i| + off) + u off; |v_i| <= R)
                const float fx = (float)rx, fy = (float)ry, fz = (float)rz, f2 = (float)r2;
                const float Rf = sqrtf((float)R2) * 1.0001f;
                const float margin = 2.4e-7f * (5.f * (fabsf(fx) + fabsf(fy) + fabsf(fz)) * Rf + 2.f * f2);
                const float foff = 0.5f * f2;
                bool out = false;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    uint32_t m = C.lm[k];
                    while (m) {
                        const int sl = (k * 32 + __ffs(m) - 1) % S_t::VD;
                        m &= m - 1u;
                        const float sdf = fmaf(fx, S.fvx[sl], fmaf(fy, S.fvy[sl], fmaf(fz, S.fvz[sl], -foff)));
                        out |= !(sdf <= -margin);
                    }
                }
                maycut = out;
            } else if (keep) {
                T nx_, ny_, nz_, off_, rn_;
                bisector(rx, ry, rz, r2, nx_, ny_, nz_, off_, rn_);
                bool out = false, amb = false;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    uint32_t m = C.lm[k];
                    while (m) {
                        const int sl = k * 32 + __ffs(m) - 1;
                        m &= m - 1u;
                        const T sd = sdist(nx_, ny_, nz_, off_, S.vx[sl], S.vy[sl], S.vz[sl]);
                        // any vertex beyond the plane may be cut (the serial
                        // test applies the FP64 form's tolerance)
                        out |= sd > (T)0;
                        if constexpr (GUARD) amb |= fabs(sd) <= fma(rn_, S.ve[sl] + (T)P.guard_rel * rn_, eC);
                    }
                }
                maycut = out || amb;
            }
            km = __ballot_sync(FULL, keep && maycut);
        }
        // Nearest first: repeatedly take the closest remaining candidate
        // (warp minimum of its distance, ties by lane), so the closest
        // bisectors shrink the cell before the farther ones are tested.
        // The key keeps the top 27 bits of r2 (a positive float orders
        // like its bits) and the lane in the low 5.
        const unsigned mykey = (__float_as_uint((float)r2) & ~31u) | (unsigned)lane;
        while (km) {
            const unsigned best = __reduce_min_sync(FULL, ((km >> lane) & 1u) ? mykey : 0xFFFFFFFFu);
            const int src = (int)(best & 31u);
            km &= ~(1u << src);
            const T cx = __shfl_sync(FULL, rx, src);
            const T cy = __shfl_sync(FULL, ry, src);
            const T cz = __shfl_sync(FULL, rz, src);
            const T c2 = __shfl_sync(FULL, r2, src);
            const uint32_t cj = __shfl_sync(FULL, j, src);
            const int32_t cidb = __shfl_sync(FULL, cid, src);
            if constexpr (sizeof(T) == 8) {
                // FP64 form: on the FP32 key (r2 rounded to FP32, truncated)
                // against the FP32 bound (margin 1e-5); a candidate beyond
                // reach that passes only costs a test (the cut decides exactly)
                const float k2 = __uint_as_float(best & ~31u), l2 = 4.f * R2f * (float)kStopMargin;
                if (!(k2 < l2)) {
                    if (k2 > l2 * 1.001f) km = 0;
                    continue;
                }
            } else {
                const T lim2 = (T)4 * R2 * (T)kStopMargin;
                if (!(c2 < lim2)) {
                    // taken in increasing distance: the rest are farther still
                    if (c2 > lim2 * (T)1.001) km = 0;
                    continue;
                }
            }
            T nx, ny, nz, off, rn;
            bisector(cx, cy, cz, c2, nx, ny, nz, off, rn);
            const int r = cut<T, K, GUARD, BASE == kFormHybrid>(S, C, nx, ny, nz, off, rn, cR, eC, cidb, cj, lane,
                                                                   P, fsite);
            if constexpr (BASE != kFormLean) ++W.tested;
            if (r < 0) return -r;
            if (r > 0) {
                if constexpr (BASE != kFormLean) {
                    ++W.cuts;
                    W.newv += (unsigned)(r - 1);
                }
                const T R2b = R2;
                if constexpr (sizeof(T) == 8) {
                    R2f = live_r2f(S, C, lane);
                    R2 = (T)R2f;
                } else {
                    R2 = live_r2(S, C, lane);
                }
                if constexpr (GUARD) cR = (T)P.guard_rel * sqrt_up(R2);
                // hybrid form: a cut never moves a vertex beyond the cell
                // (convexity), so a radius that grew (or is no longer
                // finite) means an FP32 vertex went wrong after an
                // FP64-decided test; the cell re-runs in FP64
                if (BASE == kFormHybrid && !(R2 <= R2b * (T)1.001)) return ST_GUARD;
            }
        }
        return ST_OK;
    };

    // Cut by every point of the lanes' bins, given as sorted ranges
    // [beg, beg + cnt), in lane order; or (direct) by one window of the
    // lanes' seeds of a crowded bin (S.sd*).
    auto process = [&](unsigned beg, unsigned cnt, bool direct) -> int {
        unsigned total = 32, pref = 0;
        if (!direct) {
            const unsigned inc = warp_incl_scan_u(cnt, lane);
            total = __shfl_sync(FULL, inc, 31);
            pref = inc - cnt;
        }
        // FP64 forms: the windows' kept candidates are gathered in shared
        // memory and cut 32 at a time, as each window's pre-test costs the
        // same however few of its candidates are kept (clustered 4M in FP64:
        // 1,204 -> 1,070 ms).  In the FP32 forms the pre-test is cheap and
        // gathering did not pay (measured).
        constexpr bool kGather = BASE != kFormLean && sizeof(T) == 8;
        unsigned nbuf = 0;
        for (unsigned w0 = 0;; w0 += 32) {
            const bool more = w0 < total;
            if (!more && (!kGather || direct || nbuf == 0)) break;
            bool keep = false;
            T rx = 0, ry = 0, rz = 0, r2 = 0;
            uint32_t j = 0;
            int32_t cid = 0;
            bool near = false;
            if (!more) {
            } else if (kSeedForm && direct) {
                j = S.sdj[lane];
                keep = j != 0xFFFFFFFFu;
                rx = S.sdx[lane];
                ry = S.sdy[lane];
                rz = S.sdz[lane];
                r2 = S.sd2[lane];
                cid = S.sdcid[lane];
            } else {
                if constexpr (BASE != kFormLean) ++W.windows;
                const unsigned c = w0 + lane;
                const T lim = (T)4 * R2 * (T)kStopMargin;
                // the lane's bin: the last with prefix <= c (never an empty one)
                int lo = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(FULL, pref, lo + step) <= c) lo += step;
                const unsigned bbeg = __shfl_sync(FULL, beg, lo), bpref = __shfl_sync(FULL, pref, lo);
                if (c < total) {
                    j = tess_chk(bbeg + (c - bpref), P.npts, P.check, CK_POINT);
                    cand(j, rx, ry, rz, r2);
                    if constexpr (sizeof(T) == 8) keep = (j != self) && r2 > dup2 && (float)r2 < 4.f * R2f * (float)kStopMargin;
                    else keep = (j != self) && r2 > dup2 && r2 < lim;
                    if constexpr (GUARD) near = (j != self) && !(r2 > dup2);
                    if constexpr (kSeedForm) keep = keep && j != seedj;
                    cid = (int32_t)(P.sorted[j] - pt_base);
                    if (keep && tgroup >= 0) keep = (int64_t)(P.sgroup ? P.sgroup[j] : 0u) == tgroup;
                }
            }
            if (GUARD && __any_sync(FULL, near)) return ST_GUARD;
            if (kGather && !direct) {
                const unsigned km = __ballot_sync(FULL, keep);
                const unsigned nk = __popc(km);
                const unsigned pos = nbuf + __popc(km & ((1u << lane) - 1u));
                if (keep && pos < 32) {
                    S.cbx[pos] = rx;
                    S.cby[pos] = ry;
                    S.cbz[pos] = rz;
                    S.cb2[pos] = r2;
                    S.cbj[pos] = j;
                    S.cbid[pos] = cid;
                }
                if (more && nbuf + nk < 32) {
                    nbuf += nk;
                    continue;
                }
                // a full window (or the batch's last candidates) from the buffer
                __syncwarp();
                const unsigned cw = more ? 32u : nbuf;
                const bool kw = (unsigned)lane < cw;
                const T bx = S.cbx[lane], by = S.cby[lane], bz = S.cbz[lane], b2 = S.cb2[lane];
                const uint32_t bj = S.cbj[lane];
                const int32_t bid = S.cbid[lane];
                __syncwarp();
                // the candidates beyond the full window wait for the next one
                if (keep && pos >= 32) {
                    S.cbx[pos - 32] = rx;
                    S.cby[pos - 32] = ry;
                    S.cbz[pos - 32] = rz;
                    S.cb2[pos - 32] = r2;
                    S.cbj[pos - 32] = j;
                    S.cbid[pos - 32] = cid;
                }
                nbuf = more ? nbuf + nk - 32 : 0;
                keep = kw;
                rx = bx;
                ry = by;
                rz = bz;
                r2 = b2;
                j = bj;
                cid = bid;
            }
            const int st = run_window(keep, rx, ry, rz, r2, j, cid);
            if (st != ST_OK) return st;
            if (!more) break;
        }
        __syncwarp();
        return ST_OK;
    };

    // The site's fractional position inside its bin, for a tighter per-bin
    // test than the gap key: a point of bin (b + o) lies at least
    // |o| - 1 + f (o < 0) or o - f (o > 0) bin sides from the site on each
    // axis.  Off-grid sites (cells of external points) skip the test.
    float fx, fy, fz;
    if constexpr (kF32Setup) {
        // (x - glo) * inv from the FP32 pairs: within D.frac_eps bins
        fx = ((shx - D.glo_hi[0]) + (slx - D.glo_lo[0])) * D.inv_f[0] - (float)cbx;
        fy = ((shy - D.glo_hi[1]) + (sly - D.glo_lo[1])) * D.inv_f[1] - (float)cby;
        fz = ((shz - D.glo_hi[2]) + (slz - D.glo_lo[2])) * D.inv_f[2] - (float)cbz;
    } else {
        fx = (float)(__dmul_rn(sx - D.glo[0], D.inv[0]) - (double)cbx);
        fy = (float)(__dmul_rn(sy - D.glo[1], D.inv[1]) - (double)cby);
        fz = (float)(__dmul_rn(sz - D.glo[2], D.inv[2]) - (double)cbz);
    }
    const bool near_ok = fx >= -1e-3f && fx <= 1.001f && fy >= -1e-3f && fy <= 1.001f && fz >= -1e-3f &&
                         fz <= 1.001f && D.has_extent;
    const float bsx = D.size_f[0], bsy = D.size_f[1], bsz = D.size_f[2];
    const float feps = D.frac_eps;
    // squared distance (bin units scaled by the bin sides) from the site to
    // the nearest point of the bin at offset (i, j, k), each gap shortened by
    // the in-bin position's error bound
    auto near2 = [&](int i, int j, int k) -> float {
        const float fxc = fminf(fmaxf(fx, 0.f), 1.f), fyc = fminf(fmaxf(fy, 0.f), 1.f),
                    fzc = fminf(fmaxf(fz, 0.f), 1.f);
        const float dx = i > 0 ? fmaxf((float)i - fxc - feps, 0.f) : (i < 0 ? fmaxf((float)(-i - 1) + fxc - feps, 0.f) : 0.f);
        const float dy = j > 0 ? fmaxf((float)j - fyc - feps, 0.f) : (j < 0 ? fmaxf((float)(-j - 1) + fyc - feps, 0.f) : 0.f);
        const float dz = k > 0 ? fmaxf((float)k - fzc - feps, 0.f) : (k < 0 ? fmaxf((float)(-k - 1) + fzc - feps, 0.f) : 0.f);
        const float ax = dx * bsx, ay = dy * bsy, az = dz * bsz;
        return ax * ax + ay * ay + az * az;
    };
    auto bin_of = [&](int i, int j, int k) -> long long {
        const int x = cbx + i, y = cby + j, z = cbz + k;
        if (x < 0 || x >= cpd || y < 0 || y >= cpd || z < 0 || z >= cpd) return -1;
        // no point of this bin can cut: it lies beyond twice the cell radius
        if (near_ok && near2(i, j, k) * (1.0f - 1e-4f) >= (sizeof(T) == 8 ? 4.f * R2f : round_up_f((T)4 * R2)))
            return -1;
        return (long long)tess_chk(bin_base + ((uint64_t)x * cpd + y) * cpd + z, P.nbins, P.check, CK_BIN);
    };

    // Phases of the walk:
    //   0  crowded bins (seeded forms, when the site's own bin is crowded);
    //   1  the sorted shell table, 32 entries per batch (one per lane); the
    //      next batch's entries and bin ranges are loaded before the current
    //      batch is cut, so their latency overlaps the cutting;
    //   2  Chebyshev rings beyond the table (sparse regions).
    // The seeded forms run them as one loop with one call of process(), so
    // their window and cut code is inlined once: with a copy per phase,
    // instruction fetch limited them (and the single loop takes their
    // crowded-bin pass from 238 to 214 ms on the clustered 4M set).  The lean
    // first pass keeps a loop per phase: it has no phase 0, and the single
    // loop's dispatch made it 8% slower.
    uint32_t t = 0;
    // a batch entry: offsets, key and, after the bin test, the sorted range
    struct Ent {
        int i, j, k;
        float key;
        unsigned beg, cnt;
    };
    uint32_t done = 0;   // crowded bins already handled (see below)
    auto load_entry = [&](uint32_t idx, Ent& e) {
        e.i = e.j = e.k = 0;
        e.key = INFINITY;
        e.beg = e.cnt = 0;
        if (idx < tab_len) {
            const TabEntry te = tab[idx];
            e.i = te.i;
            e.j = te.j;
            e.k = te.k;
            e.key = te.key;
            if (has_radius && gap_key(D.size, e.i, e.j, e.k) > radius) e.key = INFINITY;
            long long lb = bin_of(e.i, e.j, e.k);
            if (kSeedForm && done && abs(e.i) <= 1 && abs(e.j) <= 1 && abs(e.k) <= 1 &&
                ((done >> ((e.i + 1) * 9 + (e.j + 1) * 3 + (e.k + 1))) & 1u))
                lb = -1;   // handled among the crowded bins
            if (lb >= 0) {
                e.beg = P.delims[lb];
                e.cnt = P.delims[lb + 1] - e.beg;
            }
        }
    };
    int ph = 1;
    if constexpr (!kSeedForm) {
        Ent ea;
        load_entry(lane, ea);
        // lean first pass: a crowded own bin (table entry 0, lane 0's first
        // entry) sends the cell to the seeded pass
        if (BASE == kFormLean && P.list_dense && __shfl_sync(FULL, ea.cnt, 0) >= P.seed_min) status = ST_DENSE;
        bool rings = false;
        while (status == ST_OK) {
            // The table key is rounded toward zero and the threshold up, so
            // stopping on key >= thr never drops a bin that could hold a cutter.
            const float thr = round_up_f((T)4 * R2 * (T)kStopMargin);
            const unsigned ma = __ballot_sync(FULL, !(ea.key < thr));
            const int na = ma ? __ffs(ma) - 1 : 32;
            const unsigned ba = ea.beg;
            unsigned ca = lane < na ? ea.cnt : 0u;
            // re-test the bins against the current (smaller) radius
            if (ca && near_ok && near2(ea.i, ea.j, ea.k) * (1.0f - 1e-4f) >= round_up_f((T)4 * R2)) ca = 0;
            t += (uint32_t)na;
            if (!ma) load_entry(t + lane, ea);
            if constexpr (BASE != kFormLean) ++W.batches;
            status = process(ba, ca, false);
            if (status != ST_OK) break;
            if (ma) {
                rings = (t >= tab_len) && isfinite(D.tab_kmax);
                break;
            }
        }
        if (status == ST_OK && rings) {
            for (int ring = 1; ring <= cpd - 1 && status == ST_OK; ++ring) {
                double lbk = (double)(ring - 1) * D.min_size;
                lbk = lbk * lbk;
                if (lbk < D.tab_kmax) lbk = D.tab_kmax;
                if (lbk >= 4.0 * (double)R2 * kStopMargin) break;
                if (radius >= 0.0 && lbk > radius) break;
                const uint32_t rs = 24u * (uint32_t)ring * (uint32_t)ring + 2u;
                for (uint32_t r0 = 0; r0 < rs; r0 += 32) {
                    const double thr = 4.0 * (double)R2 * kStopMargin;
                    long long lb = -1;
                    const uint32_t r = r0 + lane;
                    if (r < rs) {
                        int i, j, k;
                        ring_offset(ring, r, i, j, k);
                        const double key = gap_key(D.size, i, j, k);
                        if (key > D.tab_kmax && key < thr && !(radius >= 0.0 && key > radius)) lb = bin_of(i, j, k);
                    }
                    if (!__any_sync(FULL, lb >= 0)) continue;
                    if constexpr (BASE != kFormLean) ++W.batches;
                    unsigned beg = 0, cnt = 0;
                    if (lb >= 0) {
                        beg = P.delims[lb];
                        cnt = P.delims[lb + 1] - beg;
                    }
                    status = process(beg, cnt, false);
                    if (status != ST_OK) break;
                }
            }
        }
        ph = 3;
    }
    // ---- phase 0: crowded bins first ----
    // When the site's own bin is crowded, it and every crowded neighbour bin
    // still within reach are handled one at a time, nearest first, in two
    // steps each: the 32 seeds (the nearest point of each lane's stride of
    // the bin) are cut nearest first, then the bin's windows, each lane
    // skipping its own seed (window lane = position mod 32, the seed's
    // stride).  The shell walk skips the bins done here (27-bit mask `done`
    // over the offsets {-1,0,1}^3).
    // (their ranges and distances wait in shared memory: in registers they
    // would stay live through every later cut)
    bool seed_step = true;       // phase 0: the next step cuts a bin's seeds
    if constexpr (kSeedForm) {
        const uint64_t sb = tess_chk(bin_base + ((uint64_t)cbx * cpd + cby) * cpd + cbz, P.nbins, P.check, CK_BIN);
        if (P.delims[sb + 1] - P.delims[sb] >= P.seed_min) {
            const int ti = lane / 9 - 1, tj = (lane / 3) % 3 - 1, tk = lane % 3 - 1;
            unsigned nb = 0, nc = 0;
            float dn = INFINITY;
            if (lane < 27) {
                const long long lb = bin_of(ti, tj, tk);
                if (lb >= 0 && !(has_radius && gap_key(D.size, ti, tj, tk) > radius)) {
                    nb = P.delims[lb];
                    nc = P.delims[lb + 1] - nb;
                }
                dn = lane == 13 ? 0.f : (near_ok ? near2(ti, tj, tk) : INFINITY);
            }
            S.nbeg[lane] = nb;
            S.ncnt[lane] = nc;
            S.nd[lane] = dn;
            S.pending = __ballot_sync(FULL, nc >= P.seed_min && dn < INFINITY);
            ph = 0;
        }
    }
    Ent ea;
    bool loaded = false;                 // phase 1: the first batch is loaded
    S.ring = 1;
    S.r0 = 0;
    while (kSeedForm && status == ST_OK) {
        unsigned ba = 0, ca = 0;
        bool direct = false;
        if (kSeedForm && ph == 0) {
            if (seed_step) {
                const unsigned pending = S.pending;
                if (!pending) {
                    ph = 1;
                    continue;
                }
                const unsigned ndkey = (__float_as_uint(S.nd[lane]) & ~31u) | (unsigned)lane;
                const unsigned best = __reduce_min_sync(FULL, ((pending >> lane) & 1u) ? ndkey : 0xFFFFFFFFu);
                const int cbin = (int)(best & 31u);
                S.pending = pending & ~(1u << cbin);
                S.cbin = cbin;
                // still within reach of the (shrinking) cell?
                if (cbin != 13 && S.nd[cbin] * (1.0f - 1e-4f) >= (sizeof(T) == 8 ? 4.f * R2f : round_up_f((T)4 * R2)))
                    continue;
                const unsigned sbeg = S.nbeg[cbin], scnt = S.ncnt[cbin];
                T drx = 0, dry = 0, drz = 0, dr2 = (T)INFINITY;
                seedj = 0xFFFFFFFFu;
                for (unsigned q = lane; q < scnt; q += 32) {
                    const uint32_t j = tess_chk(sbeg + q, P.npts, P.check, CK_POINT);
                    T rx, ry, rz, r2;
                    cand(j, rx, ry, rz, r2);
                    bool keep = (j != self) && r2 > dup2 && r2 < dr2;
                    if (keep && tgroup >= 0) keep = (int64_t)(P.sgroup ? P.sgroup[j] : 0u) == tgroup;
                    if (keep) {
                        drx = rx;
                        dry = ry;
                        drz = rz;
                        dr2 = r2;
                        seedj = j;
                    }
                }
                S.sdx[lane] = drx;
                S.sdy[lane] = dry;
                S.sdz[lane] = drz;
                S.sd2[lane] = dr2;
                S.sdj[lane] = seedj;
                S.sdcid[lane] = seedj != 0xFFFFFFFFu ? (int32_t)(P.sorted[seedj] - pt_base) : 0;
                direct = true;
                seed_step = false;
            } else {
                // the bin as lane 0's range (window lane = position mod 32)
                ba = S.nbeg[S.cbin];
                ca = lane == 0 ? S.ncnt[S.cbin] : 0u;
                seed_step = true;
            }
        } else if (ph == 1) {
            if (!loaded) {
                load_entry(lane, ea);
                loaded = true;
                // lean first pass: a crowded own bin (table entry 0, lane 0's
                // first entry) sends the cell to the seeded pass
                if (BASE == kFormLean && P.list_dense && __shfl_sync(FULL, ea.cnt, 0) >= P.seed_min) {
                    status = ST_DENSE;
                    break;
                }
            }
            // The table key is rounded toward zero and the threshold up, so
            // stopping on key >= thr never drops a bin that could hold a cutter.
            const float thr = sizeof(T) == 8 ? 4.f * R2f * (float)kStopMargin : round_up_f((T)4 * R2 * (T)kStopMargin);
            const unsigned ma = __ballot_sync(FULL, !(ea.key < thr));
            const int na = ma ? __ffs(ma) - 1 : 32;
            ba = ea.beg;
            ca = lane < na ? ea.cnt : 0u;
            // re-test the bins against the current (smaller) radius
            if (ca && near_ok &&
                near2(ea.i, ea.j, ea.k) * (1.0f - 1e-4f) >= (sizeof(T) == 8 ? 4.f * R2f : round_up_f((T)4 * R2)))
                ca = 0;
            t += (uint32_t)na;
            if (ma) {
                ph = (t >= tab_len) && isfinite(D.tab_kmax) ? 2 : 3;
            } else {
                load_entry(t + lane, ea);
            }
            if constexpr (BASE != kFormLean) ++W.batches;
        } else if (ph == 2) {
            const int ring = S.ring;
            const uint32_t r0 = S.r0;
            if (r0 == 0) {
                // a new ring: stop when even its nearest bins are out of reach
                double lbk = (double)(ring - 1) * D.min_size;
                lbk = lbk * lbk;
                if (lbk < D.tab_kmax) lbk = D.tab_kmax;
                if (ring > cpd - 1 || lbk >= 4.0 * (double)R2 * kStopMargin || (radius >= 0.0 && lbk > radius)) {
                    ph = 3;
                    continue;
                }
            }
            const uint32_t rs = 24u * (uint32_t)ring * (uint32_t)ring + 2u;
            const double thr = 4.0 * (double)R2 * kStopMargin;
            long long lb = -1;
            const uint32_t r = r0 + lane;
            if (r < rs) {
                int i, j, k;
                ring_offset(ring, r, i, j, k);
                const double key = gap_key(D.size, i, j, k);
                if (key > D.tab_kmax && key < thr && !(radius >= 0.0 && key > radius)) lb = bin_of(i, j, k);
            }
            S.r0 = r0 + 32 < rs ? r0 + 32 : 0u;
            S.ring = r0 + 32 < rs ? ring : ring + 1;
            if (!__any_sync(FULL, lb >= 0)) continue;
            if constexpr (BASE != kFormLean) ++W.batches;
            if (lb >= 0) {
                ba = P.delims[lb];
                ca = P.delims[lb + 1] - ba;
            }
        } else {
            break;
        }
        status = process(ba, ca, direct);
        if (kSeedForm && ph == 0 && seed_step) {
            // a crowded bin's windows are done
            seedj = 0xFFFFFFFFu;
            done |= 1u << S.cbin;
        }
    }

    // ---- finalize: faces, areas, volume in FP64 (polyhedron.rs:776-855) ----
    int nlive = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) nlive += __popc(C.lm[k]);
    double vol = 0.0;
    int F = 0;
    constexpr int R = (S_t::P + 31) / 32;
    double farea[R];
    int fdegr[R];
    if (status == ST_OK) {
        for (int i = lane; i < C.np; i += 32) S.fdeg[i] = 0;
        __syncwarp();
        bool fbad = false;
        bool vbad = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if ((C.lm[k] >> lane) & 1u) {
                const int s = k * 32 + lane;
                const uint32_t tt = S.tri[s];
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const int p = plane_of(tt, e);
                    if (p < C.np) {
                        atomicAdd(&S.fdeg[p], 1u);
                        S.fsta[p] = (uint8_t)s;
                    } else {
                        fbad = true;
                    }
                }
            }
        }
        __syncwarp();
        bool bad = fbad;
        double vpart = 0.0;
        if constexpr (GUARD && !EXACT) {
            // Face planes as FP32 pairs, without the FP64 pipe: the bisector of
            // the site and point q has n = q = p_j - site and h = q.q / 2
            // (vector3.rs:223-239 up to the scale of n).  q comes from the
            // points' FP32 pairs (hi + lo relative to the centre, 48 bits) by a
            // TwoSum of the high parts, so its error is ~2^-46 of the
            // distance from the centre; h = q.q / 2 follows in double-float.
            // Walls: n = +-e_a, h = the distance to the wall (FP64; only cells
            // that touch a wall have such faces).
            const double* blo = P.box_override ? P.box : D.blo;
            const double* bhi = P.box_override ? P.box + 3 : D.bhi;
            for (int p = lane; p < C.np; p += 32) {
                if (S.fdeg[p] == 0) continue;
                float q0, q1, q2, l0 = 0.f, l1 = 0.f, l2 = 0.f, hh, hl, dist;
                if (p < 6) {
                    const int a = p >> 1;
                    const bool mx = p & 1;
                    const double s_a = a == 0 ? sx : (a == 1 ? sy : sz);
                    const double h = mx ? (bhi[a] - s_a) : (s_a - blo[a]);
                    hh = (float)h;
                    hl = (float)(h - (double)hh);
                    q0 = a == 0 ? (mx ? 1.f : -1.f) : 0.f;
                    q1 = a == 1 ? (mx ? 1.f : -1.f) : 0.f;
                    q2 = a == 2 ? (mx ? 1.f : -1.f) : 0.f;
                    dist = hh;
                } else {
                    const uint32_t j = tess_chk(S.psrc[p], P.npts, P.check, CK_POINT);
                    float sh, se;
                    two_sum(P.shi[3ull * j], -shx, sh, se);
                    two_sum(sh, (P.slo[3ull * j] - slx) + se, q0, l0);
                    two_sum(P.shi[3ull * j + 1], -shy, sh, se);
                    two_sum(sh, (P.slo[3ull * j + 1] - sly) + se, q1, l1);
                    two_sum(P.shi[3ull * j + 2], -shz, sh, se);
                    two_sum(sh, (P.slo[3ull * j + 2] - slz) + se, q2, l2);
                    float p0, e0, p1, e1, p2, e2, s01, t01, s2, t2;
                    two_prod(q0, q0, p0, e0);
                    two_prod(q1, q1, p1, e1);
                    two_prod(q2, q2, p2, e2);
                    two_sum(p0, p1, s01, t01);
                    two_sum(s01, p2, s2, t2);
                    const float low = ((e0 + e1) + e2) + (t01 + t2) + 2.f * (q0 * l0 + q1 * l1 + q2 * l2);
                    float H, HL;
                    two_sum(s2, low, H, HL);
                    hh = 0.5f * H;   // exact scalings
                    hl = 0.5f * HL;
                    dist = 0.5f * sqrtf(H);
                }
                S.fqx[p] = q0;
                S.fqy[p] = q1;
                S.fqz[p] = q2;
                S.qlx[p] = l0;
                S.qly[p] = l1;
                S.qlz[p] = l2;
                S.qhh[p] = hh;
                S.qhl[p] = hl;
                S.qdist[p] = dist;
            }
        } else if constexpr (GUARD) {
            // FP64 face planes: bisector of the site and point q, n = q,
            // h = q.q / 2 (vector3.rs:223-239 up to the scale of n); walls
            // n = +-e_a, h = distance to the wall.
            const double* blo = P.box_override ? P.box : D.blo;
            const double* bhi = P.box_override ? P.box + 3 : D.bhi;
            for (int p = lane; p < C.np; p += 32) {
                if (S.fdeg[p] == 0) continue;
                double qx, qy, qz, qh;
                float dist;
                if (p < 6) {
                    const int a = p >> 1;
                    const bool mx = p & 1;
                    const double s_a = a == 0 ? sx : (a == 1 ? sy : sz);
                    qh = mx ? (bhi[a] - s_a) : (s_a - blo[a]);
                    qx = a == 0 ? (mx ? 1.0 : -1.0) : 0.0;
                    qy = a == 1 ? (mx ? 1.0 : -1.0) : 0.0;
                    qz = a == 2 ? (mx ? 1.0 : -1.0) : 0.0;
                    dist = (float)qh;
                } else {
                    const uint32_t j = tess_chk(S.psrc[p], P.npts, P.check, CK_POINT);
                    qx = P.spx[j] - sx;
                    qy = P.spy[j] - sy;
                    qz = P.spz[j] - sz;
                    const double q2 = qx * qx + qy * qy + qz * qz;
                    qh = 0.5 * q2;
                    dist = 0.5f * sqrtf((float)q2);
                }
                S.qx[p] = qx;
                S.qy[p] = qy;
                S.qz[p] = qz;
                S.qh[p] = qh;
                S.fqx[p] = (float)qx;
                S.fqy[p] = (float)qy;
                S.fqz[p] = (float)qz;
                S.qdist[p] = dist;
            }
        }
        if constexpr (GUARD) {
            __syncwarp();
            // One Newton step per vertex: residuals of its three planes in
            // double-float (FP32 form) or FP64 (FP64-accurate finish),
            // correction solved in FP32 (Cramer).  A correction larger than
            // verify_rel * R means the FP32 vertex was not trustworthy: the
            // cell re-runs in FP64.
            // The residual h - n.x of a plane kept as FP32 pairs: the high
            // parts' products exact (FMA), summed by TwoSum, the low-order
            // terms in FP32; accurate to ~2^-46 |n| |x|, far below the
            // residual of an FP32 vertex (~1e-7 |n| |x|).
            auto resid = [&](int pl, float x, float y, float z) -> float {
                float p0, e0, p1, e1, p2, e2, s1, t1, s2, t2, s3, t3;
                two_prod(S.fqx[pl], x, p0, e0);
                two_prod(S.fqy[pl], y, p1, e1);
                two_prod(S.fqz[pl], z, p2, e2);
                two_sum(S.qhh[pl], -p0, s1, t1);
                two_sum(s1, -p1, s2, t2);
                two_sum(s2, -p2, s3, t3);
                const float low = ((S.qhl[pl] - e0) - e1) - e2 + ((t1 + t2) + t3) -
                                  (S.qlx[pl] * x + S.qly[pl] * y + S.qlz[pl] * z);
                return s3 + low;
            };
            const float vlim = P.verify_rel * sqrtf((float)R2);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if ((C.lm[k] >> lane) & 1u) {
                    const int s = k * 32 + lane;
                    const uint32_t tt = S.tri[s];
                    const int a = plane_of(tt, 0), b = plane_of(tt, 1), c = plane_of(tt, 2);
                    const double x = (double)C.vx[k], y = (double)C.vy[k], z = (double)C.vz[k];
                    float ra, rb, rc;
                    if constexpr (EXACT) {
                        ra = (float)(S.qh[a] - (S.qx[a] * x + S.qy[a] * y + S.qz[a] * z));
                        rb = (float)(S.qh[b] - (S.qx[b] * x + S.qy[b] * y + S.qz[b] * z));
                        rc = (float)(S.qh[c] - (S.qx[c] * x + S.qy[c] * y + S.qz[c] * z));
                    } else {
                        ra = resid(a, C.vx[k], C.vy[k], C.vz[k]);
                        rb = resid(b, C.vx[k], C.vy[k], C.vz[k]);
                        rc = resid(c, C.vx[k], C.vy[k], C.vz[k]);
                    }
                    const float ax_ = S.fqx[a], ay_ = S.fqy[a], az_ = S.fqz[a];
                    const float bx_ = S.fqx[b], by_ = S.fqy[b], bz_ = S.fqz[b];
                    const float cx_ = S.fqx[c], cy_ = S.fqy[c], cz_ = S.fqz[c];
                    const float bcx = by_ * cz_ - bz_ * cy_, bcy = bz_ * cx_ - bx_ * cz_, bcz = bx_ * cy_ - by_ * cx_;
                    const float cax = cy_ * az_ - cz_ * ay_, cay = cz_ * ax_ - cx_ * az_, caz = cx_ * ay_ - cy_ * ax_;
                    const float abx = ay_ * bz_ - az_ * by_, aby = az_ * bx_ - ax_ * bz_, abz = ax_ * by_ - ay_ * bx_;
                    const float det = ax_ * bcx + ay_ * bcy + az_ * bcz;
                    const float inv = recip(det);
                    const float ddx = (ra * bcx + rb * cax + rc * abx) * inv;
                    const float ddy = (ra * bcy + rb * cay + rc * aby) * inv;
                    const float ddz = (ra * bcz + rb * caz + rc * abz) * inv;
                    // the correction must stay within the vertex's error bound
                    const float lim = 2.0f * C.ve[k] + vlim;
                    if (!(fabsf(ddx) <= lim && fabsf(ddy) <= lim && fabsf(ddz) <= lim)) vbad = true;
                    S.dx[s] = ddx;
                    S.dy[s] = ddy;
                    S.dz[s] = ddz;
                    if constexpr (EXACT) {
                        // a second step from x + d (exact in FP64): its residuals
                        // are ~1e-7 of the first, so the FP32 solve leaves an error
                        // at the FP64 rounding of the residuals
                        const double x1 = x + (double)ddx, y1 = y + (double)ddy, z1 = z + (double)ddz;
                        const float sa_ = (float)(S.qh[a] - (S.qx[a] * x1 + S.qy[a] * y1 + S.qz[a] * z1));
                        const float sb_ = (float)(S.qh[b] - (S.qx[b] * x1 + S.qy[b] * y1 + S.qz[b] * z1));
                        const float sc_ = (float)(S.qh[c] - (S.qx[c] * x1 + S.qy[c] * y1 + S.qz[c] * z1));
                        S.rx[s] = x1 + (double)((sa_ * bcx + sb_ * cax + sc_ * abx) * inv);
                        S.ry[s] = y1 + (double)((sa_ * bcy + sb_ * cay + sc_ * aby) * inv);
                        S.rz[s] = z1 + (double)((sa_ * bcz + sb_ * caz + sc_ * abz) * inv);
                    }
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int p = r * 32 + lane;
            farea[r] = 0.0;
            fdegr[r] = 0;
            if (p < C.np && S.fdeg[p] > 0) {
                const int start = tess_chk((int)S.fsta[p], S_t::V, P.check, CK_SLOT);
                int cur = start, steps = 0;
                if constexpr (EXACT) {
                    // The face's area from its projection on the plane normal
                    // to the dominant axis m of its normal q (shoelace on the
                    // refined FP64 positions, face-relative): w_m = 2 A q_m/|q|
                    // (walk clockwise seen from outside: next x current is
                    // outward).  Area = w_m |q| / (2 q_m); the pyramid from the
                    // site, h A / 3 with h = qh / |q|, is qh w_m / (6 q_m)
                    // (compute_volume, polyhedron.rs:838-855).
                    const double q0 = S.qx[p], q1 = S.qy[p], q2 = S.qz[p];
                    const int m = (fabs(q0) >= fabs(q1) && fabs(q0) >= fabs(q2)) ? 0 : (fabs(q1) >= fabs(q2) ? 1 : 2);
                    const double* X1 = m == 0 ? S.ry : (m == 1 ? S.rz : S.rx);
                    const double* X2 = m == 0 ? S.rz : (m == 1 ? S.rx : S.ry);
                    const double qm = m == 0 ? q0 : (m == 1 ? q1 : q2);
                    const double a1 = X1[start], a2 = X2[start];
                    double u1 = 0.0, u2 = 0.0, wm = 0.0;
                    do {
                        const uint32_t tt = S.tri[cur], aa = S.adj[cur];
                        const int i = plane_of(tt, 0) == p ? 0 : (plane_of(tt, 1) == p ? 1 : 2);
                        const int nx = plane_of(aa, i);
                        if (plane_of(tt, i) != p || nx >= S_t::V) {
                            bad = true;
                            break;
                        }
                        const double v1 = X1[nx] - a1, v2 = X2[nx] - a2;
                        if (steps > 0) wm += v1 * u2 - v2 * u1;
                        u1 = v1;
                        u2 = v2;
                        cur = nx;
                        ++steps;
                    } while (cur != start && steps <= S_t::V);
                    const double inv_qm = 1.0 / qm;
                    farea[r] = 0.5 * wm * inv_qm * sqrt(q0 * q0 + q1 * q1 + q2 * q2);
                    vpart += S.qh[p] * wm * inv_qm * 0.5;
                } else if constexpr (GUARD) {
                    // Fan from the first vertex (weighted_normal,
                    // polyhedron.rs:776-808) on refined positions:
                    // (x - anchor) = (x32 - a32) + (dx - da), in FP32.
                    const float a0 = (float)S.vx[start], a1 = (float)S.vy[start], a2 = (float)S.vz[start];
                    const float e0 = S.dx[start], e1 = S.dy[start], e2 = S.dz[start];
                    float ux = 0.f, uy = 0.f, uz = 0.f, wx = 0.f, wy = 0.f, wz = 0.f;
                    do {
                        const uint32_t tt = S.tri[cur], aa = S.adj[cur];
                        const int i = plane_of(tt, 0) == p ? 0 : (plane_of(tt, 1) == p ? 1 : 2);
                        const int nx = plane_of(aa, i);
                        if (plane_of(tt, i) != p || nx >= S_t::V) {
                            bad = true;
                            break;
                        }
                        const float vx_ = ((float)S.vx[nx] - a0) + (S.dx[nx] - e0);
                        const float vy_ = ((float)S.vy[nx] - a1) + (S.dy[nx] - e1);
                        const float vz_ = ((float)S.vz[nx] - a2) + (S.dz[nx] - e2);
                        if (steps > 0) {
                            wx += uy * vz_ - uz * vy_;
                            wy += uz * vx_ - ux * vz_;
                            wz += ux * vy_ - uy * vx_;
                        }
                        ux = vx_;
                        uy = vy_;
                        uz = vz_;
                        cur = nx;
                        ++steps;
                    } while (cur != start && steps <= S_t::V);
                    const float area = 0.5f * sqrtf(wx * wx + wy * wy + wz * wz);
                    farea[r] = (double)area;
                    vpart += (double)(area * S.qdist[p]);
                } else {
                    double ax = 0.0, ay = 0.0, az = 0.0;
                    do {
                        const uint32_t tt = S.tri[cur], aa = S.adj[cur];
                        const int i = plane_of(tt, 0) == p ? 0 : (plane_of(tt, 1) == p ? 1 : 2);
                        const int nx = plane_of(aa, i);
                        if (plane_of(tt, i) != p || nx >= S_t::V) {
                            bad = true;
                            break;
                        }
                        const double X0 = (double)S.vx[cur], X1 = (double)S.vy[cur], X2 = (double)S.vz[cur];
                        const double Y0 = (double)S.vx[nx], Y1 = (double)S.vy[nx], Y2 = (double)S.vz[nx];
                        // the walk runs clockwise seen from outside: Y x X is outward
                        ax += Y1 * X2 - Y2 * X1;
                        ay += Y2 * X0 - Y0 * X2;
                        az += Y0 * X1 - Y1 * X0;
                        cur = nx;
                        ++steps;
                    } while (cur != start && steps <= S_t::V);
                    const double A0 = (double)S.vx[start], A1 = (double)S.vy[start], A2 = (double)S.vz[start];
                    vpart += (ax * A0 + ay * A1 + az * A2) * 0.5;
                    farea[r] = 0.5 * sqrt(ax * ax + ay * ay + az * az);
                }
                bad |= (cur != start) || (steps != (int)S.fdeg[p]) || steps < 3;
                fdegr[r] = steps;
            }
        }
        // volume: sum of pyramids from the site, area * height / 3
        // (compute_volume, polyhedron.rs:838-855)
        vol = (GUARD && !EXACT) ? warp_sum_d(vpart) * (1.0 / 3.0) : warp_sum_d(vpart) / 3.0;
#pragma unroll
        for (int r = 0; r < R; ++r) F += __popc(__ballot_sync(FULL, fdegr[r] > 0));
        // Every vertex has three faces: V - E + F = 2 with E = 3V/2.
        if (nlive > 0 && F != nlive / 2 + 2) bad = true;
        if (__any_sync(FULL, bad)) status = ST_DEGEN;
        else if (GUARD && __any_sync(FULL, vbad)) status = ST_VERIFY;
    }

    // ---- outputs ----
    if (status != ST_OK) {
        if (GEO) {
            if (lane == 0) P.geo->status = status;
            return;
        }
        if (lane == 0) {
            uint32_t* list = nullptr;
            unsigned* count = nullptr;
            if (P.reasons) atomicAdd(&P.reasons[status & 7], 1u);
            if (status == ST_GUARD || status == ST_DEGEN || status == ST_VERIFY) {
                list = P.list_fp64;
                count = P.list_fp64_count;
            } else if (status == ST_VCAP || status == ST_PCAP) {
                list = P.list_cap;
                count = P.list_cap_count;
            } else if (status == ST_DENSE) {
                list = P.list_dense;
                count = P.list_dense_count;
            }
            if (list) {
                list[tess_chk(atomicAdd(count, 1u), P.npts, P.check, CK_LIST)] = gs;
                P.status[orig] = ST_PENDING;
            } else {
                P.status[orig] = (uint8_t)status;
                P.vol[orig] = 0.0;
                P.nface[orig] = 0;
                atomicAdd(P.fail_count, 1u);
            }
        }
        return;
    }
    // compact live face ids, rank faces by id (faces are reported sorted)
    {
        int base = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int p = r * 32 + lane;
            const unsigned m = __ballot_sync(FULL, fdegr[r] > 0);
            if (fdegr[r] > 0) S.flist[base + __popc(m & ((1u << lane) - 1u))] = S.pid[p];
            base += __popc(m);
        }
        __syncwarp();
    }
    int rank[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        rank[r] = 0;
        if (fdegr[r] > 0) {
            const int32_t my = S.pid[r * 32 + lane];
            for (int q = 0; q < F; ++q) rank[r] += S.flist[q] < my;
        }
    }
    if (GEO) {
        GeoOut* G = P.geo;
        // vertices: live slots renumbered in slot order
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if ((C.lm[k] >> lane) & 1u) {
                int vi = __popc(C.lm[k] & ((1u << lane) - 1u));
#pragma unroll
                for (int kk = 0; kk < K; ++kk)
                    if (kk < k) vi += __popc(C.lm[kk]);
                const int s = k * 32 + lane;
                G->verts[3 * vi] = (double)S.vx[s] + (GUARD ? (double)S.dx[s % S_t::VF] : 0.0);
                G->verts[3 * vi + 1] = (double)S.vy[s] + (GUARD ? (double)S.dy[s % S_t::VF] : 0.0);
                G->verts[3 * vi + 2] = (double)S.vz[s] + (GUARD ? (double)S.dz[s % S_t::VF] : 0.0);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (fdegr[r] > 0) {
                S.rank2p[rank[r]] = (uint8_t)(r * 32 + lane);
                G->face_nbr[rank[r]] = S.pid[r * 32 + lane];
                G->face_area[rank[r]] = farea[r];
            }
        }
        __syncwarp();
        if (lane == 0) {
            int off = 0;
            for (int q = 0; q < F; ++q) {
                const int p = S.rank2p[q];
                G->face_off[q] = off;
                const int deg = (int)S.fdeg[p];
                const int start = tess_chk((int)S.fsta[p], S_t::V, P.check, CK_SLOT);
                int cur = start;
                // reversed walk: counter-clockwise seen from outside
                for (int st = 0; st < deg; ++st) {
                    int vi = 0;
                    for (int k = 0; k < K; ++k) {
                        if ((cur >> 5) == k) vi += __popc(C.lm[k] & ((1u << (cur & 31)) - 1u));
                        else if ((cur >> 5) > k) vi += __popc(C.lm[k]);
                    }
                    G->face_vtx[tess_chk(off + (deg - st) % deg, 3 * 256, P.check, CK_FACE)] = vi;
                    const uint32_t tt = S.tri[cur], aa = S.adj[cur];
                    const int i = plane_of(tt, 0) == p ? 0 : (plane_of(tt, 1) == p ? 1 : 2);
                    cur = plane_of(aa, i) % S_t::V;
                }
                off += deg;
            }
            G->face_off[F] = off;
            G->nv = nlive;
            G->nf = F;
            G->volume = vol;
            G->status = ST_OK;
        }
        return;
    }
    unsigned long long fbase = 0;
    if (lane == 0) fbase = atomicAdd(P.face_cursor, (unsigned long long)F);
    fbase = __shfl_sync(FULL, fbase, 0);
    if (fbase + F > P.face_cap) {
        if (lane == 0) {
            P.status[orig] = ST_POOL;
            P.nface[orig] = 0;
        }
        return;   // the host sees the face cursor past the capacity and recomputes
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (fdegr[r] > 0) {
            const unsigned long long fi = tess_chk(fbase + rank[r], P.face_cap, P.check, CK_FACE);
            P.face_nbr[fi] = S.pid[r * 32 + lane];
            P.face_area[fi] = farea[r];
        }
    }
    if (lane == 0) {
        P.vol[orig] = vol;
        P.nface[orig] = (uint32_t)F;
        P.fstart[orig] = fbase;
        P.status[orig] = ST_OK;
    }
}

// K = 2: 8 warps per block, two blocks per SM (registers capped at 128).
template <typename T, int K, bool GEO, int FORM>
__global__ void __launch_bounds__(K == 2 ? 256 : 128, K == 2 ? 2 : 1) k_clip(ClipParams P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    Smem<T, K>& S = reinterpret_cast<Smem<T, K>*>(smraw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    if (P.grid_err && *P.grid_err == 1) return;   // non-finite input: nothing to clip
    Work W;
    for (;;) {
        unsigned w = 0;
        if (lane == 0) w = atomicAdd(P.cursor, 1u);
        w = __shfl_sync(FULL, w, 0);
        const unsigned total = P.work_count ? *P.work_count : P.total;
        if (w >= total) break;
        const uint32_t gs = P.work ? P.work[w] : w;
        run_cell<T, K, GEO, FORM>(P, S, gs, lane, W);
    }
    if (P.work_ctr && lane == 0) {
        atomicAdd(&P.work_ctr[0], (unsigned long long)W.tested);
        atomicAdd(&P.work_ctr[1], (unsigned long long)W.cuts);
        atomicAdd(&P.work_ctr[2], (unsigned long long)W.newv);
        atomicAdd(&P.work_ctr[3], (unsigned long long)W.windows);
        atomicAdd(&P.work_ctr[4], (unsigned long long)W.batches);
    }
}

// Raise the kernel's dynamic shared memory limit to what `bytes` needs, once
// per size and device: cudaFuncSetAttribute applies to the current device
// only, so the limit is remembered per device ordinal.  A mutex keeps two
// host threads from lowering each other's limit.  Kept out of stream capture
// by the host's warm-up calls.
constexpr int kMaxDevices = 64;
template <typename T, int K, bool GEO, int FORM>
cudaError_t configure_smem(size_t bytes) {
    static std::mutex mu;
    static size_t configured[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t* slot = (dev >= 0 && dev < kMaxDevices) ? &configured[dev] : nullptr;
    if (slot && bytes <= *slot) return cudaSuccess;
    e = cudaFuncSetAttribute(k_clip<T, K, GEO, FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && slot) *slot = bytes;
    return e;
}

template <typename T, int K, bool GEO, int FORM>
cudaError_t launch_t(const ClipParams& p, int wpb, int blocks, cudaStream_t s) {
    const size_t sm = sizeof(Smem<T, K>) * (size_t)wpb;
    cudaError_t e = configure_smem<T, K, GEO, FORM>(sm);
    if (e != cudaSuccess) return e;
    k_clip<T, K, GEO, FORM><<<blocks, 32 * wpb, sm, s>>>(p);
    return cudaGetLastError();
}

template <typename T, int K, bool GEO, int FORM>
int blocks_t(int wpb, int device) {
    const size_t sm = sizeof(Smem<T, K>) * (size_t)wpb;
    int per = 0, nsm = 0;
    if (configure_smem<T, K, GEO, FORM>(sm) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_clip<T, K, GEO, FORM>, 32 * wpb, sm) != cudaSuccess)
        per = 1;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaGetLastError();   // leave no sticky error behind a failed query
    if (per < 1) per = 1;
    return per * (nsm > 0 ? nsm : 1);
}

}  // namespace clipk
}  // namespace tess
