// tess_internal.cuh -- device data layout shared by the binning pass, the
// clipping kernels and the host driver of libtessgpu.so (sm_103a).
//
// HBM layout of one set of diagrams (a single Diagram is a set of one):
//   points   xyz[3 * total]            FP64 AoS, concatenated diagram by diagram
//   bins     bin[total], rank[total]    global bin id and arrival rank per point
//   grid     delims[total_bins + 1]     CSR offsets of the bin-sorted order
//   sorted   sorted[total]              sorted position -> point (concatenated index)
//            spx/spy/spz[total]         FP64 positions in sorted order (SoA)
//            sgroup[total]              group ids in sorted order (optional)
//   table    tab[...]                   per-diagram shell table (sorted offsets)
//   results  vol[total], nface[total], fstart[total], status[total]  (point order)
//            face_nbr[cap], face_area[cap]   face pool, filled by atomic allocation
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace tess {

constexpr double kTolerance = 1e-12;        // polyhedron.rs:221-223
constexpr double kStopMargin = 1.0 + 1e-5;  // slack on the security-radius test
constexpr int kMaxTable = 4096;             // shell-table entries per diagram (sort capacity)

// Per-cell status codes written by the clipping kernels.
enum CellStatus : uint8_t {
    ST_OK = 0,
    ST_GUARD = 1,       // FP32 plane-side test inside the guard band -> FP64 re-run
    ST_VCAP = 2,        // vertex capacity exceeded -> larger capacity re-run
    ST_PCAP = 3,        // face (plane) capacity exceeded -> larger capacity re-run
    ST_DEGEN = 4,       // inconsistent topology (degenerate input) -> FP64 re-run / error
    ST_POOL = 5,        // face pool full -> host grows the pool
    ST_VERIFY = 6,      // FP32 vertex failed the FP64 check -> FP64 re-run
    ST_DENSE = 7,       // crowded own bin (lean first pass) -> seeded re-run
    ST_PENDING = 255    // not computed yet
};

// The checked build (compiled with TESS_CHECKED=1, libtessgpu_checked.so): the
// binning and clipping kernels test every data-dependent index into a device
// array before use.  An index outside [0, n) sets bit `site` of the handle's
// check word and is replaced by 0, so the access stays in bounds; the host
// then fails the call with TESS_E_CHECK.  The regular build compiles no test.
#ifndef TESS_CHECKED
#define TESS_CHECKED 0
#endif
enum CheckSite : int {
    CK_POINT = 0,   // a point (sorted or original index)
    CK_BIN = 1,     // a bin of the grid
    CK_SLOT = 2,    // a vertex slot or free-slot stack entry of a cell
    CK_PLANE = 3,   // a plane of a cell
    CK_LIST = 4,    // an entry of a re-run list
    CK_FACE = 5,    // a face of the face pool
    CK_GRID = 6     // a position of the binning pass's sort
};
template <typename I, typename N>
__device__ __forceinline__ I tess_chk(I i, N n, int* check, int site) {
#if TESS_CHECKED
    if (!((unsigned long long)(long long)i < (unsigned long long)n)) {
        if (check) atomicOr(check, 1 << site);
        return (I)0;
    }
#else
    (void)n;
    (void)check;
    (void)site;
#endif
    return i;
}

// One diagram as the kernels see it.  Filled partly by the host (counts,
// bases, box) and partly on the device (bounds, bin sizes, table length).
struct DiagDesc {
    double glo[3], ghi[3];   // CeleryBounds (celery.rs:81-125), tight point bounds
    double ctr[3];           // centre of those bounds: the FP32 hi/lo positions are split relative to it
    double size[3];          // x/y/z_cell_size (celery.rs:165-167)
    double inv[3];           // x/y/z_inverse_cell_size (celery.rs:169-171)
    double blo[3], bhi[3];   // container box (walls)
    double tab_kmax;         // every offset with key <= tab_kmax is in the table
    double min_size;         // smallest nonzero bin side
    uint64_t bin_base;       // first global bin of this diagram
    uint64_t tab_base;       // first table entry of this diagram
    uint32_t pt_base;        // first point (concatenated order == sorted order base)
    uint32_t n;              // points
    uint32_t tab_len;        // table entries (device-written)
    uint32_t tab_cap;        // table capacity reserved by the host
    int32_t cpd;             // cells_per_dimension (host, glibc cbrt)
    int32_t cheb;            // Chebyshev radius enumerated into the table
    // FP32 forms of the grid and the box for the FP32 clipping pass (device-
    // written with the grid): offsets from ctr as FP32 pairs (hi + lo), so the
    // site's place in its bin and the box corners come out of FP32 arithmetic
    float glo_hi[3], glo_lo[3];          // point bounds' low corner - ctr
    float blo_hi[3], blo_lo[3];          // container box low corner - ctr
    float bhi_hi[3], bhi_lo[3];          // container box high corner - ctr
    float inv_f[3];                      // inverse bin sides
    float glo_f[3];                      // point bounds' low corner, rounded to FP32
    float size_f[3];                     // bin sides
    float rcp_cpd, rcp_cpd2;             // 1 / cpd, 1 / cpd^2 (bin id -> coordinates)
    float frac_eps;                      // bound on the FP32 in-bin position's error, in bins
    int32_t has_extent;                  // some bin side is nonzero (min_size > 0)
};

// Shell-table entry: a bin offset and its search-order key (celery.rs:423-427)
// rounded toward zero to FP32 so the stop test stays conservative.
struct TabEntry {
    float key;
    int8_t i, j, k, pad;
};

// Output of one cell's full geometry (single-cell queries); the leading
// fields mirror tess_cell_geometry of the C ABI.
struct GeoOut {
    double volume;
    int32_t nv, nf;
    double verts[3 * 256];          // site-relative vertex positions
    int32_t face_nbr[256];
    double face_area[256];
    int32_t face_off[257];          // offsets into face_vtx
    int32_t face_vtx[3 * 256];      // vertex indices, CCW seen from outside
    int32_t status;
};

// Order-preserving map of doubles onto uint64 (for atomicMin/atomicMax).
__device__ __forceinline__ unsigned long long ord_enc(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_dec(unsigned long long e) {
    unsigned long long b = (e >> 63) ? (e & 0x7FFFFFFFFFFFFFFFull) : ~e;
    return __longlong_as_double((long long)b);
}

// get_{x,y,z}_cell_index (celery.rs:269-314): x >= max -> cpd-1, else
// min(trunc((x - min) * inv), cpd-1), with `as usize` saturating at 0 for
// negative and NaN values.  Exact FP64 multiply, no FMA.
__device__ __forceinline__ int axis_index(double x, double lo, double hi, double inv, int cpd) {
    if (x >= hi) return cpd - 1;
    double v = __dmul_rn(__dsub_rn(x, lo), inv);
    if (!(v > 0.0)) return 0;
    if (v >= (double)(cpd - 1)) return cpd - 1;
    return (int)v;
}

// Search-order key of a bin offset (celery.rs:423-427 on the gap counts,
// celery.rs:447-639), self = -1 (celery.rs:438-443).  Exact FP64, no FMA.
__device__ __forceinline__ double gap_key(const double size[3], int i, int j, int k) {
    if (i == 0 && j == 0 && k == 0) return -1.0;
    int gi = i < 0 ? -i - 1 : (i > 0 ? i - 1 : 0);
    int gj = j < 0 ? -j - 1 : (j > 0 ? j - 1 : 0);
    int gk = k < 0 ? -k - 1 : (k > 0 ? k - 1 : 0);
    double a = __dmul_rn((double)gi, size[0]);
    double b = __dmul_rn((double)gj, size[1]);
    double c = __dmul_rn((double)gk, size[2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// ---- launchers (tess_grid.cu) ----
struct GridBuffers {
    const double* xyz;          // concatenated points, AoS
    const uint32_t* groups;     // point groups or null
    DiagDesc* diags;
    int ndiag;
    uint32_t total;             // total points
    uint64_t total_bins;
    const uint32_t* chunk_diag; // per 8192-point chunk: diagram id
    const uint32_t* chunk_start;
    uint32_t nchunks;
    unsigned long long* bounds; // 6 per diagram (encoded)
    uint32_t* bin;
    uint32_t* rank;
    uint32_t* delims;           // total_bins + 1
    uint32_t* scan_tmp;         // block sums
    uint32_t* sorted;
    uint32_t* inv;              // point -> sorted position, or null (built on demand)
    double* spx;
    double* spy;
    double* spz;
    float* shi;                 // FP32 split of the sorted positions:
    float* slo;                 // x = shi + slo, 3 floats per point each (AoS)
    uint32_t* sgroup;           // null when groups is null
    TabEntry* table;
    int table_gaps;
    int* error_flag;            // set when an input coordinate is not finite
    int* check;                 // checked build: the check word
};
constexpr uint32_t kChunk = 8192;
constexpr int kScanItems = 8;       // items per thread in the scan
constexpr int kScanThreads = 1024;

// side/fork/join (optional): a second stream and two events; the shell
// table is then built on the side stream while the histogram, scan and
// scatter run (fork after the grid parameters, join before returning).
cudaError_t launch_grid_build(const GridBuffers& g, cudaStream_t s, cudaStream_t side = nullptr,
                              cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
// inv[sorted[s]] = s for s < n (the point -> sorted position map, on demand).
cudaError_t launch_inverse(const uint32_t* sorted, uint32_t* inv, uint32_t n, int* check, cudaStream_t s);
// n bytes from src to dst by the SMs (16-byte aligned pointers; either may be
// the device address of pinned host memory).
cudaError_t launch_copy_bytes(void* dst, const void* src, size_t n, int sms, cudaStream_t s);
// out[0] = most points in one bin, out[1] = points in bins of >= crowd points
// (every bin of every diagram of the set)
cudaError_t launch_occupancy(const uint32_t* delims, uint64_t nbins, uint32_t crowd, unsigned long long* out,
                             int blocks, cudaStream_t s);
size_t scan_tmp_words(uint64_t nitems);

// ---- radius queries (tess_radius.cu) ----
// Query kinds: find_cells_in_radius (celery.rs:753-796), the points of those
// bins (find_neighbors_in_cell_radius, celery.rs:802-818), those within the
// radius (find_neighbors_in_real_radius, celery.rs:825-855), and the
// expanding-search neighbour cloud of a cell (interface.rs:348-365).
enum RadiusMode { RQ_CELLS = 0, RQ_CELL_RADIUS = 1, RQ_REAL_RADIUS = 2, RQ_CLOUD = 3 };

struct RadiusParams {
    const DiagDesc* desc;       // the diagram (a set of one)
    const uint32_t* delims;
    const uint32_t* sorted;
    const double* spx;          // FP64 positions in sorted order
    const double* spy;
    const double* spz;
    const uint32_t* sgroup;     // groups in sorted order, or null (all 0)
    const double* xyz;          // points, AoS, original order
    const uint32_t* inv;        // point -> sorted position
    const double* qxyz;         // query positions (AoS), or null: queries are cells
    const uint32_t* qcell;      // cloud query cells (original index), or null: every cell
    uint32_t nq;
    double radius;
    int64_t group;              // cloud only: < 0 keeps every group
    const short4* rtab;         // cloud only: bin offsets with key <= radius, search order
    uint32_t rtab_len;
    uint32_t* count;            // count pass: results per query
    const uint64_t* offs;       // fill pass: CSR offsets per query
    uint32_t* out;              // fill pass: bin ids or original point indices
    int* err;                   // set to 1 when a query cell is out of range
    const uint32_t* qorder;     // processing order of the queries (spatially sorted), or null
    const float* shi;           // FP32 high parts of the sorted positions (AoS), for the FP32 filter
    int f32_filter;             // real radius: pre-filter candidates in FP32 (radius in range)
    // check_cell_in_range as a table: for gaps gx <= gtab_x, gy <= gtab_y, the
    // largest gz <= gtab_z whose squared gap distance is within radius^2
    // (-1: none); null: the FP64 formula per bin
    const int16_t* gtab;
    int gtab_x, gtab_y, gtab_z;
    // bin boundaries per axis: bnd[a * cpd + i] (1 <= i < cpd) is the order
    // code (ord_enc) of the smallest double whose axis_index is >= i
    const unsigned long long* bnd;
};

// Fills RadiusParams::bnd for diagram 0 (3 * cpd entries).
cudaError_t launch_axis_bounds(const DiagDesc* desc, int cpd, unsigned long long* bnd, cudaStream_t s);

// Spatial processing order for large query batches: a counting sort of the
// queries by the coarse bin (2 x 2 x 2 grid bins) holding their position.
struct QueryOrder {
    uint32_t* qbin;             // [nq] coarse bin of each query
    uint32_t* qrank;            // [nq] arrival rank within its coarse bin
    uint32_t* cnt;              // [ncoarse] queries per coarse bin
    uint64_t* coff;             // [ncoarse + 1] offsets
    uint64_t* scan_tmp;         // csr_tmp_words(ncoarse)
    uint32_t* order;            // [nq] the result
    uint32_t ncoarse;
    int cpdc;                   // coarse bins per dimension
};
cudaError_t launch_query_order(const RadiusParams& p, const QueryOrder& o, int blocks, cudaStream_t s);

cudaError_t launch_radius(const RadiusParams& p, int mode, bool fill, int blocks, cudaStream_t s);
// Bin offsets of the search order (celery.rs:418-679) whose key is at most
// `radius`, sorted by (key, i, j, k), for a grid of cpd bins per axis with
// the given bin sizes.  Returns false if more than max_entries would be kept
// or enumerated.
bool build_radius_table(const double size[3], int cpd, double radius, size_t max_entries,
                        std::vector<short4>& out);
// The gap table of RadiusParams::gtab for this radius; false if the radius is
// not finite and non-negative or the table would exceed max_entries.
bool build_gap_table(const double size[3], const double inv[3], int cpd, double radius, size_t max_entries,
                     std::vector<int16_t>& out, int* gx, int* gy, int* gz);

// ---- launchers (tess_clip.cu) ----
struct ClipParams {
    const DiagDesc* diags;
    int ndiag;
    const double* spx;
    const double* spy;
    const double* spz;
    const float* shi;               // x = shi + slo (FP32 pair), AoS
    const float* slo;
    const uint32_t* sorted;
    const uint32_t* delims;
    const uint32_t* sgroup;
    const TabEntry* table;
    const uint32_t* bin;            // global bin of each point (original order)
    // work: sorted positions to process
    const uint32_t* work;          // null: 0 .. total-1
    const uint32_t* work_count;    // null: total
    uint32_t total;
    unsigned int* cursor;          // work cursor (zeroed before launch)
    // results, indexed by point (concatenated original order)
    double* vol;
    uint32_t* nface;
    uint64_t* fstart;
    uint8_t* status;
    int32_t* face_nbr;
    double* face_area;
    unsigned long long* face_cursor;
    uint64_t face_cap;
    // routing of failed cells
    uint32_t* list_fp64;          // guard / degenerate cells (FP32 pass) or null
    unsigned int* list_fp64_count;
    uint32_t* list_cap;           // capacity overflow cells or null
    unsigned int* list_cap_count;
    uint32_t* list_dense;         // lean first pass: cells of crowded bins, or null
    unsigned int* list_dense_count;
    unsigned int* fail_count;     // cells left with an error status
    unsigned int* reasons;        // per status code: cells routed or failed for it
    unsigned long long* work_ctr; // optional work counters (tested, cuts, new vertices, windows, batches)
    // options
    double search_radius;         // < 0: none
    int64_t target_group;         // < 0: none
    float guard_rel;
    float verify_rel;
    uint32_t seed_min;            // own-bin count from which a cell is seeded (crowded bins)
    // single-cell geometry output (queries); null for bulk runs
    GeoOut* geo;
    int at_point;                 // 1: site = point[] below, not a diagram point
    double point[3];
    int box_override;             // 1: walls from box[] instead of the diagram's box
    double box[6];                // lo xyz, hi xyz
    // the binning pass's error flag: when it reports non-finite input (1),
    // the clipping kernels return at once (the batch graph runs every pass
    // without a host check in between)
    const int* grid_err;
    // checked build: the check word, the points and the bins of the set
    int* check;
    uint32_t npts;
    uint64_t nbins;
};

// Forms of the clipping kernel:
//   kFormLean    the FP32 first pass (2 slots per lane, no window pre-test);
//   kFormStd     the re-run passes and the plain FP64 form, with the window
//                pre-test (cells next to dense clusters test hundreds of
//                candidates);
//   kFormHybrid  FP32, 2 slots per lane, with the pre-test, for cells the
//                first pass flagged: a plane test in the guard band is
//                decided in FP64 for the vertices concerned (each recomputed
//                from its three planes) instead of re-running the cell.
//   kFormExact   a flag on the FP32 forms: the finalize refines every vertex
//                with a second FP64-residual Newton step and accumulates face
//                areas and the volume in FP64 (FP64-accurate results)
enum ClipForm : int { kFormLean = 0, kFormStd = 1, kFormHybrid = 2, kFormExact = 4 };
cudaError_t launch_clip_f32(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s);
cudaError_t launch_clip_f64(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s);
int clip_blocks_f32(int slots, int form, int wpb, int device);
int clip_blocks_f64(int slots, int form, int wpb, int device);
// precision: 0 FP64, 1 FP32.  slots: 2, 4 or 8.
cudaError_t launch_clip(const ClipParams& p, int precision, int slots, int form, int warps_per_block,
                        int blocks, cudaStream_t s);
int clip_blocks_for(int precision, int slots, int form, int warps_per_block, int device);
// CSR offsets (3 launches) and the gather into them (1 launch).
cudaError_t launch_csr_offsets(const uint32_t* nface, uint32_t n, uint64_t* offs, uint64_t* scan_tmp,
                               cudaStream_t s);
cudaError_t launch_csr_gather(const uint32_t* nface, const uint64_t* fstart, const int32_t* face_nbr,
                              const double* face_area, uint32_t n, const uint64_t* offs, int32_t* nbr_out,
                              double* area_out, cudaStream_t s);
size_t csr_tmp_words(uint32_t n);

// Sets the calling thread's last error message (printf format).
void set_error(const char* fmt, ...);

}  // namespace tess
