// tess_api.cu -- host driver and C ABI of libtessgpu.so (declared in
// include/tessellator.h).  Owns the device buffers of a set of diagrams,
// sequences the binning pass and the clipping passes on one CUDA stream, and
// serves the per-cell and bulk queries of the reference's interface.rs API.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include "tess_internal.cuh"
#include "tessellator.h"

using namespace tess;

namespace {

thread_local std::string g_last_error;

tess_status fail(tess_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? TESS_E_NOMEM : TESS_E_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                       \
    } while (0)

#define TRY(call)                                                                                  \
    do {                                                                                           \
        tess_status s_ = (call);                                                                   \
        if (s_ != TESS_OK) return s_;                                                              \
    } while (0)

// Timing events of one call (TESS_FLAG_TIMING), destroyed on every return
// path, early error returns included.
struct TimingEvents {
    cudaEvent_t e[3] = {};
    TimingEvents() = default;
    TimingEvents(const TimingEvents&) = delete;
    TimingEvents& operator=(const TimingEvents&) = delete;
    ~TimingEvents() {
        for (auto& x : e)
            if (x) cudaEventDestroy(x);
    }
    cudaError_t create(int n) {
        for (int i = 0; i < n; ++i) {
            cudaError_t r = cudaEventCreate(&e[i]);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }
    // elapsed milliseconds between two recorded events (0 when unavailable)
    float ms(int a, int b) const {
        float v = 0.f;
        if (cudaEventElapsedTime(&v, e[a], e[b]) != cudaSuccess) v = 0.f;
        (void)cudaGetLastError();   // best-effort timing leaves no error behind
        return v;
    }
};

template <typename T>
tess_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    CU(cudaMalloc((void**)p, sizeof(T) * count));
    return TESS_OK;
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

// Device buffer of at least `need` elements (contents not kept).
template <typename T>
tess_status ensure(T** p, size_t& cap, size_t need) {
    if (*p && need <= cap) return TESS_OK;
    dfree(*p);
    const size_t c = std::max(need, cap + cap / 2);
    TRY(dalloc(p, c));
    cap = c;
    return TESS_OK;
}

// cells_per_dimension = (n / density).cbrt() as usize + 1 (celery.rs:159-160),
// with the host's libm cbrt.
int64_t cells_per_dim(uint64_t n, double density) {
    const double v = std::cbrt((double)n / density);
    if (!(v > 0.0)) return 1;
    return (int64_t)v + 1;
}

// Work lists of the re-run passes: FP64 (cells the FP32 passes flagged),
// CAP1/CAP2 (FP32 capacity), CAP64A/B (FP64 capacity), FP64B (cells the
// hybrid FP32 pass could not settle).
enum { L_FP64 = 0, L_CAP1 = 1, L_CAP2 = 2, L_CAP64A = 3, L_CAP64B = 4, L_FP64B = 5, L_DENSE = 6, L_COUNT = 7,
       L_FAIL = 7, L_REASON = 8 };
// Kernels launched by one binning pass (launch_grid_build).
constexpr uint64_t kGridLaunches = 11;

struct Engine {
    tess_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // the binning pass builds the shell tables on a side stream (fork/join)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    size_t ndiag = 0;
    uint32_t total = 0;
    uint64_t total_bins = 0;
    uint64_t table_total = 0;
    uint32_t nchunks = 0;
    bool has_groups = false;
    std::vector<DiagDesc> hdesc;
    // device
    double* d_xyz = nullptr;
    uint32_t* d_groups = nullptr;
    DiagDesc* d_desc = nullptr;
    uint32_t* d_chunk_diag = nullptr;
    uint32_t* d_chunk_start = nullptr;
    unsigned long long* d_bounds = nullptr;
    uint32_t* d_bin = nullptr;
    uint32_t* d_rank = nullptr;
    uint32_t* d_delims = nullptr;
    uint32_t* d_scan_tmp = nullptr;
    uint32_t* d_sorted = nullptr;
    uint32_t* d_inv = nullptr;
    double* d_spx = nullptr;
    double* d_spy = nullptr;
    double* d_spz = nullptr;
    float* d_shi = nullptr;
    float* d_slo = nullptr;
    uint32_t* d_sgroup = nullptr;
    TabEntry* d_table = nullptr;
    int* d_err = nullptr;
    int* d_check = nullptr;     // checked build: out-of-range index sites (CheckSite bits)
    bool inv_valid = false;     // d_inv matches the current binning
    // results
    double* d_vol = nullptr;
    uint32_t* d_nface = nullptr;
    uint64_t* d_fstart = nullptr;
    uint8_t* d_status = nullptr;
    int32_t* d_fnbr = nullptr;
    double* d_farea = nullptr;
    uint64_t face_cap = 0;
    // tess_diagram_compute_all_to_host: the pool is the caller's buffer for one
    // compute (never regrown), and the faces of that compute are on the host
    bool pool_fixed = false;
    bool faces_on_host = false;
    uint64_t pool_need = 0;
    unsigned long long* d_fcursor = nullptr;
    uint32_t* d_list[L_COUNT] = {};
    unsigned* d_counters = nullptr;   // [0..15] cursors, [16..31] list counts
    unsigned long long* d_work = nullptr;  // work counters (TESS_FLAG_COUNTERS)
    uint64_t* d_offs = nullptr;
    int32_t* d_cnbr = nullptr;
    double* d_carea = nullptr;
    uint64_t csr_cap = 0;
    uint64_t* d_csr_tmp = nullptr;
    GeoOut* d_geo = nullptr;
    uint32_t* d_one = nullptr;
    // radius queries: query positions / cells, per-query counts and offsets,
    // scan scratch, results, and the search-order prefix of the last radius
    double* d_rq = nullptr;
    size_t rq_cap = 0;
    uint32_t* d_rcell = nullptr;
    size_t rcell_cap = 0;
    uint32_t* d_rcnt = nullptr;
    size_t rcnt_cap = 0;
    uint64_t* d_roffs = nullptr;
    size_t roffs_cap = 0;
    uint64_t* d_rtmp = nullptr;
    size_t rtmp_cap = 0;
    uint32_t* d_rout = nullptr;
    size_t rout_cap = 0;
    short4* d_rtab = nullptr;
    size_t rtab_cap = 0;
    uint32_t rtab_len = 0;
    bool rtab_valid = false;
    uint64_t rtab_radius_bits = 0;
    int* d_rerr = nullptr;
    int sm_count = 0;
    unsigned long long* d_bnd = nullptr;   // bin boundaries per axis (3 x cpd order codes)
    size_t bnd_cap = 0;
    bool bnd_valid = false;
    DiagDesc hgrid{};             // host copy of the device-written grid fields
    bool hgrid_valid = false;
    int16_t* d_gtab = nullptr;    // gap table of the last box-query radius
    size_t gtab_cap = 0;
    bool gtab_valid = false, gtab_present = false;
    uint64_t gtab_radius_bits = 0;
    int gtab_dim[3] = {};
    // spatial order of large query batches
    uint32_t* d_qbin = nullptr;
    uint32_t* d_qrank = nullptr;
    uint32_t* d_qorder = nullptr;
    size_t qord_cap = 0, qrank_cap = 0, qorder_cap = 0;
    uint32_t* d_qcnt = nullptr;
    size_t qcnt_cap = 0;
    uint64_t* d_qcoff = nullptr;
    size_t qcoff_cap = 0;
    uint64_t* d_qtmp = nullptr;
    size_t qtmp_cap = 0;
    // state
    bool built = false;
    bool computed = false;
    bool csr_valid = false;
    uint64_t csr_total = 0;
    int last_precision = TESS_PRECISION_FP64;
    double last_radius = -1.0;
    int64_t last_group = -1;
    tess_stats stats{};
    uint64_t launches = 0;    // kernels launched so far (all passes)
    cudaGraphExec_t graph = nullptr;
    int graph_precision = -1;
    // the batch graph captured with a caller's face pool
    // (tess_batch_compute_to_host): its pointers, capacity and precision
    cudaGraphExec_t graph_host = nullptr;
    int graph_host_precision = -1;
    const void* graph_host_nbr = nullptr;
    const void* graph_host_area = nullptr;
    uint64_t graph_host_cap = 0;
    int blocks_cache[2][4][8] = {};   // [kernel type][slots][form, with the exact flag]
    // allocated capacities of the grid arrays a re-grid may grow
    uint64_t delims_alloc = 0, table_alloc = 0;
    // autotuning: the timing sample, the occupancy counters, and whether the
    // knobs were tuned for this handle
    uint32_t* d_sample = nullptr;
    size_t sample_cap = 0;
    unsigned long long* d_occ = nullptr;
    bool tuned = false;

    ~Engine() { release(); }

    void drop_graphs() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        if (graph_host) cudaGraphExecDestroy(graph_host);
        graph_host = nullptr;
    }

    void release() {
        drop_graphs();
        dfree(d_xyz); dfree(d_groups); dfree(d_desc); dfree(d_chunk_diag); dfree(d_chunk_start);
        dfree(d_bounds); dfree(d_bin); dfree(d_rank); dfree(d_delims); dfree(d_scan_tmp);
        dfree(d_sorted); dfree(d_inv); dfree(d_spx); dfree(d_spy); dfree(d_spz); dfree(d_shi); dfree(d_slo); dfree(d_sgroup);
        dfree(d_table); dfree(d_err); dfree(d_check); dfree(d_vol); dfree(d_nface); dfree(d_fstart); dfree(d_status);
        dfree(d_fnbr); dfree(d_farea); dfree(d_fcursor);
        for (auto& l : d_list) dfree(l);
        dfree(d_counters); dfree(d_work); dfree(d_offs); dfree(d_cnbr); dfree(d_carea); dfree(d_csr_tmp);
        dfree(d_geo); dfree(d_one);
        dfree(d_rq); dfree(d_rcell); dfree(d_rcnt); dfree(d_roffs); dfree(d_rtmp); dfree(d_rout); dfree(d_rtab);
        dfree(d_rerr); dfree(d_gtab); dfree(d_bnd); dfree(d_qbin); dfree(d_qrank); dfree(d_qorder); dfree(d_qcnt); dfree(d_qcoff); dfree(d_qtmp);
        dfree(d_sample); dfree(d_occ);
        if (own_stream && stream) cudaStreamDestroy(stream);
        stream = nullptr;
        if (side) cudaStreamDestroy(side);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        side = nullptr;
        ev_fork = ev_join = nullptr;
    }

    int blocks(int precision, int slots, int form = kFormStd) {
        const int si = slots <= 2 ? 0 : (slots <= 4 ? 1 : 2);
        int& b = blocks_cache[precision][si][form];
        if (!b) {
            const int wpb = wpb_for(precision, slots);
            b = clip_blocks_for(precision, slots, form, wpb, device);
        }
        return b;
    }
    int wpb_for(int precision, int slots) const {
        int w = cfg.warps_per_block;
        if (slots >= 8) w = std::min(w, 2);
        else if (slots >= 4) w = std::min(w, 4);
        return std::max(1, w);
    }
};

// Measured on the clustered 4M set (first pass + re-runs): 257.9 ms at 48,
// 238.7 ms at 24, 231.2 ms at 12; uniform inputs have no bin that large.
constexpr int32_t kDefaultCrowdedBin = 12;

void fill_defaults(tess_config* c) {
    c->guard_rel = 4e-7;
    c->verify_rel = 1e-6;
    c->bin_density = 1.25;
    c->table_gaps = 8;
    c->warps_per_block = 8;
    c->slots_per_lane = 2;
    c->device = 0;
    c->stream = nullptr;
    c->flags = 0;
    c->crowded_bin = kDefaultCrowdedBin;
}

tess_status check_config(const tess_config& c) {
    if (!(c.bin_density > 0.0) || !std::isfinite(c.bin_density)) return fail(TESS_E_INVALID, "bin_density must be > 0");
    if (c.table_gaps < 1 || c.table_gaps > 8) return fail(TESS_E_INVALID, "table_gaps must be in [1, 8]");
    if (c.warps_per_block < 1 || c.warps_per_block > 32) return fail(TESS_E_INVALID, "warps_per_block must be in [1, 32]");
    if (c.slots_per_lane != 2 && c.slots_per_lane != 4 && c.slots_per_lane != 8)
        return fail(TESS_E_INVALID, "slots_per_lane must be 2, 4 or 8");
    // below 3e-7 the guard band no longer covers an FP32 plane test's rounding
    if (!(c.guard_rel >= 3e-7) || !(c.guard_rel < 1e-2))
        return fail(TESS_E_INVALID, "guard_rel must be in [3e-7, 1e-2)");
    if (!(c.verify_rel > 0.0) || !(c.verify_rel < 1.0)) return fail(TESS_E_INVALID, "verify_rel must be in (0, 1)");
    if (c.crowded_bin != 0 && (c.crowded_bin < 2 || c.crowded_bin > (1 << 20)))
        return fail(TESS_E_INVALID, "crowded_bin must be 0 (default) or in [2, 2^20]");
    return TESS_OK;
}

// Per diagram: cells per dimension at `density`, the first global bin, and
// the shell table's capacity and offset (cpd and the table extent follow
// CeleryCellInfo::new, celery.rs:153-188).  Returns the totals.
tess_status layout_grid(std::vector<DiagDesc>& diags, double density, int table_gaps, uint64_t* bins_out,
                        uint64_t* tab_out) {
    uint64_t bins = 0, tab = 0;
    for (size_t d = 0; d < diags.size(); ++d) {
        DiagDesc& D = diags[d];
        const int64_t cpd = cells_per_dim(D.n, density);
        if (cpd > 1625) return fail(TESS_E_INVALID, "diagram %zu: %u points give %lld bins per axis (max 1625)",
                                    d, D.n, (long long)cpd);
        D.cpd = (int32_t)cpd;
        D.bin_base = bins;
        bins += (uint64_t)cpd * cpd * cpd;
        int c = table_gaps + 1;
        if (c > cpd - 1) c = (int)cpd - 1;
        if (c < 0) c = 0;
        const uint64_t cube = (uint64_t)(2 * c + 1) * (2 * c + 1) * (2 * c + 1);
        D.tab_cap = (uint32_t)std::min<uint64_t>(cube, (uint64_t)kMaxTable);
        D.tab_base = tab;
        tab += D.tab_cap;
        D.tab_len = 0;
    }
    if (bins + 1 >= 0xFFFFFFF0ull) return fail(TESS_E_INVALID, "too many bins (%llu)", (unsigned long long)bins);
    *bins_out = bins;
    *tab_out = tab;
    return TESS_OK;
}

// Allocate everything for `diags` (pt_base/n/box set) and copy the points.
tess_status engine_init(Engine& E, const tess_config* cfg, std::vector<DiagDesc>& diags, const double* xyz,
                        bool xyz_on_device, const uint32_t* groups) {
    if (cfg) E.cfg = *cfg;
    else fill_defaults(&E.cfg);
    TRY(check_config(E.cfg));
    E.device = E.cfg.device;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0)
        return fail(TESS_E_CUDA, "no CUDA device available (%s)", cudaGetErrorString(ce));
    if (E.device < 0 || E.device >= ndev) return fail(TESS_E_INVALID, "device %d out of range", E.device);
    CU(cudaSetDevice(E.device));
    if (E.cfg.stream) {
        E.stream = (cudaStream_t)E.cfg.stream;
        E.own_stream = false;
    } else {
        CU(cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking));
        E.own_stream = true;
    }
    CU(cudaStreamCreateWithFlags(&E.side, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&E.ev_fork, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&E.ev_join, cudaEventDisableTiming));
    E.ndiag = diags.size();
    uint64_t total = 0, bins = 0, tab = 0;
    std::vector<uint32_t> cdiag, cstart;
    TRY(layout_grid(diags, E.cfg.bin_density, E.cfg.table_gaps, &bins, &tab));
    for (size_t d = 0; d < diags.size(); ++d) {
        const DiagDesc& D = diags[d];
        for (uint32_t s = 0; s < D.n; s += kChunk) {
            cdiag.push_back((uint32_t)d);
            cstart.push_back(D.pt_base + s);
        }
        total += D.n;
    }
    if (total >= 0xFFFFFFF0ull) return fail(TESS_E_INVALID, "too many points (%llu)", (unsigned long long)total);
    E.total = (uint32_t)total;
    E.total_bins = bins;
    E.table_total = tab;
    E.nchunks = (uint32_t)cdiag.size();
    E.hdesc = diags;
    E.has_groups = groups != nullptr;
    const size_t n = E.total;
    TRY(dalloc(&E.d_xyz, 3 * n));
    if (xyz_on_device) CU(cudaMemcpyAsync(E.d_xyz, xyz, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, E.stream));
    else CU(cudaMemcpyAsync(E.d_xyz, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, E.stream));
    if (groups) {
        TRY(dalloc(&E.d_groups, n));
        CU(cudaMemcpyAsync(E.d_groups, groups, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, E.stream));
        TRY(dalloc(&E.d_sgroup, n));
    }
    TRY(dalloc(&E.d_desc, E.ndiag));
    CU(cudaMemcpyAsync(E.d_desc, diags.data(), sizeof(DiagDesc) * E.ndiag, cudaMemcpyHostToDevice, E.stream));
    TRY(dalloc(&E.d_chunk_diag, E.nchunks));
    TRY(dalloc(&E.d_chunk_start, E.nchunks));
    CU(cudaMemcpyAsync(E.d_chunk_diag, cdiag.data(), sizeof(uint32_t) * E.nchunks, cudaMemcpyHostToDevice, E.stream));
    CU(cudaMemcpyAsync(E.d_chunk_start, cstart.data(), sizeof(uint32_t) * E.nchunks, cudaMemcpyHostToDevice, E.stream));
    TRY(dalloc(&E.d_bounds, 6 * E.ndiag));
    TRY(dalloc(&E.d_bin, n));
    TRY(dalloc(&E.d_rank, n));
    TRY(dalloc(&E.d_delims, E.total_bins + 1));
    TRY(dalloc(&E.d_scan_tmp, scan_tmp_words(E.total_bins + 1)));
    E.delims_alloc = E.total_bins + 1;
    TRY(dalloc(&E.d_sorted, n));
    TRY(dalloc(&E.d_inv, n));
    TRY(dalloc(&E.d_spx, n));
    TRY(dalloc(&E.d_spy, n));
    TRY(dalloc(&E.d_spz, n));
    TRY(dalloc(&E.d_shi, 3 * n));
    TRY(dalloc(&E.d_slo, 3 * n));
    TRY(dalloc(&E.d_table, E.table_total));
    E.table_alloc = E.table_total;
    TRY(dalloc(&E.d_err, 1));
    TRY(dalloc(&E.d_check, 1));
    CU(cudaMemsetAsync(E.d_check, 0, sizeof(int), E.stream));
    TRY(dalloc(&E.d_vol, n));
    TRY(dalloc(&E.d_nface, n));
    TRY(dalloc(&E.d_fstart, n));
    TRY(dalloc(&E.d_status, n));
    E.face_cap = (E.cfg.flags & TESS_FLAG_SMALL_FACE_POOL) ? 1024 : (uint64_t)n * 20 + 4096;
    TRY(dalloc(&E.d_fnbr, E.face_cap));
    TRY(dalloc(&E.d_farea, E.face_cap));
    TRY(dalloc(&E.d_fcursor, 1));
    for (auto& l : E.d_list) TRY(dalloc(&l, n));
    TRY(dalloc(&E.d_counters, 32));
    TRY(dalloc(&E.d_work, 8));
    TRY(dalloc(&E.d_offs, n + 1));
    TRY(dalloc(&E.d_csr_tmp, csr_tmp_words(E.total)));
    TRY(dalloc(&E.d_geo, 1));
    TRY(dalloc(&E.d_one, 1));
    return TESS_OK;
}

GridBuffers grid_buffers(Engine& E) {
    GridBuffers g{};
    g.xyz = E.d_xyz;
    g.groups = E.d_groups;
    g.diags = E.d_desc;
    g.ndiag = (int)E.ndiag;
    g.total = E.total;
    g.total_bins = E.total_bins;
    g.chunk_diag = E.d_chunk_diag;
    g.chunk_start = E.d_chunk_start;
    g.nchunks = E.nchunks;
    g.bounds = E.d_bounds;
    g.bin = E.d_bin;
    g.rank = E.d_rank;
    g.delims = E.d_delims;
    g.scan_tmp = E.d_scan_tmp;
    g.sorted = E.d_sorted;
    g.inv = nullptr;   // built on demand (ensure_inv)
    g.spx = E.d_spx;
    g.spy = E.d_spy;
    g.spz = E.d_spz;
    g.shi = E.d_shi;
    g.slo = E.d_slo;
    g.sgroup = E.d_sgroup;
    g.table = E.d_table;
    g.table_gaps = E.cfg.table_gaps;
    g.error_flag = E.d_err;
    g.check = E.d_check;
    return g;
}

// The point -> sorted position map, built on first use after a binning pass.
tess_status ensure_inv(Engine& E) {
    if (E.inv_valid) return TESS_OK;
    CU(launch_inverse(E.d_sorted, E.d_inv, E.total, E.d_check, E.stream));
    // the handle's stream does not block with the legacy default stream:
    // finish here, so plain copies of single entries see the map
    CU(cudaStreamSynchronize(E.stream));
    E.launches += 1;
    E.inv_valid = true;
    return TESS_OK;
}

// The checked build's verdict on the launches so far: TESS_E_CHECK once any
// device index was out of range (the word stays set for the handle).  The
// regular build reads nothing.
tess_status check_word(Engine& E) {
#if TESS_CHECKED
    int w = 0;
    CU(cudaMemcpyAsync(&w, E.d_check, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaStreamSynchronize(E.stream));
    if (w)
        return fail(TESS_E_CHECK,
                    "checked build: out-of-range device index (sites 0x%x: 1 point, 2 bin, 4 slot, 8 plane, 16 list, "
                    "32 face, 64 sort)", w);
#else
    (void)E;
#endif
    return TESS_OK;
}

// The address at which kernels on `device` (the current device) may read and
// write p: pinned host memory (its device mapping), managed memory, or
// memory of that device.  Pageable host memory and another device's memory
// have none here (those go through cudaMemcpyAsync).
static bool sm_address(const void* p, int device, const void** out) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (!a.devicePointer) return false;
    const bool ok = a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged ||
                    (a.type == cudaMemoryTypeDevice && a.device == device);
    if (!ok) return false;
    *out = a.devicePointer;
    return true;
}

// n bytes between the library's buffers and a caller's, on the engine's
// stream.  When both sides have a device address and are 16-byte aligned the
// SMs move the bytes (launch_copy_bytes), else cudaMemcpyAsync does.  Right
// after a long kernel the copy engines start slowly and the SMs do not
// (GB300, after 300 ms of GPU work: 3 GB into pinned host memory in 17.7-22.4
// ms by the copy engine against 16.7 ms by the SMs, 400 MB out of it in
// 2.4-3.9 against 2.0 ms; on some hosts the copy engine took 5-10x longer).
static tess_status copy_async(Engine& E, void* dst, const void* src, size_t n) {
    if (n == 0) return TESS_OK;
    const void *dd = nullptr, *sd = nullptr;
    if (sm_address(dst, E.device, &dd) && sm_address(src, E.device, &sd) && !((reinterpret_cast<uintptr_t>(dd) |
                                                            reinterpret_cast<uintptr_t>(sd)) & 15u)) {
        if (!E.sm_count) CU(cudaDeviceGetAttribute(&E.sm_count, cudaDevAttrMultiProcessorCount, E.device));
        CU(launch_copy_bytes(const_cast<void*>(dd), sd, n, E.sm_count, E.stream));
        E.launches += 1;
        return TESS_OK;
    }
    CU(cudaMemcpyAsync(dst, src, n, cudaMemcpyDefault, E.stream));
    return TESS_OK;
}

tess_status engine_build(Engine& E, bool check) {
    CU(cudaSetDevice(E.device));
    TimingEvents ev;
    const bool timing = E.cfg.flags & TESS_FLAG_TIMING;
    if (timing) {
        CU(ev.create(2));
        CU(cudaEventRecord(ev.e[0], E.stream));
    }
    CU(launch_grid_build(grid_buffers(E), E.stream, E.side, E.ev_fork, E.ev_join));
    E.launches += kGridLaunches;
    if (timing) CU(cudaEventRecord(ev.e[1], E.stream));
    if (check) {
        int err = 0;
        CU(cudaMemcpyAsync(&err, E.d_err, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaStreamSynchronize(E.stream));
        if (err) {
            // the grid describes the bad points: nothing may use it until a
            // build succeeds
            E.built = false;
            E.computed = false;
            E.csr_valid = false;
            if (err == 1) return fail(TESS_E_INVALID, "input coordinates must be finite");
            return fail(TESS_E_CUDA, "shell table exceeded its capacity");
        }
    }
    if (timing) {
        CU(cudaEventSynchronize(ev.e[1]));
        E.stats.ms_grid = ev.ms(0, 1);
    }
    TRY(check_word(E));
    E.built = true;
    E.inv_valid = false;
    E.computed = false;
    E.csr_valid = false;
    E.rtab_valid = false;
    E.gtab_valid = false;
    E.hgrid_valid = false;
    E.bnd_valid = false;
    return TESS_OK;
}

ClipParams base_params(Engine& E) {
    ClipParams p{};
    p.diags = E.d_desc;
    p.ndiag = (int)E.ndiag;
    p.spx = E.d_spx;
    p.spy = E.d_spy;
    p.spz = E.d_spz;
    p.shi = E.d_shi;
    p.slo = E.d_slo;
    p.sorted = E.d_sorted;
    p.delims = E.d_delims;
    p.sgroup = E.d_sgroup;
    p.table = E.d_table;
    p.bin = E.d_bin;
    p.total = E.total;
    p.vol = E.d_vol;
    p.nface = E.d_nface;
    p.fstart = E.d_fstart;
    p.status = E.d_status;
    p.face_nbr = E.d_fnbr;
    p.face_area = E.d_farea;
    p.face_cursor = E.d_fcursor;
    p.face_cap = E.face_cap;
    p.guard_rel = (float)E.cfg.guard_rel;
    p.verify_rel = (float)E.cfg.verify_rel;
    p.grid_err = E.d_err;
    p.check = E.d_check;
    p.npts = E.total;
    p.nbins = E.total_bins;
    p.seed_min = (uint32_t)(E.cfg.crowded_bin > 0 ? E.cfg.crowded_bin : kDefaultCrowdedBin);
    return p;
}

// The fixed launch sequence of one compute (no host synchronisation):
// first pass, capacity re-runs, FP64 re-runs.  Counters: cursor c at
// d_counters[c], list counts at d_counters[16 + list].
tess_status enqueue_passes(Engine& E, int precision, double radius, int64_t group, bool timing,
                           cudaEvent_t* ev, const uint32_t* sample = nullptr, uint32_t nsample = 0) {
    unsigned* cur = E.d_counters;
    unsigned* cnt = E.d_counters + 16;
    CU(cudaMemsetAsync(E.d_counters, 0, sizeof(unsigned) * 32, E.stream));
    CU(cudaMemsetAsync(E.d_fcursor, 0, sizeof(unsigned long long), E.stream));
    if (E.cfg.flags & TESS_FLAG_COUNTERS) CU(cudaMemsetAsync(E.d_work, 0, sizeof(unsigned long long) * 8, E.stream));
    ClipParams base = base_params(E);
    base.search_radius = radius;
    base.target_group = group;
    const int s0 = E.cfg.slots_per_lane;
    int cursor = 0;
    // One launch over a work list (null: every cell).  Failed cells append to
    // the FP64 list (guard, degenerate, verify) and the capacity list.
    auto pass = [&](int prec, int slots, int form, const uint32_t* work, const unsigned* wcount, uint32_t* l64,
                    unsigned* c64, uint32_t* lcap, unsigned* ccap, uint32_t* ldense = nullptr,
                    unsigned* cdense = nullptr) -> tess_status {
        ClipParams p = base;
        p.list_dense = ldense;
        p.list_dense_count = cdense;
        p.work = work;
        p.work_count = wcount;
        if (work && !wcount) p.total = nsample;   // the first pass over a timing sample
        p.cursor = cur + cursor++;
        p.list_fp64 = l64;
        p.list_fp64_count = c64;
        p.list_cap = lcap;
        p.list_cap_count = ccap;
        p.fail_count = cnt + L_FAIL;
        p.reasons = cnt + L_REASON;
        p.work_ctr = (E.cfg.flags & TESS_FLAG_COUNTERS) ? E.d_work : nullptr;
        CU(launch_clip(p, prec, slots, form, E.wpb_for(prec, slots), E.blocks(prec, slots, form), E.stream));
        E.launches += 1;
        return TESS_OK;
    };
    uint32_t* const* L = E.d_list;
    if (timing) CU(cudaEventRecord(ev[0], E.stream));
    // without capacity re-runs, the capacity lists are left out: an overflowing
    // cell is then reported as failed
    const bool norerun = E.cfg.flags & TESS_FLAG_NO_CAPACITY_RERUN;
    if (precision == TESS_PRECISION_FP32_GUARD || precision == TESS_PRECISION_MIXED) {
        // with the exact flag (MIXED) every FP32 pass finishes in FP64
        const int X = precision == TESS_PRECISION_MIXED ? kFormExact : 0;
        // FP32: the lean first pass (2 slots per lane) over every cell but
        // those of crowded bins, which run seeded in the standard form;
        // capacity re-runs at 4 and 8 slots; the flagged cells re-run in the
        // hybrid form (guard-band tests decided in FP64); what that cannot
        // settle runs in the FP64 form.
        const bool two = s0 < 4, one = s0 < 8 && !norerun;
        // (with TESS_FLAG_COUNTERS the first pass runs in the standard form:
        // the lean form keeps no counters)
        const bool lean = s0 <= 2 && !(E.cfg.flags & TESS_FLAG_COUNTERS);
        TRY(pass(1, s0, (lean ? kFormLean : kFormStd) | X, sample, nullptr, L[L_FP64], cnt + L_FP64,
                 one ? L[L_CAP1] : nullptr, cnt + L_CAP1, lean ? L[L_DENSE] : nullptr, cnt + L_DENSE));
        if (lean)
            TRY(pass(1, 2, kFormStd | X, L[L_DENSE], cnt + L_DENSE, L[L_FP64], cnt + L_FP64,
                     norerun ? nullptr : L[L_CAP1], cnt + L_CAP1));
        if (timing) CU(cudaEventRecord(ev[1], E.stream));
        if (one) {
            const int s1 = two ? 4 : 8;
            TRY(pass(1, s1, kFormStd | X, L[L_CAP1], cnt + L_CAP1, L[L_FP64], cnt + L_FP64, two ? L[L_CAP2] : nullptr,
                     cnt + L_CAP2));
            if (two)
                TRY(pass(1, 8, kFormStd | X, L[L_CAP2], cnt + L_CAP2, L[L_FP64], cnt + L_FP64, nullptr, nullptr));
        }
        TRY(pass(1, 2, kFormHybrid | X, L[L_FP64], cnt + L_FP64, L[L_FP64B], cnt + L_FP64B,
                 norerun ? nullptr : L[L_FP64B], cnt + L_FP64B));
        TRY(pass(0, 2, kFormStd, L[L_FP64B], cnt + L_FP64B, nullptr, nullptr, norerun ? nullptr : L[L_CAP64A],
                 cnt + L_CAP64A));
        TRY(pass(0, 4, kFormStd, L[L_CAP64A], cnt + L_CAP64A, nullptr, nullptr, L[L_CAP64B], cnt + L_CAP64B));
        TRY(pass(0, 8, kFormStd, L[L_CAP64B], cnt + L_CAP64B, nullptr, nullptr, nullptr, nullptr));
    } else {
        const bool two = s0 < 4, one = s0 < 8 && !norerun;
        TRY(pass(0, s0, kFormStd, sample, nullptr, nullptr, nullptr, one ? L[L_CAP64A] : nullptr, cnt + L_CAP64A));
        if (timing) CU(cudaEventRecord(ev[1], E.stream));
        if (one) {
            const int s1 = two ? 4 : 8;
            TRY(pass(0, s1, kFormStd, L[L_CAP64A], cnt + L_CAP64A, nullptr, nullptr, two ? L[L_CAP64B] : nullptr,
                     cnt + L_CAP64B));
            if (two) TRY(pass(0, 8, kFormStd, L[L_CAP64B], cnt + L_CAP64B, nullptr, nullptr, nullptr, nullptr));
        }
    }
    if (timing) CU(cudaEventRecord(ev[2], E.stream));
    return TESS_OK;
}

tess_status engine_autotune(Engine& E, int precision, bool batch, const char* cache_path, tess_tuning* out);

tess_status engine_compute(Engine& E, int precision, double radius, int64_t group) {
    if (!E.built) return fail(TESS_E_STATE, "diagram is not built");
    if (precision != TESS_PRECISION_FP64 && precision != TESS_PRECISION_FP32_GUARD &&
        precision != TESS_PRECISION_MIXED)
        return fail(TESS_E_INVALID, "unknown precision %d", precision);
    if (std::isnan(radius)) return fail(TESS_E_INVALID, "search_radius is NaN");
    CU(cudaSetDevice(E.device));
    if ((E.cfg.flags & TESS_FLAG_AUTOTUNE) && !E.tuned) TRY(engine_autotune(E, precision, false, nullptr, nullptr));
    const bool timing = E.cfg.flags & TESS_FLAG_TIMING;
    TimingEvents ev;
    if (timing) CU(ev.create(3));
    for (int attempt = 0; attempt < 4; ++attempt) {
        TRY(enqueue_passes(E, precision, radius, group, timing, ev.e));
        unsigned long long used = 0;
        unsigned counts[16];
        int gerr = 0;
        CU(cudaMemcpyAsync(&used, E.d_fcursor, sizeof(used), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaMemcpyAsync(counts, E.d_counters + 16, sizeof(counts), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaMemcpyAsync(&gerr, E.d_err, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaStreamSynchronize(E.stream));
        if (gerr == 1) {
            // the device points were rebuilt without a check and hold a
            // non-finite coordinate: the clipping kernels did nothing
            E.computed = false;
            return fail(TESS_E_INVALID, "input coordinates must be finite");
        }
        if (used > E.face_cap && E.pool_fixed) {
            // the caller's pool: report the size needed
            E.pool_need = used;
            E.computed = false;
            return fail(TESS_E_CAPACITY, "%llu faces, face_cap %llu", used, (unsigned long long)E.face_cap);
        }
        if (used > E.face_cap) {
            // face pool too small: grow and recompute
            dfree(E.d_fnbr);
            dfree(E.d_farea);
            E.face_cap = std::max<uint64_t>(2 * E.face_cap, used + used / 4 + 4096);
            TRY(dalloc(&E.d_fnbr, E.face_cap));
            TRY(dalloc(&E.d_farea, E.face_cap));
            E.stats.face_pool_regrows += 1;
            continue;
        }
        E.stats.cells = E.total;
        E.stats.faces = used;
        if (precision != TESS_PRECISION_FP64) {
            E.stats.rerun_fp64 = counts[L_FP64];
            E.stats.rerun_fp64_full = counts[L_FP64B];
            E.stats.dense_cells = counts[L_DENSE];
            E.stats.rerun_capacity = (uint64_t)counts[L_CAP1] + counts[L_CAP2] + counts[L_CAP64A] + counts[L_CAP64B];
        } else {
            E.stats.rerun_fp64 = 0;
            E.stats.rerun_fp64_full = 0;
            E.stats.dense_cells = 0;
            E.stats.rerun_capacity = (uint64_t)counts[L_CAP64A] + counts[L_CAP64B];
        }
        if (E.ndiag == 1) {
            DiagDesc dd;
            CU(cudaMemcpy(&dd, E.d_desc, sizeof(DiagDesc), cudaMemcpyDeviceToHost));
            E.stats.table_entries = dd.tab_len;
        }
        if (timing) {
            E.stats.ms_clip = ev.ms(0, 1);
            E.stats.ms_rerun = ev.ms(1, 2);
        }
        E.computed = true;
        E.csr_valid = false;
        E.faces_on_host = E.pool_fixed;
        E.last_precision = precision;
        E.last_radius = radius;
        E.last_group = group;
        const uint64_t failed = counts[L_FAIL];
        E.stats.failed = failed;
        if (E.cfg.flags & TESS_FLAG_COUNTERS) {
            unsigned long long w[8];
            CU(cudaMemcpy(w, E.d_work, sizeof(w), cudaMemcpyDeviceToHost));
            E.stats.candidates_tested = w[0];
            E.stats.cuts = w[1];
            E.stats.new_vertices = w[2];
            E.stats.windows = w[3];
            E.stats.batches = w[4];
        }
        E.stats.rerun_guard = counts[L_REASON + ST_GUARD];
        E.stats.rerun_verify = counts[L_REASON + ST_VERIFY];
        E.stats.rerun_degenerate = counts[L_REASON + ST_DEGEN];
        TRY(check_word(E));
        if (failed) return fail(TESS_E_OVERFLOW, "%llu cells could not be computed", (unsigned long long)failed);
        return TESS_OK;
    }
    return fail(TESS_E_NOMEM, "face pool could not be sized");
}

tess_status engine_csr(Engine& E) {
    if (!E.computed) return fail(TESS_E_STATE, "compute_all has not run");
    if (E.faces_on_host)
        return fail(TESS_E_STATE, "the last compute wrote its faces to the caller's buffers (compute_all_to_host)");
    if (E.csr_valid) return TESS_OK;
    CU(cudaSetDevice(E.device));
    TimingEvents ev;
    const bool timing = E.cfg.flags & TESS_FLAG_TIMING;
    if (timing) CU(ev.create(2));
    // offsets first (to size the outputs), then the gather
    if (timing) CU(cudaEventRecord(ev.e[0], E.stream));
    CU(launch_csr_offsets(E.d_nface, E.total, E.d_offs, E.d_csr_tmp, E.stream));
    uint64_t total = 0;
    CU(cudaMemcpyAsync(&total, E.d_offs + E.total, sizeof(uint64_t), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaStreamSynchronize(E.stream));
    if (total > E.csr_cap || !E.d_cnbr) {
        dfree(E.d_cnbr);
        dfree(E.d_carea);
        E.csr_cap = total + total / 8 + 1024;
        TRY(dalloc(&E.d_cnbr, E.csr_cap));
        TRY(dalloc(&E.d_carea, E.csr_cap));
    }
    CU(launch_csr_gather(E.d_nface, E.d_fstart, E.d_fnbr, E.d_farea, E.total, E.d_offs, E.d_cnbr, E.d_carea,
                         E.stream));
    E.launches += 4;
    if (timing) {
        CU(cudaEventRecord(ev.e[1], E.stream));
        CU(cudaEventSynchronize(ev.e[1]));
        E.stats.ms_csr = ev.ms(0, 1);
    }
    E.csr_total = total;
    E.csr_valid = true;
    return TESS_OK;
}

// ---- autotuning ----

// Lay the grid out again at `density` (batch handles only: a diagram's grid is
// the Celery the bin queries expose) and rebuild it.
tess_status engine_regrid(Engine& E, double density) {
    std::vector<DiagDesc> diags = E.hdesc;
    uint64_t bins = 0, tab = 0;
    TRY(layout_grid(diags, density, E.cfg.table_gaps, &bins, &tab));
    CU(cudaSetDevice(E.device));
    CU(cudaStreamSynchronize(E.stream));
    if (bins + 1 > E.delims_alloc) {
        dfree(E.d_delims);
        dfree(E.d_scan_tmp);
        TRY(dalloc(&E.d_delims, bins + 1));
        TRY(dalloc(&E.d_scan_tmp, scan_tmp_words(bins + 1)));
        E.delims_alloc = bins + 1;
    }
    if (tab > E.table_alloc) {
        dfree(E.d_table);
        TRY(dalloc(&E.d_table, tab));
        E.table_alloc = tab;
    }
    E.hdesc = diags;
    E.total_bins = bins;
    E.table_total = tab;
    E.cfg.bin_density = density;
    CU(cudaMemcpyAsync(E.d_desc, E.hdesc.data(), sizeof(DiagDesc) * E.ndiag, cudaMemcpyHostToDevice, E.stream));
    E.drop_graphs();
    return engine_build(E, true);
}

// The cache file of tuned knobs: explicit path, "" for none, else
// $TESS_TUNE_CACHE, $XDG_CACHE_HOME/tessellator-gb300/tuning.txt or
// $HOME/.cache/tessellator-gb300/tuning.txt.
std::string tuning_cache_path(const char* given) {
    if (given) return std::string(given);
    if (const char* e = std::getenv("TESS_TUNE_CACHE")) return std::string(e);
    std::string dir;
    if (const char* x = std::getenv("XDG_CACHE_HOME")) dir = std::string(x) + "/tessellator-gb300";
    else if (const char* h = std::getenv("HOME")) dir = std::string(h) + "/.cache/tessellator-gb300";
    else return std::string();
    return dir + "/tuning.txt";
}

// One line per key: "<key>\t<warps_per_block> <crowded_bin> <bin_density> <ms_chosen> <ms_default> <sample>".
bool tuning_lookup(const std::string& path, const std::string& key, tess_tuning* t) {
    if (path.empty()) return false;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        const char* tab = std::strchr(line, '\t');
        if (!tab || (size_t)(tab - line) != key.size() || std::strncmp(line, key.c_str(), key.size()) != 0) continue;
        int w = 0, c = 0;
        double d = 0, a = 0, b = 0;
        unsigned long long m = 0;
        if (std::sscanf(tab + 1, "%d %d %lf %lf %lf %llu", &w, &c, &d, &a, &b, &m) == 6 && w >= 1 && w <= 8 &&
            c >= 2 && c <= (1 << 20) && d > 0.0 && std::isfinite(d)) {
            t->warps_per_block = w;
            t->crowded_bin = c;
            t->bin_density = d;
            t->ms_chosen = a;
            t->ms_default = b;
            t->sample_cells = m;
            found = true;   // the last entry of a key wins
        }
    }
    std::fclose(f);
    return found;
}

void tuning_store(const std::string& path, const std::string& key, const tess_tuning& t) {
    if (path.empty()) return;
    // create the directory (one level of parent is enough for the defaults)
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos && slash > 0) {
        const std::string dir = path.substr(0, slash);
        const size_t up = dir.find_last_of('/');
        if (up != std::string::npos && up > 0) mkdir(dir.substr(0, up).c_str(), 0755);
        mkdir(dir.c_str(), 0755);
    }
    std::vector<std::string> keep;
    if (FILE* f = std::fopen(path.c_str(), "r")) {
        char line[1024];
        while (std::fgets(line, sizeof(line), f)) {
            const char* tab = std::strchr(line, '\t');
            if (tab && (size_t)(tab - line) == key.size() && std::strncmp(line, key.c_str(), key.size()) == 0) continue;
            keep.emplace_back(line);
        }
        std::fclose(f);
    }
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s\t%d %d %.17g %.6f %.6f %llu\n", key.c_str(), t.warps_per_block, t.crowded_bin,
                  t.bin_density, t.ms_chosen, t.ms_default, (unsigned long long)t.sample_cells);
    keep.emplace_back(buf);
    const std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) return;
    bool ok = true;
    for (const auto& l : keep) ok &= std::fputs(l.c_str(), f) >= 0;
    ok &= std::fclose(f) == 0;
    if (ok) std::rename(tmp.c_str(), path.c_str());
    else std::remove(tmp.c_str());
}

// Time one compute over the sample with the current knobs (ms), the face
// pool grown first if the sample overflows it.
tess_status time_sample(Engine& E, int precision, uint32_t m, float* ms) {
    TimingEvents ev;
    CU(ev.create(2));
    for (int attempt = 0; attempt < 4; ++attempt) {
        CU(cudaEventRecord(ev.e[0], E.stream));
        TRY(enqueue_passes(E, precision, -1.0, -1, false, nullptr, E.d_sample, m));
        CU(cudaEventRecord(ev.e[1], E.stream));
        unsigned long long used = 0;
        CU(cudaMemcpyAsync(&used, E.d_fcursor, sizeof(used), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaStreamSynchronize(E.stream));
        if (used <= E.face_cap) {
            *ms = ev.ms(0, 1);
            return TESS_OK;
        }
        if (E.pool_fixed) return fail(TESS_E_CAPACITY, "face pool too small for the tuning sample");
        dfree(E.d_fnbr);
        dfree(E.d_farea);
        E.face_cap = std::max<uint64_t>(2 * E.face_cap, used + used / 4 + 4096);
        TRY(dalloc(&E.d_fnbr, E.face_cap));
        TRY(dalloc(&E.d_farea, E.face_cap));
        E.stats.face_pool_regrows += 1;
        E.drop_graphs();
    }
    return fail(TESS_E_NOMEM, "face pool could not be sized");
}

// Choose warps per block, the crowded-bin threshold and (batches) the grid
// density by timing each candidate on an evenly spaced sample of up to
// 262,144 cells in bin order (the whole box, every diagram), two runs each,
// the faster counted.  Candidates: warps per block {4, 8} (the clipping
// kernel's launch bound allows 8 at most), crowded bin {12, 8, 24, 48},
// density {0.6, 1.25, 2.5} points per bin (batches).
tess_status engine_autotune(Engine& E, int precision, bool batch, const char* cache_path, tess_tuning* out) {
    if (!E.built) return fail(TESS_E_STATE, "the grid is not built");
    if (precision != TESS_PRECISION_FP64 && precision != TESS_PRECISION_FP32_GUARD && precision != TESS_PRECISION_MIXED)
        return fail(TESS_E_INVALID, "unknown precision %d", precision);
    CU(cudaSetDevice(E.device));
    tess_tuning T{};
    // the input's occupancy at the reference density
    if (!E.d_occ) TRY(dalloc(&E.d_occ, 2));
    const double dens0 = E.cfg.bin_density;
    if (batch && dens0 != 1.25) TRY(engine_regrid(E, 1.25));
    const int ob = (int)std::min<uint64_t>(4096, (E.total_bins + 255) / 256 + 1);
    CU(launch_occupancy(E.d_delims, E.total_bins, (uint32_t)kDefaultCrowdedBin, E.d_occ, ob, E.stream));
    unsigned long long occ[2] = {0, 0};
    CU(cudaMemcpyAsync(occ, E.d_occ, sizeof(occ), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaStreamSynchronize(E.stream));
    T.max_bin_points = (uint32_t)occ[0];
    T.crowded_fraction = E.total ? (double)occ[1] / (double)E.total : 0.0;
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, E.device));
    char kb[512];
    std::snprintf(kb, sizeof(kb), "%s/%dsm|%s|prec%d|n2^%d|max2^%d|crowd%d", prop.name, prop.multiProcessorCount,
                  batch ? "batch" : "diagram", precision, (int)std::lround(std::log2((double)std::max(1u, E.total))),
                  (int)std::floor(std::log2((double)occ[0] + 1.0)), (int)std::lround(10.0 * T.crowded_fraction));
    std::string key(kb);
    for (auto& ch : key)
        if (ch == ' ' || ch == '\t' || ch == '\n') ch = '_';
    const std::string path = tuning_cache_path(cache_path);
    tess_tuning cached{};
    if (tuning_lookup(path, key, &cached)) {
        E.cfg.warps_per_block = cached.warps_per_block;
        E.cfg.crowded_bin = cached.crowded_bin;
        std::memset(E.blocks_cache, 0, sizeof(E.blocks_cache));
        if (batch && cached.bin_density != E.cfg.bin_density) TRY(engine_regrid(E, cached.bin_density));
        E.drop_graphs();
        cached.from_cache = 1;
        cached.trials = 0;
        cached.max_bin_points = T.max_bin_points;
        cached.crowded_fraction = T.crowded_fraction;
        if (!batch) cached.bin_density = E.cfg.bin_density;
        E.tuned = true;
        E.computed = false;
        E.csr_valid = false;
        if (out) *out = cached;
        return TESS_OK;
    }
    // the sample: every k-th cell in bin (sorted) order
    const uint32_t m = std::min<uint32_t>(E.total, 262144u);
    std::vector<uint32_t> hs(m);
    for (uint32_t i = 0; i < m; ++i) hs[i] = (uint32_t)(((uint64_t)i * E.total) / m);
    TRY(ensure(&E.d_sample, E.sample_cap, m));
    CU(cudaMemcpyAsync(E.d_sample, hs.data(), sizeof(uint32_t) * m, cudaMemcpyHostToDevice, E.stream));
    T.sample_cells = m;
    std::vector<double> dens = batch ? std::vector<double>{1.25, 0.6, 2.5} : std::vector<double>{E.cfg.bin_density};
    const int wpbs[] = {8, 4};
    const int crowds[] = {12, 8, 24, 48};
    float best = INFINITY;
    int bw = 8, bc = kDefaultCrowdedBin;
    double bd = dens[0];
    for (double de : dens) {
        if (batch && de != E.cfg.bin_density) {
            uint64_t nb = 0, nt = 0;
            std::vector<DiagDesc> probe = E.hdesc;
            if (layout_grid(probe, de, E.cfg.table_gaps, &nb, &nt) != TESS_OK) continue;   // too many bins
            TRY(engine_regrid(E, de));
        }
        for (int w : wpbs)
            for (int c : crowds) {
                E.cfg.warps_per_block = w;
                E.cfg.crowded_bin = c;
                std::memset(E.blocks_cache, 0, sizeof(E.blocks_cache));
                float t = INFINITY;
                for (int rep = 0; rep < 2; ++rep) {
                    float ms = 0.f;
                    TRY(time_sample(E, precision, m, &ms));
                    t = std::min(t, ms);
                }
                ++T.trials;
                if (de == 1.25 && w == 8 && c == kDefaultCrowdedBin) T.ms_default = t;
                if (t < best) {
                    best = t;
                    bw = w;
                    bc = c;
                    bd = de;
                }
            }
    }
    E.cfg.warps_per_block = bw;
    E.cfg.crowded_bin = bc;
    std::memset(E.blocks_cache, 0, sizeof(E.blocks_cache));
    if (batch && bd != E.cfg.bin_density) TRY(engine_regrid(E, bd));
    E.drop_graphs();
    T.warps_per_block = bw;
    T.crowded_bin = bc;
    T.bin_density = batch ? bd : E.cfg.bin_density;
    T.ms_chosen = best;
    if (!batch) T.ms_default = T.ms_default > 0 ? T.ms_default : best;
    E.tuned = true;
    E.computed = false;
    E.csr_valid = false;
    tuning_store(path, key, T);
    if (out) *out = T;
    return TESS_OK;
}

// One cell's full geometry: re-run the cell alone (FP64 re-run if the FP32
// form declines it) into the GeoOut buffer and copy it back.
tess_status engine_geo(Engine& E, int precision, uint32_t gs, const double* point, double radius, int64_t group,
                       const double* lo, const double* hi, GeoOut* out) {
    CU(cudaSetDevice(E.device));
    for (int prec : {precision, (int)TESS_PRECISION_FP64}) {
        ClipParams p = base_params(E);
        p.search_radius = radius;
        p.target_group = group;
        CU(cudaMemcpyAsync(E.d_one, &gs, sizeof(uint32_t), cudaMemcpyHostToDevice, E.stream));
        CU(cudaMemsetAsync(E.d_counters, 0, sizeof(unsigned) * 32, E.stream));
        p.work = E.d_one;
        p.work_count = nullptr;
        p.total = 1;
        p.cursor = E.d_counters;
        p.geo = E.d_geo;
        if (point) {
            p.at_point = 1;
            p.point[0] = point[0];
            p.point[1] = point[1];
            p.point[2] = point[2];
        }
        if (lo) {
            p.box_override = 1;
            for (int a = 0; a < 3; ++a) {
                p.box[a] = lo[a];
                p.box[3 + a] = hi[a];
            }
        }
        CU(launch_clip(p, prec == TESS_PRECISION_FP32_GUARD ? 1 : 0, 8, kFormStd, 1, 1, E.stream));
        CU(cudaMemcpyAsync(out, E.d_geo, sizeof(GeoOut), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaStreamSynchronize(E.stream));
        TRY(check_word(E));
        if (out->status == ST_OK) return TESS_OK;
        if (prec == TESS_PRECISION_FP64) break;
    }
    return fail(TESS_E_OVERFLOW, "cell could not be computed (status %d)", out->status);
}


// Largest search-order prefix a neighbour-cloud call may enumerate.
constexpr size_t kMaxRadiusTable = (size_t)1 << 26;
// Query batches at least this large are processed in spatial order.
constexpr size_t kOrderMin = 65536;
// Largest gap table (entries of int16) for box queries; beyond it the
// kernel evaluates the gap distance per bin in FP64.
constexpr size_t kMaxGapTable = 65536;

// Fixed-radius queries (tess_radius.cu) over nq queries: positions qxyz, or
// cells (cloud only; null = every cell).  Count pass, scan, then the fill
// pass into `out` when it is given and the total fits in `cap`.  With
// on_device, qxyz / cells / offs / out are device pointers.
tess_status engine_radius(Engine& E, int mode, bool by_cell, const double* qxyz, const uint32_t* cells, size_t nq,
                          double radius, int64_t group, int on_device, uint64_t* offs, uint32_t* out, size_t cap,
                          size_t* total) {
    if (!E.built) return fail(TESS_E_STATE, "the diagram has no grid");
    if (nq >= 0xFFFFFFFFull) return fail(TESS_E_INVALID, "too many queries (%zu)", nq);
    if (nq && !by_cell && !qxyz) return fail(TESS_E_INVALID, "query positions are NULL");
    CU(cudaSetDevice(E.device));
    if (!E.sm_count) CU(cudaDeviceGetAttribute(&E.sm_count, cudaDevAttrMultiProcessorCount, E.device));
    if (!E.d_rerr) TRY(dalloc(&E.d_rerr, 1));
    RadiusParams p{};
    p.desc = E.d_desc;
    p.delims = E.d_delims;
    p.sorted = E.d_sorted;
    p.spx = E.d_spx;
    p.spy = E.d_spy;
    p.spz = E.d_spz;
    p.sgroup = E.d_sgroup;
    p.xyz = E.d_xyz;
    TRY(ensure_inv(E));
    p.inv = E.d_inv;
    p.nq = (uint32_t)nq;
    p.radius = radius;
    p.group = group;
    p.err = E.d_rerr;
    if (!by_cell) {
        if (on_device) {
            p.qxyz = qxyz;
        } else if (nq) {
            TRY(ensure(&E.d_rq, E.rq_cap, 3 * nq));
            TRY(copy_async(E, E.d_rq, qxyz, sizeof(double) * 3 * nq));
            p.qxyz = E.d_rq;
        }
    } else if (cells) {
        if (on_device) {
            p.qcell = cells;
        } else if (nq) {
            for (size_t t = 0; t < nq; ++t)
                if (cells[t] >= E.total)
                    return fail(TESS_E_INVALID, "cell index %u out of range (n = %u)", cells[t], E.total);
            TRY(ensure(&E.d_rcell, E.rcell_cap, nq));
            TRY(copy_async(E, E.d_rcell, cells, sizeof(uint32_t) * nq));
            p.qcell = E.d_rcell;
        }
    } else if (nq != E.total) {
        return fail(TESS_E_INVALID, "with cells NULL, ncells must be the number of points (%u)", E.total);
    }
    uint64_t bits;
    memcpy(&bits, &radius, sizeof(bits));
    const bool need_cloud_tab = mode == RQ_CLOUD && (!E.rtab_valid || bits != E.rtab_radius_bits);
    const bool need_gap_tab = mode != RQ_CLOUD && (!E.gtab_valid || bits != E.gtab_radius_bits);
    if ((need_cloud_tab || need_gap_tab) && !E.hgrid_valid) {
        CU(cudaMemcpyAsync(&E.hgrid, E.d_desc, sizeof(DiagDesc), cudaMemcpyDeviceToHost, E.stream));
        CU(cudaStreamSynchronize(E.stream));
        E.hgrid_valid = true;
    }
    const DiagDesc& D = E.hgrid;
    if (need_gap_tab) {
        std::vector<int16_t> gt;
        E.gtab_present = build_gap_table(D.size, D.inv, D.cpd, radius, kMaxGapTable, gt, &E.gtab_dim[0],
                                         &E.gtab_dim[1], &E.gtab_dim[2]);
        if (E.gtab_present) {
            TRY(ensure(&E.d_gtab, E.gtab_cap, gt.size()));
            CU(cudaMemcpyAsync(E.d_gtab, gt.data(), sizeof(int16_t) * gt.size(), cudaMemcpyHostToDevice, E.stream));
            CU(cudaStreamSynchronize(E.stream));
        }
        E.gtab_radius_bits = bits;
        E.gtab_valid = true;
    }
    if (mode != RQ_CLOUD && E.gtab_present) {
        p.gtab = E.d_gtab;
        p.gtab_x = E.gtab_dim[0];
        p.gtab_y = E.gtab_dim[1];
        p.gtab_z = E.gtab_dim[2];
    }
    if (!E.bnd_valid) {
        const int cpd = E.hdesc[0].cpd;
        TRY(ensure(&E.d_bnd, E.bnd_cap, 3 * (size_t)cpd));
        CU(launch_axis_bounds(E.d_desc, cpd, E.d_bnd, E.stream));
        E.launches += 1;
        E.bnd_valid = true;
    }
    p.bnd = E.d_bnd;
    p.shi = E.d_shi;
    const double r2 = radius * radius;
    p.f32_filter = mode == RQ_REAL_RADIUS && std::isfinite(radius) && r2 >= 1e-30 && r2 <= 1e36;
    if (mode == RQ_CLOUD) {
        if (need_cloud_tab) {
            std::vector<short4> tab;
            if (!build_radius_table(D.size, D.cpd, radius, kMaxRadiusTable, tab))
                return fail(TESS_E_LIMIT, "radius %g reaches more than %zu bin offsets", radius, kMaxRadiusTable);
            TRY(ensure(&E.d_rtab, E.rtab_cap, tab.size()));
            if (!tab.empty()) {
                CU(cudaMemcpyAsync(E.d_rtab, tab.data(), sizeof(short4) * tab.size(), cudaMemcpyHostToDevice,
                                   E.stream));
                CU(cudaStreamSynchronize(E.stream));
            }
            E.rtab_len = (uint32_t)tab.size();
            E.rtab_radius_bits = bits;
            E.rtab_valid = true;
        }
        p.rtab = E.d_rtab;
        p.rtab_len = E.rtab_len;
    }
    TRY(ensure(&E.d_rcnt, E.rcnt_cap, nq + 1));
    TRY(ensure(&E.d_roffs, E.roffs_cap, nq + 1));
    const size_t tmp_words = csr_tmp_words((uint32_t)std::max<size_t>(nq, 1));
    TRY(ensure(&E.d_rtmp, E.rtmp_cap, tmp_words));
    p.count = E.d_rcnt;
    p.offs = E.d_roffs;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((nq + 7) / 8, (size_t)E.sm_count * 16));
    CU(cudaMemsetAsync(E.d_rerr, 0, sizeof(int), E.stream));
    const bool timing = E.cfg.flags & TESS_FLAG_TIMING;
    TimingEvents tev;
    cudaEvent_t* ev = tev.e;
    if (timing) CU(tev.create(3));
    E.stats.ms_query_count = E.stats.ms_query_fill = 0.0;
    uint64_t tot = 0;
    if (nq) {
        if (timing) CU(cudaEventRecord(ev[0], E.stream));
        if (nq >= kOrderMin && (p.qxyz || p.qcell)) {
            // process large batches in coarse-bin order: neighbouring warps then
            // read the same candidate bins
            QueryOrder o{};
            o.cpdc = (E.hdesc[0].cpd + 1) / 2;
            o.ncoarse = (uint32_t)o.cpdc * (uint32_t)o.cpdc * (uint32_t)o.cpdc;
            TRY(ensure(&E.d_qbin, E.qord_cap, nq));
            TRY(ensure(&E.d_qrank, E.qrank_cap, nq));
            TRY(ensure(&E.d_qorder, E.qorder_cap, nq));
            TRY(ensure(&E.d_qcnt, E.qcnt_cap, o.ncoarse));
            TRY(ensure(&E.d_qcoff, E.qcoff_cap, (size_t)o.ncoarse + 1));
            TRY(ensure(&E.d_qtmp, E.qtmp_cap, csr_tmp_words(o.ncoarse)));
            o.qbin = E.d_qbin;
            o.qrank = E.d_qrank;
            o.order = E.d_qorder;
            o.cnt = E.d_qcnt;
            o.coff = E.d_qcoff;
            o.scan_tmp = E.d_qtmp;
            const int eblocks = (int)std::min<size_t>((nq + 255) / 256, (size_t)E.sm_count * 8);
            CU(launch_query_order(p, o, eblocks, E.stream));
            E.launches += 5;
            p.qorder = E.d_qorder;
        }
        CU(launch_radius(p, mode, false, blocks, E.stream));
        CU(launch_csr_offsets(E.d_rcnt, (uint32_t)nq, E.d_roffs, E.d_rtmp, E.stream));
        if (timing) CU(cudaEventRecord(ev[1], E.stream));
        CU(cudaMemcpyAsync(&tot, E.d_roffs + nq, sizeof(uint64_t), cudaMemcpyDeviceToHost, E.stream));
        E.launches += 4;
    }
    int err = 0;
    CU(cudaMemcpyAsync(&err, E.d_rerr, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaStreamSynchronize(E.stream));
    if (timing && nq) E.stats.ms_query_count = tev.ms(0, 1);
    if (err) return fail(TESS_E_INVALID, "a query cell index is out of range (n = %u)", E.total);
    if (total) *total = (size_t)tot;
    if (offs) {
        if (nq) {
            TRY(copy_async(E, offs, E.d_roffs, sizeof(uint64_t) * (nq + 1)));
        } else if (on_device) {
            CU(cudaMemsetAsync(offs, 0, sizeof(uint64_t), E.stream));
        } else {
            offs[0] = 0;
        }
    }
    if (!out || tot == 0) {
        CU(cudaStreamSynchronize(E.stream));
        return TESS_OK;
    }
    if (tot > cap) {
        CU(cudaStreamSynchronize(E.stream));
        return fail(TESS_E_CAPACITY, "%llu results, capacity %zu", (unsigned long long)tot, cap);
    }
    if (on_device) {
        p.out = out;
    } else {
        TRY(ensure(&E.d_rout, E.rout_cap, tot));
        p.out = E.d_rout;
    }
    if (timing) CU(cudaEventRecord(ev[1], E.stream));
    CU(launch_radius(p, mode, true, blocks, E.stream));
    if (timing) CU(cudaEventRecord(ev[2], E.stream));
    E.launches += 1;
    if (!on_device) TRY(copy_async(E, out, E.d_rout, sizeof(uint32_t) * tot));
    CU(cudaStreamSynchronize(E.stream));
    if (timing) E.stats.ms_query_fill = tev.ms(1, 2);
    return TESS_OK;
}

tess_status validate_box(const double* lo, const double* hi) {
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(lo[a]) || !std::isfinite(hi[a]) || !(lo[a] <= hi[a]))
            return fail(TESS_E_INVALID, "container box must satisfy lo <= hi (axis %d)", a);
    return TESS_OK;
}

}  // namespace

namespace tess {
void set_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}
}  // namespace tess

struct tess_diagram {
    Engine E;
    uint32_t n = 0;
};
struct tess_batch {
    Engine E;
};

extern "C" {

void tess_config_default(tess_config* cfg) {
    if (cfg) fill_defaults(cfg);
}

size_t tess_last_error(char* buf, size_t cap) {
    const size_t n = g_last_error.size();
    if (buf && cap) {
        const size_t m = std::min(n, cap - 1);
        memcpy(buf, g_last_error.data(), m);
        buf[m] = 0;
    }
    return n;
}

const char* tess_version(void) { return "tessellator-gb300 0.1 (sm_103a)"; }

static tess_status create_common(const double* xyz, bool on_device, size_t n, const uint32_t* groups,
                                 const double lo[3], const double hi[3], const tess_config* cfg,
                                 tess_diagram** out) {
    if (!out) return fail(TESS_E_INVALID, "out is NULL");
    *out = nullptr;
    if (!xyz) return fail(TESS_E_INVALID, "xyz is NULL");
    if (n == 0) return fail(TESS_E_INVALID, "a diagram needs at least one point");
    if ((lo == nullptr) != (hi == nullptr)) return fail(TESS_E_INVALID, "give both lo and hi, or neither");
    DiagDesc D{};
    D.pt_base = 0;
    D.n = (uint32_t)n;
    if (lo) {
        TRY(validate_box(lo, hi));
        for (int a = 0; a < 3; ++a) {
            D.blo[a] = lo[a];
            D.bhi[a] = hi[a];
        }
    } else {
        // The Diagram bounding box: starts at the origin and grows to contain
        // every point (interface.rs:53-54, vector3.rs:263-288).
        std::vector<double> hx;
        const double* src = xyz;
        if (on_device) {
            hx.resize(3 * n);
            cudaError_t e = cudaMemcpy(hx.data(), xyz, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return fail(TESS_E_CUDA, "reading device points: %s", cudaGetErrorString(e));
            src = hx.data();
        }
        for (int a = 0; a < 3; ++a) D.blo[a] = D.bhi[a] = 0.0;
        for (size_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) {
                const double v = src[3 * i + a];
                if (v < D.blo[a]) D.blo[a] = v;
                if (v > D.bhi[a]) D.bhi[a] = v;
            }
    }
    tess_diagram* h = new (std::nothrow) tess_diagram();
    if (!h) return fail(TESS_E_NOMEM, "host allocation failed");
    h->n = (uint32_t)n;
    std::vector<DiagDesc> v{D};
    tess_status st = engine_init(h->E, cfg, v, xyz, on_device, groups);
    if (st == TESS_OK) st = engine_build(h->E, true);
    if (st != TESS_OK) {
        delete h;
        return st;
    }
    *out = h;
    return TESS_OK;
}

tess_status tess_diagram_create(const double* xyz, size_t n, const uint32_t* groups, const double lo[3],
                                const double hi[3], const tess_config* cfg, tess_diagram** out) {
    return create_common(xyz, false, n, groups, lo, hi, cfg, out);
}

tess_status tess_diagram_create_device(const double* d_xyz, size_t n, const uint32_t* groups, const double lo[3],
                                       const double hi[3], const tess_config* cfg, tess_diagram** out) {
    return create_common(d_xyz, true, n, groups, lo, hi, cfg, out);
}

tess_status tess_diagram_rebuild(tess_diagram* d) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_build(d->E, false);
}

tess_status tess_diagram_destroy(tess_diagram* d) {
    delete d;
    return TESS_OK;
}

tess_status tess_diagram_compute_all(tess_diagram* d, tess_precision precision, double search_radius,
                                     int64_t target_group) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_compute(d->E, (int)precision, search_radius, target_group);
}

// The address at which the clipping kernels may write a caller's face pool:
// pinned host memory (cudaHostAlloc, cudaHostRegister, tess_host_alloc),
// managed memory, or memory of the handle's device.
static tess_status device_address(void* p, int device, void** out, const char* what) {
    const void* a = nullptr;
    if (!sm_address(p, device, &a))
        return fail(TESS_E_INVALID, "%s is not pinned host or managed memory, or memory of device %d", what, device);
    *out = const_cast<void*>(a);
    return TESS_OK;
}

tess_status tess_diagram_compute_all_to_host(tess_diagram* d, tess_precision precision, double search_radius,
                                             int64_t target_group, double* volumes, uint64_t* face_start,
                                             uint32_t* face_count, int32_t* face_nbr, double* face_area,
                                             size_t face_cap, size_t* faces_used) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    if (!volumes || !face_start || !face_count || !face_nbr || !face_area)
        return fail(TESS_E_INVALID, "NULL output buffer");
    Engine& E = d->E;
    CU(cudaSetDevice(E.device));
    void *dn = nullptr, *da = nullptr;
    TRY(device_address(face_nbr, E.device, &dn, "face_nbr"));
    TRY(device_address(face_area, E.device, &da, "face_area"));
    // a pending autotune times its samples in the library's own pool
    if (E.built && (E.cfg.flags & TESS_FLAG_AUTOTUNE) && !E.tuned &&
        (precision == TESS_PRECISION_FP64 || precision == TESS_PRECISION_FP32_GUARD ||
         precision == TESS_PRECISION_MIXED))
        TRY(engine_autotune(E, (int)precision, false, nullptr, nullptr));
    // the kernels write each cell's faces straight into the caller's pool as
    // the cell finishes, so the faces cross the host link during the compute
    int32_t* const own_nbr = E.d_fnbr;
    double* const own_area = E.d_farea;
    const uint64_t own_cap = E.face_cap;
    E.d_fnbr = static_cast<int32_t*>(dn);
    E.d_farea = static_cast<double*>(da);
    E.face_cap = face_cap;
    E.pool_fixed = true;
    E.pool_need = 0;
    const tess_status st = engine_compute(E, (int)precision, search_radius, target_group);
    E.d_fnbr = own_nbr;
    E.d_farea = own_area;
    E.face_cap = own_cap;
    E.pool_fixed = false;
    if (faces_used) *faces_used = st == TESS_E_CAPACITY ? E.pool_need : E.stats.faces;
    if (st != TESS_OK && st != TESS_E_OVERFLOW) {
        if (st == TESS_E_CAPACITY) E.faces_on_host = false;
        return st;
    }
    // the per-cell results (failed cells: volume 0, no faces)
    const size_t n = d->n;
    TRY(copy_async(E, volumes, E.d_vol, sizeof(double) * n));
    TRY(copy_async(E, face_start, E.d_fstart, sizeof(uint64_t) * n));
    TRY(copy_async(E, face_count, E.d_nface, sizeof(uint32_t) * n));
    CU(cudaStreamSynchronize(E.stream));
    return st;
}

tess_status tess_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(TESS_E_INVALID, "ptr is NULL");
    *ptr = nullptr;
    if (bytes == 0) return TESS_OK;
    const cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(e == cudaErrorMemoryAllocation ? TESS_E_NOMEM : TESS_E_CUDA, "cudaHostAlloc(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    return TESS_OK;
}

tess_status tess_host_free(void* ptr) {
    if (!ptr) return TESS_OK;
    const cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(TESS_E_CUDA, "cudaFreeHost: %s", cudaGetErrorString(e));
    }
    return TESS_OK;
}

tess_status tess_diagram_stats(const tess_diagram* d, tess_stats* out) {
    if (!d || !out) return fail(TESS_E_INVALID, "NULL argument");
    *out = d->E.stats;
    out->launches = d->E.launches;
    return TESS_OK;
}

tess_status tess_diagram_update_points(tess_diagram* d, const double* xyz, int on_device) {
    if (!d || !xyz) return fail(TESS_E_INVALID, "NULL argument");
    Engine& E = d->E;
    CU(cudaSetDevice(E.device));
    TRY(copy_async(E, E.d_xyz, xyz, sizeof(double) * 3 * (size_t)E.total));
    return engine_build(E, true);
}

tess_status tess_diagram_celery(const tess_diagram* d, uint32_t* cells, uint32_t* sorted_indices,
                                uint32_t* delimiters) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    const Engine& E = d->E;
    CU(cudaSetDevice(E.device));
    if (cells) CU(cudaMemcpy(cells, E.d_bin, sizeof(uint32_t) * E.total, cudaMemcpyDeviceToHost));
    if (sorted_indices) CU(cudaMemcpy(sorted_indices, E.d_sorted, sizeof(uint32_t) * E.total, cudaMemcpyDeviceToHost));
    if (delimiters)
        CU(cudaMemcpy(delimiters, E.d_delims, sizeof(uint32_t) * (E.total_bins + 1), cudaMemcpyDeviceToHost));
    return TESS_OK;
}

tess_status tess_diagram_grid(const tess_diagram* d, int64_t* cpd, double bounds[6]) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    DiagDesc D;
    CU(cudaSetDevice(d->E.device));
    CU(cudaMemcpy(&D, d->E.d_desc, sizeof(D), cudaMemcpyDeviceToHost));
    if (cpd) *cpd = D.cpd;
    if (bounds)
        for (int a = 0; a < 3; ++a) {
            bounds[2 * a] = D.glo[a];
            bounds[2 * a + 1] = D.ghi[a];
        }
    return TESS_OK;
}

static tess_status cell_check(const tess_diagram* d, size_t i) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    if (i >= d->n) return fail(TESS_E_INVALID, "cell index %zu out of range (n = %u)", i, d->n);
    if (!d->E.computed) return fail(TESS_E_STATE, "compute_all has not run");
    return TESS_OK;
}

tess_status tess_cell_volume(const tess_diagram* d, size_t i, double* volume) {
    TRY(cell_check(d, i));
    if (!volume) return fail(TESS_E_INVALID, "volume is NULL");
    CU(cudaSetDevice(d->E.device));
    CU(cudaMemcpy(volume, d->E.d_vol + i, sizeof(double), cudaMemcpyDeviceToHost));
    return TESS_OK;
}

tess_status tess_cell_faces(const tess_diagram* d, size_t i, int32_t* nbr, double* area, size_t cap,
                            size_t* count) {
    TRY(cell_check(d, i));
    if (d->E.faces_on_host)
        return fail(TESS_E_STATE, "the last compute wrote its faces to the caller's buffers (compute_all_to_host)");
    CU(cudaSetDevice(d->E.device));
    uint32_t nf = 0;
    uint64_t fs = 0;
    CU(cudaMemcpy(&nf, d->E.d_nface + i, sizeof(nf), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(&fs, d->E.d_fstart + i, sizeof(fs), cudaMemcpyDeviceToHost));
    if (count) *count = nf;
    if (nf > cap) return fail(TESS_E_CAPACITY, "cell %zu has %u faces, capacity %zu", i, nf, cap);
    if (nf) {
        if (nbr) CU(cudaMemcpy(nbr, d->E.d_fnbr + fs, sizeof(int32_t) * nf, cudaMemcpyDeviceToHost));
        if (area) CU(cudaMemcpy(area, d->E.d_farea + fs, sizeof(double) * nf, cudaMemcpyDeviceToHost));
    }
    return TESS_OK;
}

tess_status tess_cell_neighbors(const tess_diagram* d, size_t i, int32_t* nbr, size_t cap, size_t* count) {
    return tess_cell_faces(d, i, nbr, nullptr, cap, count);
}

tess_status tess_cell_original_index(const tess_diagram* d, size_t i, size_t* original) {
    if (!d || !original) return fail(TESS_E_INVALID, "NULL argument");
    if (i >= d->n) return fail(TESS_E_INVALID, "cell index %zu out of range", i);
    *original = i;
    return TESS_OK;
}

static tess_status geo_for(tess_diagram* d, size_t i, GeoOut* g) {
    TRY(cell_check(d, i));
    uint32_t gs = 0;
    CU(cudaSetDevice(d->E.device));
    TRY(ensure_inv(d->E));
    CU(cudaMemcpy(&gs, d->E.d_inv + i, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return engine_geo(d->E, d->E.last_precision, gs, nullptr, d->E.last_radius, d->E.last_group, nullptr, nullptr, g);
}

tess_status tess_cell_vertices(tess_diagram* d, size_t i, double* xyz, size_t cap, size_t* count) {
    GeoOut* g = new (std::nothrow) GeoOut;
    if (!g) return fail(TESS_E_NOMEM, "host allocation failed");
    tess_status st = geo_for(d, i, g);
    if (st == TESS_OK) {
        if (count) *count = (size_t)g->nv;
        if ((size_t)g->nv > cap) st = fail(TESS_E_CAPACITY, "cell %zu has %d vertices, capacity %zu", i, g->nv, cap);
        else if (xyz) memcpy(xyz, g->verts, sizeof(double) * 3 * g->nv);
    }
    delete g;
    return st;
}

tess_status tess_cell_face_vertices(tess_diagram* d, size_t i, size_t face, double* xyz, size_t cap,
                                    size_t* count) {
    GeoOut* g = new (std::nothrow) GeoOut;
    if (!g) return fail(TESS_E_NOMEM, "host allocation failed");
    tess_status st = geo_for(d, i, g);
    if (st == TESS_OK) {
        if (face >= (size_t)g->nf) {
            st = fail(TESS_E_INVALID, "face %zu out of range (%d faces)", face, g->nf);
        } else {
            const int b = g->face_off[face], e = g->face_off[face + 1];
            if (count) *count = (size_t)(e - b);
            if ((size_t)(e - b) > cap) st = fail(TESS_E_CAPACITY, "face has %d vertices, capacity %zu", e - b, cap);
            else if (xyz)
                for (int t = b; t < e; ++t) memcpy(xyz + 3 * (t - b), g->verts + 3 * g->face_vtx[t], 3 * sizeof(double));
        }
    }
    delete g;
    return st;
}

static void geo_to_public(const GeoOut& g, tess_cell_geometry* out) {
    out->volume = g.volume;
    out->nvertices = g.nv;
    out->nfaces = g.nf;
    memcpy(out->vertices, g.verts, sizeof(out->vertices));
    memcpy(out->face_neighbor, g.face_nbr, sizeof(out->face_neighbor));
    memcpy(out->face_area, g.face_area, sizeof(out->face_area));
    memcpy(out->face_offset, g.face_off, sizeof(out->face_offset));
    memcpy(out->face_vertex, g.face_vtx, sizeof(out->face_vertex));
}

static tess_status single_cell(tess_diagram* d, const size_t* i, const double* p, tess_precision precision,
                               double search_radius, int64_t target_group, const double lo[3], const double hi[3],
                               tess_cell_geometry* out) {
    if (!d || !out) return fail(TESS_E_INVALID, "NULL argument");
    if (!d->E.built) return fail(TESS_E_STATE, "diagram is not built");
    if ((lo == nullptr) != (hi == nullptr)) return fail(TESS_E_INVALID, "give both lo and hi, or neither");
    if (lo) TRY(validate_box(lo, hi));
    if ((int)precision != TESS_PRECISION_FP64 && (int)precision != TESS_PRECISION_FP32_GUARD &&
        (int)precision != TESS_PRECISION_MIXED)
        return fail(TESS_E_INVALID, "unknown precision %d", (int)precision);
    if (std::isnan(search_radius)) return fail(TESS_E_INVALID, "search_radius is NaN");
    uint32_t gs = 0;
    CU(cudaSetDevice(d->E.device));
    if (i) {
        if (*i >= d->n) return fail(TESS_E_INVALID, "cell index %zu out of range (n = %u)", *i, d->n);
        TRY(ensure_inv(d->E));
        CU(cudaMemcpy(&gs, d->E.d_inv + *i, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    } else if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2])) {
        return fail(TESS_E_INVALID, "point must be finite");
    }
    GeoOut* g = new (std::nothrow) GeoOut;
    if (!g) return fail(TESS_E_NOMEM, "host allocation failed");
    tess_status st = engine_geo(d->E, (int)precision, gs, i ? nullptr : p, search_radius, target_group, lo, hi, g);
    if (st == TESS_OK) geo_to_public(*g, out);
    delete g;
    return st;
}

tess_status tess_cell_compute(tess_diagram* d, size_t i, tess_precision precision, double search_radius,
                              int64_t target_group, const double lo[3], const double hi[3],
                              tess_cell_geometry* out) {
    return single_cell(d, &i, nullptr, precision, search_radius, target_group, lo, hi, out);
}

tess_status tess_cell_compute_at(tess_diagram* d, const double p[3], tess_precision precision,
                                 double search_radius, int64_t target_group, const double lo[3],
                                 const double hi[3], tess_cell_geometry* out) {
    if (!p) return fail(TESS_E_INVALID, "point is NULL");
    return single_cell(d, nullptr, p, precision, search_radius, target_group, lo, hi, out);
}

tess_status tess_volumes(tess_diagram* d, double* volumes) {
    if (!d || !volumes) return fail(TESS_E_INVALID, "NULL argument");
    if (!d->E.computed) return fail(TESS_E_STATE, "compute_all has not run");
    CU(cudaSetDevice(d->E.device));
    TRY(copy_async(d->E, volumes, d->E.d_vol, sizeof(double) * d->n));
    CU(cudaStreamSynchronize(d->E.stream));
    return TESS_OK;
}

static tess_status csr_out(Engine& E, uint64_t* offs, int32_t* nbr, double* area, size_t cap, size_t* total) {
    TRY(engine_csr(E));
    if (total) *total = E.csr_total;
    CU(cudaSetDevice(E.device));
    if (offs) TRY(copy_async(E, offs, E.d_offs, sizeof(uint64_t) * (E.total + 1)));
    if ((nbr || area) && E.csr_total > cap) {
        CU(cudaStreamSynchronize(E.stream));
        return fail(TESS_E_CAPACITY, "%llu faces, capacity %zu", (unsigned long long)E.csr_total, cap);
    }
    if (nbr && E.csr_total)
        TRY(copy_async(E, nbr, E.d_cnbr, sizeof(int32_t) * E.csr_total));
    if (area && E.csr_total)
        TRY(copy_async(E, area, E.d_carea, sizeof(double) * E.csr_total));
    CU(cudaStreamSynchronize(E.stream));
    return TESS_OK;
}

tess_status tess_neighbors_csr(tess_diagram* d, uint64_t* offs, int32_t* nbr, double* area, size_t cap,
                               size_t* total) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return csr_out(d->E, offs, nbr, area, cap, total);
}

tess_status tess_results_device(tess_diagram* d, const double** volumes, const uint64_t** offs,
                                const int32_t** nbr, const double** area, size_t* total) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    TRY(engine_csr(d->E));
    if (volumes) *volumes = d->E.d_vol;
    if (offs) *offs = d->E.d_offs;
    if (nbr) *nbr = d->E.d_cnbr;
    if (area) *area = d->E.d_carea;
    if (total) *total = d->E.csr_total;
    return TESS_OK;
}

// ---- radius queries ----
tess_status tess_find_cells_in_radius(tess_diagram* d, const double* xyz, size_t nq, double radius, int on_device,
                                      uint64_t* offs, uint32_t* cells, size_t cap, size_t* total) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_radius(d->E, RQ_CELLS, false, xyz, nullptr, nq, radius, -1, on_device, offs, cells, cap, total);
}

tess_status tess_find_neighbors_in_radius(tess_diagram* d, const double* xyz, size_t nq, double radius,
                                          int real_radius, int on_device, uint64_t* offs, uint32_t* ids,
                                          size_t cap, size_t* total) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_radius(d->E, real_radius ? RQ_REAL_RADIUS : RQ_CELL_RADIUS, false, xyz, nullptr, nq, radius, -1,
                         on_device, offs, ids, cap, total);
}

tess_status tess_neighbor_cloud(tess_diagram* d, const uint32_t* cells, size_t ncells, double radius,
                                int64_t target_group, int on_device, uint64_t* offs, uint32_t* ids, size_t cap,
                                size_t* total) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_radius(d->E, RQ_CLOUD, true, nullptr, cells, ncells, radius, target_group, on_device, offs, ids, cap,
                         total);
}

tess_status tess_neighbor_cloud_at(tess_diagram* d, const double* xyz, size_t nq, double radius,
                                   int64_t target_group, int on_device, uint64_t* offs, uint32_t* ids, size_t cap,
                                   size_t* total) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_radius(d->E, RQ_CLOUD, false, xyz, nullptr, nq, radius, target_group, on_device, offs, ids, cap, total);
}

// ---- batch ----
tess_status tess_batch_create(size_t ndiag, const uint64_t* pt_offsets, const double* xyz, const double* boxes,
                              const tess_config* cfg, tess_batch** out) {
    if (!out) return fail(TESS_E_INVALID, "out is NULL");
    *out = nullptr;
    if (ndiag == 0 || !pt_offsets || !xyz || !boxes) return fail(TESS_E_INVALID, "NULL or empty argument");
    if (pt_offsets[0] != 0) return fail(TESS_E_INVALID, "pt_offsets[0] must be 0");
    std::vector<DiagDesc> v(ndiag);
    for (size_t d = 0; d < ndiag; ++d) {
        if (pt_offsets[d + 1] <= pt_offsets[d]) return fail(TESS_E_INVALID, "diagram %zu is empty", d);
        if (pt_offsets[d + 1] >= 0xFFFFFFF0ull) return fail(TESS_E_INVALID, "too many points");
        DiagDesc& D = v[d];
        memset(&D, 0, sizeof(D));
        D.pt_base = (uint32_t)pt_offsets[d];
        D.n = (uint32_t)(pt_offsets[d + 1] - pt_offsets[d]);
        TRY(validate_box(boxes + 6 * d, boxes + 6 * d + 3));
        for (int a = 0; a < 3; ++a) {
            D.blo[a] = boxes[6 * d + a];
            D.bhi[a] = boxes[6 * d + 3 + a];
        }
    }
    tess_batch* h = new (std::nothrow) tess_batch();
    if (!h) return fail(TESS_E_NOMEM, "host allocation failed");
    tess_status st = engine_init(h->E, cfg, v, xyz, false, nullptr);
    if (st == TESS_OK) st = engine_build(h->E, true);
    if (st != TESS_OK) {
        delete h;
        return st;
    }
    *out = h;
    return TESS_OK;
}

// One batch compute: the captured graph (grid build + passes) for this
// precision and face pool, captured again when either changed.  With a
// caller's pool (E.pool_fixed) the graph of that pool is kept beside the
// library's own.
static tess_status batch_run(tess_batch* b, int prec) {
    Engine& E = b->E;
    const bool host = E.pool_fixed;
    cudaGraphExec_t& G = host ? E.graph_host : E.graph;
    int& gprec = host ? E.graph_host_precision : E.graph_precision;
    const bool stale = !G || gprec != prec ||
                       (host && (E.graph_host_nbr != E.d_fnbr || E.graph_host_area != E.d_farea ||
                                 E.graph_host_cap != E.face_cap));
    if (stale) {
        // warm the per-kernel attributes and occupancy queries outside capture
        for (int pr : {0, 1})
            for (int s : {2, 4, 8})
                for (int f : {(int)kFormLean, (int)kFormStd, (int)kFormHybrid})
                    for (int x : {0, (int)kFormExact}) E.blocks(pr, s, f | x);
        if (G) cudaGraphExecDestroy(G);
        G = nullptr;
        cudaGraph_t g = nullptr;
        CU(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
        tess_status st = TESS_OK;
        cudaError_t ce = launch_grid_build(grid_buffers(E), E.stream, E.side, E.ev_fork, E.ev_join);
        if (ce != cudaSuccess) st = fail(TESS_E_CUDA, "capture: %s", cudaGetErrorString(ce));
        if (st == TESS_OK) st = enqueue_passes(E, prec, -1.0, -1, false, nullptr);
        cudaError_t ee = cudaStreamEndCapture(E.stream, &g);
        if (st != TESS_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (ee != cudaSuccess) return fail(TESS_E_CUDA, "end capture: %s", cudaGetErrorString(ee));
        ce = cudaGraphInstantiate(&G, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return fail(TESS_E_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
        gprec = prec;
        if (host) {
            E.graph_host_nbr = E.d_fnbr;
            E.graph_host_area = E.d_farea;
            E.graph_host_cap = E.face_cap;
        }
    }
    TimingEvents ev;
    const bool timing = E.cfg.flags & TESS_FLAG_TIMING;
    if (timing) {
        CU(ev.create(2));
        CU(cudaEventRecord(ev.e[0], E.stream));
    }
    CU(cudaGraphLaunch(G, E.stream));
    E.launches += kGridLaunches + (prec != TESS_PRECISION_FP64 ? 7 : 3);
    if (timing) CU(cudaEventRecord(ev.e[1], E.stream));
    unsigned long long used = 0;
    unsigned counts[16];
    int gerr = 0;
    CU(cudaMemcpyAsync(&used, E.d_fcursor, sizeof(used), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaMemcpyAsync(counts, E.d_counters + 16, sizeof(counts), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaMemcpyAsync(&gerr, E.d_err, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
    CU(cudaStreamSynchronize(E.stream));
    TRY(check_word(E));
    if (timing) E.stats.ms_clip = ev.ms(0, 1);
    if (gerr == 1) {
        E.computed = false;
        return fail(TESS_E_INVALID, "input coordinates must be finite");
    }
    if (gerr == 2) return fail(TESS_E_CUDA, "shell table exceeded its capacity");
    if (used > E.face_cap && host) {
        // the caller's pool: report the size needed
        E.pool_need = used;
        E.computed = false;
        return fail(TESS_E_CAPACITY, "%llu faces, face_cap %llu", used, (unsigned long long)E.face_cap);
    }
    if (used > E.face_cap) {
        // grow the pool; the captured graph holds the old pointer
        dfree(E.d_fnbr);
        dfree(E.d_farea);
        E.face_cap = used + used / 4 + 4096;
        TRY(dalloc(&E.d_fnbr, E.face_cap));
        TRY(dalloc(&E.d_farea, E.face_cap));
        E.stats.face_pool_regrows += 1;
        cudaGraphExecDestroy(E.graph);
        E.graph = nullptr;
        return batch_run(b, prec);
    }
    E.stats.cells = E.total;
    E.stats.faces = used;
    const bool f32 = prec != TESS_PRECISION_FP64;
    E.stats.rerun_fp64 = f32 ? counts[L_FP64] : 0;
    E.stats.rerun_fp64_full = f32 ? counts[L_FP64B] : 0;
    E.stats.dense_cells = f32 ? counts[L_DENSE] : 0;
    E.stats.rerun_capacity = (uint64_t)counts[L_CAP1] + counts[L_CAP2] + counts[L_CAP64A] + counts[L_CAP64B];
    E.stats.failed = counts[L_FAIL];
    E.stats.rerun_guard = counts[L_REASON + ST_GUARD];
    E.stats.rerun_verify = counts[L_REASON + ST_VERIFY];
    E.stats.rerun_degenerate = counts[L_REASON + ST_DEGEN];
    E.computed = true;
    E.csr_valid = false;
    E.faces_on_host = host;
    E.last_precision = prec;
    if (counts[L_FAIL]) return fail(TESS_E_OVERFLOW, "%u cells could not be computed", counts[L_FAIL]);
    return TESS_OK;
}

static bool known_precision(int prec) {
    return prec == TESS_PRECISION_FP64 || prec == TESS_PRECISION_FP32_GUARD || prec == TESS_PRECISION_MIXED;
}

tess_status tess_batch_compute(tess_batch* b, tess_precision precision) {
    if (!b) return fail(TESS_E_INVALID, "batch is NULL");
    Engine& E = b->E;
    const int prec = (int)precision;
    if (!known_precision(prec)) return fail(TESS_E_INVALID, "unknown precision %d", prec);
    CU(cudaSetDevice(E.device));
    if ((E.cfg.flags & TESS_FLAG_AUTOTUNE) && !E.tuned) TRY(engine_autotune(E, prec, true, nullptr, nullptr));
    return batch_run(b, prec);
}

tess_status tess_batch_compute_to_host(tess_batch* b, tess_precision precision, double* volumes,
                                       uint64_t* face_start, uint32_t* face_count, int32_t* face_nbr,
                                       double* face_area, size_t face_cap, size_t* faces_used) {
    if (!b) return fail(TESS_E_INVALID, "batch is NULL");
    if (!volumes || !face_start || !face_count || !face_nbr || !face_area)
        return fail(TESS_E_INVALID, "NULL output buffer");
    Engine& E = b->E;
    const int prec = (int)precision;
    if (!known_precision(prec)) return fail(TESS_E_INVALID, "unknown precision %d", prec);
    CU(cudaSetDevice(E.device));
    void *dn = nullptr, *da = nullptr;
    TRY(device_address(face_nbr, E.device, &dn, "face_nbr"));
    TRY(device_address(face_area, E.device, &da, "face_area"));
    // a pending autotune times its samples in the library's own pool
    if ((E.cfg.flags & TESS_FLAG_AUTOTUNE) && !E.tuned) TRY(engine_autotune(E, prec, true, nullptr, nullptr));
    int32_t* const own_nbr = E.d_fnbr;
    double* const own_area = E.d_farea;
    const uint64_t own_cap = E.face_cap;
    E.d_fnbr = static_cast<int32_t*>(dn);
    E.d_farea = static_cast<double*>(da);
    E.face_cap = face_cap;
    E.pool_fixed = true;
    E.pool_need = 0;
    const tess_status st = batch_run(b, prec);
    E.d_fnbr = own_nbr;
    E.d_farea = own_area;
    E.face_cap = own_cap;
    E.pool_fixed = false;
    if (faces_used) *faces_used = st == TESS_E_CAPACITY ? E.pool_need : E.stats.faces;
    if (st != TESS_OK && st != TESS_E_OVERFLOW) {
        if (st == TESS_E_CAPACITY) E.faces_on_host = false;
        return st;
    }
    const size_t n = E.total;
    TRY(copy_async(E, volumes, E.d_vol, sizeof(double) * n));
    TRY(copy_async(E, face_start, E.d_fstart, sizeof(uint64_t) * n));
    TRY(copy_async(E, face_count, E.d_nface, sizeof(uint32_t) * n));
    CU(cudaStreamSynchronize(E.stream));
    return st;
}

tess_status tess_batch_update_points(tess_batch* b, const double* xyz, int on_device) {
    if (!b || !xyz) return fail(TESS_E_INVALID, "NULL argument");
    Engine& E = b->E;
    CU(cudaSetDevice(E.device));
    // the captured graph re-bins from d_xyz, so only the copy is enqueued here
    TRY(copy_async(E, E.d_xyz, xyz, sizeof(double) * 3 * (size_t)E.total));
    E.computed = false;
    E.csr_valid = false;
    return TESS_OK;
}

tess_status tess_batch_stats(const tess_batch* b, tess_stats* out) {
    if (!b || !out) return fail(TESS_E_INVALID, "NULL argument");
    *out = b->E.stats;
    out->launches = b->E.launches;
    return TESS_OK;
}

tess_status tess_batch_volumes(tess_batch* b, double* volumes) {
    if (!b || !volumes) return fail(TESS_E_INVALID, "NULL argument");
    if (!b->E.computed) return fail(TESS_E_STATE, "compute has not run");
    CU(cudaSetDevice(b->E.device));
    TRY(copy_async(b->E, volumes, b->E.d_vol, sizeof(double) * b->E.total));
    CU(cudaStreamSynchronize(b->E.stream));
    return TESS_OK;
}

tess_status tess_batch_neighbors_csr(tess_batch* b, uint64_t* offs, int32_t* nbr, double* area, size_t cap,
                                     size_t* total) {
    if (!b) return fail(TESS_E_INVALID, "batch is NULL");
    return csr_out(b->E, offs, nbr, area, cap, total);
}

tess_status tess_batch_results_device(tess_batch* b, const double** volumes, const uint64_t** offs,
                                      const int32_t** nbr, const double** area, size_t* total) {
    if (!b) return fail(TESS_E_INVALID, "batch is NULL");
    TRY(engine_csr(b->E));
    if (volumes) *volumes = b->E.d_vol;
    if (offs) *offs = b->E.d_offs;
    if (nbr) *nbr = b->E.d_cnbr;
    if (area) *area = b->E.d_carea;
    if (total) *total = b->E.csr_total;
    return TESS_OK;
}

tess_status tess_diagram_autotune(tess_diagram* d, tess_precision precision, const char* cache_path,
                                  tess_tuning* out) {
    if (!d) return fail(TESS_E_INVALID, "diagram is NULL");
    return engine_autotune(d->E, (int)precision, false, cache_path, out);
}

tess_status tess_batch_autotune(tess_batch* b, tess_precision precision, const char* cache_path, tess_tuning* out) {
    if (!b) return fail(TESS_E_INVALID, "batch is NULL");
    return engine_autotune(b->E, (int)precision, true, cache_path, out);
}

tess_status tess_batch_destroy(tess_batch* b) {
    delete b;
    return TESS_OK;
}

}  // extern "C"
