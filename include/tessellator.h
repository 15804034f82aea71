/*
 * tessellator.h -- C ABI of the GB300 (sm_103a) Voronoi cell library
 * (libtessgpu.so).  It is the drop-in for the public API of
 * mcomstock/the-tessellator, src/interface.rs (Diagram, Cell, VoronoiFace).
 * Each declaration names the reference item it replaces.
 *
 * Conventions
 *  - Every call returns tess_status (0 = TESS_OK).  Nothing aborts or
 *    throws across the ABI; tess_last_error() returns the message of the
 *    calling thread's last failure.
 *  - Point indices are the caller's original indices (0 .. n-1), both for
 *    cells and for the neighbour ids that faces report
 *    (interface.rs:329, "original_indices[point_index]").
 *  - Faces of the container box report negative neighbour ids:
 *      -1 x_min, -2 x_max, -3 y_min, -4 y_max, -5 z_min, -6 z_max.
 *    (The reference leaves them as Face { point_index: None },
 *    polyhedron.rs:300-303, and panics on them in compute_neighbors.)
 *  - A cell's faces are returned sorted by neighbour id.
 *  - Vertices are returned relative to the cell's site, as the reference
 *    leaves its polyhedron translated by -position (interface.rs:266).
 *  - Output buffers are caller-owned: pass a capacity; when it is too small
 *    the call returns TESS_E_CAPACITY and still writes the needed count.
 *  - A handle may be read from several threads at once; create, compute and
 *    destroy need exclusive access.
 *  - Every computation runs on the GPU.  There is no CPU fallback: without a
 *    usable CUDA device the calls return TESS_E_CUDA.
 */
#ifndef TESSELLATOR_H
#define TESSELLATOR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TESS_OK = 0,
    TESS_E_INVALID = 1,   /* bad argument (null pointer, n == 0, NaN input, bad index) */
    TESS_E_CUDA = 2,      /* CUDA runtime error (no device, launch failure)           */
    TESS_E_CAPACITY = 3,  /* caller buffer too small; the needed size was written     */
    TESS_E_OVERFLOW = 4,  /* a cell exceeded the largest vertex/face capacity          */
    TESS_E_STATE = 5,     /* results requested before tess_diagram_compute_all         */
    TESS_E_NOMEM = 6,     /* device or host allocation failed                          */
    TESS_E_LIMIT = 7,     /* an iteration cap or wait limit was reached                */
    TESS_E_CHECK = 8      /* checked build only: a device index was out of range        */
} tess_status;

typedef enum {
    /* Plain FP64 clipping: the reference's arithmetic type (float.rs:78). */
    TESS_PRECISION_FP64 = 0,
    /* FP32 clipping; a cell whose plane-side test lands inside the guard
     * band, or whose FP32 vertices fail the FP64 check, is re-run in FP64.
     * Volumes and areas are accumulated in FP64. */
    TESS_PRECISION_FP32_GUARD = 1,
    /* The FP32 + guard clipping (its exact topology and re-runs) with an
     * FP64-accurate finish: every vertex is refined by two Newton steps on its
     * three FP64 face planes, and face areas and volumes are accumulated in
     * FP64 from those vertices.  Volumes are within 1e-11 relative of the
     * FP64 form (the worst of 1,000,000 uniform cells: 1.8e-12; typically
     * 1e-14), at close to the FP32 form's speed.
     * Single-cell geometry queries run it as TESS_PRECISION_FP64. */
    TESS_PRECISION_MIXED = 2
} tess_precision;

/* Flags for tess_config.flags */
#define TESS_FLAG_TIMING 1u     /* record per-pass device times (tess_stats)          */
#define TESS_FLAG_COUNTERS 2u   /* count the clipping work (tess_stats); the FP32 first pass then runs
                                   in its counting form, with the window pre-test (about 2% slower) */
/* Flags that exercise the recovery paths (tests and diagnostics; results are
 * unchanged except as stated): */
#define TESS_FLAG_SMALL_FACE_POOL 4u  /* start the face pool at 1,024 faces, so a compute
                                         overflows it and grows it (tess_stats.face_pool_regrows) */
#define TESS_FLAG_NO_CAPACITY_RERUN 8u /* skip the larger-capacity re-runs: a cell that outgrows
                                          the first pass's vertex or face slots is reported as
                                          failed (TESS_E_OVERFLOW, volume 0, no faces) */
#define TESS_FLAG_AUTOTUNE 16u  /* the first compute of a handle autotunes its launch knobs
                                   (tess_diagram_autotune / tess_batch_autotune with the default
                                   cache file) before it runs */

typedef struct {
    /* FP32 form, guard band: a plane test of vertex v against the bisector of
     * the site and a point at offset r is undecided (the cell re-runs in FP64)
     * when |signed distance| <= e_v + guard_rel * (|v|_1 + |r|) plus a small
     * term for the FP32 split of the positions, with e_v the vertex's tracked
     * error bound (distances normalised by |r|).  The FP32 rounding of a test
     * stays below 3e-7 (|v|_1 + |r|): keep guard_rel at or above that. */
    double guard_rel;
    /* FP32 form, final check: the FP64 correction of every vertex must stay
     * within 2 e_v + verify_rel * R, else the cell re-runs in FP64. */
    double verify_rel;
    /* Points per bin; the reference's cell_density() is 1.25 (celery.rs:185-188). */
    double bin_density;
    /* Extent of the precomputed shell table, in bins of gap (>= 1). */
    int32_t table_gaps;
    /* Warps per block of the clipping kernel (1..32). */
    int32_t warps_per_block;
    /* Vertex slots per lane of the first clipping pass (2, 4 or 8):
     * capacity = 32 x slots.  Overflowing cells re-run at the next size. */
    int32_t slots_per_lane;
    /* CUDA device ordinal. */
    int32_t device;
    /* cudaStream_t to run on; NULL: the library's own stream. */
    void* stream;
    uint32_t flags;
    /* A cell whose own bin holds at least this many points first cuts by the
     * nearest point of each lane's stride of that bin (crowded bins); 0: 12.
     * A launch knob only: results do not depend on it. */
    int32_t crowded_bin;
} tess_config;

/* Work and timing figures of the last tess_diagram_compute_all. */
typedef struct {
    uint64_t cells;             /* cells computed                                  */
    uint64_t faces;             /* faces over all cells                            */
    uint64_t rerun_fp64;        /* FP32 cells re-run in FP64 (guard band / check)  */
    uint64_t rerun_capacity;    /* cells re-run at a larger vertex capacity        */
    uint64_t failed;            /* cells with an error status                      */
    uint64_t table_entries;     /* shell-table entries (all diagrams)              */
    double ms_grid;             /* binning pass (bounds, histogram, scan, scatter) */
    double ms_clip;             /* first clipping pass                             */
    double ms_rerun;            /* re-run passes                                   */
    double ms_csr;              /* CSR compaction                                  */
    uint64_t launches;          /* kernels launched by this handle so far          */
    uint64_t rerun_guard;       /* ... of them: a plane test inside the guard band */
    uint64_t rerun_verify;      /* ... FP32 vertex too far from its FP64 position   */
    uint64_t rerun_degenerate;  /* ... inconsistent topology                        */
    /* work counters, with TESS_FLAG_COUNTERS (all passes): */
    uint64_t candidates_tested; /* bisectors tested against the cell               */
    uint64_t cuts;              /* bisectors that cut vertices off                 */
    uint64_t new_vertices;      /* vertices created by the cuts                    */
    uint64_t windows;           /* candidate windows of up to 32 points            */
    uint64_t batches;           /* batches of up to 32 bins                        */
    /* Last fixed-radius query (TESS_FLAG_TIMING): device times of its count
     * pass (with the scan of the counts) and of its fill pass. */
    double ms_query_count;
    double ms_query_fill;
    /* FP32 form: of the rerun_fp64 cells, those the hybrid re-run (guard-band
     * tests decided in FP64) could not settle, re-run entirely in FP64 */
    uint64_t rerun_fp64_full;
    /* FP32 form: cells whose own bin is crowded (>= crowded_bin points), taken out of
     * the first pass and computed by a pass that first cuts by the nearest
     * point of each lane's stride of that bin */
    uint64_t dense_cells;
    /* times the face pool was found too small and grown, followed by a
     * recompute, since the handle was created */
    uint64_t face_pool_regrows;
} tess_stats;

void tess_config_default(tess_config* cfg);
/* Message of the calling thread's last failed call ("" if none). Returns its length. */
size_t tess_last_error(char* buf, size_t cap);
/* Library version string. */
const char* tess_version(void);

/* ------------------------------------------------------------------------ */
/* Diagram                                                                    */
/* ------------------------------------------------------------------------ */
typedef struct tess_diagram tess_diagram;

/* Replaces Diagram::add_particle_with_group x n + Diagram::initialize
 * (interface.rs:52-84; both private in the reference, so it has no public
 * constructor) and Celery::new (celery.rs:231-250).
 *   xyz     host, n x 3 doubles (AoS)
 *   groups  host, n group ids (interface.rs:43), or NULL (all 0)
 *   lo, hi  the container box (the Polyhedron a caller hands to
 *           get_cell_at_index, interface.rs:186-191), or both NULL: the
 *           Diagram bounding box, which starts at the origin and grows to
 *           contain the points (interface.rs:53-54, vector3.rs:263-288).
 * The points are binned on the GPU (celery.rs:253-414). */
tess_status tess_diagram_create(const double* xyz, size_t n, const uint32_t* groups,
                                const double lo[3], const double hi[3],
                                const tess_config* cfg, tess_diagram** out);
/* Same, with xyz (n x 3 doubles) already in device memory. */
tess_status tess_diagram_create_device(const double* d_xyz, size_t n, const uint32_t* groups,
                                       const double lo[3], const double hi[3],
                                       const tess_config* cfg, tess_diagram** out);
/* Re-bin the points currently held (from device memory, no host copy). */
tess_status tess_diagram_rebuild(tess_diagram* d);
/* Replace the n points (same count) and re-bin: the points of a Diagram
 * changed, followed by Celery::reset (celery.rs:253-266).  on_device != 0:
 * xyz is a device pointer. */
tess_status tess_diagram_update_points(tess_diagram* d, const double* xyz, int on_device);
/* The Celery's public fields (celery.rs:196-217) after binning: cells[n]
 * (bin of each point), sorted_indices[n] (points in bin order, ascending
 * index within a bin) and delimiters[cpd^3 + 1].  Host buffers; any may be
 * NULL. */
tess_status tess_diagram_celery(const tess_diagram* d, uint32_t* cells, uint32_t* sorted_indices,
                                uint32_t* delimiters);
tess_status tess_diagram_destroy(tess_diagram* d);

/* Bulk Diagram::get_cell_at_index(i, box, radius, group) +
 * Cell::compute_voronoi_cell() for every i (interface.rs:186-208, 257-313).
 *   search_radius  < 0: exact cells (the reference's expand_all_no_radius,
 *                  celery.rs:971, ended by a security-radius test);
 *                  >= 0: Some(radius): only bins whose squared gap distance
 *                  is <= radius are searched, as expand_all_in_radius does
 *                  (celery.rs:1023-1036).
 *   target_group   < 0: None; else only points of that group cut
 *                  (interface.rs:280-297). */
tess_status tess_diagram_compute_all(tess_diagram* d, tess_precision precision,
                                     double search_radius, int64_t target_group);
tess_status tess_diagram_stats(const tess_diagram* d, tess_stats* out);
/* Grid figures: cells_per_dimension (celery.rs:159) and the tight point bounds
 * (celery.rs:81-125) as {xmin, xmax, ymin, ymax, zmin, zmax}. */
tess_status tess_diagram_grid(const tess_diagram* d, int64_t* cpd, double bounds[6]);

/* ---- per-cell queries (after compute_all) ---- */
/* Cell::compute_volume (interface.rs:337-339, polyhedron.rs:838-855). */
tess_status tess_cell_volume(const tess_diagram* d, size_t i, double* volume);
/* Cell::compute_neighbors (interface.rs:342-344, polyhedron.rs:871-881). */
tess_status tess_cell_neighbors(const tess_diagram* d, size_t i, int32_t* nbr, size_t cap,
                                size_t* count);
/* Cell::compute_faces + VoronoiFace::compute_neighbor / compute_area
 * (interface.rs:373-384, 408-416). */
tess_status tess_cell_faces(const tess_diagram* d, size_t i, int32_t* nbr, double* area,
                            size_t cap, size_t* count);
/* Cell::compute_vertices (interface.rs:368-370, polyhedron.rs:885-893):
 * site-relative xyz, 3 doubles per vertex.  Recomputes the cell on the GPU
 * with the last compute_all settings. */
tess_status tess_cell_vertices(tess_diagram* d, size_t i, double* xyz, size_t cap,
                               size_t* count);
/* VoronoiFace::compute_vertices (interface.rs:403-405, polyhedron.rs:897-919):
 * vertex cycle of face `face` (index into the sorted face list),
 * counter-clockwise seen from outside the cell. */
tess_status tess_cell_face_vertices(tess_diagram* d, size_t i, size_t face, double* xyz,
                                    size_t cap, size_t* count);
/* Cell::original_index (interface.rs:387-389): identity under the
 * original-index convention. */
tess_status tess_cell_original_index(const tess_diagram* d, size_t i, size_t* original);

/* One cell computed on its own, with its full geometry. */
#define TESS_MAX_CELL_VERTICES 255
#define TESS_MAX_CELL_FACES 254
typedef struct {
    double volume;                       /* polyhedron.rs:838-855                    */
    int32_t nvertices;                   /* polyhedron.rs:885-893                    */
    int32_t nfaces;
    double vertices[3 * 256];            /* site-relative xyz                        */
    int32_t face_neighbor[256];          /* sorted; walls -1 .. -6                   */
    double face_area[256];               /* interface.rs:408-410                     */
    int32_t face_offset[257];            /* face f: face_vertex[face_offset[f] ..]   */
    int32_t face_vertex[3 * 256];        /* vertex indices, CCW seen from outside    */
} tess_cell_geometry;

/* Diagram::get_cell_at_index(i, polyhedron, search_radius, target_group) +
 * Cell::compute_voronoi_cell (interface.rs:186-208, 257-313) for one cell.
 * lo/hi: the container box for this cell (the Polyhedron argument), or both
 * NULL for the diagram's box. */
tess_status tess_cell_compute(tess_diagram* d, size_t i, tess_precision precision, double search_radius,
                              int64_t target_group, const double lo[3], const double hi[3],
                              tess_cell_geometry* out);
/* Diagram::get_cell_at_particle + compute_voronoi_cell (interface.rs:211-232):
 * the cell of a point that is not in the diagram (no self exclusion). */
tess_status tess_cell_compute_at(tess_diagram* d, const double p[3], tess_precision precision,
                                 double search_radius, int64_t target_group, const double lo[3],
                                 const double hi[3], tess_cell_geometry* out);

/* ---- bulk results ---- */
/* All volumes, host buffer of n doubles. */
tess_status tess_volumes(tess_diagram* d, double* volumes);
/* CSR of all faces in original cell order: offs[n+1], nbr[total], area[total]
 * (host buffers).  Any of nbr/area may be NULL; cap is their capacity. */
tess_status tess_neighbors_csr(tess_diagram* d, uint64_t* offs, int32_t* nbr, double* area,
                               size_t cap, size_t* total);
/* Device pointers to the same results (valid until the next compute or
 * destroy): volumes[n], offs[n+1], nbr[total], area[total]. */
tess_status tess_results_device(tess_diagram* d, const double** volumes, const uint64_t** offs,
                                const int32_t** nbr, const double** area, size_t* total);
/* tess_diagram_compute_all with every cell's results delivered to the
 * caller's buffers: the Cell outputs of interface.rs:337-416 (volume,
 * neighbours, face areas) for all cells, as Diagram::compute_voronoi_cell
 * (interface.rs:257-334) gives them one at a time.  The kernels write each
 * cell's faces (neighbour id, area; sorted by id, as in the CSR) into the face
 * pool face_nbr/face_area[face_cap] as the cell finishes, so on a host buffer
 * the faces cross the host link during the compute instead of after it.  Cell
 * i's faces are face_nbr/face_area[face_start[i] .. face_start[i] +
 * face_count[i]); volumes[n], face_start[n], face_count[n] are written at the
 * end.  The two pool buffers must have a device address: pinned host memory
 * (tess_host_alloc, cudaHostAlloc, cudaHostRegister), device or managed
 * memory; pageable memory is TESS_E_INVALID.  The other three may be any
 * memory.  *faces_used (may be NULL) receives the pool positions used.  A pool
 * too small is TESS_E_CAPACITY with *faces_used = the size needed (the diagram
 * is then not computed).  Afterwards the faces exist only in the caller's
 * buffers: tess_neighbors_csr, tess_results_device and the per-cell face
 * queries return TESS_E_STATE until the next tess_diagram_compute_all. */
tess_status tess_diagram_compute_all_to_host(tess_diagram* d, tess_precision precision, double search_radius,
                                             int64_t target_group, double* volumes, uint64_t* face_start,
                                             uint32_t* face_count, int32_t* face_nbr, double* face_area,
                                             size_t face_cap, size_t* faces_used);
/* Pinned, device-mapped host memory for the buffers above (cudaHostAlloc);
 * bytes = 0 gives NULL.  Free with tess_host_free (NULL is a no-op). */
tess_status tess_host_alloc(size_t bytes, void** ptr);
tess_status tess_host_free(void* ptr);

/* ---- fixed-radius queries on the bin grid ---- */
/* Batched over nq queries.  Results come back as CSR: offs[nq+1] and out[total]
 * (u32 bin ids or original point indices), in the reference's order for each
 * query.  offs and *total are always written (offs may be NULL); out is written
 * when it is non-NULL and total <= cap, else TESS_E_CAPACITY (call again with a
 * larger buffer; the results are deterministic).  With on_device = 1 every
 * array argument is a device pointer; otherwise host memory.  These need only
 * the grid, not compute_all.  radius follows the reference's arithmetic for
 * any value, NaN and negative included. */

/* Celery::find_cells_in_radius (celery.rs:753-796) for query positions
 * xyz[nq][3]: the bins (id = i*cpd^2 + j*cpd + k) of the box [q - r, q + r]
 * clamped to the point bounds whose gap distance to q's bin is at most r
 * (check_cell_in_range, celery.rs:708-748), in i, j, k order. */
tess_status tess_find_cells_in_radius(tess_diagram* d, const double* xyz, size_t nq, double radius,
                                      int on_device, uint64_t* offs, uint32_t* cells, size_t cap,
                                      size_t* total);
/* Celery::find_neighbors_in_cell_radius (celery.rs:802-818, real_radius = 0):
 * every point of those bins; find_neighbors_in_real_radius (celery.rs:825-855,
 * real_radius = 1): those at squared distance <= radius * radius.  Bin by bin,
 * ascending index within a bin. */
tess_status tess_find_neighbors_in_radius(tess_diagram* d, const double* xyz, size_t nq, double radius,
                                          int real_radius, int on_device, uint64_t* offs, uint32_t* ids,
                                          size_t cap, size_t* total);
/* Cell::compute_neighbor_cloud (interface.rs:348-365) for the cells
 * cells[ncells] (original indices; NULL = every cell, ncells = n): the points
 * of the bins the expanding search from the cell's position reaches before
 * the first search-order key above radius (expand_all_in_radius,
 * celery.rs:1023-1075; the key is a squared gap distance compared with the
 * unsquared radius), self included, in search order (ties by i, j, k),
 * ascending index within a bin; only target_group's points when
 * target_group >= 0.  TESS_E_LIMIT if the radius reaches more than 2^26 bin
 * offsets. */
tess_status tess_neighbor_cloud(tess_diagram* d, const uint32_t* cells, size_t ncells, double radius,
                                int64_t target_group, int on_device, uint64_t* offs, uint32_t* ids,
                                size_t cap, size_t* total);
/* The same from positions xyz[nq][3] (a Cell made by get_cell_at_particle,
 * interface.rs:211-232). */
tess_status tess_neighbor_cloud_at(tess_diagram* d, const double* xyz, size_t nq, double radius,
                                   int64_t target_group, int on_device, uint64_t* offs, uint32_t* ids,
                                   size_t cap, size_t* total);

/* ------------------------------------------------------------------------ */
/* Batch: many independent diagrams, one persistent launch per pass,          */
/* captured in a CUDA graph (no reference counterpart: the reference builds   */
/* one Diagram at a time).                                                    */
/* ------------------------------------------------------------------------ */
typedef struct tess_batch tess_batch;

/*   pt_offsets  ndiag+1 offsets into xyz (host)
 *   xyz         host, total x 3 doubles
 *   boxes       host, ndiag x 6 doubles {xlo, ylo, zlo, xhi, yhi, zhi} */
tess_status tess_batch_create(size_t ndiag, const uint64_t* pt_offsets, const double* xyz,
                              const double* boxes, const tess_config* cfg, tess_batch** out);
/* Bin and clip every diagram.  The sequence of launches is captured in a CUDA
 * graph on first use and replayed afterwards. */
tess_status tess_batch_compute(tess_batch* b, tess_precision precision);
/* tess_batch_compute with the faces written into the caller's pool as the
 * cells finish, as tess_diagram_compute_all_to_host: volumes, face_start and
 * face_count over all points (total), neighbour ids local to each diagram.
 * The graph captured for a pool is kept while the pool, its capacity and the
 * precision stay the same. */
tess_status tess_batch_compute_to_host(tess_batch* b, tess_precision precision, double* volumes,
                                       uint64_t* face_start, uint32_t* face_count, int32_t* face_nbr,
                                       double* face_area, size_t face_cap, size_t* faces_used);
/* Replace every diagram's points (same offsets and boxes), from host memory or
 * (on_device != 0) device memory; the next tess_batch_compute bins them
 * again.  The batch form of Celery::reset (celery.rs:253-266) over
 * tess_diagram_update_points. */
tess_status tess_batch_update_points(tess_batch* b, const double* xyz, int on_device);
tess_status tess_batch_stats(const tess_batch* b, tess_stats* out);
/* Volumes of all points (concatenated order), host buffer. */
tess_status tess_batch_volumes(tess_batch* b, double* volumes);
/* CSR over all points (concatenated order); neighbour ids are indices local
 * to each diagram. */
tess_status tess_batch_neighbors_csr(tess_batch* b, uint64_t* offs, int32_t* nbr, double* area,
                                     size_t cap, size_t* total);
/* Device pointers to the same results (valid until the next compute, update
 * or destroy): volumes[total points], offs[total points + 1], nbr[faces],
 * area[faces]; the batch form of tess_results_device. */
tess_status tess_batch_results_device(tess_batch* b, const double** volumes, const uint64_t** offs,
                                      const int32_t** nbr, const double** area, size_t* total);
tess_status tess_batch_destroy(tess_batch* b);

/* ------------------------------------------------------------------------ */
/* Autotuning (no reference counterpart; the reference fixes its bin density  */
/* with "TODO: Experiment with different values", celery.rs:185-188)          */
/* ------------------------------------------------------------------------ */
/* The knobs a compute runs with, chosen per input by timing every candidate
 * on an evenly spaced sample of the cells (bin order, so the sample covers
 * the whole box and every diagram of a batch).  Results never depend on
 * them: they change how the work is laid out, not what is computed. */
typedef struct {
    int32_t warps_per_block;   /* chosen warps per block of the clipping kernel      */
    int32_t crowded_bin;       /* chosen crowded-bin threshold (tess_config)        */
    double bin_density;        /* batch: chosen points per bin of the batch's grid;
                                  diagram: the Celery grid's density, unchanged, as
                                  the bin queries expose that grid                  */
    double ms_chosen;          /* the sample's compute time with the chosen knobs   */
    double ms_default;         /* ... with the default knobs                        */
    uint64_t sample_cells;     /* cells in the timing sample                         */
    int32_t trials;            /* candidate knob sets timed (0: read from the cache) */
    int32_t from_cache;        /* 1: the choice came from the cache file             */
    uint32_t max_bin_points;   /* the input's most crowded bin (points)             */
    double crowded_fraction;   /* share of points in bins of >= 12 points           */
} tess_tuning;

/* Tune d's knobs for `precision`.  The choice is kept by the handle for every
 * later compute and written to a cache file, keyed by the device, the form
 * (diagram / batch), the precision, the point count (power-of-two bucket) and
 * the bin occupancy (most crowded bin, crowded share), so the next handle of
 * that kind of input reuses it without timing.  cache_path: the file; NULL:
 * $TESS_TUNE_CACHE, else $XDG_CACHE_HOME/tessellator-gb300/tuning.txt, else
 * $HOME/.cache/tessellator-gb300/tuning.txt; "" : no cache.  The timing runs
 * leave no results: call tess_diagram_compute_all afterwards. */
tess_status tess_diagram_autotune(tess_diagram* d, tess_precision precision, const char* cache_path,
                                  tess_tuning* out);
/* The same for a batch, whose grid density is tuned too (the batch exposes no
 * bin queries); the batch's CUDA graph is captured again with the choice. */
tess_status tess_batch_autotune(tess_batch* b, tess_precision precision, const char* cache_path,
                                tess_tuning* out);

/* ------------------------------------------------------------------------ */
/* No-allocation CSR offsets                                                  */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference.  For callers that may not allocate device
 * memory (a fixed device budget, an allocator that owns all device memory, or
 * a path where an allocation's implicit synchronisation is not allowed):
 * d_offs[0..n] = exclusive scan of d_counts[0..n) (per-cell face counts),
 * d_offs[n] = total, both in device memory, enqueued on `stream`
 * (cudaStream_t, NULL = the default stream).  It calls no allocator.  Its
 * scratch is a 128 KiB device array inside the library, which every GPU that
 * loads the library holds until exit; n may be at most 2^26
 * (TESS_E_CAPACITY beyond).  The first call on a device looks up that array's
 * address, so make it before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race. */
tess_status tess_csr_offsets_noalloc(const uint32_t* d_counts, size_t n, uint64_t* d_offs, void* stream);

#ifdef __cplusplus
}
#endif
#endif
