/*
 * tess_oracle.h -- CPU restatement (FP64) of The Tessellator's per-particle
 * Voronoi cell computation.  TEST INFRASTRUCTURE ONLY: this library is the
 * checker for the CUDA implementation and the timed CPU baseline.  Nothing in
 * the product path links or calls it.
 *
 * Every function names the reference file:line it restates (paths are within
 * the mcomstock/the-tessellator project).  Where the reference is unfinished
 * (polyhedron.rs:438-730 is work in progress), the intended half-space clip is
 * restated with the reference's own arithmetic: bisector construction,
 * three-way classification with absolute tolerance 1e-12, the edge
 * intersection formula, the Incident-vertex rule, fan normals and volume / 6.
 */
#ifndef TESS_ORACLE_H
#define TESS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Classification tolerance, polyhedron.rs:221-223. */
#define OR_TOLERANCE 1e-12
/* Points per bin, celery.rs:185-188. */
#define OR_CELL_DENSITY 1.25

/* Search modes of Cell::compute_voronoi_cell (interface.rs:275-278). */
enum {
    OR_MODE_SECURE = 0, /* shell walk with the security-radius stop (exact)   */
    OR_MODE_BRUTE = 1,  /* expand_all_no_radius: every point, celery.rs:971   */
    OR_MODE_RADIUS = 2  /* expand_all_in_radius(r), celery.rs:1023            */
};

/* Wall ids reported as neighbours for faces of the container box. */
enum {
    OR_WALL_XMIN = -1, OR_WALL_XMAX = -2, OR_WALL_YMIN = -3,
    OR_WALL_YMAX = -4, OR_WALL_ZMIN = -5, OR_WALL_ZMAX = -6
};

/* CeleryBounds + CeleryCellInfo (celery.rs:64-181). */
typedef struct {
    double xmin, xmax, ymin, ymax, zmin, zmax;
    double sx, sy, sz;   /* x/y/z_cell_size            */
    double ix, iy, iz;   /* x/y/z_inverse_cell_size    */
    int64_t cpd;         /* cells_per_dimension         */
} or_grid_info;

/* ---- plane / vector math (vector3.rs), exposed for known-answer tests ---- */
double or_dot(const double a[3], const double b[3]);                 /* vector3.rs:38  */
void or_cross(const double a[3], const double b[3], double out[3]); /* vector3.rs:44  */
/* Plane::halfway_from_origin_to, vector3.rs:223-239: out = {nx, ny, nz, offset} */
void or_halfway_from_origin_to(const double p[3], double out[4]);
/* Plane::build_from_non_unit_normal_and_point, vector3.rs:244-249 */
void or_plane_from_normal_and_point(const double n[3], const double p[3], double out[4]);
/* Plane::vector_location, vector3.rs:170-185: +1 Outside, 0 Incident, -1 Inside */
int or_vector_location(const double plane[4], const double v[3], double tol);
/* Plane::intersection, vector3.rs:213-219 */
void or_intersection(const double plane[4], const double a[3], const double b[3], double out[3]);

/* ---- grid (celery.rs) ---- */
int64_t or_cells_per_dimension(size_t n);                                    /* celery.rs:159-160 */
void or_grid_info_compute(const double* xyz, size_t n, or_grid_info* out);   /* celery.rs:81-181  */
int64_t or_axis_index(double x, double lo, double hi, double inv, int64_t cpd); /* celery.rs:269-282 */
void or_bin_ids(const double* xyz, size_t n, const or_grid_info* g, uint32_t* bins); /* celery.rs:342 */
/* Argsort by bin (stable by input index) + CSR delimiters, celery.rs:357-414. */
void or_sort_bins(const uint32_t* bins, size_t n, uint64_t nbins, uint32_t* sorted, uint32_t* delims);
/* Full search order (celery.rs:418-679), ties broken by (i, j, k) ascending.
 * Writes (2cpd-1)^3 entries; returns the count.  ijk has 3 ints per entry. */
size_t or_search_order(const or_grid_info* g, int32_t* ijk, double* dist);
/* Search-order key of one offset (celery.rs:423-427 applied to the gap counts). */
double or_gap_key(const or_grid_info* g, int32_t i, int32_t j, int32_t k);

/* ---- diagram ---- */
typedef struct or_diagram or_diagram;

/* Diagram constructor (the reference's private add_particle_with_group x N +
 * initialize, interface.rs:52-84).  lo/hi: container box; NULL => the
 * Diagram bounding box, which starts at the origin (interface.rs:53-54,
 * vector3.rs:263-288).  groups may be NULL (all zero). */
or_diagram* or_diagram_create(const double* xyz, size_t n, const uint32_t* groups,
                              const double* lo, const double* hi);
void or_diagram_destroy(or_diagram* d);
void or_diagram_grid(const or_diagram* d, or_grid_info* out);
void or_diagram_box(const or_diagram* d, double lo[3], double hi[3]);
const uint32_t* or_diagram_sorted(const or_diagram* d);   /* sorted_indices */
const uint32_t* or_diagram_delims(const or_diagram* d);   /* delimiters     */
const uint32_t* or_diagram_bins(const or_diagram* d);     /* cells          */

/* Per-cell work counters (for the algorithmic FLOP count). */
typedef struct {
    int64_t candidates;      /* bisectors built                              */
    int64_t classified;      /* vertex classifications                       */
    int64_t cuts;            /* planes that removed at least one vertex     */
    int64_t new_vertices;    /* intersection vertices created                */
    int64_t fan_triangles;   /* sum over final faces of (degree - 2)        */
    int64_t faces;           /* final faces                                  */
    double min_abs_sd_rel;   /* min |signed distance| / cell radius seen     */
} or_cell_stats;

/* One cell: compute_voronoi_cell (interface.rs:257-313) for the point with
 * original index i.  Returns 0 on success.  Output arrays are owned by the
 * result object. */
typedef struct or_cell or_cell;
or_cell* or_cell_compute(const or_diagram* d, size_t i, int mode, double radius,
                         int64_t target_group);
/* Cell for a point not in the diagram (get_cell_at_particle, interface.rs:211-232). */
or_cell* or_cell_compute_at(const or_diagram* d, const double p[3], int mode, double radius,
                            int64_t target_group);
void or_cell_destroy(or_cell* c);
double or_cell_volume(const or_cell* c);                     /* polyhedron.rs:838-855 */
int or_cell_nfaces(const or_cell* c);
/* Faces sorted by neighbour id: ids (original indices, walls -1..-6), areas
 * (interface.rs:408-410), face degrees. */
void or_cell_faces(const or_cell* c, int64_t* ids, double* areas, int32_t* degrees);
int or_cell_nvertices(const or_cell* c);
void or_cell_vertices(const or_cell* c, double* xyz);        /* polyhedron.rs:885-893 */
/* Vertex cycle of face f (in sorted-face order), polyhedron.rs:897-919. */
int or_cell_face_vertices(const or_cell* c, int f, double* xyz, int cap);
void or_cell_get_stats(const or_cell* c, or_cell_stats* s);

/* All cells, multi-threaded (nthreads <= 0: all cores).  Results in original
 * order: volumes[n], counts[n] (faces per cell).  Face lists are kept in the
 * result and read with or_all_faces(). */
typedef struct or_all or_all;
or_all* or_compute_all(const or_diagram* d, int mode, double radius, int64_t target_group,
                       int nthreads, const uint32_t* subset, size_t nsubset);
void or_all_destroy(or_all* a);
size_t or_all_total_faces(const or_all* a);
/* volumes/counts have one entry per computed cell (subset order, or original
 * order when subset is NULL); offs has ncells+1 entries. */
void or_all_results(const or_all* a, double* volumes, int64_t* offs, int64_t* ids, double* areas);
void or_all_stats(const or_all* a, or_cell_stats* total);
double or_all_seconds(const or_all* a);

/* ---- radius queries (celery.rs:682-855, interface.rs:348-365) ----
 * Batched over nq query positions q (AoS).  Each returns the total number of
 * results; offs (nq + 1 entries, nullable) gets CSR offsets and out the
 * results, as far as they fit in cap.  Point results are original indices. */
int or_check_cell_in_range(const or_diagram* d, const double p[3], double radius, int64_t i, int64_t j,
                           int64_t k);                                                /* celery.rs:708-748 */
size_t or_find_cells_in_radius(const or_diagram* d, const double* q, size_t nq, double radius, uint64_t* offs,
                               uint32_t* out, size_t cap);                            /* celery.rs:753-796 */
size_t or_find_neighbors_in_radius(const or_diagram* d, const double* q, size_t nq, double radius, int real_radius,
                                   uint64_t* offs, uint32_t* out, size_t cap);        /* celery.rs:802-855 */
size_t or_neighbor_cloud(const or_diagram* d, const double* q, size_t nq, double radius, int64_t target_group,
                         uint64_t* offs, uint32_t* out, size_t cap);                  /* interface.rs:348-365 */

#ifdef __cplusplus
}
#endif
#endif
