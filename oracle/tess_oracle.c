/*
 * tess_oracle.c -- CPU restatement (FP64) of The Tessellator's per-particle
 * Voronoi cell computation.  TEST INFRASTRUCTURE ONLY (checker + timed CPU
 * baseline); the product path never links it.
 *
 * Build: gcc -O3 -std=c11 -fopenmp -ffp-contract=off -fPIC -shared.
 * -ffp-contract=off keeps every multiply and add separately rounded, as the
 * reference's Float64 arithmetic (float.rs:80-118) is.
 *
 * Representation.  The reference keeps a half-edge mesh in free-list pools
 * (polyhedron.rs:204-217, pool.rs).  This restatement keeps, per face, the
 * cycle of its vertex indices (counter-clockwise seen from outside, the same
 * orientation as the reference's starting cube, polyhedron.rs:314-389).
 * Every vertex position is produced by the reference's own arithmetic:
 *   - the starting box translated by -site      polyhedron.rs:268-392, 859-867
 *   - bisector plane of site (origin) and p     vector3.rs:223-239
 *   - signed distance, 3-way location, tol      vector3.rs:170-210, polyhedron.rs:221
 *   - intersection(outside a, inside b)         vector3.rs:213-219, polyhedron.rs:566-571
 *   - Incident vertices are kept at their exact position (the reference copies
 *     them, polyhedron.rs:554-565)
 *   - fan weighted normal, volume = sum(anchor . wn) / 6, area = |wn| / 2
 *                                               polyhedron.rs:776-855, interface.rs:408-410
 */
#include "tess_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* vector / plane math (vector3.rs)                                          */
/* ------------------------------------------------------------------------ */
typedef struct { double x, y, z; } v3;
typedef struct { v3 n; double off; } pl_t;

static inline v3 mk(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
/* vector3.rs:38-40 (evaluated left to right) */
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* vector3.rs:44-50 */
static inline v3 vcross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 vscale(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); } /* :53 */
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); } /* :94  */
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); } /* :106 */
static inline double vmag(v3 a) { return sqrt(vdot(a, a)); }                       /* :69  */
static inline v3 vunit(v3 a) { return vscale(a, 1.0 / vmag(a)); }                  /* :75  */

/* build_from_normal_and_point, vector3.rs:229-239 */
static inline pl_t plane_np(v3 unit_normal, v3 point) {
    pl_t r; r.n = unit_normal; r.off = vdot(unit_normal, point); return r;
}
/* halfway_from_origin_to, vector3.rs:223-225 */
static inline pl_t halfway(v3 p) { return plane_np(vunit(p), vscale(p, 0.5)); }
/* signed_distance = offset_inverse - plane_offset, vector3.rs:191-210 */
static inline double sdist(const pl_t* pl, v3 v) { return vdot(pl->n, v) - pl->off; }
/* location, vector3.rs:170-178: +1 Outside, 0 Incident, -1 Inside */
static inline int loc_of(double sd, double tol) { return sd > tol ? 1 : (sd < -tol ? -1 : 0); }
/* intersection, vector3.rs:213-219 */
static inline v3 isect(const pl_t* pl, v3 a, v3 b) {
    double ao = vdot(pl->n, a), bo = vdot(pl->n, b);
    return vadd(a, vscale(vsub(b, a), (pl->off - ao) / (bo - ao)));
}

static v3 ld3(const double* p) { return mk(p[0], p[1], p[2]); }
static void st3(double* p, v3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

double or_dot(const double a[3], const double b[3]) { return vdot(ld3(a), ld3(b)); }
void or_cross(const double a[3], const double b[3], double out[3]) { st3(out, vcross(ld3(a), ld3(b))); }
void or_halfway_from_origin_to(const double p[3], double out[4]) {
    pl_t q = halfway(ld3(p)); st3(out, q.n); out[3] = q.off;
}
void or_plane_from_normal_and_point(const double n[3], const double p[3], double out[4]) {
    pl_t q = plane_np(vunit(ld3(n)), ld3(p)); st3(out, q.n); out[3] = q.off;
}
int or_vector_location(const double plane[4], const double v[3], double tol) {
    pl_t q; q.n = ld3(plane); q.off = plane[3];
    return loc_of(sdist(&q, ld3(v)), tol);
}
void or_intersection(const double plane[4], const double a[3], const double b[3], double out[3]) {
    pl_t q; q.n = ld3(plane); q.off = plane[3];
    st3(out, isect(&q, ld3(a), ld3(b)));
}

/* ------------------------------------------------------------------------ */
/* grid (celery.rs)                                                          */
/* ------------------------------------------------------------------------ */

/* `f64 as usize`: saturating, truncates toward zero, NaN -> 0 (float.rs:138-142). */
static uint64_t as_usize(double v) {
    if (!(v > 0.0)) return 0;
    if (v >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)v;
}

/* CeleryCellInfo::new, celery.rs:159-160: (n / 1.25).cbrt() as usize + 1 */
int64_t or_cells_per_dimension(size_t n) {
    return (int64_t)as_usize(cbrt((double)n / OR_CELL_DENSITY)) + 1;
}

/* CeleryBounds::new (celery.rs:81-125) + CeleryCellInfo::new (celery.rs:153-181) */
void or_grid_info_compute(const double* xyz, size_t n, or_grid_info* g) {
    memset(g, 0, sizeof(*g));
    if (n == 0) { g->cpd = 1; return; }
    double xmin = xyz[0], ymin = xyz[1], zmin = xyz[2];
    double xmax = xmin, ymax = ymin, zmax = zmin;
    for (size_t i = 0; i < n; ++i) {
        double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        if (x < xmin) xmin = x;
        if (x > xmax) xmax = x;
        if (y < ymin) ymin = y;
        if (y > ymax) ymax = y;
        if (z < zmin) zmin = z;
        if (z > zmax) zmax = z;
    }
    g->xmin = xmin; g->xmax = xmax; g->ymin = ymin; g->ymax = ymax; g->zmin = zmin; g->zmax = zmax;
    g->cpd = or_cells_per_dimension(n);
    double c = (double)g->cpd;
    g->sx = (xmax - xmin) / c; g->sy = (ymax - ymin) / c; g->sz = (zmax - zmin) / c;
    g->ix = c / (xmax - xmin); g->iy = c / (ymax - ymin); g->iz = c / (zmax - zmin);
}

/* get_{x,y,z}_cell_index, celery.rs:269-314 */
int64_t or_axis_index(double x, double lo, double hi, double inv, int64_t cpd) {
    if (x >= hi) return cpd - 1;
    uint64_t k = as_usize((x - lo) * inv);
    return k < (uint64_t)(cpd - 1) ? (int64_t)k : cpd - 1;
}

static inline void bin3(const or_grid_info* g, double x, double y, double z, int64_t* bx, int64_t* by, int64_t* bz) {
    *bx = or_axis_index(x, g->xmin, g->xmax, g->ix, g->cpd);
    *by = or_axis_index(y, g->ymin, g->ymax, g->iy, g->cpd);
    *bz = or_axis_index(z, g->zmin, g->zmax, g->iz, g->cpd);
}

/* get_cells + get_cell_from_indices, celery.rs:317-354 */
void or_bin_ids(const double* xyz, size_t n, const or_grid_info* g, uint32_t* bins) {
    int64_t c = g->cpd;
    for (size_t i = 0; i < n; ++i) {
        int64_t bx, by, bz;
        bin3(g, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], &bx, &by, &bz);
        bins[i] = (uint32_t)(bx * c * c + by * c + bz);
    }
}

/* get_sorted_indices + get_delimiters, celery.rs:357-414.  The reference's
 * sort_unstable_by leaves the within-bin order unspecified; this counting
 * sort keeps it ascending by input index. */
void or_sort_bins(const uint32_t* bins, size_t n, uint64_t nbins, uint32_t* sorted, uint32_t* delims) {
    memset(delims, 0, (nbins + 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) delims[bins[i] + 1]++;
    for (uint64_t b = 0; b < nbins; ++b) delims[b + 1] += delims[b];
    uint32_t* fill = (uint32_t*)malloc((nbins + 1) * sizeof(uint32_t));
    memcpy(fill, delims, (nbins + 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) sorted[fill[bins[i]]++] = (uint32_t)i;
    free(fill);
}

/* Search-order key, celery.rs:423-427, applied to the gap counts
 * (|offset| - 1, floored at 0) as get_search_order does (celery.rs:447-639). */
double or_gap_key(const or_grid_info* g, int32_t i, int32_t j, int32_t k) {
    if (i == 0 && j == 0 && k == 0) return -1.0;   /* celery.rs:438-443 */
    int32_t gi = i < 0 ? -i - 1 : (i > 0 ? i - 1 : 0);
    int32_t gj = j < 0 ? -j - 1 : (j > 0 ? j - 1 : 0);
    int32_t gk = k < 0 ? -k - 1 : (k > 0 ? k - 1 : 0);
    double a = (double)gi * g->sx, b = (double)gj * g->sy, c = (double)gk * g->sz;
    return a * a + b * b + c * c;
}

typedef struct { double key; int32_t i, j, k; } so_entry;

static int so_cmp(const void* pa, const void* pb) {
    const so_entry* a = (const so_entry*)pa;
    const so_entry* b = (const so_entry*)pb;
    if (a->key < b->key) return -1;
    if (a->key > b->key) return 1;
    if (a->i != b->i) return a->i < b->i ? -1 : 1;
    if (a->j != b->j) return a->j < b->j ? -1 : 1;
    if (a->k != b->k) return a->k < b->k ? -1 : 1;
    return 0;
}

/* All offsets within Chebyshev radius `cheb`, keeping those with key <= kmax
 * (kmax < 0: keep all), sorted by (key, i, j, k). */
static so_entry* build_order(const or_grid_info* g, int32_t cheb, double kmax, size_t* count) {
    size_t side = (size_t)(2 * cheb + 1);
    so_entry* e = (so_entry*)malloc(side * side * side * sizeof(so_entry));
    size_t m = 0;
    for (int32_t i = -cheb; i <= cheb; ++i)
        for (int32_t j = -cheb; j <= cheb; ++j)
            for (int32_t k = -cheb; k <= cheb; ++k) {
                double key = or_gap_key(g, i, j, k);
                if (kmax >= 0.0 && key > kmax) continue;
                e[m].key = key; e[m].i = i; e[m].j = j; e[m].k = k; ++m;
            }
    qsort(e, m, sizeof(so_entry), so_cmp);
    *count = m;
    return e;
}

size_t or_search_order(const or_grid_info* g, int32_t* ijk, double* dist) {
    size_t m;
    so_entry* e = build_order(g, (int32_t)(g->cpd - 1), -1.0, &m);
    for (size_t t = 0; t < m; ++t) {
        if (ijk) { ijk[3 * t] = e[t].i; ijk[3 * t + 1] = e[t].j; ijk[3 * t + 2] = e[t].k; }
        if (dist) dist[t] = e[t].key;
    }
    free(e);
    return m;
}

/* ------------------------------------------------------------------------ */
/* diagram (interface.rs:25-84)                                              */
/* ------------------------------------------------------------------------ */
struct or_diagram {
    size_t n;
    double* xyz;        /* original order */
    uint32_t* groups;
    double lo[3], hi[3];
    or_grid_info g;
    uint32_t* bins;
    uint32_t* sorted;
    uint32_t* delims;
    so_entry* table;    /* offsets with key <= table_kmax, sorted */
    size_t ntable;
    double table_kmax;
};

/* Offsets kept in the sorted table: every offset whose key is at most
 * (TABLE_GAPS * smallest bin side)^2.  Beyond it the walk continues shell by
 * shell (Chebyshev rings), which visits the same bins in a different order. */
#define TABLE_GAPS 5

or_diagram* or_diagram_create(const double* xyz, size_t n, const uint32_t* groups,
                              const double* lo, const double* hi) {
    if (n == 0 || n > 0xFFFFFFF0u) return NULL;
    or_diagram* d = (or_diagram*)calloc(1, sizeof(or_diagram));
    d->n = n;
    d->xyz = (double*)malloc(3 * n * sizeof(double));
    memcpy(d->xyz, xyz, 3 * n * sizeof(double));
    d->groups = (uint32_t*)calloc(n, sizeof(uint32_t));
    if (groups) memcpy(d->groups, groups, n * sizeof(uint32_t));
    if (lo && hi) {
        for (int a = 0; a < 3; ++a) { d->lo[a] = lo[a]; d->hi[a] = hi[a]; }
    } else {
        /* BoundingBox::default() is the origin; adjust_to_contain grows it
         * (interface.rs:53-54, vector3.rs:263-288). */
        for (int a = 0; a < 3; ++a) { d->lo[a] = 0.0; d->hi[a] = 0.0; }
        for (size_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) {
                double v = xyz[3 * i + a];
                if (v < d->lo[a]) d->lo[a] = v;
                if (v > d->hi[a]) d->hi[a] = v;
            }
    }
    or_grid_info_compute(xyz, n, &d->g);
    uint64_t c = (uint64_t)d->g.cpd, nb = c * c * c;
    d->bins = (uint32_t*)malloc(n * sizeof(uint32_t));
    d->sorted = (uint32_t*)malloc(n * sizeof(uint32_t));
    d->delims = (uint32_t*)malloc((nb + 1) * sizeof(uint32_t));
    or_bin_ids(xyz, n, &d->g, d->bins);
    or_sort_bins(d->bins, n, nb, d->sorted, d->delims);
    double m = d->g.sx;
    if (d->g.sy < m) m = d->g.sy;
    if (d->g.sz < m) m = d->g.sz;
    d->table_kmax = (TABLE_GAPS * m) * (TABLE_GAPS * m);
    int32_t cheb = TABLE_GAPS + 1;
    if (cheb > (int32_t)(c - 1)) cheb = (int32_t)(c - 1);
    /* Degenerate axes (zero extent) make every gap key zero along them; keep
     * the whole (small) grid in the table then. */
    if (!(m > 0.0)) { cheb = (int32_t)(c - 1); d->table_kmax = INFINITY; }
    d->table = build_order(&d->g, cheb, -1.0, &d->ntable);
    if (isfinite(d->table_kmax)) {
        size_t t = 0;
        while (t < d->ntable && d->table[t].key <= d->table_kmax) ++t;
        d->ntable = t;
    }
    return d;
}

void or_diagram_destroy(or_diagram* d) {
    if (!d) return;
    free(d->xyz); free(d->groups); free(d->bins); free(d->sorted); free(d->delims); free(d->table);
    free(d);
}
void or_diagram_grid(const or_diagram* d, or_grid_info* out) { *out = d->g; }
void or_diagram_box(const or_diagram* d, double lo[3], double hi[3]) {
    for (int a = 0; a < 3; ++a) { lo[a] = d->lo[a]; hi[a] = d->hi[a]; }
}
const uint32_t* or_diagram_sorted(const or_diagram* d) { return d->sorted; }
const uint32_t* or_diagram_delims(const or_diagram* d) { return d->delims; }
const uint32_t* or_diagram_bins(const or_diagram* d) { return d->bins; }

/* ------------------------------------------------------------------------ */
/* polyhedron (polyhedron.rs)                                                */
/* ------------------------------------------------------------------------ */
#define GROW(ptr, cap, need)                                                      \
    do {                                                                          \
        if ((size_t)(need) > (cap)) {                                             \
            size_t nc_ = (cap) ? (cap) : 64;                                      \
            while (nc_ < (size_t)(need)) nc_ *= 2;                                \
            (ptr) = realloc((ptr), nc_ * sizeof(*(ptr)));                         \
            (cap) = nc_;                                                          \
        }                                                                         \
    } while (0)

typedef struct {
    /* current polyhedron */
    v3* v; size_t cv; int nv;
    int64_t* fid; size_t cfid;
    int* fst; size_t cfst;
    int* fln; size_t cfln;
    int nf;
    int* cyc; size_t ccyc; int nc;
    /* rebuild buffers */
    v3* v2; size_t cv2;
    int64_t* fid2; size_t cfid2;
    int* fst2; size_t cfst2;
    int* fln2; size_t cfln2;
    int* cyc2; size_t ccyc2;
    /* scratch */
    double* sd; size_t csd;
    signed char* loc; size_t cloc;
    int* ec; size_t cec;        /* edge cache: (u, w, vertex) triples */
    int* seg; size_t cseg;      /* new-face segments: (entry, exit)   */
    int* tr; size_t ctr;        /* transitions of one face            */
    int* nxt; size_t cnxt;
    int* remap; size_t cremap;
    double* ang; size_t cang;
    int* ord; size_t cord;
} poly_t;

static void poly_free(poly_t* P) {
    free(P->v); free(P->fid); free(P->fst); free(P->fln); free(P->cyc);
    free(P->v2); free(P->fid2); free(P->fst2); free(P->fln2); free(P->cyc2);
    free(P->sd); free(P->loc); free(P->ec); free(P->seg); free(P->tr); free(P->nxt);
    free(P->remap); free(P->ang); free(P->ord);
    memset(P, 0, sizeof(*P));
}

/* build_cube (polyhedron.rs:268-392) then translate by -site (polyhedron.rs:859-867).
 * Vertex order FDL FDR FUR FUL BDL BDR BUR BUL; faces F R B L U D with the
 * vertex cycles the reference's half-edge targets give (polyhedron.rs:338-389;
 * edge DR belongs to face D, fixing the face-B typo at polyhedron.rs:383). */
static void poly_box(poly_t* P, const double lo[3], const double hi[3], v3 site) {
    static const int cyc[6][4] = {
        {3, 0, 1, 2}, /* F (y min): FUL FDL FDR FUR */
        {2, 1, 5, 6}, /* R (x max): FUR FDR BDR BUR */
        {6, 5, 4, 7}, /* B (y max): BUR BDR BDL BUL */
        {7, 4, 0, 3}, /* L (x min): BUL BDL FDL FUL */
        {2, 6, 7, 3}, /* U (z max): FUR BUR BUL FUL */
        {0, 4, 5, 1}  /* D (z min): FDL BDL BDR FDR */
    };
    static const int64_t ids[6] = {OR_WALL_YMIN, OR_WALL_XMAX, OR_WALL_YMAX,
                                   OR_WALL_XMIN, OR_WALL_ZMAX, OR_WALL_ZMIN};
    double x0 = lo[0] - site.x, x1 = hi[0] - site.x;
    double y0 = lo[1] - site.y, y1 = hi[1] - site.y;
    double z0 = lo[2] - site.z, z1 = hi[2] - site.z;
    GROW(P->v, P->cv, 8);
    P->v[0] = mk(x0, y0, z0); P->v[1] = mk(x1, y0, z0);
    P->v[2] = mk(x1, y0, z1); P->v[3] = mk(x0, y0, z1);
    P->v[4] = mk(x0, y1, z0); P->v[5] = mk(x1, y1, z0);
    P->v[6] = mk(x1, y1, z1); P->v[7] = mk(x0, y1, z1);
    P->nv = 8;
    GROW(P->fid, P->cfid, 6); GROW(P->fst, P->cfst, 6); GROW(P->fln, P->cfln, 6);
    GROW(P->cyc, P->ccyc, 24);
    for (int f = 0; f < 6; ++f) {
        P->fid[f] = ids[f]; P->fst[f] = 4 * f; P->fln[f] = 4;
        for (int t = 0; t < 4; ++t) P->cyc[4 * f + t] = cyc[f][t];
    }
    P->nf = 6; P->nc = 24;
}

static double poly_r2(const poly_t* P) {
    double r2 = 0.0;
    for (int i = 0; i < P->nv; ++i) {
        double q = vdot(P->v[i], P->v[i]);
        if (q > r2) r2 = q;
    }
    return r2;
}

static int edge_vertex(poly_t* P, int* ne, int o, int in, const pl_t* pl, or_cell_stats* st) {
    int a = o < in ? o : in, b = o < in ? in : o;
    for (int t = 0; t < *ne; ++t)
        if (P->ec[3 * t] == a && P->ec[3 * t + 1] == b) return P->ec[3 * t + 2];
    GROW(P->v, P->cv, (size_t)P->nv + 1);
    /* intersection(previous = outside vertex, current = inside vertex),
     * polyhedron.rs:566-571 */
    P->v[P->nv] = isect(pl, P->v[o], P->v[in]);
    GROW(P->ec, P->cec, 3 * (size_t)(*ne + 1));
    P->ec[3 * *ne] = a; P->ec[3 * *ne + 1] = b; P->ec[3 * *ne + 2] = P->nv;
    ++*ne;
    st->new_vertices++;
    return P->nv++;
}

/* Orders the vertices of the new face by angle around its normal; used only
 * when the segment chain is not a single simple cycle (degenerate cuts). */
static int angular_cycle(poly_t* P, const pl_t* pl, const int* pts, int m, int* out) {
    v3 c = mk(0, 0, 0);
    for (int t = 0; t < m; ++t) c = vadd(c, P->v[pts[t]]);
    c = vscale(c, 1.0 / (double)m);
    v3 n = pl->n;
    v3 h = fabs(n.x) < 0.6 ? mk(1, 0, 0) : mk(0, 1, 0);
    v3 e1 = vunit(vcross(n, h)), e2 = vcross(n, e1);
    GROW(P->ang, P->cang, (size_t)m); GROW(P->ord, P->cord, (size_t)m);
    for (int t = 0; t < m; ++t) {
        v3 q = vsub(P->v[pts[t]], c);
        P->ang[t] = atan2(vdot(q, e2), vdot(q, e1));
        P->ord[t] = pts[t];
    }
    for (int a = 1; a < m; ++a) { /* insertion sort, m is small */
        double ka = P->ang[a]; int va = P->ord[a]; int b = a - 1;
        while (b >= 0 && P->ang[b] > ka) { P->ang[b + 1] = P->ang[b]; P->ord[b + 1] = P->ord[b]; --b; }
        P->ang[b + 1] = ka; P->ord[b + 1] = va;
    }
    for (int t = 0; t < m; ++t) out[t] = P->ord[t];
    return m;
}

/* Clip by the half-space {x : n.x - off <= 0}: the intended behaviour of
 * Polyhedron::cut_with_plane (polyhedron.rs:438-642).  Returns 1 when at
 * least one vertex was Outside (a face for `id` was added), else 0. */
static int poly_cut(poly_t* P, const pl_t* pl, int64_t id, or_cell_stats* st, double rscale) {
    int nv = P->nv;
    GROW(P->sd, P->csd, (size_t)nv); GROW(P->loc, P->cloc, (size_t)nv);
    int any_out = 0;
    for (int i = 0; i < nv; ++i) {
        double s = sdist(pl, P->v[i]);
        P->sd[i] = s;
        int l = loc_of(s, OR_TOLERANCE);
        P->loc[i] = (signed char)l;
        any_out |= (l > 0);
        double r = fabs(s) / rscale;
        if (r < st->min_abs_sd_rel) st->min_abs_sd_rel = r;
    }
    st->classified += nv;
    if (!any_out) return 0;
    st->cuts++;

    int ne = 0, nseg = 0, nf2 = 0, nc2 = 0;
    GROW(P->fid2, P->cfid2, (size_t)P->nf + 1); GROW(P->fst2, P->cfst2, (size_t)P->nf + 1);
    GROW(P->fln2, P->cfln2, (size_t)P->nf + 1);
    for (int f = 0; f < P->nf; ++f) {
        int k = P->fln[f];
        const int* c = P->cyc + P->fst[f];
        int has_out = 0;
        for (int t = 0; t < k; ++t) has_out |= (P->loc[c[t]] > 0);
        int start = nc2;
        if (!has_out) {
            GROW(P->cyc2, P->ccyc2, (size_t)nc2 + (size_t)k);
            for (int t = 0; t < k; ++t) P->cyc2[nc2++] = c[t];
        } else {
            int ntr = 0;
            GROW(P->tr, P->ctr, 2 * (size_t)k);
            for (int t = 0; t < k; ++t) {
                int u = c[t], w = c[(t + 1) % k];
                int lu = P->loc[u], lw = P->loc[w];
                if (lu <= 0) { GROW(P->cyc2, P->ccyc2, (size_t)nc2 + 2); P->cyc2[nc2++] = u; }
                if (lu <= 0 && lw > 0) {            /* leaving the kept region */
                    int e = u;
                    if (lu < 0) { e = edge_vertex(P, &ne, w, u, pl, st); P->cyc2[nc2++] = e; }
                    P->tr[2 * ntr] = 0; P->tr[2 * ntr + 1] = e; ++ntr;
                } else if (lu > 0 && lw <= 0) {     /* re-entering it */
                    int e = w;
                    if (lw < 0) {
                        e = edge_vertex(P, &ne, u, w, pl, st);
                        GROW(P->cyc2, P->ccyc2, (size_t)nc2 + 1);
                        P->cyc2[nc2++] = e;
                    }
                    P->tr[2 * ntr] = 1; P->tr[2 * ntr + 1] = e; ++ntr;
                }
            }
            /* Pair each exit with the next entry: the new face runs entry -> exit. */
            int t0 = 0;
            while (t0 < ntr && P->tr[2 * t0] != 0) ++t0;
            for (int q = 0; q < ntr && t0 < ntr; q += 2) {
                int a = (t0 + q) % ntr, b = (t0 + q + 1) % ntr;
                if (P->tr[2 * a] != 0 || P->tr[2 * b] != 1) break;
                int ex = P->tr[2 * a + 1], en = P->tr[2 * b + 1];
                if (en != ex) {
                    GROW(P->seg, P->cseg, 2 * (size_t)(nseg + 1));
                    P->seg[2 * nseg] = en; P->seg[2 * nseg + 1] = ex; ++nseg;
                }
            }
        }
        if (nc2 - start >= 3) {
            P->fid2[nf2] = P->fid[f]; P->fst2[nf2] = start; P->fln2[nf2] = nc2 - start; ++nf2;
        } else {
            nc2 = start;
        }
    }

    /* The new face for `id`: chain entry -> exit segments. */
    if (nseg >= 3) {
        GROW(P->nxt, P->cnxt, (size_t)P->nv);
        for (int i = 0; i < P->nv; ++i) P->nxt[i] = -1;
        int ok = 1;
        for (int s = 0; s < nseg; ++s) {
            if (P->nxt[P->seg[2 * s]] != -1) ok = 0;
            P->nxt[P->seg[2 * s]] = P->seg[2 * s + 1];
        }
        GROW(P->cyc2, P->ccyc2, (size_t)nc2 + 2 * (size_t)nseg + 2);
        int start = nc2, cur = P->seg[0], steps = 0;
        if (ok) {
            do {
                P->cyc2[nc2++] = cur;
                cur = P->nxt[cur];
                ++steps;
            } while (cur != -1 && cur != P->seg[0] && steps <= nseg);
            if (cur != P->seg[0] || steps != nseg) ok = 0;
        }
        if (!ok) {
            nc2 = start;
            int m = 0;
            int* pts = P->cyc2 + start;
            for (int s = 0; s < 2 * nseg; ++s) {
                int v = P->seg[s], dup = 0;
                for (int t = 0; t < m; ++t) dup |= (pts[t] == v);
                if (!dup) pts[m++] = v;
            }
            if (m >= 3) nc2 = start + angular_cycle(P, pl, pts, m, pts);
        }
        if (nc2 - start >= 3) {
            GROW(P->fid2, P->cfid2, (size_t)nf2 + 1); GROW(P->fst2, P->cfst2, (size_t)nf2 + 1);
            GROW(P->fln2, P->cfln2, (size_t)nf2 + 1);
            P->fid2[nf2] = id; P->fst2[nf2] = start; P->fln2[nf2] = nc2 - start; ++nf2;
        } else {
            nc2 = start;
        }
    }

    /* Drop vertices no face references (clean_up_vertices / mark_sweep,
     * polyhedron.rs:645-730) and renumber. */
    GROW(P->remap, P->cremap, (size_t)P->nv);
    for (int i = 0; i < P->nv; ++i) P->remap[i] = -1;
    for (int t = 0; t < nc2; ++t) P->remap[P->cyc2[t]] = 0;
    GROW(P->v2, P->cv2, (size_t)P->nv);
    int m = 0;
    for (int i = 0; i < P->nv; ++i)
        if (P->remap[i] == 0) { P->remap[i] = m; P->v2[m++] = P->v[i]; }
    for (int t = 0; t < nc2; ++t) P->cyc2[t] = P->remap[P->cyc2[t]];

    /* swap buffers */
#define SWAP(a, b, ca, cb) do { void* t_ = (a); (a) = (b); (b) = t_; size_t u_ = (ca); (ca) = (cb); (cb) = u_; } while (0)
    SWAP(P->v, P->v2, P->cv, P->cv2);
    SWAP(P->fid, P->fid2, P->cfid, P->cfid2);
    SWAP(P->fst, P->fst2, P->cfst, P->cfst2);
    SWAP(P->fln, P->fln2, P->cfln, P->cfln2);
    SWAP(P->cyc, P->cyc2, P->ccyc, P->ccyc2);
#undef SWAP
    P->nv = m; P->nf = nf2; P->nc = nc2;
    return 1;
}

/* weighted_normal, polyhedron.rs:776-808: anchor = first vertex of the face,
 * sum of cross(v_i - anchor, v_{i+1} - anchor). */
static v3 face_wn(const poly_t* P, int f) {
    const int* c = P->cyc + P->fst[f];
    int k = P->fln[f];
    v3 a = P->v[c[0]], nrm = mk(0, 0, 0);
    v3 cur = vsub(P->v[c[1]], a);
    for (int t = 2; t < k; ++t) {
        v3 prev = cur;
        cur = vsub(P->v[c[t]], a);
        nrm = vadd(nrm, vcross(prev, cur));
    }
    return nrm;
}

/* ------------------------------------------------------------------------ */
/* cell driver (interface.rs:257-334, celery.rs:865-1075)                     */
/* ------------------------------------------------------------------------ */
struct or_cell {
    double volume;
    int nf, nv;
    int64_t* ids;
    double* areas;
    int32_t* deg;
    int32_t* fstart;   /* into fverts (vertex indices)       */
    int32_t* fverts;
    double* verts;     /* nv x 3, site-relative (as the reference leaves them) */
    or_cell_stats st;
};

/* Offsets > this margin times 4 R^2 can not cut: a bisector of a point at
 * distance |p| >= 2R lies outside every vertex. */
#define STOP_MARGIN (1.0 + 1e-6)

typedef struct {
    const or_diagram* d;
    poly_t* P;
    or_cell_stats* st;
    v3 site;
    int64_t self;       /* original index of the site, or -1 */
    int64_t group;      /* target group, or -1 */
    int mode;
    double radius;
    double r2;          /* current max |v|^2 */
    double rscale;
} walk_t;

/* Cut by every point of bin (bx,by,bz); returns nothing. */
static void visit_bin(walk_t* w, int64_t bx, int64_t by, int64_t bz) {
    const or_diagram* d = w->d;
    int64_t c = d->g.cpd;
    if (bx < 0 || bx >= c || by < 0 || by >= c || bz < 0 || bz >= c) return;
    uint64_t b = (uint64_t)(bx * c * c + by * c + bz);
    for (uint32_t s = d->delims[b]; s < d->delims[b + 1]; ++s) {
        uint32_t j = d->sorted[s];
        if ((int64_t)j == w->self) continue;                                   /* interface.rs:300-301 */
        if (w->group >= 0 && (int64_t)d->groups[j] != w->group) continue;     /* interface.rs:280-297 */
        v3 p = vsub(ld3(d->xyz + 3 * (size_t)j), w->site);                     /* interface.rs:322-326 */
        double p2 = vdot(p, p);
        if (p2 == 0.0) continue;   /* coincident point: the reference's NaN plane cuts nothing */
        if (w->mode == OR_MODE_SECURE && p2 >= 4.0 * w->r2 * STOP_MARGIN) continue;
        w->st->candidates++;
        pl_t pl = halfway(p);                                                  /* interface.rs:332 */
        if (poly_cut(w->P, &pl, (int64_t)j, w->st, sqrt(w->r2))) {
            w->r2 = poly_r2(w->P);
        }
    }
}

static void run_walk(walk_t* w) {
    const or_diagram* d = w->d;
    int64_t bx, by, bz;
    bin3(&d->g, w->site.x, w->site.y, w->site.z, &bx, &by, &bz);   /* celery.rs:882-902 */
    int limited = (w->mode == OR_MODE_RADIUS);
    /* phase 1: the sorted table (celery.rs:1029-1072) */
    for (size_t t = 0; t < d->ntable; ++t) {
        const so_entry* e = &d->table[t];
        if (limited && e->key > w->radius) return;                   /* celery.rs:1034-1036 */
        if (w->mode == OR_MODE_SECURE && e->key >= 4.0 * w->r2 * STOP_MARGIN) return;
        visit_bin(w, bx + e->i, by + e->j, bz + e->k);
    }
    if (!isfinite(d->table_kmax)) return;
    if (limited && d->table_kmax >= w->radius) return;
    /* phase 2: remaining offsets, Chebyshev ring by ring */
    double m = d->g.sx;
    if (d->g.sy < m) m = d->g.sy;
    if (d->g.sz < m) m = d->g.sz;
    int64_t c = d->g.cpd;
    for (int64_t s = 1; s <= c - 1; ++s) {
        double lb = (double)(s - 1) * m;
        lb = lb * lb;
        if (lb < d->table_kmax) lb = d->table_kmax;
        if (w->mode == OR_MODE_SECURE && lb >= 4.0 * w->r2 * STOP_MARGIN) return;
        if (limited && lb > w->radius) return;
        for (int64_t i = -s; i <= s; ++i)
            for (int64_t j = -s; j <= s; ++j)
                for (int64_t k = -s; k <= s; ++k) {
                    int64_t ai = i < 0 ? -i : i, aj = j < 0 ? -j : j, ak = k < 0 ? -k : k;
                    int64_t ch = ai > aj ? ai : aj;
                    if (ak > ch) ch = ak;
                    if (ch != s) continue;
                    double key = or_gap_key(&d->g, (int32_t)i, (int32_t)j, (int32_t)k);
                    if (key <= d->table_kmax) continue;       /* visited in phase 1 */
                    if (limited && key > w->radius) continue;
                    if (w->mode == OR_MODE_SECURE && key >= 4.0 * w->r2 * STOP_MARGIN) continue;
                    visit_bin(w, bx + i, by + j, bz + k);
                }
    }
}

static void finish_cell(poly_t* P, or_cell* out, int want_geometry) {
    /* compute_volume, polyhedron.rs:838-855 */
    double vol = 0.0;
    out->nf = P->nf;
    out->ids = (int64_t*)malloc((size_t)(P->nf ? P->nf : 1) * sizeof(int64_t));
    out->areas = (double*)malloc((size_t)(P->nf ? P->nf : 1) * sizeof(double));
    out->deg = (int32_t*)malloc((size_t)(P->nf ? P->nf : 1) * sizeof(int32_t));
    int* order = (int*)malloc((size_t)(P->nf ? P->nf : 1) * sizeof(int));
    double* ar = (double*)malloc((size_t)(P->nf ? P->nf : 1) * sizeof(double));
    for (int f = 0; f < P->nf; ++f) {
        v3 wn = face_wn(P, f);
        vol = vol + vdot(P->v[P->cyc[P->fst[f]]], wn);
        ar[f] = 0.5 * vmag(wn);                          /* interface.rs:408-410 */
        order[f] = f;
        out->st.fan_triangles += P->fln[f] - 2;
    }
    out->volume = vol / 6.0;
    out->st.faces = P->nf;
    /* faces reported sorted by neighbour id (walls first) */
    for (int a = 1; a < P->nf; ++a) {
        int oa = order[a], b = a - 1;
        while (b >= 0 && P->fid[order[b]] > P->fid[oa]) { order[b + 1] = order[b]; --b; }
        order[b + 1] = oa;
    }
    for (int t = 0; t < P->nf; ++t) {
        out->ids[t] = P->fid[order[t]];
        out->areas[t] = ar[order[t]];
        out->deg[t] = P->fln[order[t]];
    }
    if (want_geometry) {
        out->nv = P->nv;
        out->verts = (double*)malloc((size_t)(P->nv ? P->nv : 1) * 3 * sizeof(double));
        for (int i = 0; i < P->nv; ++i) st3(out->verts + 3 * i, P->v[i]);
        out->fstart = (int32_t*)malloc((size_t)(P->nf + 1) * sizeof(int32_t));
        out->fverts = (int32_t*)malloc((size_t)(P->nc ? P->nc : 1) * sizeof(int32_t));
        int q = 0;
        for (int t = 0; t < P->nf; ++t) {
            out->fstart[t] = q;
            int f = order[t];
            for (int u = 0; u < P->fln[f]; ++u) out->fverts[q++] = P->cyc[P->fst[f] + u];
        }
        out->fstart[P->nf] = q;
    }
    free(order);
    free(ar);
}

static void compute_into(const or_diagram* d, poly_t* P, v3 site, int64_t self, int mode,
                         double radius, int64_t group, or_cell* out, int want_geometry) {
    memset(&out->st, 0, sizeof(out->st));
    out->st.min_abs_sd_rel = INFINITY;
    poly_box(P, d->lo, d->hi, site);
    walk_t w;
    w.d = d; w.P = P; w.st = &out->st; w.site = site; w.self = self; w.group = group;
    w.mode = mode; w.radius = radius; w.r2 = poly_r2(P);
    w.rscale = sqrt(w.r2) > 0 ? sqrt(w.r2) : 1.0;
    run_walk(&w);
    finish_cell(P, out, want_geometry);
}

or_cell* or_cell_compute(const or_diagram* d, size_t i, int mode, double radius, int64_t target_group) {
    if (!d || i >= d->n) return NULL;
    or_cell* c = (or_cell*)calloc(1, sizeof(or_cell));
    poly_t P;
    memset(&P, 0, sizeof(P));
    compute_into(d, &P, ld3(d->xyz + 3 * i), (int64_t)i, mode, radius, target_group, c, 1);
    poly_free(&P);
    return c;
}

or_cell* or_cell_compute_at(const or_diagram* d, const double p[3], int mode, double radius,
                            int64_t target_group) {
    if (!d) return NULL;
    or_cell* c = (or_cell*)calloc(1, sizeof(or_cell));
    poly_t P;
    memset(&P, 0, sizeof(P));
    compute_into(d, &P, ld3(p), -1, mode, radius, target_group, c, 1);
    poly_free(&P);
    return c;
}

void or_cell_destroy(or_cell* c) {
    if (!c) return;
    free(c->ids); free(c->areas); free(c->deg); free(c->fstart); free(c->fverts); free(c->verts);
    free(c);
}
double or_cell_volume(const or_cell* c) { return c->volume; }
int or_cell_nfaces(const or_cell* c) { return c->nf; }
void or_cell_faces(const or_cell* c, int64_t* ids, double* areas, int32_t* degrees) {
    for (int t = 0; t < c->nf; ++t) {
        if (ids) ids[t] = c->ids[t];
        if (areas) areas[t] = c->areas[t];
        if (degrees) degrees[t] = c->deg[t];
    }
}
int or_cell_nvertices(const or_cell* c) { return c->nv; }
void or_cell_vertices(const or_cell* c, double* xyz) {
    memcpy(xyz, c->verts, (size_t)c->nv * 3 * sizeof(double));
}
int or_cell_face_vertices(const or_cell* c, int f, double* xyz, int cap) {
    if (f < 0 || f >= c->nf || !c->fstart) return -1;
    int k = c->fstart[f + 1] - c->fstart[f];
    for (int t = 0; t < k && t < cap; ++t) {
        int vi = c->fverts[c->fstart[f] + t];
        memcpy(xyz + 3 * t, c->verts + 3 * vi, 3 * sizeof(double));
    }
    return k;
}
void or_cell_get_stats(const or_cell* c, or_cell_stats* s) { *s = c->st; }

/* ------------------------------------------------------------------------ */
/* all cells                                                                  */
/* ------------------------------------------------------------------------ */
struct or_all {
    size_t ncells;
    double* vol;
    int64_t* cnt;
    int32_t* owner;     /* thread that stored the faces       */
    int64_t* at;        /* offset in that thread's buffer      */
    int nthr;
    int64_t** tid;      /* per-thread face ids                  */
    double** tar;       /* per-thread face areas                */
    size_t* tn;
    or_cell_stats total;
    double seconds;
};

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

or_all* or_compute_all(const or_diagram* d, int mode, double radius, int64_t target_group,
                       int nthreads, const uint32_t* subset, size_t nsubset) {
    if (!d) return NULL;
    or_all* a = (or_all*)calloc(1, sizeof(or_all));
    a->ncells = subset ? nsubset : d->n;
    size_t nc = a->ncells;
    a->vol = (double*)calloc(nc ? nc : 1, sizeof(double));
    a->cnt = (int64_t*)calloc(nc ? nc : 1, sizeof(int64_t));
    a->owner = (int32_t*)calloc(nc ? nc : 1, sizeof(int32_t));
    a->at = (int64_t*)calloc(nc ? nc : 1, sizeof(int64_t));
    int nthr = 1;
#ifdef _OPENMP
    nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
    a->nthr = nthr;
    a->tid = (int64_t**)calloc((size_t)nthr, sizeof(int64_t*));
    a->tar = (double**)calloc((size_t)nthr, sizeof(double*));
    a->tn = (size_t*)calloc((size_t)nthr, sizeof(size_t));
    or_cell_stats* per = (or_cell_stats*)calloc((size_t)nthr, sizeof(or_cell_stats));
    for (int t = 0; t < nthr; ++t) per[t].min_abs_sd_rel = INFINITY;
    double t0 = now_s();
#ifdef _OPENMP
#pragma omp parallel num_threads(nthr)
#endif
    {
        int me = 0;
#ifdef _OPENMP
        me = omp_get_thread_num();
#endif
        poly_t P;
        memset(&P, 0, sizeof(P));
        size_t cap = 0;
        or_cell cell;
        memset(&cell, 0, sizeof(cell));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (size_t q = 0; q < nc; ++q) {
            size_t i = subset ? subset[q] : q;
            if (i >= d->n) continue;
            compute_into(d, &P, ld3(d->xyz + 3 * i), (int64_t)i, mode, radius, target_group, &cell, 0);
            a->vol[q] = cell.volume;
            a->cnt[q] = cell.nf;
            a->owner[q] = me;
            a->at[q] = (int64_t)a->tn[me];
            size_t need = a->tn[me] + (size_t)cell.nf;
            if (need > cap) {
                size_t ncap = cap ? cap : 1024;
                while (ncap < need) ncap *= 2;
                a->tid[me] = (int64_t*)realloc(a->tid[me], ncap * sizeof(int64_t));
                a->tar[me] = (double*)realloc(a->tar[me], ncap * sizeof(double));
                cap = ncap;
            }
            memcpy(a->tid[me] + a->tn[me], cell.ids, (size_t)cell.nf * sizeof(int64_t));
            memcpy(a->tar[me] + a->tn[me], cell.areas, (size_t)cell.nf * sizeof(double));
            a->tn[me] = need;
            or_cell_stats* s = &per[me];
            s->candidates += cell.st.candidates; s->classified += cell.st.classified;
            s->cuts += cell.st.cuts; s->new_vertices += cell.st.new_vertices;
            s->fan_triangles += cell.st.fan_triangles; s->faces += cell.st.faces;
            if (cell.st.min_abs_sd_rel < s->min_abs_sd_rel) s->min_abs_sd_rel = cell.st.min_abs_sd_rel;
            free(cell.ids); free(cell.areas); free(cell.deg);
            cell.ids = NULL; cell.areas = NULL; cell.deg = NULL;
        }
        poly_free(&P);
    }
    a->seconds = now_s() - t0;
    a->total.min_abs_sd_rel = INFINITY;
    for (int t = 0; t < nthr; ++t) {
        a->total.candidates += per[t].candidates; a->total.classified += per[t].classified;
        a->total.cuts += per[t].cuts; a->total.new_vertices += per[t].new_vertices;
        a->total.fan_triangles += per[t].fan_triangles; a->total.faces += per[t].faces;
        if (per[t].min_abs_sd_rel < a->total.min_abs_sd_rel) a->total.min_abs_sd_rel = per[t].min_abs_sd_rel;
    }
    free(per);
    return a;
}

void or_all_destroy(or_all* a) {
    if (!a) return;
    for (int t = 0; t < a->nthr; ++t) { free(a->tid[t]); free(a->tar[t]); }
    free(a->tid); free(a->tar); free(a->tn);
    free(a->vol); free(a->cnt); free(a->owner); free(a->at);
    free(a);
}
size_t or_all_total_faces(const or_all* a) {
    size_t s = 0;
    for (size_t q = 0; q < a->ncells; ++q) s += (size_t)a->cnt[q];
    return s;
}
void or_all_results(const or_all* a, double* volumes, int64_t* offs, int64_t* ids, double* areas) {
    int64_t o = 0;
    for (size_t q = 0; q < a->ncells; ++q) {
        if (volumes) volumes[q] = a->vol[q];
        if (offs) offs[q] = o;
        int me = a->owner[q];
        for (int64_t t = 0; t < a->cnt[q]; ++t) {
            if (ids) ids[o + t] = a->tid[me][a->at[q] + t];
            if (areas) areas[o + t] = a->tar[me][a->at[q] + t];
        }
        o += a->cnt[q];
    }
    if (offs) offs[a->ncells] = o;
}
void or_all_stats(const or_all* a, or_cell_stats* total) { *total = a->total; }
double or_all_seconds(const or_all* a) { return a->seconds; }

/* ------------------------------------------------------------------------ */
/* radius queries (celery.rs:682-855, celery.rs:1023-1075, interface.rs:348-365) */
/* ------------------------------------------------------------------------ */

/* min_float / max_float, celery.rs:682-698: on ties and NaN the second
 * argument wins. */
static double rq_min(double a, double b) { return a < b ? a : b; }
static double rq_max(double a, double b) { return a > b ? a : b; }

static int64_t rq_gap(int64_t coord, int64_t index) {
    int64_t v = coord - index;
    if (v < 0) v = -v;
    v -= 1;
    return v < 0 ? 0 : v;
}

/* check_cell_in_range, celery.rs:708-748: the gap distance between the bin of
 * p and bin (i, j, k), squared, against radius * radius. */
int or_check_cell_in_range(const or_diagram* d, const double p[3], double radius, int64_t i, int64_t j,
                           int64_t k) {
    const or_grid_info* g = &d->g;
    int64_t xi = or_axis_index(p[0], g->xmin, g->xmax, g->ix, g->cpd);
    int64_t yi = or_axis_index(p[1], g->ymin, g->ymax, g->iy, g->cpd);
    int64_t zi = or_axis_index(p[2], g->zmin, g->zmax, g->iz, g->cpd);
    double a = (double)rq_gap(xi, i) * g->sx;
    double b = (double)rq_gap(yi, j) * g->sy;
    double c = (double)rq_gap(zi, k) * g->sz;
    double ds = a * a + b * b + c * c;
    return ds <= radius * radius;
}

/* find_cells_in_radius, celery.rs:753-796, for one position, in the
 * reference's i, j, k loop order: with m, counts the bins into *m and stores
 * them in out[*m..] as far as cap allows; with bins_tmp, collects them there. */
static void rq_cells(const or_diagram* d, const double p[3], double radius, uint32_t* out, size_t cap,
                     size_t* m, uint32_t** bins_tmp, size_t* bins_cap, size_t* nbins) {
    const or_grid_info* g = &d->g;
    double lx = rq_max(p[0] - radius, g->xmin), ly = rq_max(p[1] - radius, g->ymin);
    double lz = rq_max(p[2] - radius, g->zmin);
    double hx = rq_min(p[0] + radius, g->xmax), hy = rq_min(p[1] + radius, g->ymax);
    double hz = rq_min(p[2] + radius, g->zmax);
    int64_t i0 = or_axis_index(lx, g->xmin, g->xmax, g->ix, g->cpd);
    int64_t j0 = or_axis_index(ly, g->ymin, g->ymax, g->iy, g->cpd);
    int64_t k0 = or_axis_index(lz, g->zmin, g->zmax, g->iz, g->cpd);
    int64_t i1 = or_axis_index(hx, g->xmin, g->xmax, g->ix, g->cpd);
    int64_t j1 = or_axis_index(hy, g->ymin, g->ymax, g->iy, g->cpd);
    int64_t k1 = or_axis_index(hz, g->zmin, g->zmax, g->iz, g->cpd);
    *nbins = 0;
    for (int64_t i = i0; i <= i1; ++i)
        for (int64_t j = j0; j <= j1; ++j)
            for (int64_t k = k0; k <= k1; ++k) {
                if (!or_check_cell_in_range(d, p, radius, i, j, k)) continue;
                uint32_t b = (uint32_t)((i * g->cpd + j) * g->cpd + k);   /* celery.rs:317-325 */
                if (m) {
                    if (out && *m < cap) out[*m] = b;
                    ++*m;
                }
                if (bins_tmp) {
                    if (*nbins == *bins_cap) {
                        *bins_cap = *bins_cap ? 2 * *bins_cap : 64;
                        *bins_tmp = (uint32_t*)realloc(*bins_tmp, *bins_cap * sizeof(uint32_t));
                    }
                    (*bins_tmp)[(*nbins)++] = b;
                }
            }
}

size_t or_find_cells_in_radius(const or_diagram* d, const double* q, size_t nq, double radius, uint64_t* offs,
                               uint32_t* out, size_t cap) {
    size_t m = 0;
    for (size_t t = 0; t < nq; ++t) {
        if (offs) offs[t] = m;
        size_t nb = 0;
        rq_cells(d, q + 3 * t, radius, out, cap, &m, NULL, NULL, &nb);
    }
    if (offs) offs[nq] = m;
    return m;
}

/* distance_squared, celery.rs:700-702 */
static double rq_dist2(const double a[3], const double b[3]) {
    return (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
}

/* find_neighbors_in_cell_radius (celery.rs:802-818, real_radius = 0) and
 * find_neighbors_in_real_radius (celery.rs:825-855, real_radius = 1): the
 * points of the bins find_cells_in_radius returns, in bin order and
 * sorted_indices order within a bin; the real form keeps a point if its
 * squared distance is at most radius * radius. */
size_t or_find_neighbors_in_radius(const or_diagram* d, const double* q, size_t nq, double radius, int real_radius,
                                   uint64_t* offs, uint32_t* out, size_t cap) {
    size_t m = 0, bcap = 0, nb = 0;
    uint32_t* bins = NULL;
    const double r2 = radius * radius;
    for (size_t t = 0; t < nq; ++t) {
        if (offs) offs[t] = m;
        rq_cells(d, q + 3 * t, radius, NULL, 0, NULL, &bins, &bcap, &nb);
        for (size_t u = 0; u < nb; ++u)
            for (uint32_t s = d->delims[bins[u]]; s < d->delims[bins[u] + 1]; ++s) {
                uint32_t pi = d->sorted[s];
                if (real_radius && !(rq_dist2(q + 3 * t, d->xyz + 3 * (size_t)pi) <= r2)) continue;
                if (out && m < cap) out[m] = pi;
                ++m;
            }
    }
    if (offs) offs[nq] = m;
    free(bins);
    return m;
}

/* Cell::compute_neighbor_cloud, interface.rs:348-365: an ExpandingSearch
 * from the cell's position (celery.rs:882-902) walked by
 * expand_all_in_radius (celery.rs:1023-1075) over the whole search order
 * (every offset up to cpd - 1 per axis, sorted by key; ties by i, j, k), which
 * stops at the first key above the radius (a squared gap distance compared
 * with the unsquared radius); out-of-grid bins are skipped; then the points
 * of other groups are dropped when target_group >= 0. */
size_t or_neighbor_cloud(const or_diagram* d, const double* q, size_t nq, double radius, int64_t target_group,
                         uint64_t* offs, uint32_t* out, size_t cap) {
    const or_grid_info* g = &d->g;
    size_t ne = 0;
    so_entry* e = build_order(g, (int32_t)(g->cpd - 1), -1.0, &ne);
    size_t m = 0;
    const int64_t c = g->cpd;
    for (size_t t = 0; t < nq; ++t) {
        if (offs) offs[t] = m;
        const double* p = q + 3 * t;
        int64_t bx = or_axis_index(p[0], g->xmin, g->xmax, g->ix, c);
        int64_t by = or_axis_index(p[1], g->ymin, g->ymax, g->iy, c);
        int64_t bz = or_axis_index(p[2], g->zmin, g->zmax, g->iz, c);
        for (size_t u = 0; u < ne; ++u) {
            if (e[u].key > radius) break;                           /* celery.rs:1037-1039 */
            int64_t x = bx + e[u].i, y = by + e[u].j, z = bz + e[u].k;
            if (x < 0 || x >= c || y < 0 || y >= c || z < 0 || z >= c) continue;
            uint64_t b = (uint64_t)((x * c + y) * c + z);
            for (uint32_t s = d->delims[b]; s < d->delims[b + 1]; ++s) {
                uint32_t pi = d->sorted[s];
                if (target_group >= 0 && (int64_t)d->groups[pi] != target_group) continue;
                if (out && m < cap) out[m] = pi;
                ++m;
            }
        }
    }
    if (offs) offs[nq] = m;
    free(e);
    return m;
}
