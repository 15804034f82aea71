/* The C ABI of include/tessellator.h used from plain C (and, compiled as
 * C++, from C++): a diagram of 1,000 points of a jittered 10 x 10 x 10
 * lattice in the unit box, every cell in each precision, the volume sum,
 * the neighbour CSR (sizes first, then the arrays), one cell's queries
 * against the bulk results, and error reporting.
 * Exit status: 0 success, 2 no CUDA device (create reports TESS_E_CUDA),
 * 1 a failed check. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "tessellator.h"

static int fail(const char* what) {
    char msg[512];
    tess_last_error(msg, sizeof msg);
    fprintf(stderr, "%s: %s\n", what, msg);
    return 1;
}

int main(void) {
    enum { M = 10, N = M * M * M };
    double* xyz = (double*)malloc(sizeof(double) * 3 * N);
    unsigned long long s = 12345;
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < M; ++j)
            for (int k = 0; k < M; ++k) {
                const int p = (i * M + j) * M + k;
                const int ijk[3] = {i, j, k};
                for (int a = 0; a < 3; ++a) {
                    s = s * 6364136223846793005ull + 1442695040888963407ull;   /* LCG (Knuth's MMIX constants) */
                    const double u = (double)(s >> 11) / 9007199254740992.0;
                    xyz[3 * p + a] = (ijk[a] + 0.5 + 0.3 * (u - 0.5)) / M;
                }
            }
    tess_config cfg;
    tess_config_default(&cfg);
    const double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    tess_diagram* d = NULL;
    tess_status st = tess_diagram_create(xyz, N, NULL, lo, hi, &cfg, &d);
    if (st == TESS_E_CUDA) {
        printf("no CUDA device: create reported TESS_E_CUDA\n");
        free(xyz);
        return 2;
    }
    if (st != TESS_OK) return fail("create");
    /* an argument error is reported, not aborted */
    if (tess_cell_volume(d, N + 5, NULL) != TESS_E_INVALID) return fail("bad cell index accepted");
    const tess_precision precs[3] = {TESS_PRECISION_FP64, TESS_PRECISION_FP32_GUARD, TESS_PRECISION_MIXED};
    const double tol[3] = {1e-11, 1e-6, 1e-11};
    double* vol = (double*)malloc(sizeof(double) * N);
    uint64_t* offs = (uint64_t*)malloc(sizeof(uint64_t) * (N + 1));
    for (int q = 0; q < 3; ++q) {
        if (tess_diagram_compute_all(d, precs[q], -1.0, -1) != TESS_OK) return fail("compute_all");
        if (tess_volumes(d, vol) != TESS_OK) return fail("volumes");
        double sum = 0.0;
        for (int i = 0; i < N; ++i) sum += vol[i];
        if (fabs(sum - 1.0) > tol[q]) {
            fprintf(stderr, "precision %d: volume sum %.17g\n", (int)precs[q], sum);
            return 1;
        }
        size_t total = 0;
        if (tess_neighbors_csr(d, offs, NULL, NULL, 0, &total) != TESS_OK) return fail("csr sizes");
        int32_t* nbr = (int32_t*)malloc(sizeof(int32_t) * total);
        double* area = (double*)malloc(sizeof(double) * total);
        if (tess_neighbors_csr(d, NULL, nbr, area, total, &total) != TESS_OK) return fail("csr");
        /* one cell's own queries agree with the bulk results */
        const size_t c = 417;
        double v = 0.0;
        if (tess_cell_volume(d, c, &v) != TESS_OK || v != vol[c]) return fail("cell volume");
        int32_t cn[64];
        size_t nn = 0;
        if (tess_cell_neighbors(d, c, cn, 64, &nn) != TESS_OK) return fail("cell neighbours");
        if (nn != offs[c + 1] - offs[c]) return fail("cell neighbour count");
        for (size_t f = 0; f < nn; ++f)
            if (cn[f] != nbr[offs[c] + f]) return fail("cell neighbour ids");
        printf("precision %d: %d cells, %zu faces, volume sum %.15f\n", (int)precs[q], N, total, sum);
        /* the same cells with the faces written into a pinned host pool */
        {
            const size_t cap = total + 64;
            void *pn = NULL, *pa = NULL;
            double* hv = (double*)malloc(sizeof(double) * N);
            uint64_t* hs = (uint64_t*)malloc(sizeof(uint64_t) * N);
            uint32_t* hc = (uint32_t*)malloc(sizeof(uint32_t) * N);
            size_t used = 0;
            if (tess_host_alloc(sizeof(int32_t) * cap, &pn) != TESS_OK ||
                tess_host_alloc(sizeof(double) * cap, &pa) != TESS_OK)
                return fail("host alloc");
            if (tess_diagram_compute_all_to_host(d, precs[q], -1.0, -1, hv, hs, hc, (int32_t*)pn, (double*)pa, cap,
                                                 &used) != TESS_OK)
                return fail("compute_all_to_host");
            for (int i = 0; i < N; ++i) {
                if (hv[i] != vol[i] || hc[i] != offs[i + 1] - offs[i]) return fail("to_host volume or count");
                for (uint32_t f = 0; f < hc[i]; ++f)
                    if (((int32_t*)pn)[hs[i] + f] != nbr[offs[i] + f] || ((double*)pa)[hs[i] + f] != area[offs[i] + f])
                        return fail("to_host faces");
            }
            if (tess_neighbors_csr(d, offs, NULL, NULL, 0, &total) != TESS_E_STATE) return fail("csr after to_host");
            tess_host_free(pn);
            tess_host_free(pa);
            free(hv);
            free(hs);
            free(hc);
        }
        free(nbr);
        free(area);
    }
    tess_diagram_destroy(d);
    free(vol);
    free(offs);
    free(xyz);
    printf("ok\n");
    return 0;
}
