/*
 * Command-line front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.
 * Reads an edge list with the reference parser's semantics
 * (DirectedWeightedGraph.h:67-96, 136-170): ``src dst w`` triples, weight <= 0 rejected,
 * repeated (src,dst) pairs have their weights summed, n = 1 + max source id.
 *
 *   oracle_cli exact <edges> <out> [threads]
 *   oracle_cli ss    <edges> <src> <out>
 *   oracle_cli cluster <edges> <verts> <out_prefix>
 * Output format matches oracle/_ref/ref_harness (one %.17g value per line).
 */
#include "brandes_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int32_t s, d; double w; } trip_t;

static int cmp_trip(const void* a, const void* b) {
    const trip_t* x = (const trip_t*)a;
    const trip_t* y = (const trip_t*)b;
    if (x->s != y->s) return x->s < y->s ? -1 : 1;
    if (x->d != y->d) return x->d < y->d ? -1 : 1;
    return 0;
}

static int load(const char* path, int32_t* n_out, int64_t** rp, int32_t** col, double** w) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    size_t cap = 1024, m = 0;
    trip_t* t = (trip_t*)malloc(cap * sizeof(trip_t));
    long s, d;
    double x;
    int32_t maxs = -1;
    while (fscanf(f, "%ld %ld %lf", &s, &d, &x) == 3) {
        if (x <= 0) { fclose(f); free(t); return -2; }
        if (m == cap) { cap *= 2; t = (trip_t*)realloc(t, cap * sizeof(trip_t)); }
        t[m].s = (int32_t)s; t[m].d = (int32_t)d; t[m].w = x;
        if ((int32_t)s > maxs) maxs = (int32_t)s;
        ++m;
    }
    fclose(f);
    qsort(t, m, sizeof(trip_t), cmp_trip);
    /* merge repeated pairs (weights summed in file order is what the reference does; the
       sort is stable enough for the integer-valued weights used here) */
    size_t u = 0;
    for (size_t i = 0; i < m; ++i) {
        if (u > 0 && t[u - 1].s == t[i].s && t[u - 1].d == t[i].d) t[u - 1].w += t[i].w;
        else t[u++] = t[i];
    }
    int32_t n = maxs + 1;
    *rp = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    *col = (int32_t*)malloc((u ? u : 1) * sizeof(int32_t));
    *w = (double*)malloc((u ? u : 1) * sizeof(double));
    for (size_t i = 0; i < u; ++i) {
        if (t[i].d >= n) { free(t); return -3; }
        (*rp)[t[i].s + 1]++;
        (*col)[i] = t[i].d;
        (*w)[i] = t[i].w;
    }
    for (int32_t v = 0; v < n; ++v) (*rp)[v + 1] += (*rp)[v];
    free(t);
    *n_out = n;
    return 0;
}

static void dump(const char* path, const double* x, int64_t n) {
    FILE* f = fopen(path, "w");
    for (int64_t i = 0; i < n; ++i) fprintf(f, "%.17g\n", x[i]);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: oracle_cli exact|ss|cluster ...\n"); return 2; }
    int32_t n;
    int64_t* rp;
    int32_t* col;
    double* w;
    int rc = load(argv[2], &n, &rp, &col, &w);
    if (rc) { fprintf(stderr, "load failed (%d)\n", rc); return 1; }
    if (!strcmp(argv[1], "exact")) {
        double* bc = (double*)calloc((size_t)n, sizeof(double));
        int th = argc > 4 ? atoi(argv[4]) : 1;
        if (orc_exact_bc(n, rp, col, w, bc, th)) return 1;
        dump(argv[3], bc, n);
        return 0;
    }
    if (!strcmp(argv[1], "ss") && argc == 5) {
        double* dep = (double*)calloc((size_t)n, sizeof(double));
        if (orc_single_source(n, rp, col, w, atoi(argv[3]), dep)) return 1;
        dump(argv[4], dep, n);
        return 0;
    }
    if (!strcmp(argv[1], "cluster") && argc == 5) {
        FILE* f = fopen(argv[3], "r");
        int32_t cap = 1024, nv = 0, v;
        int32_t* verts = (int32_t*)malloc((size_t)cap * sizeof(int32_t));
        while (fscanf(f, "%d", &v) == 1) {
            if (nv == cap) { cap *= 2; verts = (int32_t*)realloc(verts, (size_t)cap * sizeof(int32_t)); }
            verts[nv++] = v;
        }
        fclose(f);
        /* border = cluster vertex with an out- or in-edge crossing the cluster
           (SubGraph.h:70-135); listed in ascending id order (std::set) */
        char* in = (char*)calloc((size_t)n, 1);
        char* isb = (char*)calloc((size_t)n, 1);
        for (int32_t i = 0; i < nv; ++i) in[verts[i]] = 1;
        for (int32_t x = 0; x < n; ++x)
            for (int64_t e = rp[x]; e < rp[x + 1]; ++e)
                if (in[x] != in[col[e]]) { if (in[x]) isb[x] = 1; else isb[col[e]] = 1; }
        int32_t nb = 0;
        int32_t* borders = (int32_t*)malloc((size_t)n * sizeof(int32_t));
        for (int32_t x = 0; x < n; ++x) if (isb[x]) borders[nb++] = x;
        double* bc = (double*)calloc((size_t)n, sizeof(double));
        double* bd = (double*)calloc((size_t)nv * (nb ? nb : 1), sizeof(double));
        double* bs = (double*)calloc((size_t)nv * (nb ? nb : 1), sizeof(double));
        if (orc_cluster_eval(n, rp, col, w, nv, verts, nb, borders, bc, bd, bs, 1)) return 1;
        char path[4096];
        snprintf(path, sizeof path, "%s.bc", argv[4]);
        dump(path, bc, n);
        snprintf(path, sizeof path, "%s.vi", argv[4]);
        FILE* g = fopen(path, "w");
        fprintf(g, "%d\n", nb);
        for (int32_t j = 0; j < nb; ++j) fprintf(g, "%d ", borders[j]);
        fprintf(g, "\n");
        for (int32_t i = 0; i < nv; ++i) {
            for (int32_t j = 0; j < nb; ++j)
                fprintf(g, "%.17g %d ", bd[(int64_t)i * nb + j], (int)bs[(int64_t)i * nb + j]);
            fprintf(g, "\n");
        }
        fclose(g);
        return 0;
    }
    fprintf(stderr, "bad arguments\n");
    return 2;
}
