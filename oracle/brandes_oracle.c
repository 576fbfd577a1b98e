/*
 * CPU oracle for the Brandes hot path -- TEST INFRASTRUCTURE ONLY (see brandes_oracle.h).
 *
 * Restates, in C, the reference's _dijkstra_SSSP (ExactBrandesBC.h:97-161) and the
 * reverse visit-stack walk (ExactBrandesBC.h:73-90):
 *   - dist initialised to DBL_MAX (numeric_limits<W>::max, ExactBrandesBC.h:110);
 *   - a priority queue ordered by (dist, id) ascending (the std::set comparator,
 *     ExactBrandesBC.h:113-118), here an indexed binary heap: the pop order of a strict
 *     total order does not depend on the container;
 *   - strict improvement clears the predecessor list and sigma (ExactBrandesBC.h:142-149),
 *     equality appends the predecessor and adds its sigma (ExactBrandesBC.h:152-156);
 *   - the backward walk pops the settle stack and, for each predecessor v of w in append
 *     order, adds sigma[v]/sigma[w]*(1+delta[w]) to delta[v] (ExactBrandesBC.h:79-84),
 *     then adds delta[w] to BC[w] when w is not the source (ExactBrandesBC.h:86-89).
 */
#include "brandes_oracle.h"

#include <float.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int32_t n;
    double* dist;
    double* sigma;
    double* delta;
    int32_t* stack;   /* settle order */
    int32_t nstack;
    int32_t* heap;    /* indexed binary heap of vertex ids */
    int32_t* pos;     /* heap position or -1 */
    int32_t nheap;
    int32_t** pred;   /* per-vertex predecessor lists (append order) */
    int32_t* pcnt;
    int32_t* pcap;
} ws_t;

static ws_t* ws_new(int32_t n) {
    ws_t* s = (ws_t*)calloc(1, sizeof(ws_t));
    if (!s) return NULL;
    s->n = n;
    size_t nn = n > 0 ? (size_t)n : 1;
    s->dist = (double*)malloc(nn * sizeof(double));
    s->sigma = (double*)calloc(nn, sizeof(double));
    s->delta = (double*)calloc(nn, sizeof(double));
    s->stack = (int32_t*)malloc(nn * sizeof(int32_t));
    s->heap = (int32_t*)malloc(nn * sizeof(int32_t));
    s->pos = (int32_t*)malloc(nn * sizeof(int32_t));
    s->pred = (int32_t**)calloc(nn, sizeof(int32_t*));
    s->pcnt = (int32_t*)calloc(nn, sizeof(int32_t));
    s->pcap = (int32_t*)calloc(nn, sizeof(int32_t));
    if (!s->dist || !s->sigma || !s->delta || !s->stack || !s->heap || !s->pos || !s->pred ||
        !s->pcnt || !s->pcap)
        return NULL;
    for (size_t i = 0; i < nn; ++i) { s->dist[i] = DBL_MAX; s->pos[i] = -1; }
    return s;
}

static void ws_free(ws_t* s) {
    if (!s) return;
    for (int32_t i = 0; i < s->n; ++i) free(s->pred[i]);
    free(s->dist); free(s->sigma); free(s->delta); free(s->stack); free(s->heap);
    free(s->pos); free(s->pred); free(s->pcnt); free(s->pcap); free(s);
}

/* Restore the pristine state for every vertex the last source touched: all of them
 * were settled (a relaxed vertex enters the queue and is popped before it empties). */
static void ws_reset(ws_t* s) {
    for (int32_t i = 0; i < s->nstack; ++i) {
        int32_t v = s->stack[i];
        s->dist[v] = DBL_MAX;
        s->sigma[v] = 0.0;
        s->delta[v] = 0.0;
        s->pcnt[v] = 0;
    }
    s->nstack = 0;
}

static inline int less(const ws_t* s, int32_t a, int32_t b) {
    if (s->dist[a] == s->dist[b]) return a < b;
    return s->dist[a] < s->dist[b];
}

static void sift_up(ws_t* s, int32_t i) {
    int32_t v = s->heap[i];
    while (i > 0) {
        int32_t p = (i - 1) >> 1;
        if (!less(s, v, s->heap[p])) break;
        s->heap[i] = s->heap[p];
        s->pos[s->heap[i]] = i;
        i = p;
    }
    s->heap[i] = v;
    s->pos[v] = i;
}

static void sift_down(ws_t* s, int32_t i) {
    int32_t v = s->heap[i];
    for (;;) {
        int32_t l = 2 * i + 1;
        if (l >= s->nheap) break;
        int32_t c = l;
        if (l + 1 < s->nheap && less(s, s->heap[l + 1], s->heap[l])) c = l + 1;
        if (!less(s, s->heap[c], v)) break;
        s->heap[i] = s->heap[c];
        s->pos[s->heap[i]] = i;
        i = c;
    }
    s->heap[i] = v;
    s->pos[v] = i;
}

static int pred_push(ws_t* s, int32_t w, int32_t v) {
    if (s->pcnt[w] == s->pcap[w]) {
        int32_t cap = s->pcap[w] ? 2 * s->pcap[w] : 4;
        int32_t* p = (int32_t*)realloc(s->pred[w], (size_t)cap * sizeof(int32_t));
        if (!p) return -1;
        s->pred[w] = p;
        s->pcap[w] = cap;
    }
    s->pred[w][s->pcnt[w]++] = v;
    return 0;
}

/* Forward pass from src.  cid/my_c restrict the forward star to one cluster
 * (cid == NULL: the whole graph). */
static int sssp(const int64_t* rp, const int32_t* col, const double* w, const int32_t* cid,
                int32_t my_c, int32_t src, ws_t* s) {
    s->nheap = 0;
    s->nstack = 0;
    s->sigma[src] = 1.0;
    s->dist[src] = 0.0;
    s->heap[s->nheap++] = src;
    s->pos[src] = 0;
    while (s->nheap > 0) {
        int32_t v = s->heap[0];
        s->pos[v] = -1;
        if (--s->nheap > 0) {
            s->heap[0] = s->heap[s->nheap];
            sift_down(s, 0);
        }
        s->stack[s->nstack++] = v;
        for (int64_t e = rp[v]; e < rp[v + 1]; ++e) {
            int32_t x = col[e];
            if (cid && cid[x] != my_c) continue;
            double nd = s->dist[v] + w[e];
            if (nd < s->dist[x]) {
                s->dist[x] = nd;
                if (s->pos[x] < 0) {
                    s->heap[s->nheap] = x;
                    s->pos[x] = s->nheap++;
                }
                sift_up(s, s->pos[x]);
                s->pcnt[x] = 0;
                s->sigma[x] = 0.0;
            }
            if (nd == s->dist[x]) {
                if (pred_push(s, x, v)) return -1;
                s->sigma[x] += s->sigma[v];
            }
        }
    }
    return 0;
}

/* Backward walk; bc (may be NULL) receives delta[w] for w != src, in pop order. */
static void backward(int32_t src, ws_t* s, double* bc) {
    for (int32_t i = s->nstack - 1; i >= 0; --i) {
        int32_t x = s->stack[i];
        for (int32_t k = 0; k < s->pcnt[x]; ++k) {
            int32_t v = s->pred[x][k];
            double c = s->sigma[v] / s->sigma[x] * (1.0 + s->delta[x]);
            s->delta[v] += c;
        }
        if (bc && x != src) bc[x] += s->delta[x];
    }
}

static int run_sources(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                       int64_t nsrc, const int32_t* sources, double* out_bc, int nthreads) {
    if (nthreads <= 1) {
        ws_t* s = ws_new(n);
        if (!s) return -1;
        for (int64_t i = 0; i < nsrc; ++i) {
            int32_t src = sources ? sources[i] : (int32_t)i;
            if (sssp(rp, col, w, NULL, 0, src, s)) { ws_free(s); return -1; }
            backward(src, s, out_bc);
            ws_reset(s);
        }
        ws_free(s);
        return 0;
    }
    int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        ws_t* s = ws_new(n);
        double* part = (double*)calloc(n > 0 ? (size_t)n : 1, sizeof(double));
        if (!s || !part) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
            err = 1;
        } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int64_t i = 0; i < nsrc; ++i) {
                int32_t src = sources ? sources[i] : (int32_t)i;
                if (sssp(rp, col, w, NULL, 0, src, s)) {
                    err = 1;
                    continue;
                }
                backward(src, s, part);
                ws_reset(s);
            }
#ifdef _OPENMP
#pragma omp critical
#endif
            for (int32_t v = 0; v < n; ++v) out_bc[v] += part[v];
        }
        free(part);
        ws_free(s);
    }
    return err ? -1 : 0;
}

int orc_exact_bc(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                 double* out_bc, int nthreads) {
    return run_sources(n, rp, col, w, n, NULL, out_bc, nthreads);
}

int orc_exact_bc_sources(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                         int64_t nsrc, const int32_t* sources, double* out_bc, int nthreads) {
    return run_sources(n, rp, col, w, nsrc, sources, out_bc, nthreads);
}

int orc_single_source(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                      int32_t source, double* out_dep) {
    ws_t* s = ws_new(n);
    if (!s) return -1;
    memset(out_dep, 0, (size_t)n * sizeof(double));
    int rc = sssp(rp, col, w, NULL, 0, source, s);
    if (!rc) backward(source, s, out_dep);
    ws_free(s);
    return rc;
}

int64_t orc_sssp_dump(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                      int32_t source, double* dist, double* sigma, double* delta,
                      int32_t* order, int64_t* pred_off, int32_t* pred) {
    ws_t* s = ws_new(n);
    if (!s) return -1;
    if (sssp(rp, col, w, NULL, 0, source, s)) { ws_free(s); return -1; }
    backward(source, s, NULL);
    int64_t tot = 0;
    for (int32_t v = 0; v < n; ++v) {
        if (dist) dist[v] = s->dist[v];
        if (sigma) sigma[v] = s->sigma[v];
        if (delta) delta[v] = s->delta[v];
        if (pred_off) pred_off[v] = tot;
        if (pred)
            for (int32_t k = 0; k < s->pcnt[v]; ++k) pred[tot + k] = s->pred[v][k];
        tot += s->pcnt[v];
    }
    if (pred_off) pred_off[n] = tot;
    if (order) memcpy(order, s->stack, (size_t)s->nstack * sizeof(int32_t));
    int64_t cnt = s->nstack;
    ws_free(s);
    return cnt;
}

int orc_cluster_eval(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                     int32_t nverts, const int32_t* verts, int32_t nb, const int32_t* borders,
                     double* bc_accum, double* bdist, double* bsigma, int nthreads) {
    int32_t* cid = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    if (!cid) return -1;
    for (int32_t v = 0; v < n; ++v) cid[v] = -1;
    for (int32_t i = 0; i < nverts; ++i) cid[verts[i]] = 0;
    int err = 0;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        ws_t* s = ws_new(n);
        double* part = (double*)calloc(n > 0 ? (size_t)n : 1, sizeof(double));
        if (!s || !part) {
            err = 1;
        } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int32_t i = 0; i < nverts; ++i) {
                int32_t src = verts[i];
                if (sssp(rp, col, w, cid, 0, src, s)) { err = 1; continue; }
                /* DijkstraClusterEvaluator.h:166-177: border (dist or 0, sigma) */
                for (int32_t j = 0; j < nb; ++j) {
                    int32_t b = borders[j];
                    double d = s->dist[b];
                    if (bdist) bdist[(int64_t)i * nb + j] = d != DBL_MAX ? d : 0.0;
                    if (bsigma) bsigma[(int64_t)i * nb + j] = s->sigma[b];
                }
                backward(src, s, nthreads == 1 ? bc_accum : part);
                ws_reset(s);
            }
            if (nthreads > 1) {
#ifdef _OPENMP
#pragma omp critical
#endif
                for (int32_t i = 0; i < nverts; ++i) bc_accum[verts[i]] += part[verts[i]];
            }
        }
        free(part);
        ws_free(s);
    }
    free(cid);
    return err ? -1 : 0;
}

int orc_pivot_batch(int32_t n, const int64_t* rp, const int32_t* col, const double* w,
                    int64_t npiv, const int32_t* pivots, const double* card, double* bc_accum,
                    int nthreads) {
    int err = 0;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        ws_t* s = ws_new(n);
        double* dep = (double*)calloc(n > 0 ? (size_t)n : 1, sizeof(double));
        double* part = (double*)calloc(n > 0 ? (size_t)n : 1, sizeof(double));
        if (!s || !dep || !part) {
            err = 1;
        } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int64_t p = 0; p < npiv; ++p) {
                int32_t src = pivots[p];
                if (sssp(rp, col, w, NULL, 0, src, s)) { err = 1; continue; }
                backward(src, s, dep);
                double* tgt = nthreads == 1 ? bc_accum : part;
                for (int32_t v = 0; v < n; ++v) {
                    tgt[v] += dep[v] * card[p];
                    dep[v] = 0.0;
                }
                ws_reset(s);
            }
            if (nthreads > 1) {
#ifdef _OPENMP
#pragma omp critical
#endif
                for (int32_t v = 0; v < n; ++v) bc_accum[v] += part[v];
            }
        }
        free(part);
        free(dep);
        ws_free(s);
    }
    return err ? -1 : 0;
}
