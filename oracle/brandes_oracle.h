/*
 * CPU oracle for the Brandes hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-source Dijkstra with shortest-path
 * counting and Brandes dependency back-propagation (fast-bc, V=int, W=double):
 *   libfastbc/include/brandes/ExactBrandesBC.h:45-161
 *   libfastbc/include/brandes/DijkstraSSBrandesBC.h:45-147
 *   libfastbc/include/brandes/DijkstraClusterEvaluator.h:50-180
 *   libfastbc/include/brandes/ClusteredBrandesBC.h:141-166 (pivot scatter)
 * It keeps the reference's settle order ((dist, id) ascending), predecessor append
 * order and double arithmetic, so single-threaded results are bit-identical to the
 * reference; this is checked against the reference itself (oracle/_ref) and against
 * the reference unit tests' known answers.  Only the test suite, the smoke check and
 * the benchmark's CPU-baseline leg use it; the GPU library never does.
 *
 * Graph: CSR with row_ptr[n+1] (int64), col[m] (int32) and w[m] (double), each row's
 * neighbours in ascending id order (the std::map order of forwardStar).
 */
#ifndef FBC_BRANDES_ORACLE_H
#define FBC_BRANDES_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Exact BC over every source 0..n-1 (ExactBrandesBC::computeBC).  nthreads<=1 runs
 * the sources in order on one thread, as the reference does with -t 1. */
int orc_exact_bc(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                 double* out_bc, int nthreads);

/* Exact BC restricted to the listed sources (a bounded sample of the above). */
int orc_exact_bc_sources(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                         int64_t nsrc, const int32_t* sources, double* out_bc, int nthreads);

/* One source's dependency vector with dep[source] = 0
 * (DijkstraSSBrandesBC::singleSourceBrandes). */
int orc_single_source(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                      int32_t source, double* out_dep);

/* Debug dump of one source: dist (DBL_MAX when unreached), sigma, delta, the settle
 * order (returns its length) and the predecessor lists in append order, as CSR
 * (pred_off[n+1], pred[...]; pred may be NULL to query the total via pred_off[n]). */
int64_t orc_sssp_dump(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                      int32_t source, double* dist, double* sigma, double* delta,
                      int32_t* order, int64_t* pred_off, int32_t* pred);

/* Cluster evaluation (DijkstraClusterEvaluator::evaluateCluster): every listed cluster
 * vertex is a source; the forward star is restricted to cluster members
 * (SubGraph::forwardStar).  Adds intra-cluster BC into bc_accum (global ids) and writes,
 * for source i (in list order) and border j (ascending ids), bdist[i*nb+j] (0 when
 * unreached) and bsigma[i*nb+j]. */
int orc_cluster_eval(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                     int32_t nverts, const int32_t* verts, int32_t nborders, const int32_t* borders,
                     double* bc_accum, double* bdist, double* bsigma, int nthreads);

/* The k-means step of the pivot selection for one cluster (kmeans_oracle.c): np exact-class
 * pivots with normalized border vectors L[np*b] (lengths) and Cn[np*b] (counts) and class sizes
 * wt[np]; k = max(floor(np * kfrac), 1) centroids, at most max_iter + 1 Lloyd steps.  Writes the
 * distinct chosen pivots as indices into the class list (out_idx) with their weights (out_w), in
 * centroid order, and returns how many; out_idx and out_w have room for k entries. */
int32_t orc_kmeans_pivots(int32_t np, int32_t b, const double* L, const int32_t* Cn, const int32_t* wt,
                          double kfrac, int32_t max_iter, int32_t* out_idx, int32_t* out_w);

/* Pivot scatter (ClusteredBrandesBC.h:147-155): bc_accum[v] += dep_p[v] * card[p]. */
int orc_pivot_batch(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                    int64_t npiv, const int32_t* pivots, const double* card, double* bc_accum,
                    int nthreads);

#ifdef __cplusplus
}
#endif
#endif
