/*
 * fbc_gpu.h -- C ABI of the GB300 Brandes engine (libfbcgpu.so).
 *
 * The reference fast-bc has no C ABI or FFI: its hot path sits behind three C++
 * template interfaces (V=int, W=double in the fbc CLI, main.cpp:25-31):
 *   IBrandesBC<V,W>::computeBC               libfastbc/include/brandes/IBrandesBC.h:24
 *   ISSBrandesBC<V,W>::singleSourceBrandes    libfastbc/include/brandes/ISSBrandesBC.h:26-28
 *   IClusterEvaluator<V,W>::evaluateCluster   libfastbc/include/brandes/IClusterEvaluator.h:33-36
 * Each entry point below is what an implementation of one of those interfaces calls
 * (the headers under include/fastbc_gpu hold the C++ classes that implement them on top of this ABI).
 * Plain pointers and sizes only; every call returns FBC_OK or an FBC_ERR_* status and
 * never throws; fbc_last_error_string() describes the last failure of the calling thread.
 * Calls are serialised by an internal mutex, so OpenMP worker threads may call in
 * concurrently (the reference calls singleSourceBrandes from OMP workers,
 * ClusteredBrandesBC.h:143-148).  Each call makes the device given to fbc_gpu_init current for
 * its duration and gives the calling thread its own current device back on return.
 *
 * Graphs: directed, positive integer weights (the README's input contract), vertex ids
 * 0..n-1, each CSR row sorted ascending without repeats (the std::map order of
 * IGraph::forwardStar, IGraph.h:39).  Distances are int32 on the device: a graph whose
 * (n-1)*max_weight reaches 2^31-1 is rejected with FBC_ERR_RANGE.
 */
#ifndef FBC_GPU_H
#define FBC_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FBC_OK 0
#define FBC_ERR_INVALID_ARG 1   /* bad pointer/size/id, weight <= 0, unsorted row ...   */
#define FBC_ERR_CUDA 2          /* a CUDA runtime call failed                           */
#define FBC_ERR_OOM 3           /* device allocation failed                             */
#define FBC_ERR_ITER_LIMIT 4    /* a device loop hit its iteration bound                */
#define FBC_ERR_RANGE 5         /* weights or distances do not fit the int32 device form */
#define FBC_ERR_SIGMA_OVERFLOW 6 /* a shortest-path count exceeded 2^64-1                */
#define FBC_ERR_NOT_INIT 7      /* fbc_gpu_init has not been called                     */
#define FBC_ERR_QUEUE 8         /* a device work queue overflowed (internal error)      */
#define FBC_ERR_HASH 9          /* two different border vectors share one 64-bit hash in the
                                   class grouping (reported, never merged)               */

/* dependency precision (the "precision" form of the engine) */
#define FBC_PREC_FP64 0   /* plain: FP64 dependency arithmetic                          */
#define FBC_PREC_FP32C 1  /* FP32 double-float (two-sum compensated) dependency; FP64 only
                             for sigma ratios above 2^24 and the cross-source BC sum     */

/* schedule */
#define FBC_SCHED_PLAIN 0    /* one source per thread block, per-source state in HBM     */
#define FBC_SCHED_BATCHED 1  /* persistent mixed launch: one source per warp with state in
                                shared memory for small segments, per block otherwise    */

typedef struct fbc_graph_s* fbc_graph;

/* Per-call measurements (all optional: pass NULL). */
typedef struct {
    double kernel_ms;        /* device time of the compute kernels, CUDA events on the
                                library stream                                            */
    double wall_ms;          /* host wall time of the whole call, copies included         */
    int64_t h2d_bytes;       /* host->device bytes copied by the call                     */
    int64_t d2h_bytes;       /* device->host bytes copied by the call                     */
    int64_t units;           /* (segment, source) units processed                          */
    double relaxations;      /* sum over units of the segment's edge count (TEPS numerator) */
    int32_t launches;        /* kernels launched by the call                               */
    int32_t slots;           /* concurrent block slots of the block-per-source kernel      */
    double warp_ms;          /* device time of the warp-per-source kernel (CUDA events)    */
    double block_ms;         /* device time of the block-per-source kernel (CUDA events)   */
    double warp_bytes;       /* algorithmic bytes of the warp kernel's units               */
    double block_bytes;      /* algorithmic bytes of the block kernel's units; one unit on a
                                segment of n vertices and m edges counts 40*m + 52*n bytes  */
    int64_t warp_units;
    int64_t block_units;
    int32_t group;           /* sources per block of the frontier kernel (0: not launched)  */
    int32_t retries;         /* units recomputed by the plain kernel with wider path counts */
} fbc_stats;

/* Library lifetime.  fbc_gpu_init selects the device and creates the library stream. */
int fbc_gpu_init(int device);
int fbc_gpu_shutdown(void);
const char* fbc_last_error_string(void);

/* Tuning knobs (the autotuner sets the first ones); values outside a knob's range are clamped:
 *   "delta"            bucket width of the distance pass (0 = 4 x the graph's mean weight)
 *   "block_threads"    block size of the plain kernel (32..1024)
 *   "frontier_threads" block size of the frontier kernel (32..128; above 128 the wide form)
 *   "group"            sources per frontier block: 1, 2, 4, or 0 = automatic (others refused)
 *   "chunk_max"        sources per work item of the shared-memory kernel
 *   "wide_n"           segments of at least this many vertices use the wide frontier blocks
 *   "wide_threads"     block size of the wide frontier blocks (64..1024, a multiple of 32; above 512
 *                      a 1024-thread form with 64 registers per thread; default 1024)
 *   "wide_kv"          level entries per lane of the 1024-thread form: 1 (default) or 2
 *   "bc_sweep"         1 (default): a one-segment launch of one source per block adds BC in its
 *                      restore sweep (coalesced, segment order); 0: in the dependency pass
 *   "adj4"             1 (default): wide one-source blocks on a relabelled graph with fewer than 2^24
 *                      vertices and weights below 256 read its adjacency packed in 4 bytes; 0: 8 bytes
 *   "pull_count"       1 (default): on a relabelled graph whose every edge has a reverse (weights
 *                      below 256) the frontier kernel counts each vertex's tight in-edges from its
 *                      own row and the reverse weights, without atomics; 0: atomic counts
 *   "source_order"     1 (default): the sources of a batched call on a relabelled graph run in its
 *                      locality order (sources running at once start near each other); 0: as given
 *   "warp_max_n"       largest segment run warp-per-source in shared memory
 *   "order_min_n"      batched runs relabel graphs of at least this many vertices for memory
 *                      locality (outputs stay in input ids)
 *   "csr_device_min_m" edge lists of at least this many edges are built into a CSR on the device
 *   "iter_mult"        distance-pass rounds are capped at iter_mult * (n + 2); 0 makes every unit
 *                      stop at once with FBC_ERR_ITER_LIMIT (a host-side way to exercise the
 *                      bounded-loop error path)
 *   "ws_budget_mb"     cap of the block kernels' workspace (0 = 60% of the free device memory)
 *   "debug_sched"      schedule of fbc_sssp_debug (0 plain, else batched)
 *   "scratch_keep_mb"  per-call scratch (graph builds, text parsing, class grouping) comes from a
 *                      stream-ordered memory pool that keeps up to this many MiB (default 8192)
 * Unknown key -> FBC_ERR_INVALID_ARG. */
int fbc_set_option(const char* key, int64_t value);
int fbc_get_option(const char* key, int64_t* value);

/* Device graph from CSR (row_ptr[n+1], col[m], w[m], double weights as in W=double).
 * Replaces building a DirectedWeightedGraph for the GPU (DirectedWeightedGraph.h:67-170). */
int fbc_graph_upload(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* w,
                     fbc_graph* out);

/* Device graph from an edge list with the reference parser's rules
 * (DirectedWeightedGraph.h:67-96, 136-170): weight <= 0 rejected, repeated (src,dst)
 * pairs have their weights summed, n = 1 + max source id (a destination id >= n, which
 * is undefined behaviour in the reference, is rejected). */
int fbc_graph_from_edges(int64_t count, const int32_t* src, const int32_t* dst, const double* w,
                         fbc_graph* out);

/* Device graph from edge-list text (the bytes of the file fbc reads,
 * DirectedWeightedGraph(std::istream&), DirectedWeightedGraph.h:67-96): whitespace-separated
 * triples "src dst weight", ids read as int and weights as double exactly as operator>> does
 * (correctly rounded; a weight that overflows a double ends the reading there, as the
 * reference's loop does), then the rules of fbc_graph_from_edges.  Tokenised and parsed on the
 * device; len < 2 GiB.  FBC_ERR_INVALID_ARG for a weight <= 0 or not a number ("Edge weight
 * must be greater than zero"), an id token that is not a decimal int32, or text that ends
 * inside a triple (the last two are undefined behaviour in the reference).
 * st (optional): kernel_ms = device time of the tokenising and parsing kernels, wall_ms = the
 * whole call (copy, parse, CSR build, host mirror), h2d/d2h bytes, launches of the parse. */
int fbc_graph_from_text(const char* text, int64_t len, fbc_graph* out, fbc_stats* st);

int fbc_graph_info(fbc_graph g, int32_t* n, int64_t* m);
/* Download the CSR (row_ptr[n+1], col[m], w[m]); any pointer may be NULL. */
int fbc_graph_download(fbc_graph g, int64_t* row_ptr, int32_t* col, double* w);
int fbc_graph_free(fbc_graph g);

/* Exact BC over every source (ExactBrandesBC::computeBC, ExactBrandesBC.h:45-95).
 * out_bc[n] is overwritten. */
int fbc_exact_bc(fbc_graph g, int precision, int sched, double* out_bc, fbc_stats* st);

/* One source's dependency vector, dep[source] = 0
 * (DijkstraSSBrandesBC::singleSourceBrandes, DijkstraSSBrandesBC.h:45-81).  out_dep[n]. */
int fbc_single_source(fbc_graph g, int32_t source, int precision, double* out_dep,
                      fbc_stats* st);

/* Batched pivot dependencies: out_bc_accum[v] += sum_p cards[p] * dep_p[v]
 * (the pivot loop of ClusteredBrandesBC.h:141-155; cards may be NULL for all-ones). */
int fbc_sssp_dependency_batch(fbc_graph g, int64_t count, const int32_t* sources,
                              const double* cards, int precision, int sched,
                              double* out_bc_accum, fbc_stats* st);

/* Batched cluster evaluation (DijkstraClusterEvaluator::evaluateCluster,
 * DijkstraClusterEvaluator.h:50-180) for nclusters clusters at once.  Cluster c holds
 * cluster_vertices[cluster_off[c] .. cluster_off[c+1]); each of them is a source over the
 * cluster's induced subgraph (SubGraph::forwardStar, SubGraph.h:165-176).
 * Borders: border_off/borders give each cluster's border vertices in ascending id order
 * (SubGraph::borders); pass border_off = NULL to have them computed (a vertex with an in-
 * or out-edge crossing the cluster, SubGraph.h:70-135).
 * Outputs: out_intra_bc[n] += intra-cluster BC (global ids); for the i-th vertex of
 * cluster c and its j-th border: out_border_dist[E_c + i*nb_c + j] (0 when unreached) and
 * out_border_sigma[...], E_c = sum_{c'<c} n_c' * nb_c'.  The caller sizes the border outputs
 * with fbc_cluster_border_count; either may be NULL. */
int fbc_cluster_border_count(fbc_graph g, int32_t nclusters, const int64_t* cluster_off,
                             const int32_t* cluster_vertices, const int64_t* border_off,
                             int64_t* out_nborders_total, int64_t* out_entries);
int fbc_cluster_borders(fbc_graph g, int32_t nclusters, const int64_t* cluster_off,
                        const int32_t* cluster_vertices, int64_t* out_border_off,
                        int32_t* out_borders);
int fbc_cluster_eval_batch(fbc_graph g, int32_t nclusters, const int64_t* cluster_off,
                           const int32_t* cluster_vertices, const int64_t* border_off,
                           const int32_t* borders, int precision, int sched,
                           double* out_intra_bc, double* out_border_dist,
                           uint64_t* out_border_sigma, fbc_stats* st);

/* Prepared cluster sweep for repeated evaluation of the same clusters (the Louvain-cluster
 * sweep of the clustered mode): the cluster subgraphs, units and work items are uploaded once
 * and the sweep (counter resets, the shared-memory kernel for the clusters that fit it, the
 * frontier kernel -- four sources per block, on a workspace of the plan's own -- for the larger
 * ones, downloads into pinned host buffers) is captured into CUDA graphs; fbc_plan_run replays
 * them.  A plan with a cluster of more than 32,768 vertices (or a vertex of 65,535+ in-edges) is
 * not captured, and a run whose path counts need a wider representation is redone: both are
 * evaluated with fbc_cluster_eval_batch instead (same results).  fbc_plan_results gives host views of the
 * last run's intra-cluster BC (n entries, overwritten each run) and border vectors (layout of
 * fbc_cluster_eval_batch), valid until the next run or fbc_plan_free. */
typedef struct fbc_plan_s* fbc_plan;
int fbc_cluster_plan_create(fbc_graph g, int32_t nclusters, const int64_t* cluster_off,
                            const int32_t* cluster_vertices, const int64_t* border_off,
                            const int32_t* borders, int precision, fbc_plan* out);
int fbc_plan_run(fbc_plan p, fbc_stats* st);
int fbc_plan_results(fbc_plan p, const double** intra_bc, const double** border_dist,
                     const uint64_t** border_sigma, int64_t* entries, int32_t* captured);
int fbc_plan_free(fbc_plan p);

/* Topological classes of every cluster (VertexInfoPivotSelector::selectPivots,
 * VertexInfoPivotSelector.h:30-123, for all clusters): vertices of a cluster whose border vectors
 * (bdist / bsig as fbc_cluster_eval_batch lays them out), lengths shifted by their minimum, are
 * equal form a class; classes in the order of their first member in the cluster list; a class's
 * pivot is its non-border member of least bc[v] (first in list order on ties), or its first member
 * if all members are borders; cardinality = class size.  Clusters without borders get no class.
 * Outputs: out_class_off[nclusters + 1] (classes of cluster c at [off[c], off[c+1])), out_pivots
 * and out_cards with room for cluster_off[nclusters] entries.  bc has n entries (the intra-cluster
 * BC the selection compares). */
int fbc_cluster_classes(fbc_graph g, int32_t nclusters, const int64_t* cluster_off,
                        const int32_t* cluster_vertices, const int64_t* border_off, const int32_t* borders,
                        const double* bc, const double* border_dist, const uint64_t* border_sigma,
                        int64_t* out_class_off, int32_t* out_pivots, int32_t* out_cards);

/* The k-means step of the clustered pivot selection (PlusPlusKMeans::computeCentroids,
 * PlusPlusKMeans.h:76-147, as KMeansPivotSelector.h:95-100 calls it) for nsets independent point
 * sets at once, one thread block each.  Set s has np_s = set_off[s+1] - set_off[s] points of
 * nb[s] entries: point j's lengths len[vec_off[s] + j*nb[s] + i] (integers in [0, 2^31): a
 * normalized border vector, VertexInfo::normalize) and counts cnt[...] (the int border path counts
 * VertexInfo stores), weight wt[set_off[s] + j]; k[s] centroids (1 <= k <= np_s).  The reference's
 * arithmetic and tie rules are kept (k-means++ start, each point to its first nearest centroid,
 * each centroid to the first member nearest to the members' mean, stop when no centroid moves by
 * more than min_variance or after max_iter + 1 steps), so the result equals the reference's
 * single-threaded one.  Outputs for set s at o_s = k[0] + ... + k[s-1]: out_idx[o_s + c] the point
 * index (within the set) of centroid c, duplicates kept as computeCentroids returns them
 * (KMeansPivotSelector removes them), out_w[o_s + c] the summed weights of its members in the last
 * step.  FBC_ERR_RANGE when a squared distance could pass 2^53 (the reference's double sums would
 * then round). */
int fbc_kmeans(int32_t nsets, const int64_t* set_off, const int32_t* nb, const int64_t* vec_off, const double* len,
               const int32_t* cnt, const int32_t* wt, const int32_t* k, double min_variance, int32_t max_iter,
               int32_t* out_idx, int32_t* out_w, fbc_stats* st);

/* Exact BC of several independent graphs in one persistent launch.  out_bc[g] has
 * n_g entries. */
int fbc_multi_exact_bc(int32_t ngraphs, const fbc_graph* graphs, int precision, int sched,
                       double* const* out_bc, fbc_stats* st);

/* Debug dump of one source: dist (-1 when unreached), sigma, delta (FP64 form) and the
 * number of shortest-path predecessors of each vertex; any output may be NULL. */
int fbc_sssp_debug(fbc_graph g, int32_t source, int32_t* out_dist, uint64_t* out_sigma,
                   double* out_delta, int32_t* out_npred);

/* No counterpart in the reference (which only runs on the CPU): a variant of the plain
 * block-per-source kernel for callers that cannot allocate device memory -- code inside a
 * framework's memory pool or a custom allocator that owns every device byte, or a library
 * handed device buffers and a stream by its host application.  It allocates nothing: the
 * graph (d_row_ptr: n+1 int32 row offsets, row_ptr[0] = 0 and row_ptr[n] = m; d_adj: 2*m int32,
 * (destination, weight) pairs, each row's destinations strictly ascending, weights > 0) and the
 * output (d_dep: n doubles, overwritten, d_dep[source] = 0) are the caller's device buffers, the
 * work runs on the caller's stream (NULL: the default stream), and the per-source work area is a
 * fixed device array inside the library, sized for FBC_NOALLOC_MAX_N vertices (about 12.6 MB,
 * held by every GPU that loads the library until the process exits).  Larger n is rejected with
 * FBC_ERR_RANGE; a malformed CSR (checked on the device, reading only row_ptr[0..n] and
 * d_adj[0..2m)) with FBC_ERR_INVALID_ARG.  fbc_gpu_init is not needed.
 * The first call on a device looks up that array's device address (once per device, with the
 * device current).  Every call ends by reading its status back with a synchronisation of the
 * caller's stream, so the entry point cannot be called while that stream is being captured.
 * All calls share the one array, so calls whose work overlaps on the GPU (other streams, other
 * host threads) race and must be serialised by the caller.  A source whose path counts pass
 * 2^64 - 1 is run again with FP64 counts, as fbc_single_source does; results agree with
 * fbc_single_source's within the precision form's tolerance. */
#define FBC_NOALLOC_MAX_N 262144
int fbc_single_source_noalloc(int32_t n, int64_t m, const int32_t* d_row_ptr, const int32_t* d_adj,
                              int32_t source, int precision, double* d_dep, void* stream);

#ifdef __cplusplus
}
#endif
#endif
