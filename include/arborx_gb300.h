/*
 * arborx_gb300.h -- C ABI of the GB300-native bounding volume hierarchy.
 *
 * A drop-in for the ArborX BoundingVolumeHierarchy hot path (construction,
 * intersects / nearest queries, CRS output), implemented with hand-written
 * sm_103a CUDA kernels.  Every pointer argument named d_* is DEVICE memory;
 * h_* is host memory.  Streams are cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Every call is stream-ordered; the documented
 * synchronisation points are the same as the reference's (root bounds after a
 * build, the result count of a two-pass spatial query).
 *
 * Each declaration cites the reference interface it replaces (paths relative
 * to the ArborX source tree, version 2.1.99).
 */
#ifndef ARBORX_GB300_H
#define ARBORX_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define ABX_API __attribute__((visibility("default")))
#else
#define ABX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference reports errors by throwing
 * ArborX::SearchException from ARBORX_ASSERT (src/misc/ArborX_Exception.hpp:
 * 19-37); no C++ exception crosses this ABI, each call returns one of these. */
typedef enum abx_status
{
  ABX_SUCCESS = 0,
  ABX_ERROR_INVALID_ARGUMENT = 1, /* ARBORX_ASSERT on a precondition          */
  ABX_ERROR_CUDA = 2,             /* a CUDA runtime call failed               */
  ABX_ERROR_OUT_OF_MEMORY = 3,    /* device allocation failed                 */
  ABX_ERROR_BUFFER_OVERFLOW = 4,  /* hard preallocation too small
                                     (ArborX_CrsGraphWrapperImpl.hpp:268)     */
  ABX_ERROR_DEVICE = 5,           /* a kernel raised the device error word    */
  ABX_ERROR_NOT_SUPPORTED = 6,
  ABX_ERROR_TIMEOUT = 7           /* a bounded device-side wait gave up       */
} abx_status;

/* Bits of the device error word (abx_device_errors). */
#define ABX_DEVERR_STACK_OVERFLOW 0x1u
#define ABX_DEVERR_TIMEOUT 0x2u
#define ABX_DEVERR_BAD_INPUT 0x4u
#define ABX_DEVERR_INTERNAL 0x8u

typedef struct abx_bvh abx_bvh; /* opaque tree                                */
typedef struct abx_crs abx_crs; /* opaque CRS result (offsets + indices)      */
typedef struct abx_forest abx_forest; /* opaque batch of independent trees    */
typedef struct abx_brute abx_brute;   /* opaque brute-force index             */

/* Geometry of values and predicates, float32, array-of-structures:
 *   POINT  x y z                 (12 bytes)   ArborX::Point<3>
 *   BOX    minx miny minz maxx maxy maxz (24) ArborX::Box<3>
 *   SPHERE cx cy cz r            (16 bytes)   ArborX::Sphere<3>
 *   RAY    ox oy oz dx dy dz     (24 bytes)   ArborX::Experimental::Ray<float>
 *          (predicates only; the direction is normalized by the library as
 *          the Ray constructor does, ArborX_Ray.hpp:46-55)
 * (src/geometry/ArborX_Point.hpp:24-38, ArborX_Box.hpp:32-67,
 *  ArborX_Sphere.hpp:25-47, ArborX_Ray.hpp:33-66). */
typedef enum abx_geometry
{
  ABX_POINT = 0,
  ABX_BOX = 1,
  ABX_SPHERE = 2,
  ABX_RAY = 3,
  /* Discrete oriented polytopes KDOP<3, k> (src/geometry/ArborX_KDOP.hpp:
   * 64-183), k/2 directions: the axes, for k = 18 and 26 the edge
   * directions, for k = 14 and 26 the corner directions, in the reference's
   * order.  One KDOP is 2 * (k/2) floats: min[k/2] then max[k/2]. */
  ABX_KDOP6 = 4,
  ABX_KDOP14 = 5,
  ABX_KDOP18 = 6,
  ABX_KDOP26 = 7
} abx_geometry;

/* TraversalPolicy (src/spatial/detail/ArborX_TraversalPolicy.hpp:19-47):
 * buffer_size 0 = two-pass count/fill; > 0 = single pass into a per-query
 * buffer, second pass on overflow; < 0 = single pass, overflow is an error.
 * sort_predicates: reorder queries along Morton32 of their centroids
 * (ArborX_LinearBVH.hpp:287-306), default 1. */
typedef struct abx_traversal_policy
{
  int32_t buffer_size;
  int32_t sort_predicates;
} abx_traversal_policy;

/* ---------------------------------------------------------------------- */
/* Library                                                                  */
/* ---------------------------------------------------------------------- */

/* Human-readable name of a status. */
ABX_API const char *abx_status_string(abx_status status);

/* Detailed message of the last failing call on this host thread. */
ABX_API const char *abx_last_error(void);

/* Library version "major.minor.patch". */
ABX_API const char *abx_version(void);

/* Read and clear the device error word of the current device
 * (ABX_DEVERR_* bits); synchronises `stream`.  Replaces the reference's
 * device-side KOKKOS_ASSERT/abort (ArborX_HappyTreeFriends.hpp:28-62),
 * which would kill the context. */
ABX_API abx_status abx_device_errors(void *stream, uint32_t *h_bits);

/* Stage timing, the counterpart of the reference's Kokkos Tools regions
 * (ArborX_LinearBVH.hpp:201-255, ArborX_CrsGraphWrapperImpl.hpp:394-431).
 * While enabled, every kernel stage of every call records a pair of CUDA
 * events on the stream it runs on.  abx_profiling_stage waits for the
 * recorded events and returns the summed device time and the number of
 * kernel launches of one stage ("bounds", "morton64", "sort64",
 * "hierarchy", "morton32", "sort32", "spatial", "scan", "compact",
 * "nearest"); "*" sums all stages.  abx_profiling_reset drops the records. */
ABX_API abx_status abx_profiling_enable(int32_t enable);
ABX_API abx_status abx_profiling_stage(const char *stage, double *h_total_ms,
                                       int64_t *h_launches);
ABX_API abx_status abx_profiling_reset(void);

/* Launch-shape and kernel-variant knobs (no counterpart in the reference,
 * whose launch shapes are Kokkos' RangePolicy defaults).  Known names:
 * "SPATIAL_BUCKET" / "NEAREST_BUCKET" (a spatial / nearest traversal scans
 * the leaves of any subtree of at most this many leaves from the
 * Morton-ordered leaf copy instead of descending into it; 1-32, defaults 8
 * and 1; read at query time).
 * Unset knobs read the environment variable ABX_TUNE_<name>, then the
 * built-in default.  Results never depend on a knob. */
ABX_API abx_status abx_tuning_set(const char *name, int32_t value);
ABX_API abx_status abx_tuning_reset(void);

/* ---------------------------------------------------------------------- */
/* Tree                                                                     */
/* ---------------------------------------------------------------------- */

/* BoundingVolumeHierarchy(space, values[, indexable_getter, Morton64{}])
 * (src/spatial/ArborX_LinearBVH.hpp:68-73,167-256).  `d_values` holds n
 * points (ABX_POINT) or boxes (ABX_BOX) in device memory; the value stored in
 * every leaf is its index in d_values (the benchmark form
 * BVH<MemorySpace, int, IndexableGetter>, benchmarks/bvh_driver/
 * benchmark_registration.hpp:151-161).  The geometry is copied; d_values may
 * be freed after the call returns.  Asynchronous on `stream`. */
ABX_API abx_status abx_bvh_create(void *stream, abx_geometry kind,
                          const float *d_values, int64_t n, abx_bvh **out);

/* Values through access traits (ArborX_AccessTraits.hpp:36-76: a rank-2
 * View of n rows, any layout): coordinate d of value i is
 * data[i * value_stride + d * coord_stride], d < 3 for points, < 6 for boxes
 * (min x y z, max x y z).  Row-major n x 3 is (3, 1), column-major (SoA,
 * Kokkos::LayoutLeft) is (1, n), padded float4 rows are (4, 1).  Strides are
 * in floats and may be any non-negative values; the tree is the one
 * abx_bvh_create builds from the same values packed row-major. */
typedef struct abx_values
{
  const float *data;
  int64_t value_stride;
  int64_t coord_stride;
} abx_values;

ABX_API abx_status abx_bvh_create_strided(void *stream, abx_geometry kind, abx_values values,
                                          int64_t n, abx_bvh **out);

/* Values of query results (PairValueIndex values, ArborX_PairValueIndex.hpp:
 * 23-44, or any record the caller stores per value): d_dst row j = d_src row
 * d_rows[j] for j < m, rows of row_bytes bytes (a multiple of 4); d_src holds
 * n_src rows (device memory).  An index outside [0, n_src) sets the device
 * error word and gives a zero row.  Asynchronous on `stream`. */
ABX_API abx_status abx_gather_rows(void *stream, const void *d_src, int64_t n_src,
                                   int64_t row_bytes, const int32_t *d_rows, int64_t m,
                                   void *d_dst);

/* KDOP bounding volumes (src/geometry/ArborX_KDOP.hpp; the BoundingVolume
 * parameter of BoundingVolumeHierarchy, src/spatial/ArborX_LinearBVH.hpp:
 * 56-60).  abx_bvh_create with kind ABX_KDOP6/14/18/26 builds a tree over n
 * KDOP values (2 * (k/2) floats each) whose nodes are bounded by KDOPs of
 * the same directions; it answers intersects(Box) and intersects(KDOP of the
 * same k) predicates (abx_bvh_query_intersects), with the reference's
 * KDOP-box and KDOP-KDOP tests (ArborX_Intersects.hpp:317-368).  KDOP
 * predicates (kind ABX_KDOPk, any k) also run on point and box trees and on
 * brute force.  The reference defines no distance to a KDOP and no
 * sphere- or ray-KDOP test: nearest, sphere and ray queries on a KDOP tree
 * return ABX_ERROR_INVALID_ARGUMENT.  Forests and BruteForce take points and
 * boxes only.
 *
 * abx_kdop_from_geometry: KDOP{} expanded by each of n points or boxes
 * (ArborX_Expand.hpp:128-208), written to d_kdops (device, 2 * (k/2) floats
 * per value): the conversion the reference's test trees apply to their
 * primitives (test/ArborXTest_LegacyTree.hpp:50-60).
 * abx_bvh_kdop_bounds: the KDOP of the whole tree (bounds() of a KDOP-bounded
 * tree), 2 * (k/2) floats to host memory; waits for the build. */
ABX_API abx_status abx_kdop_from_geometry(void *stream, abx_geometry kind, const float *d_values,
                                          int64_t n, abx_geometry kdop_kind, float *d_kdops);
ABX_API abx_status abx_bvh_kdop_bounds(const abx_bvh *bvh, float *h_kdop);

/* On-disk trees (warm restarts of a serving process; no counterpart in the
 * reference).  abx_bvh_save writes the tree (geometry kind, size, bounds,
 * child-pair nodes, Morton-ordered leaves, and for KDOP trees the KDOP
 * records) to `path`; abx_bvh_load reads it back to the current device: the
 * loaded tree answers every query exactly like the saved one.  The file
 * starts with the 8 bytes "ABXBVH01" followed by little-endian int32 kind,
 * int32 reserved, int64 size, float bounds[6], then the arrays. */
ABX_API abx_status abx_bvh_save(const abx_bvh *bvh, const char *path);
ABX_API abx_status abx_bvh_load(void *stream, const char *path, abx_bvh **out);

/* Destroy a tree (frees stream-ordered on the stream it was built on). */
ABX_API abx_status abx_bvh_destroy(abx_bvh *bvh);

/* size() / empty() (ArborX_LinearBVH.hpp:75-79). */
ABX_API int64_t abx_bvh_size(const abx_bvh *bvh);

/* bounds() (ArborX_LinearBVH.hpp:81-82): the root bounding box, the empty
 * box [FLT_MAX, -FLT_MAX] for an empty tree.  Waits for the build. */
ABX_API abx_status abx_bvh_bounds(const abx_bvh *bvh, float h_box[6]);

/* Geometry kind of the leaves. */
ABX_API abx_geometry abx_bvh_geometry(const abx_bvh *bvh);

/* Copy the node arrays in the reference layout to device buffers
 * (src/spatial/detail/ArborX_Node.hpp:24-51): d_leaves receives n
 * {int32 rope, int32 value}; d_internal receives n-1 {int32 left_child,
 * int32 rope, float box[6]} (32 bytes each).  Node numbering follows
 * ArborX_HappyTreeFriends.hpp:23-86.  Either pointer may be NULL. */
ABX_API abx_status abx_bvh_export_nodes(const abx_bvh *bvh, void *stream,
                                int32_t *d_leaves, void *d_internal);

/* Device view of a tree, for user kernels that traverse it themselves (the
 * PerThread query, ArborX_LinearBVH.hpp:112-122; the callback query,
 * :258-313).  `nodes` holds max(size - 1, 1) 64-byte child-pair nodes:
 *   float4 a = L.lo.x L.lo.y L.lo.z L.hi.x
 *   float4 b = L.hi.y L.hi.z R.lo.x R.lo.y
 *   float4 c = R.lo.z R.hi.x R.hi.y R.hi.z
 *   int4   d = left ref, right ref, left count, right count
 * (root = node 0).  A ref >= 0 is an internal node.  A ref < 0 is a leaf with
 * value ~ref whose bounding volume is the child box (count 1), or no child
 * (count 0, one-leaf tree).  The count of an internal child is its number of
 * leaves when at most 32 (bit 16 set: its index is the right end of its leaf
 * range), else 0.  `leaves` holds the leaves in Morton order: points as
 * float4 {x, y, z, value}, boxes as two float4 {lo, value} {hi, 0}.  Valid
 * while the tree lives, once its build has completed on its stream. */
typedef struct abx_device_view
{
  const void *nodes;
  const void *leaves;
  int64_t size;
  int32_t geometry;
  int32_t reserved;
} abx_device_view;

ABX_API abx_status abx_bvh_device_view(const abx_bvh *bvh, abx_device_view *out);

/* ---------------------------------------------------------------------- */
/* Queries with CRS output                                                  */
/* ---------------------------------------------------------------------- */

/* query(space, intersects(geometry)..., indices, offsets, policy)
 * (ArborX_LinearBVH.hpp:90-110; ArborX_CrsGraphWrapper.hpp:22-34;
 * ArborX_CrsGraphWrapperImpl.hpp:378-432).  `kind` is the predicate geometry
 * (ABX_SPHERE or ABX_BOX), d_predicates holds nq of them.  The result owns
 * its device arrays (the reference reallocates out/offset in the callee,
 * ArborX_CrsGraphWrapperImpl.hpp:286,376-377).  The call synchronises
 * `stream` once to size the output, like the reference's lastElement
 * (ArborX_CrsGraphWrapperImpl.hpp:248). */
ABX_API abx_status abx_bvh_query_intersects(const abx_bvh *bvh, void *stream,
                                    abx_geometry kind,
                                    const float *d_predicates, int64_t nq,
                                    abx_traversal_policy policy,
                                    abx_crs **out);

/* query(space, nearest(point, k)..., indices, offsets[, policy])
 * (ArborX_CrsGraphWrapperImpl.hpp:353-374; TreeTraversal<Nearest>,
 * ArborX_TreeTraversal.hpp:122-336).  d_queries: nq points.  d_k: one k per
 * query (device int32) or NULL to use `k` for all.  Each query returns
 * min(k, size()) values ordered by ascending (distance, index): the k
 * smallest float32 distances, ties at equal distance broken by the smaller
 * value index.  With with_distances != 0 the distances are kept
 * (abx_crs_distances).  Asynchronous unless d_k is given (then one
 * synchronisation to size the output). */
ABX_API abx_status abx_bvh_query_nearest(const abx_bvh *bvh, void *stream,
                                 const float *d_queries, int64_t nq,
                                 const int32_t *d_k, int32_t k,
                                 abx_traversal_policy policy,
                                 int32_t with_distances, abx_crs **out);

/* ---------------------------------------------------------------------- */
/* Batched trees (forest)                                                 */
/* ---------------------------------------------------------------------- */
/* Replaces the many-trees pattern of the reference
 * (benchmarks/execution_space_instances/execution_space_instances_driver.cpp:
 * 187-233: one BoundingVolumeHierarchy per subview of a values array, each
 * built and queried through its own call) by one build and one query launch
 * sequence over all trees.  Tree t holds the values
 * d_values[h_offsets[t] .. h_offsets[t + 1]) (h_offsets: host, ntrees + 1
 * entries, h_offsets[0] = 0, non-decreasing; empty trees allowed).  Each tree
 * is exactly the tree abx_bvh_create builds from its subview alone: same
 * scene box, node arrays (abx_forest_export_nodes), tree-local values. */
ABX_API abx_status abx_forest_create(void *stream, abx_geometry kind,
                                     const float *d_values,
                                     const int64_t *h_offsets, int32_t ntrees,
                                     abx_forest **out);
ABX_API abx_status abx_forest_destroy(abx_forest *forest);
ABX_API int32_t abx_forest_num_trees(const abx_forest *forest);
/* Number of values in tree `tree` (0 for a bad index). */
ABX_API int64_t abx_forest_size(const abx_forest *forest, int32_t tree);
/* Bounds of one tree (ArborX_LinearBVH.hpp:104): 6 host floats. */
ABX_API abx_status abx_forest_bounds(const abx_forest *forest, int32_t tree,
                                     float h_box[6]);
/* The node arrays of one tree, in the layout of abx_bvh_export_nodes. */
ABX_API abx_status abx_forest_export_nodes(const abx_forest *forest,
                                           int32_t tree, void *stream,
                                           int32_t *d_leaves, void *d_internal);

/* Queries grouped by tree: the predicates
 * d_predicates[h_query_offsets[t] .. h_query_offsets[t + 1]) run on tree t
 * (h_query_offsets: host, ntrees + 1 entries).  One CRS result over all
 * queries; its indices are tree-local values, so query q of tree t returns
 * what abx_bvh_query_intersects / abx_bvh_query_nearest on tree t alone
 * return for it, in the same order.  Both calls synchronise `stream` once. */
ABX_API abx_status abx_forest_query_intersects(const abx_forest *forest,
                                               void *stream, abx_geometry kind,
                                               const float *d_predicates,
                                               const int64_t *h_query_offsets,
                                               abx_traversal_policy policy,
                                               abx_crs **out);
ABX_API abx_status abx_forest_query_nearest(const abx_forest *forest,
                                            void *stream,
                                            const float *d_queries,
                                            const int64_t *h_query_offsets,
                                            const int32_t *d_k, int32_t k,
                                            abx_traversal_policy policy,
                                            int32_t with_distances,
                                            abx_crs **out);

/* ---------------------------------------------------------------------- */
/* Neighbor lists (src/spatial/detail/ArborX_NeighborList.hpp:47-188)      */
/* ---------------------------------------------------------------------- */
/* findFullNeighborList / findHalfNeighborList(space, points, radius,
 * offsets, indices): the radius self-join of n points (a tree is built
 * internally).  Full (half = 0): row p lists every other point q with
 * distance(p, q) <= radius.  Half (half != 0): row p lists the points q
 * within radius whose leaf precedes p's leaf in the tree's Morton order (the
 * pairs of HalfTraversal, ArborX_HalfTraversal.hpp:52-73), so every pair
 * appears once.  The reference fills rows through atomics (any order); here a
 * row is in the tree's depth-first order.  CRS over n rows. */
ABX_API abx_status abx_find_neighbor_list(void *stream, const float *d_points, int64_t n,
                                          float radius, int32_t half, abx_crs **out);

/* expandHalfToFull (src/spatial/detail/ArborX_ExpandHalfToFull.hpp:23-69):
 * from a half list (device offsets n + 1, indices) the full list, row i = its
 * half row followed by every k whose half row lists i, in ascending k.
 * Synchronises once (the input size). */
ABX_API abx_status abx_expand_half_to_full(void *stream, int64_t n, const int32_t *d_offsets,
                                           const int32_t *d_indices, abx_crs **out);

/* ---------------------------------------------------------------------- */
/* Brute force (src/spatial/ArborX_BruteForce.hpp:40-176)                  */
/* ---------------------------------------------------------------------- */
/* BruteForce(space, values): every predicate is tested against every value
 * (ArborX_BruteForceImpl.hpp:29-229), values staged through shared memory.
 * Same predicates, policies and CRS output as the tree queries:
 * intersects returns each query's matches in ascending value order (the
 * reference's order is that of its atomic inserts); nearest returns exactly
 * what abx_bvh_query_nearest returns on a tree of the same values (k smallest
 * (distance, index), ascending).  Predicate sorting is a no-op here. */
ABX_API abx_status abx_brute_create(void *stream, abx_geometry kind, const float *d_values,
                                    int64_t n, abx_brute **out);
ABX_API abx_status abx_brute_destroy(abx_brute *brute);
ABX_API int64_t abx_brute_size(const abx_brute *brute);
ABX_API abx_status abx_brute_bounds(const abx_brute *brute, float h_box[6]);
ABX_API abx_status abx_brute_query_intersects(const abx_brute *brute, void *stream,
                                              abx_geometry kind, const float *d_predicates,
                                              int64_t nq, abx_traversal_policy policy,
                                              abx_crs **out);
ABX_API abx_status abx_brute_query_nearest(const abx_brute *brute, void *stream,
                                           const float *d_queries, int64_t nq,
                                           const int32_t *d_k, int32_t k,
                                           abx_traversal_policy policy, int32_t with_distances,
                                           abx_crs **out);

/* ---------------------------------------------------------------------- */
/* Serving: a request loop over trees resident in HBM                      */
/* ---------------------------------------------------------------------- */
/* No counterpart in the reference (it is the loop around
 * BoundingVolumeHierarchy::query, ArborX_LinearBVH.hpp:90-110).  Worker
 * threads, each on its own CUDA stream, coalesce the pending requests on one
 * tree and of one kind into a single query launch (mixed k and radii
 * allowed), admit batches while their device memory fits
 * max_inflight_bytes, and run up to `workers` batches at once; requests that
 * arrive meanwhile join the next batch.  A request's results are those of
 * the same query run alone: nearest as abx_bvh_query_nearest (with
 * distances), intersects as abx_bvh_query_intersects on spheres. */
typedef struct abx_server abx_server;

#define ABX_REQ_NEAREST 0    /* h_queries: nq points (3 floats), k          */
#define ABX_REQ_INTERSECTS 1 /* h_queries: nq spheres (4 floats: x y z r)   */

typedef struct abx_server_config
{
  int32_t workers;            /* concurrent batches (streams), default 4      */
  int32_t l2_persist;         /* 1: the nodes of the tree a batch queries are
                                 held L2-persisting while it runs (access
                                 policy window on the worker's stream; the
                                 context's persisting-L2 limit is raised while
                                 the server lives and restored after)        */
  int64_t max_inflight_bytes; /* device-memory budget of running batches      */
  int64_t max_batch_queries;  /* cap of one coalesced launch                  */
} abx_server_config;

typedef struct abx_request
{
  int32_t tree;             /* id from abx_server_add_tree                  */
  int32_t kind;             /* ABX_REQ_NEAREST or ABX_REQ_INTERSECTS        */
  const float *h_queries;   /* host rows; copied by abx_server_submit       */
  int64_t nq;
  int32_t k;                /* nearest only                                  */
  int32_t reserved;
} abx_request;

typedef struct abx_server_statistics
{
  int64_t completed_requests;
  int64_t completed_queries;
  int64_t batches;          /* coalesced launches                            */
  double p50_ms;            /* request latency, submit to completion        */
  double p99_ms;
  double span_s;            /* first submit to last completion               */
} abx_server_statistics;

/* cfg may be NULL (defaults: 4 workers, no L2 persistence, 8 GiB, 2^20
 * queries per launch).  On the 64-tree serving workload L2 persistence was
 * measured slower (saturation 12.8k vs 14.4k requests/s), so it is off by
 * default. */
ABX_API abx_status abx_server_create(const abx_server_config *cfg, abx_server **out);
ABX_API abx_status abx_server_destroy(abx_server *srv);
/* The tree must outlive the server. */
ABX_API abx_status abx_server_add_tree(abx_server *srv, const abx_bvh *tree, int32_t *tree_id);
ABX_API abx_status abx_server_submit(abx_server *srv, const abx_request *req, int64_t *ticket);
/* Blocks until the request completed; its number of results and latency. */
ABX_API abx_status abx_server_wait(abx_server *srv, int64_t ticket, int64_t *num_results,
                                   double *latency_ms);
/* Copies the results to host arrays (offsets nq + 1, indices, distances for
 * nearest; any may be NULL) and releases the request. */
ABX_API abx_status abx_server_result(abx_server *srv, int64_t ticket, int32_t *h_offsets,
                                     int32_t *h_indices, float *h_distances);
ABX_API abx_status abx_server_stats(abx_server *srv, abx_server_statistics *out);
ABX_API abx_status abx_server_reset_stats(abx_server *srv);

/* ordered_intersects(Ray) (Experimental::OrderedSpatial,
 * ArborX_Predicates.hpp:103-125; traversal ArborX_TreeTraversal.hpp:338-489):
 * per ray, the leaves in front of it by increasing distance(Ray, Box)
 * (ArborX_Ray.hpp:435-447, the entry distance), equal distances by value
 * (the reference reports them in heap order).  k > 0 keeps the first k per
 * ray, which is nearest(Ray, k) (leaves the ray misses are never
 * candidates).  For 1 <= k <= 32 on a tree the first k come from a pruned
 * walk that never lists the other hits (same rows and distances).
 * d_rays: nq rows of ABX_RAY.  with_distances keeps the distances
 * (abx_crs_distances).  Synchronises the stream. */
ABX_API abx_status abx_bvh_query_ordered_intersects(const abx_bvh *bvh, void *stream,
                                                    const float *d_rays, int64_t nq, int32_t k,
                                                    abx_traversal_policy policy,
                                                    int32_t with_distances, abx_crs **out);

/* nearest(point, k) with one k for all queries into caller-provided device
 * arrays and no host synchronisation, so that the call can be captured in a
 * CUDA graph and replayed (the queries' contents may change between
 * replays).  d_offsets (nq + 1), d_indices (nq * min(k, size())) and, if not
 * NULL, d_distances receive what abx_bvh_query_nearest returns.  While the
 * stream is capturing, the tree's build must already have completed (for
 * instance abx_bvh_bounds returned): the call does not wait on it then. */
ABX_API abx_status abx_bvh_query_nearest_into(const abx_bvh *bvh, void *stream,
                                              const float *d_queries, int64_t nq, int32_t k,
                                              abx_traversal_policy policy, int32_t *d_offsets,
                                              int32_t *d_indices, float *d_distances);

/* nearest(point, k) with the queries and the results in HOST memory: the
 * call a host-side plugin makes (the reference's query(space, predicates,
 * indices, offsets) with host Views).  The queries go to the device in
 * chunks of `chunk` queries (<= 0: 40% of them, at least 2^18) over two
 * copy streams, so that
 * chunk i + 1 moves in and the results of chunk i - 1 move out while chunk i
 * is traversed; each chunk is ordered by Morton code by itself when
 * policy.sort_predicates is set.  When chunk <= 0 and the result buffers
 * are page-locked and mapped (cudaHostAlloc, cudaHostRegister: every pinned
 * buffer on a unified-address system), there are no chunks: the traversal
 * writes the results straight into them over the CPU-GPU link.  h_offsets
 * (nq + 1), h_indices (nq * min(k, size())) and, if not NULL, h_distances
 * receive exactly what abx_bvh_query_nearest returns.  Returns when the
 * results are on the host. */
ABX_API abx_status abx_bvh_query_nearest_host(const abx_bvh *bvh, void *stream,
                                              const float *h_queries, int64_t nq, int32_t k,
                                              abx_traversal_policy policy, int64_t chunk,
                                              int32_t *h_offsets, int32_t *h_indices,
                                              float *h_distances);

/* Accessors of a CRS result: device offsets (nq + 1), device indices
 * (num_results), device distances (nearest only, else NULL). */
ABX_API int64_t abx_crs_num_queries(const abx_crs *crs);
ABX_API int64_t abx_crs_num_results(const abx_crs *crs);
ABX_API const int32_t *abx_crs_offsets(const abx_crs *crs);
ABX_API const int32_t *abx_crs_indices(const abx_crs *crs);
ABX_API const float *abx_crs_distances(const abx_crs *crs);
ABX_API abx_status abx_crs_destroy(abx_crs *crs);

/* ---------------------------------------------------------------------- */
/* Building blocks (the reference's Details functions, exposed for parity  */
/* tests and for callers that assemble their own pipelines)               */
/* ---------------------------------------------------------------------- */

/* calculateBoundingBoxOfTheScene (spatial/detail/
 * ArborX_TreeConstruction.hpp:26-39): d_box_out receives 6 floats. */
ABX_API abx_status abx_scene_bounds(void *stream, abx_geometry kind,
                            const float *d_values, int64_t n,
                            float *d_box_out);

/* projectOntoSpaceFillingCurve with Morton64 (spatial/detail/
 * ArborX_SpaceFillingCurves.hpp:45-57,64-84) against the scene box
 * d_scene (6 floats). */
ABX_API abx_status abx_morton64(void *stream, abx_geometry kind,
                        const float *d_values, int64_t n,
                        const float *d_scene, uint64_t *d_codes);

/* Morton32 of predicate centroids (ArborX_SpaceFillingCurves.hpp:30-43). */
ABX_API abx_status abx_morton32(void *stream, abx_geometry kind,
                        const float *d_values, int64_t n,
                        const float *d_scene, uint32_t *d_codes);

/* sortObjects (misc/ArborX_SortUtils.hpp:28-39): sort d_keys in place
 * (stable: equal keys keep their input order) and write the permutation. */
ABX_API abx_status abx_sort_u64(void *stream, uint64_t *d_keys, int64_t n,
                        uint32_t *d_permutation);
ABX_API abx_status abx_sort_u32(void *stream, uint32_t *d_keys, int64_t n,
                        uint32_t *d_permutation);

/* generateHierarchy (spatial/detail/ArborX_TreeConstruction.hpp:71-348)
 * from already sorted Morton codes and the permutation: writes the node
 * arrays in the layout of abx_bvh_export_nodes.  n >= 2. */
ABX_API abx_status abx_generate_hierarchy(void *stream, abx_geometry kind,
                                  const float *d_values, int64_t n,
                                  const uint32_t *d_permutation,
                                  const uint64_t *d_sorted_codes,
                                  int32_t *d_leaves, void *d_internal);

/* exclusive_scan (kokkos_ext/ArborX_KokkosExtStdAlgorithms.hpp:24) of n
 * int32 into n + 1 outputs (the last is the total).  In-place allowed. */
ABX_API abx_status abx_exclusive_scan_i32(void *stream, const int32_t *d_in,
                                  int64_t n, int32_t *d_out);

/* Allocation-free exclusive scan.  No counterpart in the reference: ArborX
 * always allocates its scratch through Kokkos.
 *
 * For callers that must not allocate device memory: code that runs under a
 * device-memory budget owned by another allocator (a framework that has
 * reserved the GPU's memory for its own pool, where an extra cudaMalloc can
 * fail or break that pool's accounting), and latency-critical loops that
 * must not take the allocator's locks or the device-wide synchronisation of
 * cudaFree.  It computes exactly what abx_exclusive_scan_i32 computes (n
 * int32 inputs, n + 1 outputs, in place allowed) for
 * n <= ABX_NOALLOC_SCAN_MAX_N and rejects larger n with
 * ABX_ERROR_INVALID_ARGUMENT.  It allocates nothing: its scratch (one 64-bit
 * partial sum per 4096 inputs, 32 KB in all) is a static array in the
 * library's device memory, which every GPU that loads the library holds
 * until the process exits.
 *
 * The first call on a device, with that device current, looks up the
 * array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture.  All calls share the one array: calls that
 * overlap on the GPU (on different streams with no ordering between them)
 * race and corrupt each other's result, so order them on one stream or with
 * events.  Each call writes every scratch entry before reading it, so no
 * entry has to start at zero.  The total must fit in int32: unlike
 * abx_exclusive_scan_i32, this variant does not report an overflowing total
 * in the device error word. */
#define ABX_NOALLOC_SCAN_MAX_N 16777216
ABX_API abx_status abx_exclusive_scan_i32_noalloc(void *stream,
                                                  const int32_t *d_in,
                                                  int64_t n, int32_t *d_out);

#ifdef __cplusplus
}
#endif

#endif /* ARBORX_GB300_H */
