// abx_build.h -- host launchers of the construction and query kernels.
#pragma once

#include "abx_common.cuh"
#include "abx_internal.h"

namespace abx
{

abx_status scene_bounds(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                        float *d_out);

// d_hist (optional, zeroed, 8 x 256) receives the radix digit histograms.
abx_status morton64_codes(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                          const float *d_scene, uint64_t *d_codes, uint32_t *d_hist);

// d_hist (optional, zeroed, 4 x 256).
abx_status morton32_codes(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                          const float *d_scene, uint32_t *d_codes, uint32_t *d_hist);

// n >= 2.  d_tnodes and d_sorted (Morton-ordered leaf geometry, SortedLeaf)
// may be null: scratch is used for them then.
abx_status generate_hierarchy(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                              const uint32_t *d_perm, const uint64_t *d_codes,
                              LeafNode *d_leaves, InternalNode *d_internal, TNode *d_tnodes,
                              float4 *d_sorted);

// Hierarchy over trees stored as segments [off[s], off[s+1]) of the sorted
// positions (nseg trees; d_off on the device).  Node records of the
// internal node with Karras index k of tree s go to slot off[s] + k; a
// one-leaf tree has its traversal node in slot off[s].  Values and node
// numbers in the records are tree-local.
abx_status generate_hierarchy_segments(cudaStream_t s, abx_geometry kind, const float *d_g,
                                       int64_t total, const int64_t *d_off, int nseg,
                                       const uint32_t *d_perm, const uint64_t *d_codes,
                                       TNode *d_tnodes, float4 *d_sorted);

// The reference-layout arrays (leaves {rope, value}, internal nodes
// {left_child, rope, box}; ArborX_Node.hpp:24-51) of the tree whose sorted
// positions and node slots start at lo, derived from its child-pair nodes
// and Morton-ordered leaves.  Either output may be null.
abx_status export_reference_layout(cudaStream_t s, abx_geometry kind, const TNode *d_tnodes,
                                   const float4 *d_sorted, int64_t lo, int64_t n,
                                   LeafNode *d_leaves, InternalNode *d_internal);

// Batched build of nseg trees given as segments of d_g (d_off on the device):
// per-tree bounds (d_bounds, 6 floats per tree), per-tree Morton codes, a
// stable sort of every tree, the segmented hierarchy.
abx_status forest_build(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t total,
                        const int64_t *d_off, int nseg, float *d_bounds, TNode *d_tnodes,
                        float4 *d_sorted);

// Query order of a forest batch: by tree, then Morton32 within the tree's box.
abx_status forest_query_order(cudaStream_t s, abx_geometry pred_kind, const float *d_preds,
                              int64_t nq, const int64_t *d_qoff, int nseg,
                              const float *d_bounds, uint32_t *d_perm);

abx_status single_leaf(cudaStream_t s, abx_geometry kind, const float *d_g,
                       LeafNode *d_leaves, TNode *d_tnodes, float4 *d_sorted, float *d_bounds);

// Spatial queries with the default (two-pass) policy: from this many queries
// on, a buffer of about twice the sampled mean hit count takes the counting
// pass's results (up to kOnePassMaxBuffer per query and kOnePassMaxBytes in
// all), and only overflowing queries are traversed again.
constexpr int64_t kOnePassMinQueries = 65536;
constexpr int64_t kOnePassSample = 4096;
constexpr int64_t kOnePassMaxBuffer = 256;
constexpr int64_t kOnePassMaxBytes = (int64_t)4 << 30;

// Leaves per CTA of the block-local hierarchy climb.
constexpr int kHierBlock = 256;

// Largest subtree whose leaves a query may scan as one bucket, the flag of a
// child slot's count field marking "Karras index = right end of the range",
// and the default bucket limits of the query kernels.
constexpr int kMaxBucket = 32;
constexpr int kBucketRightEnd = 1 << 16;
constexpr int kDefaultSpatialBucket = 8;
constexpr int kDefaultNearestBucket = 1;

// Tree view used by the query launchers.
struct TreeView
{
  const TNode *tnodes;
  int64_t n;
  const float *d_bounds; // 6 floats, the tree bounds
  const float4 *sorted;  // leaf geometry in Morton order (SortedLeaf<kind>)
  abx_geometry kind;     // ABX_POINT or ABX_BOX leaves
  // KDOP-bounded trees (abx_kdop.cu): directions (0: box-bounded), node slot
  // and leaf KDOP records
  int ndir = 0;
  const float *knodes = nullptr;
  const float *kleaves = nullptr;
  // brute force over points: the values again in Morton order ({x, y, z,
  // value}) with their sorted Morton64 codes (scan start of a query block)
  const float4 *morton_sorted = nullptr;
  const uint64_t *morton_codes = nullptr;
};

// Trees of a batch seen by a query launch: tree s owns the sorted positions
// [tree_off[s], tree_off[s+1]) and the queries [qoff[s], qoff[s+1]).  A null
// view means one tree (root node 0, TreeView::n leaves).
struct ForestView
{
  const int64_t *tree_off;
  const int64_t *qoff;
  int nseg;
};

// Row-major copy (cols floats per value) of values read through strides.
abx_status pack_strided(cudaStream_t s, const float *d_data, int64_t value_stride,
                        int64_t coord_stride, int64_t n, int cols, float *d_out);

// Values of a brute-force index packed in input order like the Morton-ordered
// leaves ({x, y, z, index}; two float4 per box).  A TreeView with null
// tnodes is a brute-force index over such values: the query launchers then
// test every predicate against every value.
abx_status brute_pack(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                      float4 *d_values);

// Spatial query modes.
enum SpatialMode
{
  kCount = 0,  // counts[q] = number of hits
  kFill = 1,   // out[offsets[q] + j] = j-th hit
  kBuffered = 2 // out[q * buffer + j] for j < buffer, counts[q] = hits
};

// KDOPs (abx_kdop.cu).  kdop_from_geometry: expand(KDOP{}, point or box)
// for n points or boxes into the host KDOP format.  kdop_axis_boxes: the axis
// box of every KDOP.  kdop_records: the node slot and leaf records of a KDOP
// tree of n >= 1 values over its box topology (d_knodes: 2 max(n - 1, 1) + 1
// records, d_kleaves: n records of kdop_pad(ndir) floats).
abx_status kdop_from_geometry(cudaStream_t s, abx_geometry src_kind, const float *d_src, int64_t n,
                              abx_geometry kdop_kind, float *d_out);
abx_status kdop_axis_boxes(cudaStream_t s, abx_geometry kdop_kind, const float *d_kdops, int64_t n,
                           float *d_boxes);
abx_status kdop_records(cudaStream_t s, abx_geometry kdop_kind, const TNode *d_tnodes,
                        const float4 *d_sorted, int64_t n, const float *d_kdops, float4 *d_knodes,
                        float4 *d_kleaves);
// Spatial launches that involve KDOPs: KDOP predicates on any tree or brute
// force, and box or KDOP predicates on KDOP trees.
abx_status launch_spatial_kdop(cudaStream_t s, TreeView const &t, ForestView const &f,
                               abx_geometry pred_kind, const float *d_preds, int64_t nq,
                               const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                               const int32_t *d_offsets, int32_t *d_out, int32_t buffer,
                               unsigned *d_overflow);

abx_status launch_spatial(cudaStream_t s, TreeView const &t, ForestView const *f,
                          abx_geometry pred_kind, const float *d_preds, int64_t nq,
                          const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                          const int32_t *d_offsets, int32_t *d_out, int32_t buffer,
                          unsigned *d_overflow);

abx_status launch_compact(cudaStream_t s, const int32_t *d_tmp, int64_t nq, int32_t buffer,
                          const int32_t *d_offsets, int32_t *d_out);

// Spatial self-query of a point tree with spheres built from its own values
// (neighbor lists): filter 1 drops each value from its own result, filter 2
// keeps only values whose leaf precedes the query value's leaf
// (d_leaf_pos[value] = Morton position).  Count and fill modes.
abx_status launch_spatial_self(cudaStream_t s, TreeView const &t, int filter,
                               const int32_t *d_leaf_pos, const float *d_spheres, int64_t nq,
                               const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                               const int32_t *d_offsets, int32_t *d_out);

// Neighbor lists: spheres (p, r) of every point; the tree's leaf order
// (order[t] = value at Morton position t, pos[value] = t); the full list from
// a half list (row i = its half row, then the rows k listing i, ascending k).
abx_status self_spheres(cudaStream_t s, const float *d_points, int64_t n, float r,
                        float *d_spheres);
abx_status leaf_order(cudaStream_t s, abx_geometry kind, const float4 *d_sorted, int64_t n,
                      uint32_t *d_order, int32_t *d_pos);
abx_status expand_half_to_full(cudaStream_t s, int64_t n, const int32_t *d_half_off,
                               const int32_t *d_half_idx, int64_t m, int32_t *d_full_off,
                               int32_t *d_full_idx);

// Rays: Ray{origin, direction} construction (direction normalized in
// double); the ordering pass of ordered_intersects: the m results of a ray
// CRS (d_offsets, d_indices) sorted per ray by (distance, value), at most k
// per ray (k <= 0: all), into d_new_offsets (nq + 1) and d_out_idx /
// d_out_dist (room for m); the kept total in *h_new_total (synchronises s).
abx_status ray_normalize(cudaStream_t s, const float *d_raw, int64_t n, float *d_out);
abx_status order_ray_results(cudaStream_t s, abx_geometry leaf_kind, const float4 *d_sorted,
                             int64_t n, const float *d_rays, int64_t nq, const int32_t *d_offsets,
                             const int32_t *d_indices, int64_t m, int32_t k,
                             int32_t *d_new_offsets, int32_t *d_out_idx, float *d_out_dist,
                             int64_t *h_new_total);

// nearest(Ray, k) for 1 <= k <= kRayNearestMaxK on a tree of n >= 1 leaves,
// by a pruned walk (no full hit list): the same rows as the first k of
// ordered_intersects.  Offsets into d_offsets (nq + 1); indices and, when
// with_dist, distances allocated on s (*d_idx, *d_dist; released with
// dfree); the total in *h_total (synchronises s).
constexpr int kRayNearestMaxK = 32;
abx_status ray_nearest(cudaStream_t s, abx_geometry leaf_kind, const TNode *d_nodes,
                       const float4 *d_sorted, int64_t n, const float *d_rays, int64_t nq,
                       const uint32_t *d_perm, int32_t k, bool with_dist, int32_t *d_offsets,
                       int32_t **d_idx, float **d_dist, int64_t *h_total);

// The queries whose result count (from CRS offsets) exceeds `buffer`, into
// d_list (nq entries of room); their number in *h_count (synchronises s).
abx_status launch_overflow_list(cudaStream_t s, const int32_t *d_offsets, int64_t nq,
                                int32_t buffer, uint32_t *d_list, int64_t *h_count);

// Mean number of results per query over a strided sample of at most
// max_sample queries (counts land in d_counts at the sampled queries;
// synchronises s).
abx_status sample_mean_hits(cudaStream_t s, TreeView const &t, ForestView const *f,
                            abx_geometry pred_kind, const float *d_preds, int64_t nq,
                            const uint32_t *d_perm, int32_t *d_counts, int64_t max_sample,
                            double *h_mean);

// kNN: d_offsets null means uniform k (offset q * min(k, n)), and then
// d_offsets_out (nq + 1) is filled by the kernel.  max_k bounds every k.
abx_status launch_nearest(cudaStream_t s, TreeView const &t, ForestView const *f,
                          const float *d_queries, int64_t nq, const uint32_t *d_perm,
                          const int32_t *d_k, int32_t k, int32_t max_k, const int32_t *d_offsets,
                          int32_t *d_offsets_out, int32_t *d_idx, float *d_dist);

// d_dst row j = d_src row d_rows[j] (rows of `words` 32-bit words; rows
// outside [0, n_src) raise the device error word and give zeros).
abx_status gather_rows(cudaStream_t s, const void *d_src, int64_t n_src, int words,
                       const int32_t *d_rows, int64_t m, void *d_dst);

// d_out[i] = {point d_g[d_perm[i]], value d_perm[i]} (brute force in Morton
// order).
abx_status brute_pack_sorted(cudaStream_t s, const float *d_g, const uint32_t *d_perm, int64_t n,
                             float4 *d_out);

// d_out[i] = (first + i) * step for i < count (CRS offsets of a fixed k).
abx_status fill_offsets_iota(cudaStream_t s, int32_t *d_out, int64_t count, int64_t first,
                             int64_t step);

// counts[q] = min(max(k_q, 0), size of q's tree) with k_q = d_k[q] (or k
// when d_k is null); max of k_q over queries into *d_max (zeroed).
abx_status launch_knn_counts(cudaStream_t s, TreeView const &t, ForestView const *f,
                             const int32_t *d_k, int32_t k, int64_t nq, int32_t *d_counts,
                             int32_t *d_max);

} // namespace abx
