// abx_kdop.cu -- KDOP bounding volumes (src/geometry/ArborX_KDOP.hpp; the
// BoundingVolume parameter of BoundingVolumeHierarchy, ArborX_LinearBVH.hpp:
// 56-60, exercised by test/CMakeLists.txt:126-151 with KDOP<3,14> and
// KDOP<3,18>).
//
// A tree over KDOP values keeps the child-pair topology of the box tree of
// the values' axis ranges: the reference sorts KDOP values by the centroid of
// that same box (centroid(KDOP), ArborX_Centroid.hpp:84-94) inside the scene
// box expanded by those boxes (expand(Box, KDOP), ArborX_Expand.hpp:210-225),
// so its hierarchy is the box tree's.  Beside the topology it stores
//   knodes   one KDOP record per child slot: slot s of node i is record
//            2 i + s; a single leaf's slot holds the leaf's own KDOP, an
//            internal child's slot the union of its subtree (expand(KDOP,
//            KDOP), ArborX_Expand.hpp:110-126); record 2 (n - 1) (2 for one
//            leaf) holds the union of the whole tree
//   kleaves  the values' KDOPs in Morton order with the value in the spare
//            float (bucket scans)
// and the traversal (k_spatial with NDIR > 0) tests KDOPs only.  Also here:
// the conversion of points and boxes to KDOPs (the LegacyTree pattern of the
// reference's test suite, test/ArborXTest_LegacyTree.hpp:50-60) and the
// launches of intersects(KDOP) predicates.
#include "abx_spatial.cuh"

namespace abx
{
namespace
{

template <int NDIR>
__device__ __forceinline__ void kdop_load_cg(const float4 *rec, Kdop<NDIR> &k)
{
  constexpr int n4 = kdop_pad(NDIR) / 4;
  float f[4 * n4];
#pragma unroll
  for (int j = 0; j < n4; ++j)
  {
    const float4 v = __ldcg(rec + j);
    f[4 * j] = v.x;
    f[4 * j + 1] = v.y;
    f[4 * j + 2] = v.z;
    f[4 * j + 3] = v.w;
  }
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
  {
    k.mn[i] = f[i];
    k.mx[i] = f[NDIR + i];
  }
}

// expand(KDOP{}, point or box) for every input geometry (KIND 0 points, 1
// boxes), written in the host format.
template <int NDIR, int KIND>
__global__ void k_kdop_from_geometry(const float *__restrict__ g, int64_t n, float *__restrict__ out)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  Kdop<NDIR> k;
  kdop_empty<NDIR>(k);
  if (KIND == 0)
    kdop_expand_point<NDIR>(k, g[3 * i], g[3 * i + 1], g[3 * i + 2]);
  else
  {
    Box3 b;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      b.lo[d] = g[6 * i + d];
      b.hi[d] = g[6 * i + 3 + d];
    }
    kdop_expand_box<NDIR>(k, b);
  }
#pragma unroll
  for (int j = 0; j < NDIR; ++j)
  {
    out[2 * NDIR * i + j] = k.mn[j];
    out[2 * NDIR * i + NDIR + j] = k.mx[j];
  }
}

// The axis box of every KDOP value (the geometry the box tree is built on).
template <int NDIR>
__global__ void k_kdop_axis_boxes(const float *__restrict__ kd, int64_t n, float *__restrict__ boxes)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  Kdop<NDIR> k;
  kdop_load_raw<NDIR>(kd, i, k);
  const Box3 b = kdop_axis_box<NDIR>(k);
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    boxes[6 * i + d] = b.lo[d];
    boxes[6 * i + 3 + d] = b.hi[d];
  }
}

// kleaves[t] = KDOP of the value at sorted position t, with the value.
template <int NDIR>
__global__ void k_kdop_leaves(const float4 *__restrict__ sorted, int64_t n,
                              const float *__restrict__ kd, float4 *__restrict__ kleaves,
                              unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n)
    return;
  const int v = __float_as_int(__ldg(sorted + 2 * t).w);
  Kdop<NDIR> k;
  if ((uint64_t)v < (uint64_t)n)
    kdop_load_raw<NDIR>(kd, v, k);
  else
  {
    raise_error(err, ABX_DEVERR_INTERNAL);
    kdop_empty<NDIR>(k);
  }
  kdop_store<NDIR>(kleaves + t * (kdop_pad(NDIR) / 4), k, v);
}

// parent[c] = 2 i + s for the internal node c in slot s of node i.
__global__ void k_kdop_parents(const TNode *__restrict__ tnodes, int64_t nint,
                               int *__restrict__ parent, unsigned *__restrict__ err)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nint)
    return;
  const int4 d = tnodes[i].d;
  const int refs[2] = {d.x, d.y};
#pragma unroll
  for (int s = 0; s < 2; ++s)
  {
    if (refs[s] < 0)
      continue;
    if ((int64_t)refs[s] >= nint)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      continue;
    }
    parent[refs[s]] = (int)(2 * i + s);
  }
}

// Bottom-up KDOP unions.  Thread i writes the records of node i's leaf slots
// and adds their number to the node's counter; whoever brings a counter to 2
// owns the node: it forms the union of the two records, writes it into the
// parent's slot and counts there in turn (each count an acquire-release
// atomic add: the counting thread's record stores are released with it, and
// the owner acquires the other record; records are read through L2).  The
// climb ends at the root, which writes the record of the whole tree.
template <int NDIR>
__global__ void k_kdop_refit(const TNode *__restrict__ tnodes, int64_t nint,
                             const float *__restrict__ kd, int64_t n, const int *__restrict__ parent,
                             unsigned *__restrict__ counters, float4 *__restrict__ knodes,
                             unsigned *__restrict__ err)
{
  constexpr int R = kdop_pad(NDIR) / 4;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nint)
    return;
  const int4 d = tnodes[i].d;
  const int refs[2] = {d.x, d.y}, cfs[2] = {d.z, d.w};
  unsigned leaves = 0;
#pragma unroll
  for (int s = 0; s < 2; ++s)
  {
    if (refs[s] >= 0)
      continue;
    Kdop<NDIR> k;
    const int v = bucket_start(refs[s]);
    if (cfs[s] == 0) // absent child of a one-leaf tree
      kdop_empty<NDIR>(k);
    else if ((int64_t)v < n)
      kdop_load_raw<NDIR>(kd, v, k);
    else
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      kdop_empty<NDIR>(k);
    }
    kdop_store<NDIR>(knodes + (2 * i + s) * R, k);
    ++leaves;
  }
  if (leaves == 0)
    return;
  if (atomic_add_acq_rel(counters + i, leaves) + leaves < 2)
    return;
  int64_t node = i;
  for (int64_t steps = 0;; ++steps)
  {
    if (steps > nint)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      return;
    }
    Kdop<NDIR> a, b;
    kdop_load_cg<NDIR>(knodes + 2 * node * R, a);
    kdop_load_cg<NDIR>(knodes + (2 * node + 1) * R, b);
#pragma unroll
    for (int j = 0; j < NDIR; ++j)
    {
      a.mn[j] = kokkos_min(a.mn[j], b.mn[j]);
      a.mx[j] = kokkos_max(a.mx[j], b.mx[j]);
    }
    const int p = node == 0 ? -1 : parent[node];
    if (p < 0)
    {
      kdop_store<NDIR>(knodes + 2 * nint * R, a);
      return;
    }
    kdop_store<NDIR>(knodes + (int64_t)p * R, a);
    if (atomic_add_acq_rel(counters + (p >> 1), 1u) == 0)
      return;
    node = p >> 1;
  }
}

template <int NDIR>
abx_status kdop_tree_records(cudaStream_t s, const TNode *d_tnodes, const float4 *d_sorted,
                             int64_t n, const float *d_kdops, float4 *d_knodes, float4 *d_kleaves)
{
  unsigned *err = device_state().d_error;
  const int64_t nint = n > 1 ? n - 1 : 1;
  StageScope scope(s, "kdop", 4);
  k_kdop_leaves<NDIR><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_sorted, n, d_kdops, d_kleaves,
                                                                   err);
  ABX_CUDA_TRY(cudaGetLastError());
  Scratch<int> parent;
  Scratch<unsigned> counters;
  ABX_CUDA_TRY(parent.alloc(nint, s));
  ABX_CUDA_TRY(counters.alloc(nint, s));
  ABX_CUDA_TRY(cudaMemsetAsync(parent.ptr, 0xff, nint * sizeof(int), s));
  ABX_CUDA_TRY(cudaMemsetAsync(counters.ptr, 0, nint * sizeof(unsigned), s));
  const unsigned blocks = (unsigned)((nint + 255) / 256);
  k_kdop_parents<<<blocks, 256, 0, s>>>(d_tnodes, nint, parent.ptr, err);
  ABX_CUDA_TRY(cudaGetLastError());
  k_kdop_refit<NDIR><<<blocks, 256, 0, s>>>(d_tnodes, nint, d_kdops, n, parent.ptr, counters.ptr,
                                            d_knodes, err);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

template <int NDIR, int PRED>
abx_status kdop_tree_spatial(cudaStream_t s, TreeView const &t, const float *d_preds, int64_t nq,
                             const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                             const int32_t *d_offsets, int32_t *d_out, int32_t buffer,
                             unsigned *d_overflow)
{
  unsigned *err = device_state().d_error;
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("SPATIAL_BUCKET", kDefaultSpatialBucket)));
  const ForestView f{nullptr, nullptr, 1};
  const float4 *kn = reinterpret_cast<const float4 *>(t.knodes);
  const float4 *kl = reinterpret_cast<const float4 *>(t.kleaves);
#define ABX_KDOP_SPATIAL(M)                                                                      \
  k_spatial<PRED, M, 1, kKeepAll, NDIR><<<blocks, kQueryThreads, 0, s>>>(                         \
      t.tnodes, t.sorted, t.n, f, d_preds, nq, d_perm, d_counts, d_offsets, d_out, buffer, bucket, \
      d_overflow, err, nullptr, kn, kl)
  if (mode == kCount)
    ABX_KDOP_SPATIAL(kCount);
  else if (mode == kFill)
    ABX_KDOP_SPATIAL(kFill);
  else
    ABX_KDOP_SPATIAL(kBuffered);
#undef ABX_KDOP_SPATIAL
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

// intersects(KDOP) predicates on point or box trees, forests and brute force.
template <int PRED, int KIND>
abx_status kdop_pred_spatial(cudaStream_t s, TreeView const &t, ForestView const &f,
                             const float *d_preds, int64_t nq, const uint32_t *d_perm,
                             SpatialMode mode, int32_t *d_counts, const int32_t *d_offsets,
                             int32_t *d_out, int32_t buffer, unsigned *d_overflow)
{
  unsigned *err = device_state().d_error;
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("SPATIAL_BUCKET", kDefaultSpatialBucket)));
#define ABX_SPATIAL(M)                                                                         \
  k_spatial<PRED, M, KIND><<<blocks, kQueryThreads, 0, s>>>(t.tnodes, t.sorted, t.n, f, d_preds, \
                                                            nq, d_perm, d_counts, d_offsets,   \
                                                            d_out, buffer, bucket, d_overflow, err)
#define ABX_BRUTE(M)                                                                           \
  k_brute_spatial<PRED, M, KIND><<<blocks, kQueryThreads, 0, s>>>(                               \
      t.sorted, t.n, d_preds, nq, d_perm, d_counts, d_offsets, d_out, buffer, d_overflow)
  if (!t.tnodes)
  {
    if (mode == kCount)
      ABX_BRUTE(kCount);
    else if (mode == kFill)
      ABX_BRUTE(kFill);
    else
      ABX_BRUTE(kBuffered);
  }
  else if (mode == kCount)
    ABX_SPATIAL(kCount);
  else if (mode == kFill)
    ABX_SPATIAL(kFill);
  else
    ABX_SPATIAL(kBuffered);
#undef ABX_BRUTE
#undef ABX_SPATIAL
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

template <int PRED>
abx_status kdop_pred_dispatch(cudaStream_t s, TreeView const &t, ForestView const &f,
                              const float *d_preds, int64_t nq, const uint32_t *d_perm,
                              SpatialMode mode, int32_t *d_counts, const int32_t *d_offsets,
                              int32_t *d_out, int32_t buffer, unsigned *d_overflow)
{
  constexpr int nd = kdop_ndir(PRED);
  if (t.ndir > 0)
  {
    if (t.ndir != nd)
      return fail(ABX_ERROR_INVALID_ARGUMENT,
                  "intersects(KDOP) on a KDOP tree needs the tree's number of directions");
    return kdop_tree_spatial<nd, PRED>(s, t, d_preds, nq, d_perm, mode, d_counts, d_offsets, d_out,
                                       buffer, d_overflow);
  }
  if (t.kind == ABX_BOX)
    return kdop_pred_spatial<PRED, 1>(s, t, f, d_preds, nq, d_perm, mode, d_counts, d_offsets,
                                      d_out, buffer, d_overflow);
  return kdop_pred_spatial<PRED, 0>(s, t, f, d_preds, nq, d_perm, mode, d_counts, d_offsets, d_out,
                                    buffer, d_overflow);
}

} // namespace

abx_status kdop_from_geometry(cudaStream_t s, abx_geometry src_kind, const float *d_src, int64_t n,
                              abx_geometry kdop_kind, float *d_out)
{
  if (n <= 0)
    return ABX_SUCCESS;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  const bool box = src_kind == ABX_BOX;
#define ABX_FROM(ND)                                                                     \
  (box ? k_kdop_from_geometry<ND, 1><<<blocks, 256, 0, s>>>(d_src, n, d_out)             \
       : k_kdop_from_geometry<ND, 0><<<blocks, 256, 0, s>>>(d_src, n, d_out))
  switch (kdop_ndir(kdop_kind))
  {
  case 3: ABX_FROM(3); break;
  case 7: ABX_FROM(7); break;
  case 9: ABX_FROM(9); break;
  case 13: ABX_FROM(13); break;
  default: return fail(ABX_ERROR_INVALID_ARGUMENT, "not a KDOP kind");
  }
#undef ABX_FROM
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status kdop_axis_boxes(cudaStream_t s, abx_geometry kdop_kind, const float *d_kdops, int64_t n,
                           float *d_boxes)
{
  if (n <= 0)
    return ABX_SUCCESS;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  switch (kdop_ndir(kdop_kind))
  {
  case 3: k_kdop_axis_boxes<3><<<blocks, 256, 0, s>>>(d_kdops, n, d_boxes); break;
  case 7: k_kdop_axis_boxes<7><<<blocks, 256, 0, s>>>(d_kdops, n, d_boxes); break;
  case 9: k_kdop_axis_boxes<9><<<blocks, 256, 0, s>>>(d_kdops, n, d_boxes); break;
  case 13: k_kdop_axis_boxes<13><<<blocks, 256, 0, s>>>(d_kdops, n, d_boxes); break;
  default: return fail(ABX_ERROR_INVALID_ARGUMENT, "not a KDOP kind");
  }
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status kdop_records(cudaStream_t s, abx_geometry kdop_kind, const TNode *d_tnodes,
                        const float4 *d_sorted, int64_t n, const float *d_kdops, float4 *d_knodes,
                        float4 *d_kleaves)
{
  if (n <= 0)
    return ABX_SUCCESS;
  switch (kdop_ndir(kdop_kind))
  {
  case 3: return kdop_tree_records<3>(s, d_tnodes, d_sorted, n, d_kdops, d_knodes, d_kleaves);
  case 7: return kdop_tree_records<7>(s, d_tnodes, d_sorted, n, d_kdops, d_knodes, d_kleaves);
  case 9: return kdop_tree_records<9>(s, d_tnodes, d_sorted, n, d_kdops, d_knodes, d_kleaves);
  case 13: return kdop_tree_records<13>(s, d_tnodes, d_sorted, n, d_kdops, d_knodes, d_kleaves);
  default: return fail(ABX_ERROR_INVALID_ARGUMENT, "not a KDOP kind");
  }
}

abx_status launch_spatial_kdop(cudaStream_t s, TreeView const &t, ForestView const &f,
                               abx_geometry pred_kind, const float *d_preds, int64_t nq,
                               const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                               const int32_t *d_offsets, int32_t *d_out, int32_t buffer,
                               unsigned *d_overflow)
{
#define ABX_ARGS s, t, f, d_preds, nq, d_perm, mode, d_counts, d_offsets, d_out, buffer, d_overflow
  switch (pred_kind)
  {
  case ABX_KDOP6: return kdop_pred_dispatch<ABX_KDOP6>(ABX_ARGS);
  case ABX_KDOP14: return kdop_pred_dispatch<ABX_KDOP14>(ABX_ARGS);
  case ABX_KDOP18: return kdop_pred_dispatch<ABX_KDOP18>(ABX_ARGS);
  case ABX_KDOP26: return kdop_pred_dispatch<ABX_KDOP26>(ABX_ARGS);
  default: break;
  }
#undef ABX_ARGS
  if (pred_kind != ABX_BOX || t.ndir == 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "KDOP trees answer intersects(Box) and intersects(KDOP) predicates only");
  switch (t.ndir)
  {
#define ABX_BOXQ(ND)                                                                               \
  return kdop_tree_spatial<ND, ABX_BOX>(s, t, d_preds, nq, d_perm, mode, d_counts, d_offsets, d_out, \
                                        buffer, d_overflow)
  case 3: ABX_BOXQ(3);
  case 7: ABX_BOXQ(7);
  case 9: ABX_BOXQ(9);
  case 13: ABX_BOXQ(13);
#undef ABX_BOXQ
  default: return fail(ABX_ERROR_INVALID_ARGUMENT, "bad KDOP tree");
  }
}

} // namespace abx
