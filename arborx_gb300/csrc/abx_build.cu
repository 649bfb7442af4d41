// abx_build.cu -- BVH construction kernels.
//
//   k_bounds_partial / k_bounds_final   scene bounding box
//       (calculateBoundingBoxOfTheScene, ArborX_TreeConstruction.hpp:26-39)
//   k_morton64                          63-bit Morton code of every centroid,
//       with the radix sort's 8 digit histograms accumulated on the fly
//       (Morton64, ArborX_SpaceFillingCurves.hpp:45-84)
//   k_morton32                          Morton32 of predicate centroids
//       (ArborX_SpaceFillingCurves.hpp:30-43,86-104) + 4 digit histograms
//   k_hierarchy                         Apetrei bottom-up build with the
//       Karras rule for equal codes (GenerateHierarchy,
//       ArborX_TreeConstruction.hpp:71-348), writing the reference node
//       layout and the 64-byte child-pair traversal layout in one pass.
#include <climits>

#include "abx_build.h"
#include "abx_common.cuh"
#include "abx_internal.h"

namespace abx
{
namespace
{

constexpr int kBoundsThreads = 256;

__device__ __forceinline__ void warp_minmax(float &lo, float &hi)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
}

// Block-reduce a box; thread 0 returns the result.
__device__ __forceinline__ Box3 block_reduce_box(Box3 b)
{
  __shared__ float sh[6][kBoundsThreads / 32];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    warp_minmax(b.lo[d], b.hi[d]);
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      sh[d][w] = b.lo[d];
      sh[3 + d][w] = b.hi[d];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i)
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        b.lo[d] = fminf(b.lo[d], sh[d][i]);
        b.hi[d] = fmaxf(b.hi[d], sh[3 + d][i]);
      }
    }
  }
  return b;
}

// Points: each thread consumes 4 points (three 16-byte loads) per step when
// the array is 16-byte aligned; otherwise scalar loads.
template <int KIND>
__global__ void __launch_bounds__(kBoundsThreads)
    k_bounds_partial(const float *__restrict__ g, int64_t n, float *__restrict__ partial)
{
  Box3 b = empty_box();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (KIND == 0 && (reinterpret_cast<uintptr_t>(g) & 15) == 0)
  {
    const float4 *g4 = reinterpret_cast<const float4 *>(g);
    const int64_t groups = n / 4; // 4 points = 3 float4
    for (int64_t i = tid; i < groups; i += stride)
    {
      float4 u = __ldg(g4 + 3 * i), v = __ldg(g4 + 3 * i + 1), w = __ldg(g4 + 3 * i + 2);
      float xs[4] = {u.x, u.w, v.z, w.y};
      float ys[4] = {u.y, v.x, v.w, w.z};
      float zs[4] = {u.z, v.y, w.x, w.w};
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        b.lo[0] = fminf(b.lo[0], xs[j]); b.hi[0] = fmaxf(b.hi[0], xs[j]);
        b.lo[1] = fminf(b.lo[1], ys[j]); b.hi[1] = fmaxf(b.hi[1], ys[j]);
        b.lo[2] = fminf(b.lo[2], zs[j]); b.hi[2] = fmaxf(b.hi[2], zs[j]);
      }
    }
    for (int64_t i = groups * 4 + tid; i < n; i += stride)
      expand(b, load_leaf_box<0>(g, i));
  }
  else
  {
    for (int64_t i = tid; i < n; i += stride)
      expand(b, load_leaf_box<KIND>(g, i));
  }
  b = block_reduce_box(b);
  if (threadIdx.x == 0)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      partial[6 * blockIdx.x + d] = b.lo[d];
      partial[6 * blockIdx.x + 3 + d] = b.hi[d];
    }
  }
}

__global__ void __launch_bounds__(kBoundsThreads)
    k_bounds_final(const float *__restrict__ partial, int np, float *__restrict__ out)
{
  Box3 b = empty_box();
  for (int i = threadIdx.x; i < np; i += blockDim.x)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      b.lo[d] = fminf(b.lo[d], partial[6 * i + d]);
      b.hi[d] = fmaxf(b.hi[d], partial[6 * i + 3 + d]);
    }
  }
  b = block_reduce_box(b);
  if (threadIdx.x == 0)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      out[d] = b.lo[d];
      out[3 + d] = b.hi[d];
    }
  }
}

// Morton64 codes + digit histograms of the 8 radix passes.
template <int KIND>
__global__ void __launch_bounds__(256)
    k_morton64(const float *__restrict__ g, int64_t n, const float *__restrict__ scene,
               uint64_t *__restrict__ codes, uint32_t *__restrict__ hist)
{
  __shared__ uint32_t sh[8 * 256];
  __shared__ float sc[6];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
    sh[i] = 0;
  if (threadIdx.x < 6)
    sc[threadIdx.x] = scene[threadIdx.x];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    float x, y, z;
    load_centroid<KIND>(g, i, x, y, z);
    uint64_t c = morton64_unit(translate_scale(x, sc[0], sc[3]),
                               translate_scale(y, sc[1], sc[4]),
                               translate_scale(z, sc[2], sc[5]));
    codes[i] = c;
    if (hist)
    {
#pragma unroll
      for (int p = 0; p < 8; ++p)
        atomicAdd(&sh[p * 256 + ((c >> (8 * p)) & 0xff)], 1u);
    }
  }
  if (hist)
  {
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
      if (sh[i])
        atomicAdd(&hist[i], sh[i]);
  }
}

template <int KIND>
__global__ void __launch_bounds__(256)
    k_morton32(const float *__restrict__ g, int64_t n, const float *__restrict__ scene,
               uint32_t *__restrict__ codes, uint32_t *__restrict__ hist)
{
  __shared__ uint32_t sh[4 * 256];
  __shared__ float sc[6];
  for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
    sh[i] = 0;
  if (threadIdx.x < 6)
    sc[threadIdx.x] = scene[threadIdx.x];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    float x, y, z;
    load_centroid<KIND>(g, i, x, y, z);
    uint32_t c = morton32_unit(translate_scale(x, sc[0], sc[3]),
                               translate_scale(y, sc[1], sc[4]),
                               translate_scale(z, sc[2], sc[5]));
    codes[i] = c;
    if (hist)
    {
#pragma unroll
      for (int p = 0; p < 4; ++p)
        atomicAdd(&sh[p * 256 + ((c >> (8 * p)) & 0xff)], 1u);
    }
  }
  if (hist)
  {
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
      if (sh[i])
        atomicAdd(&hist[i], sh[i]);
  }
}

// GenerateHierarchy::delta (ArborX_TreeConstruction.hpp:131-170): xor of
// adjacent sorted codes; equal codes fall back to LLONG_MIN + (i ^ (i + 1));
// the sum is formed in unsigned 64-bit arithmetic and shifted down by one.
__device__ __forceinline__ int64_t h_delta(const uint64_t *__restrict__ codes, int i,
                                           int num_internal)
{
  if (i < 0 || i >= num_internal)
    return INT64_MAX;
  uint64_t x = __ldg(codes + i) ^ __ldg(codes + i + 1);
  uint64_t add = x == 0 ? (0x8000000000000000ull + (uint64_t)(int64_t)(i ^ (i + 1))) : 0ull;
  return (int64_t)(x + add - 1ull);
}

__device__ __forceinline__ Box3 load_internal_box_cg(const InternalNode *node)
{
  const float *f = reinterpret_cast<const float *>(node);
  float2 a = __ldcg(reinterpret_cast<const float2 *>(f + 2));
  float4 b = __ldcg(reinterpret_cast<const float4 *>(f + 4));
  Box3 r;
  r.lo[0] = a.x; r.lo[1] = a.y; r.lo[2] = b.x;
  r.hi[0] = b.y; r.hi[1] = b.z; r.hi[2] = b.w;
  return r;
}

// Count field of a child slot in a TNode: a leaf child is 1; an internal
// child covering c <= kMaxBucket leaves is c, plus kBucketRightEnd when its
// Karras index is the right end of its leaf range (its leaves then start at
// index - c + 1, else at index); larger subtrees are 0.  Query kernels may
// scan such a child's leaves from the Morton-ordered copy instead of
// descending into it.
__device__ __forceinline__ int child_count_field(int kidx, int lo, int hi)
{
  const int c = hi - lo + 1;
  if (c > kMaxBucket)
    return 0;
  return c | (kidx == hi ? kBucketRightEnd : 0);
}

// State of a climb that leaves its CTA (handed from k_hierarchy_local to
// k_hierarchy_global): the node completed last and its leaf range.
struct __align__(16) ClimbState
{
  int i;           // node number (leaf index or n + Karras index)
  int range_left;
  int range_right;
  int cur_node;    // Karras index, or -1 when the node is a leaf
  int original;    // leaf value when cur_node == -1
  int pad[3];
  float lo[3];
  float hi[3];
  float pad2[2];
};
static_assert(sizeof(ClimbState) == 64, "climb state is 64 B");

// Apetrei's climb with global flags (ArborX_TreeConstruction.hpp:197-311):
// relaxed compare-and-swap on the parent's range slot; a release fence before
// it once this thread has written a node record in this kernel (`wrote`;
// records written by an earlier kernel are already visible); an acquire
// fence before reading an internal sibling's box through L2.  The first
// arriver at a parent stops; nothing spins.
template <int KIND>
__device__ __forceinline__ void climb_global(const float *__restrict__ g, int n,
                                             const uint32_t *__restrict__ perm,
                                             const uint64_t *__restrict__ codes,
                                             int *__restrict__ ranges,
                                             InternalNode *__restrict__ internal,
                                             TNode *__restrict__ tnodes, int i, int range_left,
                                             int range_right, int cur_node, int original,
                                             Box3 box, bool wrote)
{
  const int num_internal = n - 1;
  const int root = num_internal + 1;
  long long delta_left = h_delta(codes, range_left - 1, num_internal);
  long long delta_right = h_delta(codes, range_right, num_internal);
  auto rope_of = [&](int rr, long long dr) -> int {
    if (rr != num_internal)
      return dr < h_delta(codes, rr + 1, num_internal) ? rr + 1 : rr + 1 + num_internal + 1;
    return kRopeSentinel;
  };
  do
  {
    const bool is_left_child = delta_right < delta_left;
    const int p = is_left_child ? range_right : range_left - 1;
    const int own_lo = range_left, own_hi = range_right;
    if (wrote)
      fence_acq_rel_gpu(); // release internal[cur_node]
    const int old = atomic_cas_relaxed(ranges + p, -1, is_left_child ? range_left : range_right);
    if (old == -1)
      return;
    int left_child, sib_lo, sib_hi, sib_node;
    if (is_left_child)
    {
      range_right = old;
      left_child = i;
      sib_lo = p + 1;
      sib_hi = range_right;
      sib_node = p + 1;
      delta_right = h_delta(codes, range_right, num_internal);
    }
    else
    {
      range_left = old;
      left_child = (p == range_left) ? p : p + num_internal + 1;
      sib_lo = range_left;
      sib_hi = p;
      sib_node = p;
      delta_left = h_delta(codes, range_left - 1, num_internal);
    }
    const bool sib_leaf = (sib_lo == sib_hi);
    Box3 sib;
    int sib_value = 0;
    if (sib_leaf)
    {
      sib_value = (int)__ldg(perm + sib_lo);
      sib = load_leaf_box<KIND>(g, sib_value);
    }
    else
    {
      fence_acq_rel_gpu(); // acquire internal[sib_node]
      sib = load_internal_box_cg(internal + sib_node);
    }
    const int karras_parent = delta_right < delta_left ? range_right : range_left;
    const int own_ref = cur_node < 0 ? bucket_ref(original) : cur_node;
    const int own_c = cur_node < 0 ? 1 : child_count_field(cur_node, own_lo, own_hi);
    const int sib_ref = sib_leaf ? bucket_ref(sib_value) : sib_node;
    const int sib_c = sib_leaf ? 1 : child_count_field(sib_node, sib_lo, sib_hi);
    tnodes[karras_parent] = is_left_child ? make_tnode(box, own_ref, own_c, sib, sib_ref, sib_c)
                                          : make_tnode(sib, sib_ref, sib_c, box, own_ref, own_c);
    expand(box, sib);
    InternalNode node;
    node.left_child = left_child;
    node.rope = rope_of(range_right, delta_right);
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      node.lo[d] = box.lo[d];
      node.hi[d] = box.hi[d];
    }
    internal[karras_parent] = node;
    wrote = true;
    cur_node = karras_parent;
    i = karras_parent + num_internal + 1;
  } while (i != root);
}

// Apetrei's climb (ArborX_TreeConstruction.hpp:197-311), first regime.
//
// Each CTA owns kHierBlock consecutive leaves [b0, b1].  While the parent a
// thread climbs to covers only leaves of its CTA, the flag exchange and the
// sibling's box go through shared memory (block-scope fences, no global
// atomics).  The parent of a node [L, R] lies inside the CTA iff its other
// child ends inside it: for a left child (split p = R) iff some j in
// [p + 1, b1] has delta(j) >= delta(p), for a right child (split p = L - 1)
// iff some j in [b0 - 1, p - 1] has delta(j) > delta(p) -- read from suffix
// and prefix maxima of the CTA's deltas.  Both children of a parent reach the
// same verdict, so they meet on the same flag.  A thread whose parent leaves
// the CTA records its state in the frontier list and stops, so the CTA
// retires at once; k_hierarchy_global finishes those climbs (when the list is
// full the thread finishes its climb with climb_global itself).  Nothing
// spins: the first arriver at a parent stops.
//
// Every internal node gets its reference-layout record and its 64-byte
// child-pair node; leaf geometry is copied into Morton order on the way.
template <int KIND>
__global__ void __launch_bounds__(kHierBlock)
    k_hierarchy_local(const float *__restrict__ g, int n, const uint32_t *__restrict__ perm,
                      const uint64_t *__restrict__ codes, int *__restrict__ ranges,
                      LeafNode *__restrict__ leaves, InternalNode *__restrict__ internal,
                      TNode *__restrict__ tnodes, float4 *__restrict__ sorted,
                      ClimbState *__restrict__ frontier, unsigned *__restrict__ frontier_count,
                      int frontier_capacity)
{
  __shared__ long long s_delta[kHierBlock + 1]; // delta(b0 - 1 + k)
  __shared__ long long s_pre[kHierBlock + 1];   // max of s_delta[0 .. k]
  __shared__ long long s_suf[kHierBlock + 1];   // max of s_delta[k .. nb]
  __shared__ int s_flag[kHierBlock];            // split p -> s_flag[p - b0]
  __shared__ Box3 s_box[kHierBlock];           // internal node with Karras index in [b0, b1]
  __shared__ Box3 s_leaf[kHierBlock];
  __shared__ int s_value[kHierBlock];

  const int num_internal = n - 1;
  const int root = num_internal + 1;
  const int b0 = blockIdx.x * kHierBlock;
  const int b1 = min(b0 + kHierBlock - 1, n - 1);
  const int nb = b1 - b0 + 1;
  const int tid = threadIdx.x;

  for (int k = tid; k <= nb; k += blockDim.x)
    s_delta[k] = h_delta(codes, b0 - 1 + k, num_internal);
  s_flag[tid] = -1;
  int i = b0 + tid;
  Box3 box = empty_box();
  int original = 0;
  if (i <= b1)
  {
    original = (int)__ldg(perm + i);
    box = load_leaf_box<KIND>(g, original);
    s_leaf[tid] = box;
    s_value[tid] = original;
    SortedLeaf<KIND>::store(sorted, i, box, original);
  }
  __syncthreads();
  // inclusive prefix maxima s_pre[k] = max(s_delta[0..k]) and suffix maxima
  // s_suf[k] = max(s_delta[k..nb]) for k in [0, nb], nb <= kHierBlock:
  // warp shuffles, then the maxima of the warps before / after
  {
    __shared__ long long w_pre[kHierBlock / 32];
    __shared__ long long w_suf[kHierBlock / 32];
    const int lane = tid & 31, warp = tid >> 5;
    const long long v = tid <= nb ? s_delta[tid] : LLONG_MIN;
    long long pre = v, suf = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const long long a = __shfl_up_sync(0xffffffffu, pre, o);
      const long long b = __shfl_down_sync(0xffffffffu, suf, o);
      if (lane >= o)
        pre = max(pre, a);
      if (lane + o < 32)
        suf = max(suf, b);
    }
    if (lane == 31)
      w_pre[warp] = pre;
    if (lane == 0)
      w_suf[warp] = suf;
    __syncthreads();
    for (int w = 0; w < warp; ++w)
      pre = max(pre, w_pre[w]);
    for (int w = warp + 1; w < kHierBlock / 32; ++w)
      suf = max(suf, w_suf[w]);
    // entry nb = kHierBlock (a full CTA) lies past the last thread
    const long long last = nb == kHierBlock ? s_delta[kHierBlock] : LLONG_MIN;
    if (tid <= nb)
    {
      s_pre[tid] = pre;
      s_suf[tid] = max(suf, last);
    }
    if (nb == kHierBlock && tid == kHierBlock - 1)
    {
      s_pre[kHierBlock] = max(pre, last);
      s_suf[kHierBlock] = last;
    }
    __syncthreads();
  }
  if (i > b1)
    return;

  // delta(j) for j in [b0 - 1, b1]
  auto delta_at = [&](int j) -> long long { return s_delta[j - b0 + 1]; };
  // GenerateHierarchy::setRope (ArborX_TreeConstruction.hpp:173-195)
  auto rope_of = [&](int range_right, long long delta_right) -> int {
    if (range_right != num_internal)
    {
      const long long next = range_right + 1 <= b1 ? delta_at(range_right + 1)
                                                    : h_delta(codes, range_right + 1, num_internal);
      return delta_right < next ? range_right + 1 : range_right + 1 + num_internal + 1;
    }
    return kRopeSentinel;
  };

  int range_left = i, range_right = i;
  long long delta_left = delta_at(range_left - 1);
  long long delta_right = delta_at(range_right);
  LeafNode leaf;
  leaf.rope = rope_of(range_right, delta_right);
  leaf.value = original;
  leaves[i] = leaf;

  int cur_node = -1; // Karras index of the node this thread completed last
  do
  {
    const bool is_left_child = delta_right < delta_left;
    const int p = is_left_child ? range_right : range_left - 1;
    const bool inside = is_left_child ? (p < b1 && s_suf[p - b0 + 2] >= delta_right)
                                      : (p >= b0 && s_pre[p - b0] > delta_left);
    if (!inside)
    {
      const unsigned slot = atomicAdd(frontier_count, 1u);
      if ((int)slot >= frontier_capacity)
      {
        // list full (very deep trees): finish this climb here instead
        climb_global<KIND>(g, n, perm, codes, ranges, internal, tnodes, i, range_left,
                           range_right, cur_node, original, box, cur_node >= 0);
        return;
      }
      ClimbState st;
      st.i = i;
      st.range_left = range_left;
      st.range_right = range_right;
      st.cur_node = cur_node;
      st.original = original;
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        st.lo[d] = box.lo[d];
        st.hi[d] = box.hi[d];
      }
      frontier[slot] = st;
      return;
    }
    const int own_lo = range_left, own_hi = range_right;
    __threadfence_block(); // release s_box[cur_node - b0]
    const int old = atomicCAS(s_flag + (p - b0), -1, is_left_child ? range_left : range_right);
    if (old == -1)
      return;
    __threadfence_block(); // acquire the sibling's s_box entry
    int left_child, sib_lo, sib_hi, sib_node;
    if (is_left_child)
    {
      range_right = old;
      left_child = i;
      sib_lo = p + 1;
      sib_hi = range_right;
      sib_node = p + 1;
      delta_right = delta_at(range_right);
    }
    else
    {
      range_left = old;
      left_child = (p == range_left) ? p : p + num_internal + 1;
      sib_lo = range_left;
      sib_hi = p;
      sib_node = p;
      delta_left = delta_at(range_left - 1);
    }
    const bool sib_leaf = (sib_lo == sib_hi);
    const Box3 sib = sib_leaf ? s_leaf[sib_lo - b0] : s_box[sib_node - b0];
    const int sib_value = sib_leaf ? s_value[sib_lo - b0] : 0;
    const int karras_parent = delta_right < delta_left ? range_right : range_left;

    const int own_ref = cur_node < 0 ? bucket_ref(original) : cur_node;
    const int own_c = cur_node < 0 ? 1 : child_count_field(cur_node, own_lo, own_hi);
    const int sib_ref = sib_leaf ? bucket_ref(sib_value) : sib_node;
    const int sib_c = sib_leaf ? 1 : child_count_field(sib_node, sib_lo, sib_hi);
    tnodes[karras_parent] = is_left_child ? make_tnode(box, own_ref, own_c, sib, sib_ref, sib_c)
                                          : make_tnode(sib, sib_ref, sib_c, box, own_ref, own_c);
    expand(box, sib);
    InternalNode node;
    node.left_child = left_child;
    node.rope = rope_of(range_right, delta_right);
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      node.lo[d] = box.lo[d];
      node.hi[d] = box.hi[d];
    }
    internal[karras_parent] = node;
    s_box[karras_parent - b0] = box;
    cur_node = karras_parent;
    i = karras_parent + num_internal + 1;
  } while (i != root);
}

// Second regime: the climbs handed over by k_hierarchy_local.  Their node
// records were written by the previous kernel.
template <int KIND>
__global__ void __launch_bounds__(256)
    k_hierarchy_global(const float *__restrict__ g, int n, const uint32_t *__restrict__ perm,
                       const uint64_t *__restrict__ codes, int *__restrict__ ranges,
                       InternalNode *__restrict__ internal, TNode *__restrict__ tnodes,
                       const ClimbState *__restrict__ frontier,
                       const unsigned *__restrict__ frontier_count, int capacity)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= min((int)*frontier_count, capacity))
    return;
  const ClimbState st = frontier[e];
  Box3 box;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    box.lo[d] = st.lo[d];
    box.hi[d] = st.hi[d];
  }
  climb_global<KIND>(g, n, perm, codes, ranges, internal, tnodes, st.i, st.range_left,
                     st.range_right, st.cur_node, st.original, box, false);
}

// One-leaf tree (ArborX_TreeConstruction.hpp:41-69): leaf {-1, 0}; the
// traversal node holds a one-leaf bucket on the left and nothing on the
// right (count 0).
template <int KIND>
__global__ void k_single_leaf(const float *__restrict__ g, LeafNode *__restrict__ leaves,
                              TNode *__restrict__ tnodes, float4 *__restrict__ sorted,
                              float *__restrict__ bounds)
{
  Box3 b = load_leaf_box<KIND>(g, 0);
  leaves[0].rope = kRopeSentinel;
  leaves[0].value = 0;
  SortedLeaf<KIND>::store(sorted, 0, b, 0);
  tnodes[0] = make_tnode(b, bucket_ref(0), 1, empty_box(), bucket_ref(0), 0); // leaf value 0
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    bounds[d] = b.lo[d];
    bounds[3 + d] = b.hi[d];
  }
}

template <int KIND>
abx_status launch_bounds_t(cudaStream_t s, const float *g, int64_t n, float *out)
{
  DeviceState &ds = device_state();
  int blocks = (int)std::min<int64_t>(std::max<int64_t>((n + 4 * kBoundsThreads - 1) /
                                                            (4 * kBoundsThreads),
                                                        1),
                                      (int64_t)ds.num_sms * 4);
  Scratch<float> partial;
  ABX_CUDA_TRY(partial.alloc(6 * (size_t)blocks, s));
  StageScope scope(s, "bounds", 2);
  k_bounds_partial<KIND><<<blocks, kBoundsThreads, 0, s>>>(g, n, partial.ptr);
  k_bounds_final<<<1, kBoundsThreads, 0, s>>>(partial.ptr, blocks, out);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

int grid_for(int64_t n, int threads, int per_sm)
{
  DeviceState &ds = device_state();
  int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ds.num_sms * per_sm));
}

} // namespace

abx_status scene_bounds(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                        float *d_out)
{
  if (kind == ABX_POINT)
    return launch_bounds_t<0>(s, d_g, n, d_out);
  if (kind == ABX_BOX)
    return launch_bounds_t<1>(s, d_g, n, d_out);
  return fail(ABX_ERROR_INVALID_ARGUMENT, "scene bounds: values must be points or boxes");
}

abx_status morton64_codes(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                          const float *d_scene, uint64_t *d_codes, uint32_t *d_hist)
{
  if (n <= 0)
    return ABX_SUCCESS;
  int blocks = grid_for(n, 256, 8);
  StageScope scope(s, "morton64", 1);
  if (kind == ABX_POINT)
    k_morton64<0><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_BOX)
    k_morton64<1><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_SPHERE)
    k_morton64<2><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status morton32_codes(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                          const float *d_scene, uint32_t *d_codes, uint32_t *d_hist)
{
  if (n <= 0)
    return ABX_SUCCESS;
  int blocks = grid_for(n, 256, 8);
  StageScope scope(s, "morton32", 1);
  if (kind == ABX_POINT)
    k_morton32<0><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_BOX)
    k_morton32<1><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_SPHERE)
    k_morton32<2><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status generate_hierarchy(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                              const uint32_t *d_perm, const uint64_t *d_codes,
                              LeafNode *d_leaves, InternalNode *d_internal, TNode *d_tnodes,
                              float4 *d_sorted)
{
  if (n < 2)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "generate_hierarchy needs at least 2 values");
  if (n > (int64_t)INT32_MAX / 2)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "generate_hierarchy: too many values");
  Scratch<int> ranges;
  ABX_CUDA_TRY(ranges.alloc(n - 1, s));
  ABX_CUDA_TRY(cudaMemsetAsync(ranges.ptr, 0xff, sizeof(int) * (n - 1), s));
  Scratch<TNode> tmp_t;
  if (!d_tnodes)
  {
    ABX_CUDA_TRY(tmp_t.alloc(n - 1, s));
    d_tnodes = tmp_t.ptr;
  }
  Scratch<float4> tmp_sorted;
  if (!d_sorted)
  {
    ABX_CUDA_TRY(tmp_sorted.alloc((size_t)n * (kind == ABX_BOX ? 2 : 1), s));
    d_sorted = tmp_sorted.ptr;
  }
  const unsigned blocks = (unsigned)((n + kHierBlock - 1) / kHierBlock);
  // a CTA's leaf range splits into a few maximal subtrees (2 log2(512) + 2
  // for a balanced tree), each handing over at most one climb; deeper trees
  // that overflow the list finish those climbs in the first kernel
  const int capacity = (int)blocks * 24;
  Scratch<ClimbState> frontier;
  Scratch<unsigned> count;
  ABX_CUDA_TRY(frontier.alloc((size_t)capacity, s));
  ABX_CUDA_TRY(count.alloc(1, s));
  ABX_CUDA_TRY(cudaMemsetAsync(count.ptr, 0, sizeof(unsigned), s));
  const unsigned gblocks = (unsigned)((capacity + 255) / 256);
  StageScope scope(s, "hierarchy", 2);
  if (kind == ABX_POINT)
  {
    k_hierarchy_local<0><<<blocks, kHierBlock, 0, s>>>(d_g, (int)n, d_perm, d_codes, ranges.ptr,
                                                       d_leaves, d_internal, d_tnodes, d_sorted,
                                                       frontier.ptr, count.ptr, capacity);
    k_hierarchy_global<0><<<gblocks, 256, 0, s>>>(d_g, (int)n, d_perm, d_codes, ranges.ptr,
                                                  d_internal, d_tnodes, frontier.ptr, count.ptr,
                                                  capacity);
  }
  else
  {
    k_hierarchy_local<1><<<blocks, kHierBlock, 0, s>>>(d_g, (int)n, d_perm, d_codes, ranges.ptr,
                                                       d_leaves, d_internal, d_tnodes, d_sorted,
                                                       frontier.ptr, count.ptr, capacity);
    k_hierarchy_global<1><<<gblocks, 256, 0, s>>>(d_g, (int)n, d_perm, d_codes, ranges.ptr,
                                                  d_internal, d_tnodes, frontier.ptr, count.ptr,
                                                  capacity);
  }
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status single_leaf(cudaStream_t s, abx_geometry kind, const float *d_g,
                       LeafNode *d_leaves, TNode *d_tnodes, float4 *d_sorted, float *d_bounds)
{
  StageScope scope(s, "hierarchy", 1);
  if (kind == ABX_POINT)
    k_single_leaf<0><<<1, 1, 0, s>>>(d_g, d_leaves, d_tnodes, d_sorted, d_bounds);
  else
    k_single_leaf<1><<<1, 1, 0, s>>>(d_g, d_leaves, d_tnodes, d_sorted, d_bounds);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace abx
