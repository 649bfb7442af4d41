// abx_hierarchy.cu -- Apetrei's bottom-up hierarchy over one or many trees,
// and the per-tree stages of a batched (forest) build.
//
// Trees are segments of one array of Morton-sorted positions: tree s owns
// positions [off[s], off[s + 1]).  Every formula of GenerateHierarchy
// (ArborX_TreeConstruction.hpp:71-348) is evaluated in the tree's own
// numbering: delta() is +inf across a tree boundary and breaks ties of equal
// codes with the tree-local index, leaves and internal nodes are numbered
// inside the tree, values are tree-local input indices.  So a tree built in a
// batch has exactly the node arrays of the same tree built alone.  Storage is
// global: the internal node with Karras index k (a tree-local position) lives
// in slot off[s] + k, i.e. at its global sorted position; a one-leaf tree
// uses slot off[s] for its single traversal node.
#include <climits>

#include "abx_build.h"

namespace abx
{
namespace
{

// GenerateHierarchy::delta (ArborX_TreeConstruction.hpp:131-170) at global
// position j of the tree [lo, hi]: xor of adjacent codes; equal codes fall
// back to LLONG_MIN + (jl ^ (jl + 1)) with the tree-local index jl; the sum is
// formed in unsigned 64-bit arithmetic and shifted down by one; +inf outside
// [lo, hi - 1].
__device__ __forceinline__ long long seg_delta(const uint64_t *__restrict__ codes, int j, int lo,
                                               int hi)
{
  if (j < lo || j >= hi)
    return LLONG_MAX;
  const uint64_t x = __ldg(codes + j) ^ __ldg(codes + j + 1);
  const int jl = j - lo;
  const uint64_t add =
      x == 0 ? (0x8000000000000000ull + (uint64_t)(int64_t)(jl ^ (jl + 1))) : 0ull;
  return (long long)(x + add - 1ull);
}

// delta at global position j, whatever tree j belongs to (its tree among
// segments s_lo..s_hi).
__device__ __forceinline__ long long pos_delta(const uint64_t *__restrict__ codes,
                                               const int64_t *__restrict__ off, int s_lo,
                                               int s_hi, int64_t total, int j)
{
  if (j < 0 || (int64_t)j >= total - 1)
    return LLONG_MAX;
  const int s = find_segment_in(off, s_lo, s_hi, j);
  return seg_delta(codes, j, (int)__ldg(off + s), (int)__ldg(off + s + 1) - 1);
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

// Box of an internal node written by another CTA: the union of the two
// child boxes of its child-pair node, read through L2.
__device__ __forceinline__ Box3 load_tnode_box_cg(const TNode *node)
{
  const float4 *f = reinterpret_cast<const float4 *>(node);
  TNode t;
  t.a = __ldcg(f);
  t.b = __ldcg(f + 1);
  t.c = __ldcg(f + 2);
  Box3 l, r;
  tnode_children(t, l, r);
  expand(l, r);
  return l;
}

// State of a climb that leaves its CTA (handed from k_hierarchy_local to
// k_hierarchy_global).
struct __align__(16) ClimbState
{
  int range_left, range_right; // global positions
  int cur_node;                // global slot of the node completed last, -1 for a leaf
  int value;                   // leaf value when cur_node == -1
  int lo, hi;                  // the tree's positions
  int pad[2];
  float blo[3];
  float bhi[3];
  float pad2[2];
};
static_assert(sizeof(ClimbState) == 64, "climb state is 64 B");

// Child-pair node of the parent with Karras index kp; `box` (the climbing
// child's) becomes the parent's box.
__device__ __forceinline__ void write_parent(TNode *__restrict__ tnodes, int kp,
                                             bool is_left_child, Box3 &box, int own_ref,
                                             int own_c, Box3 const &sib, int sib_ref, int sib_c)
{
  tnodes[kp] = is_left_child ? make_tnode(box, own_ref, own_c, sib, sib_ref, sib_c)
                             : make_tnode(sib, sib_ref, sib_c, box, own_ref, own_c);
  expand(box, sib);
}

// Apetrei's climb with global flags (ArborX_TreeConstruction.hpp:197-311):
// relaxed compare-and-swap on the parent's range slot, preceded by a release
// fence once this thread's node may have been written in this kernel
// (`wrote`); an acquire fence before reading an internal sibling's node
// through L2.  The first arriver at a parent stops; nothing spins.  Stops at
// the tree's root.
template <int KIND>
__device__ void climb_global(const float *__restrict__ g, const uint32_t *__restrict__ perm,
                             const uint64_t *__restrict__ codes, int *__restrict__ ranges,
                             TNode *__restrict__ tnodes, ClimbState st, bool wrote)
{
  const int lo = st.lo, hi = st.hi;
  int range_left = st.range_left, range_right = st.range_right;
  int cur_node = st.cur_node;
  Box3 box;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    box.lo[d] = st.blo[d];
    box.hi[d] = st.bhi[d];
  }
  long long delta_left = seg_delta(codes, range_left - 1, lo, hi);
  long long delta_right = seg_delta(codes, range_right, lo, hi);
  while (!(range_left == lo && range_right == hi))
  {
    const bool is_left_child = delta_right < delta_left;
    const int p = is_left_child ? range_right : range_left - 1;
    const int own_lo = range_left, own_hi = range_right;
    if (wrote)
      fence_acq_rel_gpu(); // release tnodes[cur_node]
    const int old = atomic_cas_relaxed(ranges + p, -1, is_left_child ? range_left : range_right);
    if (old == -1)
      return;
    int sib_lo, sib_hi;
    if (is_left_child)
    {
      range_right = old;
      sib_lo = p + 1;
      sib_hi = range_right;
      delta_right = seg_delta(codes, range_right, lo, hi);
    }
    else
    {
      range_left = old;
      sib_lo = range_left;
      sib_hi = p;
      delta_left = seg_delta(codes, range_left - 1, lo, hi);
    }
    const int sib_node = is_left_child ? p + 1 : p;
    const bool sib_leaf = (sib_lo == sib_hi);
    Box3 sib;
    int sib_value = 0;
    if (sib_leaf)
    {
      sib_value = (int)__ldg(perm + sib_lo) - lo;
      sib = load_leaf_box<KIND>(g, sib_value + lo);
    }
    else
    {
      fence_acq_rel_gpu(); // acquire tnodes[sib_node]
      sib = load_tnode_box_cg(tnodes + sib_node);
    }
    const int kp = delta_right < delta_left ? range_right : range_left;
    const int own_ref = cur_node < 0 ? bucket_ref(st.value) : cur_node;
    const int own_c = cur_node < 0 ? 1 : child_count_field(cur_node, own_lo, own_hi);
    const int sib_ref = sib_leaf ? bucket_ref(sib_value) : sib_node;
    const int sib_c = sib_leaf ? 1 : child_count_field(sib_node, sib_lo, sib_hi);
    write_parent(tnodes, kp, is_left_child, box, own_ref, own_c, sib, sib_ref, sib_c);
    wrote = true;
    cur_node = kp;
  }
}

// The second arriver at the flag of split p creates the parent of its node
// [L, R] (slot `node`, -1 for the leaf L) and the sibling: writes the
// parent's child-pair node and box, and moves (L, R, node) up to the parent.
__device__ __forceinline__ void make_parent(TNode *__restrict__ tnodes, const long long *s_delta,
                                            const Box3 *s_leaf, const int *s_value, Box3 *s_box,
                                            int b0, bool is_left_child, int p, int old, int &L,
                                            int &R, int &node)
{
  int nl = L, nr = R, sib_lo, sib_hi;
  if (is_left_child)
  {
    nr = old;
    sib_lo = p + 1;
    sib_hi = nr;
  }
  else
  {
    nl = old;
    sib_lo = nl;
    sib_hi = p;
  }
  const int sib_node = is_left_child ? p + 1 : p;
  const bool sib_leaf = sib_lo == sib_hi;
  Box3 box = node < 0 ? s_leaf[L - b0] : s_box[node - b0];
  const Box3 sib = sib_leaf ? s_leaf[sib_lo - b0] : s_box[sib_node - b0];
  const int sib_ref = sib_leaf ? bucket_ref(s_value[sib_lo - b0]) : sib_node;
  const int sib_c = sib_leaf ? 1 : child_count_field(sib_node, sib_lo, sib_hi);
  const int own_ref = node < 0 ? bucket_ref(s_value[L - b0]) : node;
  const int own_c = node < 0 ? 1 : child_count_field(node, L, R);
  const int kp = s_delta[nr - b0 + 1] < s_delta[nl - b0] ? nr : nl;
  write_parent(tnodes, kp, is_left_child, box, own_ref, own_c, sib, sib_ref, sib_c);
  s_box[kp - b0] = box;
  L = nl;
  R = nr;
  node = kp;
}

// Apetrei's climb, first regime.
//
// Each CTA owns kHierBlock consecutive positions [b0, b1].  Work items are
// the nodes whose parent is still to be reached: (range, node), the leaves
// first.  In a round every item tries its parent's flag in shared memory; the
// second arriver creates the parent, which is an item of the next round.
// Every sibling an item reads was created in an earlier round, so the
// barrier (or __syncwarp) between rounds orders all shared-memory boxes.  The
// list is compacted every round while it holds more than 32 items (about
// log2(kHierBlock / 32) rounds); warp 0 then finishes alone, one item per
// lane, so idle warps do not cycle through the tail rounds.
//
// The parent of a node [L, R] lies inside the CTA iff its other child ends
// inside it: for a left child (split p = R) iff some j in [p + 1, b1] has
// delta(j) >= delta(p), for a right child (split p = L - 1) iff some j in
// [b0 - 1, p - 1] has delta(j) > delta(p) -- read from suffix and prefix
// maxima of the CTA's deltas (tree boundaries have delta = +inf).  Both
// children of a parent reach the same verdict, so they meet on the same
// flag.  An item whose parent leaves the CTA goes to the frontier list,
// finished by k_hierarchy_global (or in place when the list is full).
//
// Writes the 64-byte child-pair node of every internal node and the leaf
// geometry in Morton order; the reference-layout arrays are derived from
// them on demand (export_reference_layout).
// Five CTAs per SM (at most 51 registers): with four the climb is ~15% slower.
template <int KIND>
__global__ void __launch_bounds__(kHierBlock, 5)
    k_hierarchy_local(const float *__restrict__ g, int64_t total, const int64_t *__restrict__ off,
                      int nseg, const uint32_t *__restrict__ perm,
                      const uint64_t *__restrict__ codes, int *__restrict__ ranges,
                      TNode *__restrict__ tnodes, float4 *__restrict__ sorted,
                      ClimbState *__restrict__ frontier, unsigned *__restrict__ frontier_count,
                      int frontier_capacity)
{
  __shared__ long long s_delta[kHierBlock + 1]; // delta(b0 - 1 + k)
  __shared__ long long s_pre[kHierBlock + 1];   // max of s_delta[0 .. k]
  __shared__ long long s_suf[kHierBlock + 1];   // max of s_delta[k .. nb]
  __shared__ int s_flag[kHierBlock];            // split p -> s_flag[p - b0]
  __shared__ Box3 s_box[kHierBlock];           // internal node with slot in [b0, b1]
  __shared__ Box3 s_leaf[kHierBlock];
  __shared__ int s_value[kHierBlock];
  __shared__ int3 s_items[2][kHierBlock];       // (range_left, range_right, node or -1)
  __shared__ int s_count[2];

  __shared__ int s_seg[2]; // the trees of positions b0 - 1 .. b1 + 1
  const int b0 = blockIdx.x * kHierBlock;
  const int b1 = (int)min((int64_t)b0 + kHierBlock - 1, total - 1);
  const int nb = b1 - b0 + 1;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  if (tid < 2)
    s_seg[tid] = nseg > 1 ? find_segment(off, nseg,
                                         tid == 0 ? max(b0 - 1, 0) : min((int64_t)b1 + 1, total - 1))
                          : 0;
  __syncthreads();
  const int seg_lo = s_seg[0], seg_hi = s_seg[1];

  for (int k = tid; k <= nb; k += blockDim.x)
    s_delta[k] = pos_delta(codes, off, seg_lo, seg_hi, total, b0 - 1 + k);
  s_flag[tid] = -1;
  if (tid < 2)
    s_count[tid] = 0;
  const int i = b0 + tid;
  if (i <= b1)
  {
    const int s = find_segment_in(off, seg_lo, seg_hi, i);
    const int lo = (int)__ldg(off + s);
    const int hi = (int)__ldg(off + s + 1) - 1;
    const int original = (int)__ldg(perm + i);
    const int value = original - lo;
    const Box3 box = load_leaf_box<KIND>(g, original);
    s_leaf[tid] = box;
    s_value[tid] = value;
    SortedLeaf<KIND>::store(sorted, i, box, value);
    s_items[0][tid] = make_int3(i, i, -1);
    if (lo == hi)
      // one-leaf tree (ArborX_TreeConstruction.hpp:41-69): a one-leaf
      // bucket on the left, nothing on the right (count 0)
      tnodes[lo] = make_tnode(box, bucket_ref(value), 1, empty_box(), bucket_ref(0), 0);
  }
  __syncthreads();
  // inclusive prefix maxima s_pre[k] = max(s_delta[0..k]) and suffix maxima
  // s_suf[k] = max(s_delta[k..nb]) for k in [0, nb], nb <= kHierBlock:
  // warp shuffles, then the maxima of the warps before / after
  {
    __shared__ long long w_pre[kHierBlock / 32];
    __shared__ long long w_suf[kHierBlock / 32];
    const int warp = tid >> 5;
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

  // One climb step of the item (L, R, node): returns true when the item
  // moves up to the parent it created.
  auto step = [&](int &L, int &R, int &node) -> bool {
    const long long dl = s_delta[L - b0];
    const long long dr = s_delta[R - b0 + 1];
    if (dl == LLONG_MAX && dr == LLONG_MAX) // the root of a tree
      return false;
    const bool is_left_child = dr < dl;
    const int p = is_left_child ? R : L - 1;
    const bool inside = is_left_child ? (p < b1 && s_suf[p - b0 + 2] >= dr)
                                      : (p >= b0 && s_pre[p - b0] > dl);
    if (!inside)
    {
      const Box3 box = node < 0 ? s_leaf[L - b0] : s_box[node - b0];
      ClimbState st;
      st.range_left = L;
      st.range_right = R;
      st.cur_node = node;
      st.value = node < 0 ? s_value[L - b0] : 0;
      const int s = find_segment_in(off, seg_lo, seg_hi, L);
      st.lo = (int)__ldg(off + s);
      st.hi = (int)__ldg(off + s + 1) - 1;
      st.pad[0] = st.pad[1] = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        st.blo[d] = box.lo[d];
        st.bhi[d] = box.hi[d];
      }
      st.pad2[0] = st.pad2[1] = 0.f;
      const unsigned slot = atomicAdd(frontier_count, 1u);
      if ((int)slot < frontier_capacity)
        frontier[slot] = st;
      else // list full (very deep trees): finish this climb here
        climb_global<KIND>(g, perm, codes, ranges, tnodes, st, true);
      return false;
    }
    const int old = atomicCAS(s_flag + (p - b0), -1, is_left_child ? L : R);
    if (old == -1)
      return false;
    make_parent(tnodes, s_delta, s_leaf, s_value, s_box, b0, is_left_child, p, old, L, R, node);
    return true;
  };

  // CTA-wide rounds over a compacted item list while it holds more than a
  // warp's worth of items
  int cur = 0;
  int count = nb;
  while (count > 32)
  {
    bool emit = false;
    int L = 0, R = 0, node = -1;
    if (tid < count)
    {
      const int3 it = s_items[cur][tid];
      L = it.x;
      R = it.y;
      node = it.z;
      emit = step(L, R, node);
    }
    const int nxt = cur ^ 1;
    const unsigned mask = __ballot_sync(0xffffffffu, emit);
    if (mask)
    {
      const int leader = __ffs(mask) - 1;
      int base = 0;
      if (lane == leader)
        base = atomicAdd(&s_count[nxt], __popc(mask));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (emit)
        s_items[nxt][base + __popc(mask & lanemask_lt())] = make_int3(L, R, node);
    }
    __syncthreads();
    count = s_count[nxt];
    if (tid == 0)
      s_count[cur] = 0;
    cur = nxt;
    __syncthreads();
  }
  // the rest by warp 0 alone: one item per lane, warp-synchronous rounds
  if (tid >= 32)
    return;
  int L = 0, R = 0, node = -1;
  bool active = lane < count;
  if (active)
  {
    const int3 it = s_items[cur][lane];
    L = it.x;
    R = it.y;
    node = it.z;
  }
  while (__any_sync(0xffffffffu, active))
  {
    if (active)
      active = step(L, R, node);
    __syncwarp();
  }
}

// Second regime: the climbs handed over by k_hierarchy_local.  Their nodes
// were written by the previous kernel.
template <int KIND>
__global__ void __launch_bounds__(256)
    k_hierarchy_global(const float *__restrict__ g, const uint32_t *__restrict__ perm,
                       const uint64_t *__restrict__ codes, int *__restrict__ ranges,
                       TNode *__restrict__ tnodes, const ClimbState *__restrict__ frontier,
                       const unsigned *__restrict__ frontier_count, int capacity)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= min((int)*frontier_count, capacity))
    return;
  climb_global<KIND>(g, perm, codes, ranges, tnodes, frontier[e], false);
}

// ---------------------------------------------------------------------------
// Reference-layout node arrays, derived from the child-pair nodes
// ---------------------------------------------------------------------------

// Leaf values in Morton order and their inverse (value -> leaf number).
template <int KIND>
__global__ void k_export_values(const float4 *__restrict__ sorted, int64_t lo, int n,
                                LeafNode *__restrict__ leaves, int *__restrict__ inv,
                                unsigned *__restrict__ err)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n)
    return;
  Box3 b;
  int v;
  SortedLeaf<KIND>::load(sorted, lo + p, b, v);
  leaves[p].value = v;
  if (n == 1)
    leaves[p].rope = kRopeSentinel;
  if ((unsigned)v < (unsigned)n)
    inv[v] = p;
  else
    raise_error(err, ABX_DEVERR_INTERNAL);
}

// Node number of a child reference of the tree whose slots start at lo.
__device__ __forceinline__ int child_number(int ref, int64_t lo, int n, const int *__restrict__ inv)
{
  return ref >= 0 ? (int)(ref - lo) + n : inv[bucket_start(ref)];
}

// Left child, box and parent links of every internal node (Karras index k,
// node number n + k; ArborX_HappyTreeFriends.hpp:23-86 numbering).
__global__ void k_export_internal(const TNode *__restrict__ tnodes, int64_t lo, int n,
                                  const int *__restrict__ inv, InternalNode *__restrict__ internal,
                                  int *__restrict__ parent, int *__restrict__ right,
                                  unsigned *__restrict__ err)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n - 1)
    return;
  const TNode t = tnodes[lo + k];
  Box3 l, r;
  tnode_children(t, l, r);
  expand(l, r);
  const int lc = child_number(t.d.x, lo, n, inv);
  const int rc = child_number(t.d.y, lo, n, inv);
  if ((unsigned)lc >= (unsigned)(2 * n - 1) || (unsigned)rc >= (unsigned)(2 * n - 1))
  {
    raise_error(err, ABX_DEVERR_INTERNAL);
    return;
  }
  InternalNode node;
  node.left_child = lc;
  node.rope = kRopeSentinel;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    node.lo[d] = l.lo[d];
    node.hi[d] = l.hi[d];
  }
  internal[k] = node;
  parent[lc] = 2 * k;
  parent[rc] = 2 * k + 1;
  right[k] = rc;
}

// Ropes (GenerateHierarchy::setRope, ArborX_TreeConstruction.hpp:173-195):
// the rope of a node is the right sibling of its nearest ancestor-or-self
// that is a left child; the sentinel when there is none.
__global__ void k_export_ropes(int n, const int *__restrict__ parent, const int *__restrict__ right,
                               LeafNode *__restrict__ leaves, InternalNode *__restrict__ internal,
                               unsigned *__restrict__ err)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= 2 * n - 1)
    return;
  int y = x, rope = kRopeSentinel;
  for (int steps = 0; y != n; ++steps)
  {
    const int e = parent[y];
    if (steps > 2 * n || (unsigned)(e >> 1) >= (unsigned)(n - 1))
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      break;
    }
    if ((e & 1) == 0)
    {
      rope = right[e >> 1];
      break;
    }
    y = (e >> 1) + n;
  }
  if (x < n)
    leaves[x].rope = rope;
  else
    internal[x - n].rope = rope;
}

// ---------------------------------------------------------------------------
// Per-tree stages of a forest build
// ---------------------------------------------------------------------------

__device__ __forceinline__ void block_reduce_box(Box3 &b)
{
  __shared__ float sh[6][8];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      b.lo[d] = fminf(b.lo[d], __shfl_xor_sync(0xffffffffu, b.lo[d], o));
      b.hi[d] = fmaxf(b.hi[d], __shfl_xor_sync(0xffffffffu, b.hi[d], o));
    }
  }
  const int w = threadIdx.x >> 5;
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
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        b.lo[d] = fminf(b.lo[d], sh[d][k]);
        b.hi[d] = fmaxf(b.hi[d], sh[3 + d][k]);
      }
    }
  }
}

// Bounding box of every tree (one CTA per tree; empty trees get the empty box).
template <int KIND>
__global__ void __launch_bounds__(256)
    k_forest_bounds(const float *__restrict__ g, const int64_t *__restrict__ off,
                    float *__restrict__ bounds)
{
  const int s = blockIdx.x;
  const int64_t a = off[s], e = off[s + 1];
  Box3 b = empty_box();
  for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x)
    expand(b, load_leaf_box<KIND>(g, i));
  block_reduce_box(b);
  if (threadIdx.x == 0)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      bounds[6 * s + d] = b.lo[d];
      bounds[6 * s + 3 + d] = b.hi[d];
    }
  }
}

__device__ __forceinline__ uint64_t morton64_in(float x, float y, float z, const float *sc)
{
  return morton64_unit(translate_scale(x, sc[0], sc[3]), translate_scale(y, sc[1], sc[4]),
                       translate_scale(z, sc[2], sc[5]));
}

// Morton64 code of every value against its own tree's box (one CTA per
// tree), with the 8 digit histograms of the radix sort.
template <int KIND>
__global__ void __launch_bounds__(256)
    k_forest_morton64(const float *__restrict__ g, const int64_t *__restrict__ off,
                      const float *__restrict__ bounds, uint64_t *__restrict__ codes,
                      uint32_t *__restrict__ hist)
{
  __shared__ uint32_t sh[8 * 256];
  __shared__ float sc[6];
  const int s = blockIdx.x;
  for (int k = threadIdx.x; k < 8 * 256; k += blockDim.x)
    sh[k] = 0;
  if (threadIdx.x < 6)
    sc[threadIdx.x] = bounds[6 * s + threadIdx.x];
  __syncthreads();
  const int64_t a = off[s], e = off[s + 1];
  for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x)
  {
    float x, y, z;
    load_centroid<KIND>(g, i, x, y, z);
    const uint64_t c = morton64_in(x, y, z, sc);
    codes[i] = c;
#pragma unroll
    for (int p = 0; p < 8; ++p)
      atomicAdd(&sh[p * 256 + ((c >> (8 * p)) & 0xff)], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 8 * 256; k += blockDim.x)
    if (sh[k])
      atomicAdd(&hist[k], sh[k]);
}

// keys[i] = tree of the value at sorted position i (its original index is
// random, so the search runs over a shared-memory copy of the offsets when
// they fit).
constexpr int kSmemOffsets = 6144;

__global__ void k_tree_keys(const uint32_t *__restrict__ perm, const int64_t *__restrict__ off,
                            int nseg, int64_t total, uint32_t *__restrict__ keys)
{
  __shared__ int64_t s_off[kSmemOffsets];
  const bool staged = nseg + 1 <= kSmemOffsets;
  if (staged)
    for (int k = threadIdx.x; k <= nseg; k += blockDim.x)
      s_off[k] = off[k];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total)
    keys[i] = (uint32_t)(staged ? find_segment_in(s_off, 0, nseg - 1, perm[i])
                                : find_segment(off, nseg, perm[i]));
}

// The trees of a CTA's consecutive positions [first, first + blockDim.x):
// thread 0 and 1 find the two ends once.
__device__ __forceinline__ void block_segments(const int64_t *__restrict__ off, int nseg,
                                               int64_t first, int64_t total, int *s_seg)
{
  if (threadIdx.x < 2)
  {
    const int64_t p =
        threadIdx.x == 0 ? first : min(first + (int64_t)blockDim.x - 1, total - 1);
    s_seg[threadIdx.x] = find_segment(off, nseg, p);
  }
  __syncthreads();
}

// Morton64 code of the value at every sorted position (after the regroup by
// tree), recomputed with the same arithmetic as k_forest_morton64.
template <int KIND>
__global__ void k_forest_codes(const float *__restrict__ g, const uint32_t *__restrict__ perm,
                               const int64_t *__restrict__ off, int nseg, int64_t total,
                               const float *__restrict__ bounds, uint64_t *__restrict__ codes)
{
  __shared__ int s_seg[2];
  const int64_t first = (int64_t)blockIdx.x * blockDim.x;
  block_segments(off, nseg, first, total, s_seg);
  const int64_t i = first + threadIdx.x;
  if (i >= total)
    return;
  const int s = find_segment_in(off, s_seg[0], s_seg[1], i);
  float sc[6];
#pragma unroll
  for (int d = 0; d < 6; ++d)
    sc[d] = __ldg(bounds + 6 * s + d);
  float x, y, z;
  load_centroid<KIND>(g, perm[i], x, y, z);
  codes[i] = morton64_in(x, y, z, sc);
}

// Predicate ordering key of a forest query: its tree above the Morton32 code
// of its centroid in that tree's box (ArborX_LinearBVH.hpp:287-306 per tree).
// A 32-bit key keeps the top 32 - tree_bits bits of the 30-bit code (the
// order only serves coherence); otherwise tree << 32 | code.
template <int KIND, class Key>
__global__ void k_forest_query_keys(const float *__restrict__ preds,
                                    const int64_t *__restrict__ qoff, int nseg, int tree_bits,
                                    int64_t nq, const float *__restrict__ bounds,
                                    Key *__restrict__ keys)
{
  __shared__ int s_seg[2];
  const int64_t first = (int64_t)blockIdx.x * blockDim.x;
  block_segments(qoff, nseg, first, nq, s_seg);
  const int64_t q = first + threadIdx.x;
  if (q >= nq)
    return;
  const int s = find_segment_in(qoff, s_seg[0], s_seg[1], q);
  const float *sc = bounds + 6 * s;
  float x, y, z;
  load_centroid<KIND>(preds, q, x, y, z);
  const uint32_t c = morton32_unit(translate_scale(x, __ldg(sc), __ldg(sc + 3)),
                                   translate_scale(y, __ldg(sc + 1), __ldg(sc + 4)),
                                   translate_scale(z, __ldg(sc + 2), __ldg(sc + 5)));
  if (sizeof(Key) == 8)
    keys[q] = (Key)(((uint64_t)s << 32) | c);
  else
  {
    const int shift = tree_bits > 2 ? tree_bits - 2 : 0;
    keys[q] = (Key)((tree_bits ? ((uint32_t)s << (32 - tree_bits)) : 0u) | (c >> shift));
  }
}

__global__ void k_one_segment(int64_t *off, int64_t n)
{
  off[0] = 0;
  off[1] = n;
}

} // namespace

abx_status generate_hierarchy_segments(cudaStream_t s, abx_geometry kind, const float *d_g,
                                       int64_t total, const int64_t *d_off, int nseg,
                                       const uint32_t *d_perm, const uint64_t *d_codes,
                                       TNode *d_tnodes, float4 *d_sorted)
{
  if (total < 1)
    return ABX_SUCCESS;
  if (total > (int64_t)INT32_MAX / 2)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "generate_hierarchy: too many values");
  Scratch<int> ranges;
  ABX_CUDA_TRY(ranges.alloc(total, s));
  ABX_CUDA_TRY(cudaMemsetAsync(ranges.ptr, 0xff, sizeof(int) * total, s));
  Scratch<float4> tmp_sorted;
  if (!d_sorted)
  {
    ABX_CUDA_TRY(tmp_sorted.alloc((size_t)total * (kind == ABX_BOX ? 2 : 1), s));
    d_sorted = tmp_sorted.ptr;
  }
  const unsigned blocks = (unsigned)((total + kHierBlock - 1) / kHierBlock);
  // a CTA's positions split into a few maximal subtrees (2 log2(kHierBlock) + 2 for
  // a balanced tree), each handing over at most one climb; deeper trees that
  // overflow the list finish those climbs in the first kernel
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
    k_hierarchy_local<0><<<blocks, kHierBlock, 0, s>>>(d_g, total, d_off, nseg, d_perm, d_codes,
                                                       ranges.ptr, d_tnodes, d_sorted,
                                                       frontier.ptr, count.ptr, capacity);
    k_hierarchy_global<0><<<gblocks, 256, 0, s>>>(d_g, d_perm, d_codes, ranges.ptr, d_tnodes,
                                                  frontier.ptr, count.ptr, capacity);
  }
  else
  {
    k_hierarchy_local<1><<<blocks, kHierBlock, 0, s>>>(d_g, total, d_off, nseg, d_perm, d_codes,
                                                       ranges.ptr, d_tnodes, d_sorted,
                                                       frontier.ptr, count.ptr, capacity);
    k_hierarchy_global<1><<<gblocks, 256, 0, s>>>(d_g, d_perm, d_codes, ranges.ptr, d_tnodes,
                                                  frontier.ptr, count.ptr, capacity);
  }
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
  Scratch<TNode> tmp_t;
  if (!d_tnodes)
  {
    ABX_CUDA_TRY(tmp_t.alloc(n, s));
    d_tnodes = tmp_t.ptr;
  }
  Scratch<float4> tmp_sorted;
  if (!d_sorted)
  {
    ABX_CUDA_TRY(tmp_sorted.alloc((size_t)n * (kind == ABX_BOX ? 2 : 1), s));
    d_sorted = tmp_sorted.ptr;
  }
  Scratch<int64_t> off;
  ABX_CUDA_TRY(off.alloc(2, s));
  k_one_segment<<<1, 1, 0, s>>>(off.ptr, n);
  ABX_TRY(generate_hierarchy_segments(s, kind, d_g, n, off.ptr, 1, d_perm, d_codes, d_tnodes,
                                      d_sorted));
  if (d_leaves || d_internal)
    ABX_TRY(export_reference_layout(s, kind, d_tnodes, d_sorted, 0, n, d_leaves, d_internal));
  return ABX_SUCCESS;
}

abx_status export_reference_layout(cudaStream_t s, abx_geometry kind, const TNode *d_tnodes,
                                   const float4 *d_sorted, int64_t lo, int64_t n,
                                   LeafNode *d_leaves, InternalNode *d_internal)
{
  if (n <= 0)
    return ABX_SUCCESS;
  if (n > (int64_t)INT32_MAX / 2)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "export: too many values");
  DeviceState &ds = device_state();
  Scratch<LeafNode> tmp_leaves;
  Scratch<InternalNode> tmp_internal;
  if (!d_leaves)
  {
    ABX_CUDA_TRY(tmp_leaves.alloc(n, s));
    d_leaves = tmp_leaves.ptr;
  }
  if (!d_internal && n > 1)
  {
    ABX_CUDA_TRY(tmp_internal.alloc(n - 1, s));
    d_internal = tmp_internal.ptr;
  }
  const int nn = (int)n;
  Scratch<int> inv, parent, right;
  ABX_CUDA_TRY(inv.alloc(n, s));
  const unsigned b1 = (unsigned)((n + 255) / 256);
  if (kind == ABX_BOX)
    k_export_values<1><<<b1, 256, 0, s>>>(d_sorted, lo, nn, d_leaves, inv.ptr, ds.d_error);
  else
    k_export_values<0><<<b1, 256, 0, s>>>(d_sorted, lo, nn, d_leaves, inv.ptr, ds.d_error);
  ABX_CUDA_TRY(cudaGetLastError());
  if (n == 1)
    return ABX_SUCCESS;
  ABX_CUDA_TRY(parent.alloc(2 * n - 1, s));
  ABX_CUDA_TRY(right.alloc(n - 1, s));
  k_export_internal<<<(unsigned)((n - 1 + 255) / 256), 256, 0, s>>>(
      d_tnodes, lo, nn, inv.ptr, d_internal, parent.ptr, right.ptr, ds.d_error);
  k_export_ropes<<<(unsigned)((2 * n - 1 + 255) / 256), 256, 0, s>>>(
      nn, parent.ptr, right.ptr, d_leaves, d_internal, ds.d_error);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status forest_build(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t total,
                        const int64_t *d_off, int nseg, float *d_bounds, TNode *d_tnodes,
                        float4 *d_sorted)
{
  if (nseg < 1)
    return ABX_SUCCESS;
  {
    StageScope scope(s, "bounds", 1);
    if (kind == ABX_POINT)
      k_forest_bounds<0><<<nseg, 256, 0, s>>>(d_g, d_off, d_bounds);
    else
      k_forest_bounds<1><<<nseg, 256, 0, s>>>(d_g, d_off, d_bounds);
    ABX_CUDA_TRY(cudaGetLastError());
  }
  if (total < 1)
    return ABX_SUCCESS;
  Scratch<uint64_t> codes;
  Scratch<uint32_t> perm, perm2, keys, hist;
  ABX_CUDA_TRY(codes.alloc(total, s));
  ABX_CUDA_TRY(perm.alloc(total, s));
  ABX_CUDA_TRY(hist.alloc(8 * 256, s));
  ABX_CUDA_TRY(cudaMemsetAsync(hist.ptr, 0, 8 * 256 * sizeof(uint32_t), s));
  {
    StageScope scope(s, "morton64", 1);
    if (kind == ABX_POINT)
      k_forest_morton64<0><<<nseg, 256, 0, s>>>(d_g, d_off, d_bounds, codes.ptr, hist.ptr);
    else
      k_forest_morton64<1><<<nseg, 256, 0, s>>>(d_g, d_off, d_bounds, codes.ptr, hist.ptr);
    ABX_CUDA_TRY(cudaGetLastError());
  }
  // stable by code over all trees, then stable by tree: a stable sort of
  // every tree by its own codes
  ABX_TRY(radix_sort_u64(s, codes.ptr, perm.ptr, nullptr, total, 8, hist.ptr,
                         top_passes_from_hist(s, hist.ptr, total)));
  const uint32_t *final_perm = perm.ptr;
  int tree_bits = 0;
  while ((1ll << tree_bits) < nseg)
    ++tree_bits;
  if (tree_bits > 0)
  {
    ABX_CUDA_TRY(perm2.alloc(total, s));
    ABX_CUDA_TRY(keys.alloc(total, s));
    const unsigned blocks = (unsigned)((total + 255) / 256);
    k_tree_keys<<<blocks, 256, 0, s>>>(perm.ptr, d_off, nseg, total, keys.ptr);
    ABX_TRY(radix_sort_u32(s, keys.ptr, perm2.ptr, perm.ptr, total, (tree_bits + 7) / 8, nullptr));
    final_perm = perm2.ptr;
    if (kind == ABX_POINT)
      k_forest_codes<0><<<blocks, 256, 0, s>>>(d_g, final_perm, d_off, nseg, total, d_bounds,
                                               codes.ptr);
    else
      k_forest_codes<1><<<blocks, 256, 0, s>>>(d_g, final_perm, d_off, nseg, total, d_bounds,
                                               codes.ptr);
    ABX_CUDA_TRY(cudaGetLastError());
  }
  return generate_hierarchy_segments(s, kind, d_g, total, d_off, nseg, final_perm, codes.ptr,
                                     d_tnodes, d_sorted);
}

abx_status forest_query_order(cudaStream_t s, abx_geometry pred_kind, const float *d_preds,
                              int64_t nq, const int64_t *d_qoff, int nseg,
                              const float *d_bounds, uint32_t *d_perm)
{
  if (nq < 1)
    return ABX_SUCCESS;
  int tree_bits = 0;
  while ((1ll << tree_bits) < nseg)
    ++tree_bits;
  const unsigned blocks = (unsigned)((nq + 255) / 256);
#define ABX_QK(KIND, KEY)                                                                      \
  k_forest_query_keys<KIND, KEY><<<blocks, 256, 0, s>>>(d_preds, d_qoff, nseg, tree_bits, nq,   \
                                                       d_bounds, keys.ptr)
#define ABX_QKEYS(KEY)                                                                        \
  do                                                                                          \
  {                                                                                           \
    switch (pred_kind)                                                                        \
    {                                                                                         \
    case ABX_POINT: ABX_QK(0, KEY); break;                                                    \
    case ABX_BOX: ABX_QK(1, KEY); break;                                                      \
    case ABX_SPHERE: ABX_QK(2, KEY); break;                                                   \
    case ABX_RAY: ABX_QK(3, KEY); break;                                                      \
    case ABX_KDOP6: ABX_QK(4, KEY); break;                                                    \
    case ABX_KDOP14: ABX_QK(5, KEY); break;                                                   \
    case ABX_KDOP18: ABX_QK(6, KEY); break;                                                   \
    case ABX_KDOP26: ABX_QK(7, KEY); break;                                                   \
    default: return fail(ABX_ERROR_INVALID_ARGUMENT, "predicate kind");                       \
    }                                                                                         \
    ABX_CUDA_TRY(cudaGetLastError());                                                         \
  } while (0)
  if (tree_bits <= 16)
  {
    Scratch<uint32_t> keys;
    ABX_CUDA_TRY(keys.alloc(nq, s));
    ABX_QKEYS(uint32_t);
    // the order only schedules the queries: the top three digits (tree, then
    // the high Morton bits) suffice (4096 clouds, 5.85e7 box queries: order
    // 2.91 vs 3.84 ms for all four digits, traversal 9.91 vs 9.82 ms); 0 asks
    // for the full sort
    const int digits = tuning_value("FOREST_ORDER_DIGITS", 3);
    if (digits >= 1 && digits <= 3)
      return radix_order_top_u32(s, keys.ptr, d_perm, nq, 4, nullptr, digits);
    return radix_sort_u32(s, keys.ptr, d_perm, nullptr, nq, 4, nullptr, 0);
  }
  Scratch<uint64_t> keys;
  ABX_CUDA_TRY(keys.alloc(nq, s));
  ABX_QKEYS(uint64_t);
#undef ABX_QKEYS
#undef ABX_QK
  return radix_sort_u64(s, keys.ptr, d_perm, nullptr, nq, (32 + tree_bits + 7) / 8, nullptr);
}

} // namespace abx
