// abx_query.cu -- query traversal kernels over the 64-byte child-pair nodes
// and the Morton-ordered leaf buckets.
//
//   k_spatial   (abx_spatial.cuh) launched for sphere, box and ray
//               predicates; compaction, overflow lists and sampling of the
//               one-pass CRS.
//   k_nearest   nearest(Point, k) keeping the k best (distance, index) keys in
//               registers (k <= 32), closer child first, pruning by the k-th
//               distance (TreeTraversal<Nearest>, ArborX_TreeTraversal.hpp:
//               180-335, with the heap replaced by a sorted register list).
//   k_nearest_large  the same for k > 32 with a bounded max-heap kept in the
//               query's slice of the output arrays (misc/ArborX_Heap.hpp).
//
// Distances are compared squared: sqrt_rn is monotone, so a squared distance
// s passes "distance <= r" exactly when s <= sq_threshold(r), the largest
// float whose correctly rounded square root is <= r.  Square roots are taken
// only for candidates that can enter a result, which keeps every decision
// and every reported distance bit-identical to the sqrt-per-test formula.
#include <algorithm>
#include <cmath>

#include "abx_spatial.cuh"

namespace abx
{
namespace
{

// Compaction of per-query buffers into the CRS.  A warp owns 32 consecutive
// queries and copies their contiguous output range: each lane takes output
// positions with stride 32, finds its query by a binary search over the 33
// offsets held in the lanes' registers, and reads entry (position - offset)
// of that query's buffer.  Stores are coalesced for any row length.  An
// overflowed query keeps its first `buffer` results here; the fill pass
// rewrites all of them.
__global__ void k_compact(const int32_t *__restrict__ tmp, int64_t nq, int32_t buffer,
                          const int32_t *__restrict__ offsets, int32_t *__restrict__ out)
{
  const int64_t q0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5 << 5;
  const int lane = threadIdx.x & 31;
  if (q0 >= nq)
    return;
  const int m = (int)min((int64_t)32, nq - q0); // queries of this warp
  // lane l holds offsets[q0 + l] for l < m
  const int32_t my_off = lane < m ? offsets[q0 + lane] : INT32_MAX;
  const int32_t begin = __shfl_sync(0xffffffffu, my_off, 0);
  const int32_t end = offsets[q0 + m];
  for (int32_t base = begin; base < end; base += 32) // warp-uniform trips
  {
    const int32_t j = base + lane;
    // the largest r < m with offsets[q0 + r] <= j
    int lo = 0, hi = m - 1;
#pragma unroll
    for (int step = 0; step < 5; ++step)
    {
      const int mid = (lo + hi + 1) >> 1;
      const int32_t om = __shfl_sync(0xffffffffu, my_off, mid);
      if (lo < hi)
      {
        if (om <= j)
          lo = mid;
        else
          hi = mid - 1;
      }
    }
    const int32_t e = j - __shfl_sync(0xffffffffu, my_off, lo);
    if (j < end && e < buffer)
      out[j] = tmp[(q0 + lo) * (int64_t)buffer + e];
  }
}

// Queries whose result count exceeds the buffer: flag[q] = 1.
__global__ void k_overflow_flags(const int32_t *__restrict__ offsets, int64_t nq, int32_t buffer,
                                 int32_t *__restrict__ flags)
{
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq)
    flags[q] = offsets[q + 1] - offsets[q] > buffer;
}

// list[pos[q]] = q for every flagged query (pos: exclusive scan of flags).
__global__ void k_overflow_list(const int32_t *__restrict__ flags, const int32_t *__restrict__ pos,
                                int64_t nq, uint32_t *__restrict__ list)
{
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq && flags[q])
    list[pos[q]] = (uint32_t)q;
}

// Strided sample of the queries (in traversal order): sample[t] = query of
// position t * stride.
__global__ void k_sample_queries(const uint32_t *__restrict__ perm, int64_t stride, int64_t m,
                                 uint32_t *__restrict__ sample)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m)
    sample[t] = perm ? perm[t * stride] : (uint32_t)(t * stride);
}

// Sum of counts[sample[t]] into *total (zeroed).
__global__ void k_sample_sum(const int32_t *__restrict__ counts, const uint32_t *__restrict__ sample,
                             int64_t m, unsigned long long *__restrict__ total)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v = t < m ? (unsigned long long)counts[sample[t]] : 0ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v)
    atomicAdd(total, v);
}

// ---------------------------------------------------------------------------
// Nearest
// ---------------------------------------------------------------------------

// A k-nearest candidate as one 64-bit key: the distance's bit pattern (a
// non-negative float, so unsigned order = numeric order) above the value + 1.
// Unsigned key order is exactly the (distance, index) order; 0 sorts before
// every candidate and ~0 after every candidate.
constexpr uint64_t kKeyEmpty = ~0ull;

__device__ __forceinline__ uint64_t knn_key(float d, int value)
{
  return ((uint64_t)__float_as_uint(d) << 32) | (uint32_t)(value + 1);
}
__device__ __forceinline__ float key_dist(uint64_t k) { return __uint_as_float((uint32_t)(k >> 32)); }
__device__ __forceinline__ int key_value(uint64_t k) { return (int)(uint32_t)k - 1; }

// Insert c into the ascending list (precondition: c < key[K-1]).
template <int K>
__device__ __forceinline__ void list_insert(uint64_t (&key)[K], uint64_t c)
{
  bool lt[K];
#pragma unroll
  for (int j = 0; j < K; ++j)
    lt[j] = c < key[j];
#pragma unroll
  for (int j = K - 1; j >= 1; --j)
    key[j] = lt[j - 1] ? key[j - 1] : (lt[j] ? c : key[j]);
  key[0] = lt[0] ? c : key[0];
}

struct KnnTask
{
  int64_t q;
  int k;
  int kk;
  int64_t base;
};

__device__ __forceinline__ KnnTask knn_task(int64_t t, int64_t n, ForestView const &f,
                                            QueryTree &tree, int64_t nq,
                                            const uint32_t *__restrict__ perm,
                                            const int32_t *__restrict__ kq, int32_t k_all,
                                            const int32_t *__restrict__ offsets,
                                            int32_t *__restrict__ offsets_out)
{
  KnnTask task;
  task.q = perm ? (int64_t)__ldg(perm + t) : t;
  tree = query_tree(task.q, n, f);
  n = tree.size;
  const int k = kq ? __ldg(kq + task.q) : k_all;
  task.k = k < 0 ? 0 : k;
  task.kk = (int)((int64_t)task.k < n ? (int64_t)task.k : n);
  task.base = offsets ? (int64_t)__ldg(offsets + task.q) : task.q * (int64_t)task.kk;
  if (offsets_out)
  {
    offsets_out[task.q] = (int32_t)task.base;
    if (task.q == nq - 1)
      offsets_out[nq] = (int32_t)(task.base + task.kk);
  }
  return task;
}

// One query per thread.  The list keeps K slots; the first K - k hold the
// key 0 (never displaced), so the k-th best is always slot K - 1.  thr is
// sq_bound of the k-th best distance (+inf until the list is full): a node
// or leaf whose squared distance s satisfies s <= thr may hold a better
// candidate (and every one that can passes).  Buckets are scanned as soon as their box passes; of two
// passing internal children the closer is visited first and the other waits
// on the stack with its squared distance.
// Up to 16 keys the register list fits in 64 registers per thread, which
// lets 8 CTAs share an SM (2-3% faster at 1e7 points than 7); the 32-key
// list needs more.
template <int K, int KIND, bool SCAN>
__global__ void __launch_bounds__(kQueryThreads, K <= 16 ? 8 : 1)
    k_nearest(const TNode *__restrict__ nodes, const float4 *__restrict__ sorted, int64_t n,
              ForestView f, const float *__restrict__ queries, int64_t nq,
              const uint32_t *__restrict__ perm,
              const int32_t *__restrict__ kq, int32_t k_all, const int32_t *__restrict__ offsets,
              int32_t *__restrict__ offsets_out, int32_t *__restrict__ out_idx,
              float *__restrict__ out_dist, int bucket, unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  QueryTree tree;
  const KnnTask task = knn_task(t, n, f, tree, nq, perm, kq, k_all, offsets, offsets_out);
  if (task.kk == 0)
    return;
  uint64_t key[K];
  const int first = K - task.k;
#pragma unroll
  for (int j = 0; j < K; ++j)
    key[j] = j < first ? 0ull : kKeyEmpty;
  float thr = INFINITY;
  const float qx = __ldg(queries + 3 * task.q), qy = __ldg(queries + 3 * task.q + 1),
              qz = __ldg(queries + 3 * task.q + 2);

  auto offer = [&](float s, int v) {
    const uint64_t c = knn_key(__fsqrt_rn(s), v);
    if (c < key[K - 1])
    {
      list_insert<K>(key, c);
      if (key[K - 1] != kKeyEmpty)
        thr = sq_bound(key_dist(key[K - 1]));
    }
  };
  // s_box: squared distance to the bucket's box (for a single leaf, its
  // own squared distance)
  // a child whose box passed (squared distance s_box); returns true when it
  // is an internal node to descend into
  auto visit = [&](int ref, int cf, float s_box) -> bool {
    int start = 0, cnt = 0;
    const ChildKind kind = child_kind<SCAN>(ref, cf, bucket, start, cnt);
    if (kind == kLeaf)
      offer(s_box, bucket_start(ref));
    else if (SCAN && kind == kScan)
    {
      for (int j = 0; j < cnt; ++j)
      {
        Box3 b;
        int v;
        SortedLeaf<KIND>::load(sorted, start + j, b, v);
        const float s = leaf_dist2<KIND>(qx, qy, qz, b);
        if (s <= thr)
          offer(s, v);
      }
    }
    return kind == kDescend;
  };

  int sref[kStackDepth];
  float sdist[kStackDepth];
  int sp = 0;
  int node = tree.root;
  const int64_t num_nodes = tree.size > 1 ? tree.size - 1 : 1;
  int64_t budget = num_nodes;
  while (true)
  {
    if (--budget < 0 || (uint64_t)(node - tree.root) >= (uint64_t)num_nodes)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      break;
    }
    const TNode tn = load_tnode(nodes, node);
    Box3 l, r;
    tnode_children(tn, l, r);
    const int lref = tn.d.x, rref = tn.d.y;
    const bool rnone = is_bucket_ref(rref) && tn.d.w == 0; // one-leaf tree: no right child
    const float sl = dist2_pb(qx, qy, qz, l);
    const float sr = rnone ? INFINITY : dist2_pb(qx, qy, qz, r);
    // leaves and scanned subtrees first (they may tighten thr), then the
    // internal children that still pass
    bool dl = sl <= thr && visit(lref, tn.d.z, sl);
    bool dr = sr <= thr && visit(rref, tn.d.w, sr);
    const bool gl = dl && sl <= thr;
    const bool gr = dr && sr <= thr;
    if (gl && gr)
    {
      const bool left_first = sl <= sr;
      node = left_first ? lref : rref;
      if (sp < kStackDepth)
      {
        sref[sp] = left_first ? rref : lref;
        sdist[sp] = left_first ? sr : sl;
        ++sp;
      }
      else
        raise_error(err, ABX_DEVERR_STACK_OVERFLOW);
      continue;
    }
    if (gl || gr)
    {
      node = gl ? lref : rref;
      continue;
    }
    bool found = false;
    while (sp > 0)
    {
      --sp;
      if (sdist[sp] <= thr)
      {
        node = sref[sp];
        found = true;
        break;
      }
    }
    if (!found)
      break;
  }
  if (K % 4 == 0 && first == 0 && task.kk == K && (task.base & 3) == 0)
  {
    // a full list at a 16-byte aligned offset: vector stores, so each
    // query's results leave as whole sectors
    int4 *oi = reinterpret_cast<int4 *>(out_idx + task.base);
#pragma unroll
    for (int j = 0; j < K; j += 4)
      oi[j / 4] = make_int4(key_value(key[j]), key_value(key[j + 1]), key_value(key[j + 2]),
                            key_value(key[j + 3]));
    if (out_dist)
    {
      float4 *od = reinterpret_cast<float4 *>(out_dist + task.base);
#pragma unroll
      for (int j = 0; j < K; j += 4)
        od[j / 4] = make_float4(key_dist(key[j]), key_dist(key[j + 1]), key_dist(key[j + 2]),
                                key_dist(key[j + 3]));
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    if (j >= first && j < first + task.kk)
    {
      out_idx[task.base + (j - first)] = key_value(key[j]);
      if (out_dist)
        out_dist[task.base + (j - first)] = key_dist(key[j]);
    }
  }
}

// (distance, index) order of the k-nearest result.
__device__ __forceinline__ bool pair_lt(float da, int ia, float db, int ib)
{
  return da < db || (da == db && ia < ib);
}

// Bounded max-heap on (distance, index) in global memory: the farthest of
// the current best is at the top (PriorityQueue / bubbleUp / bubbleDown of
// misc/ArborX_PriorityQueue.hpp:63-93 and misc/ArborX_Heap.hpp:40-92, with
// the (distance, index) order).
__device__ void heap_sift_down(float *hd, int *hi, int pos, int len, float d, int v)
{
  int child = 2 * pos + 1;
  while (child < len)
  {
    if (child + 1 < len && pair_lt(hd[child], hi[child], hd[child + 1], hi[child + 1]))
      ++child;
    if (!pair_lt(d, v, hd[child], hi[child]))
      break;
    hd[pos] = hd[child];
    hi[pos] = hi[child];
    pos = child;
    child = 2 * pos + 1;
  }
  hd[pos] = d;
  hi[pos] = v;
}

__device__ void heap_push(float *hd, int *hi, int &size, float d, int v)
{
  int pos = size++;
  while (pos > 0)
  {
    const int parent = (pos - 1) / 2;
    if (!pair_lt(hd[parent], hi[parent], d, v))
      break;
    hd[pos] = hd[parent];
    hi[pos] = hi[parent];
    pos = parent;
  }
  hd[pos] = d;
  hi[pos] = v;
}

template <int KIND>
__global__ void __launch_bounds__(kQueryThreads)
    k_nearest_large(const TNode *__restrict__ nodes, const float4 *__restrict__ sorted,
                    int64_t n, ForestView f, const float *__restrict__ queries, int64_t nq,
                    const uint32_t *__restrict__ perm, const int32_t *__restrict__ kq,
                    int32_t k_all, const int32_t *__restrict__ offsets,
                    int32_t *__restrict__ offsets_out, int32_t *__restrict__ out_idx,
                    float *__restrict__ out_dist, int bucket, unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  QueryTree tree;
  const KnnTask task = knn_task(t, n, f, tree, nq, perm, kq, k_all, offsets, offsets_out);
  const int kk = task.kk;
  if (kk == 0)
    return;
  float *hd = out_dist + task.base;
  int *hi = out_idx + task.base;
  int size = 0;
  float thr = INFINITY;
  const float qx = queries[3 * task.q], qy = queries[3 * task.q + 1], qz = queries[3 * task.q + 2];
  auto offer = [&](float s, int v) {
    const float d = __fsqrt_rn(s);
    if (size < kk)
      heap_push(hd, hi, size, d, v);
    else if (pair_lt(d, v, hd[0], hi[0]))
      heap_sift_down(hd, hi, 0, size, d, v);
    else
      return;
    if (size == kk)
      thr = sq_threshold(hd[0]);
  };
  // a child whose box passed (squared distance s_box); returns true when it
  // is an internal node to descend into
  auto visit = [&](int ref, int cf, float s_box) -> bool {
    int start = 0, cnt = 0;
    const ChildKind kind = child_kind<true>(ref, cf, bucket, start, cnt);
    if (kind == kLeaf)
      offer(s_box, bucket_start(ref));
    else if (kind == kScan)
    {
      for (int j = 0; j < cnt; ++j)
      {
        Box3 b;
        int v;
        SortedLeaf<KIND>::load(sorted, start + j, b, v);
        const float s = leaf_dist2<KIND>(qx, qy, qz, b);
        if (s <= thr)
          offer(s, v);
      }
    }
    return kind == kDescend;
  };
  int sref[kStackDepth];
  float sdist[kStackDepth];
  int sp = 0;
  int node = tree.root;
  const int64_t num_nodes = tree.size > 1 ? tree.size - 1 : 1;
  int64_t budget = num_nodes;
  while (true)
  {
    if (--budget < 0 || (uint64_t)(node - tree.root) >= (uint64_t)num_nodes)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      break;
    }
    const TNode tn = load_tnode(nodes, node);
    Box3 l, r;
    tnode_children(tn, l, r);
    const int lref = tn.d.x, rref = tn.d.y;
    const bool rnone = is_bucket_ref(rref) && tn.d.w == 0; // one-leaf tree: no right child
    const float sl = dist2_pb(qx, qy, qz, l);
    const float sr = rnone ? INFINITY : dist2_pb(qx, qy, qz, r);
    // leaves and scanned subtrees first (they may tighten thr), then the
    // internal children that still pass
    bool dl = sl <= thr && visit(lref, tn.d.z, sl);
    bool dr = sr <= thr && visit(rref, tn.d.w, sr);
    const bool gl = dl && sl <= thr;
    const bool gr = dr && sr <= thr;
    if (gl && gr)
    {
      const bool left_first = sl <= sr;
      node = left_first ? lref : rref;
      if (sp < kStackDepth)
      {
        sref[sp] = left_first ? rref : lref;
        sdist[sp] = left_first ? sr : sl;
        ++sp;
      }
      else
        raise_error(err, ABX_DEVERR_STACK_OVERFLOW);
      continue;
    }
    if (gl || gr)
    {
      node = gl ? lref : rref;
      continue;
    }
    bool found = false;
    while (sp > 0)
    {
      --sp;
      if (sdist[sp] <= thr)
      {
        node = sref[sp];
        found = true;
        break;
      }
    }
    if (!found)
      break;
  }
  // heap sort into ascending (distance, index) order
  for (int len = size; len > 1; --len)
  {
    const float d0 = hd[0];
    const int i0 = hi[0];
    heap_sift_down(hd, hi, 0, len - 1, hd[len - 1], hi[len - 1]);
    hd[len - 1] = d0;
    hi[len - 1] = i0;
  }
}

__global__ void k_knn_counts(int64_t n, ForestView f, const int32_t *__restrict__ kq, int32_t k_all,
                             int64_t nq, int32_t *__restrict__ counts, int32_t *__restrict__ kmax)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int32_t m = 0;
  if (i < nq)
  {
    int32_t k = kq ? kq[i] : k_all;
    k = k < 0 ? 0 : k;
    const int64_t size = query_tree(i, n, f).size;
    counts[i] = (int32_t)((int64_t)k < size ? (int64_t)k : size);
    m = k;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0)
    atomicMax(kmax, m);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

// Brute force: tiles and k_brute_spatial in abx_spatial.cuh.

// Nearest: the same sorted key list and (distance, index) rule as k_nearest,
// so the results equal the tree's.
template <int K, int KIND>
__global__ void __launch_bounds__(kQueryThreads)
    k_brute_nearest(const float4 *__restrict__ values, int64_t n, const float *__restrict__ queries,
                    int64_t nq, const int32_t *__restrict__ kq, int32_t k_all,
                    const int32_t *__restrict__ offsets, int32_t *__restrict__ offsets_out,
                    int32_t *__restrict__ out_idx, float *__restrict__ out_dist)
{
  __shared__ float4 tile[kBruteTile * (KIND == 1 ? 2 : 1)];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < nq;
  KnnTask task{};
  if (active)
  {
    QueryTree tree;
    task = knn_task(t, n, ForestView{nullptr, nullptr, 1}, tree, nq, nullptr, kq, k_all,
                    offsets, offsets_out);
  }
  const bool work = active && task.kk > 0;
  uint64_t key[K];
  const int first = K - (work ? task.k : 0);
#pragma unroll
  for (int j = 0; j < K; ++j)
    key[j] = j < first ? 0ull : kKeyEmpty;
  float thr = INFINITY;
  float qx = 0, qy = 0, qz = 0;
  if (work)
  {
    qx = __ldg(queries + 3 * task.q);
    qy = __ldg(queries + 3 * task.q + 1);
    qz = __ldg(queries + 3 * task.q + 2);
  }
  for (int64_t t0 = 0; t0 < n; t0 += kBruteTile)
  {
    const int m = load_tile<KIND>(tile, values, n, t0);
    if (!work)
      continue;
    for (int j = 0; j < m; ++j)
    {
      Box3 b;
      int v;
      tile_leaf<KIND>(tile, j, b, v);
      const float s = leaf_dist2<KIND>(qx, qy, qz, b);
      if (s <= thr)
      {
        const uint64_t c = knn_key(__fsqrt_rn(s), v);
        if (c < key[K - 1])
        {
          list_insert<K>(key, c);
          if (key[K - 1] != kKeyEmpty)
            thr = sq_bound(key_dist(key[K - 1]));
        }
      }
    }
  }
  if (!work)
    return;
  const int kk = task.kk;
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    const int r = j - first;
    if (r >= 0 && r < kk)
    {
      out_idx[task.base + r] = key_value(key[j]);
      if (out_dist)
        out_dist[task.base + r] = key_dist(key[j]);
    }
  }
}

// Nearest over point values with the all-pairs product on tensor cores as a
// candidate filter (mma.sync m16n8k8 tf32).  The points are scanned in
// Morton order, each CTA starting at the tile where the Morton64 code of its
// first query falls and wrapping around: with the queries in Morton order too,
// a query's list reaches its final neighbours within the first tiles, so
// later tiles rarely produce candidates.  A warp owns 32 queries; per
// group of 8 points it forms, for its two 16-query row blocks,
//   C'(q, p) = |p|^2 (1 - e) - 2 q.p,   e = 2^-16,
// from A rows (qx, qy, qz, 1) and B columns (-2px, -2py, -2pz, |p|^2 (1 - e))
// split into tf32 high and low parts: one product with K = 8 takes
// [A_hi | A_lo] x [B_hi ; B_hi], a second A_hi x B_lo (the low x low term is
// dropped).  The product and accumulation errors stay below 2^-18 (|q|^2 +
// 2 |p|^2), so V = |q|^2 (1 - e) + C' lies below the real squared distance
// by more than the float formula's own error: V <= the exact squared
// distance of the tree's formula.  A pair whose V exceeds the query's
// pruning bound thr cannot enter its list; every other pair is a candidate,
// queued per query in shared memory and rescored by the owner lane with the
// exact formula and key rule of k_brute_nearest.  Results are identical to
// that kernel's.  Points or queries with non-finite coordinates or squared
// norms above 1e30 are always candidates (exact path).
constexpr int kTcTile = 512; // points per shared-memory stage
constexpr float kTcSlack = 1.52587890625e-05f; // e = 2^-16
constexpr float kTcBig = 1e30f;

__device__ __forceinline__ uint32_t tf32_rna(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// D = A B + C for one m16n8k8 tile: lane (g, t) gives A[g][t], A[g + 8][t],
// A[g][t + 4], A[g + 8][t + 4] and B[t][g], B[t + 4][g].
__device__ __forceinline__ void mma_k8(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                       uint32_t a3, uint32_t b0, uint32_t b1)
{
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
               "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int K>
__global__ void __launch_bounds__(kQueryThreads)
    k_brute_nearest_tc(const float4 *__restrict__ values, int64_t n,
                       const uint64_t *__restrict__ codes, const float *__restrict__ scene,
                       const float *__restrict__ queries, int64_t nq,
                       const uint32_t *__restrict__ perm,
                       const int32_t *__restrict__ kq, int32_t k_all,
                       const int32_t *__restrict__ offsets, int32_t *__restrict__ offsets_out,
                       int32_t *__restrict__ out_idx, float *__restrict__ out_dist,
                       uint64_t *__restrict__ partial)
{
  constexpr unsigned kAll = 0xffffffffu;
  constexpr int kWarps = kQueryThreads / 32;
  __shared__ float4 s_pt[kTcTile];
  __shared__ float4 s_hi[kTcTile];
  __shared__ float4 s_lo[kTcTile];
  __shared__ int s_cand[kWarps][32][8];
  __shared__ int s_cnt[kWarps][32];
  __shared__ int64_t s_start;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < nq;
  KnnTask task{};
  if (active)
  {
    QueryTree tree;
    task = knn_task(t, n, ForestView{nullptr, nullptr, 1}, tree, nq, perm, kq, k_all, offsets,
                    blockIdx.y == 0 ? offsets_out : nullptr);
  }
  const bool work = active && task.kk > 0;
  uint64_t key[K];
  const int first = K - (work ? task.k : 0);
#pragma unroll
  for (int j = 0; j < K; ++j)
    key[j] = j < first ? 0ull : kKeyEmpty;
  float thr = INFINITY;
  float qx = 0, qy = 0, qz = 0;
  if (work)
  {
    qx = __ldg(queries + 3 * task.q);
    qy = __ldg(queries + 3 * task.q + 1);
    qz = __ldg(queries + 3 * task.q + 2);
  }
  // the tile of the first query's Morton code: the CTA's scan starts there
  if (threadIdx.x == 0)
  {
    int64_t pos = 0;
    if (active)
    {
      const uint64_t c = morton64_unit(translate_scale(qx, __ldg(scene), __ldg(scene + 3)),
                                       translate_scale(qy, __ldg(scene + 1), __ldg(scene + 4)),
                                       translate_scale(qz, __ldg(scene + 2), __ldg(scene + 5)));
      int64_t a = 0, b = n; // first position with code >= c
      while (a < b)
      {
        const int64_t mid = (a + b) >> 1;
        if (__ldg(codes + mid) < c)
          a = mid + 1;
        else
          b = mid;
      }
      pos = a;
    }
    s_start = pos;
  }
  __syncthreads();
  // this CTA's share of the tiles (gridDim.y chunks when few queries would
  // leave SMs idle; the partial lists are merged afterwards)
  const int64_t all_tiles = (n + kTcTile - 1) / kTcTile;
  const int64_t per_chunk = (all_tiles + gridDim.y - 1) / gridDim.y;
  const int64_t tile_lo = (int64_t)blockIdx.y * per_chunk;
  const int64_t num_tiles = max((int64_t)0, min(per_chunk, all_tiles - tile_lo));
  int64_t start_tile = s_start / kTcTile - tile_lo;
  start_tile = start_tile < 0 || start_tile >= num_tiles ? 0 : start_tile;
  const float qn = __fadd_rn(__fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy)), __fmul_rn(qz, qz));
  // a query outside the filter's range takes every pair (T = +inf, NaN pairs
  // count as candidates through !(c > T))
  const bool q_exact = !(qn <= kTcBig);
  const float qn_lo = __fmul_rd(qn, 1.f - kTcSlack);
  // the per-row bound the filter compares C' with
  auto row_bound = [&]() -> float {
    if (!work)
      return -INFINITY;
    if (q_exact || thr == INFINITY)
      return INFINITY;
    return __fsub_ru(thr, qn_lo);
  };
  float T = row_bound();
  // A fragments of the rows g, g + 8, 16 + g, 24 + g: component tq of
  // (qx, qy, qz, 1), high and low tf32 parts
  uint32_t ahi[4], alo[4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
  {
    const int row = (r >> 1) * 16 + (r & 1) * 8 + g;
    const float x = __shfl_sync(kAll, qx, row), y = __shfl_sync(kAll, qy, row),
                z = __shfl_sync(kAll, qz, row);
    const float a = tq == 0 ? x : tq == 1 ? y : tq == 2 ? z : 1.f;
    ahi[r] = tf32_rna(a);
    alo[r] = tf32_rna(__fsub_rn(a, __uint_as_float(ahi[r])));
  }
  float Trow[4];
  auto load_bounds = [&]() {
#pragma unroll
    for (int r = 0; r < 4; ++r)
      Trow[r] = __shfl_sync(kAll, T, (r >> 1) * 16 + (r & 1) * 8 + g);
  };
  load_bounds();
  s_cnt[warp][lane] = 0;
  auto offer = [&](float s, int v) {
    if (s <= thr)
    {
      const uint64_t c = knn_key(__fsqrt_rn(s), v);
      if (c < key[K - 1])
      {
        list_insert<K>(key, c);
        if (key[K - 1] != kKeyEmpty)
          thr = sq_bound(key_dist(key[K - 1]));
      }
    }
  };
  for (int64_t it = 0; it < num_tiles; ++it)
  {
    int64_t tile = start_tile + it;
    if (tile >= num_tiles)
      tile -= num_tiles;
    const int64_t t0 = (tile_lo + tile) * kTcTile;
    const int m = (int)min((int64_t)kTcTile, n - t0);
    __syncthreads();
    for (int j = threadIdx.x; j < kTcTile; j += blockDim.x)
    {
      float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
      if (j < m)
      {
        p = __ldg(values + t0 + j);
        const float pn =
            __fadd_rn(__fadd_rn(__fmul_rn(p.x, p.x), __fmul_rn(p.y, p.y)), __fmul_rn(p.z, p.z));
        if (pn <= kTcBig)
        {
          const float b[4] = {__fmul_rn(-2.f, p.x), __fmul_rn(-2.f, p.y), __fmul_rn(-2.f, p.z),
                              __fmul_rn(pn, 1.f - kTcSlack)};
          float h[4], l[4];
#pragma unroll
          for (int c = 0; c < 4; ++c)
          {
            h[c] = __uint_as_float(tf32_rna(b[c]));
            l[c] = __uint_as_float(tf32_rna(__fsub_rn(b[c], h[c])));
          }
          hi = make_float4(h[0], h[1], h[2], h[3]);
          lo = make_float4(l[0], l[1], l[2], l[3]);
        }
        else // outside the filter's range: C' = -FLT_MAX, always a candidate
          hi.w = -FLT_MAX;
      }
      else
        p.w = __int_as_float(-1); // padding: never offered
      s_pt[j] = p;
      s_hi[j] = hi;
      s_lo[j] = lo;
    }
    __syncthreads();
    for (int p0 = 0; p0 < m; p0 += 8)
    {
      const float *bh = reinterpret_cast<const float *>(s_hi + p0 + g);
      const float *bl = reinterpret_cast<const float *>(s_lo + p0 + g);
      const uint32_t bhi = __float_as_uint(bh[tq]), blo = __float_as_uint(bl[tq]);
      float c[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
      for (int blk = 0; blk < 2; ++blk)
      {
        mma_k8(c[blk], ahi[2 * blk], ahi[2 * blk + 1], 0u, 0u, blo, 0u);
        mma_k8(c[blk], ahi[2 * blk], ahi[2 * blk + 1], alo[2 * blk], alo[2 * blk + 1], bhi, bhi);
      }
      // c[blk][e]: row blk * 16 + (e >> 1) * 8 + g, point p0 + 2 tq + (e & 1)
      unsigned mask = 0;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        mask |= (unsigned)!(c[e >> 2][e & 3] > Trow[2 * (e >> 2) + ((e & 3) >> 1)]) << e;
      if (__any_sync(kAll, mask != 0))
      {
#pragma unroll
        for (int e = 0; e < 8; ++e)
        {
          const int row = (e >> 2) * 16 + ((e & 3) >> 1) * 8 + g;
          const int pj = p0 + 2 * tq + (e & 1);
          if (((mask >> e) & 1) && pj < m)
          {
            const int slot = atomicAdd(&s_cnt[warp][row], 1);
            s_cand[warp][row][slot] = pj;
          }
        }
        __syncwarp();
        const int cnt = s_cnt[warp][lane];
        for (int i = 0; i < cnt; ++i)
        {
          const float4 p = s_pt[s_cand[warp][lane][i]];
          if (__float_as_int(p.w) >= 0)
            offer(dist2_pp(qx, qy, qz, p.x, p.y, p.z), __float_as_int(p.w));
        }
        s_cnt[warp][lane] = 0;
        T = row_bound();
        __syncwarp();
        load_bounds();
      }
    }
  }
  if (partial)
  {
    if (active)
    {
#pragma unroll
      for (int m = 0; m < K; ++m)
        partial[((int64_t)blockIdx.y * nq + t) * K + m] = work ? key[m] : kKeyEmpty;
    }
    return;
  }
  if (!work)
    return;
  const int kk = task.kk;
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    const int r = j - first;
    if (r >= 0 && r < kk)
    {
      out_idx[task.base + r] = key_value(key[j]);
      if (out_dist)
        out_dist[task.base + r] = key_dist(key[j]);
    }
  }
}

// The k best of a query over the point chunks of a split k_brute_nearest_tc
// launch: the chunks' sorted key lists merged by the same key rule.
template <int K>
__global__ void __launch_bounds__(kQueryThreads)
    k_brute_merge(const uint64_t *__restrict__ partial, int chunks, int64_t n,
                  int64_t nq, const uint32_t *__restrict__ perm, const int32_t *__restrict__ kq,
                  int32_t k_all, const int32_t *__restrict__ offsets,
                  int32_t *__restrict__ out_idx, float *__restrict__ out_dist)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  QueryTree tree;
  const KnnTask task = knn_task(t, n, ForestView{nullptr, nullptr, 1}, tree, nq, perm, kq, k_all,
                                offsets, nullptr);
  if (task.kk == 0)
    return;
  uint64_t key[K];
  const int first = K - task.k;
#pragma unroll
  for (int j = 0; j < K; ++j)
    key[j] = j < first ? 0ull : kKeyEmpty;
  for (int c = 0; c < chunks; ++c)
  {
    const uint64_t *row = partial + ((int64_t)c * nq + t) * K;
    for (int m = 0; m < K; ++m)
    {
      const uint64_t v = __ldg(row + m);
      if (v == 0ull || v == kKeyEmpty) // placeholders of k < K, unfilled slots
        continue;
      if (!(v < key[K - 1]))
        break; // the chunk's list is ascending
      list_insert<K>(key, v);
    }
  }
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    const int r = j - first;
    if (r >= 0 && r < task.kk)
    {
      out_idx[task.base + r] = key_value(key[j]);
      if (out_dist)
        out_dist[task.base + r] = key_dist(key[j]);
    }
  }
}

// intersects(Sphere) over point values with the same tensor-core filter:
// the pair (q, p) can match only if |q|^2 (1 - e) + C'(q, p) <= r2, r2 the
// query's exact squared-radius threshold; passing pairs are marked per query
// in a shared-memory bit mask (one bit per point of the 8-point group) and
// the owner lane tests them exactly in ascending point order, so the matches
// come out in ascending value order like k_brute_spatial's (the points are
// scanned in input order).
template <int MODE>
__global__ void __launch_bounds__(kQueryThreads)
    k_brute_spatial_tc(const float4 *__restrict__ values, int64_t n,
                       const float *__restrict__ preds, int64_t nq,
                       const uint32_t *__restrict__ list, int32_t *__restrict__ counts,
                       const int32_t *__restrict__ offsets, int32_t *__restrict__ out,
                       int32_t buffer, unsigned *__restrict__ overflow)
{
  constexpr unsigned kAll = 0xffffffffu;
  constexpr int kWarps = kQueryThreads / 32;
  __shared__ float4 s_pt[kTcTile];
  __shared__ float4 s_hi[kTcTile];
  __shared__ float4 s_lo[kTcTile];
  __shared__ unsigned s_mask[kWarps][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < nq;
  const int64_t q = active && list ? (int64_t)__ldg(list + t) : t;
  float qx = 0.f, qy = 0.f, qz = 0.f, r2 = -1.f;
  if (active)
  {
    const SpherePred sp = PredOf<ABX_SPHERE>::load(preds, q);
    qx = sp.cx;
    qy = sp.cy;
    qz = sp.cz;
    r2 = sp.r2;
  }
  int32_t *dst = nullptr;
  if (MODE == kFill && active)
    dst = out + __ldg(offsets + q);
  if (MODE == kBuffered && active)
    dst = out + q * (int64_t)buffer;
  int32_t count = 0;
  const float qn = __fadd_rn(__fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy)), __fmul_rn(qz, qz));
  // r2 < 0 (negative radius) matches nothing; a query outside the filter's
  // range takes every pair (NaN pairs count through !(c > T))
  float T = -INFINITY;
  if (active && r2 >= 0.f)
    T = qn <= kTcBig ? __fsub_ru(r2, __fmul_rd(qn, 1.f - kTcSlack)) : INFINITY;
  uint32_t ahi[4], alo[4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
  {
    const int row = (r >> 1) * 16 + (r & 1) * 8 + g;
    const float x = __shfl_sync(kAll, qx, row), y = __shfl_sync(kAll, qy, row),
                z = __shfl_sync(kAll, qz, row);
    const float a = tq == 0 ? x : tq == 1 ? y : tq == 2 ? z : 1.f;
    ahi[r] = tf32_rna(a);
    alo[r] = tf32_rna(__fsub_rn(a, __uint_as_float(ahi[r])));
  }
  float Trow[4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
    Trow[r] = __shfl_sync(kAll, T, (r >> 1) * 16 + (r & 1) * 8 + g);
  s_mask[warp][lane] = 0;
  for (int64_t t0 = 0; t0 < n; t0 += kTcTile)
  {
    const int m = (int)min((int64_t)kTcTile, n - t0);
    __syncthreads();
    for (int j = threadIdx.x; j < kTcTile; j += blockDim.x)
    {
      float4 p = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
      float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
      if (j < m)
      {
        p = __ldg(values + t0 + j);
        const float pn =
            __fadd_rn(__fadd_rn(__fmul_rn(p.x, p.x), __fmul_rn(p.y, p.y)), __fmul_rn(p.z, p.z));
        if (pn <= kTcBig)
        {
          const float b[4] = {__fmul_rn(-2.f, p.x), __fmul_rn(-2.f, p.y), __fmul_rn(-2.f, p.z),
                              __fmul_rn(pn, 1.f - kTcSlack)};
          float h[4], l[4];
#pragma unroll
          for (int c = 0; c < 4; ++c)
          {
            h[c] = __uint_as_float(tf32_rna(b[c]));
            l[c] = __uint_as_float(tf32_rna(__fsub_rn(b[c], h[c])));
          }
          hi = make_float4(h[0], h[1], h[2], h[3]);
          lo = make_float4(l[0], l[1], l[2], l[3]);
        }
        else
          hi.w = -FLT_MAX;
      }
      s_pt[j] = p;
      s_hi[j] = hi;
      s_lo[j] = lo;
    }
    __syncthreads();
    for (int p0 = 0; p0 < m; p0 += 8)
    {
      const float *bh = reinterpret_cast<const float *>(s_hi + p0 + g);
      const float *bl = reinterpret_cast<const float *>(s_lo + p0 + g);
      const uint32_t bhi = __float_as_uint(bh[tq]), blo = __float_as_uint(bl[tq]);
      float c[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
      for (int blk = 0; blk < 2; ++blk)
      {
        mma_k8(c[blk], ahi[2 * blk], ahi[2 * blk + 1], 0u, 0u, blo, 0u);
        mma_k8(c[blk], ahi[2 * blk], ahi[2 * blk + 1], alo[2 * blk], alo[2 * blk + 1], bhi, bhi);
      }
      unsigned mask = 0;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        mask |= (unsigned)!(c[e >> 2][e & 3] > Trow[2 * (e >> 2) + ((e & 3) >> 1)]) << e;
      if (__any_sync(kAll, mask != 0))
      {
#pragma unroll
        for (int e = 0; e < 8; ++e)
          if ((mask >> e) & 1)
            atomicOr(&s_mask[warp][(e >> 2) * 16 + ((e & 3) >> 1) * 8 + g],
                     1u << (2 * tq + (e & 1)));
        __syncwarp();
        unsigned bits = s_mask[warp][lane];
        while (bits)
        {
          const int col = __ffs(bits) - 1;
          bits &= bits - 1;
          const int pj = p0 + col;
          if (pj >= m)
            break;
          const float4 p = s_pt[pj];
          if (dist2_pp(qx, qy, qz, p.x, p.y, p.z) <= r2)
          {
            if (MODE == kFill || (MODE == kBuffered && count < buffer))
              dst[count] = __float_as_int(p.w);
            ++count;
          }
        }
        s_mask[warp][lane] = 0;
        __syncwarp();
      }
    }
  }
  if (!active)
    return;
  if (MODE != kFill)
    counts[q] = count;
  if (MODE == kBuffered && count > buffer)
    atomicOr(overflow, 1u);
}

// Nearest with k above 32: a binary heap per query in the output arrays.
template <int KIND>
__global__ void __launch_bounds__(kQueryThreads)
    k_brute_nearest_large(const float4 *__restrict__ values, int64_t n,
                          const float *__restrict__ queries, int64_t nq,
                          const int32_t *__restrict__ kq, int32_t k_all,
                          const int32_t *__restrict__ offsets, int32_t *__restrict__ offsets_out,
                          int32_t *__restrict__ out_idx, float *__restrict__ out_dist)
{
  __shared__ float4 tile[kBruteTile * (KIND == 1 ? 2 : 1)];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < nq;
  KnnTask task{};
  if (active)
  {
    QueryTree tree;
    task = knn_task(t, n, ForestView{nullptr, nullptr, 1}, tree, nq, nullptr, kq, k_all,
                    offsets, offsets_out);
  }
  const bool work = active && task.kk > 0;
  const int kk = work ? task.kk : 0;
  float *hd = work ? out_dist + task.base : nullptr;
  int *hi = work ? out_idx + task.base : nullptr;
  int size = 0;
  float qx = 0, qy = 0, qz = 0;
  if (work)
  {
    qx = __ldg(queries + 3 * task.q);
    qy = __ldg(queries + 3 * task.q + 1);
    qz = __ldg(queries + 3 * task.q + 2);
  }
  float thr = INFINITY;
  for (int64_t t0 = 0; t0 < n; t0 += kBruteTile)
  {
    const int m = load_tile<KIND>(tile, values, n, t0);
    if (!work)
      continue;
    for (int j = 0; j < m; ++j)
    {
      Box3 b;
      int v;
      tile_leaf<KIND>(tile, j, b, v);
      const float s = leaf_dist2<KIND>(qx, qy, qz, b);
      if (s > thr)
        continue;
      const float d = __fsqrt_rn(s);
      if (size < kk)
        heap_push(hd, hi, size, d, v);
      else if (pair_lt(d, v, hd[0], hi[0]))
        heap_sift_down(hd, hi, 0, size, d, v);
      if (size == kk)
        thr = sq_threshold(hd[0]);
    }
  }
  if (!work)
    return;
  for (int len = size; len > 1; --len)
  {
    const float d0 = hd[0];
    const int i0 = hi[0];
    heap_sift_down(hd, hi, 0, len - 1, hd[len - 1], hi[len - 1]);
    hd[len - 1] = d0;
    hi[len - 1] = i0;
  }
}

// Points in Morton order for the filtered brute force: {x, y, z, index}.
__global__ void k_brute_pack_sorted(const float *__restrict__ g, const uint32_t *__restrict__ perm,
                                    int64_t n, float4 *__restrict__ out)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    const uint32_t v = __ldg(perm + i);
    out[i] = make_float4(__ldg(g + 3 * (int64_t)v), __ldg(g + 3 * (int64_t)v + 1),
                         __ldg(g + 3 * (int64_t)v + 2), __int_as_float((int)v));
  }
}

// Pack values in input order: {x, y, z, index} (two float4 per box).
template <int KIND>
__global__ void k_brute_pack(const float *__restrict__ g, int64_t n, float4 *__restrict__ values)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    SortedLeaf<KIND>::store(values, i, load_leaf_box<KIND>(g, i), (int)i);
}

template <int PRED, int KIND>
abx_status spatial_dispatch(cudaStream_t s, TreeView const &t, ForestView const &f,
                            const float *d_preds,
                            int64_t nq, const uint32_t *d_perm, SpatialMode mode,
                            int32_t *d_counts, const int32_t *d_offsets, int32_t *d_out,
                            int32_t buffer, unsigned *d_overflow)
{
  unsigned *err = device_state().d_error;
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("SPATIAL_BUCKET", kDefaultSpatialBucket)));
#define ABX_SPATIAL(M)                                                                      \
  k_spatial<PRED, M, KIND><<<blocks, kQueryThreads, 0, s>>>(t.tnodes, t.sorted, t.n, f, d_preds, \
                                                            nq, d_perm, d_counts, d_offsets,  \
                                                            d_out, buffer, bucket, d_overflow, \
                                                            err)
#define ABX_BRUTE(M)                                                                         \
  k_brute_spatial<PRED, M, KIND><<<blocks, kQueryThreads, 0, s>>>(                               \
      t.sorted, t.n, d_preds, nq, d_perm, d_counts, d_offsets, d_out, buffer, d_overflow)
#define ABX_BRUTE_TC(M)                                                                    \
  k_brute_spatial_tc<M><<<blocks, kQueryThreads, 0, s>>>(t.sorted, t.n, d_preds, nq, d_perm,     \
                                                         d_counts, d_offsets, d_out, buffer,    \
                                                         d_overflow)
  if (!t.tnodes && PRED == ABX_SPHERE && KIND == 0 && t.morton_sorted &&
      tuning_value("BRUTE_TENSOR", 1))
  {
    if (mode == kCount)
      ABX_BRUTE_TC(kCount);
    else if (mode == kFill)
      ABX_BRUTE_TC(kFill);
    else
      ABX_BRUTE_TC(kBuffered);
  }
  else if (!t.tnodes) // brute force: every predicate against every value
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
#undef ABX_BRUTE_TC
#undef ABX_BRUTE
#undef ABX_SPATIAL
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

template <int K, int KIND>
abx_status nearest_k(cudaStream_t s, TreeView const &t, ForestView const &f,
                     const float *d_queries, int64_t nq,
                     const uint32_t *d_perm, const int32_t *d_k, int32_t k,
                     const int32_t *d_offsets, int32_t *d_offsets_out, int32_t *d_idx,
                     float *d_dist, unsigned *err)
{
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("NEAREST_BUCKET", kDefaultNearestBucket)));
  if (!t.tnodes && t.morton_sorted && tuning_value("BRUTE_TENSOR", 1))
  {
    // few queries: split the points into chunks so that about two CTAs per
    // SM run, then merge the chunks' lists
    const int64_t tiles = (t.n + kTcTile - 1) / kTcTile;
    const int64_t want = 2 * (int64_t)device_state().num_sms;
    const int chunks = (int)std::max<int64_t>(
        1, std::min<int64_t>({tiles, (int64_t)64, (want + blocks - 1) / blocks}));
    Scratch<uint64_t> partial;
    if (chunks > 1)
      ABX_CUDA_TRY(partial.alloc((size_t)chunks * nq * K, s));
    k_brute_nearest_tc<K><<<dim3(blocks, chunks), kQueryThreads, 0, s>>>(
        t.morton_sorted, t.n, t.morton_codes, t.d_bounds, d_queries, nq, d_perm, d_k, k, d_offsets,
        d_offsets_out, d_idx, d_dist, chunks > 1 ? partial.ptr : nullptr);
    if (chunks > 1)
      k_brute_merge<K><<<blocks, kQueryThreads, 0, s>>>(partial.ptr, chunks, t.n, nq, d_perm, d_k,
                                                        k, d_offsets, d_idx, d_dist);
  }
  else if (!t.tnodes) // brute force
    k_brute_nearest<K, KIND><<<blocks, kQueryThreads, 0, s>>>(
        t.sorted, t.n, d_queries, nq, d_k, k, d_offsets, d_offsets_out, d_idx, d_dist);
  else if (bucket >= 2)
    k_nearest<K, KIND, true><<<blocks, kQueryThreads, 0, s>>>(
        t.tnodes, t.sorted, t.n, f, d_queries, nq, d_perm, d_k, k, d_offsets, d_offsets_out, d_idx,
        d_dist, bucket, err);
  else
    k_nearest<K, KIND, false><<<blocks, kQueryThreads, 0, s>>>(
        t.tnodes, t.sorted, t.n, f, d_queries, nq, d_perm, d_k, k, d_offsets, d_offsets_out, d_idx,
        d_dist, bucket, err);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

template <int KIND>
abx_status nearest_dispatch(cudaStream_t s, TreeView const &t, ForestView const &f,
                            const float *d_queries,
                            int64_t nq, const uint32_t *d_perm, const int32_t *d_k, int32_t k,
                            int32_t max_k, const int32_t *d_offsets, int32_t *d_offsets_out,
                            int32_t *d_idx, float *d_dist)
{
  unsigned *err = device_state().d_error;
#define ABX_KNN(KV)                                                                             \
  return nearest_k<KV, KIND>(s, t, f, d_queries, nq, d_perm, d_k, k, d_offsets, d_offsets_out, \
                             d_idx, d_dist, err)
  if (max_k <= 1)
    ABX_KNN(1);
  if (max_k <= 2)
    ABX_KNN(2);
  if (max_k <= 4)
    ABX_KNN(4);
  if (max_k <= 8)
    ABX_KNN(8);
  if (max_k <= 16)
    ABX_KNN(16);
  if (max_k <= 32)
    ABX_KNN(32);
#undef ABX_KNN
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("NEAREST_BUCKET", kDefaultNearestBucket)));
  if (!t.tnodes)
    k_brute_nearest_large<KIND><<<blocks, kQueryThreads, 0, s>>>(
        t.sorted, t.n, d_queries, nq, d_k, k, d_offsets, d_offsets_out, d_idx, d_dist);
  else
  k_nearest_large<KIND><<<blocks, kQueryThreads, 0, s>>>(t.tnodes, t.sorted, t.n, f, d_queries, nq,
                                                         d_perm, d_k, k, d_offsets,
                                                         d_offsets_out, d_idx, d_dist, bucket,
                                                         err);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace

abx_status launch_spatial(cudaStream_t s, TreeView const &t, ForestView const *fp,
                          abx_geometry pred_kind, const float *d_preds, int64_t nq,
                          const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                          const int32_t *d_offsets, int32_t *d_out, int32_t buffer,
                          unsigned *d_overflow)
{
  if (nq <= 0 || t.n <= 0)
    return ABX_SUCCESS;
  const ForestView f = fp ? *fp : ForestView{nullptr, nullptr, 1};
  StageScope scope(s, "spatial", 1);
  if (t.ndir > 0 || kdop_ndir(pred_kind) > 0)
    return launch_spatial_kdop(s, t, f, pred_kind, d_preds, nq, d_perm, mode, d_counts, d_offsets,
                               d_out, buffer, d_overflow);
  const bool box_leaves = t.kind == ABX_BOX;
  if (pred_kind == ABX_SPHERE)
    return box_leaves ? spatial_dispatch<ABX_SPHERE, 1>(s, t, f, d_preds, nq, d_perm, mode, d_counts,
                                                        d_offsets, d_out, buffer, d_overflow)
                      : spatial_dispatch<ABX_SPHERE, 0>(s, t, f, d_preds, nq, d_perm, mode, d_counts,
                                                        d_offsets, d_out, buffer, d_overflow);
  if (pred_kind == ABX_BOX)
    return box_leaves ? spatial_dispatch<ABX_BOX, 1>(s, t, f, d_preds, nq, d_perm, mode, d_counts,
                                                     d_offsets, d_out, buffer, d_overflow)
                      : spatial_dispatch<ABX_BOX, 0>(s, t, f, d_preds, nq, d_perm, mode, d_counts,
                                                     d_offsets, d_out, buffer, d_overflow);
  if (pred_kind == ABX_RAY)
    return box_leaves ? spatial_dispatch<ABX_RAY, 1>(s, t, f, d_preds, nq, d_perm, mode, d_counts,
                                                     d_offsets, d_out, buffer, d_overflow)
                      : spatial_dispatch<ABX_RAY, 0>(s, t, f, d_preds, nq, d_perm, mode, d_counts,
                                                     d_offsets, d_out, buffer, d_overflow);
  return fail(ABX_ERROR_INVALID_ARGUMENT, "intersects predicates must be spheres, boxes, rays or KDOPs");
}

abx_status brute_pack_sorted(cudaStream_t s, const float *d_g, const uint32_t *d_perm, int64_t n,
                             float4 *d_out)
{
  if (n <= 0)
    return ABX_SUCCESS;
  k_brute_pack_sorted<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_g, d_perm, n, d_out);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status brute_pack(cudaStream_t s, abx_geometry kind, const float *d_g, int64_t n,
                      float4 *d_values)
{
  if (n <= 0)
    return ABX_SUCCESS;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (kind == ABX_BOX)
    k_brute_pack<1><<<blocks, 256, 0, s>>>(d_g, n, d_values);
  else
    k_brute_pack<0><<<blocks, 256, 0, s>>>(d_g, n, d_values);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status launch_spatial_self(cudaStream_t s, TreeView const &t, int filter,
                               const int32_t *d_leaf_pos, const float *d_spheres, int64_t nq,
                               const uint32_t *d_perm, SpatialMode mode, int32_t *d_counts,
                               const int32_t *d_offsets, int32_t *d_out)
{
  if (nq <= 0 || t.n <= 0)
    return ABX_SUCCESS;
  if (t.kind != ABX_POINT || !t.tnodes)
    return fail(ABX_ERROR_NOT_SUPPORTED, "neighbor lists: point trees only");
  unsigned *err = device_state().d_error;
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("SPATIAL_BUCKET", kDefaultSpatialBucket)));
  const ForestView f{nullptr, nullptr, 1};
  StageScope scope(s, "spatial", 1);
#define ABX_SELF(M, F)                                                                          \
  k_spatial<ABX_SPHERE, M, 0, F><<<blocks, kQueryThreads, 0, s>>>(                              \
      t.tnodes, t.sorted, t.n, f, d_spheres, nq, d_perm, d_counts, d_offsets, d_out, 0, bucket, \
      nullptr, err, d_leaf_pos)
  if (filter == kSkipSelf)
  {
    if (mode == kCount)
      ABX_SELF(kCount, kSkipSelf);
    else
      ABX_SELF(kFill, kSkipSelf);
  }
  else
  {
    if (mode == kCount)
      ABX_SELF(kCount, kEarlierLeaves);
    else
      ABX_SELF(kFill, kEarlierLeaves);
  }
#undef ABX_SELF
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status launch_overflow_list(cudaStream_t s, const int32_t *d_offsets, int64_t nq,
                                int32_t buffer, uint32_t *d_list, int64_t *h_count)
{
  *h_count = 0;
  if (nq <= 0)
    return ABX_SUCCESS;
  Scratch<int32_t> flags, pos;
  ABX_CUDA_TRY(flags.alloc(nq, s));
  ABX_CUDA_TRY(pos.alloc(nq + 1, s));
  const unsigned blocks = (unsigned)((nq + 255) / 256);
  k_overflow_flags<<<blocks, 256, 0, s>>>(d_offsets, nq, buffer, flags.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  ABX_TRY(exclusive_scan_i32(s, flags.ptr, nq, pos.ptr));
  k_overflow_list<<<blocks, 256, 0, s>>>(flags.ptr, pos.ptr, nq, d_list);
  ABX_CUDA_TRY(cudaGetLastError());
  int32_t count = 0;
  ABX_CUDA_TRY(cudaMemcpyAsync(&count, pos.ptr + nq, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  *h_count = count;
  return ABX_SUCCESS;
}

abx_status sample_mean_hits(cudaStream_t s, TreeView const &t, ForestView const *f,
                            abx_geometry pred_kind, const float *d_preds, int64_t nq,
                            const uint32_t *d_perm, int32_t *d_counts, int64_t max_sample,
                            double *h_mean)
{
  *h_mean = 0;
  if (nq <= 0)
    return ABX_SUCCESS;
  const int64_t m = std::min(nq, max_sample);
  const int64_t stride = nq / m;
  Scratch<uint32_t> sample;
  Scratch<unsigned long long> total;
  ABX_CUDA_TRY(sample.alloc(m, s));
  ABX_CUDA_TRY(total.alloc(1, s));
  ABX_CUDA_TRY(cudaMemsetAsync(total.ptr, 0, sizeof(unsigned long long), s));
  const unsigned blocks = (unsigned)((m + 255) / 256);
  k_sample_queries<<<blocks, 256, 0, s>>>(d_perm, stride, m, sample.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  ABX_TRY(launch_spatial(s, t, f, pred_kind, d_preds, m, sample.ptr, kCount, d_counts, nullptr,
                         nullptr, 0, nullptr));
  k_sample_sum<<<blocks, 256, 0, s>>>(d_counts, sample.ptr, m, total.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  unsigned long long sum = 0;
  ABX_CUDA_TRY(cudaMemcpyAsync(&sum, total.ptr, sizeof(sum), cudaMemcpyDeviceToHost, s));
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  *h_mean = (double)sum / (double)m;
  return ABX_SUCCESS;
}

abx_status launch_compact(cudaStream_t s, const int32_t *d_tmp, int64_t nq, int32_t buffer,
                          const int32_t *d_offsets, int32_t *d_out)
{
  if (nq <= 0)
    return ABX_SUCCESS;
  const unsigned blocks = (unsigned)((nq + 255) / 256); // a warp per 32 queries
  StageScope scope(s, "compact", 1);
  k_compact<<<blocks, 256, 0, s>>>(d_tmp, nq, buffer, d_offsets, d_out);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

namespace
{
// dst row j = src row rows[j], rows of w 32-bit words (a value gather of the
// query results).
__global__ void k_gather_rows(const uint32_t *__restrict__ src, int64_t n_src, int w,
                              const int32_t *__restrict__ rows, int64_t m,
                              uint32_t *__restrict__ dst, unsigned *__restrict__ err)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * w)
    return;
  const int64_t j = i / w;
  const int c = (int)(i - j * w);
  const int32_t r = __ldg(rows + j);
  if ((uint64_t)r >= (uint64_t)n_src)
  {
    raise_error(err, ABX_DEVERR_INTERNAL);
    dst[i] = 0;
    return;
  }
  dst[i] = __ldg(src + (int64_t)r * w + c);
}

__global__ void k_offsets_iota(int32_t *__restrict__ out, int64_t count, int64_t first, int64_t step)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count)
    out[i] = (int32_t)((first + i) * step);
}
} // namespace

abx_status gather_rows(cudaStream_t s, const void *d_src, int64_t n_src, int words,
                       const int32_t *d_rows, int64_t m, void *d_dst)
{
  if (m <= 0)
    return ABX_SUCCESS;
  const int64_t total = m * words;
  k_gather_rows<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
      static_cast<const uint32_t *>(d_src), n_src, words, d_rows, m, static_cast<uint32_t *>(d_dst),
      device_state().d_error);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status fill_offsets_iota(cudaStream_t s, int32_t *d_out, int64_t count, int64_t first,
                             int64_t step)
{
  if (count <= 0)
    return ABX_SUCCESS;
  k_offsets_iota<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(d_out, count, first, step);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status launch_nearest(cudaStream_t s, TreeView const &t, ForestView const *fp,
                          const float *d_queries, int64_t nq, const uint32_t *d_perm,
                          const int32_t *d_k, int32_t k, int32_t max_k, const int32_t *d_offsets,
                          int32_t *d_offsets_out, int32_t *d_idx, float *d_dist)
{
  if (nq <= 0)
    return ABX_SUCCESS;
  const ForestView f = fp ? *fp : ForestView{nullptr, nullptr, 1};
  StageScope scope(s, "nearest", 1);
  if (t.kind == ABX_BOX)
    return nearest_dispatch<1>(s, t, f, d_queries, nq, d_perm, d_k, k, max_k, d_offsets,
                               d_offsets_out, d_idx, d_dist);
  return nearest_dispatch<0>(s, t, f, d_queries, nq, d_perm, d_k, k, max_k, d_offsets,
                             d_offsets_out, d_idx, d_dist);
}

abx_status launch_knn_counts(cudaStream_t s, TreeView const &t, ForestView const *fp,
                             const int32_t *d_k, int32_t k, int64_t nq, int32_t *d_counts,
                             int32_t *d_max)
{
  if (nq <= 0)
    return ABX_SUCCESS;
  const ForestView f = fp ? *fp : ForestView{nullptr, nullptr, 1};
  const unsigned blocks = (unsigned)((nq + 255) / 256);
  StageScope scope(s, "knn_counts", 1);
  k_knn_counts<<<blocks, 256, 0, s>>>(t.n, f, d_k, k, nq, d_counts, d_max);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace abx
