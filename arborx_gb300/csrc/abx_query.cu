// abx_query.cu -- query traversal kernels over the 64-byte child-pair nodes.
//
//   k_spatial   intersects(Sphere | Box) predicates, one thread per query,
//               depth-first with the left subtree first.  Hits come out in
//               the same order as the reference's rope walk
//               (TreeTraversal<Spatial>, ArborX_TreeTraversal.hpp:97-119);
//               modes count / fill / buffered implement the CRS passes of
//               ArborX_CrsGraphWrapperImpl.hpp:148-323.
//   k_nearest   nearest(Point, k) with the k best (distance, index) pairs in
//               registers (k <= 32), closer child first, pruning by the k-th
//               distance (TreeTraversal<Nearest>, ArborX_TreeTraversal.hpp:
//               180-335, with the heap replaced by a sorted register list).
//   k_nearest_large  the same for k > 32 with a bounded max-heap kept in the
//               query's slice of the output arrays (misc/ArborX_Heap.hpp).
#include <algorithm>
#include <cmath>

#include "abx_build.h"

namespace abx
{
namespace
{

constexpr int kQueryThreads = 128;

__device__ __forceinline__ TNode load_tnode(const TNode *__restrict__ nodes, int i)
{
  const float4 *p = reinterpret_cast<const float4 *>(nodes + i);
  TNode t;
  t.a = __ldg(p);
  t.b = __ldg(p + 1);
  t.c = __ldg(p + 2);
  float4 d = __ldg(p + 3);
  t.d = make_int4(__float_as_int(d.x), __float_as_int(d.y), 0, 0);
  return t;
}

struct SpherePred
{
  float cx, cy, cz, r;
  __device__ __forceinline__ bool test(Box3 const &b) const
  {
    // intersects(Sphere, Box) (ArborX_Intersects.hpp:83-92)
    return dist_pb(cx, cy, cz, b) <= r;
  }
};

struct BoxPred
{
  Box3 b;
  __device__ __forceinline__ bool test(Box3 const &o) const { return isect_bb(b, o); }
};

template <int PRED>
struct PredOf;
template <>
struct PredOf<ABX_SPHERE>
{
  using type = SpherePred;
  static __device__ __forceinline__ SpherePred load(const float *p, int64_t q)
  {
    const float *s = p + 4 * q;
    return SpherePred{__ldg(s), __ldg(s + 1), __ldg(s + 2), __ldg(s + 3)};
  }
};
template <>
struct PredOf<ABX_BOX>
{
  using type = BoxPred;
  static __device__ __forceinline__ BoxPred load(const float *p, int64_t q)
  {
    const float *s = p + 6 * q;
    BoxPred b;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      b.b.lo[d] = __ldg(s + d);
      b.b.hi[d] = __ldg(s + 3 + d);
    }
    return b;
  }
};

template <int PRED, int MODE>
__global__ void __launch_bounds__(kQueryThreads)
    k_spatial(const TNode *__restrict__ nodes, int64_t n, const float *__restrict__ preds,
              int64_t nq, const uint32_t *__restrict__ perm, int32_t *__restrict__ counts,
              const int32_t *__restrict__ offsets, int32_t *__restrict__ out, int32_t buffer,
              unsigned *__restrict__ overflow, unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int64_t q = perm ? (int64_t)__ldg(perm + t) : t;
  const auto pred = PredOf<PRED>::load(preds, q);

  int32_t *dst = nullptr;
  int32_t cap = 0;
  if (MODE == kFill)
    dst = out + __ldg(offsets + q);
  if (MODE == kBuffered)
  {
    dst = out + q * (int64_t)buffer;
    cap = buffer;
  }
  int32_t count = 0;
  auto emit = [&](int ref) {
    const int v = leaf_value(ref);
    if (MODE == kFill)
      dst[count] = v;
    if (MODE == kBuffered && count < cap)
      dst[count] = v;
    ++count;
  };

  if (n == 1)
  {
    TNode tn = load_tnode(nodes, 0);
    Box3 l, r;
    tnode_children(tn, l, r);
    if (pred.test(l))
      emit(tn.d.x);
  }
  else
  {
    int stack[kStackDepth];
    int sp = 0;
    int node = 0;
    // a depth-first walk visits each of the n - 1 internal nodes at most once
    int64_t budget = n;
    while (true)
    {
      if (--budget < 0 || (uint64_t)node >= (uint64_t)(n - 1))
      {
        raise_error(err, ABX_DEVERR_INTERNAL);
        break;
      }
      const TNode tn = load_tnode(nodes, node);
      Box3 l, r;
      tnode_children(tn, l, r);
      const int lref = tn.d.x, rref = tn.d.y;
      const bool hl = pred.test(l);
      const bool hr = pred.test(r);
      bool has_next = false;
      int next = 0;
      if (hl)
      {
        if (is_leaf_ref(lref))
          emit(lref);
        else
        {
          next = lref;
          has_next = true;
        }
      }
      if (hr)
      {
        if (!has_next && is_leaf_ref(rref))
          emit(rref);
        else if (!has_next)
        {
          next = rref;
          has_next = true;
        }
        else if (sp < kStackDepth)
          stack[sp++] = rref;
        else
          raise_error(err, ABX_DEVERR_STACK_OVERFLOW);
      }
      while (!has_next && sp > 0)
      {
        const int ref = stack[--sp];
        if (is_leaf_ref(ref))
          emit(ref);
        else
        {
          next = ref;
          has_next = true;
        }
      }
      if (!has_next)
        break;
      node = next;
    }
  }
  if (MODE != kFill)
    counts[q] = count;
  if (MODE == kBuffered && count > cap)
    atomicOr(overflow, 1u);
}

__global__ void k_compact(const int32_t *__restrict__ tmp, int64_t nq, int32_t buffer,
                          const int32_t *__restrict__ offsets, int32_t *__restrict__ out)
{
  // one warp per query
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= nq)
    return;
  const int32_t o = offsets[q];
  const int32_t c = offsets[q + 1] - o;
  const int32_t *src = tmp + q * (int64_t)buffer;
  for (int j = lane; j < c; j += 32)
    out[o + j] = src[j];
}

// (distance, index) order of the k-nearest result.
__device__ __forceinline__ bool pair_lt(float da, int ia, float db, int ib)
{
  return da < db || (da == db && ia < ib);
}

template <int K>
__device__ __forceinline__ void list_insert(float (&bd)[K], int (&bi)[K], float d, int v)
{
  bool done = false;
#pragma unroll
  for (int j = K - 1; j >= 1; --j)
  {
    const bool move = !done && pair_lt(d, v, bd[j - 1], bi[j - 1]);
    const bool place = !done && !move;
    bd[j] = move ? bd[j - 1] : (place ? d : bd[j]);
    bi[j] = move ? bi[j - 1] : (place ? v : bi[j]);
    done = done || place;
  }
  if (!done)
  {
    bd[0] = d;
    bi[0] = v;
  }
}

// The list keeps K slots; the first K - k hold (-inf, -1) sentinels that no
// candidate displaces, so the k-th best is always slot K - 1 (static index).
template <int K>
__global__ void __launch_bounds__(kQueryThreads)
    k_nearest(const TNode *__restrict__ nodes, int64_t n, const float *__restrict__ queries,
              int64_t nq, const uint32_t *__restrict__ perm, const int32_t *__restrict__ kq,
              int32_t k_all, const int32_t *__restrict__ offsets,
              int32_t *__restrict__ offsets_out, int32_t *__restrict__ out_idx,
              float *__restrict__ out_dist, unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int64_t q = perm ? (int64_t)__ldg(perm + t) : t;
  int k = kq ? __ldg(kq + q) : k_all;
  k = k < 0 ? 0 : k;
  const int kk = (int)((int64_t)k < n ? (int64_t)k : n);
  const int64_t base = offsets ? (int64_t)__ldg(offsets + q) : q * (int64_t)kk;
  if (offsets_out)
  {
    offsets_out[q] = (int32_t)base;
    if (q == nq - 1)
      offsets_out[nq] = (int32_t)(base + kk);
  }
  if (kk == 0)
    return;

  float bd[K];
  int bi[K];
  const int first = K - k;
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    bd[j] = j < first ? -INFINITY : INFINITY;
    bi[j] = j < first ? -1 : 0x7fffffff;
  }
  const float qx = __ldg(queries + 3 * q), qy = __ldg(queries + 3 * q + 1),
              qz = __ldg(queries + 3 * q + 2);

  if (n == 1)
  {
    TNode tn = load_tnode(nodes, 0);
    Box3 l, r;
    tnode_children(tn, l, r);
    list_insert<K>(bd, bi, dist_pb(qx, qy, qz, l), leaf_value(tn.d.x));
  }
  else
  {
    int sref[kStackDepth];
    float sdist[kStackDepth];
    int sp = 0;
    int node = 0;
    int64_t budget = n; // each internal node is visited at most once
    while (true)
    {
      if (--budget < 0 || (uint64_t)node >= (uint64_t)(n - 1))
      {
        raise_error(err, ABX_DEVERR_INTERNAL);
        break;
      }
      const TNode tn = load_tnode(nodes, node);
      Box3 l, r;
      tnode_children(tn, l, r);
      const int lref = tn.d.x, rref = tn.d.y;
      const float dl = dist_pb(qx, qy, qz, l);
      const float dr = dist_pb(qx, qy, qz, r);
      const bool ll = is_leaf_ref(lref), rl = is_leaf_ref(rref);
      if (ll && pair_lt(dl, leaf_value(lref), bd[K - 1], bi[K - 1]))
        list_insert<K>(bd, bi, dl, leaf_value(lref));
      if (rl && pair_lt(dr, leaf_value(rref), bd[K - 1], bi[K - 1]))
        list_insert<K>(bd, bi, dr, leaf_value(rref));
      const float rad = bd[K - 1];
      const bool gl = !ll && dl <= rad;
      const bool gr = !rl && dr <= rad;
      if (gl && gr)
      {
        const bool left_first = dl <= dr;
        node = left_first ? lref : rref;
        if (sp < kStackDepth)
        {
          sref[sp] = left_first ? rref : lref;
          sdist[sp] = left_first ? dr : dl;
          ++sp;
        }
        else
          raise_error(err, ABX_DEVERR_STACK_OVERFLOW);
      }
      else if (gl)
        node = lref;
      else if (gr)
        node = rref;
      else
      {
        bool found = false;
        while (sp > 0)
        {
          --sp;
          if (sdist[sp] <= bd[K - 1])
          {
            node = sref[sp];
            found = true;
            break;
          }
        }
        if (!found)
          break;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    if (j >= first && j < first + kk)
    {
      out_idx[base + (j - first)] = bi[j];
      if (out_dist)
        out_dist[base + (j - first)] = bd[j];
    }
  }
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
    int parent = (pos - 1) / 2;
    if (!pair_lt(hd[parent], hi[parent], d, v))
      break;
    hd[pos] = hd[parent];
    hi[pos] = hi[parent];
    pos = parent;
  }
  hd[pos] = d;
  hi[pos] = v;
}

__device__ void heap_offer(float *hd, int *hi, int &size, int k, float d, int v)
{
  if (size < k)
    heap_push(hd, hi, size, d, v);
  else if (pair_lt(d, v, hd[0], hi[0]))
    heap_sift_down(hd, hi, 0, size, d, v);
}

__global__ void __launch_bounds__(kQueryThreads)
    k_nearest_large(const TNode *__restrict__ nodes, int64_t n,
                    const float *__restrict__ queries, int64_t nq,
                    const uint32_t *__restrict__ perm, const int32_t *__restrict__ kq,
                    int32_t k_all, const int32_t *__restrict__ offsets,
                    int32_t *__restrict__ offsets_out, int32_t *__restrict__ out_idx,
                    float *__restrict__ out_dist, unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int64_t q = perm ? (int64_t)__ldg(perm + t) : t;
  int k = kq ? __ldg(kq + q) : k_all;
  k = k < 0 ? 0 : k;
  const int kk = (int)((int64_t)k < n ? (int64_t)k : n);
  const int64_t base = offsets ? (int64_t)__ldg(offsets + q) : q * (int64_t)kk;
  if (offsets_out)
  {
    offsets_out[q] = (int32_t)base;
    if (q == nq - 1)
      offsets_out[nq] = (int32_t)(base + kk);
  }
  if (kk == 0)
    return;
  float *hd = out_dist + base;
  int *hi = out_idx + base;
  int size = 0;
  const float qx = queries[3 * q], qy = queries[3 * q + 1], qz = queries[3 * q + 2];
  if (n == 1)
  {
    TNode tn = load_tnode(nodes, 0);
    Box3 l, r;
    tnode_children(tn, l, r);
    heap_offer(hd, hi, size, kk, dist_pb(qx, qy, qz, l), leaf_value(tn.d.x));
  }
  else
  {
    int sref[kStackDepth];
    float sdist[kStackDepth];
    int sp = 0;
    int node = 0;
    int64_t budget = n; // each internal node is visited at most once
    while (true)
    {
      if (--budget < 0 || (uint64_t)node >= (uint64_t)(n - 1))
      {
        raise_error(err, ABX_DEVERR_INTERNAL);
        break;
      }
      const TNode tn = load_tnode(nodes, node);
      Box3 l, r;
      tnode_children(tn, l, r);
      const int lref = tn.d.x, rref = tn.d.y;
      const float dl = dist_pb(qx, qy, qz, l);
      const float dr = dist_pb(qx, qy, qz, r);
      const bool ll = is_leaf_ref(lref), rl = is_leaf_ref(rref);
      if (ll)
        heap_offer(hd, hi, size, kk, dl, leaf_value(lref));
      if (rl)
        heap_offer(hd, hi, size, kk, dr, leaf_value(rref));
      const float rad = size == kk ? hd[0] : INFINITY;
      const bool gl = !ll && dl <= rad;
      const bool gr = !rl && dr <= rad;
      if (gl && gr)
      {
        const bool left_first = dl <= dr;
        node = left_first ? lref : rref;
        if (sp < kStackDepth)
        {
          sref[sp] = left_first ? rref : lref;
          sdist[sp] = left_first ? dr : dl;
          ++sp;
        }
        else
          raise_error(err, ABX_DEVERR_STACK_OVERFLOW);
      }
      else if (gl)
        node = lref;
      else if (gr)
        node = rref;
      else
      {
        bool found = false;
        while (sp > 0)
        {
          --sp;
          const float radn = size == kk ? hd[0] : INFINITY;
          if (sdist[sp] <= radn)
          {
            node = sref[sp];
            found = true;
            break;
          }
        }
        if (!found)
          break;
      }
    }
  }
  // heap sort into ascending (distance, index) order
  for (int len = size; len > 1; --len)
  {
    float d0 = hd[0];
    int i0 = hi[0];
    float dl = hd[len - 1];
    int il = hi[len - 1];
    heap_sift_down(hd, hi, 0, len - 1, dl, il);
    hd[len - 1] = d0;
    hi[len - 1] = i0;
  }
}

__global__ void k_knn_counts(const int32_t *__restrict__ kq, int64_t nq, int64_t n,
                             int32_t *__restrict__ counts, int32_t *__restrict__ kmax)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int32_t m = 0;
  if (i < nq)
  {
    int32_t k = kq[i];
    k = k < 0 ? 0 : k;
    counts[i] = (int32_t)((int64_t)k < n ? (int64_t)k : n);
    m = k;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0)
    atomicMax(kmax, m);
}

template <int PRED>
abx_status spatial_dispatch(cudaStream_t s, TreeView const &t, const float *d_preds,
                            int64_t nq, const uint32_t *d_perm, SpatialMode mode,
                            int32_t *d_counts, const int32_t *d_offsets, int32_t *d_out,
                            int32_t buffer, unsigned *d_overflow)
{
  unsigned *err = device_state().d_error;
  unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  StageScope scope(s, "spatial", 1);
  if (mode == kCount)
    k_spatial<PRED, kCount><<<blocks, kQueryThreads, 0, s>>>(
        t.tnodes, t.n, d_preds, nq, d_perm, d_counts, d_offsets, d_out, buffer, d_overflow, err);
  else if (mode == kFill)
    k_spatial<PRED, kFill><<<blocks, kQueryThreads, 0, s>>>(
        t.tnodes, t.n, d_preds, nq, d_perm, d_counts, d_offsets, d_out, buffer, d_overflow, err);
  else
    k_spatial<PRED, kBuffered><<<blocks, kQueryThreads, 0, s>>>(
        t.tnodes, t.n, d_preds, nq, d_perm, d_counts, d_offsets, d_out, buffer, d_overflow, err);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace

abx_status launch_spatial(cudaStream_t s, TreeView const &t, abx_geometry pred_kind,
                          const float *d_preds, int64_t nq, const uint32_t *d_perm,
                          SpatialMode mode, int32_t *d_counts, const int32_t *d_offsets,
                          int32_t *d_out, int32_t buffer, unsigned *d_overflow)
{
  if (nq <= 0 || t.n <= 0)
    return ABX_SUCCESS;
  if (pred_kind == ABX_SPHERE)
    return spatial_dispatch<ABX_SPHERE>(s, t, d_preds, nq, d_perm, mode, d_counts, d_offsets,
                                        d_out, buffer, d_overflow);
  if (pred_kind == ABX_BOX)
    return spatial_dispatch<ABX_BOX>(s, t, d_preds, nq, d_perm, mode, d_counts, d_offsets,
                                     d_out, buffer, d_overflow);
  return fail(ABX_ERROR_INVALID_ARGUMENT, "intersects predicates must be spheres or boxes");
}

abx_status launch_compact(cudaStream_t s, const int32_t *d_tmp, int64_t nq, int32_t buffer,
                          const int32_t *d_offsets, int32_t *d_out)
{
  if (nq <= 0)
    return ABX_SUCCESS;
  unsigned blocks = (unsigned)((nq * 32 + 255) / 256);
  StageScope scope(s, "compact", 1);
  k_compact<<<blocks, 256, 0, s>>>(d_tmp, nq, buffer, d_offsets, d_out);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status launch_nearest(cudaStream_t s, TreeView const &t, const float *d_queries,
                          int64_t nq, const uint32_t *d_perm, const int32_t *d_k,
                          int32_t k, int32_t max_k, const int32_t *d_offsets,
                          int32_t *d_offsets_out, int32_t *d_idx, float *d_dist)
{
  if (nq <= 0)
    return ABX_SUCCESS;
  unsigned *err = device_state().d_error;
  unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  StageScope scope(s, "nearest", 1);
#define ABX_KNN(KV)                                                                        \
  k_nearest<KV><<<blocks, kQueryThreads, 0, s>>>(t.tnodes, t.n, d_queries, nq, d_perm, d_k, \
                                                 k, d_offsets, d_offsets_out, d_idx, d_dist, \
                                                 err)
  if (max_k <= 1)
    ABX_KNN(1);
  else if (max_k <= 2)
    ABX_KNN(2);
  else if (max_k <= 4)
    ABX_KNN(4);
  else if (max_k <= 8)
    ABX_KNN(8);
  else if (max_k <= 16)
    ABX_KNN(16);
  else if (max_k <= 32)
    ABX_KNN(32);
  else
    k_nearest_large<<<blocks, kQueryThreads, 0, s>>>(t.tnodes, t.n, d_queries, nq, d_perm, d_k,
                                                     k, d_offsets, d_offsets_out, d_idx,
                                                     d_dist, err);
#undef ABX_KNN
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status launch_knn_counts(cudaStream_t s, const int32_t *d_k, int64_t nq, int64_t n,
                             int32_t *d_counts, int32_t *d_max)
{
  if (nq <= 0)
    return ABX_SUCCESS;
  unsigned blocks = (unsigned)((nq + 255) / 256);
  StageScope scope(s, "knn_counts", 1);
  k_knn_counts<<<blocks, 256, 0, s>>>(d_k, nq, n, d_counts, d_max);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace abx
