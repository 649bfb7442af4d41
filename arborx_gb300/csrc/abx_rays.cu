// abx_rays.cu -- ray predicates: construction of Ray values and the
// ordering pass of ordered_intersects(Ray)
// (src/spatial/detail/ArborX_TreeTraversal.hpp:338-489: leaves reported by
// increasing distance along the ray), and nearest(Ray, k), the first k of
// those leaves, by a pruned walk.  The intersection test of intersects(Ray)
// runs in the spatial traversal (RayPred, abx_spatial.cuh).
#include "abx_spatial.cuh"

namespace abx
{
namespace
{

// Ray{origin, direction} (ArborX_Ray.hpp:46-55, misc/ArborX_Vector.hpp:40-88):
// the direction divided by its norm, both in double, rounded to float.
__global__ void k_ray_normalize(const float *__restrict__ raw, int64_t n, float *__restrict__ out)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const float *r = raw + 6 * i;
  double s = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    s = __dadd_rn(s, __dmul_rn((double)r[3 + d], (double)r[3 + d]));
  const double mag = __dsqrt_rn(s);
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    out[6 * i + d] = r[d];
    out[6 * i + 3 + d] = __double2float_rn(__ddiv_rn((double)r[3 + d], mag));
  }
}

// For every result e of ray q: its value, row and distance along the ray
// (one thread per ray).
template <int KIND>
__global__ void k_ray_entries(const float *__restrict__ rays, int64_t nq,
                              const int32_t *__restrict__ offsets,
                              const int32_t *__restrict__ indices,
                              const float4 *__restrict__ sorted, const int32_t *__restrict__ pos,
                              uint32_t *__restrict__ values, uint32_t *__restrict__ rows,
                              float *__restrict__ dist, int64_t n, unsigned *__restrict__ err)
{
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  float o[3], d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    o[k] = rays[6 * q + k];
    d[k] = rays[6 * q + 3 + k];
  }
  for (int32_t e = offsets[q]; e < offsets[q + 1]; ++e)
  {
    const int v = indices[e];
    values[e] = (uint32_t)v;
    rows[e] = (uint32_t)q;
    const int p = (uint64_t)v < (uint64_t)n ? pos[v] : -1;
    if ((uint64_t)p >= (uint64_t)n)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      dist[e] = INFINITY;
      continue;
    }
    Box3 b;
    int vv;
    SortedLeaf<KIND>::load(sorted, p, b, vv);
    dist[e] = ray_box_distance(o, d, b);
  }
}

// key of entry perm[j]: its row above the bits of its (non-negative)
// distance, so that the unsigned order is (row, distance).  A ray starting on
// a box has the distance -0 (max(-0, 0) keeps -0), equal to 0 in the
// reference's comparisons: adding +0 makes it +0 in the key.
__global__ void k_ray_keys(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ rows,
                           const float *__restrict__ dist, int64_t m, uint64_t *__restrict__ keys)
{
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m)
  {
    const uint32_t e = perm[j];
    keys[j] = ((uint64_t)rows[e] << 32) | __float_as_uint(__fadd_rn(dist[e], 0.f));
  }
}

__global__ void k_truncated_counts(const int32_t *__restrict__ offsets, int64_t nq, int32_t k,
                                   int32_t *__restrict__ counts)
{
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq)
    counts[q] = min(offsets[q + 1] - offsets[q], k);
}

// Row q of the output: the first (new_off[q+1] - new_off[q]) entries of its
// ordered row (one warp per row).
__global__ void k_ordered_gather(const int32_t *__restrict__ offsets,
                                 const int32_t *__restrict__ new_off, int64_t nq,
                                 const uint32_t *__restrict__ order,
                                 const int32_t *__restrict__ indices,
                                 const float *__restrict__ dist, int32_t *__restrict__ out_idx,
                                 float *__restrict__ out_dist)
{
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= nq)
    return;
  const int32_t o = offsets[q], no = new_off[q], c = new_off[q + 1] - no;
  for (int32_t j = lane; j < c; j += 32)
  {
    const uint32_t e = order[o + j];
    out_idx[no + j] = indices[e];
    if (out_dist)
      out_dist[no + j] = dist[e];
  }
}

// nearest(Ray, k): the first k leaves of the ray's ordered_intersects row,
// ordered by (entry distance, value) with -0 equal to +0.  One ray per
// thread keeps its best k as sorted 64-bit keys (the bits of the distance
// plus 0, above value + 1) in registers, the first K - k slots holding the
// key 0 that is never displaced; bit j of `neg` records that slot j's
// distance was -0 (a ray starting on the box's entry face), which the output
// restores.  The walk visits the nearer passing child first and skips a
// child whose entry distance exceeds the k-th best: a box inside another has
// an entry distance at least the outer one's (each slab time is a rounded
// (bound - origin) / direction, monotone in the bound, and the entry is
// their maximum clamped at 0), and node boxes are exact unions of their
// children, so no leaf of the row is lost.  Equal distances are kept
// (ties go by value).  The leaf test and distance are those of the
// intersects traversal and of the ordering pass (ray_box_intersection with
// t1 >= 0, entry max(t0, 0)).
constexpr uint64_t kRayKeyEmpty = ~0ull;

template <int K, int KIND>
__global__ void __launch_bounds__(kQueryThreads)
    k_ray_nearest(const TNode *__restrict__ nodes, const float4 *__restrict__ sorted, int64_t n,
                  const float *__restrict__ rays, int64_t nq, const uint32_t *__restrict__ perm,
                  int32_t k, int bucket, int32_t *__restrict__ counts,
                  int32_t *__restrict__ dense_idx, float *__restrict__ dense_dist,
                  unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int64_t q = perm ? (int64_t)__ldg(perm + t) : t;
  const RayPred ray = PredOf<ABX_RAY>::load(rays, q);
  uint64_t key[K];
  uint64_t neg = 0;
  const int first = K - k;
#pragma unroll
  for (int j = 0; j < K; ++j)
    key[j] = j < first ? 0ull : kRayKeyEmpty;
  float thr = INFINITY;

  // entry distance of a box the ray passes (the intersects test), else false
  auto entry = [&](Box3 const &b, float &dist) -> bool {
    float t0, t1;
    if (!(ray_box_intersection(ray.o, ray.d, b, t0, t1) && t1 >= 0.f))
      return false;
    dist = t0 < 0.f ? 0.f : t0;
    return true;
  };
  auto offer = [&](float dist, int v) {
    const float c = __fadd_rn(dist, 0.f);
    const uint64_t ck = ((uint64_t)__float_as_uint(c) << 32) | (uint32_t)(v + 1);
    if (!(ck < key[K - 1]))
      return;
    bool lt[K];
    int p = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
    {
      lt[j] = ck < key[j];
      p += lt[j] ? 0 : 1;
    }
#pragma unroll
    for (int j = K - 1; j >= 1; --j)
      key[j] = lt[j - 1] ? key[j - 1] : (lt[j] ? ck : key[j]);
    key[0] = lt[0] ? ck : key[0];
    const uint64_t below = neg & ((1ull << p) - 1);
    neg = below | ((neg >> p) << (p + 1)) | ((uint64_t)signbit(dist) << p);
    if (key[K - 1] != kRayKeyEmpty)
      thr = __uint_as_float((uint32_t)(key[K - 1] >> 32));
  };
  // a child that passed with entry distance dist; true for an internal node
  // to descend into
  auto visit = [&](int ref, int cf, float dist) -> bool {
    int start = 0, cnt = 0;
    const ChildKind kind = child_kind<true>(ref, cf, bucket, start, cnt);
    if (kind == kLeaf)
      offer(dist, bucket_start(ref));
    else if (kind == kScan)
    {
      for (int j = 0; j < cnt; ++j)
      {
        Box3 b;
        int v;
        SortedLeaf<KIND>::load(sorted, start + j, b, v);
        float d;
        if (entry(b, d) && __fadd_rn(d, 0.f) <= thr)
          offer(d, v);
      }
    }
    return kind == kDescend;
  };

  int sref[kStackDepth];
  float sdist[kStackDepth];
  int sp = 0;
  int node = 0;
  const int64_t num_nodes = n > 1 ? n - 1 : 1;
  int64_t budget = num_nodes; // each node is visited at most once
  while (true)
  {
    if (--budget < 0 || (uint64_t)node >= (uint64_t)num_nodes)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      break;
    }
    const TNode tn = load_tnode(nodes, node);
    Box3 l, r;
    tnode_children(tn, l, r);
    const int lref = tn.d.x, rref = tn.d.y;
    const bool rnone = is_bucket_ref(rref) && tn.d.w == 0; // one-leaf tree
    float dl = 0.f, dr = 0.f;
    const bool hl = entry(l, dl);
    const bool hr = !rnone && entry(r, dr);
    const float cl = hl ? __fadd_rn(dl, 0.f) : INFINITY;
    const float cr = hr ? __fadd_rn(dr, 0.f) : INFINITY;
    // leaves and scanned buckets first (they may lower thr), then the
    // internal children that still pass
    const bool vl = hl && cl <= thr && visit(lref, tn.d.z, dl);
    const bool vr = hr && cr <= thr && visit(rref, tn.d.w, dr);
    const bool gl = vl && cl <= thr;
    const bool gr = vr && cr <= thr;
    if (gl && gr)
    {
      const bool left_first = cl <= cr;
      node = left_first ? lref : rref;
      if (sp < kStackDepth)
      {
        sref[sp] = left_first ? rref : lref;
        sdist[sp] = left_first ? cr : cl;
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
  int c = 0;
  const int64_t base = q * (int64_t)k;
#pragma unroll
  for (int j = 0; j < K; ++j)
  {
    if (j >= first && key[j] != kRayKeyEmpty)
    {
      dense_idx[base + c] = (int)(uint32_t)key[j] - 1;
      if (dense_dist)
        dense_dist[base + c] =
            ((neg >> j) & 1) ? -0.f : __uint_as_float((uint32_t)(key[j] >> 32));
      ++c;
    }
  }
  counts[q] = c;
}

// Row q of the output: the first counts[q] entries of ray q's dense row of k.
__global__ void k_ray_nearest_compact(const int32_t *__restrict__ offsets, int64_t nq, int32_t k,
                                      const int32_t *__restrict__ dense_idx,
                                      const float *__restrict__ dense_dist,
                                      int32_t *__restrict__ out_idx, float *__restrict__ out_dist)
{
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nq * (int64_t)k)
    return;
  const int64_t q = e / k;
  const int j = (int)(e - q * k);
  const int32_t o = offsets[q];
  if (j >= offsets[q + 1] - o)
    return;
  out_idx[o + j] = dense_idx[e];
  if (out_dist)
    out_dist[o + j] = dense_dist[e];
}

template <int K>
void launch_ray_nearest(cudaStream_t s, abx_geometry leaf_kind, const TNode *nodes,
                        const float4 *sorted, int64_t n, const float *rays, int64_t nq,
                        const uint32_t *perm, int32_t k, int bucket, int32_t *counts,
                        int32_t *dense_idx, float *dense_dist, unsigned *err)
{
  const unsigned blocks = (unsigned)((nq + kQueryThreads - 1) / kQueryThreads);
  if (leaf_kind == ABX_BOX)
    k_ray_nearest<K, 1><<<blocks, kQueryThreads, 0, s>>>(nodes, sorted, n, rays, nq, perm, k,
                                                          bucket, counts, dense_idx, dense_dist,
                                                          err);
  else
    k_ray_nearest<K, 0><<<blocks, kQueryThreads, 0, s>>>(nodes, sorted, n, rays, nq, perm, k,
                                                          bucket, counts, dense_idx, dense_dist,
                                                          err);
}

} // namespace

abx_status ray_normalize(cudaStream_t s, const float *d_raw, int64_t n, float *d_out)
{
  if (n <= 0)
    return ABX_SUCCESS;
  k_ray_normalize<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_raw, n, d_out);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status order_ray_results(cudaStream_t s, abx_geometry leaf_kind, const float4 *d_sorted,
                             int64_t n, const float *d_rays, int64_t nq, const int32_t *d_offsets,
                             const int32_t *d_indices, int64_t m, int32_t k,
                             int32_t *d_new_offsets, int32_t *d_out_idx, float *d_out_dist,
                             int64_t *h_new_total)
{
  *h_new_total = 0;
  if (nq <= 0)
    return ABX_SUCCESS;
  const unsigned qblocks = (unsigned)((nq + 255) / 256);
  if (m == 0)
  {
    ABX_CUDA_TRY(cudaMemsetAsync(d_new_offsets, 0, (nq + 1) * sizeof(int32_t), s));
    return ABX_SUCCESS;
  }
  Scratch<uint32_t> order_leaf, values, rows, perm1, perm2;
  Scratch<int32_t> pos, counts;
  Scratch<float> dist;
  Scratch<uint64_t> keys;
  ABX_CUDA_TRY(order_leaf.alloc(n, s));
  ABX_CUDA_TRY(pos.alloc(n, s));
  ABX_CUDA_TRY(values.alloc(m, s));
  ABX_CUDA_TRY(rows.alloc(m, s));
  ABX_CUDA_TRY(perm1.alloc(m, s));
  ABX_CUDA_TRY(perm2.alloc(m, s));
  ABX_CUDA_TRY(dist.alloc(m, s));
  ABX_CUDA_TRY(keys.alloc(m, s));
  ABX_CUDA_TRY(counts.alloc(nq, s));
  ABX_TRY(leaf_order(s, leaf_kind, d_sorted, n, order_leaf.ptr, pos.ptr));
  unsigned *err = device_state().d_error;
  if (leaf_kind == ABX_BOX)
    k_ray_entries<1><<<qblocks, 256, 0, s>>>(d_rays, nq, d_offsets, d_indices, d_sorted, pos.ptr,
                                             values.ptr, rows.ptr, dist.ptr, n, err);
  else
    k_ray_entries<0><<<qblocks, 256, 0, s>>>(d_rays, nq, d_offsets, d_indices, d_sorted, pos.ptr,
                                             values.ptr, rows.ptr, dist.ptr, n, err);
  ABX_CUDA_TRY(cudaGetLastError());
  // stable by value, then stable by (row, distance): rows in order, each by
  // increasing distance, equal distances by value
  int vbits = 0;
  while ((1ll << vbits) < n)
    ++vbits;
  ABX_TRY(radix_sort_u32(s, values.ptr, perm1.ptr, nullptr, m, std::max(1, (vbits + 7) / 8),
                         nullptr));
  const unsigned eblocks = (unsigned)((m + 255) / 256);
  k_ray_keys<<<eblocks, 256, 0, s>>>(perm1.ptr, rows.ptr, dist.ptr, m, keys.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  int rbits = 0;
  while ((1ll << rbits) < nq)
    ++rbits;
  ABX_TRY(radix_sort_u64(s, keys.ptr, perm2.ptr, perm1.ptr, m, (32 + rbits + 7) / 8, nullptr));
  const int32_t kk = k > 0 ? k : INT32_MAX;
  k_truncated_counts<<<qblocks, 256, 0, s>>>(d_offsets, nq, kk, counts.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  ABX_TRY(exclusive_scan_i32(s, counts.ptr, nq, d_new_offsets));
  int32_t total = 0;
  ABX_CUDA_TRY(cudaMemcpyAsync(&total, d_new_offsets + nq, sizeof(int32_t),
                               cudaMemcpyDeviceToHost, s));
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  *h_new_total = total;
  k_ordered_gather<<<(unsigned)((nq * 32 + 255) / 256), 256, 0, s>>>(
      d_offsets, d_new_offsets, nq, perm2.ptr, d_indices, dist.ptr, d_out_idx, d_out_dist);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status ray_nearest(cudaStream_t s, abx_geometry leaf_kind, const TNode *d_nodes,
                       const float4 *d_sorted, int64_t n, const float *d_rays, int64_t nq,
                       const uint32_t *d_perm, int32_t k, bool with_dist, int32_t *d_offsets,
                       int32_t **d_idx, float **d_dist, int64_t *h_total)
{
  *d_idx = nullptr;
  *d_dist = nullptr;
  *h_total = 0;
  if (n < 1 || k < 1 || k > kRayNearestMaxK)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "ray_nearest: needs a tree and 1 <= k <= 32");
  if (nq <= 0)
  {
    ABX_CUDA_TRY(cudaMemsetAsync(d_offsets, 0, sizeof(int32_t), s));
    ABX_CUDA_TRY(dmalloc_n(d_idx, 0, s));
    if (with_dist)
      ABX_CUDA_TRY(dmalloc_n(d_dist, 0, s));
    return ABX_SUCCESS;
  }
  Scratch<int32_t> counts, dense_idx;
  Scratch<float> dense_dist;
  ABX_CUDA_TRY(counts.alloc(nq, s));
  ABX_CUDA_TRY(dense_idx.alloc((size_t)nq * k, s));
  if (with_dist)
    ABX_CUDA_TRY(dense_dist.alloc((size_t)nq * k, s));
  unsigned *err = device_state().d_error;
  const int bucket =
      std::max(1, std::min(kMaxBucket, tuning_value("RAY_BUCKET", kDefaultSpatialBucket)));
  float *dd = with_dist ? dense_dist.ptr : nullptr;
#define ABX_RAY_NEAREST(KK)                                                                     \
  launch_ray_nearest<KK>(s, leaf_kind, d_nodes, d_sorted, n, d_rays, nq, d_perm, k, bucket,     \
                         counts.ptr, dense_idx.ptr, dd, err)
  if (k <= 1)
    ABX_RAY_NEAREST(1);
  else if (k <= 2)
    ABX_RAY_NEAREST(2);
  else if (k <= 4)
    ABX_RAY_NEAREST(4);
  else if (k <= 8)
    ABX_RAY_NEAREST(8);
  else if (k <= 16)
    ABX_RAY_NEAREST(16);
  else
    ABX_RAY_NEAREST(32);
#undef ABX_RAY_NEAREST
  ABX_CUDA_TRY(cudaGetLastError());
  ABX_TRY(exclusive_scan_i32(s, counts.ptr, nq, d_offsets));
  int32_t total = 0;
  ABX_CUDA_TRY(
      cudaMemcpyAsync(&total, d_offsets + nq, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  ABX_CUDA_TRY(dmalloc_n(d_idx, (size_t)total, s));
  if (with_dist && dmalloc_n(d_dist, (size_t)total, s) != cudaSuccess)
  {
    dfree(*d_idx, s);
    *d_idx = nullptr;
    return fail(ABX_ERROR_OUT_OF_MEMORY, "ray_nearest: distances");
  }
  const int64_t m = nq * (int64_t)k;
  k_ray_nearest_compact<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(
      d_offsets, nq, k, dense_idx.ptr, dd, *d_idx, *d_dist);
  ABX_CUDA_TRY(cudaGetLastError());
  *h_total = total;
  return ABX_SUCCESS;
}

} // namespace abx
