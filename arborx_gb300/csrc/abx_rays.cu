// abx_rays.cu -- ray predicates: construction of Ray values and the
// ordering pass of ordered_intersects(Ray)
// (src/spatial/detail/ArborX_TreeTraversal.hpp:338-489: leaves reported by
// increasing distance along the ray).  The intersection test itself runs in
// the spatial traversal (RayPred, abx_query.cu).
#include "abx_build.h"

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

} // namespace abx
