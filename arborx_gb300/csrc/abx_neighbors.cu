// abx_neighbors.cu -- kernels of the radius self-join neighbor lists
// (src/spatial/detail/ArborX_NeighborList.hpp:47-188) and of the half-to-full
// expansion (ArborX_ExpandHalfToFull.hpp:23-69).  The traversal itself is the
// spatial kernel with a leaf filter (k_spatial in abx_spatial.cuh, launched
// from abx_query.cu; the half list's walk ends at the point's own leaf).
#include "abx_build.h"

namespace abx
{
namespace
{

// intersects(Sphere{p, r}) for every point (NeighborListPredicateGetter,
// ArborX_NeighborList.hpp:27-45).
__global__ void k_self_spheres(const float *__restrict__ pts, int64_t n, float r,
                               float4 *__restrict__ spheres)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    spheres[i] = make_float4(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], r);
}

// The tree's leaf order: order[t] = value of the leaf at Morton position t,
// pos[value] = t (a box leaf spans two float4, its value in the first).
template <int KIND>
__global__ void k_leaf_order(const float4 *__restrict__ sorted, int64_t n,
                             uint32_t *__restrict__ order, int32_t *__restrict__ pos,
                             unsigned *__restrict__ err)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n)
    return;
  const int v = __float_as_int(sorted[KIND == 1 ? 2 * t : t].w);
  order[t] = (uint32_t)v;
  if ((uint64_t)v < (uint64_t)n)
    pos[v] = (int32_t)t;
  else
    raise_error(err, ABX_DEVERR_INTERNAL);
}

// Mirrored pairs of a half list: entry j of row k (value i) gives the pair
// (key i, value k); rows are taken in order, so pairs are ordered by k.
__global__ void k_mirror_pairs(const int32_t *__restrict__ offsets,
                               const int32_t *__restrict__ indices, int64_t n,
                               uint32_t *__restrict__ keys, uint32_t *__restrict__ vals,
                               int32_t *__restrict__ mirror_count)
{
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n)
    return;
  for (int32_t j = offsets[k]; j < offsets[k + 1]; ++j)
  {
    const int32_t i = indices[j];
    keys[j] = (uint32_t)i;
    vals[j] = (uint32_t)k;
    atomicAdd(mirror_count + i, 1);
  }
}

// counts[i] = half row length + mirrored count.
__global__ void k_full_counts(const int32_t *__restrict__ offsets,
                              const int32_t *__restrict__ mirror_count, int64_t n,
                              int32_t *__restrict__ counts)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    counts[i] = offsets[i + 1] - offsets[i] + mirror_count[i];
}

// Row i of the full list: its half row, then the rows k that list i, in
// ascending k (one warp per row).
__global__ void k_full_fill(const int32_t *__restrict__ half_off, const int32_t *__restrict__ half_idx,
                            const int32_t *__restrict__ mirror_off,
                            const uint32_t *__restrict__ mirror_vals, int64_t n,
                            const int32_t *__restrict__ full_off, int32_t *__restrict__ full_idx)
{
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n)
    return;
  const int32_t h0 = half_off[i], hc = half_off[i + 1] - h0;
  const int32_t m0 = mirror_off[i], mc = mirror_off[i + 1] - m0;
  int32_t *dst = full_idx + full_off[i];
  for (int32_t j = lane; j < hc; j += 32)
    dst[j] = half_idx[h0 + j];
  for (int32_t j = lane; j < mc; j += 32)
    dst[hc + j] = (int32_t)mirror_vals[m0 + j];
}

} // namespace

abx_status self_spheres(cudaStream_t s, const float *d_points, int64_t n, float r,
                        float *d_spheres)
{
  if (n <= 0)
    return ABX_SUCCESS;
  k_self_spheres<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_points, n, r,
                                                             reinterpret_cast<float4 *>(d_spheres));
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status leaf_order(cudaStream_t s, abx_geometry kind, const float4 *d_sorted, int64_t n,
                      uint32_t *d_order, int32_t *d_pos)
{
  if (n <= 0)
    return ABX_SUCCESS;
  unsigned *err = device_state().d_error;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (kind == ABX_BOX)
    k_leaf_order<1><<<blocks, 256, 0, s>>>(d_sorted, n, d_order, d_pos, err);
  else
    k_leaf_order<0><<<blocks, 256, 0, s>>>(d_sorted, n, d_order, d_pos, err);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

abx_status expand_half_to_full(cudaStream_t s, int64_t n, const int32_t *d_half_off,
                               const int32_t *d_half_idx, int64_t m, int32_t *d_full_off,
                               int32_t *d_full_idx)
{
  if (n <= 0)
    return ABX_SUCCESS;
  Scratch<uint32_t> keys, vals, sorted_vals;
  Scratch<int32_t> mirror_count, mirror_off, counts;
  ABX_CUDA_TRY(keys.alloc(std::max<int64_t>(m, 1), s));
  ABX_CUDA_TRY(vals.alloc(std::max<int64_t>(m, 1), s));
  ABX_CUDA_TRY(sorted_vals.alloc(std::max<int64_t>(m, 1), s));
  ABX_CUDA_TRY(mirror_count.alloc(n, s));
  ABX_CUDA_TRY(mirror_off.alloc(n + 1, s));
  ABX_CUDA_TRY(counts.alloc(n, s));
  ABX_CUDA_TRY(cudaMemsetAsync(mirror_count.ptr, 0, n * sizeof(int32_t), s));
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_mirror_pairs<<<blocks, 256, 0, s>>>(d_half_off, d_half_idx, n, keys.ptr, vals.ptr,
                                        mirror_count.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  // stable by key: grouped by i, ascending k inside each group
  int key_bits = 0;
  while ((1ll << key_bits) < n)
    ++key_bits;
  if (m > 0)
    ABX_TRY(radix_sort_u32(s, keys.ptr, sorted_vals.ptr, vals.ptr, m,
                           std::max(1, (key_bits + 7) / 8), nullptr));
  ABX_TRY(exclusive_scan_i32(s, mirror_count.ptr, n, mirror_off.ptr));
  k_full_counts<<<blocks, 256, 0, s>>>(d_half_off, mirror_count.ptr, n, counts.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  ABX_TRY(exclusive_scan_i32(s, counts.ptr, n, d_full_off));
  k_full_fill<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(
      d_half_off, d_half_idx, mirror_off.ptr, sorted_vals.ptr, n, d_full_off, d_full_idx);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace abx
