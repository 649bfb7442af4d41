// abx_build.cu -- BVH construction kernels.
//
//   k_bounds_partial / k_bounds_final   scene bounding box
//       (calculateBoundingBoxOfTheScene, ArborX_TreeConstruction.hpp:26-39)
//   k_morton64                          63-bit Morton code of every centroid,
//       with the radix sort's 8 digit histograms accumulated on the fly
//       (Morton64, ArborX_SpaceFillingCurves.hpp:45-84)
//   k_morton32                          Morton32 of predicate centroids
//       (ArborX_SpaceFillingCurves.hpp:30-43,86-104) + 4 digit histograms
//   k_single_leaf                       the one-leaf tree
//       (ArborX_TreeConstruction.hpp:41-69)
// The hierarchy itself is in abx_hierarchy.cu.
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

// One-leaf tree (ArborX_TreeConstruction.hpp:41-69): leaf {-1, 0}; the
// traversal node holds a one-leaf bucket on the left and nothing on the
// right (count 0).
template <int KIND>
__global__ void k_single_leaf(const float *__restrict__ g, LeafNode *__restrict__ leaves,
                              TNode *__restrict__ tnodes, float4 *__restrict__ sorted,
                              float *__restrict__ bounds)
{
  Box3 b = load_leaf_box<KIND>(g, 0);
  if (leaves)
  {
    leaves[0].rope = kRopeSentinel;
    leaves[0].value = 0;
  }
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

// Row-major copy of values read through strides (access traits).
__global__ void k_pack_strided(const float *__restrict__ data, int64_t value_stride,
                               int64_t coord_stride, int64_t n, int cols, float *__restrict__ out)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  for (int d = 0; d < cols; ++d)
    out[i * cols + d] = __ldg(data + i * value_stride + d * coord_stride);
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
  else if (kind == ABX_RAY)
    k_morton32<3><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_KDOP6)
    k_morton32<4><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_KDOP14)
    k_morton32<5><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_KDOP18)
    k_morton32<6><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else if (kind == ABX_KDOP26)
    k_morton32<7><<<blocks, 256, 0, s>>>(d_g, n, d_scene, d_codes, d_hist);
  else
    return fail(ABX_ERROR_INVALID_ARGUMENT, "predicate kind");
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

abx_status pack_strided(cudaStream_t s, const float *d_data, int64_t value_stride,
                        int64_t coord_stride, int64_t n, int cols, float *d_out)
{
  if (n <= 0)
    return ABX_SUCCESS;
  k_pack_strided<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_data, value_stride, coord_stride,
                                                              n, cols, d_out);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

} // namespace abx
