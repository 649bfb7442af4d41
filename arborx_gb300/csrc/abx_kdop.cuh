// abx_kdop.cuh -- discrete oriented polytopes KDOP<3, k>, k = 6, 14, 18, 26
// (src/geometry/ArborX_KDOP.hpp:30-183): for each of the k/2 directions a
// [min, max] range of the projections of the geometry on that direction.
//
// A KDOP record in device memory is kdop_pad(NDIR) floats: min[NDIR],
// max[NDIR], then zero padding to a multiple of 4 floats so that every record
// is a whole number of float4 (16-byte aligned).  The host format of a KDOP
// value or predicate is the reference's struct layout: min[NDIR] then
// max[NDIR], 2 * NDIR floats.
//
// Arithmetic restates the reference's formulas exactly: a projection is
// p[0]*dir[0], then += p[1]*dir[1], then += p[2]*dir[2], each operation one
// binary32 rounding (ArborX_Expand.hpp:136-140, ArborX_Intersects.hpp:
// 336-340); min/max are Kokkos::min/max, (b < a ? b : a) and (a < b ? b : a).
#pragma once

#include "abx_common.cuh"

namespace abx
{

// Number of directions of a KDOP geometry kind (0 for other kinds).
__host__ __device__ constexpr int kdop_ndir(int kind)
{
  return kind == ABX_KDOP6 ? 3 : kind == ABX_KDOP14 ? 7 : kind == ABX_KDOP18 ? 9
                               : kind == ABX_KDOP26 ? 13 : 0;
}

// Floats of a padded device record.
__host__ __device__ constexpr int kdop_pad(int ndir) { return (2 * ndir + 3) / 4 * 4; }

// Component a of direction i of KDOP<3, 2 * ndir> (ArborX_KDOP.hpp:64-151):
// the three axes, then for k = 18 and 26 the six edge directions (1,1,0),
// (1,0,1), (0,1,1), (1,-1,0), (1,0,-1), (0,1,-1), then for k = 14 and 26 the
// four corner directions (1,1,1), (1,-1,1), (1,1,-1), (1,-1,-1).
__host__ __device__ constexpr int kdop_dir(int ndir, int i, int a)
{
  if (i < 3)
    return a == i ? 1 : 0;
  const int first_corner = ndir == 7 ? 3 : 9;
  if (ndir != 7 && i < 9)
  {
    const int e = i - 3, j = e % 3;
    const int f = j == 2 ? 1 : 0, s = j == 0 ? 1 : 2;
    return a == f ? 1 : a == s ? (e < 3 ? 1 : -1) : 0;
  }
  const int c = i - first_corner;
  return a == 0 ? 1 : a == 1 ? ((c & 1) ? -1 : 1) : (c >= 2 ? -1 : 1);
}

__device__ __forceinline__ float kokkos_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float kokkos_max(float a, float b) { return (a < b) ? b : a; }

template <int NDIR>
__device__ __forceinline__ float kdop_proj(int i, float x, float y, float z)
{
  float p = __fmul_rn(x, (float)kdop_dir(NDIR, i, 0));
  p = __fadd_rn(p, __fmul_rn(y, (float)kdop_dir(NDIR, i, 1)));
  return __fadd_rn(p, __fmul_rn(z, (float)kdop_dir(NDIR, i, 2)));
}

template <int NDIR>
struct Kdop
{
  float mn[NDIR];
  float mx[NDIR];
};

// KDOP() (ArborX_KDOP.hpp:164-172): every range empty.
template <int NDIR>
__device__ __forceinline__ void kdop_empty(Kdop<NDIR> &k)
{
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
  {
    k.mn[i] = FLT_MAX;
    k.mx[i] = -FLT_MAX;
  }
}

// expand(KDOP, Point) (ArborX_Expand.hpp:128-148).
template <int NDIR>
__device__ __forceinline__ void kdop_expand_point(Kdop<NDIR> &k, float x, float y, float z)
{
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
  {
    const float p = kdop_proj<NDIR>(i, x, y, z);
    k.mn[i] = kokkos_min(k.mn[i], p);
    k.mx[i] = kokkos_max(k.mx[i], p);
  }
}

// expand(KDOP, Box) (ArborX_Expand.hpp:151-208): nothing for a box with an
// inverted range, else the eight corners in the reference's order.
template <int NDIR>
__device__ __forceinline__ void kdop_expand_box(Kdop<NDIR> &k, Box3 const &b)
{
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (b.lo[d] > b.hi[d])
      return;
  const float x[2] = {b.lo[0], b.hi[0]}, y[2] = {b.lo[1], b.hi[1]}, z[2] = {b.lo[2], b.hi[2]};
  // (xmin,ymin,zmin), (xmin,ymax,zmin), (xmin,ymin,zmax), (xmin,ymax,zmax),
  // then the same four with xmax
#pragma unroll
  for (int c = 0; c < 8; ++c)
    kdop_expand_point<NDIR>(k, x[c >> 2], y[c & 1], z[(c >> 1) & 1]);
}

// The KDOP of a box, equal in value to KDOP{} expanded by the box.  For a
// valid box with finite coordinates every projection is finite or an
// overflow to +-inf (never NaN), and a rounded sum is monotone in each term,
// so the eight-corner minimum (maximum) is the projection of the corner
// taking, on each axis, the smaller (larger) term: two projections per
// direction instead of eight.  Other boxes take the eight-corner loop.
template <int NDIR>
__device__ __forceinline__ void kdop_of_box(Kdop<NDIR> &k, Box3 const &b)
{
  bool fast = true;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    fast = fast && b.lo[d] <= b.hi[d] && fabsf(b.lo[d]) <= FLT_MAX && fabsf(b.hi[d]) <= FLT_MAX;
  if (!fast)
  {
    kdop_empty<NDIR>(k);
    kdop_expand_box<NDIR>(k, b);
    return;
  }
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
  {
    constexpr int nd = NDIR;
    const int dx = kdop_dir(nd, i, 0), dy = kdop_dir(nd, i, 1), dz = kdop_dir(nd, i, 2);
    k.mn[i] = kdop_proj<NDIR>(i, dx < 0 ? b.hi[0] : b.lo[0], dy < 0 ? b.hi[1] : b.lo[1],
                              dz < 0 ? b.hi[2] : b.lo[2]);
    k.mx[i] = kdop_proj<NDIR>(i, dx > 0 ? b.hi[0] : b.lo[0], dy > 0 ? b.hi[1] : b.lo[1],
                              dz > 0 ? b.hi[2] : b.lo[2]);
  }
}

// intersects(KDOP, KDOP) (ArborX_Intersects.hpp:350-368); symmetric.
template <int NDIR>
__device__ __forceinline__ bool kdop_overlap(Kdop<NDIR> const &a, Kdop<NDIR> const &b)
{
  bool ok = true;
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
    ok = ok && !(b.mx[i] < a.mn[i] || b.mn[i] > a.mx[i]);
  return ok;
}

// intersects(Point, KDOP) (ArborX_Intersects.hpp:328-348).
template <int NDIR>
__device__ __forceinline__ bool kdop_contains(Kdop<NDIR> const &k, float x, float y, float z)
{
  bool ok = true;
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
  {
    const float p = kdop_proj<NDIR>(i, x, y, z);
    ok = ok && !(p < k.mn[i] || p > k.mx[i]);
  }
  return ok;
}

// A padded device record (kdop_pad(NDIR) / 4 float4).  2 * NDIR is 2 mod 4
// for the odd direction counts, so a record has two spare floats; a leaf
// record keeps its value's bits in the first (returned by kdop_load).
template <int NDIR>
__device__ __forceinline__ int kdop_load(const float4 *__restrict__ rec, Kdop<NDIR> &k)
{
  constexpr int n4 = kdop_pad(NDIR) / 4;
  float f[4 * n4];
#pragma unroll
  for (int j = 0; j < n4; ++j)
  {
    const float4 v = __ldg(rec + j);
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
  return __float_as_int(f[2 * NDIR]);
}

template <int NDIR>
__device__ __forceinline__ void kdop_store(float4 *__restrict__ rec, Kdop<NDIR> const &k,
                                           int value = 0)
{
  static_assert(NDIR % 2 == 1, "records keep a spare float for the value");
  constexpr int n4 = kdop_pad(NDIR) / 4;
  float f[4 * n4];
#pragma unroll
  for (int i = 0; i < 4 * n4; ++i)
    f[i] = 0.f;
#pragma unroll
  for (int i = 0; i < NDIR; ++i)
  {
    f[i] = k.mn[i];
    f[NDIR + i] = k.mx[i];
  }
  f[2 * NDIR] = __int_as_float(value);
#pragma unroll
  for (int j = 0; j < n4; ++j)
    rec[j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
}

// A KDOP in the host format (2 * NDIR floats).
template <int NDIR>
__device__ __forceinline__ void kdop_load_raw(const float *__restrict__ g, int64_t i, Kdop<NDIR> &k)
{
  const float *r = g + 2 * NDIR * i;
#pragma unroll
  for (int j = 0; j < NDIR; ++j)
  {
    k.mn[j] = __ldg(r + j);
    k.mx[j] = __ldg(r + NDIR + j);
  }
}

// Box of a KDOP, expand(Box{}, KDOP) (ArborX_Expand.hpp:210-225): the ranges
// of the first three (axis) directions.
template <int NDIR>
__device__ __forceinline__ Box3 kdop_axis_box(Kdop<NDIR> const &k)
{
  Box3 b;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    b.lo[d] = kokkos_min(FLT_MAX, k.mn[d]);
    b.hi[d] = kokkos_max(-FLT_MAX, k.mx[d]);
  }
  return b;
}

} // namespace abx
