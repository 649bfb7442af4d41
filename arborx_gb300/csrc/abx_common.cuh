// abx_common.cuh -- shared device code of the GB300 BVH library: exact
// binary32 geometry, node layouts, memory-ordering primitives.
//
// Floating point: every operation that decides a result uses an explicit
// round-to-nearest intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn),
// which the compiler never contracts into an FMA, so device results equal the
// reference formulas evaluated one IEEE operation at a time in source order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>

namespace abx
{

constexpr int kRopeSentinel = -1;

// Traversal stack depth.  A node's split bit strictly decreases from parent
// to child over the 94-bit augmented key (63-bit Morton code + 31-bit index
// used for equal codes, ArborX_TreeConstruction.hpp:131-170), so the depth of
// any tree with fewer than 2^31 leaves is at most 95 and a depth-first walk
// never holds more than 95 deferred nodes.
constexpr int kStackDepth = 96;

// ---------------------------------------------------------------------------
// Node layouts
// ---------------------------------------------------------------------------

// Reference layout (src/spatial/detail/ArborX_Node.hpp:24-51).
struct LeafNode
{
  int rope;
  int value;
};

struct __align__(16) InternalNode
{
  int left_child;
  int rope;
  float lo[3];
  float hi[3];
};
static_assert(sizeof(InternalNode) == 32, "reference internal node is 32 B");

// Traversal layout: one 64-byte node per internal node holding the bounding
// boxes of BOTH children plus their references, so a visit is a single
// 64-byte line and both child tests come from one dependent load.
//   a = L.lo.x L.lo.y L.lo.z L.hi.x
//   b = L.hi.y L.hi.z R.lo.x R.lo.y
//   c = R.lo.z R.hi.x R.hi.y R.hi.z
//   d = left ref, right ref, left count, right count
// A reference >= 0 is an internal node (index into the node array, Karras
// numbering, root = 0).  A reference < 0 is a leaf bucket of `count` leaves:
// count 1 is a single leaf whose value is ~ref and whose bounding volume is
// the child box stored in the node itself; count >= 2 covers the leaves at
// sorted positions ~ref .. ~ref + count - 1, whose geometry and values are
// stored contiguously in Morton order (the subtree of every node covering at
// most `leaf size` leaves is collapsed into one bucket); count 0 marks an
// absent child (one-leaf tree).  For point leaves a single leaf's box is the
// degenerate box [p, p]: the point-box distance and intersection formulas
// then reduce bit-for-bit to the point-point ones (closestPoint returns p
// exactly).
struct __align__(64) TNode
{
  float4 a;
  float4 b;
  float4 c;
  int4 d;
};
static_assert(sizeof(TNode) == 64, "traversal node is 64 B");

__host__ __device__ __forceinline__ int bucket_ref(int start) { return ~start; }
__host__ __device__ __forceinline__ bool is_bucket_ref(int ref) { return ref < 0; }
__host__ __device__ __forceinline__ int bucket_start(int ref) { return ~ref; }

struct Box3
{
  float lo[3];
  float hi[3];
};

__device__ __forceinline__ Box3 empty_box()
{
  Box3 b;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    b.lo[d] = FLT_MAX;
    b.hi[d] = -FLT_MAX;
  }
  return b;
}

// expand(Box, Box) (geometry/algorithms/ArborX_Expand.hpp:61-77); min/max are
// exact, fminf/fmaxf equal Kokkos::min/max on non-NaN input.
__device__ __forceinline__ void expand(Box3 &b, Box3 const &o)
{
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    b.lo[d] = fminf(b.lo[d], o.lo[d]);
    b.hi[d] = fmaxf(b.hi[d], o.hi[d]);
  }
}

__device__ __forceinline__ void tnode_children(TNode const &t, Box3 &l, Box3 &r)
{
  l.lo[0] = t.a.x; l.lo[1] = t.a.y; l.lo[2] = t.a.z;
  l.hi[0] = t.a.w; l.hi[1] = t.b.x; l.hi[2] = t.b.y;
  r.lo[0] = t.b.z; r.lo[1] = t.b.w; r.lo[2] = t.c.x;
  r.hi[0] = t.c.y; r.hi[1] = t.c.z; r.hi[2] = t.c.w;
}

__device__ __forceinline__ TNode make_tnode(Box3 const &l, int lref, int lcount, Box3 const &r,
                                            int rref, int rcount)
{
  TNode t;
  t.a = make_float4(l.lo[0], l.lo[1], l.lo[2], l.hi[0]);
  t.b = make_float4(l.hi[1], l.hi[2], r.lo[0], r.lo[1]);
  t.c = make_float4(r.lo[2], r.hi[0], r.hi[1], r.hi[2]);
  t.d = make_int4(lref, rref, lcount, rcount);
  return t;
}

// ---------------------------------------------------------------------------
// Exact geometry
// ---------------------------------------------------------------------------

// distance(Point a, Point b) (geometry/algorithms/ArborX_Distance.hpp:52-70):
// tmp = b - a per dimension, squares accumulated from 0 in order, sqrt.
__device__ __forceinline__ float dist_pp(float ax, float ay, float az, float bx,
                                         float by, float bz)
{
  float tx = __fsub_rn(bx, ax);
  float ty = __fsub_rn(by, ay);
  float tz = __fsub_rn(bz, az);
  float s = __fmul_rn(tx, tx);
  s = __fadd_rn(s, __fmul_rn(ty, ty));
  s = __fadd_rn(s, __fmul_rn(tz, tz));
  return __fsqrt_rn(s);
}

// Squared form of dist_pp (the value whose sqrt is taken).
__device__ __forceinline__ float dist2_pp(float ax, float ay, float az, float bx,
                                          float by, float bz)
{
  float tx = __fsub_rn(bx, ax);
  float ty = __fsub_rn(by, ay);
  float tz = __fsub_rn(bz, az);
  float s = __fmul_rn(tx, tx);
  s = __fadd_rn(s, __fmul_rn(ty, ty));
  return __fadd_rn(s, __fmul_rn(tz, tz));
}

// closestPoint(Point, Box) (geometry/algorithms/ArborX_ClosestPoint.hpp:48-66)
__device__ __forceinline__ float clamp_to_box(float p, float lo, float hi)
{
  return p < lo ? lo : (p > hi ? hi : p);
}

// distance(Point, Box) = distance(p, closestPoint(p, box))
// (geometry/algorithms/ArborX_Distance.hpp:72-80).
__device__ __forceinline__ float dist2_pb(float px, float py, float pz,
                                          Box3 const &b)
{
  return dist2_pp(px, py, pz, clamp_to_box(px, b.lo[0], b.hi[0]),
                  clamp_to_box(py, b.lo[1], b.hi[1]),
                  clamp_to_box(pz, b.lo[2], b.hi[2]));
}

__device__ __forceinline__ float dist_pb(float px, float py, float pz,
                                         Box3 const &b)
{
  return __fsqrt_rn(dist2_pb(px, py, pz, b));
}

// intersects(Box, Box) (geometry/algorithms/ArborX_Intersects.hpp:52-65); for
// a degenerate box [p, p] it equals intersects(Point, Box) (:68-80).
__device__ __forceinline__ bool isect_bb(Box3 const &a, Box3 const &b)
{
  return !(a.lo[0] > b.hi[0] || a.hi[0] < b.lo[0] || a.lo[1] > b.hi[1] ||
           a.hi[1] < b.lo[1] || a.lo[2] > b.hi[2] || a.hi[2] < b.lo[2]);
}

// translateAndScale (geometry/algorithms/ArborX_TranslateAndScale.hpp:25-35).
__device__ __forceinline__ float translate_scale(float x, float a, float b)
{
  return a != b ? __fdiv_rn(__fsub_rn(x, a), __fsub_rn(b, a)) : 0.f;
}

// Bit interleaving by a shift-and-mask ladder.  Stage b moves every source
// bit i whose bit b is set up by 2^(b+1), so that after the stages for bits
// B..0 source bit i sits at 3i.  ladder_mask() derives the set of positions
// occupied after the stages for bits >= b, i.e. the mask of that stage.
__host__ __device__ constexpr uint64_t ladder_mask(int nbits, int b)
{
  uint64_t m = 0;
  for (int i = 0; i < nbits; ++i)
  {
    int handled = i & ~((1 << b) - 1);
    m |= 1ull << (i + 2 * handled);
  }
  return m;
}

// Spread the low 21 bits of x so that bit i lands on bit 3i.
__device__ __forceinline__ uint64_t spread3_21(uint64_t x)
{
  constexpr uint64_t m4 = ladder_mask(21, 4), m3 = ladder_mask(21, 3),
                     m2 = ladder_mask(21, 2), m1 = ladder_mask(21, 1),
                     m0 = ladder_mask(21, 0);
  x &= 0x1fffffull;
  x = (x | (x << 32)) & m4;
  x = (x | (x << 16)) & m3;
  x = (x | (x << 8)) & m2;
  x = (x | (x << 4)) & m1;
  x = (x | (x << 2)) & m0;
  return x;
}

// Spread the low 10 bits of x so that bit i lands on bit 3i.
__device__ __forceinline__ uint32_t spread3_10(uint32_t x)
{
  constexpr uint32_t m3 = (uint32_t)ladder_mask(10, 3), m2 = (uint32_t)ladder_mask(10, 2),
                     m1 = (uint32_t)ladder_mask(10, 1), m0 = (uint32_t)ladder_mask(10, 0);
  x &= 0x3ffu;
  x = (x | (x << 16)) & m3;
  x = (x | (x << 8)) & m2;
  x = (x | (x << 4)) & m1;
  x = (x | (x << 2)) & m0;
  return x;
}

// morton64 for a 3-D point already mapped to the unit cube
// (spatial/detail/ArborX_MortonCode.hpp:318-347): per axis
// clamp(x * 2^21, 0, 2^21 - 1) in float, truncated, interleaved with x on the
// highest bit of each triplet.
__device__ __forceinline__ uint64_t morton64_unit(float x, float y, float z)
{
  const float N = 2097152.f;
  const float M = 2097151.f;
  float fx = __fmul_rn(x, N), fy = __fmul_rn(y, N), fz = __fmul_rn(z, N);
  fx = fx < 0.f ? 0.f : (M < fx ? M : fx);
  fy = fy < 0.f ? 0.f : (M < fy ? M : fy);
  fz = fz < 0.f ? 0.f : (M < fz ? M : fz);
  uint64_t ux = (uint64_t)fx, uy = (uint64_t)fy, uz = (uint64_t)fz;
  return (spread3_21(ux) << 2) + (spread3_21(uy) << 1) + spread3_21(uz);
}

// morton32 for a 3-D point in the unit cube (ArborX_MortonCode.hpp:291-316):
// 10 bits per axis, clamp(x * 1024, 0, 1023) in float.
__device__ __forceinline__ uint32_t morton32_unit(float x, float y, float z)
{
  const float N = 1024.f;
  const float M = 1023.f;
  float fx = __fmul_rn(x, N), fy = __fmul_rn(y, N), fz = __fmul_rn(z, N);
  fx = fx < 0.f ? 0.f : (M < fx ? M : fx);
  fy = fy < 0.f ? 0.f : (M < fy ? M : fy);
  fz = fz < 0.f ? 0.f : (M < fz ? M : fz);
  uint32_t ux = (uint32_t)fx, uy = (uint32_t)fy, uz = (uint32_t)fz;
  return (spread3_10(ux) << 2) + (spread3_10(uy) << 1) + spread3_10(uz);
}

// ---------------------------------------------------------------------------
// Geometry access
// ---------------------------------------------------------------------------

// Centroid of a value (geometry/algorithms/ArborX_Centroid.hpp:40-60).  The
// general form takes the KDOP kinds 4..7 (2 * ndir floats each): the centroid
// of the KDOP's axis box, Box{} expanded by the first three directions'
// ranges (ArborX_Centroid.hpp:84-94).
template <int KIND>
__device__ __forceinline__ void load_centroid(const float *g, int64_t i, float &x,
                                              float &y, float &z)
{
  static_assert(KIND >= 4 && KIND <= 7, "geometry kind");
  constexpr int nd = KIND == 4 ? 3 : KIND == 5 ? 7 : KIND == 6 ? 9 : 13;
  const float *k = g + 2 * nd * i;
  float c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    const float mn = __ldg(k + d), mx = __ldg(k + nd + d);
    const float lo = mn < FLT_MAX ? mn : FLT_MAX;
    const float hi = -FLT_MAX < mx ? mx : -FLT_MAX;
    c[d] = __fdiv_rn(__fadd_rn(lo, hi), 2.f);
  }
  x = c[0];
  y = c[1];
  z = c[2];
}

// KIND: 0 point (3 floats), 1 box (6 floats), 2 sphere (4 floats).
template <>
__device__ __forceinline__ void load_centroid<0>(const float *g, int64_t i,
                                                 float &x, float &y, float &z)
{
  x = __ldg(g + 3 * i);
  y = __ldg(g + 3 * i + 1);
  z = __ldg(g + 3 * i + 2);
}

template <>
__device__ __forceinline__ void load_centroid<1>(const float *g, int64_t i,
                                                 float &x, float &y, float &z)
{
  const float *b = g + 6 * i;
  x = __fdiv_rn(__fadd_rn(__ldg(b + 0), __ldg(b + 3)), 2.f);
  y = __fdiv_rn(__fadd_rn(__ldg(b + 1), __ldg(b + 4)), 2.f);
  z = __fdiv_rn(__fadd_rn(__ldg(b + 2), __ldg(b + 5)), 2.f);
}

template <>
__device__ __forceinline__ void load_centroid<2>(const float *g, int64_t i,
                                                 float &x, float &y, float &z)
{
  x = __ldg(g + 4 * i);
  y = __ldg(g + 4 * i + 1);
  z = __ldg(g + 4 * i + 2);
}

// A ray's centroid is its origin (returnCentroid, ArborX_Ray.hpp:78-82).
template <>
__device__ __forceinline__ void load_centroid<3>(const float *g, int64_t i,
                                                 float &x, float &y, float &z)
{
  x = __ldg(g + 6 * i);
  y = __ldg(g + 6 * i + 1);
  z = __ldg(g + 6 * i + 2);
}

// intersection(Ray, Box, tmin, tmax) (ArborX_Ray.hpp:107-158): slab test of
// a ray (origin o, normalized direction d) with a zero direction component
// handled through signs; the comparisons never let a NaN update the bounds.
__device__ __forceinline__ bool ray_box_intersection(float const (&o)[3], float const (&d)[3],
                                                     Box3 const &b, float &tmin, float &tmax)
{
  tmin = -INFINITY;
  tmax = INFINITY;
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    float tdmin, tdmax;
    if (d[k] == 0.f)
    {
      const float min_orig = __fsub_rn(b.lo[k], o[k]);
      if (min_orig == 0.f)
        continue;
      const float max_orig = __fsub_rn(b.hi[k], o[k]);
      tdmin = signbit(__fmul_rn(d[k], max_orig)) ? INFINITY : -INFINITY;
      tdmax = signbit(__fmul_rn(d[k], min_orig)) ? INFINITY : -INFINITY;
    }
    else if (d[k] > 0.f)
    {
      tdmin = __fdiv_rn(__fsub_rn(b.lo[k], o[k]), d[k]);
      tdmax = __fdiv_rn(__fsub_rn(b.hi[k], o[k]), d[k]);
    }
    else
    {
      tdmin = __fdiv_rn(__fsub_rn(b.hi[k], o[k]), d[k]);
      tdmax = __fdiv_rn(__fsub_rn(b.lo[k], o[k]), d[k]);
    }
    if (tmin < tdmin)
      tmin = tdmin;
    if (tmax > tdmax)
      tmax = tdmax;
  }
  return tmin <= tmax;
}

// distance(Ray, Box) (ArborX_Ray.hpp:435-447): entry distance max(tmin, 0)
// of a box in front of the ray, +inf otherwise.
__device__ __forceinline__ float ray_box_distance(float const (&o)[3], float const (&d)[3],
                                                  Box3 const &b)
{
  float t0, t1;
  const bool hit = ray_box_intersection(o, d, b, t0, t1) && t1 >= 0.f;
  return hit ? (t0 < 0.f ? 0.f : t0) : INFINITY;
}

// Bounding box of a leaf value: expand(empty, indexable).
template <int KIND>
__device__ __forceinline__ Box3 load_leaf_box(const float *g, int64_t i)
{
  Box3 b;
  if (KIND == 0)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      float v = __ldg(g + 3 * i + d);
      b.lo[d] = fminf(FLT_MAX, v);
      b.hi[d] = fmaxf(-FLT_MAX, v);
    }
  }
  else
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      b.lo[d] = fminf(FLT_MAX, __ldg(g + 6 * i + d));
      b.hi[d] = fmaxf(-FLT_MAX, __ldg(g + 6 * i + 3 + d));
    }
  }
  return b;
}

// Leaf geometry in Morton order (the buckets' storage): points as
// {x, y, z, value}; boxes as {lo.x, lo.y, lo.z, value}, {hi.x, hi.y, hi.z, 0}.
template <int KIND>
struct SortedLeaf;

template <>
struct SortedLeaf<0>
{
  static constexpr int kFloat4s = 1;
  static __device__ __forceinline__ void store(float4 *s, int64_t i, Box3 const &b, int value)
  {
    s[i] = make_float4(b.lo[0], b.lo[1], b.lo[2], __int_as_float(value));
  }
  static __device__ __forceinline__ void load(const float4 *__restrict__ s, int64_t i, Box3 &b,
                                              int &value)
  {
    const float4 v = __ldg(s + i);
    b.lo[0] = b.hi[0] = v.x;
    b.lo[1] = b.hi[1] = v.y;
    b.lo[2] = b.hi[2] = v.z;
    value = __float_as_int(v.w);
  }
};

template <>
struct SortedLeaf<1>
{
  static constexpr int kFloat4s = 2;
  static __device__ __forceinline__ void store(float4 *s, int64_t i, Box3 const &b, int value)
  {
    s[2 * i] = make_float4(b.lo[0], b.lo[1], b.lo[2], __int_as_float(value));
    s[2 * i + 1] = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.f);
  }
  static __device__ __forceinline__ void load(const float4 *__restrict__ s, int64_t i, Box3 &b,
                                              int &value)
  {
    const float4 u = __ldg(s + 2 * i);
    const float4 v = __ldg(s + 2 * i + 1);
    b.lo[0] = u.x;
    b.lo[1] = u.y;
    b.lo[2] = u.z;
    b.hi[0] = v.x;
    b.hi[1] = v.y;
    b.hi[2] = v.z;
    value = __float_as_int(u.w);
  }
};

// Segment containing global position i of a batch of trees: the largest s
// in [lo, hi] with off[s] <= i (empty trees share offsets with their
// successor and are skipped).  The caller knows i lies in segments lo..hi.
__device__ __forceinline__ int find_segment_in(const int64_t *off, int lo, int hi, int64_t i)
{
  while (lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_segment(const int64_t *__restrict__ off, int nseg, int64_t i)
{
  return find_segment_in(off, 0, nseg - 1, i);
}

// ---------------------------------------------------------------------------
// Memory ordering
// ---------------------------------------------------------------------------

__device__ __forceinline__ int atomic_cas_acq_rel(int *addr, int expected, int desired)
{
  int old;
  asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;"
               : "=r"(old)
               : "l"(addr), "r"(expected), "r"(desired)
               : "memory");
  return old;
}

__device__ __forceinline__ int atomic_cas_relaxed(int *addr, int expected, int desired)
{
  int old;
  asm volatile("atom.relaxed.gpu.global.cas.b32 %0, [%1], %2, %3;"
               : "=r"(old)
               : "l"(addr), "r"(expected), "r"(desired)
               : "memory");
  return old;
}

// atomicAdd with acquire-release semantics at GPU scope: the adder's earlier
// stores are visible to whoever later reads the count, and the adder sees
// the stores that preceded the earlier adds.
__device__ __forceinline__ unsigned atomic_add_acq_rel(unsigned *addr, unsigned v)
{
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(addr), "r"(v)
               : "memory");
  return old;
}

__device__ __forceinline__ void fence_acq_rel_gpu()
{
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v)
{
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned lanemask_lt()
{
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ void raise_error(unsigned *err, unsigned bits)
{
  if (err)
    atomicOr(err, bits);
}

} // namespace abx
