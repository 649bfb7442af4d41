// abx_spatial.cuh -- the spatial traversal kernel k_spatial and what it
// shares with the nearest kernels: the query's tree, node loads, the exact
// squared-distance threshold and the predicate types.  Included by the query
// translation units (abx_query.cu; abx_kdop.cu instantiates the KDOP forms;
// abx_rays.cu uses the node loads and the ray predicate for nearest(Ray, k)).
//
//   k_spatial   intersects(Sphere | Box | Ray | KDOP) predicates, one thread
//               per query, depth-first with the left subtree first and the
//               leaves of a bucket in Morton order.  Hits come out in the same
//               order as the reference's rope walk (TreeTraversal<Spatial>,
//               ArborX_TreeTraversal.hpp:97-119); modes count / fill /
//               buffered implement the CRS passes of
//               ArborX_CrsGraphWrapperImpl.hpp:148-323.
#pragma once

#include "abx_build.h"
#include "abx_kdop.cuh"

namespace abx
{
namespace
{

constexpr int kQueryThreads = 128;

// The tree a query runs on: root node slot and number of leaves (a forest
// query finds its tree from the query offsets).
struct QueryTree
{
  int root;
  int64_t size;
};

__device__ __forceinline__ QueryTree query_tree(int64_t q, int64_t n, ForestView const &f)
{
  if (!f.qoff)
    return QueryTree{0, n};
  const int s = find_segment(f.qoff, f.nseg, q);
  const int64_t lo = __ldg(f.tree_off + s);
  return QueryTree{(int)lo, __ldg(f.tree_off + s + 1) - lo};
}

__device__ __forceinline__ TNode load_tnode(const TNode *__restrict__ nodes, int i)
{
  const float4 *p = reinterpret_cast<const float4 *>(nodes + i);
  TNode t;
  t.a = __ldg(p);
  t.b = __ldg(p + 1);
  t.c = __ldg(p + 2);
  const float4 d = __ldg(p + 3);
  t.d = make_int4(__float_as_int(d.x), __float_as_int(d.y), __float_as_int(d.z),
                  __float_as_int(d.w));
  return t;
}

// Largest float s with sqrt_rn(s) <= r, for r >= 0 (+inf for r = +inf).
// RN(r * r) lies within a couple of ulps of the answer (sqrt_rn(RN(r*r)) = r
// without overflow or underflow), so the two bounded walks always finish.
__device__ __forceinline__ float sq_threshold(float r)
{
  if (!(r < INFINITY))
    return INFINITY;
  float t = __fmul_rn(r, r);
#pragma unroll 1
  for (int i = 0; i < 8 && __fsqrt_rn(t) > r; ++i)
    t = __int_as_float(__float_as_int(t) - 1);
#pragma unroll 1
  for (int i = 0; i < 8; ++i)
  {
    const float u = __int_as_float(__float_as_int(t) + 1);
    if (__fsqrt_rn(u) <= r)
      t = u;
    else
      break;
  }
  return t;
}

// A bound above sq_threshold(r) within a few ulps, without square roots.
// sqrt_rn(s) <= r needs sqrt(s) <= r + ulp(r)/2, i.e. s <= r^2 + r ulp(r) +
// ulp(r)^2/4, and r ulp(r) <= 2 ulp(r^2): RU(r r) + 3 ulps lies above every
// such s (subnormal squares included).  Pruning with it visits a few more
// candidates than the exact threshold and keeps every result exact, because
// a candidate enters the k-nearest list only by its exact key.
__device__ __forceinline__ float sq_bound(float r)
{
  const float t = __fmul_ru(r, r);
  return t < INFINITY ? __uint_as_float(__float_as_uint(t) + 3u) : INFINITY;
}

// Squared distance from a point to a leaf's bounding volume.
template <int KIND>
__device__ __forceinline__ float leaf_dist2(float qx, float qy, float qz, Box3 const &b)
{
  if (KIND == 0)
    return dist2_pp(qx, qy, qz, b.lo[0], b.lo[1], b.lo[2]);
  return dist2_pb(qx, qy, qz, b);
}

// intersects(Sphere, .) with the radius test done on squared distances:
// sphere-box (ArborX_Intersects.hpp:83-92) and, for point leaves,
// sphere-point (:106-115).
struct SpherePred
{
  static constexpr bool kRetestLeaf = false;
  float cx, cy, cz, r, r2;
  __device__ __forceinline__ bool test(Box3 const &b) const { return dist2_pb(cx, cy, cz, b) <= r2; }
  template <int KIND>
  __device__ __forceinline__ bool test_leaf(Box3 const &b) const
  {
    return leaf_dist2<KIND>(cx, cy, cz, b) <= r2;
  }
};

// intersects(Box, .): box-box (ArborX_Intersects.hpp:52-65), for point leaves
// point-box through reverse dispatch (:68-80; the degenerate box [p, p] gives
// the same comparisons).
struct BoxPred
{
  static constexpr bool kRetestLeaf = false;
  Box3 b;
  __device__ __forceinline__ bool test(Box3 const &o) const { return isect_bb(b, o); }
  template <int KIND>
  __device__ __forceinline__ bool test_leaf(Box3 const &o) const
  {
    return isect_bb(b, o);
  }
};

// intersects(Ray, .): the box in front of the ray (ArborX_Ray.hpp:160-168);
// point leaves are degenerate boxes.  Rows hold the normalized ray.
struct RayPred
{
  static constexpr bool kRetestLeaf = false;
  float o[3], d[3];
  __device__ __forceinline__ bool test(Box3 const &b) const
  {
    float t0, t1;
    return ray_box_intersection(o, d, b, t0, t1) && t1 >= 0.f;
  }
  template <int KIND>
  __device__ __forceinline__ bool test_leaf(Box3 const &b) const
  {
    return test(b);
  }
};

// intersects(KDOP, .): against a box, the KDOP of the box's corners
// (ArborX_Intersects.hpp:317-326); against a point leaf, the point test
// (:328-348, through reverse dispatch).  A single point leaf is stored as the
// child box [p, p], whose KDOP test equals the point test only for finite
// coordinates, so single leaves are tested again as points (kRetestLeaf).
template <int NDIR>
struct KdopPred
{
  static constexpr bool kRetestLeaf = true;
  Kdop<NDIR> k;
  __device__ __forceinline__ bool test(Box3 const &b) const
  {
    Kdop<NDIR> o;
    kdop_of_box<NDIR>(o, b);
    return kdop_overlap<NDIR>(k, o);
  }
  template <int KIND>
  __device__ __forceinline__ bool test_leaf(Box3 const &b) const
  {
    if (KIND == 0)
      return kdop_contains<NDIR>(k, b.lo[0], b.lo[1], b.lo[2]);
    return test(b);
  }
};

template <int PRED>
struct PredOf;
template <>
struct PredOf<ABX_RAY>
{
  static __device__ __forceinline__ RayPred load(const float *p, int64_t q)
  {
    const float *r = p + 6 * q;
    RayPred rp;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
      rp.o[k] = __ldg(r + k);
      rp.d[k] = __ldg(r + 3 + k);
    }
    return rp;
  }
};
template <>
struct PredOf<ABX_SPHERE>
{
  static __device__ __forceinline__ SpherePred load(const float *p, int64_t q)
  {
    const float *s = p + 4 * q;
    SpherePred sp{__ldg(s), __ldg(s + 1), __ldg(s + 2), __ldg(s + 3), 0.f};
    // a negative radius matches nothing (sqrt_rn(s) >= 0 > r)
    sp.r2 = sp.r >= 0.f ? sq_threshold(sp.r) : -1.f;
    return sp;
  }
};
template <>
struct PredOf<ABX_BOX>
{
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

template <int PRED, int NDIR = kdop_ndir(PRED)>
struct KdopPredOf
{
  static __device__ __forceinline__ KdopPred<NDIR> load(const float *p, int64_t q)
  {
    KdopPred<NDIR> kp;
    kdop_load_raw<NDIR>(p, q, kp.k);
    return kp;
  }
};
template <>
struct PredOf<ABX_KDOP6> : KdopPredOf<ABX_KDOP6>
{
};
template <>
struct PredOf<ABX_KDOP14> : KdopPredOf<ABX_KDOP14>
{
};
template <>
struct PredOf<ABX_KDOP18> : KdopPredOf<ABX_KDOP18>
{
};
template <>
struct PredOf<ABX_KDOP26> : KdopPredOf<ABX_KDOP26>
{
};

// The predicate of a query on a KDOP-bounded tree as a KDOP: a box predicate
// becomes the KDOP of its corners (intersects(Box, KDOP) reverses to
// ArborX_Intersects.hpp:317-326), a KDOP predicate stays itself.
template <int NDIR>
__device__ __forceinline__ Kdop<NDIR> as_kdop(BoxPred const &p)
{
  Kdop<NDIR> k;
  kdop_of_box<NDIR>(k, p.b);
  return k;
}
template <int NDIR>
__device__ __forceinline__ Kdop<NDIR> as_kdop(KdopPred<NDIR> const &p)
{
  return p.k;
}
template <int NDIR, class P>
__device__ __forceinline__ Kdop<NDIR> as_kdop(P const &)
{
  Kdop<NDIR> k; // not reached: the launcher admits box and KDOP predicates only
  kdop_empty<NDIR>(k);
  return k;
}

// ---------------------------------------------------------------------------
// Spatial
// ---------------------------------------------------------------------------

// How a traversal handles a child slot (ref, count field): descend into an
// internal node, take a single leaf (its box is the child box), or scan the
// leaves of a small internal subtree from the Morton-ordered copy.
enum ChildKind
{
  kDescend = 0,
  kLeaf = 1,
  kScan = 2,
  kNone = 3
};

template <bool SCAN>
__device__ __forceinline__ ChildKind child_kind(int ref, int cf, int bucket, int &start, int &cnt)
{
  if (is_bucket_ref(ref))
    return cf == 0 ? kNone : kLeaf;
  if (!SCAN)
    return kDescend;
  const int c = cf & 0xffff;
  if (c >= 2 && c <= bucket)
  {
    cnt = c;
    start = (cf & kBucketRightEnd) ? ref - c + 1 : ref;
    return kScan;
  }
  return kDescend;
}

// Leaf filters of a self-query (predicate q built from the value q itself):
// kKeepAll, kSkipSelf (a value never matches its own predicate) or
// kEarlierLeaves (only values whose leaf precedes q's leaf in Morton order,
// leaf_pos[value] = its position: the pairs of the reference's
// HalfTraversal, ArborX_HalfTraversal.hpp:52-73).
enum LeafFilter
{
  kKeepAll = 0,
  kSkipSelf = 1,
  kEarlierLeaves = 2
};

// NDIR > 0: a KDOP-bounded tree (KIND 1 leaf boxes give the values; node
// slot s of node i is the KDOP record knodes[(2 i + s) * kdop_pad(NDIR) / 4],
// the leaf at sorted position t is kleaves[t * kdop_pad(NDIR) / 4]); every
// node and leaf test is the KDOP overlap with the predicate's KDOP.
template <int PRED, int MODE, int KIND, int FILTER = kKeepAll, int NDIR = 0>
__global__ void __launch_bounds__(kQueryThreads)
    k_spatial(const TNode *__restrict__ nodes, const float4 *__restrict__ sorted, int64_t n,
              ForestView f, const float *__restrict__ preds, int64_t nq,
              const uint32_t *__restrict__ perm, int32_t *__restrict__ counts,
              const int32_t *__restrict__ offsets, int32_t *__restrict__ out, int32_t buffer,
              int bucket, unsigned *__restrict__ overflow, unsigned *__restrict__ err,
              const int32_t *__restrict__ leaf_pos = nullptr,
              const float4 *__restrict__ knodes = nullptr,
              const float4 *__restrict__ kleaves = nullptr)
{
  constexpr int kRec = kdop_pad(NDIR) / 4; // float4 per KDOP record
  using QK = Kdop<(NDIR > 0 ? NDIR : 1)>;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int64_t q = perm ? (int64_t)__ldg(perm + t) : t;
  const QueryTree tree = query_tree(q, n, f);
  if (tree.size <= 0)
  {
    if (MODE != kFill)
      counts[q] = 0;
    return;
  }
  const auto pred = PredOf<PRED>::load(preds, q);
  QK qk;
  if constexpr (NDIR > 0)
    qk = as_kdop<NDIR>(pred);

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
  const int32_t own_pos = FILTER == kEarlierLeaves ? __ldg(leaf_pos + q) : 0;
  // kEarlierLeaves: the walk reaches leaves in Morton order (left child
  // first, buckets scanned in order), so after a passing leaf at or past the
  // query's own position every later leaf is filtered too: the walk ends
  // there (in the reference, the half traversal starts at the leaf's rope)
  bool done = false;
  auto emit = [&](int v) {
    if (FILTER == kSkipSelf && v == q)
      return;
    if (FILTER == kEarlierLeaves && __ldg(leaf_pos + v) >= own_pos)
    {
      done = true;
      return;
    }
    if (MODE == kFill)
      dst[count] = v;
    if (MODE == kBuffered && count < cap)
      dst[count] = v;
    ++count;
  };
  // the leaves of a small subtree, in Morton (= rope walk) order
  auto scan = [&](int start, int cnt) {
    for (int j = 0; j < cnt; ++j)
    {
      if constexpr (NDIR > 0)
      {
        QK lk;
        const int v = kdop_load<NDIR>(kleaves + (int64_t)(start + j) * kRec, lk);
        if (kdop_overlap<NDIR>(qk, lk))
          emit(v);
      }
      else
      {
        Box3 b;
        int v;
        SortedLeaf<KIND>::load(sorted, start + j, b, v);
        if (pred.template test_leaf<KIND>(b))
          emit(v);
      }
    }
  };
  // a child that passed its box test; returns true when it is to be
  // descended into
  auto visit = [&](int ref, int cf) -> bool {
    int start = 0, cnt = 0;
    const ChildKind k = child_kind<true>(ref, cf, bucket, start, cnt);
    if (k == kLeaf)
      emit(bucket_start(ref));
    else if (k == kScan)
      scan(start, cnt);
    return k == kDescend;
  };

  int sref[kStackDepth];
  int scf[kStackDepth];
  int sp = 0;
  int node = tree.root;
  const int64_t num_nodes = tree.size > 1 ? tree.size - 1 : 1;
  int64_t budget = num_nodes; // a depth-first walk visits each node at most once
  while (true)
  {
    if (--budget < 0 || (uint64_t)(node - tree.root) >= (uint64_t)num_nodes)
    {
      raise_error(err, ABX_DEVERR_INTERNAL);
      break;
    }
    int lref, rref, lcf, rcf;
    bool hl, hr;
    if constexpr (NDIR > 0)
    {
      // a single leaf's slot holds the leaf's own KDOP: the slot test is the
      // leaf test
      const float4 d = __ldg(reinterpret_cast<const float4 *>(nodes + node) + 3);
      lref = __float_as_int(d.x);
      rref = __float_as_int(d.y);
      lcf = __float_as_int(d.z);
      rcf = __float_as_int(d.w);
      QK a;
      kdop_load<NDIR>(knodes + (int64_t)node * 2 * kRec, a);
      hl = kdop_overlap<NDIR>(qk, a);
      hr = false;
      if (!(is_bucket_ref(rref) && rcf == 0))
      {
        kdop_load<NDIR>(knodes + ((int64_t)node * 2 + 1) * kRec, a);
        hr = kdop_overlap<NDIR>(qk, a);
      }
    }
    else
    {
      const TNode tn = load_tnode(nodes, node);
      Box3 l, r;
      tnode_children(tn, l, r);
      lref = tn.d.x;
      rref = tn.d.y;
      lcf = tn.d.z;
      rcf = tn.d.w;
      const bool rnone = is_bucket_ref(rref) && rcf == 0; // one-leaf tree
      hl = pred.test(l);
      hr = !rnone && pred.test(r);
      if constexpr (decltype(pred)::kRetestLeaf)
      {
        // a single leaf's child box stands for the leaf: take its own test
        hl = hl && (!is_bucket_ref(lref) || pred.template test_leaf<KIND>(l));
        hr = hr && (!is_bucket_ref(rref) || pred.template test_leaf<KIND>(r));
      }
    }
    bool has_next = false;
    int next = 0;
    if (hl && visit(lref, lcf))
    {
      next = lref;
      has_next = true;
    }
    if (hr)
    {
      if (!has_next)
      {
        if (visit(rref, rcf))
        {
          next = rref;
          has_next = true;
        }
      }
      else if (sp < kStackDepth)
      {
        sref[sp] = rref;
        scf[sp] = rcf;
        ++sp;
      }
      else
        raise_error(err, ABX_DEVERR_STACK_OVERFLOW);
    }
    while (!has_next && sp > 0 && !done)
    {
      --sp;
      if (visit(sref[sp], scf[sp]))
      {
        next = sref[sp];
        has_next = true;
      }
    }
    if (!has_next || done)
      break;
    node = next;
  }
  if (MODE != kFill)
    counts[q] = count;
  if (MODE == kBuffered && count > cap)
    atomicOr(overflow, 1u);
}

// ---------------------------------------------------------------------------
// Brute force (ArborX_BruteForce.hpp:40-176, ArborX_BruteForceImpl.hpp:29-229):
// every predicate against every value, values staged through shared memory
// in tiles.  Values are packed like the Morton-ordered leaves, in input
// order ({x, y, z, value} per point, two float4 per box).
// ---------------------------------------------------------------------------

constexpr int kBruteTile = 1024;

template <int KIND>
__device__ __forceinline__ void tile_leaf(const float4 *tile, int j, Box3 &b, int &v)
{
  const float4 u = tile[KIND == 1 ? 2 * j : j];
  b.lo[0] = u.x;
  b.lo[1] = u.y;
  b.lo[2] = u.z;
  if (KIND == 1)
  {
    const float4 w = tile[2 * j + 1];
    b.hi[0] = w.x;
    b.hi[1] = w.y;
    b.hi[2] = w.z;
  }
  else
  {
    b.hi[0] = u.x;
    b.hi[1] = u.y;
    b.hi[2] = u.z;
  }
  v = __float_as_int(u.w);
}

// Load tile [t0, t0 + m) of the packed values into shared memory.
template <int KIND>
__device__ __forceinline__ int load_tile(float4 *tile, const float4 *__restrict__ values, int64_t n,
                                         int64_t t0)
{
  constexpr int f4 = KIND == 1 ? 2 : 1;
  const int m = (int)min((int64_t)kBruteTile, n - t0);
  __syncthreads();
  for (int j = threadIdx.x; j < m * f4; j += blockDim.x)
    tile[j] = __ldg(values + t0 * f4 + j);
  __syncthreads();
  return m;
}

// Spatial: the matches of a predicate come out in ascending value order.
template <int PRED, int MODE, int KIND>
__global__ void __launch_bounds__(kQueryThreads)
    k_brute_spatial(const float4 *__restrict__ values, int64_t n, const float *__restrict__ preds,
                    int64_t nq, const uint32_t *__restrict__ list, int32_t *__restrict__ counts,
                    const int32_t *__restrict__ offsets, int32_t *__restrict__ out,
                    int32_t buffer, unsigned *__restrict__ overflow)
{
  __shared__ float4 tile[kBruteTile * (KIND == 1 ? 2 : 1)];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < nq;
  // the predicate of thread t: list[t] when a query list is given
  const int64_t q = active && list ? (int64_t)__ldg(list + t) : t;
  const auto pred = PredOf<PRED>::load(preds, active ? q : 0);
  int32_t *dst = nullptr;
  if (MODE == kFill && active)
    dst = out + __ldg(offsets + q);
  if (MODE == kBuffered && active)
    dst = out + q * (int64_t)buffer;
  int32_t count = 0;
  for (int64_t t0 = 0; t0 < n; t0 += kBruteTile)
  {
    const int m = load_tile<KIND>(tile, values, n, t0);
    if (!active)
      continue;
    for (int j = 0; j < m; ++j)
    {
      Box3 b;
      int v;
      tile_leaf<KIND>(tile, j, b, v);
      if (pred.template test_leaf<KIND>(b))
      {
        if (MODE == kFill || (MODE == kBuffered && count < buffer))
          dst[count] = v;
        ++count;
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

} // namespace
} // namespace abx
