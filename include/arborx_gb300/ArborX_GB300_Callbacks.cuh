// ArborX_GB300_Callbacks.cuh -- user callbacks on GB300 trees (nvcc only).
//
// The reference lets users run their own functor on every match, from the
// host (bvh.query(space, predicates, callback, policy),
// src/spatial/ArborX_LinearBVH.hpp:84-88,258-313) and from device code
// (bvh.query(PerThread, predicate, callback), :112-122); a spatial callback
// may stop the traversal by returning CallbackTreeTraversalControl::early_exit
// (src/spatial/detail/ArborX_Callbacks.hpp:24-28, honoured at
// ArborX_TreeTraversal.hpp:105-108).  A callback is a device functor, so this
// path is a header instantiated in the user's translation unit; it walks the
// tree's device view (abx_bvh_device_view) with the same arithmetic as the
// library's own kernels:
//   spatial  depth-first, left subtree first: matches in the rope-walk order;
//            sphere tests compare squared distances with the exact threshold
//            (the largest float whose correctly rounded root is <= r);
//   nearest  the k smallest (distance, value) pairs, reported in ascending
//            order (ties at equal distance: smaller value first).
#ifndef ARBORX_GB300_CALLBACKS_CUH
#define ARBORX_GB300_CALLBACKS_CUH

#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <type_traits>
#include <utility>

#include "ArborX_GB300.hpp"

namespace ArborXGB
{

// ArborX::CallbackTreeTraversalControl (ArborX_Callbacks.hpp:24-28).
enum class CallbackTreeTraversalControl
{
  early_exit,
  normal_continuation
};

namespace Experimental
{
struct PerThread
{
};
} // namespace Experimental

// Device handle of a tree (see abx_device_view in arborx_gb300.h).
struct DeviceTree
{
  const float4 *nodes;
  const float4 *leaves;
  int64_t size;
  int geometry;
};

inline DeviceTree device_tree(BoundingVolumeHierarchy const &bvh)
{
  abx_device_view v;
  Details::check(abx_bvh_device_view(bvh.handle(), &v));
  return DeviceTree{static_cast<const float4 *>(v.nodes), static_cast<const float4 *>(v.leaves),
                    v.size, v.geometry};
}

// Predicates for one query, usable on the device.
template <class Geometry>
struct SpatialPredicate
{
  Geometry geometry;
};

struct NearestPredicate
{
  Point point;
  int k;
};

__host__ __device__ inline SpatialPredicate<Sphere> intersects(Sphere const &s) { return {s}; }
__host__ __device__ inline SpatialPredicate<Box> intersects(Box const &b) { return {b}; }
__host__ __device__ inline NearestPredicate nearest(Point const &p, int k = 1) { return {p, k}; }

namespace Details
{

struct DBox
{
  float lo[3], hi[3];
};

__device__ inline void node_children(const float4 *nodes, int i, DBox &l, DBox &r, int4 &d)
{
  const float4 a = __ldg(nodes + 4 * i), b = __ldg(nodes + 4 * i + 1), c = __ldg(nodes + 4 * i + 2);
  const float4 e = __ldg(nodes + 4 * i + 3);
  l = DBox{{a.x, a.y, a.z}, {a.w, b.x, b.y}};
  r = DBox{{b.z, b.w, c.x}, {c.y, c.z, c.w}};
  d = make_int4(__float_as_int(e.x), __float_as_int(e.y), __float_as_int(e.z), __float_as_int(e.w));
}

// distance(Point, closestPoint(Point, Box)) squared, one rounding per
// operation (geometry/algorithms/ArborX_Distance.hpp:52-80,
// ArborX_ClosestPoint.hpp:48-66).
__device__ inline float dist2_point_box(float px, float py, float pz, DBox const &b)
{
  const float cx = px < b.lo[0] ? b.lo[0] : (px > b.hi[0] ? b.hi[0] : px);
  const float cy = py < b.lo[1] ? b.lo[1] : (py > b.hi[1] ? b.hi[1] : py);
  const float cz = pz < b.lo[2] ? b.lo[2] : (pz > b.hi[2] ? b.hi[2] : pz);
  const float tx = __fsub_rn(cx, px), ty = __fsub_rn(cy, py), tz = __fsub_rn(cz, pz);
  float s = __fmul_rn(tx, tx);
  s = __fadd_rn(s, __fmul_rn(ty, ty));
  return __fadd_rn(s, __fmul_rn(tz, tz));
}

// Largest float s with sqrt_rn(s) <= r (r >= 0; +inf for +inf).
__device__ inline float sq_threshold(float r)
{
  if (!(r < INFINITY))
    return INFINITY;
  float t = __fmul_rn(r, r);
  for (int i = 0; i < 8 && __fsqrt_rn(t) > r; ++i)
    t = __int_as_float(__float_as_int(t) - 1);
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

struct SphereTest
{
  float cx, cy, cz, r2;
  __device__ bool operator()(DBox const &b) const { return dist2_point_box(cx, cy, cz, b) <= r2; }
};

struct BoxTest
{
  DBox q;
  __device__ bool operator()(DBox const &b) const
  {
    return !(q.lo[0] > b.hi[0] || q.hi[0] < b.lo[0] || q.lo[1] > b.hi[1] || q.hi[1] < b.lo[1] ||
             q.lo[2] > b.hi[2] || q.hi[2] < b.lo[2]);
  }
};

__device__ inline SphereTest make_test(Sphere const &s)
{
  return SphereTest{s.centre[0], s.centre[1], s.centre[2],
                    s.r >= 0.f ? sq_threshold(s.r) : -1.f};
}
__device__ inline BoxTest make_test(Box const &b)
{
  return BoxTest{DBox{{b.min_corner[0], b.min_corner[1], b.min_corner[2]},
                      {b.max_corner[0], b.max_corner[1], b.max_corner[2]}}};
}

// Invoke a spatial callback; true when it asks for an early exit
// (invoke_callback_and_check_early_exit, ArborX_Callbacks.hpp:85-108).
template <class Callback>
__device__ inline bool invoke_and_check_exit(Callback &&cb, int value)
{
  if constexpr (std::is_same_v<decltype(cb(value)), CallbackTreeTraversalControl>)
    return cb(value) == CallbackTreeTraversalControl::early_exit;
  else
  {
    cb(value);
    return false;
  }
}

constexpr int kDepth = 96; // bound on the tree depth, see abx_common.cuh

} // namespace Details

// bvh.query(PerThread, intersects(geometry), callback): callback(value) for
// every leaf value whose geometry intersects, in rope-walk order.
template <class Geometry, class Callback>
__device__ void query(Experimental::PerThread, DeviceTree const &tree,
                      SpatialPredicate<Geometry> const &pred, Callback &&callback)
{
  if (tree.size <= 0)
    return;
  const auto test = Details::make_test(pred.geometry);
  int stack[Details::kDepth];
  int sp = 0;
  int node = 0;
  int64_t budget = tree.size > 1 ? tree.size - 1 : 1;
  while (budget-- > 0)
  {
    Details::DBox l, r;
    int4 d;
    Details::node_children(tree.nodes, node, l, r, d);
    const bool rnone = d.y < 0 && d.w == 0;
    const bool hl = test(l);
    const bool hr = !rnone && test(r);
    bool has_next = false;
    int next = 0;
    if (hl)
    {
      if (d.x < 0)
      {
        if (Details::invoke_and_check_exit(callback, ~d.x))
          return;
      }
      else
      {
        next = d.x;
        has_next = true;
      }
    }
    if (hr)
    {
      if (!has_next)
      {
        if (d.y < 0)
        {
          if (Details::invoke_and_check_exit(callback, ~d.y))
            return;
        }
        else
        {
          next = d.y;
          has_next = true;
        }
      }
      else if (sp < Details::kDepth)
        stack[sp++] = d.y;
    }
    while (!has_next && sp > 0)
    {
      const int ref = stack[--sp];
      if (ref < 0)
      {
        if (Details::invoke_and_check_exit(callback, ~ref))
          return;
      }
      else
      {
        next = ref;
        has_next = true;
      }
    }
    if (!has_next)
      return;
    node = next;
  }
}

// bvh.query(PerThread, nearest(point, k), callback): callback(value,
// distance) for the min(k, size) nearest values in ascending (distance,
// value) order; k <= K.
template <int K, class Callback>
__device__ void query(Experimental::PerThread, DeviceTree const &tree,
                      NearestPredicate const &pred, Callback &&callback)
{
  const int k = pred.k < K ? pred.k : K;
  if (tree.size <= 0 || k <= 0)
    return;
  // keys: distance bits << 32 | value + 1; unsigned order = (distance, value)
  unsigned long long key[K];
  for (int j = 0; j < K; ++j)
    key[j] = j < K - k ? 0ull : ~0ull;
  float thr = INFINITY;
  const float qx = pred.point[0], qy = pred.point[1], qz = pred.point[2];
  auto offer = [&](float s, int v) {
    const unsigned long long c =
        ((unsigned long long)__float_as_uint(__fsqrt_rn(s)) << 32) | (unsigned)(v + 1);
    if (c < key[K - 1])
    {
      bool lt[K];
#pragma unroll
      for (int j = 0; j < K; ++j)
        lt[j] = c < key[j];
#pragma unroll
      for (int j = K - 1; j >= 1; --j)
        key[j] = lt[j - 1] ? key[j - 1] : (lt[j] ? c : key[j]);
      key[0] = lt[0] ? c : key[0];
      if (key[K - 1] != ~0ull)
        thr = Details::sq_threshold(__uint_as_float((unsigned)(key[K - 1] >> 32)));
    }
  };
  int sref[Details::kDepth];
  float sdist[Details::kDepth];
  int sp = 0;
  int node = 0;
  int64_t budget = tree.size > 1 ? tree.size - 1 : 1;
  while (budget-- > 0)
  {
    Details::DBox l, r;
    int4 d;
    Details::node_children(tree.nodes, node, l, r, d);
    const bool rnone = d.y < 0 && d.w == 0;
    const float sl = Details::dist2_point_box(qx, qy, qz, l);
    const float sr = rnone ? INFINITY : Details::dist2_point_box(qx, qy, qz, r);
    if (d.x < 0 && sl <= thr)
      offer(sl, ~d.x);
    if (d.y < 0 && !rnone && sr <= thr)
      offer(sr, ~d.y);
    const bool gl = d.x >= 0 && sl <= thr;
    const bool gr = d.y >= 0 && sr <= thr;
    if (gl && gr)
    {
      const bool left_first = sl <= sr;
      node = left_first ? d.x : d.y;
      if (sp < Details::kDepth)
      {
        sref[sp] = left_first ? d.y : d.x;
        sdist[sp] = left_first ? sr : sl;
        ++sp;
      }
      continue;
    }
    if (gl || gr)
    {
      node = gl ? d.x : d.y;
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
  for (int j = K - k; j < K; ++j)
    if (key[j] != ~0ull)
      callback((int)(unsigned)key[j] - 1, __uint_as_float((unsigned)(key[j] >> 32)));
}

namespace Details
{

template <class Geometry, class Callback>
__global__ void callback_spatial_kernel(DeviceTree tree, const Geometry *preds, int64_t nq,
                                        const unsigned *perm, Callback cb)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int q = (int)(perm ? perm[t] : t);
  query(Experimental::PerThread{}, tree, SpatialPredicate<Geometry>{preds[q]},
        [&](int value) { return cb(q, value); });
}

template <int K, class Callback>
__global__ void callback_nearest_kernel(DeviceTree tree, const Point *points, int64_t nq, int k,
                                        const int *ks, const unsigned *perm, Callback cb)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const int q = (int)(perm ? perm[t] : t);
  query<K>(Experimental::PerThread{}, tree, NearestPredicate{points[q], ks ? ks[q] : k},
           [&](int value, float dist) { cb(q, value, dist); });
}

// Morton32 order of the predicates' centroids within the tree bounds, the
// reference's predicate sorting (ArborX_LinearBVH.hpp:287-306).
inline DeviceView<unsigned> predicate_order(BoundingVolumeHierarchy const &bvh, cudaStream_t s,
                                            abx_geometry kind, const float *geometry, int64_t nq)
{
  DeviceView<unsigned> perm;
  if (nq < 2 || bvh.empty())
    return perm;
  Box b = bvh.bounds();
  std::vector<float> scene = {b.min_corner[0], b.min_corner[1], b.min_corner[2],
                              b.max_corner[0], b.max_corner[1], b.max_corner[2]};
  DeviceView<float> d_scene(scene, s);
  DeviceView<unsigned> codes((size_t)nq);
  perm.realloc((size_t)nq);
  check(abx_morton32(s, kind, geometry, nq, d_scene.data(), codes.data()));
  check(abx_sort_u32(s, codes.data(), nq, perm.data()));
  check_cuda(cudaStreamSynchronize(s));
  return perm;
}

} // namespace Details

// bvh.query(space, predicates, callback, policy) for spatial predicates:
// callback(query_index, value) on the device, returning void or
// CallbackTreeTraversalControl.
template <class Geometry, class Callback>
void query(BoundingVolumeHierarchy const &bvh, cudaStream_t space,
           Intersects<Geometry> const &preds, Callback const &callback,
           Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy())
{
  const int64_t nq = (int64_t)preds.geometries.size();
  if (nq == 0 || bvh.empty())
    return;
  constexpr abx_geometry kind = std::is_same_v<Geometry, Sphere> ? ABX_SPHERE : ABX_BOX;
  DeviceView<unsigned> perm;
  if (policy._sort_predicates)
    perm = Details::predicate_order(bvh, space, kind,
                                    reinterpret_cast<const float *>(preds.geometries.data()), nq);
  Details::callback_spatial_kernel<<<(unsigned)((nq + 127) / 128), 128, 0, space>>>(
      device_tree(bvh), preds.geometries.data(), nq, perm.size() ? perm.data() : nullptr,
      callback);
  Details::check_cuda(cudaGetLastError());
  Details::check_cuda(cudaStreamSynchronize(space));
}

// bvh.query(space, nearest predicates, callback, policy):
// callback(query_index, value, distance) on the device, ascending order per
// query; every k <= K.
template <int K = 32, class Callback>
void query(BoundingVolumeHierarchy const &bvh, cudaStream_t space, Nearest const &preds,
           Callback const &callback,
           Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy())
{
  const int64_t nq = (int64_t)preds.points.size();
  if (nq == 0 || bvh.empty())
    return;
  DeviceView<unsigned> perm;
  if (policy._sort_predicates)
    perm = Details::predicate_order(bvh, space, ABX_POINT,
                                    reinterpret_cast<const float *>(preds.points.data()), nq);
  Details::callback_nearest_kernel<K><<<(unsigned)((nq + 127) / 128), 128, 0, space>>>(
      device_tree(bvh), preds.points.data(), nq, preds.k,
      preds.ks.size() ? preds.ks.data() : nullptr, perm.size() ? perm.data() : nullptr, callback);
  Details::check_cuda(cudaGetLastError());
  Details::check_cuda(cudaStreamSynchronize(space));
}

} // namespace ArborXGB

#endif // ARBORX_GB300_CALLBACKS_CUH
