// ArborX_GB300.hpp -- C++ face of the GB300 BVH, shaped like ArborX's API.
//
// Header-only host code over the C ABI of arborx_gb300.h.  The names, the
// argument meaning and the error behaviour follow the reference:
//   BoundingVolumeHierarchy / BVH      src/spatial/ArborX_LinearBVH.hpp:57-142
//   query(tree, space, preds, indices, offsets[, policy])
//                                      src/spatial/ArborX_CrsGraphWrapper.hpp:22-34
//   intersects / nearest               src/spatial/detail/ArborX_Predicates.hpp:57-142
//   Experimental::make_intersects / make_nearest
//                                      src/spatial/detail/ArborX_PredicateHelpers.hpp:92-206
//   Experimental::TraversalPolicy      src/spatial/detail/ArborX_TraversalPolicy.hpp:19-47
//   SearchException                    src/misc/ArborX_Exception.hpp:19-37
// Device arrays play the role of Kokkos::View<T*, CudaSpace>; the execution
// space instance is a cudaStream_t.  Values stored in the tree are the
// indices of the input rows (the benchmark form BVH<MemorySpace, int, ...>).
#ifndef ARBORX_GB300_HPP
#define ARBORX_GB300_HPP

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../arborx_gb300.h"

namespace ArborXGB
{

// ArborX::SearchException (src/misc/ArborX_Exception.hpp:19-37).
class SearchException : public std::logic_error
{
public:
  explicit SearchException(std::string const &msg) : std::logic_error(msg) {}
};

template <class T>
class DeviceView;

namespace Details
{
inline void check(abx_status s)
{
  if (s == ABX_SUCCESS)
    return;
  std::string msg = std::string(abx_status_string(s)) + ": " + abx_last_error();
  if (s == ABX_ERROR_BUFFER_OVERFLOW || s == ABX_ERROR_INVALID_ARGUMENT)
    throw SearchException(msg);
  throw std::runtime_error(msg);
}
inline void check_cuda(cudaError_t e)
{
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e));
}
} // namespace Details

// Geometries, memory-compatible with the ABI rows (and with ArborX::Point<3>,
// ArborX::Box<3>, ArborX::Sphere<3> of float).
struct Point
{
  float coords[3];
  __host__ __device__ float &operator[](int d) { return coords[d]; }
  __host__ __device__ float operator[](int d) const { return coords[d]; }
};

struct Box
{
  Point min_corner{{3.40282347e38f, 3.40282347e38f, 3.40282347e38f}};
  Point max_corner{{-3.40282347e38f, -3.40282347e38f, -3.40282347e38f}};
  Box() = default; // the empty box, ArborX_Box.hpp:35-42
  __host__ __device__ Box(Point lo, Point hi) : min_corner(lo), max_corner(hi) {}
  __host__ __device__ Point &minCorner() { return min_corner; }
  __host__ __device__ Point const &minCorner() const { return min_corner; }
  __host__ __device__ Point &maxCorner() { return max_corner; }
  __host__ __device__ Point const &maxCorner() const { return max_corner; }
};

struct Sphere
{
  Point centre;
  float r;
  __host__ __device__ Point const &centroid() const { return centre; }
  __host__ __device__ float radius() const { return r; }
};

namespace Experimental
{
// ArborX::Experimental::Ray (src/geometry/ArborX_Ray.hpp:33-66).  The
// direction is stored as given; the library normalizes it (in double, as
// the reference's constructor does) when it runs a query.
struct Ray
{
  Point origin;
  Point direction;
  __host__ __device__ Point const &origin_point() const { return origin; }
};

// ArborX::Experimental::KDOP<3, k> (src/geometry/ArborX_KDOP.hpp:155-183),
// k = 6, 14, 18, 26: the ranges of the k/2 directions, min then max, as in
// the reference's struct and the C ABI rows.  Default: every range empty.
template <int DIM, int k, class Coordinate = float>
struct KDOP
{
  static_assert(DIM == 3 && std::is_same_v<Coordinate, float> &&
                    (k == 6 || k == 14 || k == 18 || k == 26),
                "KDOP<3, 6 | 14 | 18 | 26, float>");
  static constexpr int n_directions = k / 2;
  float _min_values[k / 2];
  float _max_values[k / 2];
  KDOP()
  {
    for (int i = 0; i < n_directions; ++i)
    {
      _min_values[i] = 3.40282347e38f;
      _max_values[i] = -3.40282347e38f;
    }
  }
};
} // namespace Experimental

namespace Details
{
// Direction i of KDOP<3, 2 n> (ArborX_KDOP.hpp:64-151): the axes, then the
// edges (k = 18, 26), then the corners (k = 14, 26).
inline void kdop_direction(int n, int i, float d[3])
{
  static const float edges[6][3] = {{1, 1, 0}, {1, 0, 1}, {0, 1, 1},
                                    {1, -1, 0}, {1, 0, -1}, {0, 1, -1}};
  static const float corners[4][3] = {{1, 1, 1}, {1, -1, 1}, {1, 1, -1}, {1, -1, -1}};
  const float *v = nullptr;
  float axis[3] = {0, 0, 0};
  if (i < 3)
  {
    axis[i] = 1;
    v = axis;
  }
  else if (n == 7)
    v = corners[i - 3];
  else if (i < 9)
    v = edges[i - 3];
  else
    v = corners[i - 9];
  d[0] = v[0];
  d[1] = v[1];
  d[2] = v[2];
}
} // namespace Details

// expand(KDOP, Point) and expand(KDOP, Box) on the host
// (algorithms/ArborX_Expand.hpp:128-208): the same projections (one rounding
// per operation; compile without FMA contraction to match bit for bit) and
// Kokkos::min/max.
template <int k>
void expand(Experimental::KDOP<3, k> &x, Point const &p)
{
  for (int i = 0; i < k / 2; ++i)
  {
    float d[3];
    Details::kdop_direction(k / 2, i, d);
    float proj = p[0] * d[0];
    proj += p[1] * d[1];
    proj += p[2] * d[2];
    x._min_values[i] = proj < x._min_values[i] ? proj : x._min_values[i];
    x._max_values[i] = x._max_values[i] < proj ? proj : x._max_values[i];
  }
}
template <int k>
void expand(Experimental::KDOP<3, k> &x, Box const &b)
{
  for (int d = 0; d < 3; ++d)
    if (b.minCorner()[d] > b.maxCorner()[d])
      return;
  for (int c = 0; c < 8; ++c)
  {
    Point const &px = (c >> 2) & 1 ? b.maxCorner() : b.minCorner();
    Point const &py = c & 1 ? b.maxCorner() : b.minCorner();
    Point const &pz = (c >> 1) & 1 ? b.maxCorner() : b.minCorner();
    expand(x, Point{{px[0], py[1], pz[2]}});
  }
}

// ArborX::PairValueIndex (src/spatial/detail/ArborX_PairValueIndex.hpp:
// 23-44): a value stored with the caller's index; a tree over them indexes
// their geometry and returns the pairs themselves.
template <class Value, class Index = int>
struct PairValueIndex
{
  static_assert(std::is_same_v<Value, Point> || std::is_same_v<Value, Box>,
                "PairValueIndex of points or boxes");
  static_assert(std::is_same_v<Index, int> || std::is_same_v<Index, unsigned>,
                "32-bit indices");
  Value value;
  Index index;
};

template <class T>
struct is_pair_value_index : std::false_type
{
};
template <class V, class I>
struct is_pair_value_index<PairValueIndex<V, I>> : std::true_type
{
};

static_assert(sizeof(Point) == 12 && sizeof(Box) == 24 && sizeof(Sphere) == 16 &&
                  sizeof(Experimental::Ray) == 24,
              "geometry rows must match the C ABI");

// A device array owning its memory: the counterpart of
// Kokkos::View<T*, Kokkos::CudaSpace>.
template <class T>
class DeviceView
{
public:
  DeviceView() = default;
  explicit DeviceView(size_t n) { realloc(n); }
  DeviceView(std::vector<T> const &host, cudaStream_t s = nullptr)
  {
    realloc(host.size());
    if (!host.empty())
    {
      Details::check_cuda(cudaMemcpyAsync(_ptr.get(), host.data(), host.size() * sizeof(T),
                                          cudaMemcpyHostToDevice, s));
      Details::check_cuda(cudaStreamSynchronize(s));
    }
  }
  void realloc(size_t n)
  {
    _size = n;
    T *p = nullptr;
    if (n > 0)
      Details::check_cuda(cudaMalloc(&p, n * sizeof(T)));
    _ptr.reset(p, [](T *q) {
      if (q)
        cudaFree(q);
    });
  }
  T *data() const { return _ptr.get(); }
  size_t size() const { return _size; }
  std::vector<T> to_host(cudaStream_t s = nullptr) const
  {
    std::vector<T> h(_size);
    if (_size)
    {
      Details::check_cuda(
          cudaMemcpyAsync(h.data(), _ptr.get(), _size * sizeof(T), cudaMemcpyDeviceToHost, s));
      Details::check_cuda(cudaStreamSynchronize(s));
    }
    return h;
  }

private:
  std::shared_ptr<T> _ptr;
  size_t _size = 0;
};

namespace Details
{
// Move a CRS result of the library into the caller's arrays (the reference
// reallocates indices and offsets in the callee,
// ArborX_CrsGraphWrapperImpl.hpp:376-377).
inline void take(cudaStream_t space, abx_crs *crs, int64_t nq, DeviceView<int> &indices,
                 DeviceView<int> &offsets, DeviceView<float> *distances)
{
  std::unique_ptr<abx_crs, abx_status (*)(abx_crs *)> guard(crs, abx_crs_destroy);
  const int64_t nres = abx_crs_num_results(crs);
  offsets.realloc((size_t)nq + 1);
  indices.realloc((size_t)nres);
  check_cuda(cudaMemcpyAsync(offsets.data(), abx_crs_offsets(crs), (nq + 1) * sizeof(int),
                             cudaMemcpyDeviceToDevice, space));
  if (nres)
    check_cuda(cudaMemcpyAsync(indices.data(), abx_crs_indices(crs), nres * sizeof(int),
                               cudaMemcpyDeviceToDevice, space));
  if (distances)
  {
    distances->realloc((size_t)nres);
    if (nres)
      check_cuda(cudaMemcpyAsync(distances->data(), abx_crs_distances(crs), nres * sizeof(float),
                                 cudaMemcpyDeviceToDevice, space));
  }
  // the result's arrays are released stream-ordered after the copies
}

template <class Policy>
inline abx_traversal_policy c_policy(Policy const &p)
{
  return abx_traversal_policy{p._buffer_size, p._sort_predicates ? 1 : 0};
}

template <class T>
struct kdop_kind
{
  static constexpr abx_geometry value = ABX_POINT; // not a KDOP
};
template <int k>
struct kdop_kind<Experimental::KDOP<3, k>>
{
  static constexpr abx_geometry value =
      k == 6 ? ABX_KDOP6 : k == 14 ? ABX_KDOP14 : k == 18 ? ABX_KDOP18 : ABX_KDOP26;
};

template <class Geometry>
constexpr abx_geometry predicate_kind()
{
  if constexpr (std::is_same_v<Geometry, Sphere>)
    return ABX_SPHERE;
  else if constexpr (std::is_same_v<Geometry, Box>)
    return ABX_BOX;
  else if constexpr (kdop_kind<Geometry>::value != ABX_POINT)
    return kdop_kind<Geometry>::value;
  else
    return ABX_RAY;
}
} // namespace Details

namespace Experimental
{
// ArborX::Experimental::TraversalPolicy (ArborX_TraversalPolicy.hpp:19-47).
struct TraversalPolicy
{
  int _buffer_size = 0;
  bool _sort_predicates = true;
  TraversalPolicy &setBufferSize(int buffer_size)
  {
    _buffer_size = buffer_size;
    return *this;
  }
  TraversalPolicy &setPredicateSorting(bool sort_predicates)
  {
    _sort_predicates = sort_predicates;
    return *this;
  }
};
} // namespace Experimental

// A batch of intersects(geometry) predicates over a device array.
template <class Geometry>
struct Intersects
{
  static_assert(std::is_same_v<Geometry, Sphere> || std::is_same_v<Geometry, Box> ||
                    std::is_same_v<Geometry, Experimental::Ray> ||
                    Details::kdop_kind<Geometry>::value != ABX_POINT,
                "intersects predicates are spheres, boxes, rays or KDOPs");
  DeviceView<Geometry> geometries;
};

// A batch of nearest(point, k) predicates (one k for all, or one per query).
struct Nearest
{
  DeviceView<Point> points;
  int k = 1;
  DeviceView<int> ks; // empty = use k
};

template <class Geometry>
Intersects<Geometry> intersects(DeviceView<Geometry> const &geometries)
{
  return Intersects<Geometry>{geometries};
}

inline Nearest nearest(DeviceView<Point> const &points, int k = 1) { return Nearest{points, k, {}}; }
inline Nearest nearest(DeviceView<Point> const &points, DeviceView<int> const &ks)
{
  return Nearest{points, 0, ks};
}

namespace Experimental
{
// A batch of ordered_intersects(Ray) predicates (ArborX_Predicates.hpp:
// 103-156): the hits of each ray by increasing distance along it; k > 0
// keeps the first k (nearest(Ray, k)).
struct OrderedIntersects
{
  DeviceView<Ray> rays;
  int k = 0;
};
inline OrderedIntersects make_ordered_intersects(DeviceView<Ray> const &rays, int k = 0)
{
  return OrderedIntersects{rays, k};
}

// make_intersects(points, r) (ArborX_PredicateHelpers.hpp:99-105): spheres of
// radius r around host points.
inline Intersects<Sphere> make_intersects(std::vector<Point> const &points, float r,
                                          cudaStream_t s = nullptr)
{
  std::vector<Sphere> spheres(points.size());
  for (size_t i = 0; i < points.size(); ++i)
    spheres[i] = Sphere{points[i], r};
  return Intersects<Sphere>{DeviceView<Sphere>(spheres, s)};
}
inline Nearest make_nearest(DeviceView<Point> const &points, int k) { return nearest(points, k); }
} // namespace Experimental

class BoundingVolumeHierarchy
{
public:
  using size_type = int64_t;
  using bounding_volume_type = Box;
  using value_type = int;

  BoundingVolumeHierarchy() : BoundingVolumeHierarchy(nullptr, DeviceView<Point>()) {}

  // BoundingVolumeHierarchy(space, values) (ArborX_LinearBVH.hpp:68-73)
  BoundingVolumeHierarchy(cudaStream_t space, DeviceView<Point> const &points)
  {
    create(space, ABX_POINT, reinterpret_cast<const float *>(points.data()),
           (int64_t)points.size());
  }
  BoundingVolumeHierarchy(cudaStream_t space, DeviceView<Box> const &boxes)
  {
    create(space, ABX_BOX, reinterpret_cast<const float *>(boxes.data()), (int64_t)boxes.size());
  }
  // BVH<MemorySpace, PairValueIndex<KDOP>, DefaultIndexableGetter, KDOP>: KDOP
  // values, nodes bounded by KDOPs of the same directions
  // (ArborX_LinearBVH.hpp:56-60; test/CMakeLists.txt:126-151)
  template <int k>
  BoundingVolumeHierarchy(cudaStream_t space, DeviceView<Experimental::KDOP<3, k>> const &kdops)
  {
    create(space, Details::kdop_kind<Experimental::KDOP<3, k>>::value,
           reinterpret_cast<const float *>(kdops.data()), (int64_t)kdops.size());
  }

  // BVH<MemorySpace, PairValueIndex<Point | Box>>: the tree indexes the
  // pairs' geometry (read through their stride, ArborX_AccessTraits.hpp:
  // 36-76) and keeps a copy of the pairs, which value queries return.
  template <class V, class I>
  BoundingVolumeHierarchy(cudaStream_t space, DeviceView<PairValueIndex<V, I>> const &values)
  {
    using P = PairValueIndex<V, I>;
    static_assert(sizeof(P) % 4 == 0, "pairs of 32-bit words");
    const abx_geometry kind = std::is_same_v<V, Point> ? ABX_POINT : ABX_BOX;
    abx_values strided{reinterpret_cast<const float *>(values.data()), (int64_t)(sizeof(P) / 4), 1};
    abx_bvh *t = nullptr;
    Details::check(abx_bvh_create_strided(space, kind, strided, (int64_t)values.size(), &t));
    _tree.reset(t, [](abx_bvh *p) { abx_bvh_destroy(p); });
    _values.realloc(values.size() * sizeof(P) / 4);
    if (values.size())
      Details::check_cuda(cudaMemcpyAsync(_values.data(), values.data(), values.size() * sizeof(P),
                                          cudaMemcpyDeviceToDevice, space));
    _value_bytes = sizeof(P);
  }

  size_type size() const noexcept { return abx_bvh_size(_tree.get()); }
  bool empty() const noexcept { return size() == 0; }
  Box bounds() const
  {
    float b[6];
    Details::check(abx_bvh_bounds(_tree.get(), b));
    return Box(Point{{b[0], b[1], b[2]}}, Point{{b[3], b[4], b[5]}});
  }

  // query(space, predicates, values, offsets[, policy]) on a tree of pairs:
  // the matching pairs themselves in the CRS order of the indices.
  template <class Predicates, class V, class I>
  void query(cudaStream_t space, Predicates const &preds, DeviceView<PairValueIndex<V, I>> &values,
             DeviceView<int> &offsets,
             Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy()) const
  {
    using P = PairValueIndex<V, I>;
    if (_value_bytes != sizeof(P))
      throw SearchException("query: the tree was not built from these PairValueIndex values");
    DeviceView<int> indices;
    query(space, preds, indices, offsets, policy);
    values.realloc(indices.size());
    Details::check(abx_gather_rows(space, _values.data(), size(), (int64_t)sizeof(P),
                                   indices.data(), (int64_t)indices.size(), values.data()));
  }

  // query(space, predicates, indices, offsets[, policy]): the callee
  // reallocates indices and offsets (ArborX_CrsGraphWrapperImpl.hpp:376-377).
  template <class Geometry>
  void query(cudaStream_t space, Intersects<Geometry> const &preds, DeviceView<int> &indices,
             DeviceView<int> &offsets,
             Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy()) const
  {
    abx_crs *crs = nullptr;
    constexpr abx_geometry kind = Details::predicate_kind<Geometry>();
    Details::check(abx_bvh_query_intersects(
        _tree.get(), space, kind, reinterpret_cast<const float *>(preds.geometries.data()),
        (int64_t)preds.geometries.size(), c_policy(policy), &crs));
    Details::take(space, crs, (int64_t)preds.geometries.size(), indices, offsets, nullptr);
  }

  void query(cudaStream_t space, Nearest const &preds, DeviceView<int> &indices,
             DeviceView<int> &offsets,
             Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy(),
             DeviceView<float> *distances = nullptr) const
  {
    abx_crs *crs = nullptr;
    Details::check(abx_bvh_query_nearest(
        _tree.get(), space, reinterpret_cast<const float *>(preds.points.data()),
        (int64_t)preds.points.size(), preds.ks.size() ? preds.ks.data() : nullptr, preds.k,
        c_policy(policy), distances ? 1 : 0, &crs));
    Details::take(space, crs, (int64_t)preds.points.size(), indices, offsets, distances);
  }

  // query(space, ordered_intersects(rays), indices, offsets[, policy])
  void query(cudaStream_t space, Experimental::OrderedIntersects const &preds,
             DeviceView<int> &indices, DeviceView<int> &offsets,
             Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy(),
             DeviceView<float> *distances = nullptr) const
  {
    abx_crs *crs = nullptr;
    Details::check(abx_bvh_query_ordered_intersects(
        _tree.get(), space, reinterpret_cast<const float *>(preds.rays.data()),
        (int64_t)preds.rays.size(), preds.k, c_policy(policy), distances ? 1 : 0, &crs));
    Details::take(space, crs, (int64_t)preds.rays.size(), indices, offsets, distances);
  }

  // nearest(points, k) with the queries and the CRS in host memory (a
  // host-side plugin's call; abx_bvh_query_nearest_host): the copies are
  // pipelined against the traversal.  Returns when the results are on the host.
  void query_host(cudaStream_t space, std::vector<Point> const &queries, int k,
                  std::vector<int> &indices, std::vector<int> &offsets,
                  Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy(),
                  std::vector<float> *distances = nullptr) const
  {
    const int64_t nq = (int64_t)queries.size();
    const int64_t kk = std::min<int64_t>(std::max(k, 0), size());
    offsets.resize((size_t)nq + 1);
    indices.resize((size_t)(nq * kk));
    if (distances)
      distances->resize((size_t)(nq * kk));
    Details::check(abx_bvh_query_nearest_host(
        _tree.get(), space, reinterpret_cast<const float *>(queries.data()), nq, k,
        c_policy(policy), 0, offsets.data(), indices.data(),
        distances ? distances->data() : nullptr));
  }

  abx_bvh const *handle() const { return _tree.get(); }

private:
  void create(cudaStream_t space, abx_geometry kind, const float *values, int64_t n)
  {
    abx_bvh *t = nullptr;
    Details::check(abx_bvh_create(space, kind, values, n, &t));
    _tree.reset(t, [](abx_bvh *p) { abx_bvh_destroy(p); });
  }
  static abx_traversal_policy c_policy(Experimental::TraversalPolicy const &p)
  {
    return Details::c_policy(p);
  }
  std::shared_ptr<abx_bvh> _tree;
  DeviceView<float> _values; // the pairs of a PairValueIndex tree
  size_t _value_bytes = 0;
};

using BVH = BoundingVolumeHierarchy;

// ArborX::BruteForce (src/spatial/ArborX_BruteForce.hpp:40-176): every
// predicate against every value; the same query interface.
class BruteForce
{
public:
  using size_type = int64_t;
  using bounding_volume_type = Box;
  using value_type = int;

  BruteForce(cudaStream_t space, DeviceView<Point> const &points)
  {
    create(space, ABX_POINT, reinterpret_cast<const float *>(points.data()),
           (int64_t)points.size());
  }
  BruteForce(cudaStream_t space, DeviceView<Box> const &boxes)
  {
    create(space, ABX_BOX, reinterpret_cast<const float *>(boxes.data()), (int64_t)boxes.size());
  }
  size_type size() const noexcept { return abx_brute_size(_index.get()); }
  bool empty() const noexcept { return size() == 0; }
  Box bounds() const
  {
    float b[6];
    Details::check(abx_brute_bounds(_index.get(), b));
    return Box(Point{{b[0], b[1], b[2]}}, Point{{b[3], b[4], b[5]}});
  }
  template <class Geometry>
  void query(cudaStream_t space, Intersects<Geometry> const &preds, DeviceView<int> &indices,
             DeviceView<int> &offsets,
             Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy()) const
  {
    abx_crs *crs = nullptr;
    Details::check(abx_brute_query_intersects(
        _index.get(), space, Details::predicate_kind<Geometry>(),
        reinterpret_cast<const float *>(preds.geometries.data()), (int64_t)preds.geometries.size(),
        Details::c_policy(policy), &crs));
    Details::take(space, crs, (int64_t)preds.geometries.size(), indices, offsets, nullptr);
  }
  void query(cudaStream_t space, Nearest const &preds, DeviceView<int> &indices,
             DeviceView<int> &offsets,
             Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy(),
             DeviceView<float> *distances = nullptr) const
  {
    abx_crs *crs = nullptr;
    Details::check(abx_brute_query_nearest(
        _index.get(), space, reinterpret_cast<const float *>(preds.points.data()),
        (int64_t)preds.points.size(), preds.ks.size() ? preds.ks.data() : nullptr, preds.k,
        Details::c_policy(policy), distances ? 1 : 0, &crs));
    Details::take(space, crs, (int64_t)preds.points.size(), indices, offsets, distances);
  }

private:
  void create(cudaStream_t space, abx_geometry kind, const float *values, int64_t n)
  {
    abx_brute *b = nullptr;
    Details::check(abx_brute_create(space, kind, values, n, &b));
    _index.reset(b, [](abx_brute *p) { abx_brute_destroy(p); });
  }
  std::shared_ptr<abx_brute> _index;
};

namespace Experimental
{
// findFullNeighborList / findHalfNeighborList (src/spatial/detail/
// ArborX_NeighborList.hpp:47-188): the radius self-join of the points.
inline void findFullNeighborList(cudaStream_t space, DeviceView<Point> const &points, float radius,
                                 DeviceView<int> &offsets, DeviceView<int> &indices)
{
  abx_crs *crs = nullptr;
  Details::check(abx_find_neighbor_list(space, reinterpret_cast<const float *>(points.data()),
                                        (int64_t)points.size(), radius, 0, &crs));
  Details::take(space, crs, (int64_t)points.size(), indices, offsets, nullptr);
}
inline void findHalfNeighborList(cudaStream_t space, DeviceView<Point> const &points, float radius,
                                 DeviceView<int> &offsets, DeviceView<int> &indices)
{
  abx_crs *crs = nullptr;
  Details::check(abx_find_neighbor_list(space, reinterpret_cast<const float *>(points.data()),
                                        (int64_t)points.size(), radius, 1, &crs));
  Details::take(space, crs, (int64_t)points.size(), indices, offsets, nullptr);
}
} // namespace Experimental

namespace Details
{
// expandHalfToFull (src/spatial/detail/ArborX_ExpandHalfToFull.hpp:23-69):
// offsets and indices replaced by the full list.
inline void expandHalfToFull(cudaStream_t space, DeviceView<int> &offsets, DeviceView<int> &indices)
{
  abx_crs *crs = nullptr;
  const int64_t n = (int64_t)offsets.size() - 1;
  check(abx_expand_half_to_full(space, n, offsets.data(), indices.data(), &crs));
  DeviceView<int> new_offsets, new_indices;
  take(space, crs, n, new_indices, new_offsets, nullptr);
  offsets = new_offsets;
  indices = new_indices;
}
} // namespace Details

// ArborX::query(tree, space, predicates, indices, offsets[, policy])
// (src/spatial/ArborX_CrsGraphWrapper.hpp:22-34).
template <class Predicates>
void query(BoundingVolumeHierarchy const &tree, cudaStream_t space, Predicates const &preds,
           DeviceView<int> &indices, DeviceView<int> &offsets,
           Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy())
{
  tree.query(space, preds, indices, offsets, policy);
}

} // namespace ArborXGB

#endif // ARBORX_GB300_HPP
