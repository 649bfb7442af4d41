/*
 * abx_oracle.c -- CPU restatement of the ArborX BoundingVolumeHierarchy hot
 * path (construction, spatial and nearest queries, CRS output).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library in
 * arborx_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product path never calls into it.
 *
 * Every function names the reference file:line it restates (paths are
 * relative to the ArborX source tree, version 2.1.99).  The reference itself
 * cannot be compiled here (it needs Kokkos >= 4.5), so parity is pinned by
 * the known-answer vectors of the reference's own tests (tests/golden/) and
 * by exact brute-force checks.
 *
 * Floating point: compiled with -ffp-contract=off and without fast-math, so
 * every +, -, *, /, sqrt below is one IEEE-754 binary32 operation rounded to
 * nearest, in source order.  That is the "uncontracted source semantics"
 * parity definition used by the CUDA kernels as well.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ABXO_ROPE_SENTINEL (-1)

/* Kokkos::min / Kokkos::max as used by expand (Expand.hpp:43-77). */
static inline float kmin(float a, float b) { return (b < a) ? b : a; }
static inline float kmax(float a, float b) { return (a < b) ? b : a; }

int abxo_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void abxo_set_num_threads(int n)
{
#ifdef _OPENMP
  if (n > 0)
    omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Geometry                                                                  */
/* ------------------------------------------------------------------------ */

/* Empty box = [finite_max, finite_min] (geometry/ArborX_Box.hpp:32-42). */
static inline void box_empty(float b[6])
{
  for (int d = 0; d < 3; ++d)
  {
    b[d] = FLT_MAX;
    b[3 + d] = -FLT_MAX;
  }
}

/* expand(Box, Point) (geometry/algorithms/ArborX_Expand.hpp:43-59). */
static inline void expand_point(float b[6], const float p[3])
{
  for (int d = 0; d < 3; ++d)
  {
    b[d] = kmin(b[d], p[d]);
    b[3 + d] = kmax(b[3 + d], p[d]);
  }
}

/* expand(Box, Box) (geometry/algorithms/ArborX_Expand.hpp:61-77). */
static inline void expand_box(float b[6], const float o[6])
{
  for (int d = 0; d < 3; ++d)
  {
    b[d] = kmin(b[d], o[d]);
    b[3 + d] = kmax(b[3 + d], o[3 + d]);
  }
}

/* distance(Point, Point) (geometry/algorithms/ArborX_Distance.hpp:52-70):
 * squared sum accumulated from 0 in dimension order, tmp = b - a. */
static inline float dist_pp(const float a[3], const float b[3])
{
  float ds = 0.f;
  for (int d = 0; d < 3; ++d)
  {
    float t = b[d] - a[d];
    ds += t * t;
  }
  return sqrtf(ds);
}

/* closestPoint(Point, Box) (geometry/algorithms/ArborX_ClosestPoint.hpp:48-66)
 * followed by distance(Point, Point) (ArborX_Distance.hpp:72-80). */
static inline float dist_pb(const float p[3], const float b[6])
{
  float q[3];
  for (int d = 0; d < 3; ++d)
  {
    if (p[d] < b[d])
      q[d] = b[d];
    else if (p[d] > b[3 + d])
      q[d] = b[3 + d];
    else
      q[d] = p[d];
  }
  return dist_pp(p, q);
}

/* intersects(Box, Box) (geometry/algorithms/ArborX_Intersects.hpp:52-65). */
static inline int isect_bb(const float a[6], const float b[6])
{
  for (int d = 0; d < 3; ++d)
    if (a[d] > b[3 + d] || a[3 + d] < b[d])
      return 0;
  return 1;
}

/* intersects(Point, Box) (ArborX_Intersects.hpp:68-80), reached from
 * intersects(Box, Point) through reverse dispatch
 * (geometry/algorithms/ArborX_ReverseDispatch.hpp:36-45). */
static inline int isect_pb(const float p[3], const float b[6])
{
  for (int d = 0; d < 3; ++d)
    if (p[d] > b[3 + d] || p[d] < b[d])
      return 0;
  return 1;
}

/* centroid: Point -> itself, Box -> (min + max) / 2
 * (geometry/algorithms/ArborX_Centroid.hpp:40-60). */
static inline void centroid_box(const float b[6], float c[3])
{
  for (int d = 0; d < 3; ++d)
    c[d] = (b[d] + b[3 + d]) / 2;
}

/* translateAndScale (geometry/algorithms/ArborX_TranslateAndScale.hpp:25-35) */
static inline void translate_and_scale(const float in[3], float out[3],
                                       const float ref[6])
{
  for (int d = 0; d < 3; ++d)
  {
    float a = ref[d];
    float b = ref[3 + d];
    out[d] = (a != b ? (in[d] - a) / (b - a) : 0.f);
  }
}

/* Kokkos::clamp(v, lo, hi). */
static inline float kclamp(float v, float lo, float hi)
{
  return (v < lo) ? lo : ((hi < v) ? hi : v);
}

/* expandBitsBy<N>: insert N zero bits after each of the low bits of x
 * (spatial/detail/ArborX_MortonCode.hpp:35-197).  Written as a plain bit loop
 * so that it shares nothing with the shift-and-mask form used on the GPU. */
uint64_t abxo_expand_bits64(uint64_t x, int n_zero)
{
  int nbits = 63 / (n_zero + 1);
  if (n_zero == 0)
    return x;
  uint64_t r = 0;
  for (int i = 0; i < nbits; ++i)
    if ((x >> i) & 1ull)
      r |= 1ull << (i * (n_zero + 1));
  return r;
}

uint32_t abxo_expand_bits32(uint32_t x, int n_zero)
{
  /* number of bits kept for N = 1..9, as the reference masks them
   * (ArborX_MortonCode.hpp:42-135): 16, 10, 8, 6, 5, 4, 4, 3, 3 */
  static const int kept[10] = {32, 16, 10, 8, 6, 5, 4, 4, 3, 3};
  if (n_zero == 0)
    return x;
  uint32_t r = 0;
  for (int i = 0; i < kept[n_zero]; ++i)
    if ((x >> i) & 1u)
      r |= 1u << (i * (n_zero + 1));
  return r;
}

/* expandBitsBy<N> for 64-bit values keeps 63/(N+1) bits except for N = 8,
 * which keeps 7 (ArborX_MortonCode.hpp:233-240).  The helper above uses
 * 63/(N+1); N = 8 gives 7 as well. */

/* morton64 (spatial/detail/ArborX_MortonCode.hpp:318-347) for DIM in 1..3:
 * N = 2^(63/DIM); x = clamp(p*N, 0, N-1) in float (NeedDouble is false for
 * DIM >= 3; for DIM = 1, 2 the reference computes in double). */
uint64_t abxo_morton64(const float *p, int dim)
{
  uint64_t N = 1ull << (63 / dim);
  int need_double = N > 16777217ull;
  uint64_t r = 0;
  for (int d = 0; d < dim; ++d)
  {
    uint64_t u;
    if (need_double)
    {
      double x = (double)p[d] * (double)N;
      x = (x < 0.0) ? 0.0 : ((double)(N - 1) < x ? (double)(N - 1) : x);
      u = (uint64_t)x;
    }
    else
    {
      float x = kclamp(p[d] * (float)N, 0.f, (float)(N - 1));
      u = (uint64_t)x;
    }
    r += abxo_expand_bits64(u, dim - 1) << (dim - d - 1);
  }
  return r;
}

/* morton32 (spatial/detail/ArborX_MortonCode.hpp:291-316):
 * N = 2^(32/DIM) (2^31 for DIM = 1), clamp in float. */
uint32_t abxo_morton32(const float *p, int dim)
{
  uint32_t N = 1u << (dim == 1 ? 31 : 32 / dim);
  uint32_t r = 0;
  for (int d = 0; d < dim; ++d)
  {
    float x = kclamp(p[d] * (float)N, 0.f, (float)(N - 1));
    r += abxo_expand_bits32((uint32_t)x, dim - 1) << (dim - d - 1);
  }
  return r;
}

/* ------------------------------------------------------------------------ */
/* Construction                                                              */
/* ------------------------------------------------------------------------ */

/* Leaf geometry: points (3 floats) or boxes (6 floats: min xyz, max xyz). */
static inline void leaf_box(const float *geom, int is_box, int64_t i,
                            float b[6])
{
  if (is_box)
  {
    box_empty(b);
    expand_box(b, geom + 6 * i);
  }
  else
  {
    const float *p = geom + 3 * i;
    box_empty(b);
    expand_point(b, p);
  }
}

/* calculateBoundingBoxOfTheScene
 * (spatial/detail/ArborX_TreeConstruction.hpp:26-39): reduction with
 * expand.  min/max are exact, so the reduction order does not matter. */
void abxo_scene_bounds(const float *geom, int64_t n, int is_box, float out[6])
{
  float b[6];
  box_empty(b);
  for (int64_t i = 0; i < n; ++i)
  {
    if (is_box)
      expand_box(b, geom + 6 * i);
    else
      expand_point(b, geom + 3 * i);
  }
  memcpy(out, b, sizeof(b));
}

/* Morton64 curve applied to the centroid of every value
 * (spatial/detail/ArborX_SpaceFillingCurves.hpp:45-57,64-84). */
void abxo_morton64_codes(const float *geom, int64_t n, int is_box,
                         const float scene[6], uint64_t *codes)
{
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
  {
    float c[3], s[3];
    if (is_box)
      centroid_box(geom + 6 * i, c);
    else
      memcpy(c, geom + 3 * i, sizeof(c));
    translate_and_scale(c, s, scene);
    codes[i] = abxo_morton64(s, 3);
  }
}

/* Morton32 curve of predicate centroids (used for predicate sorting,
 * spatial/detail/ArborX_SpaceFillingCurves.hpp:86-104;
 * spatial/ArborX_LinearBVH.hpp:287-298).  kind: 0 point (3), 1 sphere (4:
 * centre, radius), 2 box (6). */
void abxo_morton32_codes(const float *geom, int64_t n, int kind,
                         const float scene[6], uint32_t *codes)
{
  int stride = kind == 0 ? 3 : (kind == 1 ? 4 : 6);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
  {
    float c[3], s[3];
    const float *g = geom + stride * i;
    if (kind == 2)
      centroid_box(g, c);
    else
      memcpy(c, g, sizeof(c));
    translate_and_scale(c, s, scene);
    codes[i] = abxo_morton32(s, 3);
  }
}

/* sortObjects (misc/ArborX_SortUtils.hpp:28-39): sort keys, return the
 * permutation.  Restated as a STABLE LSD radix sort (8-bit digits): equal
 * keys keep their input order.  The reference's equal-key order is not
 * pinned by its tests (Kokkos::BinSort on host backends, Thrust on CUDA);
 * this build fixes it to "stable". */
void abxo_sort_u64(uint64_t *keys, int64_t n, uint32_t *perm)
{
  uint64_t *k2 = (uint64_t *)malloc(sizeof(uint64_t) * (n > 0 ? n : 1));
  uint32_t *p2 = (uint32_t *)malloc(sizeof(uint32_t) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; ++i)
    perm[i] = (uint32_t)i;
  uint64_t *ka = keys, *kb = k2;
  uint32_t *pa = perm, *pb = p2;
  for (int shift = 0; shift < 64; shift += 8)
  {
    int64_t count[257];
    memset(count, 0, sizeof(count));
    for (int64_t i = 0; i < n; ++i)
      count[((ka[i] >> shift) & 255u) + 1]++;
    for (int b = 0; b < 256; ++b)
      count[b + 1] += count[b];
    for (int64_t i = 0; i < n; ++i)
    {
      int64_t dst = count[(ka[i] >> shift) & 255u]++;
      kb[dst] = ka[i];
      pb[dst] = pa[i];
    }
    uint64_t *tk = ka;
    ka = kb;
    kb = tk;
    uint32_t *tp = pa;
    pa = pb;
    pb = tp;
  }
  /* 8 passes: the data ends in the original buffers */
  free(k2);
  free(p2);
}

void abxo_sort_u32(uint32_t *keys, int64_t n, uint32_t *perm)
{
  uint32_t *k2 = (uint32_t *)malloc(sizeof(uint32_t) * (n > 0 ? n : 1));
  uint32_t *p2 = (uint32_t *)malloc(sizeof(uint32_t) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; ++i)
    perm[i] = (uint32_t)i;
  uint32_t *ka = keys, *kb = k2, *pa = perm, *pb = p2;
  for (int shift = 0; shift < 32; shift += 8)
  {
    int64_t count[257];
    memset(count, 0, sizeof(count));
    for (int64_t i = 0; i < n; ++i)
      count[((ka[i] >> shift) & 255u) + 1]++;
    for (int b = 0; b < 256; ++b)
      count[b + 1] += count[b];
    for (int64_t i = 0; i < n; ++i)
    {
      int64_t dst = count[(ka[i] >> shift) & 255u]++;
      kb[dst] = ka[i];
      pb[dst] = pa[i];
    }
    uint32_t *t = ka;
    ka = kb;
    kb = t;
    t = pa;
    pa = pb;
    pb = t;
  }
  free(k2);
  free(p2);
}

/* Node arrays in the reference layout (spatial/detail/ArborX_Node.hpp:24-51):
 *   leaf     = {int32 rope, int32 value}                      8 bytes
 *   internal = {int32 left_child, int32 rope, float box[6]}  32 bytes
 * Node numbering (spatial/detail/ArborX_HappyTreeFriends.hpp:23-86): leaves
 * are [0, n), internal node i is node n + i, the root is node n and the
 * right child of a node is the rope of its left child. */
typedef struct
{
  int32_t left_child;
  int32_t rope;
  float box[6];
} abxo_internal;

typedef struct
{
  int32_t rope;
  int32_t value;
} abxo_leaf;

/* GenerateHierarchy::delta (spatial/detail/ArborX_TreeConstruction.hpp:131-170)
 * evaluated in unsigned 64-bit arithmetic and reinterpreted as signed, as the
 * reference's expression does. */
static inline int64_t h_delta(const uint64_t *codes, int i, int num_internal)
{
  if (i < 0 || i >= num_internal)
    return INT64_MAX;
  uint64_t x = codes[i] ^ codes[i + 1];
  uint64_t add = (x == 0)
                     ? ((uint64_t)INT64_MIN + (uint64_t)(int64_t)(i ^ (i + 1)))
                     : 0ull;
  return (int64_t)(x + add - 1ull);
}

/* GenerateHierarchy::setRope (ArborX_TreeConstruction.hpp:173-195). */
static inline int32_t h_rope(const uint64_t *codes, int range_right,
                             int64_t delta_right, int num_internal)
{
  if (range_right != num_internal)
    return (delta_right < h_delta(codes, range_right + 1, num_internal))
               ? range_right + 1
               : range_right + 1 + num_internal + 1;
  return ABXO_ROPE_SENTINEL;
}

/* GenerateHierarchy::operator() (ArborX_TreeConstruction.hpp:197-311):
 * Apetrei's bottom-up build with the Karras rule for equal codes.  Leaves are
 * processed by OpenMP threads; the per-node flag uses a compare-and-swap with
 * acquire/release ordering like the reference's atomic_compare_exchange plus
 * load_fence, so every thread order gives the same arrays. */
void abxo_generate_hierarchy(const float *geom, int64_t n64, int is_box,
                             const uint32_t *perm, const uint64_t *codes,
                             abxo_leaf *leaves, abxo_internal *internal)
{
  int n = (int)n64;
  int num_internal = n - 1;
  int root = num_internal + 1; /* internalIndex(0) */
  int32_t *ranges = (int32_t *)malloc(sizeof(int32_t) * (n > 1 ? n - 1 : 1));
  for (int i = 0; i < num_internal; ++i)
    ranges[i] = -1;

#pragma omp parallel for schedule(static)
  for (int leaf = 0; leaf < n; ++leaf)
  {
    int i = leaf;
    int32_t original = (int32_t)perm[i];
    leaves[i].rope = ABXO_ROPE_SENTINEL;
    leaves[i].value = original;
    float bv[6];
    leaf_box(geom, is_box, original, bv);

    int range_left = i, range_right = i;
    int64_t delta_left = h_delta(codes, range_left - 1, num_internal);
    int64_t delta_right = h_delta(codes, range_right, num_internal);
    leaves[i].rope = h_rope(codes, range_right, delta_right, num_internal);
    if (n == 1)
      continue;
    do
    {
      int is_left_child = delta_right < delta_left;
      int left_child;
      if (is_left_child)
      {
        int apetrei_parent = range_right;
        int32_t expected = -1;
        int won = __atomic_compare_exchange_n(&ranges[apetrei_parent],
                                              &expected, range_left, 0,
                                              __ATOMIC_ACQ_REL,
                                              __ATOMIC_ACQUIRE);
        if (won)
          break;
        range_right = expected;
        left_child = i;
        int right_child = apetrei_parent + 1;
        int right_is_leaf = (right_child == range_right);
        delta_right = h_delta(codes, range_right, num_internal);
        float ob[6];
        if (right_is_leaf)
          leaf_box(geom, is_box, leaves[right_child].value, ob);
        else
          memcpy(ob, internal[right_child].box, sizeof(ob));
        expand_box(bv, ob);
      }
      else
      {
        int apetrei_parent = range_left - 1;
        int32_t expected = -1;
        int won = __atomic_compare_exchange_n(&ranges[apetrei_parent],
                                              &expected, range_right, 0,
                                              __ATOMIC_ACQ_REL,
                                              __ATOMIC_ACQUIRE);
        if (won)
          break;
        range_left = expected;
        left_child = apetrei_parent;
        int left_is_leaf = (left_child == range_left);
        delta_left = h_delta(codes, range_left - 1, num_internal);
        float ob[6];
        if (left_is_leaf)
          leaf_box(geom, is_box, leaves[left_child].value, ob);
        else
          memcpy(ob, internal[left_child].box, sizeof(ob));
        expand_box(bv, ob);
        if (!left_is_leaf)
          left_child = left_child + num_internal + 1;
      }
      int karras_parent = delta_right < delta_left ? range_right : range_left;
      abxo_internal *pn = &internal[karras_parent];
      pn->left_child = left_child;
      pn->rope = h_rope(codes, range_right, delta_right, num_internal);
      memcpy(pn->box, bv, sizeof(bv));
      __atomic_thread_fence(__ATOMIC_RELEASE);
      i = karras_parent + num_internal + 1;
    } while (i != root);
  }
  free(ranges);
}

/* BoundingVolumeHierarchy constructor (spatial/ArborX_LinearBVH.hpp:167-256):
 * scene bounds -> Morton64 -> sortObjects -> generateHierarchy.  Empty and
 * one-leaf trees follow :203-213 (initializeSingleLeafTree,
 * ArborX_TreeConstruction.hpp:41-69).  `bounds` receives the tree bounds
 * (root box, or the single leaf's box, or the empty box). */
void abxo_build(const float *geom, int64_t n, int is_box, float bounds[6],
                uint64_t *sorted_codes, uint32_t *perm, abxo_leaf *leaves,
                abxo_internal *internal)
{
  box_empty(bounds);
  if (n == 0)
    return;
  if (n == 1)
  {
    leaves[0].rope = ABXO_ROPE_SENTINEL;
    leaves[0].value = 0;
    leaf_box(geom, is_box, 0, bounds);
    perm[0] = 0;
    return;
  }
  float scene[6];
  abxo_scene_bounds(geom, n, is_box, scene);
  abxo_morton64_codes(geom, n, is_box, scene, sorted_codes);
  abxo_sort_u64(sorted_codes, n, perm);
  abxo_generate_hierarchy(geom, n, is_box, perm, sorted_codes, leaves,
                          internal);
  memcpy(bounds, internal[0].box, sizeof(float) * 6);
}

/* ------------------------------------------------------------------------ */
/* Traversal                                                                 */
/* ------------------------------------------------------------------------ */

typedef struct
{
  int64_t n;
  int is_box;
  const float *geom; /* original order */
  const abxo_leaf *leaves;
  const abxo_internal *internal;
} tree_t;

static inline void node_box(const tree_t *t, int node, float b[6])
{
  if (node < t->n)
    leaf_box(t->geom, t->is_box, t->leaves[node].value, b);
  else
    memcpy(b, t->internal[node - t->n].box, sizeof(float) * 6);
}

static inline int node_rope(const tree_t *t, int node)
{
  return node < t->n ? t->leaves[node].rope : t->internal[node - t->n].rope;
}

/* Spatial predicate test against a node's bounding volume / a leaf's
 * indexable.  kind 1: intersects(Sphere) -- sphere-point
 * (ArborX_Intersects.hpp:106-115) for point leaves, sphere-box (:83-92)
 * otherwise; kind 2: intersects(Box) -- point-box through reverse dispatch
 * for point leaves (:68-80), box-box (:52-65) otherwise. */
static inline int spatial_test(const tree_t *t, int kind, const float *pred,
                               int node)
{
  if (node < t->n && !t->is_box)
  {
    const float *p = t->geom + 3 * (int64_t)t->leaves[node].value;
    if (kind == 1)
      return dist_pp(pred, p) <= pred[3];
    return isect_pb(p, pred);
  }
  float b[6];
  node_box(t, node, b);
  if (kind == 1)
    return dist_pb(pred, b) <= pred[3];
  return isect_bb(pred, b);
}

/* TreeTraversal<Spatial>::operator() (spatial/detail/ArborX_TreeTraversal.hpp:
 * 97-119): stackless rope walk.  Calls emit(value) for every hit in visit
 * order; the one-leaf tree case follows :79-89. */
static int64_t spatial_walk(const tree_t *t, int kind, const float *pred,
                            int32_t *out, int64_t cap)
{
  int64_t count = 0;
  if (t->n == 0)
    return 0;
  if (t->n == 1)
  {
    if (spatial_test(t, kind, pred, 0))
    {
      if (count < cap)
        out[count] = t->leaves[0].value;
      count++;
    }
    return count;
  }
  int node = (int)t->n;
  do
  {
    if (node < t->n)
    {
      if (spatial_test(t, kind, pred, node))
      {
        if (count < cap)
          out[count] = t->leaves[node].value;
        count++;
      }
      node = t->leaves[node].rope;
    }
    else
    {
      node = spatial_test(t, kind, pred, node) ? t->internal[node - t->n].left_child
                                               : t->internal[node - t->n].rope;
    }
  } while (node != ABXO_ROPE_SENTINEL);
  return count;
}

/* Two-pass CRS for spatial predicates (spatial/detail/
 * ArborX_CrsGraphWrapperImpl.hpp:148-323 with buffer size 0): counts, then
 * an exclusive scan into offsets (nq + 1), then a fill pass.  Results of a
 * query are in traversal (rope walk) order. */
int64_t abxo_spatial_count(int64_t n, int is_box, const float *geom,
                           const abxo_leaf *leaves, const abxo_internal *internal,
                           int kind, const float *preds, int64_t nq,
                           int32_t *offsets)
{
  tree_t t = {n, is_box, geom, leaves, internal};
  int stride = kind == 1 ? 4 : 6;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t q = 0; q < nq; ++q)
    offsets[q] = (int32_t)spatial_walk(&t, kind, preds + stride * q, NULL, 0);
  int64_t sum = 0;
  for (int64_t q = 0; q < nq; ++q)
  {
    int64_t c = offsets[q];
    offsets[q] = (int32_t)sum;
    sum += c;
  }
  offsets[nq] = (int32_t)sum;
  return sum;
}

void abxo_spatial_fill(int64_t n, int is_box, const float *geom,
                       const abxo_leaf *leaves, const abxo_internal *internal,
                       int kind, const float *preds, int64_t nq,
                       const int32_t *offsets, int32_t *indices)
{
  tree_t t = {n, is_box, geom, leaves, internal};
  int stride = kind == 1 ? 4 : 6;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t q = 0; q < nq; ++q)
    spatial_walk(&t, kind, preds + stride * q, indices + offsets[q],
                 offsets[q + 1] - offsets[q]);
}

/* ---- binary max-heap on (index, distance) pairs, ordered by distance ----
 * bubbleUp / bubbleDown / popHeap / sortHeap (misc/ArborX_Heap.hpp:40-126)
 * and PriorityQueue::push / popPush (misc/ArborX_PriorityQueue.hpp:63-93)
 * with the comparison lhs.second < rhs.second
 * (ArborX_TreeTraversal.hpp:188-197). */
typedef struct
{
  int32_t idx;
  float dist;
} pair_t;

static inline int cmp_less(pair_t a, pair_t b) { return a.dist < b.dist; }

static void heap_bubble_up(pair_t *h, int64_t pos, int64_t top, pair_t val)
{
  int64_t parent = (pos - 1) / 2;
  while (pos > top && cmp_less(h[parent], val))
  {
    h[pos] = h[parent];
    pos = parent;
    parent = (pos - 1) / 2;
  }
  h[pos] = val;
}

static void heap_bubble_down(pair_t *h, int64_t pos, int64_t len, pair_t val)
{
  int64_t child = 2 * pos + 1;
  if (child + 1 < len && cmp_less(h[child], h[child + 1]))
    ++child;
  while (child < len && cmp_less(val, h[child]))
  {
    h[pos] = h[child];
    pos = child;
    child = 2 * pos + 1;
    if (child + 1 < len && cmp_less(h[child], h[child + 1]))
      ++child;
  }
  h[pos] = val;
}

static void heap_push(pair_t *h, int64_t *size, pair_t v)
{
  h[*size] = v;
  (*size)++;
  if (*size > 1)
    heap_bubble_up(h, *size - 1, 0, h[*size - 1]);
}

static void heap_pop_push(pair_t *h, int64_t size, pair_t v)
{
  heap_bubble_down(h, 0, size, v);
}

static void heap_pop(pair_t *h, int64_t n)
{
  if (n > 1)
  {
    pair_t value = h[0];
    heap_bubble_down(h, 0, n - 1, h[n - 1]);
    h[n - 1] = value;
  }
}

static void heap_sort(pair_t *h, int64_t n)
{
  while (n > 0)
  {
    heap_pop(h, n);
    n--;
  }
}

static inline float nearest_dist(const tree_t *t, const float q[3], int node)
{
  if (node < t->n && !t->is_box)
    return dist_pp(q, t->geom + 3 * (int64_t)t->leaves[node].value);
  float b[6];
  node_box(t, node, b);
  return dist_pb(q, b);
}

/* TreeTraversal<Nearest>::operator() (spatial/detail/ArborX_TreeTraversal.hpp:
 * 180-335), verbatim tie behaviour: candidates enter the bounded max-heap
 * only when strictly closer than the current k-th distance, the closer child
 * is visited first (ties -> left), and the final order is the heap sort's.
 * `buf` has room for k pairs.  Returns the number of results (min(k, n)). */
static int64_t nearest_arborx_walk(const tree_t *t, const float *q, int is_ray, int k,
                                   pair_t *buf, int64_t *visits);

static int64_t nearest_arborx_counted(const tree_t *t, const float q[3], int k,
                                      pair_t *buf, int64_t *visits)
{
  return nearest_arborx_walk(t, q, 0, k, buf, visits);
}

static int64_t nearest_arborx(const tree_t *t, const float q[3], int k,
                              pair_t *buf)
{
  return nearest_arborx_counted(t, q, k, buf, NULL);
}

float abxo_ray_box_distance(const float *ray, const float *box);

/* distance(predicate geometry, node): a point (q[0..2]) or a normalized ray
 * (q[0..5], distance(Ray, Box) of ArborX_Ray.hpp:435-447, point leaves as
 * degenerate boxes). */
static inline float walk_dist(const tree_t *t, const float *q, int is_ray, int node)
{
  if (!is_ray)
    return nearest_dist(t, q, node);
  float b[6];
  node_box(t, node, b);
  return abxo_ray_box_distance(q, b);
}

/* visits (optional): [0] internal nodes read (root + internal children whose
 * distance is computed), [1] leaves read (leaf children whose distance is
 * computed).  These are the node reads of the reference traversal. */
static int64_t nearest_arborx_walk(const tree_t *t, const float *q, int is_ray, int k,
                                   pair_t *buf, int64_t *visits)
{
  if (k < 1 || t->n == 0)
    return 0;
  if (t->n == 1)
  {
    buf[0].idx = 0;
    buf[0].dist = walk_dist(t, q, is_ray, 0);
    return 1;
  }
  int64_t hsize = 0;
  int stack[64];
  float stack_dist[64];
  int sp = 0;
  stack[sp] = -1;
  stack_dist[sp] = 0.f;
  sp++;
  int node = (int)t->n;
  int left_child = 0, right_child = 0;
  float distance_left = 0.f, distance_right = 0.f, distance_node = 0.f;
  float radius = INFINITY;
  if (visits)
    visits[0]++;
  do
  {
    int traverse_left = 0, traverse_right = 0;
    if (distance_node < radius)
    {
      left_child = t->internal[node - t->n].left_child;
      right_child = node_rope(t, left_child);
      if (visits)
      {
        visits[left_child < t->n ? 1 : 0]++;
        visits[right_child < t->n ? 1 : 0]++;
      }
      distance_left = walk_dist(t, q, is_ray, left_child);
      distance_right = walk_dist(t, q, is_ray, right_child);
      if (distance_left < radius)
      {
        if (left_child < t->n)
        {
          pair_t p = {left_child, distance_left};
          if (hsize < k)
            heap_push(buf, &hsize, p);
          else
            heap_pop_push(buf, hsize, p);
          if (hsize == k)
            radius = buf[0].dist;
        }
        else
          traverse_left = 1;
      }
      if (distance_right < radius)
      {
        if (right_child < t->n)
        {
          pair_t p = {right_child, distance_right};
          if (hsize < k)
            heap_push(buf, &hsize, p);
          else
            heap_pop_push(buf, hsize, p);
          if (hsize == k)
            radius = buf[0].dist;
        }
        else
          traverse_right = 1;
      }
    }
    if (!traverse_left && !traverse_right)
    {
      --sp;
      node = stack[sp];
      distance_node = stack_dist[sp];
    }
    else
    {
      node = (traverse_left && (distance_left <= distance_right || !traverse_right))
                 ? left_child
                 : right_child;
      distance_node = (node == left_child ? distance_left : distance_right);
      if (traverse_left && traverse_right)
      {
        if (sp >= 64)
          return -1; /* the reference's int stack[64] would overflow */
        stack[sp] = (node == left_child ? right_child : left_child);
        stack_dist[sp] = (node == left_child ? distance_right : distance_left);
        sp++;
      }
    }
  } while (node != -1);
  heap_sort(buf, hsize);
  for (int64_t i = 0; i < hsize; ++i)
    buf[i].idx = t->leaves[buf[i].idx].value;
  return hsize;
}

/* Tie-rule kNN used by this build: the k smallest (distance, index) pairs,
 * ascending.  Same traversal skeleton; a node is skipped only when its
 * distance is strictly larger than the k-th best distance, a leaf enters
 * when (d, idx) < (d_k, idx_k).  Pure function of the point set (the box
 * distance never exceeds the distance to any point in the box). */
static inline int pair_lt(float da, int32_t ia, float db, int32_t ib)
{
  return da < db || (da == db && ia < ib);
}

static void sorted_insert(pair_t *list, int64_t *size, int k, float d,
                          int32_t idx)
{
  int64_t pos = *size < k ? *size : k - 1;
  if (*size < k)
    (*size)++;
  else if (!pair_lt(d, idx, list[k - 1].dist, list[k - 1].idx))
    return;
  while (pos > 0 && pair_lt(d, idx, list[pos - 1].dist, list[pos - 1].idx))
  {
    list[pos] = list[pos - 1];
    pos--;
  }
  list[pos].dist = d;
  list[pos].idx = idx;
}

static int64_t nearest_ordered(const tree_t *t, const float q[3], int k,
                               pair_t *list, int *stack_nodes,
                               float *stack_d, int64_t stack_cap)
{
  if (k < 1 || t->n == 0)
    return 0;
  int64_t size = 0;
  if (t->n == 1)
  {
    sorted_insert(list, &size, k, nearest_dist(t, q, 0), t->leaves[0].value);
    return size;
  }
  int64_t sp = 0;
  stack_nodes[sp] = (int)t->n;
  stack_d[sp] = 0.f;
  sp++;
  while (sp > 0)
  {
    sp--;
    int node = stack_nodes[sp];
    float dn = stack_d[sp];
    if (size == k && dn > list[k - 1].dist)
      continue;
    if (node < t->n)
    {
      sorted_insert(list, &size, k, dn, t->leaves[node].value);
      continue;
    }
    int l = t->internal[node - t->n].left_child;
    int r = node_rope(t, l);
    float dl = nearest_dist(t, q, l);
    float dr = nearest_dist(t, q, r);
    /* push the farther first so the closer is popped first */
    if (dl <= dr)
    {
      stack_nodes[sp] = r;
      stack_d[sp++] = dr;
      stack_nodes[sp] = l;
      stack_d[sp++] = dl;
    }
    else
    {
      stack_nodes[sp] = l;
      stack_d[sp++] = dl;
      stack_nodes[sp] = r;
      stack_d[sp++] = dr;
    }
    if (sp + 2 > stack_cap)
      return -1;
  }
  return size;
}

/* kNN with CRS output.  mode 0: verbatim ArborX rule; mode 1: (distance,
 * index) rule.  k_per_query may be NULL (then k applies to all).
 * offsets (nq + 1) receive the exclusive scan of min(k_i, n), indices and
 * distances (may be NULL) the results.  Returns the total, or -1 when a
 * query overflowed the 64-entry stack of the verbatim traversal. */
int64_t abxo_nearest(int64_t n, int is_box, const float *geom,
                     const abxo_leaf *leaves, const abxo_internal *internal,
                     const float *queries, int64_t nq, const int32_t *k_per_query,
                     int32_t k, int mode, int32_t *offsets, int32_t *indices,
                     float *distances)
{
  tree_t t = {n, is_box, geom, leaves, internal};
  int64_t sum = 0;
  for (int64_t q = 0; q < nq; ++q)
  {
    int64_t kq = k_per_query ? k_per_query[q] : k;
    if (kq < 0)
      kq = 0;
    offsets[q] = (int32_t)sum;
    sum += kq < n ? kq : n;
  }
  offsets[nq] = (int32_t)sum;
  int failed = 0;
#pragma omp parallel
  {
    int64_t kmax = 0;
    for (int64_t q = 0; q < nq; ++q)
    {
      int64_t kq = k_per_query ? k_per_query[q] : k;
      if (kq > kmax)
        kmax = kq;
    }
    pair_t *buf = (pair_t *)malloc(sizeof(pair_t) * (kmax > 0 ? kmax : 1));
    int64_t cap = 2 * 64 + 2 * (n > 0 ? n : 1);
    int *sn = (int *)malloc(sizeof(int) * cap);
    float *sd = (float *)malloc(sizeof(float) * cap);
#pragma omp for schedule(dynamic, 256)
    for (int64_t q = 0; q < nq; ++q)
    {
      int kq = k_per_query ? k_per_query[q] : k;
      int64_t c = mode == 0 ? nearest_arborx(&t, queries + 3 * q, kq, buf)
                            : nearest_ordered(&t, queries + 3 * q, kq, buf, sn,
                                              sd, cap);
      if (c < 0)
      {
        failed = 1;
        continue;
      }
      for (int64_t j = 0; j < c; ++j)
      {
        indices[offsets[q] + j] = buf[j].idx;
        if (distances)
          distances[offsets[q] + j] = buf[j].dist;
      }
    }
    free(buf);
    free(sn);
    free(sd);
  }
  return failed ? -1 : sum;
}

/* Exact brute force with the (distance, index) rule: every point's
 * distance with the same binary32 formula, k smallest kept.  Independent of
 * any tree; used to check the tree oracles. */
void abxo_knn_brute(const float *geom, int64_t n, int is_box,
                    const float *queries, int64_t nq, int32_t k,
                    int32_t *indices, float *distances)
{
  int64_t kk = k < n ? k : n;
#pragma omp parallel
  {
    pair_t *list = (pair_t *)malloc(sizeof(pair_t) * (k > 0 ? k : 1));
#pragma omp for schedule(dynamic, 64)
    for (int64_t q = 0; q < nq; ++q)
    {
      int64_t size = 0;
      const float *qp = queries + 3 * q;
      for (int64_t j = 0; j < n; ++j)
      {
        float b[6];
        float d;
        if (is_box)
        {
          leaf_box(geom, 1, j, b);
          d = dist_pb(qp, b);
        }
        else
          d = dist_pp(qp, geom + 3 * j);
        sorted_insert(list, &size, k, d, (int32_t)j);
      }
      for (int64_t j = 0; j < kk; ++j)
      {
        indices[q * kk + j] = list[j].idx;
        distances[q * kk + j] = list[j].dist;
      }
    }
    free(list);
  }
}

/* Exact brute-force spatial search: the sorted set of matching indices per
 * query (kind 1 sphere, kind 2 box), two passes like the CRS path. */
int64_t abxo_spatial_brute(const float *geom, int64_t n, int is_box, int kind,
                           const float *preds, int64_t nq, int32_t *offsets,
                           int32_t *indices)
{
  int stride = kind == 1 ? 4 : 6;
  int pass;
  int64_t total = 0;
  for (pass = 0; pass < 2; ++pass)
  {
    if (pass == 1 && indices == NULL)
      break;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t q = 0; q < nq; ++q)
    {
      const float *pr = preds + stride * q;
      int64_t c = 0;
      for (int64_t j = 0; j < n; ++j)
      {
        int hit;
        if (is_box)
        {
          const float *b = geom + 6 * j;
          hit = kind == 1 ? dist_pb(pr, b) <= pr[3] : isect_bb(pr, b);
        }
        else
        {
          const float *p = geom + 3 * j;
          hit = kind == 1 ? dist_pp(pr, p) <= pr[3] : isect_pb(p, pr);
        }
        if (hit)
        {
          if (pass == 1)
            indices[offsets[q] + c] = (int32_t)j;
          c++;
        }
      }
      if (pass == 0)
        offsets[q] = (int32_t)c;
    }
    if (pass == 0)
    {
      int64_t sum = 0;
      for (int64_t q = 0; q < nq; ++q)
      {
        int64_t c = offsets[q];
        offsets[q] = (int32_t)sum;
        sum += c;
      }
      offsets[nq] = (int32_t)sum;
      total = sum;
    }
  }
  return total;
}

/* Exclusive scan (kokkos_ext/ArborX_KokkosExtStdAlgorithms.hpp:24). */
void abxo_exclusive_scan_i32(const int32_t *in, int64_t n, int32_t *out)
{
  int64_t s = 0;
  for (int64_t i = 0; i < n; ++i)
  {
    int32_t v = in[i];
    out[i] = (int32_t)s;
    s += v;
  }
}

/* Node reads of the rope walk: [0] internal nodes tested, [1] leaves tested. */
static void spatial_visits(const tree_t *t, int kind, const float *pred, int64_t *visits)
{
  if (t->n < 2)
  {
    visits[1] += t->n;
    return;
  }
  int node = (int)t->n;
  do
  {
    if (node < t->n)
    {
      visits[1]++;
      node = t->leaves[node].rope;
    }
    else
    {
      visits[0]++;
      node = spatial_test(t, kind, pred, node) ? t->internal[node - t->n].left_child
                                               : t->internal[node - t->n].rope;
    }
  } while (node != ABXO_ROPE_SENTINEL);
}

/* Sum of node reads over a batch of queries, for algorithmic byte counts.
 * mode 0: nearest (queries are points, k), mode 1: spatial (kind, preds). */
void abxo_visit_counts(int64_t n, int is_box, const float *geom,
                       const abxo_leaf *leaves, const abxo_internal *internal,
                       int mode, int kind, const float *preds, int64_t nq,
                       int32_t k, int64_t *out_internal, int64_t *out_leaves)
{
  tree_t t = {n, is_box, geom, leaves, internal};
  int64_t vi = 0, vl = 0;
  int stride = mode == 0 ? 3 : (kind == 1 ? 4 : 6);
#pragma omp parallel reduction(+ : vi, vl)
  {
    pair_t *buf = (pair_t *)malloc(sizeof(pair_t) * (k > 0 ? k : 1));
#pragma omp for schedule(dynamic, 64)
    for (int64_t q = 0; q < nq; ++q)
    {
      int64_t v[2] = {0, 0};
      if (mode == 0)
        nearest_arborx_counted(&t, preds + stride * q, k, buf, v);
      else
        spatial_visits(&t, kind, preds + stride * q, v);
      vi += v[0];
      vl += v[1];
    }
    free(buf);
  }
  *out_internal = vi;
  *out_leaves = vl;
}

/* ------------------------------------------------------------------------ */
/* Rays                                                                      */
/* ------------------------------------------------------------------------ */

/* Ray{origin, direction} (src/geometry/ArborX_Ray.hpp:33-66): the constructor
 * normalizes the direction in double (misc/ArborX_Vector.hpp:40-88): the
 * double norm sqrt(((0 + x*x) + y*y) + z*z) of the float components, each
 * component divided by it in double and rounded to float.  Rows of 6 floats. */
void abxo_ray_normalize(const float *raw, int64_t n, float *out)
{
  for (int64_t i = 0; i < n; ++i)
  {
    const float *r = raw + 6 * i;
    double s = 0;
    for (int d = 0; d < 3; ++d)
      s += (double)r[3 + d] * (double)r[3 + d];
    const double mag = sqrt(s);
    for (int d = 0; d < 3; ++d)
    {
      out[6 * i + d] = r[d];
      out[6 * i + 3 + d] = (float)((double)r[3 + d] / mag);
    }
  }
}

/* intersection(Ray, Box, tmin, tmax) (ArborX_Ray.hpp:107-158): the slab test
 * with a zero direction component handled through the signs, and the
 * comparisons written so that a NaN never updates tmin / tmax. */
int abxo_ray_box_intersection(const float *ray, const float *box, float *tmin_out,
                              float *tmax_out)
{
  const float inf = INFINITY;
  float tmin = -inf, tmax = inf;
  for (int d = 0; d < 3; ++d)
  {
    const float o = ray[d], dir = ray[3 + d], lo = box[d], hi = box[3 + d];
    float tdmin, tdmax;
    if (dir == 0)
    {
      const float min_orig = lo - o;
      if (min_orig == 0)
        continue;
      const float max_orig = hi - o;
      tdmin = signbit(dir * max_orig) ? inf : -inf;
      tdmax = signbit(dir * min_orig) ? inf : -inf;
    }
    else if (dir > 0)
    {
      tdmin = (lo - o) / dir;
      tdmax = (hi - o) / dir;
    }
    else
    {
      tdmin = (hi - o) / dir;
      tdmax = (lo - o) / dir;
    }
    if (tmin < tdmin)
      tmin = tdmin;
    if (tmax > tdmax)
      tmax = tdmax;
  }
  *tmin_out = tmin;
  *tmax_out = tmax;
  return tmin <= tmax;
}

/* intersects(Ray, Box) (ArborX_Ray.hpp:160-168) and distance(Ray, Box)
 * (:435-447): the entry distance max(tmin, 0) of a box in front of the ray,
 * +inf otherwise. */
int abxo_ray_box_intersects(const float *ray, const float *box)
{
  float t0, t1;
  return abxo_ray_box_intersection(ray, box, &t0, &t1) && t1 >= 0;
}

float abxo_ray_box_distance(const float *ray, const float *box)
{
  float t0, t1;
  const int hit = abxo_ray_box_intersection(ray, box, &t0, &t1) && t1 >= 0;
  return hit ? (t0 < 0.f ? 0.f : t0) : INFINITY;
}

/* Brute force over n values (points as degenerate boxes) for nq normalized
 * rays: intersects (ordered = 0: ascending index) or ordered_intersects
 * (ordered = 1: ascending (distance, index)).  Two calls: indices NULL
 * returns the total and fills offsets. */
int64_t abxo_ray_brute(const float *geom, int64_t n, int is_box, const float *rays, int64_t nq,
                       int ordered, int32_t *offsets, int32_t *indices, float *dist)
{
  int64_t total = 0;
  typedef struct
  {
    float d;
    int32_t i;
  } hit_t;
  hit_t *hits = indices ? (hit_t *)malloc(sizeof(hit_t) * (size_t)(n > 0 ? n : 1)) : NULL;
  if (offsets)
    offsets[0] = 0;
  for (int64_t q = 0; q < nq; ++q)
  {
    const float *ray = rays + 6 * q;
    int64_t m = 0;
    for (int64_t j = 0; j < n; ++j)
    {
      float b[6];
      for (int d = 0; d < 3; ++d)
      {
        b[d] = geom[(is_box ? 6 : 3) * j + d];
        b[3 + d] = geom[(is_box ? 6 : 3) * j + (is_box ? 3 : 0) + d];
      }
      if (abxo_ray_box_intersects(ray, b))
      {
        if (hits)
        {
          hits[m].d = abxo_ray_box_distance(ray, b);
          hits[m].i = (int32_t)j;
        }
        ++m;
      }
    }
    if (hits)
    {
      if (ordered) /* insertion sort by (distance, index) */
        for (int64_t a = 1; a < m; ++a)
        {
          hit_t h = hits[a];
          int64_t b = a - 1;
          while (b >= 0 && (hits[b].d > h.d || (hits[b].d == h.d && hits[b].i > h.i)))
          {
            hits[b + 1] = hits[b];
            --b;
          }
          hits[b + 1] = h;
        }
      for (int64_t a = 0; a < m; ++a)
      {
        indices[total + a] = hits[a].i;
        if (dist)
          dist[total + a] = hits[a].d;
      }
    }
    total += m;
    if (offsets)
      offsets[q + 1] = (int32_t)total;
  }
  free(hits);
  return total;
}

/* ---------------------------------------------------------------------------
 * KDOP<3, k> bounding volumes (src/geometry/ArborX_KDOP.hpp:30-183).  A KDOP
 * with ndir = k/2 directions is 2 * ndir floats: min[ndir] then max[ndir].
 * ------------------------------------------------------------------------- */

/* Directions, ArborX_KDOP.hpp:64-151: axes; for k = 18, 26 the edges; for
 * k = 14, 26 the corners. */
static const signed char kdop_axes[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
static const signed char kdop_edges[6][3] = {{1, 1, 0}, {1, 0, 1}, {0, 1, 1},
                                             {1, -1, 0}, {1, 0, -1}, {0, 1, -1}};
static const signed char kdop_corners[4][3] = {{1, 1, 1}, {1, -1, 1}, {1, 1, -1}, {1, -1, -1}};

static const signed char *kdop_direction(int ndir, int i)
{
  if (i < 3)
    return kdop_axes[i];
  if (ndir == 7)
    return kdop_corners[i - 3];
  if (i < 9)
    return kdop_edges[i - 3];
  return kdop_corners[i - 9];
}

/* proj_i = point[0] * dir[0]; proj_i += point[d] * dir[d]
 * (ArborX_Expand.hpp:136-140, ArborX_Intersects.hpp:336-340). */
static float kdop_proj(int ndir, int i, const float *p)
{
  const signed char *d = kdop_direction(ndir, i);
  float proj = p[0] * (float)d[0];
  proj += p[1] * (float)d[1];
  proj += p[2] * (float)d[2];
  return proj;
}

/* KDOP() (ArborX_KDOP.hpp:164-172). */
void abxo_kdop_empty(int ndir, float *k)
{
  for (int i = 0; i < ndir; ++i)
  {
    k[i] = FLT_MAX;
    k[ndir + i] = -FLT_MAX;
  }
}

/* expand(KDOP, Point) (ArborX_Expand.hpp:128-148). */
void abxo_kdop_expand_point(int ndir, float *k, const float *p)
{
  for (int i = 0; i < ndir; ++i)
  {
    const float proj = kdop_proj(ndir, i, p);
    k[i] = kmin(k[i], proj);
    k[ndir + i] = kmax(k[ndir + i], proj);
  }
}

/* expand(KDOP, Box) (ArborX_Expand.hpp:151-208): an inverted range leaves the
 * KDOP unchanged; else the eight corners in the reference's order. */
void abxo_kdop_expand_box(int ndir, float *k, const float *b)
{
  for (int d = 0; d < 3; ++d)
    if (b[d] > b[3 + d])
      return;
  const float xs[2] = {b[0], b[3]}, ys[2] = {b[1], b[4]}, zs[2] = {b[2], b[5]};
  const int order[8][3] = {{0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1},
                           {1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 1, 1}};
  for (int c = 0; c < 8; ++c)
  {
    const float p[3] = {xs[order[c][0]], ys[order[c][1]], zs[order[c][2]]};
    abxo_kdop_expand_point(ndir, k, p);
  }
}

/* intersects(KDOP, KDOP) (ArborX_Intersects.hpp:350-368). */
int abxo_kdop_intersects_kdop(int ndir, const float *kdop, const float *other)
{
  for (int i = 0; i < ndir; ++i)
    if (other[ndir + i] < kdop[i] || other[i] > kdop[ndir + i])
      return 0;
  return 1;
}

/* intersects(KDOP, Box) (ArborX_Intersects.hpp:317-326). */
int abxo_kdop_intersects_box(int ndir, const float *kdop, const float *box)
{
  float other[26];
  abxo_kdop_empty(ndir, other);
  abxo_kdop_expand_box(ndir, other, box);
  return abxo_kdop_intersects_kdop(ndir, kdop, other);
}

/* intersects(Point, KDOP) (ArborX_Intersects.hpp:328-348). */
int abxo_point_intersects_kdop(int ndir, const float *p, const float *kdop)
{
  for (int i = 0; i < ndir; ++i)
  {
    const float proj = kdop_proj(ndir, i, p);
    if (proj < kdop[i] || proj > kdop[ndir + i])
      return 0;
  }
  return 1;
}

/* KDOP{} expanded by each point (is_box 0) or box (is_box 1). */
void abxo_kdop_from_geometry(int ndir, int is_box, const float *g, int64_t n, float *out)
{
  for (int64_t i = 0; i < n; ++i)
  {
    float *k = out + 2 * ndir * i;
    abxo_kdop_empty(ndir, k);
    if (is_box)
      abxo_kdop_expand_box(ndir, k, g + 6 * i);
    else
      abxo_kdop_expand_point(ndir, k, g + 3 * i);
  }
}

/* Box{} expanded by each KDOP (expand(Box, KDOP), ArborX_Expand.hpp:210-225,
 * through expand(Box, Box), :60-77): the ranges of the three axes. */
void abxo_kdop_axis_boxes(int ndir, const float *kd, int64_t n, float *boxes)
{
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d)
    {
      boxes[6 * i + d] = kmin(FLT_MAX, kd[2 * ndir * i + d]);
      boxes[6 * i + 3 + d] = kmax(-FLT_MAX, kd[2 * ndir * i + ndir + d]);
    }
}

/* One value-predicate test.  vkind/pkind: 0 point, 1 box, 2 KDOP (vndir /
 * pndir directions).  intersects is symmetric through reverse dispatch
 * (algorithms/ArborX_ReverseDispatch.hpp). */
static int kdop_leaf_test(int vkind, int vndir, const float *v, int pkind, int pndir,
                          const float *p)
{
  if (pkind == 1 && vkind == 0) /* intersects(Point, Box), Intersects.hpp:67-80 */
  {
    for (int d = 0; d < 3; ++d)
      if (v[d] < p[d] || v[d] > p[3 + d])
        return 0;
    return 1;
  }
  if (pkind == 1 && vkind == 1) /* intersects(Box, Box), Intersects.hpp:51-65 */
  {
    for (int d = 0; d < 3; ++d)
      if (p[d] > v[3 + d] || p[3 + d] < v[d])
        return 0;
    return 1;
  }
  if (pkind == 1 && vkind == 2)
    return abxo_kdop_intersects_box(vndir, v, p);
  if (pkind == 2 && vkind == 0)
    return abxo_point_intersects_kdop(pndir, v, p);
  if (pkind == 2 && vkind == 1)
    return abxo_kdop_intersects_box(pndir, p, v);
  return abxo_kdop_intersects_kdop(pndir, p, v);
}

/* Every predicate against every value, matches in ascending value order
 * (indices may be null: counts only).  Returns the number of matches. */
int64_t abxo_kdop_spatial_brute(const float *values, int64_t n, int vkind, int vndir,
                                const float *preds, int64_t nq, int pkind, int pndir,
                                int32_t *offsets, int32_t *indices)
{
  const int vs = vkind == 0 ? 3 : vkind == 1 ? 6 : 2 * vndir;
  const int ps = pkind == 1 ? 6 : 2 * pndir;
  int64_t total = 0;
  offsets[0] = 0;
  for (int64_t q = 0; q < nq; ++q)
  {
    for (int64_t i = 0; i < n; ++i)
      if (kdop_leaf_test(vkind, vndir, values + vs * i, pkind, pndir, preds + ps * q))
      {
        if (indices)
          indices[total] = (int32_t)i;
        ++total;
      }
    offsets[q + 1] = (int32_t)total;
  }
  return total;
}

/* TreeTraversal<OrderedSpatial>::operator() (spatial/detail/
 * ArborX_TreeTraversal.hpp:406-488) restated step for step: distance(Ray,
 * Box) (ArborX_Ray.hpp:435-447) of both children of an internal node; the
 * closer one (ties -> the right child) is visited next unless the queue's
 * top is strictly closer, in which case the top is popped and the closer
 * child queued; the further child is queued when its distance is finite; a
 * leaf is reported, then the walk continues from the popped top or ends on
 * an empty queue.  The queue is ArborX's PriorityQueue with CompareDistance
 * (lhs.second > rhs.second, the nearest on top), kept here as the max-heap
 * above over negated distances, which makes the same comparisons and so the
 * same tie order.  Point leaves are degenerate boxes.  The one-leaf tree
 * follows :388-401.  Reports (value, distance) in callback order; `heap` has
 * room for 2n entries (the reference's buffer holds 64). */
static int64_t ray_ordered_walk(const tree_t *t, const float *ray, pair_t *heap,
                                int32_t *idx, float *dist, int64_t cap)
{
  int64_t count = 0;
  float b[6];
#define ABXO_REPORT(v, d)                                                      \
  do                                                                           \
  {                                                                            \
    if (count < cap)                                                           \
    {                                                                          \
      idx[count] = (v);                                                        \
      dist[count] = (d);                                                       \
    }                                                                          \
    ++count;                                                                   \
  } while (0)
  if (t->n == 0)
    return 0;
  if (t->n == 1)
  {
    node_box(t, 0, b);
    const float d = abxo_ray_box_distance(ray, b);
    if (d != INFINITY)
      ABXO_REPORT(t->leaves[0].value, d);
    return count;
  }
  int64_t hs = 0;
  int node = (int)t->n;
  while (1)
  {
    if (node < t->n)
    {
      node_box(t, node, b);
      ABXO_REPORT(t->leaves[node].value, abxo_ray_box_distance(ray, b));
      if (hs == 0)
        return count;
      node = heap[0].idx;
      heap_pop(heap, hs);
      --hs;
    }
    else
    {
      const int left = t->internal[node - t->n].left_child;
      const int right = node_rope(t, left);
      node_box(t, left, b);
      const float dl = abxo_ray_box_distance(ray, b);
      node_box(t, right, b);
      const float dr = abxo_ray_box_distance(ray, b);
      const pair_t lp = {left, dl}, rp = {right, dr};
      const pair_t closer = dl < dr ? lp : rp;
      const pair_t further = dl < dr ? rp : lp;
      if (hs > 0 && -heap[0].dist < closer.dist)
      {
        node = heap[0].idx;
        heap_pop(heap, hs);
        --hs;
        if (closer.dist < INFINITY)
          heap_push(heap, &hs, (pair_t){closer.idx, -closer.dist});
      }
      else
        node = closer.idx;
      if (further.dist < INFINITY)
        heap_push(heap, &hs, (pair_t){further.idx, -further.dist});
    }
  }
#undef ABXO_REPORT
}

/* CRS of the restated ordered traversal for nq normalized rays: indices NULL
 * fills offsets (nq + 1) and returns the total; then a second call fills
 * indices and dist (callback order). */
int64_t abxo_ray_ordered_tree(int64_t n, int is_box, const float *geom, const abxo_leaf *leaves,
                              const abxo_internal *internal, const float *rays, int64_t nq,
                              int32_t *offsets, int32_t *indices, float *dist)
{
  tree_t t = {n, is_box, geom, leaves, internal};
  const int64_t hcap = 2 * (n > 0 ? n : 1) + 2;
#pragma omp parallel
  {
    pair_t *heap = (pair_t *)malloc(sizeof(pair_t) * (size_t)hcap);
#pragma omp for schedule(dynamic, 64)
    for (int64_t q = 0; q < nq; ++q)
    {
      if (!indices)
        offsets[q] = (int32_t)ray_ordered_walk(&t, rays + 6 * q, heap, NULL, NULL, 0);
      else
        ray_ordered_walk(&t, rays + 6 * q, heap, indices + offsets[q], dist + offsets[q],
                         offsets[q + 1] - offsets[q]);
    }
    free(heap);
  }
  if (indices)
    return offsets[nq];
  int64_t sum = 0;
  for (int64_t q = 0; q < nq; ++q)
  {
    const int64_t c = offsets[q];
    offsets[q] = (int32_t)sum;
    sum += c;
  }
  offsets[nq] = (int32_t)sum;
  return sum;
}

/* nearest(Ray, k) by the reference's nearest traversal
 * (ArborX_TreeTraversal.hpp:122-336, the verbatim walk above with
 * distance(Ray, Box)): candidates only at a distance below the current k-th
 * (so a missed leaf, at +inf, never enters on a tree of two or more leaves;
 * the one-leaf tree reports its leaf whatever the distance, :158-167), in
 * heap-sort order.  indices NULL fills offsets (nq + 1) and returns the
 * total; a second call fills indices and dist.  Returns -1 if a walk would
 * overflow the reference's 64-entry stack. */
int64_t abxo_ray_nearest_arborx(int64_t n, int is_box, const float *geom,
                                const abxo_leaf *leaves, const abxo_internal *internal,
                                const float *rays, int64_t nq, int k, int32_t *offsets,
                                int32_t *indices, float *dist)
{
  tree_t t = {n, is_box, geom, leaves, internal};
  int failed = 0;
#pragma omp parallel
  {
    pair_t *buf = (pair_t *)malloc(sizeof(pair_t) * (size_t)(k > 0 ? k : 1));
#pragma omp for schedule(dynamic, 64)
    for (int64_t q = 0; q < nq; ++q)
    {
      const int64_t c = nearest_arborx_walk(&t, rays + 6 * q, 1, k, buf, NULL);
      if (c < 0)
      {
#pragma omp atomic write
        failed = 1;
        continue;
      }
      if (!indices)
        offsets[q] = (int32_t)c;
      else
        for (int64_t j = 0; j < c; ++j)
        {
          indices[offsets[q] + j] = buf[j].idx;
          dist[offsets[q] + j] = buf[j].dist;
        }
    }
    free(buf);
  }
  if (failed)
    return -1;
  if (indices)
    return offsets[nq];
  int64_t sum = 0;
  for (int64_t q = 0; q < nq; ++q)
  {
    const int64_t c = offsets[q];
    offsets[q] = (int32_t)sum;
    sum += c;
  }
  offsets[nq] = (int32_t)sum;
  return sum;
}

/* findHalfNeighborList (spatial/detail/ArborX_NeighborList.hpp:47-111) with
 * HalfTraversal (ArborX_HalfTraversal.hpp:23-75) restated: the sphere of
 * leaf i (its point, radius r) walks the ropes from the leaf's own rope, so
 * only the leaves after it in Morton order, and each leaf it intersects
 * lists i's value in its row.  Trees of fewer than two leaves list nothing.
 * Leaves run here by increasing position (the reference runs them in
 * parallel with atomic row cursors, so its order inside a row is free).
 * indices NULL fills offsets (n + 1) and returns the total; a second call
 * fills indices. */
int64_t abxo_half_neighbors(int64_t n, const float *geom, const abxo_leaf *leaves,
                            const abxo_internal *internal, float r, int32_t *offsets,
                            int32_t *indices)
{
  tree_t t = {n, 0, geom, leaves, internal};
  int32_t *cursor = NULL;
  if (!indices)
    for (int64_t q = 0; q <= n; ++q)
      offsets[q] = 0;
  else
  {
    cursor = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t q = 0; q < n; ++q)
      cursor[q] = offsets[q];
  }
  for (int64_t i = 0; n >= 2 && i < n; ++i)
  {
    const int32_t v1 = leaves[i].value;
    const float pred[4] = {geom[3 * (int64_t)v1], geom[3 * (int64_t)v1 + 1],
                           geom[3 * (int64_t)v1 + 2], r};
    int node = leaves[i].rope;
    while (node != ABXO_ROPE_SENTINEL)
    {
      if (node < n)
      {
        if (spatial_test(&t, 1, pred, node))
        {
          const int32_t v2 = leaves[node].value;
          if (!indices)
            offsets[v2]++;
          else
            indices[cursor[v2]++] = v1;
        }
        node = leaves[node].rope;
      }
      else
        node = spatial_test(&t, 1, pred, node) ? internal[node - n].left_child
                                               : internal[node - n].rope;
    }
  }
  if (indices)
  {
    free(cursor);
    return offsets[n];
  }
  int64_t sum = 0;
  for (int64_t q = 0; q < n; ++q)
  {
    const int64_t c = offsets[q];
    offsets[q] = (int32_t)sum;
    sum += c;
  }
  offsets[n] = (int32_t)sum;
  return sum;
}
