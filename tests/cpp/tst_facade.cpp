// tst_facade.cpp -- the reference's query tests, restated against the C++
// face (include/arborx_gb300/ArborX_GB300.hpp) of the GB300 library.
//
// Cases follow test/tstQueryTreeDegenerate.cpp, test/tstQueryTreeTraversalPolicy.cpp,
// test/tstQueryTreeManufacturedSolution.cpp and test/tstQueryTreeComparisonWithBoost.cpp
// (the Boost R-tree replaced by a brute-force loop with the same float formula).
// Results are compared like make_compressed_storage does: offsets exactly, the
// indices of each query as a multiset.  Build with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include <arborx_gb300/ArborX_GB300.hpp>

using namespace ArborXGB;

static int g_failures = 0;
static int g_checks = 0;
#define CHECK(cond)                                                                          \
  do                                                                                         \
  {                                                                                          \
    ++g_checks;                                                                              \
    if (!(cond))                                                                             \
    {                                                                                        \
      ++g_failures;                                                                          \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);                          \
    }                                                                                        \
  } while (0)

using Crs = std::pair<std::vector<int>, std::vector<int>>; // offsets, indices

static bool same_crs(Crs const &got, std::vector<int> const &offsets,
                     std::vector<int> const &indices)
{
  if (got.first != offsets)
    return false;
  for (size_t q = 0; q + 1 < offsets.size(); ++q)
  {
    std::vector<int> a(got.second.begin() + offsets[q], got.second.begin() + offsets[q + 1]);
    std::vector<int> b(indices.begin() + offsets[q], indices.begin() + offsets[q + 1]);
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b)
      return false;
  }
  return true;
}

template <class Preds>
static Crs run(BVH const &tree, Preds const &preds,
               Experimental::TraversalPolicy const &policy = Experimental::TraversalPolicy())
{
  DeviceView<int> indices, offsets;
  query(tree, nullptr, preds, indices, offsets, policy);
  return {offsets.to_host(), indices.to_host()};
}

static Box pbox(float x, float y, float z) { return Box(Point{{x, y, z}}, Point{{x, y, z}}); }

static BVH make_boxes(std::vector<Box> const &boxes) { return BVH(nullptr, DeviceView<Box>(boxes)); }

// test/tstQueryTreeDegenerate.cpp:25-123
static void empty_tree()
{
  BVH tree;
  CHECK(tree.empty() && tree.size() == 0);
  Box b = tree.bounds();
  CHECK(b.minCorner()[0] > 3e38f && b.maxCorner()[0] < -3e38f);
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{}))), {0}, {}));
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{Box(), Box()}))),
                 {0, 0, 0}, {}));
  CHECK(same_crs(run(tree, intersects(DeviceView<Sphere>(std::vector<Sphere>{
                               {{{0, 0, 0}}, 1}, {{{1, 1, 1}}, 2}}))),
                 {0, 0, 0}, {}));
  CHECK(same_crs(run(tree, nearest(DeviceView<Point>(std::vector<Point>{{{0, 0, 0}}, {{1, 1, 1}}}),
                                   2)),
                 {0, 0, 0}, {}));
}

// test/tstQueryTreeDegenerate.cpp:125-223
static void single_leaf_tree()
{
  BVH tree = make_boxes({Box(Point{{0, 0, 0}}, Point{{1, 1, 1}})});
  CHECK(!tree.empty() && tree.size() == 1);
  Box b = tree.bounds();
  CHECK(b.minCorner()[0] == 0 && b.maxCorner()[2] == 1);
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{pbox(5, 5, 5),
                                                                        pbox(.5, .5, .5)}))),
                 {0, 0, 1}, {0}));
  CHECK(same_crs(run(tree, intersects(DeviceView<Sphere>(std::vector<Sphere>{
                               {{{0, 0, 0}}, 1}, {{{1, 1, 1}}, 3}, {{{5, 5, 5}}, 2}}))),
                 {0, 1, 2, 2}, {0, 0}));
  std::vector<Point> q = {{{0, 0, 0}}, {{4, 5, 1}}};
  CHECK(same_crs(run(tree, nearest(DeviceView<Point>(q), DeviceView<int>(std::vector<int>{3, 1}))),
                 {0, 1, 2}, {0, 0}));
}

// test/tstQueryTreeDegenerate.cpp:212-323
static void couple_leaves_tree()
{
  BVH tree = make_boxes({pbox(0, 0, 0), pbox(1, 1, 1)});
  CHECK(tree.size() == 2);
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{Box()}))), {0, 0}, {}));
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{
                               Box(Point{{0, 0, 0}}, Point{{1, 1, 1}})}))),
                 {0, 2}, {1, 0}));
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{
                               Box(Point{{.5, .5, .5}}, Point{{1.5, 1.5, 1.5}})}))),
                 {0, 1}, {1}));
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(std::vector<Box>{Box(), pbox(0, 0, 0)}))),
                 {0, 0, 1}, {0}));
  std::vector<Point> q = {{{0, 0, 0}}, {{1, 0, 0}}};
  CHECK(same_crs(run(tree, nearest(DeviceView<Point>(q), DeviceView<int>(std::vector<int>{2, 4}))),
                 {0, 2, 4}, {0, 1, 0, 1}));
}

// test/tstQueryTreeDegenerate.cpp:325-361
static void duplicated_leaves()
{
  BVH tree = make_boxes({pbox(0, 0, 0), pbox(1, 1, 1), pbox(1, 1, 1), pbox(1, 1, 1)});
  CHECK(same_crs(run(tree, intersects(DeviceView<Sphere>(std::vector<Sphere>{
                               {{{0, 0, 0}}, 1}, {{{1, 1, 1}}, 1}, {{{.5, .5, .5}}, 1}}))),
                 {0, 1, 4, 8}, {0, 1, 2, 3, 0, 1, 2, 3}));
}

// test/tstQueryTreeTraversalPolicy.cpp:32-130
static void buffer_optimization()
{
  BVH tree = make_boxes({pbox(0, 0, 0), pbox(1, 0, 0), pbox(2, 0, 0), pbox(3, 0, 0)});
  auto preds = intersects(DeviceView<Box>(
      std::vector<Box>{Box(), Box(Point{{0, 0, 0}}, Point{{3, 3, 3}}), Box()}));
  std::vector<int> offsets_ref = {0, 0, 4, 4}, indices_ref = {0, 1, 2, 3};
  for (int b : {0, -4, 5, -5, 1})
    CHECK(same_crs(run(tree, preds, Experimental::TraversalPolicy().setBufferSize(b)), offsets_ref,
                   indices_ref));
  bool thrown = false;
  try
  {
    run(tree, preds, Experimental::TraversalPolicy().setBufferSize(-1));
  }
  catch (SearchException const &)
  {
    thrown = true;
  }
  CHECK(thrown);
}

// test/tstQueryTreeTraversalPolicy.cpp:132-202
static void unsorted_predicates()
{
  BVH tree = make_boxes({pbox(0, 0, 0), pbox(1, 1, 1), pbox(2, 2, 2), pbox(3, 3, 3)});
  auto boxes = intersects(DeviceView<Box>(std::vector<Box>{
      Box(Point{{2, 2, 2}}, Point{{3, 3, 3}}), Box(Point{{0, 0, 0}}, Point{{1, 1, 1}})}));
  auto near = nearest(DeviceView<Point>(std::vector<Point>{{{2.5, 2.5, 2.5}}, {{.5, .5, .5}}}), 2);
  for (bool sort : {true, false})
  {
    auto policy = Experimental::TraversalPolicy().setPredicateSorting(sort);
    CHECK(same_crs(run(tree, boxes, policy), {0, 2, 4}, {2, 3, 0, 1}));
    CHECK(same_crs(run(tree, near, policy), {0, 2, 4}, {2, 3, 0, 1}));
  }
}

// test/tstQueryTreeManufacturedSolution.cpp:29-270, parts (i) and (ii)
static void structured_grid()
{
  const int nx = 11;
  const float h = 100.f / (nx - 1);
  auto ind = [&](int i, int j, int k) { return i + j * nx + k * nx * nx; };
  std::vector<Box> leaves(nx * nx * nx), first(nx * nx * nx);
  std::vector<int> off2(nx * nx * nx + 1, 0), ind2;
  for (int k = 0; k < nx; ++k)
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nx; ++i)
      {
        leaves[ind(i, j, k)] = pbox(i * h, j * h, k * h);
        first[ind(i, j, k)] = Box(Point{{(i - 1) * h, (j - 1) * h, (k - 1) * h}},
                                  Point{{(i + 1) * h, (j + 1) * h, (k + 1) * h}});
      }
  for (int q = 0; q < nx * nx * nx; ++q)
  {
    int i = q % nx, j = (q / nx) % nx, k = q / (nx * nx);
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di)
          if (i + di >= 0 && i + di < nx && j + dj >= 0 && j + dj < nx && k + dk >= 0 &&
              k + dk < nx)
            ind2.push_back(ind(i + di, j + dj, k + dk));
    off2[q + 1] = (int)ind2.size();
  }
  BVH tree = make_boxes(leaves);
  std::vector<int> off1(nx * nx * nx + 1), ind1(nx * nx * nx);
  for (size_t q = 0; q < off1.size(); ++q)
    off1[q] = (int)q;
  for (size_t q = 0; q < ind1.size(); ++q)
    ind1[q] = (int)q;
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(leaves))), off1, ind1));
  CHECK(same_crs(run(tree, intersects(DeviceView<Box>(first))), off2, ind2));
}

// test/tstQueryTreeDegenerate.cpp:367-446
static void stack_capacity()
{
  const int n = 4096;
  std::vector<Box> boxes;
  for (int i = 0; i < n; ++i)
    boxes.push_back(Box(Point{{(float)i, (float)i, (float)i}},
                        Point{{(float)i + 1, (float)i + 1, (float)i + 1}}));
  BVH tree = make_boxes(boxes);
  auto all = run(tree, intersects(DeviceView<Box>(std::vector<Box>{
                           Box(), Box(Point{{0, 0, 0}}, Point{{(float)n, (float)n, (float)n}})})));
  CHECK(all.first.back() == n);
  auto knn = run(tree, nearest(DeviceView<Point>(std::vector<Point>{{{0, 0, 0}}}), n));
  CHECK(knn.first.back() == n);
}

// test/tstQueryTreeComparisonWithBoost.cpp:50-231 with a brute-force
// reference: the k smallest float distances, ties by index, in order.
static void knn_against_brute_force()
{
  std::mt19937 gen(7);
  std::uniform_real_distribution<float> u(0.f, 1.f);
  const int n = 3000, nq = 200, k = 10;
  std::vector<Point> pts(n), qs(nq);
  for (auto &p : pts)
    p = Point{{u(gen), u(gen), u(gen)}};
  for (auto &p : qs)
    p = Point{{u(gen), u(gen), u(gen)}};
  BVH tree(nullptr, DeviceView<Point>(pts));
  DeviceView<int> indices, offsets;
  DeviceView<float> dist;
  tree.query(nullptr, nearest(DeviceView<Point>(qs), k), indices, offsets,
             Experimental::TraversalPolicy(), &dist);
  auto got = indices.to_host();
  auto gotd = dist.to_host();
  bool ok = offsets.to_host().back() == nq * k;
  for (int q = 0; q < nq && ok; ++q)
  {
    std::vector<std::pair<float, int>> all;
    for (int j = 0; j < n; ++j)
    {
      float ds = 0.f;
      for (int d = 0; d < 3; ++d)
      {
        float t = pts[j][d] - qs[q][d];
        ds += t * t;
      }
      all.push_back({std::sqrt(ds), j});
    }
    std::partial_sort(all.begin(), all.begin() + k, all.end());
    for (int j = 0; j < k; ++j)
      ok = ok && got[q * k + j] == all[j].second && gotd[q * k + j] == all[j].first;
  }
  CHECK(ok);
}

// BruteForce (src/spatial/ArborX_BruteForce.hpp) answers like the tree:
// nearest exactly, intersects as multisets.
static void brute_force_matches_tree()
{
  std::mt19937 gen(11);
  std::uniform_real_distribution<float> u(0.f, 1.f);
  std::vector<Point> pts(3000), qs(500);
  for (auto &p : pts)
    p = Point{{u(gen), u(gen), u(gen)}};
  for (auto &q : qs)
    q = Point{{u(gen), u(gen), u(gen)}};
  DeviceView<Point> dp(pts), dq(qs);
  BVH tree(nullptr, dp);
  BruteForce brute(nullptr, dp);
  CHECK(brute.size() == 3000);
  DeviceView<int> ti, to, bi, bo;
  tree.query(nullptr, nearest(dq, 7), ti, to);
  brute.query(nullptr, nearest(dq, 7), bi, bo);
  CHECK(ti.to_host() == bi.to_host() && to.to_host() == bo.to_host());
  auto spheres = Experimental::make_intersects(qs, 0.05f);
  tree.query(nullptr, spheres, ti, to);
  brute.query(nullptr, spheres, bi, bo);
  CHECK(same_crs({bo.to_host(), bi.to_host()}, to.to_host(), ti.to_host()));
}

// test/tstNeighborList.cpp:136-171 (rows as multisets).
static void neighbor_lists()
{
  DeviceView<Point> pts(std::vector<Point>{{{0, 0, 0}}, {{1, 1, 1}}, {{2, 2, 2}}, {{3, 3, 3}}});
  DeviceView<int> off, ind;
  Experimental::findFullNeighborList(nullptr, pts, 2.f, off, ind);
  CHECK(same_crs({off.to_host(), ind.to_host()}, {0, 1, 3, 5, 6}, {1, 0, 2, 1, 3, 2}));
  Experimental::findHalfNeighborList(nullptr, pts, 4.f, off, ind);
  Details::expandHalfToFull(nullptr, off, ind);
  CHECK(same_crs({off.to_host(), ind.to_host()}, {0, 2, 5, 8, 10},
                 {1, 2, 0, 2, 3, 0, 1, 3, 1, 2}));
}

// test/tstQueryTreeRay.cpp:62-171: rays through ten boxes on the diagonal.
static void ordered_rays()
{
  std::vector<Box> boxes;
  for (int i = 0; i < 10; ++i)
    boxes.emplace_back(Point{{(float)i, (float)i, (float)i}},
                       Point{{(float)i + 1, (float)i + 1, (float)i + 1}});
  DeviceView<Box> db(boxes);
  BVH tree(nullptr, db);
  using Experimental::Ray;
  DeviceView<Ray> rays(std::vector<Ray>{Ray{{{0, 0, 0}}, {{.1f, .1f, .1f}}},
                                        Ray{{{10, 10, 10}}, {{-.1f, -.1f, -.1f}}}});
  DeviceView<int> ind, off;
  tree.query(nullptr, Experimental::make_ordered_intersects(rays), ind, off);
  std::vector<int> want{0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 9, 8, 7, 6, 5, 4, 3, 2, 1, 0};
  CHECK(ind.to_host() == want);
  CHECK((off.to_host() == std::vector<int>{0, 10, 20}));
  tree.query(nullptr, intersects(rays), ind, off);
  CHECK((off.to_host() == std::vector<int>{0, 10, 20}));
  tree.query(nullptr, Experimental::make_ordered_intersects(rays, 1), ind, off);
  CHECK((ind.to_host() == std::vector<int>{0, 9}));
}

// test/tstQueryTreeIntersectsKDOP.cpp:26-91: a KDOP<3, 18> (a box with an
// edge cut off) over 13 points; then the same points as KDOP<3, 18> values
// in a KDOP-bounded tree.
static void intersects_kdop()
{
  std::vector<Point> prims = {{{0, 0, 0}}, {{1, 1, 1}}, {{2, 2, 2}}, {{3, 3, 3}}, {{1, 0, 0}},
                              {{2, 0, 0}}, {{3, 0, 0}}, {{0, 1, 0}}, {{0, 2, 0}}, {{0, 3, 0}},
                              {{0, 0, 1}}, {{0, 0, 2}}, {{0, 0, 3}}};
  BVH tree(nullptr, DeviceView<Point>(prims));
  using K18 = Experimental::KDOP<3, 18>;
  K18 x;
  for (Point p : std::vector<Point>{{{0.25f, 0, 0}}, {{1, 0, 0}}, {{1, 2, 0}}, {{0, 2, 0}},
                                    {{0, 0.25f, 0}}, {{0.25f, 0, 3}}, {{1, 0, 3}}, {{1, 2, 3}},
                                    {{0, 2, 3}}, {{0, 0.25f, 3}}})
    expand(x, p);
  DeviceView<K18> preds(std::vector<K18>{x});
  DeviceView<int> ind, off;
  tree.query(nullptr, intersects(preds), ind, off);
  CHECK(same_crs({off.to_host(), ind.to_host()}, {0, 4}, {1, 4, 7, 8}));
  tree.query(nullptr, intersects(DeviceView<K18>()), ind, off);
  CHECK((off.to_host() == std::vector<int>{0}));
  std::vector<K18> values(prims.size());
  for (size_t i = 0; i < prims.size(); ++i)
    expand(values[i], prims[i]);
  BVH ktree(nullptr, DeviceView<K18>(values));
  ktree.query(nullptr, intersects(preds), ind, off);
  CHECK(same_crs({off.to_host(), ind.to_host()}, {0, 4}, {1, 4, 7, 8}));
  DeviceView<Box> unit(std::vector<Box>{Box(Point{{0, 0, 0}}, Point{{1, 1, 1}})});
  ktree.query(nullptr, intersects(unit), ind, off);
  CHECK(same_crs({off.to_host(), ind.to_host()}, {0, 5}, {0, 1, 4, 7, 10}));
}

// PairValueIndex values (ArborX_PairValueIndex.hpp:23-44; the test suite's
// trees, test/ArborXTest_LegacyTree.hpp:38-60): queries return the pairs.
static void pair_value_index()
{
  std::vector<PairValueIndex<Point>> pairs;
  for (int i = 0; i < 10; ++i)
    pairs.push_back({Point{{(float)i, (float)i, (float)i}}, 100 + i});
  BVH tree(nullptr, DeviceView<PairValueIndex<Point>>(pairs));
  DeviceView<Box> q(std::vector<Box>{Box(Point{{2.5f, 2.5f, 2.5f}}, Point{{5, 5, 5}}),
                                     Box(Point{{-1, -1, -1}}, Point{{0, 0, 0}})});
  DeviceView<PairValueIndex<Point>> values;
  DeviceView<int> off;
  tree.query(nullptr, intersects(q), values, off);
  CHECK((off.to_host() == std::vector<int>{0, 3, 4}));
  std::vector<int> idx;
  for (auto const &v : values.to_host())
  {
    idx.push_back(v.index);
    CHECK(v.value[0] == (float)(v.index - 100));
  }
  CHECK((idx == std::vector<int>{103, 104, 105, 100}));
  DeviceView<Point> pts(std::vector<Point>{{{7.2f, 7.2f, 7.2f}}});
  tree.query(nullptr, nearest(pts, 2), values, off);
  idx.clear();
  for (auto const &v : values.to_host())
    idx.push_back(v.index);
  CHECK((idx == std::vector<int>{107, 108}));
}

// Host queries and host results: the same CRS as the device query.
static void host_buffers()
{
  std::vector<Point> pts;
  for (int i = 0; i < 500; ++i)
    pts.push_back(Point{{(float)(i % 10), (float)((i / 10) % 10), (float)(i / 100)}});
  BVH tree(nullptr, DeviceView<Point>(pts));
  std::vector<Point> q = {{{0.2f, 0.1f, 0.3f}}, {{4.4f, 5.6f, 2.1f}}, {{9, 9, 4}}};
  std::vector<int> hi, ho;
  std::vector<float> hd;
  tree.query_host(nullptr, q, 4, hi, ho, Experimental::TraversalPolicy(), &hd);
  DeviceView<int> di, doff;
  DeviceView<float> dd;
  tree.query(nullptr, nearest(DeviceView<Point>(q), 4), di, doff, Experimental::TraversalPolicy(),
             &dd);
  CHECK(hi == di.to_host());
  CHECK(ho == doff.to_host());
  CHECK(hd == dd.to_host());
  CHECK((ho == std::vector<int>{0, 4, 8, 12}));
}

int main()
{
  empty_tree();
  single_leaf_tree();
  couple_leaves_tree();
  duplicated_leaves();
  buffer_optimization();
  unsorted_predicates();
  structured_grid();
  stack_capacity();
  knn_against_brute_force();
  brute_force_matches_tree();
  neighbor_lists();
  ordered_rays();
  intersects_kdop();
  pair_value_index();
  host_buffers();
  std::printf("%d checks, %d failures\n", g_checks, g_failures);
  return g_failures == 0 ? 0 : 1;
}
