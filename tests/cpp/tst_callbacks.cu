// tst_callbacks.cu -- callback and PerThread queries (include/arborx_gb300/
// ArborX_GB300_Callbacks.cuh) against the library's CRS results, after
// test/tstQueryTreeCallbacks.cpp:96-379 (inline callbacks, early exit with 1..4
// matches) and test/tstQueryTreeCallbackQueryPerThread.cpp:35-115.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include <arborx_gb300/ArborX_GB300_Callbacks.cuh>

using namespace ArborXGB;

static int g_failures = 0, g_checks = 0;
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

struct Count
{
  int *counts;
  __device__ void operator()(int q, int) const { atomicAdd(counts + q, 1); }
};

// records the matches of each query in callback order
struct Record
{
  const int *offsets;
  int *cursor;
  int *out;
  __device__ void operator()(int q, int v) const { out[offsets[q] + atomicAdd(cursor + q, 1)] = v; }
};

// stops after `m` matches (ArborX_Callbacks.hpp:24-28)
struct StopAfter
{
  int *counts;
  int m;
  __device__ CallbackTreeTraversalControl operator()(int q, int) const
  {
    return atomicAdd(counts + q, 1) + 1 >= m ? CallbackTreeTraversalControl::early_exit
                                             : CallbackTreeTraversalControl::normal_continuation;
  }
};

struct RecordNearest
{
  int k;
  int *cursor;
  int *idx;
  float *dist;
  __device__ void operator()(int q, int v, float d) const
  {
    const int j = atomicAdd(cursor + q, 1);
    idx[q * k + j] = v;
    dist[q * k + j] = d;
  }
};

// user kernel calling the device-side single query
__global__ void first_hit(DeviceTree tree, const Sphere *spheres, int nq, int *first)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  int found = -1;
  query(Experimental::PerThread{}, tree, intersects(spheres[q]), [&](int v) {
    found = v;
    return CallbackTreeTraversalControl::early_exit;
  });
  first[q] = found;
}

int main()
{
  std::mt19937 gen(11);
  std::uniform_real_distribution<float> u(0.f, 1.f);
  const int n = 20000, nq = 2000, k = 12;
  std::vector<Point> pts(n), qs(nq);
  for (auto &p : pts)
    p = Point{{u(gen), u(gen), u(gen)}};
  for (auto &p : qs)
    p = Point{{u(gen), u(gen), u(gen)}};
  std::vector<Sphere> sph(nq);
  for (int q = 0; q < nq; ++q)
    sph[q] = Sphere{qs[q], 0.05f};
  BVH tree(nullptr, DeviceView<Point>(pts));
  DeviceView<Sphere> d_sph(sph);

  DeviceView<int> indices, offsets;
  ArborXGB::query(tree, nullptr, intersects(d_sph), indices, offsets);
  auto off = offsets.to_host();
  auto ind = indices.to_host();

  for (bool sort : {true, false})
  {
    auto policy = Experimental::TraversalPolicy().setPredicateSorting(sort);
    DeviceView<int> counts(std::vector<int>(nq, 0));
    query(tree, nullptr, intersects(d_sph), Count{counts.data()}, policy);
    auto c = counts.to_host();
    bool ok = true;
    for (int q = 0; q < nq; ++q)
      ok = ok && c[q] == off[q + 1] - off[q];
    CHECK(ok);

    DeviceView<int> cursor(std::vector<int>(nq, 0));
    DeviceView<int> out(ind.size());
    query(tree, nullptr, intersects(d_sph), Record{offsets.data(), cursor.data(), out.data()},
          policy);
    CHECK(out.to_host() == ind); // same order as the rope walk
  }

  for (int m = 1; m <= 4; ++m)
  {
    DeviceView<int> counts(std::vector<int>(nq, 0));
    query(tree, nullptr, intersects(d_sph), StopAfter{counts.data(), m});
    auto c = counts.to_host();
    bool ok = true;
    for (int q = 0; q < nq; ++q)
      ok = ok && c[q] == std::min(m, off[q + 1] - off[q]);
    CHECK(ok);
  }

  DeviceView<int> first(nq);
  first_hit<<<(nq + 127) / 128, 128>>>(device_tree(tree), d_sph.data(), nq, first.data());
  auto f = first.to_host();
  bool ok_first = true;
  for (int q = 0; q < nq; ++q)
    ok_first = ok_first && f[q] == (off[q + 1] > off[q] ? ind[off[q]] : -1);
  CHECK(ok_first);

  DeviceView<Point> d_qs(qs);
  DeviceView<int> nidx, noff;
  DeviceView<float> ndist;
  tree.query(nullptr, nearest(d_qs, k), nidx, noff, Experimental::TraversalPolicy(), &ndist);
  DeviceView<int> cursor(std::vector<int>(nq, 0));
  DeviceView<int> cidx((size_t)nq * k);
  DeviceView<float> cdist((size_t)nq * k);
  query<16>(tree, nullptr, nearest(d_qs, k),
            RecordNearest{k, cursor.data(), cidx.data(), cdist.data()});
  CHECK(cidx.to_host() == nidx.to_host());
  CHECK(cdist.to_host() == ndist.to_host());

  std::printf("%d checks, %d failures\n", g_checks, g_failures);
  return g_failures == 0 ? 0 : 1;
}
