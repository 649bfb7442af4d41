// abx_capi.cu -- the extern "C" entry points of include/arborx_gb300.h:
// tree construction pipeline, CRS query drivers, result objects, per-device
// state and error reporting.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "abx_build.h"
#include "abx_kdop.cuh"

// ---------------------------------------------------------------------------
// Opaque objects
// ---------------------------------------------------------------------------

struct abx_bvh
{
  int device = 0;
  cudaStream_t stream = nullptr;
  abx_geometry kind = ABX_POINT;
  int64_t n = 0;
  abx::TNode *tnodes = nullptr; // child-pair nodes, one slot per Karras index
  float4 *sorted = nullptr;  // leaf geometry in Morton order (bucket scans)
  float *d_bounds = nullptr; // tree bounds on the device (6 floats per tree)
  float *h_bounds = nullptr; // pinned copy, valid once `ready` completed
  cudaEvent_t ready = nullptr;
  // a batch of trees (abx_forest): tree s owns the sorted positions
  // [h_off[s], h_off[s + 1]); empty for a single tree
  int32_t ntrees = 1;
  std::vector<int64_t> h_off;
  int64_t *d_off = nullptr;
  // a tree over KDOP values (abx_kdop.cu): `kind` is ABX_BOX (the values'
  // axis boxes give the topology and `sorted`), kdop_kind the values' kind,
  // ndir its number of directions, knodes / kleaves the KDOP records
  int ndir = 0;
  abx_geometry kdop_kind = ABX_BOX;
  float4 *knodes = nullptr;
  float4 *kleaves = nullptr;
  // brute force over points: values in Morton order and their codes
  float4 *morton_sorted = nullptr;
  uint64_t *morton_codes = nullptr;
};

struct abx_forest : abx_bvh
{
};

// Brute-force index: the values packed in input order (`sorted`), no nodes.
struct abx_brute : abx_bvh
{
};

struct abx_crs
{
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t nq = 0;
  int64_t nres = 0;
  int32_t *offsets = nullptr;
  int32_t *indices = nullptr;
  float *distances = nullptr;
};

namespace abx
{

namespace
{
thread_local std::string g_last_error;
std::mutex g_state_mutex;
constexpr int kMaxDevices = 64;
DeviceState g_states[kMaxDevices];
} // namespace

bool stream_capturing(cudaStream_t s)
{
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) == cudaSuccess && st == cudaStreamCaptureStatusActive;
}

DeviceState &device_state()
{
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices)
    dev = 0;
  DeviceState &st = g_states[dev];
  if (st.device >= 0)
    return st;
  std::lock_guard<std::mutex> lock(g_state_mutex);
  if (st.device < 0)
  {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned *err = nullptr;
    if (cudaMalloc(&err, sizeof(unsigned)) == cudaSuccess)
      cudaMemset(err, 0, sizeof(unsigned));
    // keep freed stream-ordered memory in the pool between calls
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
    {
      uint64_t threshold = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    st.num_sms = sms > 0 ? sms : 1;
    st.d_error = err;
    init_sort_kernels();
    st.device = dev;
  }
  return st;
}

abx_status fail(abx_status status, std::string const &message)
{
  g_last_error = message;
  return status;
}

abx_status fail_cuda(cudaError_t err, char const *what)
{
  cudaGetLastError(); // clear a sticky launch error
  std::string msg = std::string(what) + ": " + cudaGetErrorName(err) + " (" +
                    cudaGetErrorString(err) + ")";
  return fail(err == cudaErrorMemoryAllocation ? ABX_ERROR_OUT_OF_MEMORY : ABX_ERROR_CUDA, msg);
}

namespace
{
struct StageRecord
{
  std::string stage;
  cudaEvent_t start;
  cudaEvent_t end;
  int kernels;
};
std::mutex g_prof_mutex;
std::vector<StageRecord> g_prof;
std::atomic<bool> g_prof_on{false};
} // namespace

namespace
{
std::mutex g_tuning_mutex;
std::map<std::string, int> g_tuning;
} // namespace

int tuning_value(char const *name, int def)
{
  {
    std::lock_guard<std::mutex> lock(g_tuning_mutex);
    auto it = g_tuning.find(name);
    if (it != g_tuning.end())
      return it->second;
  }
  std::string env = std::string("ABX_TUNE_") + name;
  if (char const *v = std::getenv(env.c_str()))
    return std::atoi(v);
  return def;
}

StageScope::StageScope(cudaStream_t s, char const *stage, int kernels)
    : stream_(s), stage_(stage), kernels_(kernels)
{
  if (g_prof_on.load(std::memory_order_relaxed))
  {
    if (cudaEventCreate(&start_) == cudaSuccess)
      cudaEventRecord(start_, s);
    else
      start_ = nullptr;
  }
}

StageScope::~StageScope()
{
  if (!start_)
    return;
  cudaEvent_t end;
  if (cudaEventCreate(&end) != cudaSuccess)
  {
    cudaEventDestroy(start_);
    return;
  }
  cudaEventRecord(end, stream_);
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  g_prof.push_back(StageRecord{stage_, start_, end, kernels_});
}

cudaError_t dmalloc(void **p, size_t bytes, cudaStream_t s)
{
  return cudaMallocAsync(p, bytes, s);
}

void dfree(void *p, cudaStream_t s)
{
  if (p)
    cudaFreeAsync(p, s);
}

// Top passes of the code sort from the Morton kernel's digit histograms
// (one small read back; plain sort choice for clustered codes).
int top_passes_from_hist(cudaStream_t s, const uint32_t *d_hist, int64_t n)
{
  if (hybrid_top_passes(n, 8) <= 0)
    return 0;
  uint32_t h[8 * 256];
  if (cudaMemcpyAsync(h, d_hist, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return hybrid_top_passes(n, 8);
  return choose_top_passes(h, n, 8);
}

// The child-pair nodes of a tree (the array every query reads most).
void tree_node_memory(const abx_bvh *t, const void **ptr, size_t *bytes)
{
  *ptr = t ? t->tnodes : nullptr;
  *bytes = t && t->tnodes ? (size_t)std::max<int64_t>(t->n - 1, 1) * sizeof(TNode) : 0;
}

} // namespace abx

using namespace abx;

namespace
{

cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Synchronise the stream and report the device error word (cleared).
abx_status sync_and_check(cudaStream_t s)
{
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  DeviceState &ds = device_state();
  unsigned bits = 0;
  ABX_CUDA_TRY(cudaMemcpy(&bits, ds.d_error, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (bits)
  {
    cudaMemset(ds.d_error, 0, sizeof(unsigned));
    return fail(bits & ABX_DEVERR_TIMEOUT ? ABX_ERROR_TIMEOUT : ABX_ERROR_DEVICE,
                "device error word 0x" + std::to_string(bits));
  }
  return ABX_SUCCESS;
}

void destroy_tree(abx_bvh *t)
{
  if (!t)
    return;
  cudaStream_t s = t->stream;
  dfree(t->tnodes, s);
  dfree(t->sorted, s);
  dfree(t->d_bounds, s);
  dfree(t->d_off, s);
  dfree(t->knodes, s);
  dfree(t->kleaves, s);
  dfree(t->morton_sorted, s);
  dfree(t->morton_codes, s);
  if (t->h_bounds)
  {
    if (t->ready)
      cudaEventSynchronize(t->ready);
    cudaFreeHost(t->h_bounds);
  }
  if (t->ready)
    cudaEventDestroy(t->ready);
  delete t;
}

void destroy_crs(abx_crs *c)
{
  if (!c)
    return;
  dfree(c->offsets, c->stream);
  dfree(c->indices, c->stream);
  dfree(c->distances, c->stream);
  delete c;
}

abx_status build_tree(abx_bvh *t, const float *d_values)
{
  cudaStream_t s = t->stream;
  const int64_t n = t->n;
  const float empty[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
  std::memcpy(t->h_bounds, empty, sizeof(empty));
  ABX_CUDA_TRY(dmalloc_n(&t->d_bounds, 6, s));
  if (n == 0)
  {
    ABX_CUDA_TRY(cudaMemcpyAsync(t->d_bounds, empty, sizeof(empty), cudaMemcpyHostToDevice, s));
    // the copy reads a stack array: finish it before returning
    ABX_CUDA_TRY(cudaStreamSynchronize(s));
    return ABX_SUCCESS;
  }
  const int f4 = t->kind == ABX_BOX ? 2 : 1;
  ABX_CUDA_TRY(dmalloc_n(&t->sorted, (size_t)n * f4, s));
  if (n == 1)
  {
    ABX_CUDA_TRY(dmalloc_n(&t->tnodes, 1, s));
    ABX_TRY(single_leaf(s, t->kind, d_values, nullptr, t->tnodes, t->sorted, t->d_bounds));
  }
  else
  {
    ABX_CUDA_TRY(dmalloc_n(&t->tnodes, n - 1, s));
    Scratch<uint64_t> codes;
    Scratch<uint32_t> perm;
    Scratch<uint32_t> hist;
    ABX_CUDA_TRY(codes.alloc(n, s));
    ABX_CUDA_TRY(perm.alloc(n, s));
    ABX_CUDA_TRY(hist.alloc(8 * 256, s));
    ABX_CUDA_TRY(cudaMemsetAsync(hist.ptr, 0, 8 * 256 * sizeof(uint32_t), s));
    // the scene box equals the root box (min/max are exact), so it is
    // computed straight into the tree bounds
    ABX_TRY(scene_bounds(s, t->kind, d_values, n, t->d_bounds));
    ABX_TRY(morton64_codes(s, t->kind, d_values, n, t->d_bounds, codes.ptr, hist.ptr));
    ABX_TRY(radix_sort_u64(s, codes.ptr, perm.ptr, nullptr, n, 8, hist.ptr,
                           top_passes_from_hist(s, hist.ptr, n)));
    ABX_TRY(generate_hierarchy(s, t->kind, d_values, n, perm.ptr, codes.ptr, nullptr, nullptr,
                               t->tnodes, t->sorted));
  }
  ABX_CUDA_TRY(cudaMemcpyAsync(t->h_bounds, t->d_bounds, 6 * sizeof(float),
                               cudaMemcpyDeviceToHost, s));
  return ABX_SUCCESS;
}

// Batched build: every tree of the forest in one pipeline (per-tree scene
// boxes and Morton codes, one sort over all trees regrouped stably by tree,
// one hierarchy pass over all segments).
abx_status build_forest(abx_bvh *t, const float *d_values)
{
  cudaStream_t s = t->stream;
  const int nt = t->ntrees;
  const int64_t total = t->n;
  ABX_CUDA_TRY(dmalloc_n(&t->d_bounds, (size_t)6 * nt, s));
  ABX_CUDA_TRY(dmalloc_n(&t->d_off, (size_t)nt + 1, s));
  ABX_CUDA_TRY(cudaMemcpyAsync(t->d_off, t->h_off.data(), ((size_t)nt + 1) * sizeof(int64_t),
                               cudaMemcpyHostToDevice, s));
  if (total > 0)
  {
    const int f4 = t->kind == ABX_BOX ? 2 : 1;
    ABX_CUDA_TRY(dmalloc_n(&t->tnodes, total, s));
    ABX_CUDA_TRY(dmalloc_n(&t->sorted, (size_t)total * f4, s));
  }
  ABX_TRY(forest_build(s, t->kind, d_values, total, t->d_off, nt, t->d_bounds, t->tnodes,
                       t->sorted));
  ABX_CUDA_TRY(cudaMemcpyAsync(t->h_bounds, t->d_bounds, (size_t)6 * nt * sizeof(float),
                               cudaMemcpyDeviceToHost, s));
  return ABX_SUCCESS;
}

// Query order: Morton32 codes of the predicates in the scene box; in a
// forest the tree index ranks above the code, the code taken in the tree's
// own box.
// Digits of the predicates' Morton32 codes that order the queries.
constexpr int kQueryOrderDigits = 3;

abx_status sort_predicates(cudaStream_t s, const abx_bvh *t, abx_geometry kind,
                           const float *d_preds, int64_t nq, const int64_t *qoff,
                           Scratch<uint32_t> &perm)
{
  ABX_CUDA_TRY(perm.alloc(nq, s));
  if (t->d_off)
    return forest_query_order(s, kind, d_preds, nq, qoff, t->ntrees, t->d_bounds, perm.ptr);
  Scratch<uint32_t> codes;
  Scratch<uint32_t> hist;
  ABX_CUDA_TRY(codes.alloc(nq, s));
  ABX_CUDA_TRY(hist.alloc(4 * 256, s));
  ABX_CUDA_TRY(cudaMemsetAsync(hist.ptr, 0, 4 * 256 * sizeof(uint32_t), s));
  ABX_TRY(morton32_codes(s, kind, d_preds, nq, t->d_bounds, codes.ptr, hist.ptr));
  // the order only schedules the queries: the top three digits of the code
  // give the traversal the same coherence as a full sort (1e7 uniform
  // queries: kNN 17.93 ms either way, ordering 0.39 vs 0.49 ms; two digits
  // cost the traversal 1.3 ms); 0 asks for the full sort
  const int digits = tuning_value("QUERY_ORDER_DIGITS", kQueryOrderDigits);
  if (digits >= 1 && digits <= 3)
    return radix_order_top_u32(s, codes.ptr, perm.ptr, nq, 4, hist.ptr, digits);
  // the hybrid sort reads a count back to the host: not while capturing
  ABX_TRY(radix_sort_u32(s, codes.ptr, perm.ptr, nullptr, nq, 4, hist.ptr,
                         stream_capturing(s) ? 0 : hybrid_top_passes(nq, 4)));
  return ABX_SUCCESS;
}

TreeView view_of(const abx_bvh *t)
{
  TreeView v{t->tnodes, t->n, t->d_bounds, t->sorted, t->kind};
  v.ndir = t->ndir;
  v.knodes = reinterpret_cast<const float *>(t->knodes);
  v.kleaves = reinterpret_cast<const float *>(t->kleaves);
  v.morton_sorted = t->morton_sorted;
  v.morton_codes = t->morton_codes;
  return v;
}

// Check a forest's query offsets (0 first, non-decreasing, one entry per
// tree plus one) and copy them to the device.
abx_status upload_query_offsets(cudaStream_t s, const abx_bvh *t, const int64_t *h_qoff,
                                Scratch<int64_t> &qoff, ForestView &fv)
{
  const int nt = t->ntrees;
  ABX_CUDA_TRY(qoff.alloc((size_t)nt + 1, s));
  ABX_CUDA_TRY(cudaMemcpyAsync(qoff.ptr, h_qoff, ((size_t)nt + 1) * sizeof(int64_t),
                               cudaMemcpyHostToDevice, s));
  // the source is the caller's host array: finish the copy before returning
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  fv = ForestView{t->d_off, qoff.ptr, nt};
  return ABX_SUCCESS;
}

// Spatial query driver of a tree or a forest (h_qoff: the forest's query
// offsets on the host, null for a tree).  Count, scan, fill
// (ArborX_CrsGraphWrapperImpl.hpp:240-313), or one buffered pass with the
// two-pass form as its overflow path (ArborX_CrsGraphWrapperImpl.hpp:117-238).
abx_status query_intersects(const abx_bvh *bvh, cudaStream_t s, abx_geometry kind,
                            const float *d_predicates, int64_t nq, const int64_t *h_qoff,
                            abx_traversal_policy policy, abx_crs **out)
{
  device_state();
  ABX_CUDA_TRY(cudaStreamWaitEvent(s, bvh->ready, 0));

  abx_crs *c = new (std::nothrow) abx_crs;
  if (!c)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_crs");
  cudaGetDevice(&c->device);
  c->stream = s;
  c->nq = nq;
  auto bail = [&](abx_status st) {
    cudaStreamSynchronize(s);
    destroy_crs(c);
    return st;
  };
  if (dmalloc_n(&c->offsets, nq + 1, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS offsets"));
  if (bvh->n == 0 || nq == 0)
  {
    cudaMemsetAsync(c->offsets, 0, (nq + 1) * sizeof(int32_t), s);
    dmalloc_n(&c->indices, 0, s);
    *out = c;
    return ABX_SUCCESS;
  }
  Scratch<int64_t> qoff;
  ForestView fv{nullptr, nullptr, 1};
  if (h_qoff)
  {
    abx_status st = upload_query_offsets(s, bvh, h_qoff, qoff, fv);
    if (st != ABX_SUCCESS)
      return bail(st);
  }
  const ForestView *f = h_qoff ? &fv : nullptr;
  Scratch<uint32_t> perm;
  if (policy.sort_predicates && nq > 1 && bvh->tnodes)
  {
    abx_status st = sort_predicates(s, bvh, kind, d_predicates, nq, qoff.ptr, perm);
    if (st != ABX_SUCCESS)
      return bail(st);
  }
  const TreeView tv = view_of(bvh);
  int64_t buffer = policy.buffer_size < 0 ? -(int64_t)policy.buffer_size
                                          : (int64_t)policy.buffer_size;
  if (buffer == 0 && nq >= kOnePassMinQueries && tuning_value("SPATIAL_ONE_PASS", 1))
  {
    // same CRS result in about one traversal: a buffer sized from a sample
    // of the queries takes the results of the counting pass; only the
    // queries that overflow it are traversed again
    double mean = 0;
    abx_status st = sample_mean_hits(s, tv, f, kind, d_predicates, nq, perm.ptr, c->offsets,
                                     kOnePassSample, &mean);
    if (st != ABX_SUCCESS)
      return bail(st);
    const int64_t b = ((int64_t)std::ceil(2.0 * mean + 8.0) + 7) / 8 * 8;
    if (b <= kOnePassMaxBuffer && b * nq * (int64_t)sizeof(int32_t) <= kOnePassMaxBytes)
      buffer = b;
  }
  int32_t total = 0;
  if (buffer == 0)
  {
    abx_status st = launch_spatial(s, tv, f, kind, d_predicates, nq, perm.ptr, kCount, c->offsets,
                                   nullptr, nullptr, 0, nullptr);
    if (st == ABX_SUCCESS)
      st = exclusive_scan_i32(s, c->offsets, nq, c->offsets);
    if (st != ABX_SUCCESS)
      return bail(st);
    cudaMemcpyAsync(&total, c->offsets + nq, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    st = sync_and_check(s);
    if (st != ABX_SUCCESS)
      return bail(st);
    if (dmalloc_n(&c->indices, (size_t)total, s) != cudaSuccess)
      return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS indices"));
    st = launch_spatial(s, tv, f, kind, d_predicates, nq, perm.ptr, kFill, nullptr, c->offsets,
                        c->indices, 0, nullptr);
    if (st != ABX_SUCCESS)
      return bail(st);
  }
  else
  {
    if (buffer * nq > ((int64_t)1 << 33))
      return bail(fail(ABX_ERROR_INVALID_ARGUMENT, "buffer_size x queries too large"));
    Scratch<int32_t> tmp;
    Scratch<unsigned> flag;
    if (tmp.alloc((size_t)(buffer * nq), s) != cudaSuccess || flag.alloc(1, s) != cudaSuccess)
      return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS buffer"));
    cudaMemsetAsync(flag.ptr, 0, sizeof(unsigned), s);
    abx_status st = launch_spatial(s, tv, f, kind, d_predicates, nq, perm.ptr, kBuffered,
                                   c->offsets, nullptr, tmp.ptr, (int32_t)buffer, flag.ptr);
    if (st == ABX_SUCCESS)
      st = exclusive_scan_i32(s, c->offsets, nq, c->offsets);
    if (st != ABX_SUCCESS)
      return bail(st);
    unsigned overflow = 0;
    cudaMemcpyAsync(&total, c->offsets + nq, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&overflow, flag.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    st = sync_and_check(s);
    if (st != ABX_SUCCESS)
      return bail(st);
    if (overflow && policy.buffer_size < 0)
      return bail(fail(ABX_ERROR_BUFFER_OVERFLOW,
                       "buffer_size " + std::to_string(policy.buffer_size) +
                           " is too small for the results of some query"));
    if (dmalloc_n(&c->indices, (size_t)total, s) != cudaSuccess)
      return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS indices"));
    st = launch_compact(s, tmp.ptr, nq, (int32_t)buffer, c->offsets, c->indices);
    if (st == ABX_SUCCESS && overflow)
    {
      // traverse again only the queries whose results did not fit
      Scratch<uint32_t> list;
      int64_t m = 0;
      if (list.alloc(nq, s) != cudaSuccess)
        return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "overflow list"));
      st = launch_overflow_list(s, c->offsets, nq, (int32_t)buffer, list.ptr, &m);
      if (st == ABX_SUCCESS && m > 0)
        st = launch_spatial(s, tv, f, kind, d_predicates, m, list.ptr, kFill, nullptr, c->offsets,
                            c->indices, 0, nullptr);
    }
    if (st != ABX_SUCCESS)
      return bail(st);
  }
  c->nres = total;
  *out = c;
  return ABX_SUCCESS;
}

// Nearest query driver of a tree or a forest: offsets from the per-query
// counts min(k, size of the query's tree) when k varies or trees differ,
// else the fixed stride min(k, n); one traversal fills the CRS arrays.
abx_status query_nearest(const abx_bvh *bvh, cudaStream_t s, const float *d_queries, int64_t nq,
                         const int64_t *h_qoff, const int32_t *d_k, int32_t k,
                         abx_traversal_policy policy, int32_t with_distances, abx_crs **out)
{
  device_state();
  ABX_CUDA_TRY(cudaStreamWaitEvent(s, bvh->ready, 0));

  abx_crs *c = new (std::nothrow) abx_crs;
  if (!c)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_crs");
  cudaGetDevice(&c->device);
  c->stream = s;
  c->nq = nq;
  auto bail = [&](abx_status st) {
    cudaStreamSynchronize(s);
    destroy_crs(c);
    return st;
  };
  if (dmalloc_n(&c->offsets, nq + 1, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS offsets"));
  const int64_t n = bvh->n;
  if (n == 0 || nq == 0)
  {
    cudaMemsetAsync(c->offsets, 0, (nq + 1) * sizeof(int32_t), s);
    dmalloc_n(&c->indices, 0, s);
    if (with_distances)
      dmalloc_n(&c->distances, 0, s);
    *out = c;
    return ABX_SUCCESS;
  }
  Scratch<int64_t> qoff;
  ForestView fv{nullptr, nullptr, 1};
  if (h_qoff)
  {
    abx_status st = upload_query_offsets(s, bvh, h_qoff, qoff, fv);
    if (st != ABX_SUCCESS)
      return bail(st);
  }
  const ForestView *f = h_qoff ? &fv : nullptr;
  Scratch<uint32_t> perm;
  if (policy.sort_predicates && nq > 1 && (bvh->tnodes || bvh->morton_sorted))
  {
    abx_status st = sort_predicates(s, bvh, ABX_POINT, d_queries, nq, qoff.ptr, perm);
    if (st != ABX_SUCCESS)
      return bail(st);
  }
  const TreeView tv = view_of(bvh);
  int64_t total = 0;
  int32_t max_k = k;
  const bool counted = d_k || f;
  if (!counted)
  {
    if (k < 0)
      k = 0;
    const int64_t kk = std::min<int64_t>(k, n);
    total = kk * nq;
    if (total >= (int64_t)INT32_MAX)
      return bail(fail(ABX_ERROR_INVALID_ARGUMENT, "nearest: more than 2^31-1 results"));
  }
  else
  {
    Scratch<int32_t> kmax;
    if (kmax.alloc(1, s) != cudaSuccess)
      return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "scratch"));
    cudaMemsetAsync(kmax.ptr, 0, sizeof(int32_t), s);
    abx_status st = launch_knn_counts(s, tv, f, d_k, k, nq, c->offsets, kmax.ptr);
    if (st == ABX_SUCCESS)
      st = exclusive_scan_i32(s, c->offsets, nq, c->offsets);
    if (st != ABX_SUCCESS)
      return bail(st);
    int32_t t32 = 0;
    cudaMemcpyAsync(&t32, c->offsets + nq, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&max_k, kmax.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    st = sync_and_check(s);
    if (st != ABX_SUCCESS)
      return bail(st);
    total = t32;
  }
  if (dmalloc_n(&c->indices, (size_t)total, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS indices"));
  Scratch<float> dist_tmp;
  float *dist = nullptr;
  if (with_distances)
  {
    if (dmalloc_n(&c->distances, (size_t)total, s) != cudaSuccess)
      return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS distances"));
    dist = c->distances;
  }
  else if (max_k > 32)
  {
    if (dist_tmp.alloc((size_t)total, s) != cudaSuccess)
      return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "kNN heap"));
    dist = dist_tmp.ptr;
  }
  abx_status st = launch_nearest(s, tv, f, d_queries, nq, perm.ptr, d_k, k, max_k,
                                 counted ? c->offsets : nullptr, counted ? nullptr : c->offsets,
                                 c->indices, dist);
  if (st != ABX_SUCCESS)
    return bail(st);
  c->nres = total;
  *out = c;
  return ABX_SUCCESS;
}

} // namespace

extern "C" {

const char *abx_status_string(abx_status status)
{
  switch (status)
  {
  case ABX_SUCCESS: return "ABX_SUCCESS";
  case ABX_ERROR_INVALID_ARGUMENT: return "ABX_ERROR_INVALID_ARGUMENT";
  case ABX_ERROR_CUDA: return "ABX_ERROR_CUDA";
  case ABX_ERROR_OUT_OF_MEMORY: return "ABX_ERROR_OUT_OF_MEMORY";
  case ABX_ERROR_BUFFER_OVERFLOW: return "ABX_ERROR_BUFFER_OVERFLOW";
  case ABX_ERROR_DEVICE: return "ABX_ERROR_DEVICE";
  case ABX_ERROR_NOT_SUPPORTED: return "ABX_ERROR_NOT_SUPPORTED";
  case ABX_ERROR_TIMEOUT: return "ABX_ERROR_TIMEOUT";
  }
  return "ABX_UNKNOWN_STATUS";
}

const char *abx_last_error(void) { return g_last_error.c_str(); }

const char *abx_version(void) { return "0.1.0"; }

abx_status abx_device_errors(void *stream, uint32_t *h_bits)
{
  if (!h_bits)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_device_errors: null output");
  ABX_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  DeviceState &ds = device_state();
  ABX_CUDA_TRY(cudaMemcpy(h_bits, ds.d_error, sizeof(unsigned), cudaMemcpyDeviceToHost));
  ABX_CUDA_TRY(cudaMemset(ds.d_error, 0, sizeof(unsigned)));
  return ABX_SUCCESS;
}

abx_status abx_tuning_set(const char *name, int32_t value)
{
  if (!name)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_tuning_set: null name");
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  g_tuning[name] = value;
  return ABX_SUCCESS;
}

abx_status abx_tuning_reset(void)
{
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  g_tuning.clear();
  return ABX_SUCCESS;
}

abx_status abx_profiling_enable(int32_t enable)
{
  g_prof_on.store(enable != 0);
  return ABX_SUCCESS;
}

abx_status abx_profiling_stage(const char *stage, double *h_total_ms, int64_t *h_launches)
{
  if (!stage)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_profiling_stage: null stage");
  const bool all = std::strcmp(stage, "*") == 0;
  double total = 0;
  int64_t launches = 0;
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  for (auto const &r : g_prof)
  {
    if (!all && r.stage != stage)
      continue;
    ABX_CUDA_TRY(cudaEventSynchronize(r.end));
    float ms = 0;
    ABX_CUDA_TRY(cudaEventElapsedTime(&ms, r.start, r.end));
    total += ms;
    launches += r.kernels;
  }
  if (h_total_ms)
    *h_total_ms = total;
  if (h_launches)
    *h_launches = launches;
  return ABX_SUCCESS;
}

abx_status abx_profiling_reset(void)
{
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  for (auto const &r : g_prof)
  {
    cudaEventSynchronize(r.end);
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.end);
  }
  g_prof.clear();
  return ABX_SUCCESS;
}

namespace abx
{
// Records of a KDOP tree: (2 max(n - 1, 1) + 1) node slot records and n leaf
// records, kdop_pad(ndir) / 4 float4 each.
size_t kdop_node_records(int64_t n) { return n > 0 ? 2 * (size_t)std::max<int64_t>(n - 1, 1) + 1 : 1; }

// A tree over n KDOP values (t->ndir set): the box tree of the values' axis
// boxes, then the KDOP records.  An empty tree keeps one empty root record.
abx_status build_kdop_tree(abx_bvh *t, const float *d_kdops)
{
  cudaStream_t s = t->stream;
  const int64_t n = t->n;
  const int rec = kdop_pad(t->ndir) / 4;
  Scratch<float> boxes;
  ABX_CUDA_TRY(boxes.alloc((size_t)std::max<int64_t>(n, 1) * 6, s));
  ABX_TRY(kdop_axis_boxes(s, t->kdop_kind, d_kdops, n, boxes.ptr));
  ABX_TRY(build_tree(t, boxes.ptr));
  ABX_CUDA_TRY(dmalloc_n(&t->knodes, kdop_node_records(n) * rec, s));
  ABX_CUDA_TRY(dmalloc_n(&t->kleaves, (size_t)std::max<int64_t>(n, 1) * rec, s));
  if (n == 0)
  {
    std::vector<float> empty(4 * rec, 0.f);
    for (int i = 0; i < t->ndir; ++i)
    {
      empty[i] = FLT_MAX;
      empty[t->ndir + i] = -FLT_MAX;
    }
    ABX_CUDA_TRY(cudaMemcpyAsync(t->knodes, empty.data(), empty.size() * sizeof(float),
                                 cudaMemcpyHostToDevice, s));
    // the copy reads a host vector: finish it before returning
    ABX_CUDA_TRY(cudaStreamSynchronize(s));
    return ABX_SUCCESS;
  }
  return kdop_records(s, t->kdop_kind, t->tnodes, t->sorted, n, d_kdops, t->knodes, t->kleaves);
}
} // namespace abx

abx_status abx_bvh_create(void *stream, abx_geometry kind, const float *d_values, int64_t n,
                          abx_bvh **out)
{
  if (!out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create: null output handle");
  *out = nullptr;
  if (kind != ABX_POINT && kind != ABX_BOX && kdop_ndir(kind) == 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_bvh_create: values must be points, boxes or KDOPs");
  if (n < 0 || n >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create: size out of range [0, 2^31-1)");
  if (n > 0 && !d_values)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create: null values");
  device_state();
  abx_bvh *t = new (std::nothrow) abx_bvh;
  if (!t)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_bvh_create: host allocation");
  cudaGetDevice(&t->device);
  t->stream = as_stream(stream);
  t->kind = kdop_ndir(kind) ? ABX_BOX : kind;
  t->ndir = kdop_ndir(kind);
  t->kdop_kind = kind;
  t->n = n;
  cudaError_t e = cudaMallocHost(&t->h_bounds, 6 * sizeof(float));
  if (e != cudaSuccess)
  {
    t->h_bounds = nullptr;
    destroy_tree(t);
    return fail_cuda(e, "cudaMallocHost");
  }
  e = cudaEventCreateWithFlags(&t->ready, cudaEventDisableTiming);
  if (e != cudaSuccess)
  {
    t->ready = nullptr;
    destroy_tree(t);
    return fail_cuda(e, "cudaEventCreate");
  }
  abx_status st = t->ndir ? build_kdop_tree(t, d_values) : build_tree(t, d_values);
  if (st == ABX_SUCCESS)
  {
    e = cudaEventRecord(t->ready, t->stream);
    if (e != cudaSuccess)
      st = fail_cuda(e, "cudaEventRecord");
  }
  if (st != ABX_SUCCESS)
  {
    cudaStreamSynchronize(t->stream);
    destroy_tree(t);
    return st;
  }
  *out = t;
  return ABX_SUCCESS;
}

abx_status abx_bvh_create_strided(void *stream, abx_geometry kind, abx_values values, int64_t n,
                                  abx_bvh **out)
{
  if (!out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create_strided: null output handle");
  *out = nullptr;
  if (kind != ABX_POINT && kind != ABX_BOX && kdop_ndir(kind) == 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create_strided: points, boxes or KDOPs");
  if (n < 0 || n >= (int64_t)INT32_MAX || values.value_stride < 0 || values.coord_stride < 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create_strided: bad size or strides");
  if (n > 0 && !values.data)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_create_strided: null values");
  const int cols = kdop_ndir(kind) ? 2 * kdop_ndir(kind) : kind == ABX_BOX ? 6 : 3;
  if (values.value_stride == cols && values.coord_stride == 1)
    return abx_bvh_create(stream, kind, values.data, n, out);
  cudaStream_t s = as_stream(stream);
  device_state();
  Scratch<float> packed;
  ABX_CUDA_TRY(packed.alloc((size_t)std::max<int64_t>(n, 1) * cols, s));
  ABX_TRY(pack_strided(s, values.data, values.value_stride, values.coord_stride, n, cols,
                       packed.ptr));
  // the build reads the packed rows on the same stream; the scratch is
  // released stream-ordered after it
  return abx_bvh_create(stream, kind, packed.ptr, n, out);
}

namespace
{
constexpr char kTreeMagic[8] = {'A', 'B', 'X', 'B', 'V', 'H', '0', '1'};

struct TreeFileHeader
{
  char magic[8];
  int32_t kind;
  int32_t reserved;
  int64_t n;
  float bounds[6];
};
static_assert(sizeof(TreeFileHeader) == 48, "tree file header is 48 bytes");

size_t tree_tnode_count(int64_t n) { return n > 1 ? (size_t)(n - 1) : (n == 1 ? 1 : 0); }
size_t tree_sorted_count(abx_geometry kind, int64_t n)
{
  return (size_t)n * (kind == ABX_BOX ? 2 : 1);
}
// float4 of the KDOP records of a tree (0 for other trees)
size_t tree_knode_count(int ndir, int64_t n)
{
  return ndir ? kdop_node_records(n) * (kdop_pad(ndir) / 4) : 0;
}
size_t tree_kleaf_count(int ndir, int64_t n)
{
  return ndir ? (size_t)std::max<int64_t>(n, 1) * (kdop_pad(ndir) / 4) : 0;
}

// Every reference a traversal follows stays inside the tree: a file read
// from disk is checked before it reaches the device (the kernels' own
// range checks stop walks, but a bucket scan reads leaf positions
// [start, start + count) straight from a node's count field).
bool valid_tree_arrays(const std::vector<TNode> &tn, const std::vector<float4> &so, int64_t n,
                       int leaf_float4s)
{
  const int64_t nt = (int64_t)tn.size();
  for (int64_t t = 0; t < n; ++t)
  {
    int v;
    std::memcpy(&v, &so[(size_t)(t * leaf_float4s)].w, sizeof(int));
    if (v < 0 || v >= n)
      return false;
  }
  for (int64_t i = 0; i < nt; ++i)
  {
    const int refs[2] = {tn[i].d.x, tn[i].d.y}, cfs[2] = {tn[i].d.z, tn[i].d.w};
    for (int side = 0; side < 2; ++side)
    {
      const int ref = refs[side], cf = cfs[side];
      if (ref < 0)
      {
        const int64_t v = bucket_start(ref);
        const bool absent = n == 1 && side == 1 && cf == 0; // one-leaf tree
        if (!absent && (cf != 1 || v >= n))
          return false;
        continue;
      }
      if (ref >= nt || (cf & ~(0xffff | kBucketRightEnd)) != 0)
        return false;
      const int c = cf & 0xffff;
      if (c == 0)
        continue;
      if (c < 2 || c > kMaxBucket)
        return false;
      const int64_t start = (cf & kBucketRightEnd) ? (int64_t)ref - c + 1 : ref;
      if (start < 0 || start + c > n)
        return false;
    }
  }
  return true;
}
} // namespace

abx_status abx_bvh_save(const abx_bvh *bvh, const char *path)
{
  if (!bvh || !path || bvh->d_off)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_save: bad argument");
  ABX_CUDA_TRY(cudaEventSynchronize(bvh->ready));
  TreeFileHeader h{};
  std::memcpy(h.magic, kTreeMagic, 8);
  h.kind = abx_bvh_geometry(bvh);
  h.n = bvh->n;
  std::memcpy(h.bounds, bvh->h_bounds, sizeof(h.bounds));
  const size_t nt = tree_tnode_count(bvh->n), ns = tree_sorted_count(bvh->kind, bvh->n);
  const size_t nkn = tree_knode_count(bvh->ndir, bvh->n), nkl = tree_kleaf_count(bvh->ndir, bvh->n);
  std::vector<TNode> tn(nt);
  std::vector<float4> so(ns), kn(nkn), kl(nkl);
  if (nt)
    ABX_CUDA_TRY(cudaMemcpy(tn.data(), bvh->tnodes, nt * sizeof(TNode), cudaMemcpyDeviceToHost));
  if (ns)
    ABX_CUDA_TRY(cudaMemcpy(so.data(), bvh->sorted, ns * sizeof(float4), cudaMemcpyDeviceToHost));
  if (nkn)
    ABX_CUDA_TRY(cudaMemcpy(kn.data(), bvh->knodes, nkn * sizeof(float4), cudaMemcpyDeviceToHost));
  if (nkl)
    ABX_CUDA_TRY(cudaMemcpy(kl.data(), bvh->kleaves, nkl * sizeof(float4), cudaMemcpyDeviceToHost));
  FILE *f = std::fopen(path, "wb");
  if (!f)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string("abx_bvh_save: cannot open ") + path);
  const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
                  (nt == 0 || std::fwrite(tn.data(), sizeof(TNode), nt, f) == nt) &&
                  (ns == 0 || std::fwrite(so.data(), sizeof(float4), ns, f) == ns) &&
                  (nkn == 0 || std::fwrite(kn.data(), sizeof(float4), nkn, f) == nkn) &&
                  (nkl == 0 || std::fwrite(kl.data(), sizeof(float4), nkl, f) == nkl);
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string("abx_bvh_save: write failed: ") + path);
  return ABX_SUCCESS;
}

abx_status abx_bvh_load(void *stream, const char *path, abx_bvh **out)
{
  if (!path || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_load: null argument");
  *out = nullptr;
  FILE *f = std::fopen(path, "rb");
  if (!f)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string("abx_bvh_load: cannot open ") + path);
  TreeFileHeader h{};
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, kTreeMagic, 8) == 0 &&
            (h.kind == ABX_POINT || h.kind == ABX_BOX || kdop_ndir(h.kind) > 0) && h.n >= 0 &&
            h.n < (int64_t)INT32_MAX;
  const int ndir = ok ? kdop_ndir(h.kind) : 0;
  const abx_geometry kind = ok ? (ndir ? ABX_BOX : (abx_geometry)h.kind) : ABX_POINT;
  const size_t nt = ok ? tree_tnode_count(h.n) : 0, ns = ok ? tree_sorted_count(kind, h.n) : 0;
  const size_t nkn = ok ? tree_knode_count(ndir, h.n) : 0;
  const size_t nkl = ok ? tree_kleaf_count(ndir, h.n) : 0;
  std::vector<TNode> tn(nt);
  std::vector<float4> so(ns), kn(nkn), kl(nkl);
  ok = ok && (nt == 0 || std::fread(tn.data(), sizeof(TNode), nt, f) == nt) &&
       (ns == 0 || std::fread(so.data(), sizeof(float4), ns, f) == ns) &&
       (nkn == 0 || std::fread(kn.data(), sizeof(float4), nkn, f) == nkn) &&
       (nkl == 0 || std::fread(kl.data(), sizeof(float4), nkl, f) == nkl);
  std::fclose(f);
  if (ok)
    ok = valid_tree_arrays(tn, so, h.n, kind == ABX_BOX ? 2 : 1);
  if (!ok)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string("abx_bvh_load: not a tree file: ") + path);
  device_state();
  abx_bvh *t = new (std::nothrow) abx_bvh;
  if (!t)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_bvh_load");
  cudaGetDevice(&t->device);
  t->stream = as_stream(stream);
  t->kind = kind;
  t->ndir = ndir;
  t->kdop_kind = ndir ? (abx_geometry)h.kind : ABX_BOX;
  t->n = h.n;
  cudaStream_t s = t->stream;
  cudaError_t e = cudaMallocHost(&t->h_bounds, 6 * sizeof(float));
  if (e == cudaSuccess)
    e = cudaEventCreateWithFlags(&t->ready, cudaEventDisableTiming);
  if (e == cudaSuccess)
    e = dmalloc_n(&t->d_bounds, 6, s);
  if (e == cudaSuccess && nt)
    e = dmalloc_n(&t->tnodes, nt, s);
  if (e == cudaSuccess && ns)
    e = dmalloc_n(&t->sorted, ns, s);
  if (e == cudaSuccess && nkn)
    e = dmalloc_n(&t->knodes, nkn, s);
  if (e == cudaSuccess && nkl)
    e = dmalloc_n(&t->kleaves, nkl, s);
  if (e == cudaSuccess)
  {
    std::memcpy(t->h_bounds, h.bounds, sizeof(h.bounds));
    e = cudaMemcpyAsync(t->d_bounds, t->h_bounds, 6 * sizeof(float), cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess && nt)
    e = cudaMemcpyAsync(t->tnodes, tn.data(), nt * sizeof(TNode), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && ns)
    e = cudaMemcpyAsync(t->sorted, so.data(), ns * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && nkn)
    e = cudaMemcpyAsync(t->knodes, kn.data(), nkn * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && nkl)
    e = cudaMemcpyAsync(t->kleaves, kl.data(), nkl * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaEventRecord(t->ready, s);
  // the host staging vectors are released on return: finish the copies first
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
  {
    cudaStreamSynchronize(s);
    destroy_tree(t);
    return fail_cuda(e, "abx_bvh_load");
  }
  *out = t;
  return ABX_SUCCESS;
}

abx_status abx_bvh_destroy(abx_bvh *bvh)
{
  destroy_tree(bvh);
  return ABX_SUCCESS;
}

int64_t abx_bvh_size(const abx_bvh *bvh) { return bvh ? bvh->n : 0; }

abx_geometry abx_bvh_geometry(const abx_bvh *bvh)
{
  return bvh ? (bvh->ndir ? bvh->kdop_kind : bvh->kind) : ABX_POINT;
}

abx_status abx_bvh_kdop_bounds(const abx_bvh *bvh, float *h_kdop)
{
  if (!bvh || !h_kdop)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_kdop_bounds: null argument");
  if (!bvh->ndir)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_kdop_bounds: not a KDOP tree");
  ABX_CUDA_TRY(cudaEventSynchronize(bvh->ready));
  const int rec = kdop_pad(bvh->ndir);
  std::vector<float> r(rec);
  const size_t root = (kdop_node_records(bvh->n) - 1) * rec;
  ABX_CUDA_TRY(cudaMemcpy(r.data(), reinterpret_cast<const float *>(bvh->knodes) + root,
                          rec * sizeof(float), cudaMemcpyDeviceToHost));
  std::memcpy(h_kdop, r.data(), 2 * bvh->ndir * sizeof(float));
  return ABX_SUCCESS;
}

abx_status abx_gather_rows(void *stream, const void *d_src, int64_t n_src, int64_t row_bytes,
                           const int32_t *d_rows, int64_t m, void *d_dst)
{
  if (row_bytes <= 0 || row_bytes % 4 != 0 || row_bytes > ((int64_t)1 << 20) || n_src < 0 ||
      m < 0 || (m > 0 && (!d_src || !d_rows || !d_dst)))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_gather_rows: bad arguments");
  device_state();
  return gather_rows(as_stream(stream), d_src, n_src, (int)(row_bytes / 4), d_rows, m, d_dst);
}

abx_status abx_kdop_from_geometry(void *stream, abx_geometry kind, const float *d_values,
                                  int64_t n, abx_geometry kdop_kind, float *d_kdops)
{
  if ((kind != ABX_POINT && kind != ABX_BOX) || kdop_ndir(kdop_kind) == 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_kdop_from_geometry: points or boxes to a KDOP kind");
  if (n < 0 || (n > 0 && (!d_values || !d_kdops)))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_kdop_from_geometry: bad arrays");
  device_state();
  return kdop_from_geometry(as_stream(stream), kind, d_values, n, kdop_kind, d_kdops);
}

abx_status abx_bvh_bounds(const abx_bvh *bvh, float h_box[6])
{
  if (!bvh || !h_box)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_bounds: null argument");
  ABX_CUDA_TRY(cudaEventSynchronize(bvh->ready));
  std::memcpy(h_box, bvh->h_bounds, 6 * sizeof(float));
  return ABX_SUCCESS;
}

abx_status abx_bvh_export_nodes(const abx_bvh *bvh, void *stream, int32_t *d_leaves,
                                void *d_internal)
{
  if (!bvh)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_export_nodes: null tree");
  cudaStream_t s = as_stream(stream);
  ABX_CUDA_TRY(cudaStreamWaitEvent(s, bvh->ready, 0));
  if (bvh->ndir)
    return fail(ABX_ERROR_NOT_SUPPORTED, "abx_bvh_export_nodes: KDOP-bounded tree");
  if (!d_leaves && !d_internal)
    return ABX_SUCCESS;
  device_state();
  return export_reference_layout(s, bvh->kind, bvh->tnodes, bvh->sorted, 0, bvh->n,
                                 reinterpret_cast<LeafNode *>(d_leaves),
                                 reinterpret_cast<InternalNode *>(d_internal));
}

abx_status abx_bvh_device_view(const abx_bvh *bvh, abx_device_view *out)
{
  if (!bvh || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_device_view: null argument");
  if (bvh->ndir)
    return fail(ABX_ERROR_NOT_SUPPORTED, "abx_bvh_device_view: KDOP-bounded tree");
  out->nodes = bvh->tnodes;
  out->leaves = bvh->sorted;
  out->size = bvh->n;
  out->geometry = bvh->kind;
  out->reserved = 0;
  return ABX_SUCCESS;
}

abx_status abx_bvh_query_intersects(const abx_bvh *bvh, void *stream, abx_geometry kind,
                                    const float *d_predicates, int64_t nq,
                                    abx_traversal_policy policy, abx_crs **out)
{
  if (!bvh || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_intersects: null argument");
  *out = nullptr;
  if (bvh->d_off)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_intersects: a forest handle");
  if (kind != ABX_SPHERE && kind != ABX_BOX && kind != ABX_RAY && kdop_ndir(kind) == 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_bvh_query_intersects: predicates must be spheres, boxes, rays or KDOPs");
  if (bvh->ndir && kind != ABX_BOX && kdop_ndir(kind) != bvh->ndir)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_bvh_query_intersects: a KDOP tree answers intersects(Box) and "
                "intersects(KDOP) with its own directions");
  if (nq < 0 || nq >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_intersects: bad number of queries");
  if (nq > 0 && !d_predicates)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_intersects: null predicates");
  cudaStream_t s = as_stream(stream);
  if (kind == ABX_RAY)
  {
    device_state();
    Scratch<float> rays;
    ABX_CUDA_TRY(rays.alloc((size_t)std::max<int64_t>(nq, 1) * 6, s));
    ABX_TRY(ray_normalize(s, d_predicates, nq, rays.ptr));
    return query_intersects(bvh, s, kind, rays.ptr, nq, nullptr, policy, out);
  }
  return query_intersects(bvh, s, kind, d_predicates, nq, nullptr, policy, out);
}

abx_status abx_bvh_query_nearest(const abx_bvh *bvh, void *stream, const float *d_queries,
                                 int64_t nq, const int32_t *d_k, int32_t k,
                                 abx_traversal_policy policy, int32_t with_distances,
                                 abx_crs **out)
{
  if (!bvh || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest: null argument");
  *out = nullptr;
  if (bvh->d_off)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest: a forest handle");
  if (bvh->ndir)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_bvh_query_nearest: no distance to a KDOP (nearest queries need points or boxes)");
  if (nq < 0 || nq >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest: bad number of queries");
  if (nq > 0 && !d_queries)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest: null queries");
  return query_nearest(bvh, as_stream(stream), d_queries, nq, nullptr, d_k, k, policy,
                       with_distances, out);
}

namespace abx
{
// Device address of page-locked host memory mapped into the device's address
// space (cudaHostAlloc / cudaHostRegister on a unified-address system); null
// for any other pointer.
void *mapped_host_pointer(void *h)
{
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess)
  {
    cudaGetLastError(); // clear the error of an unknown pointer
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Smallest chunk of the default schedule of abx_bvh_query_nearest_host.
constexpr int64_t kHostMinChunk = (int64_t)1 << 18;

// nearest(point, k) of nq >= 1 device queries into caller buffers (offsets
// optional), no allocation visible to the caller; plain_sort orders the
// predicates without reading anything back to the host.
abx_status nearest_into(const abx_bvh *bvh, cudaStream_t s, const float *d_queries, int64_t nq,
                        int32_t k, abx_traversal_policy policy, bool plain_sort,
                        int32_t *d_offsets, int32_t *d_indices, float *d_distances)
{
  Scratch<uint32_t> perm;
  if (policy.sort_predicates && nq > 1 && bvh->tnodes)
  {
    ABX_CUDA_TRY(perm.alloc(nq, s));
    Scratch<uint32_t> codes, hist;
    ABX_CUDA_TRY(codes.alloc(nq, s));
    ABX_CUDA_TRY(hist.alloc(4 * 256, s));
    ABX_CUDA_TRY(cudaMemsetAsync(hist.ptr, 0, 4 * 256 * sizeof(uint32_t), s));
    ABX_TRY(morton32_codes(s, ABX_POINT, d_queries, nq, bvh->d_bounds, codes.ptr, hist.ptr));
    const int digits = tuning_value("QUERY_ORDER_DIGITS", kQueryOrderDigits);
    if (digits >= 1 && digits <= 3)
      ABX_TRY(radix_order_top_u32(s, codes.ptr, perm.ptr, nq, 4, hist.ptr, digits));
    else
      ABX_TRY(radix_sort_u32(s, codes.ptr, perm.ptr, nullptr, nq, 4, hist.ptr,
                             plain_sort ? 0 : hybrid_top_passes(nq, 4)));
  }
  const int64_t kk = std::min<int64_t>(k, bvh->n);
  Scratch<float> dist_tmp;
  float *dist = d_distances;
  if (!dist && k > 32)
  {
    ABX_CUDA_TRY(dist_tmp.alloc((size_t)(kk * nq), s));
    dist = dist_tmp.ptr;
  }
  return launch_nearest(s, view_of(bvh), nullptr, d_queries, nq, perm.ptr, nullptr, k, k, nullptr,
                        d_offsets, d_indices, dist);
}
} // namespace abx

abx_status abx_bvh_query_nearest_into(const abx_bvh *bvh, void *stream, const float *d_queries,
                                      int64_t nq, int32_t k, abx_traversal_policy policy,
                                      int32_t *d_offsets, int32_t *d_indices, float *d_distances)
{
  if (!bvh || !d_offsets)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_into: null argument");
  if (bvh->d_off)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_into: a forest handle");
  if (bvh->ndir)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_into: no distance to a KDOP");
  if (nq < 0 || nq >= (int64_t)INT32_MAX || (nq > 0 && !d_queries))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_into: bad queries");
  cudaStream_t s = as_stream(stream);
  device_state();
  if (!stream_capturing(s))
    ABX_CUDA_TRY(cudaStreamWaitEvent(s, bvh->ready, 0));
  if (k < 0)
    k = 0;
  const int64_t kk = std::min<int64_t>(k, bvh->n);
  if (kk * nq >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_into: too many results");
  if (nq > 0 && kk > 0 && !d_indices)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_into: null indices");
  if (nq == 0 || kk == 0)
  {
    ABX_CUDA_TRY(cudaMemsetAsync(d_offsets, 0, (nq + 1) * sizeof(int32_t), s));
    return ABX_SUCCESS;
  }
  return nearest_into(bvh, s, d_queries, nq, k, policy, stream_capturing(s), d_offsets, d_indices,
                      d_distances);
}

abx_status abx_bvh_query_nearest_host(const abx_bvh *bvh, void *stream, const float *h_queries,
                                      int64_t nq, int32_t k, abx_traversal_policy policy,
                                      int64_t chunk, int32_t *h_offsets, int32_t *h_indices,
                                      float *h_distances)
{
  if (!bvh || !h_offsets)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_host: null argument");
  if (bvh->d_off)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_host: a forest handle");
  if (bvh->ndir)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_host: no distance to a KDOP");
  if (nq < 0 || nq >= (int64_t)INT32_MAX || (nq > 0 && !h_queries))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_host: bad queries");
  cudaStream_t s = as_stream(stream);
  device_state();
  if (k < 0)
    k = 0;
  const int64_t kk = std::min<int64_t>(k, bvh->n);
  if (kk * nq >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_host: too many results");
  if (nq > 0 && kk > 0 && !h_indices)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_nearest_host: null indices");
  if (nq == 0 || kk == 0)
  {
    std::memset(h_offsets, 0, (size_t)(nq + 1) * sizeof(int32_t));
    return ABX_SUCCESS;
  }
  ABX_CUDA_TRY(cudaStreamWaitEvent(s, bvh->ready, 0));
  // Pinned (page-locked, device-mapped) result buffers are written by the
  // traversal itself over the CPU-GPU link: no result copy after the last
  // query, no chunking.  Other host memory takes the chunked copies below.
  void *dev_off = mapped_host_pointer(h_offsets), *dev_idx = mapped_host_pointer(h_indices);
  void *dev_dist = h_distances ? mapped_host_pointer(h_distances) : nullptr;
  if (chunk <= 0 && dev_off && dev_idx && (!h_distances || dev_dist) &&
      tuning_value("HOST_DIRECT", 1))
  {
    // the queries move in on their own stream, alongside whatever the tree's
    // build still runs on s
    struct Copy
    {
      cudaStream_t st = nullptr;
      cudaEvent_t in = nullptr, off = nullptr, done = nullptr;
      ~Copy()
      {
        for (cudaEvent_t e : {in, off, done})
          if (e)
            cudaEventDestroy(e);
        if (st)
          cudaStreamDestroy(st);
      }
    } c;
    ABX_CUDA_TRY(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    ABX_CUDA_TRY(cudaEventCreateWithFlags(&c.in, cudaEventDisableTiming));
    ABX_CUDA_TRY(cudaEventCreateWithFlags(&c.off, cudaEventDisableTiming));
    ABX_CUDA_TRY(cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming));
    Scratch<float> dq; // allocated and released on the copy stream
    ABX_CUDA_TRY(dq.alloc((size_t)nq * 3, c.st));
    ABX_CUDA_TRY(cudaMemcpyAsync(dq.ptr, h_queries, (size_t)nq * 3 * sizeof(float),
                                 cudaMemcpyHostToDevice, c.st));
    ABX_CUDA_TRY(cudaEventRecord(c.in, c.st));
    // the offsets (a fixed k) go to the host alongside the traversal
    ABX_TRY(fill_offsets_iota(c.st, static_cast<int32_t *>(dev_off), nq + 1, 0, kk));
    ABX_CUDA_TRY(cudaEventRecord(c.off, c.st));
    ABX_CUDA_TRY(cudaStreamWaitEvent(s, c.in, 0));
    abx_status st = nearest_into(bvh, s, dq.ptr, nq, k, policy, false, nullptr,
                                 static_cast<int32_t *>(dev_idx), static_cast<float *>(dev_dist));
    cudaStreamWaitEvent(s, c.off, 0);
    // the copy stream frees the queries after the traversal read them
    cudaEventRecord(c.done, s);
    cudaStreamWaitEvent(c.st, c.done, 0);
    if (st != ABX_SUCCESS)
    {
      cudaStreamSynchronize(s);
      return st;
    }
    return sync_and_check(s);
  }
  // chunk boundaries: a fixed size, by default 40% of the queries (at least
  // kHostMinChunk): the traversal of a chunk gets slower as its Morton-sorted
  // queries thin out in space (1e7 uniform queries, k = 16: chunks of 40%
  // 20.8 ms, halves of what is left 21.6 ms, 10% 23.9 ms, one chunk 22.6
  // ms), while the copy of the last chunk's results is not hidden
  if (chunk <= 0)
    chunk = std::max(kHostMinChunk, (nq * 2 + 4) / 5);
  std::vector<int64_t> bounds{0};
  while (bounds.back() < nq)
    bounds.push_back(bounds.back() + std::min(chunk, nq - bounds.back()));
  const int64_t nchunks = (int64_t)bounds.size() - 1;
  int64_t max_chunk = 0;
  for (int64_t i = 0; i < nchunks; ++i)
    max_chunk = std::max(max_chunk, bounds[i + 1] - bounds[i]);
  chunk = max_chunk;
  // two buffer sets; the copy streams move chunk i + 1 in and chunk i - 1 out
  // while chunk i is traversed on s
  Scratch<float> qbuf[2], dbuf[2];
  Scratch<int32_t> ibuf[2], obuf[2];
  for (int b = 0; b < 2; ++b)
  {
    ABX_CUDA_TRY(qbuf[b].alloc((size_t)chunk * 3, s));
    ABX_CUDA_TRY(ibuf[b].alloc((size_t)(chunk * kk), s));
    ABX_CUDA_TRY(obuf[b].alloc((size_t)chunk + 1, s));
    if (h_distances)
      ABX_CUDA_TRY(dbuf[b].alloc((size_t)(chunk * kk), s));
  }
  struct Pipe
  {
    cudaStream_t in = nullptr, out = nullptr;
    cudaEvent_t ev[7] = {}; // alloc, in_done[2], knn_done[2], out_done[2]
    ~Pipe()
    {
      for (cudaEvent_t e : ev)
        if (e)
          cudaEventDestroy(e);
      for (cudaStream_t st : {in, out})
        if (st)
          cudaStreamDestroy(st);
    }
  } p;
  ABX_CUDA_TRY(cudaStreamCreateWithFlags(&p.in, cudaStreamNonBlocking));
  ABX_CUDA_TRY(cudaStreamCreateWithFlags(&p.out, cudaStreamNonBlocking));
  for (cudaEvent_t &e : p.ev)
    ABX_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaEvent_t alloc = p.ev[0], *in_done = p.ev + 1, *knn_done = p.ev + 3, *out_done = p.ev + 5;
  // one traversal stream: two chunks traversed at once on two streams were
  // slower than in turn (their queries compete for the caches)
  ABX_CUDA_TRY(cudaEventRecord(alloc, s));
  ABX_CUDA_TRY(cudaStreamWaitEvent(p.in, alloc, 0));
  ABX_CUDA_TRY(cudaStreamWaitEvent(p.out, alloc, 0));
  for (int b = 0; b < 2; ++b)
  {
    ABX_CUDA_TRY(cudaEventRecord(knn_done[b], s));
    ABX_CUDA_TRY(cudaEventRecord(out_done[b], p.out));
  }
  abx_status st = ABX_SUCCESS;
  for (int64_t i = 0; i < nchunks && st == ABX_SUCCESS; ++i)
  {
    const int b = (int)(i & 1);
    const int64_t a = bounds[i], m = bounds[i + 1] - a;
    const bool last = i == nchunks - 1;
    cudaError_t e = cudaStreamWaitEvent(p.in, knn_done[b], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(qbuf[b].ptr, h_queries + 3 * a, (size_t)m * 3 * sizeof(float),
                          cudaMemcpyHostToDevice, p.in);
    if (e == cudaSuccess)
      e = cudaEventRecord(in_done[b], p.in);
    if (e == cudaSuccess)
      e = cudaStreamWaitEvent(s, in_done[b], 0);
    if (e == cudaSuccess)
      e = cudaStreamWaitEvent(s, out_done[b], 0);
    if (e != cudaSuccess)
    {
      st = fail_cuda(e, "abx_bvh_query_nearest_host");
      break;
    }
    // no host synchronisation inside the chunk: the plain predicate sort
    st = nearest_into(bvh, s, qbuf[b].ptr, m, k, policy, true, nullptr, ibuf[b].ptr,
                      h_distances ? dbuf[b].ptr : nullptr);
    if (st == ABX_SUCCESS)
      st = fill_offsets_iota(s, obuf[b].ptr, m + (last ? 1 : 0), a, kk);
    if (st != ABX_SUCCESS)
      break;
    e = cudaEventRecord(knn_done[b], s);
    if (e == cudaSuccess)
      e = cudaStreamWaitEvent(p.out, knn_done[b], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_indices + a * kk, ibuf[b].ptr, (size_t)(m * kk) * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, p.out);
    if (e == cudaSuccess && h_distances)
      e = cudaMemcpyAsync(h_distances + a * kk, dbuf[b].ptr, (size_t)(m * kk) * sizeof(float),
                          cudaMemcpyDeviceToHost, p.out);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_offsets + a, obuf[b].ptr, (size_t)(m + (last ? 1 : 0)) * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, p.out);
    if (e == cudaSuccess)
      e = cudaEventRecord(out_done[b], p.out);
    if (e != cudaSuccess)
      st = fail_cuda(e, "abx_bvh_query_nearest_host");
  }
  // the buffers are released stream-ordered on s after the last copies
  for (int b = 0; b < 2; ++b)
    cudaStreamWaitEvent(s, out_done[b], 0);
  cudaStreamSynchronize(p.in);
  cudaStreamSynchronize(p.out);
  if (st != ABX_SUCCESS)
  {
    cudaStreamSynchronize(s);
    return st;
  }
  return sync_and_check(s);
}

abx_status abx_bvh_query_ordered_intersects(const abx_bvh *bvh, void *stream, const float *d_rays,
                                            int64_t nq, int32_t k, abx_traversal_policy policy,
                                            int32_t with_distances, abx_crs **out)
{
  if (!bvh || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_ordered_intersects: null argument");
  *out = nullptr;
  if (bvh->d_off)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_ordered_intersects: a forest handle");
  if (bvh->ndir)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_bvh_query_ordered_intersects: no ray test for KDOP values");
  if (nq < 0 || nq >= (int64_t)INT32_MAX || (nq > 0 && !d_rays))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_bvh_query_ordered_intersects: bad rays");
  cudaStream_t s = as_stream(stream);
  device_state();
  Scratch<float> rays;
  ABX_CUDA_TRY(rays.alloc((size_t)std::max<int64_t>(nq, 1) * 6, s));
  ABX_TRY(ray_normalize(s, d_rays, nq, rays.ptr));
  if (k >= 1 && k <= kRayNearestMaxK && bvh->n >= 1 && bvh->tnodes &&
      tuning_value("RAY_NEAREST", 1))
  {
    // nearest(Ray, k): a pruned walk keeps each ray's first k hits, with no
    // full hit list and no ordering pass (same rows)
    Scratch<uint32_t> perm;
    if (policy.sort_predicates && nq > 1)
      ABX_TRY(sort_predicates(s, bvh, ABX_RAY, rays.ptr, nq, nullptr, perm));
    abx_crs *c = new (std::nothrow) abx_crs;
    if (!c)
      return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_crs");
    cudaGetDevice(&c->device);
    c->stream = s;
    c->nq = nq;
    int64_t total = 0;
    abx_status st = dmalloc_n(&c->offsets, nq + 1, s) == cudaSuccess
                        ? ray_nearest(s, bvh->kind, bvh->tnodes, bvh->sorted, bvh->n, rays.ptr,
                                      nq, perm.ptr, k, with_distances != 0, c->offsets,
                                      &c->indices, &c->distances, &total)
                        : fail(ABX_ERROR_OUT_OF_MEMORY, "CRS");
    if (st != ABX_SUCCESS)
    {
      cudaStreamSynchronize(s);
      destroy_crs(c);
      return st;
    }
    c->nres = total;
    *out = c;
    return ABX_SUCCESS;
  }
  abx_crs *raw = nullptr;
  ABX_TRY(query_intersects(bvh, s, ABX_RAY, rays.ptr, nq, nullptr, policy, &raw));
  std::unique_ptr<abx_crs, void (*)(abx_crs *)> hits(raw, destroy_crs);
  abx_crs *c = new (std::nothrow) abx_crs;
  if (!c)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_crs");
  cudaGetDevice(&c->device);
  c->stream = s;
  c->nq = nq;
  auto bail = [&](abx_status st) {
    cudaStreamSynchronize(s);
    destroy_crs(c);
    return st;
  };
  const int64_t m = raw->nres;
  if (dmalloc_n(&c->offsets, nq + 1, s) != cudaSuccess ||
      dmalloc_n(&c->indices, (size_t)m, s) != cudaSuccess ||
      (with_distances && dmalloc_n(&c->distances, (size_t)m, s) != cudaSuccess))
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS"));
  if (nq == 0)
    cudaMemsetAsync(c->offsets, 0, sizeof(int32_t), s);
  int64_t total = 0;
  abx_status st = order_ray_results(s, bvh->kind, bvh->sorted, bvh->n, rays.ptr, nq, raw->offsets,
                                    raw->indices, m, k, c->offsets, c->indices, c->distances,
                                    &total);
  if (st != ABX_SUCCESS)
    return bail(st);
  c->nres = total;
  *out = c;
  return ABX_SUCCESS;
}

abx_status abx_forest_create(void *stream, abx_geometry kind, const float *d_values,
                             const int64_t *h_offsets, int32_t ntrees, abx_forest **out)
{
  if (!out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: null output handle");
  *out = nullptr;
  if (kind != ABX_POINT && kind != ABX_BOX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: values must be points or boxes");
  if (ntrees < 1 || !h_offsets)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: need at least one tree");
  if (h_offsets[0] != 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: offsets[0] must be 0");
  for (int32_t i = 0; i < ntrees; ++i)
    if (h_offsets[i + 1] < h_offsets[i])
      return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: offsets must not decrease");
  const int64_t total = h_offsets[ntrees];
  if (total >= (int64_t)INT32_MAX / 2)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: more than 2^30-1 values");
  if (total > 0 && !d_values)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_create: null values");
  device_state();
  abx_forest *t = new (std::nothrow) abx_forest;
  if (!t)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_forest_create: host allocation");
  cudaGetDevice(&t->device);
  t->stream = as_stream(stream);
  t->kind = kind;
  t->n = total;
  t->ntrees = ntrees;
  t->h_off.assign(h_offsets, h_offsets + ntrees + 1);
  cudaError_t e = cudaMallocHost(&t->h_bounds, (size_t)6 * ntrees * sizeof(float));
  if (e != cudaSuccess)
  {
    t->h_bounds = nullptr;
    destroy_tree(t);
    return fail_cuda(e, "cudaMallocHost");
  }
  e = cudaEventCreateWithFlags(&t->ready, cudaEventDisableTiming);
  if (e != cudaSuccess)
  {
    t->ready = nullptr;
    destroy_tree(t);
    return fail_cuda(e, "cudaEventCreate");
  }
  abx_status st = build_forest(t, d_values);
  if (st == ABX_SUCCESS)
  {
    e = cudaEventRecord(t->ready, t->stream);
    if (e != cudaSuccess)
      st = fail_cuda(e, "cudaEventRecord");
  }
  if (st != ABX_SUCCESS)
  {
    cudaStreamSynchronize(t->stream);
    destroy_tree(t);
    return st;
  }
  *out = t;
  return ABX_SUCCESS;
}

abx_status abx_forest_destroy(abx_forest *forest)
{
  destroy_tree(forest);
  return ABX_SUCCESS;
}

int32_t abx_forest_num_trees(const abx_forest *forest) { return forest ? forest->ntrees : 0; }

int64_t abx_forest_size(const abx_forest *forest, int32_t tree)
{
  if (!forest || tree < 0 || tree >= forest->ntrees)
    return 0;
  return forest->h_off[tree + 1] - forest->h_off[tree];
}

abx_status abx_forest_bounds(const abx_forest *forest, int32_t tree, float h_box[6])
{
  if (!forest || !h_box || tree < 0 || tree >= forest->ntrees)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_bounds: bad argument");
  ABX_CUDA_TRY(cudaEventSynchronize(forest->ready));
  std::memcpy(h_box, forest->h_bounds + 6 * (size_t)tree, 6 * sizeof(float));
  return ABX_SUCCESS;
}

abx_status abx_forest_export_nodes(const abx_forest *forest, int32_t tree, void *stream,
                                   int32_t *d_leaves, void *d_internal)
{
  if (!forest || tree < 0 || tree >= forest->ntrees)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_export_nodes: bad argument");
  cudaStream_t s = as_stream(stream);
  ABX_CUDA_TRY(cudaStreamWaitEvent(s, forest->ready, 0));
  const int64_t lo = forest->h_off[tree];
  const int64_t n = forest->h_off[tree + 1] - lo;
  if (!d_leaves && !d_internal)
    return ABX_SUCCESS;
  device_state();
  return export_reference_layout(s, forest->kind, forest->tnodes, forest->sorted, lo, n,
                                 reinterpret_cast<LeafNode *>(d_leaves),
                                 reinterpret_cast<InternalNode *>(d_internal));
}

namespace
{
abx_status check_query_offsets(const abx_forest *forest, const int64_t *h_qoff, const char *who)
{
  if (!h_qoff)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string(who) + ": null query offsets");
  if (h_qoff[0] != 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string(who) + ": query offsets[0] must be 0");
  for (int32_t i = 0; i < forest->ntrees; ++i)
    if (h_qoff[i + 1] < h_qoff[i])
      return fail(ABX_ERROR_INVALID_ARGUMENT,
                  std::string(who) + ": query offsets must not decrease");
  if (h_qoff[forest->ntrees] >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, std::string(who) + ": bad number of queries");
  return ABX_SUCCESS;
}
} // namespace

abx_status abx_forest_query_intersects(const abx_forest *forest, void *stream,
                                       abx_geometry kind, const float *d_predicates,
                                       const int64_t *h_query_offsets,
                                       abx_traversal_policy policy, abx_crs **out)
{
  if (!forest || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_query_intersects: null argument");
  *out = nullptr;
  if (kind != ABX_SPHERE && kind != ABX_BOX && kdop_ndir(kind) == 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_forest_query_intersects: predicates must be spheres, boxes or KDOPs");
  ABX_TRY(check_query_offsets(forest, h_query_offsets, "abx_forest_query_intersects"));
  const int64_t nq = h_query_offsets[forest->ntrees];
  if (nq > 0 && !d_predicates)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_query_intersects: null predicates");
  return query_intersects(forest, as_stream(stream), kind, d_predicates, nq, h_query_offsets,
                          policy, out);
}

abx_status abx_forest_query_nearest(const abx_forest *forest, void *stream,
                                    const float *d_queries, const int64_t *h_query_offsets,
                                    const int32_t *d_k, int32_t k, abx_traversal_policy policy,
                                    int32_t with_distances, abx_crs **out)
{
  if (!forest || !out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_query_nearest: null argument");
  *out = nullptr;
  ABX_TRY(check_query_offsets(forest, h_query_offsets, "abx_forest_query_nearest"));
  const int64_t nq = h_query_offsets[forest->ntrees];
  if (nq > 0 && !d_queries)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_forest_query_nearest: null queries");
  return query_nearest(forest, as_stream(stream), d_queries, nq, h_query_offsets, d_k, k, policy,
                       with_distances, out);
}

// Brute-force point sets from this size on keep a Morton-ordered copy.
constexpr int64_t kBruteMortonMin = 64;

abx_status abx_brute_create(void *stream, abx_geometry kind, const float *d_values, int64_t n,
                            abx_brute **out)
{
  if (!out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_brute_create: null output handle");
  *out = nullptr;
  if (kind != ABX_POINT && kind != ABX_BOX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_brute_create: values must be points or boxes");
  if (n < 0 || n >= (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_brute_create: size out of range [0, 2^31-1)");
  if (n > 0 && !d_values)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_brute_create: null values");
  device_state();
  abx_brute *t = new (std::nothrow) abx_brute;
  if (!t)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_brute_create: host allocation");
  cudaGetDevice(&t->device);
  t->stream = as_stream(stream);
  t->kind = kind;
  t->n = n;
  cudaError_t e = cudaMallocHost(&t->h_bounds, 6 * sizeof(float));
  if (e == cudaSuccess)
    e = cudaEventCreateWithFlags(&t->ready, cudaEventDisableTiming);
  abx_status st = e == cudaSuccess ? ABX_SUCCESS : fail_cuda(e, "abx_brute_create");
  cudaStream_t s = t->stream;
  if (st == ABX_SUCCESS)
  {
    const float empty[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    std::memcpy(t->h_bounds, empty, sizeof(empty));
    if (dmalloc_n(&t->d_bounds, 6, s) != cudaSuccess ||
        (n > 0 && dmalloc_n(&t->sorted, (size_t)n * (kind == ABX_BOX ? 2 : 1), s) != cudaSuccess))
      st = fail(ABX_ERROR_OUT_OF_MEMORY, "abx_brute_create: device allocation");
  }
  if (st == ABX_SUCCESS && n > 0)
  {
    st = scene_bounds(s, kind, d_values, n, t->d_bounds);
    if (st == ABX_SUCCESS)
      st = brute_pack(s, kind, d_values, n, t->sorted);
    if (st == ABX_SUCCESS && kind == ABX_POINT && n >= kBruteMortonMin)
    {
      // the points again in Morton order for the tensor-core filter's
      // coherent scan (nearest); intersects keep the input order
      Scratch<uint32_t> perm, hist;
      if (dmalloc_n(&t->morton_codes, (size_t)n, s) != cudaSuccess ||
          dmalloc_n(&t->morton_sorted, (size_t)n, s) != cudaSuccess ||
          perm.alloc((size_t)n, s) != cudaSuccess || hist.alloc(8 * 256, s) != cudaSuccess)
        st = fail(ABX_ERROR_OUT_OF_MEMORY, "abx_brute_create: device allocation");
      if (st == ABX_SUCCESS && cudaMemsetAsync(hist.ptr, 0, 8 * 256 * sizeof(uint32_t), s) != cudaSuccess)
        st = fail(ABX_ERROR_CUDA, "abx_brute_create: memset");
      if (st == ABX_SUCCESS)
        st = morton64_codes(s, kind, d_values, n, t->d_bounds, t->morton_codes, hist.ptr);
      if (st == ABX_SUCCESS)
        st = radix_sort_u64(s, t->morton_codes, perm.ptr, nullptr, n, 8, hist.ptr,
                            stream_capturing(s) ? 0 : hybrid_top_passes(n, 8));
      if (st == ABX_SUCCESS)
        st = brute_pack_sorted(s, d_values, perm.ptr, n, t->morton_sorted);
    }
    if (st == ABX_SUCCESS &&
        cudaMemcpyAsync(t->h_bounds, t->d_bounds, 6 * sizeof(float), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess)
      st = fail(ABX_ERROR_CUDA, "abx_brute_create: bounds copy");
  }
  if (st == ABX_SUCCESS && cudaEventRecord(t->ready, s) != cudaSuccess)
    st = fail(ABX_ERROR_CUDA, "abx_brute_create: event");
  if (st != ABX_SUCCESS)
  {
    cudaStreamSynchronize(s);
    destroy_tree(t);
    return st;
  }
  *out = t;
  return ABX_SUCCESS;
}

abx_status abx_brute_destroy(abx_brute *brute)
{
  destroy_tree(brute);
  return ABX_SUCCESS;
}

int64_t abx_brute_size(const abx_brute *brute) { return brute ? brute->n : 0; }

abx_status abx_brute_bounds(const abx_brute *brute, float h_box[6])
{
  return abx_bvh_bounds(brute, h_box);
}

abx_status abx_brute_query_intersects(const abx_brute *brute, void *stream, abx_geometry kind,
                                      const float *d_predicates, int64_t nq,
                                      abx_traversal_policy policy, abx_crs **out)
{
  return abx_bvh_query_intersects(brute, stream, kind, d_predicates, nq, policy, out);
}

abx_status abx_brute_query_nearest(const abx_brute *brute, void *stream, const float *d_queries,
                                   int64_t nq, const int32_t *d_k, int32_t k,
                                   abx_traversal_policy policy, int32_t with_distances,
                                   abx_crs **out)
{
  return abx_bvh_query_nearest(brute, stream, d_queries, nq, d_k, k, policy, with_distances, out);
}

abx_status abx_find_neighbor_list(void *stream, const float *d_points, int64_t n, float radius,
                                  int32_t half, abx_crs **out)
{
  if (!out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_find_neighbor_list: null output");
  *out = nullptr;
  if (n < 0 || n >= (int64_t)INT32_MAX || (n > 0 && !d_points))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_find_neighbor_list: bad points");
  cudaStream_t s = as_stream(stream);
  abx_bvh *t = nullptr;
  ABX_TRY(abx_bvh_create(stream, ABX_POINT, d_points, n, &t));
  std::unique_ptr<abx_bvh, void (*)(abx_bvh *)> tree(t, destroy_tree);
  abx_crs *c = new (std::nothrow) abx_crs;
  if (!c)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_crs");
  cudaGetDevice(&c->device);
  c->stream = s;
  c->nq = n;
  auto bail = [&](abx_status st) {
    cudaStreamSynchronize(s);
    destroy_crs(c);
    return st;
  };
  if (dmalloc_n(&c->offsets, n + 1, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS offsets"));
  if (n <= 1)
  {
    cudaMemsetAsync(c->offsets, 0, (n + 1) * sizeof(int32_t), s);
    dmalloc_n(&c->indices, 0, s);
    *out = c;
    return ABX_SUCCESS;
  }
  Scratch<float> spheres;
  Scratch<uint32_t> order;
  Scratch<int32_t> pos;
  if (spheres.alloc(4 * n, s) != cudaSuccess || order.alloc(n, s) != cudaSuccess ||
      pos.alloc(n, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "neighbor list scratch"));
  // queries in the tree's leaf order: Morton-coherent without a sort
  abx_status st = self_spheres(s, d_points, n, radius, spheres.ptr);
  if (st == ABX_SUCCESS)
    st = leaf_order(s, t->kind, t->sorted, n, order.ptr, pos.ptr);
  const TreeView tv = view_of(t);
  const int filter = half ? 2 : 1;
  if (st == ABX_SUCCESS)
    st = launch_spatial_self(s, tv, filter, pos.ptr, spheres.ptr, n, order.ptr, kCount,
                             c->offsets, nullptr, nullptr);
  if (st == ABX_SUCCESS)
    st = exclusive_scan_i32(s, c->offsets, n, c->offsets);
  if (st != ABX_SUCCESS)
    return bail(st);
  int32_t total = 0;
  cudaMemcpyAsync(&total, c->offsets + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  st = sync_and_check(s);
  if (st != ABX_SUCCESS)
    return bail(st);
  if (dmalloc_n(&c->indices, (size_t)total, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS indices"));
  st = launch_spatial_self(s, tv, filter, pos.ptr, spheres.ptr, n, order.ptr, kFill, nullptr,
                           c->offsets, c->indices);
  if (st != ABX_SUCCESS)
    return bail(st);
  c->nres = total;
  *out = c;
  return ABX_SUCCESS;
}

abx_status abx_expand_half_to_full(void *stream, int64_t n, const int32_t *d_offsets,
                                   const int32_t *d_indices, abx_crs **out)
{
  if (!out)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_expand_half_to_full: null output");
  *out = nullptr;
  if (n < 0 || n >= (int64_t)INT32_MAX || !d_offsets)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_expand_half_to_full: bad arguments");
  cudaStream_t s = as_stream(stream);
  device_state();
  int32_t m = 0;
  ABX_CUDA_TRY(cudaMemcpyAsync(&m, d_offsets + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  if (m < 0 || (int64_t)m * 2 >= (int64_t)INT32_MAX || (m > 0 && !d_indices))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_expand_half_to_full: bad half list");
  abx_crs *c = new (std::nothrow) abx_crs;
  if (!c)
    return fail(ABX_ERROR_OUT_OF_MEMORY, "abx_crs");
  cudaGetDevice(&c->device);
  c->stream = s;
  c->nq = n;
  auto bail = [&](abx_status st) {
    cudaStreamSynchronize(s);
    destroy_crs(c);
    return st;
  };
  if (dmalloc_n(&c->offsets, n + 1, s) != cudaSuccess ||
      dmalloc_n(&c->indices, (size_t)m * 2, s) != cudaSuccess)
    return bail(fail(ABX_ERROR_OUT_OF_MEMORY, "CRS"));
  if (n == 0)
    cudaMemsetAsync(c->offsets, 0, sizeof(int32_t), s);
  abx_status st = expand_half_to_full(s, n, d_offsets, d_indices, m, c->offsets, c->indices);
  if (st != ABX_SUCCESS)
    return bail(st);
  c->nres = 2 * (int64_t)m;
  *out = c;
  return ABX_SUCCESS;
}

int64_t abx_crs_num_queries(const abx_crs *crs) { return crs ? crs->nq : 0; }
int64_t abx_crs_num_results(const abx_crs *crs) { return crs ? crs->nres : 0; }
const int32_t *abx_crs_offsets(const abx_crs *crs) { return crs ? crs->offsets : nullptr; }
const int32_t *abx_crs_indices(const abx_crs *crs) { return crs ? crs->indices : nullptr; }
const float *abx_crs_distances(const abx_crs *crs) { return crs ? crs->distances : nullptr; }

abx_status abx_crs_destroy(abx_crs *crs)
{
  destroy_crs(crs);
  return ABX_SUCCESS;
}

abx_status abx_scene_bounds(void *stream, abx_geometry kind, const float *d_values, int64_t n,
                            float *d_box_out)
{
  if (!d_box_out || n < 0 || (n > 0 && !d_values))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_scene_bounds: bad argument");
  return scene_bounds(as_stream(stream), kind, d_values, n, d_box_out);
}

abx_status abx_morton64(void *stream, abx_geometry kind, const float *d_values, int64_t n,
                        const float *d_scene, uint64_t *d_codes)
{
  if (n < 0 || (n > 0 && (!d_values || !d_scene || !d_codes)))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_morton64: bad argument");
  return morton64_codes(as_stream(stream), kind, d_values, n, d_scene, d_codes, nullptr);
}

abx_status abx_morton32(void *stream, abx_geometry kind, const float *d_values, int64_t n,
                        const float *d_scene, uint32_t *d_codes)
{
  if (n < 0 || (n > 0 && (!d_values || !d_scene || !d_codes)))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_morton32: bad argument");
  return morton32_codes(as_stream(stream), kind, d_values, n, d_scene, d_codes, nullptr);
}

abx_status abx_sort_u64(void *stream, uint64_t *d_keys, int64_t n, uint32_t *d_permutation)
{
  if (n < 0 || (n > 0 && (!d_keys || !d_permutation)))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_sort_u64: bad argument");
  device_state();
  return radix_sort_u64(as_stream(stream), d_keys, d_permutation, nullptr, n, 8, nullptr,
                        hybrid_top_passes(n, 8));
}

abx_status abx_sort_u32(void *stream, uint32_t *d_keys, int64_t n, uint32_t *d_permutation)
{
  if (n < 0 || (n > 0 && (!d_keys || !d_permutation)))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_sort_u32: bad argument");
  device_state();
  return radix_sort_u32(as_stream(stream), d_keys, d_permutation, nullptr, n, 4, nullptr,
                        hybrid_top_passes(n, 4));
}

abx_status abx_generate_hierarchy(void *stream, abx_geometry kind, const float *d_values,
                                  int64_t n, const uint32_t *d_permutation,
                                  const uint64_t *d_sorted_codes, int32_t *d_leaves,
                                  void *d_internal)
{
  if (n < 2 || !d_values || !d_permutation || !d_sorted_codes || !d_leaves || !d_internal)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_generate_hierarchy: bad argument");
  if (kind != ABX_POINT && kind != ABX_BOX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_generate_hierarchy: points or boxes");
  device_state();
  return generate_hierarchy(as_stream(stream), kind, d_values, n, d_permutation, d_sorted_codes,
                            reinterpret_cast<LeafNode *>(d_leaves),
                            reinterpret_cast<InternalNode *>(d_internal), nullptr, nullptr);
}

abx_status abx_exclusive_scan_i32(void *stream, const int32_t *d_in, int64_t n, int32_t *d_out)
{
  if (n < 0 || !d_out || (n > 0 && !d_in))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_exclusive_scan_i32: bad argument");
  device_state();
  return exclusive_scan_i32(as_stream(stream), d_in, n, d_out);
}

} // extern "C"
