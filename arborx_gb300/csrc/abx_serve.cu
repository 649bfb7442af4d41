// abx_serve.cu -- request loop over trees resident in HBM (host code).
//
// Requests (nearest(k) or intersects(sphere) batches on one tree) are queued
// by abx_server_submit.  Worker threads, each with its own CUDA stream, take
// the oldest pending request and coalesce every other pending request on the
// same tree and of the same kind into one query launch (mixed k go through
// the per-query k array, mixed radii through the spheres themselves), as
// long as the batch stays under the query cap and the in-flight device
// memory stays under the budget.  Requests that arrive while batches run are
// admitted into the next batch of a free worker: continuous batching, with
// up to `workers` batches overlapping on the device.  A query's result does
// not depend on the batch it ran in (each query is traversed on its own), so
// results alone and in a mix are identical.
//
// There is no counterpart in the reference: it is the serving loop around
// BoundingVolumeHierarchy::query (src/spatial/ArborX_LinearBVH.hpp:90-110).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "abx_internal.h"

namespace
{

using Clock = std::chrono::steady_clock;

struct Request
{
  int64_t ticket = 0;
  int32_t tree = 0;
  int32_t kind = 0;
  int32_t k = 0;
  int64_t nq = 0;
  std::vector<float> queries; // nq rows of 3 (nearest) or 4 (intersects) floats
  Clock::time_point submitted;
  // results
  bool done = false;
  abx_status status = ABX_SUCCESS;
  std::string error;
  std::vector<int32_t> offsets;
  std::vector<int32_t> indices;
  std::vector<float> distances;
  double latency_ms = 0;
  int32_t batch_requests = 0;
};

int row_floats(int32_t kind) { return kind == ABX_REQ_NEAREST ? 3 : 4; }

} // namespace

struct abx_server
{
  abx_server_config cfg{};
  int device = 0;
  std::vector<const abx_bvh *> trees;

  std::mutex mu;
  std::condition_variable cv_work; // workers: pending requests or stop
  std::condition_variable cv_done; // waiters: a request completed
  std::condition_variable cv_mem;  // workers: in-flight memory released
  std::deque<std::shared_ptr<Request>> pending;
  std::map<int64_t, std::shared_ptr<Request>> by_ticket;
  int64_t next_ticket = 1;
  int64_t inflight_bytes = 0;
  int inflight_batches = 0;
  bool stop = false;

  // statistics
  std::vector<double> latencies;
  int64_t completed_queries = 0;
  int64_t batches = 0;
  Clock::time_point first_submit{};
  Clock::time_point last_done{};
  bool any_submit = false;

  std::vector<std::thread> workers;
  // L2 persistence: the context limit before the server raised it
  size_t persist_max = 0;
  size_t persist_old = 0;
  int max_window = 0;
};

namespace
{

// Device bytes a batch holds while it runs: queries, k array, offsets,
// results (nearest: k indices + distances per query; intersects: an estimate
// of 64 hits per query, the CRS arrays being sized by the call itself).
int64_t batch_bytes(std::vector<std::shared_ptr<Request>> const &b)
{
  int64_t bytes = 0;
  for (auto const &r : b)
  {
    const int64_t per = r->kind == ABX_REQ_NEAREST ? 12 + 4 + 4 + 8 * (int64_t)std::max(r->k, 0)
                                                   : 16 + 4 + 4 * 64;
    bytes += r->nq * per;
  }
  return bytes;
}

void complete(abx_server *srv, std::vector<std::shared_ptr<Request>> const &batch, abx_status st,
              std::string const &err)
{
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lock(srv->mu);
  for (auto const &r : batch)
  {
    r->status = st;
    r->error = err;
    r->done = true;
    r->latency_ms = std::chrono::duration<double, std::milli>(now - r->submitted).count();
    r->batch_requests = (int32_t)batch.size();
    if (st == ABX_SUCCESS)
    {
      srv->latencies.push_back(r->latency_ms);
      srv->completed_queries += r->nq;
    }
  }
  srv->batches += 1;
  srv->last_done = now;
  srv->cv_done.notify_all();
}

// Pinned host buffer of a worker, grown on demand and reused across batches.
struct Pinned
{
  void *p = nullptr;
  size_t cap = 0;
  ~Pinned() { cudaFreeHost(p); }
  template <class T>
  T *get(size_t n, cudaError_t &e)
  {
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (bytes > cap)
    {
      cudaFreeHost(p);
      p = nullptr;
      cap = 0;
      e = cudaMallocHost(&p, bytes + bytes / 2);
      if (e != cudaSuccess)
        return nullptr;
      cap = bytes + bytes / 2;
    }
    return static_cast<T *>(p);
  }
};

struct WorkerBuffers
{
  Pinned q, k, off, idx, dist;
};

// Run one coalesced batch on the worker's stream.
abx_status run_batch(abx_server *srv, cudaStream_t s, WorkerBuffers &wb,
                     std::vector<std::shared_ptr<Request>> &batch, std::string &err)
{
  const abx_bvh *tree = srv->trees[batch[0]->tree];
  const int32_t kind = batch[0]->kind;
  const int rf = row_floats(kind);
  int64_t nq = 0;
  bool same_k = true;
  for (auto const &r : batch)
  {
    nq += r->nq;
    same_k = same_k && r->k == batch[0]->k;
  }
  // pinned staging of the concatenated queries (and per-query k)
  float *h_q = nullptr;
  int32_t *h_k = nullptr;
  float *d_q = nullptr;
  int32_t *d_k = nullptr;
  abx_crs *crs = nullptr;
  int32_t *h_off = nullptr;
  int32_t *h_idx = nullptr;
  float *h_dist = nullptr;
  abx_status st = ABX_SUCCESS;
  auto cuda_fail = [&](cudaError_t e, const char *what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return ABX_ERROR_CUDA;
  };
  do
  {
    cudaError_t e = cudaSuccess;
    h_q = wb.q.get<float>(nq * rf, e);
    if (e != cudaSuccess)
    {
      st = cuda_fail(e, "cudaMallocHost");
      break;
    }
    int64_t q0 = 0;
    for (auto const &r : batch)
    {
      std::memcpy(h_q + q0 * rf, r->queries.data(), r->nq * rf * sizeof(float));
      q0 += r->nq;
    }
    e = cudaMallocAsync(reinterpret_cast<void **>(&d_q), std::max<int64_t>(nq, 1) * rf * sizeof(float), s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_q, h_q, nq * rf * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess)
    {
      st = cuda_fail(e, "queries to device");
      break;
    }
    if (kind == ABX_REQ_NEAREST && !same_k)
    {
      h_k = wb.k.get<int32_t>(nq, e);
      if (e == cudaSuccess)
      {
        int64_t q = 0;
        for (auto const &r : batch)
          for (int64_t j = 0; j < r->nq; ++j)
            h_k[q++] = r->k;
        e = cudaMallocAsync(reinterpret_cast<void **>(&d_k), nq * sizeof(int32_t), s);
      }
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_k, h_k, nq * sizeof(int32_t), cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess)
      {
        st = cuda_fail(e, "k to device");
        break;
      }
    }
    if (srv->persist_max > 0)
    {
      // keep this tree's nodes in L2 against the streaming queries and results
      const void *base = nullptr;
      size_t bytes = 0;
      abx::tree_node_memory(tree, &base, &bytes);
      cudaStreamAttrValue attr = {};
      attr.accessPolicyWindow.base_ptr = const_cast<void *>(base);
      attr.accessPolicyWindow.num_bytes = std::min<size_t>(bytes, (size_t)srv->max_window);
      attr.accessPolicyWindow.hitRatio =
          attr.accessPolicyWindow.num_bytes
              ? (float)std::min(1.0, (double)srv->persist_max /
                                         (double)attr.accessPolicyWindow.num_bytes)
              : 0.f;
      attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
      attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
      cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &attr);
    }
    abx_traversal_policy policy{0, 1};
    if (kind == ABX_REQ_NEAREST)
      st = abx_bvh_query_nearest(tree, s, d_q, nq, d_k, batch[0]->k, policy, 1, &crs);
    else
      st = abx_bvh_query_intersects(tree, s, ABX_SPHERE, d_q, nq, policy, &crs);
    if (st != ABX_SUCCESS)
    {
      err = abx_last_error();
      break;
    }
    const int64_t nres = abx_crs_num_results(crs);
    h_off = wb.off.get<int32_t>(nq + 1, e);
    if (e == cudaSuccess)
      h_idx = wb.idx.get<int32_t>(nres, e);
    if (e == cudaSuccess && kind == ABX_REQ_NEAREST)
      h_dist = wb.dist.get<float>(nres, e);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_off, abx_crs_offsets(crs), (nq + 1) * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && nres)
      e = cudaMemcpyAsync(h_idx, abx_crs_indices(crs), nres * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && nres && h_dist)
      e = cudaMemcpyAsync(h_dist, abx_crs_distances(crs), nres * sizeof(float),
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
    {
      st = cuda_fail(e, "results to host");
      break;
    }
    uint32_t bits = 0;
    st = abx_device_errors(s, &bits);
    if (st == ABX_SUCCESS && bits)
    {
      st = ABX_ERROR_DEVICE;
      err = "device error word " + std::to_string(bits);
    }
    if (st != ABX_SUCCESS)
      break;
    // split per request, offsets rebased to the request's first result
    q0 = 0;
    for (auto const &r : batch)
    {
      const int32_t base = h_off[q0];
      const int32_t end = h_off[q0 + r->nq];
      r->offsets.resize(r->nq + 1);
      for (int64_t j = 0; j <= r->nq; ++j)
        r->offsets[j] = h_off[q0 + j] - base;
      r->indices.assign(h_idx + base, h_idx + end);
      if (h_dist)
        r->distances.assign(h_dist + base, h_dist + end);
      q0 += r->nq;
    }
  } while (false);
  if (crs)
    abx_crs_destroy(crs);
  if (d_q)
    cudaFreeAsync(d_q, s);
  if (d_k)
    cudaFreeAsync(d_k, s);
  cudaStreamSynchronize(s);
  return st;
}

// Take the oldest pending request and every pending request on the same tree
// and of the same kind, up to the query cap (the oldest always fits).
std::vector<std::shared_ptr<Request>> form_batch(abx_server *srv)
{
  std::vector<std::shared_ptr<Request>> batch;
  const auto head = srv->pending.front();
  int64_t nq = 0;
  for (auto it = srv->pending.begin(); it != srv->pending.end();)
  {
    auto const &r = *it;
    const bool same = r->tree == head->tree && r->kind == head->kind;
    if (same && (batch.empty() || nq + r->nq <= srv->cfg.max_batch_queries))
    {
      nq += r->nq;
      batch.push_back(r);
      it = srv->pending.erase(it);
    }
    else
      ++it;
  }
  return batch;
}

void worker_loop(abx_server *srv)
{
  cudaSetDevice(srv->device);
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  WorkerBuffers wb;
  while (true)
  {
    std::vector<std::shared_ptr<Request>> batch;
    int64_t bytes = 0;
    {
      std::unique_lock<std::mutex> lock(srv->mu);
      srv->cv_work.wait(lock, [&] { return srv->stop || !srv->pending.empty(); });
      if (srv->stop && srv->pending.empty())
        break;
      batch = form_batch(srv);
      bytes = batch_bytes(batch);
      // admission by memory: wait while other batches hold the budget (a
      // batch alone is always admitted)
      srv->cv_mem.wait(lock, [&] {
        return srv->inflight_batches == 0 ||
               srv->inflight_bytes + bytes <= srv->cfg.max_inflight_bytes;
      });
      srv->inflight_bytes += bytes;
      srv->inflight_batches += 1;
      if (!srv->pending.empty())
        srv->cv_work.notify_one();
    }
    std::string err;
    const abx_status st = run_batch(srv, s, wb, batch, err);
    {
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->inflight_bytes -= bytes;
      srv->inflight_batches -= 1;
    }
    srv->cv_mem.notify_all();
    complete(srv, batch, st, err);
  }
  cudaStreamDestroy(s);
}

double percentile(std::vector<double> v, double q)
{
  if (v.empty())
    return 0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

} // namespace

extern "C" {

abx_status abx_server_create(const abx_server_config *cfg, abx_server **out)
{
  if (!out)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_create: null output");
  *out = nullptr;
  abx_server_config c{4, 0, (int64_t)8 << 30, 1 << 20};
  if (cfg)
    c = *cfg;
  if (c.workers < 1 || c.workers > 64 || c.max_inflight_bytes <= 0 || c.max_batch_queries < 1)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_create: bad configuration");
  abx_server *srv = new (std::nothrow) abx_server;
  if (!srv)
    return abx::fail(ABX_ERROR_OUT_OF_MEMORY, "abx_server_create");
  srv->cfg = c;
  cudaGetDevice(&srv->device);
  abx::device_state();
  if (c.l2_persist)
  {
    int max_persist = 0, max_window = 0;
    cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, srv->device);
    cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, srv->device);
    size_t old = 0;
    if (max_persist > 0 && max_window > 0 &&
        cudaDeviceGetLimit(&old, cudaLimitPersistingL2CacheSize) == cudaSuccess &&
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)max_persist) == cudaSuccess)
    {
      srv->persist_old = old;
      srv->persist_max = (size_t)max_persist;
      srv->max_window = max_window;
    }
  }
  try
  {
    for (int w = 0; w < c.workers; ++w)
      srv->workers.emplace_back(worker_loop, srv);
  }
  catch (...)
  {
    {
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (auto &t : srv->workers)
      t.join();
    delete srv;
    return abx::fail(ABX_ERROR_OUT_OF_MEMORY, "abx_server_create: worker threads");
  }
  *out = srv;
  return ABX_SUCCESS;
}

abx_status abx_server_destroy(abx_server *srv)
{
  if (!srv)
    return ABX_SUCCESS;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  srv->cv_mem.notify_all();
  for (auto &t : srv->workers)
    t.join();
  if (srv->persist_max > 0)
  {
    // give the persisting lines back and restore the context's limit
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, srv->persist_old);
  }
  delete srv;
  return ABX_SUCCESS;
}

abx_status abx_server_add_tree(abx_server *srv, const abx_bvh *tree, int32_t *tree_id)
{
  if (!srv || !tree || !tree_id)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_add_tree: null argument");
  std::lock_guard<std::mutex> lock(srv->mu);
  *tree_id = (int32_t)srv->trees.size();
  srv->trees.push_back(tree);
  return ABX_SUCCESS;
}

abx_status abx_server_submit(abx_server *srv, const abx_request *req, int64_t *ticket)
{
  if (!srv || !req || !ticket)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_submit: null argument");
  if (req->kind != ABX_REQ_NEAREST && req->kind != ABX_REQ_INTERSECTS)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_submit: bad request kind");
  if (req->nq < 0 || req->nq >= (int64_t)INT32_MAX || (req->nq > 0 && !req->h_queries))
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_submit: bad queries");
  auto r = std::make_shared<Request>();
  r->tree = req->tree;
  r->kind = req->kind;
  r->k = req->k;
  r->nq = req->nq;
  r->queries.assign(req->h_queries, req->h_queries + req->nq * row_floats(req->kind));
  std::lock_guard<std::mutex> lock(srv->mu);
  if (req->tree < 0 || req->tree >= (int32_t)srv->trees.size())
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_submit: unknown tree");
  r->ticket = srv->next_ticket++;
  r->submitted = Clock::now();
  if (!srv->any_submit)
  {
    srv->first_submit = r->submitted;
    srv->any_submit = true;
  }
  srv->by_ticket[r->ticket] = r;
  srv->pending.push_back(r);
  *ticket = r->ticket;
  srv->cv_work.notify_one();
  return ABX_SUCCESS;
}

abx_status abx_server_wait(abx_server *srv, int64_t ticket, int64_t *num_results,
                           double *latency_ms)
{
  if (!srv)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_wait: null server");
  std::unique_lock<std::mutex> lock(srv->mu);
  auto it = srv->by_ticket.find(ticket);
  if (it == srv->by_ticket.end())
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_wait: unknown ticket");
  auto r = it->second;
  srv->cv_done.wait(lock, [&] { return r->done; });
  if (r->status != ABX_SUCCESS)
    return abx::fail(r->status, r->error);
  if (num_results)
    *num_results = (int64_t)r->indices.size();
  if (latency_ms)
    *latency_ms = r->latency_ms;
  return ABX_SUCCESS;
}

abx_status abx_server_result(abx_server *srv, int64_t ticket, int32_t *h_offsets,
                             int32_t *h_indices, float *h_distances)
{
  if (!srv)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_result: null server");
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->by_ticket.find(ticket);
    if (it == srv->by_ticket.end())
      return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_result: unknown ticket");
    r = it->second;
    srv->cv_done.wait(lock, [&] { return r->done; });
    srv->by_ticket.erase(it);
  }
  if (r->status != ABX_SUCCESS)
    return abx::fail(r->status, r->error);
  if (h_offsets)
    std::memcpy(h_offsets, r->offsets.data(), r->offsets.size() * sizeof(int32_t));
  if (h_indices && !r->indices.empty())
    std::memcpy(h_indices, r->indices.data(), r->indices.size() * sizeof(int32_t));
  if (h_distances && !r->distances.empty())
    std::memcpy(h_distances, r->distances.data(), r->distances.size() * sizeof(float));
  return ABX_SUCCESS;
}

abx_status abx_server_stats(abx_server *srv, abx_server_statistics *out)
{
  if (!srv || !out)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_stats: null argument");
  std::lock_guard<std::mutex> lock(srv->mu);
  out->completed_requests = (int64_t)srv->latencies.size();
  out->completed_queries = srv->completed_queries;
  out->batches = srv->batches;
  out->p50_ms = percentile(srv->latencies, 0.50);
  out->p99_ms = percentile(srv->latencies, 0.99);
  out->span_s = srv->any_submit
                    ? std::chrono::duration<double>(srv->last_done - srv->first_submit).count()
                    : 0.0;
  return ABX_SUCCESS;
}

abx_status abx_server_reset_stats(abx_server *srv)
{
  if (!srv)
    return abx::fail(ABX_ERROR_INVALID_ARGUMENT, "abx_server_reset_stats: null server");
  std::lock_guard<std::mutex> lock(srv->mu);
  srv->latencies.clear();
  srv->completed_queries = 0;
  srv->batches = 0;
  srv->any_submit = false;
  return ABX_SUCCESS;
}

} // extern "C"
