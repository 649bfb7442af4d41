// abx_internal.h -- host-side internals shared by the library's translation
// units: per-device state, stream-ordered scratch allocation, error plumbing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/arborx_gb300.h"

namespace abx
{

struct DeviceState
{
  int device = -1;
  int num_sms = 0;
  unsigned *d_error = nullptr; // device error word (ABX_DEVERR_* bits)
};

// State of the current device, initialised on first use (thread-safe).
DeviceState &device_state();

// Record a failure message for abx_last_error() and return `status`.
abx_status fail(abx_status status, std::string const &message);
abx_status fail_cuda(cudaError_t err, char const *what);

// Stream-ordered device allocation from the device's default memory pool.
cudaError_t dmalloc(void **p, size_t bytes, cudaStream_t s);
void dfree(void *p, cudaStream_t s);

template <class T>
cudaError_t dmalloc_n(T **p, size_t count, cudaStream_t s)
{
  return dmalloc(reinterpret_cast<void **>(p), count * sizeof(T) + (count == 0 ? 16 : 0),
                 s);
}

// Scoped stream-ordered scratch buffer.
template <class T>
struct Scratch
{
  T *ptr = nullptr;
  cudaStream_t stream = nullptr;
  Scratch() = default;
  Scratch(Scratch const &) = delete;
  Scratch &operator=(Scratch const &) = delete;
  cudaError_t alloc(size_t count, cudaStream_t s)
  {
    stream = s;
    return dmalloc_n(&ptr, count, s);
  }
  ~Scratch()
  {
    if (ptr)
      dfree(ptr, stream);
  }
  T *release()
  {
    T *p = ptr;
    ptr = nullptr;
    return p;
  }
};

#define ABX_CUDA_TRY(expr)                                                      \
  do                                                                            \
  {                                                                             \
    cudaError_t abx_e_ = (expr);                                                \
    if (abx_e_ != cudaSuccess)                                                  \
      return ::abx::fail_cuda(abx_e_, #expr);                                   \
  } while (0)

#define ABX_TRY(expr)                                                           \
  do                                                                            \
  {                                                                             \
    abx_status abx_s_ = (expr);                                                 \
    if (abx_s_ != ABX_SUCCESS)                                                  \
      return abx_s_;                                                            \
  } while (0)

// Tuning knob `name` (kernel variant, launch shape): the value set through
// abx_tuning_set, else the environment variable ABX_TUNE_<name>, else `def`.
int tuning_value(char const *name, int def);

// Records a CUDA event pair around a kernel stage while profiling is enabled
// (abx_profiling_enable); `kernels` is the number of launches in the stage.
class StageScope
{
public:
  StageScope(cudaStream_t s, char const *stage, int kernels);
  ~StageScope();
  StageScope(StageScope const &) = delete;
  StageScope &operator=(StageScope const &) = delete;
  void add_kernels(int k) { kernels_ += k; }

private:
  cudaStream_t stream_;
  char const *stage_;
  int kernels_;
  cudaEvent_t start_ = nullptr;
};

// ---------------------------------------------------------------------------
// Kernels exposed across translation units (host launchers)
// ---------------------------------------------------------------------------

// Stable LSD radix sort of (key, value) pairs with one onesweep pass per
// 8-bit digit.  If d_hist is null the digit histograms are computed first;
// otherwise d_hist holds num_passes x 256 counts (e.g. produced by the
// Morton kernel).  When d_vals_in is null, the values start as 0..n-1.
// On return the sorted keys and values are in d_keys / d_vals.
//
// top_passes > 0 (and < num_passes): only the top `top_passes` digits are
// sorted by passes; a fix-up kernel then orders every run of equal top digits
// (stable, exact), runs longer than kRunMax through a segmented sort of just
// their elements.  Same result as the full sort, fewer passes over memory
// when the top digits already spread the keys (Morton codes of n points with
// n << 2^(8 top_passes)).  This variant synchronises the stream once.
abx_status radix_sort_u64(cudaStream_t s, uint64_t *d_keys, uint32_t *d_vals,
                          const uint32_t *d_vals_in, int64_t n, int num_passes,
                          const uint32_t *d_hist, int top_passes = 0);
// Stable order of n u32 keys by their top `top` of num_passes 8-bit digits
// only (keys equal there keep their input order): d_perm receives the
// permutation; d_keys is clobbered.  An ordering for coherence, not a sort.
abx_status radix_order_top_u32(cudaStream_t s, uint32_t *d_keys, uint32_t *d_perm, int64_t n,
                               int num_passes, const uint32_t *d_hist, int top);
abx_status radix_sort_u32(cudaStream_t s, uint32_t *d_keys, uint32_t *d_vals,
                          const uint32_t *d_vals_in, int64_t n, int num_passes,
                          const uint32_t *d_hist, int top_passes = 0);

// The child-pair node array of a tree (pointer and bytes).
void tree_node_memory(const abx_bvh *t, const void **ptr, size_t *bytes);

// Kernel attributes of the sort, set once per device by device_state().
abx_status init_sort_kernels();

// True when s is capturing a CUDA graph (no host synchronisation allowed).
bool stream_capturing(cudaStream_t s);

// Number of top passes of the hybrid sort for n keys of num_passes digits
// (0 = plain LSD).
int hybrid_top_passes(int64_t n, int num_passes);

// Top passes of a Morton64 code sort from the device digit histograms
// (reads them back: synchronises s).
int top_passes_from_hist(cudaStream_t s, const uint32_t *d_hist, int64_t n);

// Top passes chosen from the digit histograms (host copy, num_passes x 256)
// of the keys: 3 or 4 when runs of equal top digits stay short, else 0.
int choose_top_passes(const uint32_t *h_hist, int64_t n, int num_passes);

// Exclusive scan of n int32 into n + 1 outputs; *d_total_out (optional,
// device int64) receives the 64-bit total.  Raises ABX_DEVERR_BAD_INPUT when
// the total does not fit in int32.
abx_status exclusive_scan_i32(cudaStream_t s, const int32_t *d_in, int64_t n,
                              int32_t *d_out);

} // namespace abx
