// abx_sort.cu -- stable LSD radix sort of (key, uint32 value) pairs, one
// onesweep pass per 8-bit digit (decoupled look-back over per-digit tile
// prefixes), plus the digit histogram and small scan kernels.
//
// Replaces sortByKey / sortObjects (src/kokkos_ext/ArborX_KokkosExtSort.hpp:
// 79-148, src/misc/ArborX_SortUtils.hpp:28-39), which call thrust::sort_by_key
// on CUDA.  The order of equal keys is fixed here: stable (input order).
//
// Pass structure (per tile of 4096 keys, one CTA of 256 threads):
//   1. load 16 keys per thread in warp-striped order (coalesced);
//   2. rank every key among the equal digits of its warp with match_any,
//      keeping a per-warp 256-bin histogram in shared memory;
//   3. turn the warp histograms into per-digit tile offsets;
//   4. publish the tile's 256 digit counts, look back over earlier tiles to
//      get each digit's exclusive prefix (bounded spin, error word on
//      timeout), publish the inclusive prefix;
//   5. scatter the tile into shared memory in digit order, then write it out
//      so that equal-digit runs land on consecutive global addresses.
#include <algorithm>
#include <mutex>

#include "abx_common.cuh"
#include "abx_internal.h"

namespace abx
{
namespace
{

constexpr int kBins = 256;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kSortThreads * kItems;
constexpr int kMaxPasses = 8;
constexpr int kSpinLimit = 1 << 22;

template <class K>
__device__ __forceinline__ unsigned digit_of(K key, int shift)
{
  return (unsigned)(key >> shift) & 0xffu;
}

// Per-pass digit histograms of all keys (hist: passes x 256, zeroed).
template <class K>
__global__ void __launch_bounds__(256) k_histogram(const K *__restrict__ keys, int64_t n,
                                                   int num_passes,
                                                   uint32_t *__restrict__ hist)
{
  __shared__ uint32_t sh[kMaxPasses * kBins];
  for (int i = threadIdx.x; i < num_passes * kBins; i += blockDim.x)
    sh[i] = 0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    K k = keys[i];
    for (int p = 0; p < num_passes; ++p)
      atomicAdd(&sh[p * kBins + digit_of(k, 8 * p)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < num_passes * kBins; i += blockDim.x)
    if (sh[i])
      atomicAdd(&hist[i], sh[i]);
}

// offsets[p][d] = sum of hist[p][d'] for d' < d.  One CTA of 256 per pass.
__global__ void __launch_bounds__(256) k_hist_scan(const uint32_t *__restrict__ hist,
                                                   uint32_t *__restrict__ offsets)
{
  __shared__ uint32_t warp_sums[kSortWarps];
  int t = threadIdx.x;
  uint32_t v = hist[blockIdx.x * kBins + t];
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if ((t & 31) >= o)
      x += y;
  }
  if ((t & 31) == 31)
    warp_sums[t >> 5] = x;
  __syncthreads();
  uint32_t pre = 0;
  for (int w = 0; w < (t >> 5); ++w)
    pre += warp_sums[w];
  offsets[blockIdx.x * kBins + t] = pre + x - v;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v)
{
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <class K>
struct PassSmem
{
  union
  {
    uint32_t whist[kSortWarps][kBins + 1];
    struct
    {
      K keys[kTile];
      uint32_t vals[kTile];
    } exch;
  } u;
  uint32_t digit_start[kBins + 1];
  uint32_t gbase[kBins];
  uint32_t warp_tot[kSortWarps];
  uint32_t tile;
};

// One onesweep pass.  Look-back words: (tag << 32) | count with
// tag = 2 (pass + 1) for a tile aggregate and 2 (pass + 1) + 1 for an
// inclusive prefix; words of earlier passes read as "not ready", so one
// buffer (zeroed once per sort) serves every pass.
template <class K>
__global__ void __launch_bounds__(kSortThreads, 3)
    k_onesweep(const K *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
               K *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int64_t n,
               int shift, int pass, const uint32_t *__restrict__ goffsets,
               unsigned long long *__restrict__ lookback, unsigned *__restrict__ tile_counter,
               unsigned *__restrict__ err)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassSmem<K> &sm = *reinterpret_cast<PassSmem<K> *>(smem_raw);
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;

  if (tid == 0)
    sm.tile = atomicAdd(tile_counter, 1u);
  for (int i = tid; i < kSortWarps * (kBins + 1); i += kSortThreads)
    (&sm.u.whist[0][0])[i] = 0;
  __syncthreads();
  const unsigned tile = sm.tile;
  const int64_t tile_base = (int64_t)tile * kTile;

  // 1. load
  K key[kItems];
  uint32_t val[kItems];
  const int64_t warp_base = tile_base + (int64_t)warp * 32 * kItems + lane;
#pragma unroll
  for (int j = 0; j < kItems; ++j)
  {
    int64_t idx = warp_base + j * 32;
    if (idx < n)
    {
      key[j] = keys_in[idx];
      val[j] = vals_in ? vals_in[idx] : (uint32_t)idx;
    }
    else
    {
      key[j] = 0;
      val[j] = 0;
    }
  }

  // 2. warp-level stable ranking; dr[j] = digit << 16 | rank in the warp
  uint32_t dr[kItems];
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int j = 0; j < kItems; ++j)
  {
    int64_t idx = warp_base + j * 32;
    unsigned d = idx < n ? digit_of(key[j], shift) : (unsigned)kBins;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader)
    {
      base = sm.u.whist[warp][d];
      sm.u.whist[warp][d] = base + __popc(peers);
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    dr[j] = (d << 16) | (base + __popc(peers & lt));
    __syncwarp();
  }
  __syncthreads();

  // 3. per-digit warp offsets and tile totals; exclusive scan over digits
  uint32_t total = 0;
  {
    int d = tid;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w)
    {
      uint32_t c = sm.u.whist[w][d];
      sm.u.whist[w][d] = total;
      total += c;
    }
    if (tid == 0)
    {
      uint32_t s = 0;
      for (int w = 0; w < kSortWarps; ++w)
      {
        uint32_t c = sm.u.whist[w][kBins];
        sm.u.whist[w][kBins] = s;
        s += c;
      }
    }
    uint32_t x = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o)
        x += y;
    }
    if (lane == 31)
      sm.warp_tot[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; ++w)
      pre += sm.warp_tot[w];
    sm.digit_start[d] = pre + x - total;
    if (tid == kSortThreads - 1)
      sm.digit_start[kBins] = pre + x;
  }
  __syncthreads();

#pragma unroll
  for (int j = 0; j < kItems; ++j)
  {
    const unsigned d = dr[j] >> 16;
    dr[j] = sm.digit_start[d] + sm.u.whist[warp][d] + (dr[j] & 0xffffu); // tile position
  }

  // 4. decoupled look-back, one digit per thread
  {
    const int d = tid;
    const unsigned long long tag_agg = 2ull * (pass + 1);
    const unsigned long long tag_inc = tag_agg + 1;
    unsigned long long *row = lookback + (size_t)tile * kBins;
    uint32_t excl = 0;
    if (tile == 0)
    {
      st_relaxed_u64(&row[d], (tag_inc << 32) | total);
    }
    else
    {
      st_relaxed_u64(&row[d], (tag_agg << 32) | total);
      int64_t pred = (int64_t)tile - 1;
      int spins = 0;
      while (pred >= 0)
      {
        unsigned long long v = ld_relaxed_u64(lookback + (size_t)pred * kBins + d);
        unsigned long long tag = v >> 32;
        if (tag < tag_agg)
        {
          if (++spins > kSpinLimit)
          {
            raise_error(err, ABX_DEVERR_TIMEOUT);
            break;
          }
          continue;
        }
        excl += (uint32_t)v;
        if (tag == tag_inc)
          break;
        --pred;
      }
      st_relaxed_u64(&row[d], (tag_inc << 32) | (unsigned long long)(excl + total));
    }
    sm.gbase[d] = goffsets[d] + excl;
  }
  __syncthreads();

  // 5. local scatter in digit order, then coalesced global write
#pragma unroll
  for (int j = 0; j < kItems; ++j)
  {
    sm.u.exch.keys[dr[j]] = key[j];
    sm.u.exch.vals[dr[j]] = val[j];
  }
  __syncthreads();
  const uint32_t valid = sm.digit_start[kBins];
  for (uint32_t i = tid; i < valid; i += kSortThreads)
  {
    K k = sm.u.exch.keys[i];
    unsigned d = digit_of(k, shift);
    uint32_t g = sm.gbase[d] + (i - sm.digit_start[d]);
    if (g < n)
    {
      keys_out[g] = k;
      vals_out[g] = sm.u.exch.vals[i];
    }
    else
      raise_error(err, ABX_DEVERR_INTERNAL);
  }
}

// ---------------------------------------------------------------------------
// Run fix-up of the hybrid sort
// ---------------------------------------------------------------------------

constexpr int kRunMax = 32;

// Bounds [a, b) of the run of equal top bits (key >> shift) around i, the
// scan stopping once the run is known to exceed kRunMax.
template <class K>
__device__ __forceinline__ void run_bounds(const K *__restrict__ keys, int64_t n, int64_t i,
                                           K top, int shift, int64_t &a, int64_t &b)
{
  a = i;
  while (a > 0 && i - a <= kRunMax && (keys[a - 1] >> shift) == top)
    --a;
  b = i + 1;
  while (b < n && b - a <= kRunMax && (keys[b] >> shift) == top)
    ++b;
}

// Keys sorted (stably) by their top bits: place every key of a run of at
// most kRunMax equal top-bit keys at its rank by (key, position), which is the
// stable order; keys of longer runs are copied in place and counted.  A CTA
// stages its keys with a halo of kFixHalo on each side in shared memory,
// with the top bits (key >> shift, shift >= 8, so never all ones) and two
// all-ones sentinels past both ends of the array.
constexpr int kFixThreads = 256;
constexpr int kFixHalo = kRunMax + 2;

template <class K>
__global__ void __launch_bounds__(kFixThreads)
    k_run_fixup(const K *__restrict__ kin, const uint32_t *__restrict__ vin, K *__restrict__ kout,
                uint32_t *__restrict__ vout, int64_t n, int shift,
                unsigned long long *__restrict__ long_count)
{
  constexpr int kSpan = kFixThreads + 2 * kFixHalo;
  __shared__ K s_key[kSpan];
  __shared__ K s_top[kSpan];
  const int64_t b = (int64_t)blockIdx.x * kFixThreads;
  for (int j = threadIdx.x; j < kSpan; j += kFixThreads)
  {
    const int64_t g = b - kFixHalo + j;
    const bool in = g >= 0 && g < n;
    const K k = in ? kin[g] : (K)0;
    s_key[j] = k;
    // a top is below 2^(bits - 8); the sentinels differ from it and each other
    s_top[j] = in ? (K)(k >> shift) : (g < 0 ? ~(K)0 : ~(K)1);
  }
  __syncthreads();
  const int64_t i = b + threadIdx.x;
  bool is_long = false;
  if (i < n)
  {
    const int li = threadIdx.x + kFixHalo;
    const K top = s_top[li];
    int a = li;
    while (li - a <= kRunMax && s_top[a - 1] == top)
      --a;
    int e = li + 1;
    while (e - a <= kRunMax && s_top[e] == top)
      ++e;
    const K k = s_key[li];
    int64_t r = i;
    if (e - a > kRunMax)
      is_long = true;
    else
    {
      int rank = a;
      for (int j = a; j < e; ++j)
      {
        const K kj = s_key[j];
        rank += (kj < k) || (kj == k && j < li);
      }
      r = b - kFixHalo + rank;
    }
    kout[r] = k;
    vout[r] = vin[i];
  }
  const unsigned ballot = __ballot_sync(0xffffffffu, is_long);
  if (ballot && (threadIdx.x & 31) == (unsigned)(__ffs(ballot) - 1))
    atomicAdd(long_count, (unsigned long long)__popc(ballot));
}

// Flags of the keys in long runs, and of the first key of each long run.
template <class K>
__global__ void __launch_bounds__(256)
    k_long_flags(const K *__restrict__ kin, int64_t n, int shift, int32_t *__restrict__ is_long,
                 int32_t *__restrict__ is_start)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const K top = kin[i] >> shift;
  int64_t a, b;
  run_bounds(kin, n, i, top, shift, a, b);
  const bool lg = b - a > kRunMax;
  is_long[i] = lg;
  is_start[i] = lg && (i == 0 || (kin[i - 1] >> shift) != top);
}

// Compact the long-run keys: composite key (run index above the low bits)
// and their positions.
template <class K>
__global__ void __launch_bounds__(256)
    k_long_compact(const K *__restrict__ kin, int64_t n, int shift,
                   const int32_t *__restrict__ is_long, const int32_t *__restrict__ long_pos,
                   const int32_t *__restrict__ is_start, const int32_t *__restrict__ run_excl,
                   K *__restrict__ ckeys, uint32_t *__restrict__ cpos)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !is_long[i])
    return;
  const int64_t c = long_pos[i];
  const K run = (K)(run_excl[i] + is_start[i] - 1);
  const K low = kin[i] & (((K)1 << shift) - 1);
  ckeys[c] = (run << shift) | low;
  cpos[c] = (uint32_t)i;
}

// Position c of the long-run list receives the key ranked c-th.
template <class K>
__global__ void __launch_bounds__(256)
    k_long_gather(const K *__restrict__ kin, const uint32_t *__restrict__ vin,
                  K *__restrict__ kout, uint32_t *__restrict__ vout,
                  const uint32_t *__restrict__ cpos, const uint32_t *__restrict__ cperm, int64_t m)
{
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m)
    return;
  const uint32_t src = cpos[cperm[c]];
  const uint32_t dst = cpos[c];
  kout[dst] = kin[src];
  vout[dst] = vin[src];
}

// The passes of digits [first, num_passes) (LSD order), from (d_keys,
// d_vals_in or the identity) to *kin_out / *vin_out, which are d_keys / d_vals
// or the alternate buffers.  Returns the number of kernels launched in
// *launches.
template <class K>
abx_status sort_passes(cudaStream_t s, K *d_keys, uint32_t *d_vals, const uint32_t *d_vals_in,
                       int64_t n, int first, int num_passes, const uint32_t *d_hist,
                       K *keys_alt, uint32_t *vals_alt, const K **kin_out,
                       const uint32_t **vin_out, int &launches)
{
  DeviceState &ds = device_state();
  const int64_t num_tiles = (n + kTile - 1) / kTile;

  // scratch: [hist passes*256][offsets passes*256][counters 8] lookback
  const size_t lookback_words = (size_t)num_tiles * kBins;
  const size_t head_u32 = 2 * kMaxPasses * kBins + kMaxPasses;
  const size_t head_bytes = (head_u32 * 4 + 255) / 256 * 256;
  Scratch<unsigned char> work;
  ABX_CUDA_TRY(work.alloc(head_bytes + lookback_words * 8, s));
  uint32_t *hist = reinterpret_cast<uint32_t *>(work.ptr);
  uint32_t *offsets = hist + kMaxPasses * kBins;
  unsigned *counters = offsets + kMaxPasses * kBins;
  unsigned long long *lookback = reinterpret_cast<unsigned long long *>(work.ptr + head_bytes);
  ABX_CUDA_TRY(cudaMemsetAsync(work.ptr, 0, head_bytes + lookback_words * 8, s));

  const uint32_t *hsrc = d_hist;
  if (!hsrc)
  {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ds.num_sms * 8);
    k_histogram<K><<<blocks, 256, 0, s>>>(d_keys, n, num_passes, hist);
    hsrc = hist;
    ++launches;
  }
  k_hist_scan<<<num_passes, kBins, 0, s>>>(hsrc, offsets);
  ++launches;

  const size_t smem = sizeof(PassSmem<K>);

  const K *kin = d_keys;
  const uint32_t *vin = d_vals_in;
  K *kout = keys_alt;
  uint32_t *vout = vals_alt;
  for (int p = first; p < num_passes; ++p)
  {
    k_onesweep<K><<<(unsigned)num_tiles, kSortThreads, smem, s>>>(
        kin, vin, kout, vout, n, 8 * p, p, offsets + p * kBins, lookback, counters + p,
        ds.d_error);
    ABX_CUDA_TRY(cudaGetLastError());
    ++launches;
    const K *nk = kout;
    const uint32_t *nv = vout;
    kout = (kout == keys_alt) ? d_keys : keys_alt;
    vout = (vout == vals_alt) ? d_vals : vals_alt;
    kin = nk;
    vin = nv;
  }
  *kin_out = kin;
  *vin_out = vin;
  return ABX_SUCCESS;
}

template <class K>
abx_status radix_sort_full(cudaStream_t s, K *d_keys, uint32_t *d_vals,
                           const uint32_t *d_vals_in, int64_t n, int num_passes,
                           const uint32_t *d_hist, int &launches)
{
  Scratch<K> keys_alt;
  Scratch<uint32_t> vals_alt;
  ABX_CUDA_TRY(keys_alt.alloc(n, s));
  ABX_CUDA_TRY(vals_alt.alloc(n, s));
  const K *kin;
  const uint32_t *vin;
  ABX_TRY(sort_passes<K>(s, d_keys, d_vals, d_vals_in, n, 0, num_passes, d_hist, keys_alt.ptr,
                         vals_alt.ptr, &kin, &vin, launches));
  if (kin != d_keys)
    ABX_CUDA_TRY(cudaMemcpyAsync(d_keys, kin, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
  if (vin != d_vals)
    ABX_CUDA_TRY(cudaMemcpyAsync(d_vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  return ABX_SUCCESS;
}

// Top passes, run fix-up, long runs through a segmented sort of their keys.
template <class K>
abx_status radix_sort_hybrid(cudaStream_t s, K *d_keys, uint32_t *d_vals,
                             const uint32_t *d_vals_in, int64_t n, int num_passes,
                             const uint32_t *d_hist, int top, int &launches)
{
  const int first = num_passes - top;
  const int shift = 8 * first;
  Scratch<K> keys_alt;
  Scratch<uint32_t> vals_alt;
  ABX_CUDA_TRY(keys_alt.alloc(n, s));
  ABX_CUDA_TRY(vals_alt.alloc(n, s));
  const K *kin;
  const uint32_t *vin;
  ABX_TRY(sort_passes<K>(s, d_keys, d_vals, d_vals_in, n, first, num_passes, d_hist,
                         keys_alt.ptr, vals_alt.ptr, &kin, &vin, launches));
  // the fix-up is out of place: into d_keys / d_vals, or through the
  // alternate buffers when the passes ended in d_keys
  const bool via_alt = kin == d_keys;
  K *kout = via_alt ? keys_alt.ptr : d_keys;
  uint32_t *vout = via_alt ? vals_alt.ptr : d_vals;
  Scratch<unsigned long long> long_count;
  ABX_CUDA_TRY(long_count.alloc(1, s));
  ABX_CUDA_TRY(cudaMemsetAsync(long_count.ptr, 0, sizeof(unsigned long long), s));
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_run_fixup<K><<<(unsigned)((n + kFixThreads - 1) / kFixThreads), kFixThreads, 0, s>>>(
      kin, vin, kout, vout, n, shift, long_count.ptr);
  ABX_CUDA_TRY(cudaGetLastError());
  ++launches;
  unsigned long long m = 0;
  ABX_CUDA_TRY(cudaMemcpyAsync(&m, long_count.ptr, sizeof(m), cudaMemcpyDeviceToHost, s));
  ABX_CUDA_TRY(cudaStreamSynchronize(s));
  if (m > 0)
  {
    // runs have more than kRunMax keys: fewer than n / (kRunMax + 1) of them
    const int64_t max_runs = (int64_t)m / (kRunMax + 1) + 1;
    int run_bits = 0;
    while ((1ll << run_bits) < max_runs)
      ++run_bits;
    if (shift + run_bits > (int)(8 * sizeof(K)))
      return fail(ABX_ERROR_NOT_SUPPORTED, "radix sort: too many long runs");
    Scratch<int32_t> is_long, is_start, long_pos, run_excl;
    ABX_CUDA_TRY(is_long.alloc(n, s));
    ABX_CUDA_TRY(is_start.alloc(n, s));
    ABX_CUDA_TRY(long_pos.alloc(n + 1, s));
    ABX_CUDA_TRY(run_excl.alloc(n + 1, s));
    k_long_flags<K><<<blocks, 256, 0, s>>>(kin, n, shift, is_long.ptr, is_start.ptr);
    ABX_CUDA_TRY(cudaGetLastError());
    ABX_TRY(exclusive_scan_i32(s, is_long.ptr, n, long_pos.ptr));
    ABX_TRY(exclusive_scan_i32(s, is_start.ptr, n, run_excl.ptr));
    Scratch<K> ckeys;
    Scratch<uint32_t> cpos, cperm;
    ABX_CUDA_TRY(ckeys.alloc(m, s));
    ABX_CUDA_TRY(cpos.alloc(m, s));
    ABX_CUDA_TRY(cperm.alloc(m, s));
    k_long_compact<K><<<blocks, 256, 0, s>>>(kin, n, shift, is_long.ptr, long_pos.ptr,
                                              is_start.ptr, run_excl.ptr, ckeys.ptr, cpos.ptr);
    ABX_CUDA_TRY(cudaGetLastError());
    launches += 3 + 2 * 3; // flags, compact, gather; two scans of 3 kernels
    ABX_TRY(radix_sort_full<K>(s, ckeys.ptr, cperm.ptr, nullptr, (int64_t)m,
                               (shift + run_bits + 7) / 8, nullptr, launches));
    k_long_gather<K><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(kin, vin, kout, vout, cpos.ptr,
                                                                cperm.ptr, (int64_t)m);
    ABX_CUDA_TRY(cudaGetLastError());
  }
  if (via_alt)
  {
    ABX_CUDA_TRY(cudaMemcpyAsync(d_keys, kout, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
    ABX_CUDA_TRY(cudaMemcpyAsync(d_vals, vout, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
  return ABX_SUCCESS;
}

template <class K>
abx_status radix_sort_impl(cudaStream_t s, K *d_keys, uint32_t *d_vals,
                           const uint32_t *d_vals_in, int64_t n, int num_passes,
                           const uint32_t *d_hist, int top)
{
  if (n <= 0)
    return ABX_SUCCESS;
  if (n > (int64_t)INT32_MAX)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "radix sort: more than 2^31-1 keys");
  if (num_passes < 1 || num_passes > (int)(sizeof(K) * 8 / 8))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "radix sort: bad number of passes");
  if (top < 0 || top >= num_passes)
    top = 0;
  StageScope scope(s, sizeof(K) == 8 ? "sort64" : "sort32", 0);
  int launches = 0;
  abx_status st = top > 0
                      ? radix_sort_hybrid<K>(s, d_keys, d_vals, d_vals_in, n, num_passes, d_hist,
                                             top, launches)
                      : radix_sort_full<K>(s, d_keys, d_vals, d_vals_in, n, num_passes, d_hist,
                                           launches);
  scope.add_kernels(launches);
  return st;
}

// ---------------------------------------------------------------------------
// Exclusive scan: reduce per chunk, scan the chunk sums, apply.
// ---------------------------------------------------------------------------

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ long long block_sum_ll(long long v, long long *sh)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  __syncthreads();
  long long t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      t += sh[w];
  return t;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int32_t *__restrict__ in,
                                                              int64_t n,
                                                              long long *__restrict__ sums)
{
  __shared__ long long sh[kScanThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanChunk;
  long long v = 0;
  for (int j = 0; j < kScanItems; ++j)
  {
    int64_t i = base + j * kScanThreads + threadIdx.x;
    if (i < n)
      v += in[i];
  }
  long long t = block_sum_ll(v, sh);
  if (threadIdx.x == 0)
    sums[blockIdx.x] = t;
}

// Single CTA: exclusive scan of the chunk sums in place (nblocks entries).
__global__ void __launch_bounds__(1024) k_scan_sums(long long *__restrict__ sums, int64_t nb)
{
  __shared__ long long warp_tot[32];
  __shared__ long long carry;
  if (threadIdx.x == 0)
    carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x)
  {
    int64_t i = base + threadIdx.x;
    long long v = i < nb ? sums[i] : 0;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      long long y = __shfl_up_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) >= o)
        x += y;
    }
    if ((threadIdx.x & 31) == 31)
      warp_tot[threadIdx.x >> 5] = x;
    __syncthreads();
    long long pre = carry;
    for (int w = 0; w < (int)(threadIdx.x >> 5); ++w)
      pre += warp_tot[w];
    if (i < nb)
      sums[i] = pre + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1)
      carry = pre + x;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int32_t *__restrict__ in,
                                                             int64_t n,
                                                             const long long *__restrict__ sums,
                                                             int32_t *__restrict__ out,
                                                             unsigned *__restrict__ err)
{
  __shared__ long long warp_tot[kScanThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanChunk;
  // each thread owns kScanItems consecutive elements
  int64_t first = base + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  long long local = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
  {
    int64_t i = first + j;
    v[j] = i < n ? in[i] : 0;
    local += v[j];
  }
  long long x = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) >= o)
      x += y;
  }
  if ((threadIdx.x & 31) == 31)
    warp_tot[threadIdx.x >> 5] = x;
  __syncthreads();
  long long pre = sums[blockIdx.x];
  for (int w = 0; w < (int)(threadIdx.x >> 5); ++w)
    pre += warp_tot[w];
  long long run = pre + x - local;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
  {
    int64_t i = first + j;
    if (i <= n)
    {
      if (run > INT32_MAX)
        raise_error(err, ABX_DEVERR_BAD_INPUT);
      if (i < n || j == 0 || first + j - 1 < n)
        out[i] = (int32_t)run;
    }
    run += v[j];
  }
}

} // namespace

abx_status init_sort_kernels()
{
  // dynamic shared memory of the onesweep passes (above the 48 KB default);
  // set once per device, outside any stream capture
  ABX_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint64_t>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sizeof(PassSmem<uint64_t>)));
  ABX_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<uint32_t>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sizeof(PassSmem<uint32_t>)));
  return ABX_SUCCESS;
}

abx_status radix_sort_u64(cudaStream_t s, uint64_t *d_keys, uint32_t *d_vals,
                          const uint32_t *d_vals_in, int64_t n, int num_passes,
                          const uint32_t *d_hist, int top_passes)
{
  return radix_sort_impl<uint64_t>(s, d_keys, d_vals, d_vals_in, n, num_passes, d_hist,
                                   top_passes);
}

abx_status radix_sort_u32(cudaStream_t s, uint32_t *d_keys, uint32_t *d_vals,
                          const uint32_t *d_vals_in, int64_t n, int num_passes,
                          const uint32_t *d_hist, int top_passes)
{
  return radix_sort_impl<uint32_t>(s, d_keys, d_vals, d_vals_in, n, num_passes, d_hist,
                                   top_passes);
}

abx_status radix_order_top_u32(cudaStream_t s, uint32_t *d_keys, uint32_t *d_perm, int64_t n,
                               int num_passes, const uint32_t *d_hist, int top)
{
  if (n <= 0)
    return ABX_SUCCESS;
  if (top < 1 || top > num_passes || num_passes > 4)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "radix order: bad number of digits");
  StageScope scope(s, "sort32", 0);
  int launches = 0;
  Scratch<uint32_t> keys_alt, vals_alt;
  ABX_CUDA_TRY(keys_alt.alloc(n, s));
  ABX_CUDA_TRY(vals_alt.alloc(n, s));
  const uint32_t *kin;
  const uint32_t *vin;
  ABX_TRY(sort_passes<uint32_t>(s, d_keys, d_perm, nullptr, n, num_passes - top, num_passes,
                                d_hist, keys_alt.ptr, vals_alt.ptr, &kin, &vin, launches));
  if (vin != d_perm)
    ABX_CUDA_TRY(cudaMemcpyAsync(d_perm, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  scope.add_kernels(launches);
  return ABX_SUCCESS;
}

int choose_top_passes(const uint32_t *h_hist, int64_t n, int num_passes)
{
  const int cap = hybrid_top_passes(n, num_passes);
  if (cap <= 0 || !h_hist)
    return cap;
  // expected keys sharing a key's top-digit cell, digits taken independent:
  // n * prod_d sum_b p_d(b)^2 (about 1.2 for 1e7 uniform Morton codes with 3
  // digits); clustered keys make it large
  double collide = 1.0;
  for (int t = 1; t <= 4 && t < num_passes; ++t)
  {
    const uint32_t *h = h_hist + (size_t)(num_passes - t) * kBins;
    double sq = 0.0;
    for (int b = 0; b < kBins; ++b)
    {
      const double p = (double)h[b] / (double)n;
      sq += p * p;
    }
    collide *= sq;
    if (t >= 3 && (double)n * collide <= 4.0)
      return t;
  }
  return 0;
}

int hybrid_top_passes(int64_t n, int num_passes)
{
  // 3 top digits (24 bits) spread up to ~2^24 keys into short runs, 4 digits
  // up to ~2^32; below 2^16 keys the plain sort is as cheap
  if (n < (1 << 16) || num_passes <= 3)
    return 0;
  const int def = n <= (int64_t)(1 << 24) ? 3 : 4;
  return std::min(tuning_value("SORT_TOP_PASSES", def), num_passes - 1);
}

abx_status exclusive_scan_i32(cudaStream_t s, const int32_t *d_in, int64_t n, int32_t *d_out)
{
  DeviceState &ds = device_state();
  if (n < 0)
    return fail(ABX_ERROR_INVALID_ARGUMENT, "exclusive_scan: negative size");
  int64_t nb = (n + kScanChunk) / kScanChunk; // covers index n as well
  Scratch<long long> sums;
  ABX_CUDA_TRY(sums.alloc(nb, s));
  StageScope scope(s, "scan", 3);
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(d_in, n, sums.ptr);
  k_scan_sums<<<1, 1024, 0, s>>>(sums.ptr, nb);
  k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(d_in, n, sums.ptr, d_out, ds.d_error);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}

// ---------------------------------------------------------------------------
// Allocation-free exclusive scan (abx_exclusive_scan_i32_noalloc)
// ---------------------------------------------------------------------------

namespace
{

constexpr int64_t kNoAllocScanMaxN = ABX_NOALLOC_SCAN_MAX_N;
constexpr int64_t kNoAllocScanChunks = kNoAllocScanMaxN / kScanChunk + 1;

// The scan's chunk sums live in the library's static device memory: no call
// allocates.  Shared by every call on a device (see the header for the
// consequences: overlapping calls race).
static __device__ __align__(256) long long g_noalloc_scan_sums[kNoAllocScanChunks];

std::mutex g_noalloc_mutex;
long long *g_noalloc_sums_ptr[64] = {};

// Device address of g_noalloc_scan_sums for the current device, looked up
// once per device.  In host code the array's name is only a host-side
// stand-in, never a device address.
abx_status noalloc_scan_scratch(long long **out)
{
  int dev = 0;
  ABX_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64)
    return fail(ABX_ERROR_NOT_SUPPORTED, "abx_exclusive_scan_i32_noalloc: device id >= 64");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_sums_ptr[dev])
  {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_sums);
    if (e != cudaSuccess)
      return fail_cuda(e, "cudaGetSymbolAddress(g_noalloc_scan_sums)");
    g_noalloc_sums_ptr[dev] = static_cast<long long *>(p);
  }
  *out = g_noalloc_sums_ptr[dev];
  return ABX_SUCCESS;
}

} // namespace

} // namespace abx

extern "C" abx_status abx_exclusive_scan_i32_noalloc(void *stream, const int32_t *d_in,
                                                      int64_t n, int32_t *d_out)
{
  using namespace abx;
  if (n < 0 || !d_out || (n > 0 && !d_in))
    return fail(ABX_ERROR_INVALID_ARGUMENT, "abx_exclusive_scan_i32_noalloc: bad argument");
  if (n > kNoAllocScanMaxN)
    return fail(ABX_ERROR_INVALID_ARGUMENT,
                "abx_exclusive_scan_i32_noalloc: n = " + std::to_string(n) +
                    " exceeds the maximum of " + std::to_string(kNoAllocScanMaxN) +
                    " inputs this allocation-free variant supports");
  long long *sums = nullptr;
  ABX_TRY(noalloc_scan_scratch(&sums));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t nb = (n + kScanChunk) / kScanChunk; // <= kNoAllocScanChunks
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(d_in, n, sums);
  k_scan_sums<<<1, 1024, 0, s>>>(sums, nb);
  k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(d_in, n, sums, d_out, nullptr);
  ABX_CUDA_TRY(cudaGetLastError());
  return ABX_SUCCESS;
}
