// primitives.cuh - hand-written device-wide scan and LSD radix sort.
//
// Both are tile-based (2048 items per 256-thread block).  The scan is
// reduce-then-scan: per-tile sums, a scan of them (recursive), then a pass
// that scans each tile with its offset.  The radix
// sort is stable, with 8-bit digits; segmented sorting is done by sorting on
// the key and then, stably, on the segment id (see unbind.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace hbtg
{

constexpr int kScanThreads = 256;

// Rows per warp of a scan tile: 8 for 4/8-byte types, 4 for the 12-byte I3
// and 32-byte I4.
template <typename T>
__host__ __device__ constexpr int scan_items()
{
  return sizeof(T) > 8 ? 4 : 8;
}
template <typename T>
__host__ __device__ constexpr int scan_tile()
{
  return kScanThreads * scan_items<T>();
}

// Four 64-bit fixed-point sums, modulo 2^64 (exact, so any summation order
// gives the same result; a difference of two prefixes is exact whenever the
// true difference fits in 63 bits).
struct I4
{
  unsigned long long m, x, y, z;
  __host__ __device__ I4 operator+(const I4 &o) const { return I4{m + o.m, x + o.x, y + o.y, z + o.z}; }
};

// Three counts scanned together (one pass, one host read of the totals).
struct I3
{
  int a, b, c;
  __host__ __device__ I3 operator+(const I3 &o) const { return I3{a + o.a, b + o.b, c + o.c}; }
};

// Four counts scanned together (one pass, one host read of the totals).
struct I4c
{
  int a, b, c, d;
  __host__ __device__ I4c operator+(const I4c &o) const { return I4c{a + o.a, b + o.b, c + o.c, d + o.d}; }
};

// Segmented double sum: head marks the first item of a segment, where the
// running sum restarts.  Associative, not commutative.
struct SegD
{
  double v;
  int head;
  __host__ __device__ SegD operator+(const SegD &o) const { return o.head ? o : SegD{v + o.v, head}; }
};

// Types whose + is not commutative: the reduce pass keeps item order.
template <typename T>
struct ordered_sum
{
  static constexpr bool value = false;
};
template <>
struct ordered_sum<SegD>
{
  static constexpr bool value = true;
};

template <typename T>
__device__ __forceinline__ T zero_of();
template <>
__device__ __forceinline__ int zero_of<int>() { return 0; }
template <>
__device__ __forceinline__ long long zero_of<long long>() { return 0; }
template <>
__device__ __forceinline__ I4 zero_of<I4>() { return I4{0, 0, 0, 0}; }
template <>
__device__ __forceinline__ I3 zero_of<I3>() { return I3{0, 0, 0}; }
template <>
__device__ __forceinline__ I4c zero_of<I4c>() { return I4c{0, 0, 0, 0}; }
template <>
__device__ __forceinline__ SegD zero_of<SegD>() { return SegD{0., 0}; }

template <typename T>
__device__ __forceinline__ T shfl_up(T v, int d)
{
  return __shfl_up_sync(0xffffffffu, v, d);
}
template <>
__device__ __forceinline__ I3 shfl_up<I3>(I3 v, int d)
{
  return I3{__shfl_up_sync(0xffffffffu, v.a, d), __shfl_up_sync(0xffffffffu, v.b, d),
            __shfl_up_sync(0xffffffffu, v.c, d)};
}
template <>
__device__ __forceinline__ I4c shfl_up<I4c>(I4c v, int d)
{
  return I4c{__shfl_up_sync(0xffffffffu, v.a, d), __shfl_up_sync(0xffffffffu, v.b, d),
             __shfl_up_sync(0xffffffffu, v.c, d), __shfl_up_sync(0xffffffffu, v.d, d)};
}
template <>
__device__ __forceinline__ I4 shfl_up<I4>(I4 v, int d)
{
  return I4{__shfl_up_sync(0xffffffffu, v.m, d), __shfl_up_sync(0xffffffffu, v.x, d),
            __shfl_up_sync(0xffffffffu, v.y, d), __shfl_up_sync(0xffffffffu, v.z, d)};
}

template <>
__device__ __forceinline__ SegD shfl_up<SegD>(SegD v, int d)
{
  return SegD{__shfl_up_sync(0xffffffffu, v.v, d), __shfl_up_sync(0xffffffffu, v.head, d)};
}

template <typename T>
__device__ __forceinline__ T shfl_idx(T v, int src)
{
  return __shfl_sync(0xffffffffu, v, src);
}
template <>
__device__ __forceinline__ I3 shfl_idx<I3>(I3 v, int src)
{
  return I3{__shfl_sync(0xffffffffu, v.a, src), __shfl_sync(0xffffffffu, v.b, src),
            __shfl_sync(0xffffffffu, v.c, src)};
}
template <>
__device__ __forceinline__ I4c shfl_idx<I4c>(I4c v, int src)
{
  return I4c{__shfl_sync(0xffffffffu, v.a, src), __shfl_sync(0xffffffffu, v.b, src),
             __shfl_sync(0xffffffffu, v.c, src), __shfl_sync(0xffffffffu, v.d, src)};
}
template <>
__device__ __forceinline__ I4 shfl_idx<I4>(I4 v, int src)
{
  return I4{__shfl_sync(0xffffffffu, v.m, src), __shfl_sync(0xffffffffu, v.x, src),
            __shfl_sync(0xffffffffu, v.y, src), __shfl_sync(0xffffffffu, v.z, src)};
}

// Every combine in the scans below is (earlier items) + (later items), so a
// non-commutative associative + (the segmented sum SegD) scans correctly.
template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v, int lane)
{
#pragma unroll
  for (int d = 1; d < 32; d <<= 1)
  {
    const T o = shfl_up(v, d);
    if (lane >= d)
      v = o + v;
  }
  return v;
}

template <>
__device__ __forceinline__ SegD shfl_idx<SegD>(SegD v, int src)
{
  return SegD{__shfl_sync(0xffffffffu, v.v, src), __shfl_sync(0xffffffffu, v.head, src)};
}

// Scan input read straight from an array, output written to one.
template <typename T>
struct ArrayLoad
{
  const T *in;
  __device__ __forceinline__ T operator()(long long i) const { return in[i]; }
};
template <typename T>
struct ArrayStore
{
  T *out;
  __device__ __forceinline__ void operator()(long long i, const T &v) const { out[i] = v; }
};

// Reduce-then-scan.  A tile is 8 warps x 32 lanes x scan_items<T>() rows;
// warp w owns the contiguous items [w*32*rows, (w+1)*32*rows) of its tile and
// reads them one coalesced row of 32 at a time.  Pass 1 sums each tile, the
// tile sums are scanned (recursively), pass 2 scans each tile row by row with
// warp shuffles and adds the tile's offset.  `Load` supplies item i, so an
// input that is a function of other arrays needs no array of its own.
template <typename T, typename Load>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(Load load, T *__restrict__ tile_sums, long long n)
{
  constexpr int kTile = scan_tile<T>(), kRows = scan_items<T>();
  __shared__ T warp_tot[kScanThreads / kWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long wbase = (long long)blockIdx.x * kTile + (long long)warp * kWarp * kRows;
  T acc = zero_of<T>();
  if constexpr (ordered_sum<T>::value)
  { // row by row, in item order
#pragma unroll
    for (int k = 0; k < kRows; k++)
    {
      const long long i = wbase + k * kWarp + lane;
      const T x = (i < n) ? load(i) : zero_of<T>();
      acc = acc + shfl_idx(warp_inclusive_scan(x, lane), 31);
    }
  }
  else
  {
#pragma unroll
    for (int k = 0; k < kRows; k++)
    {
      const long long i = wbase + k * kWarp + lane;
      if (i < n)
        acc = acc + load(i);
    }
    acc = warp_inclusive_scan(acc, lane);
  }
  if (lane == 31)
    warp_tot[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    T tot = zero_of<T>();
#pragma unroll
    for (int w = 0; w < kScanThreads / kWarp; w++)
      tot = tot + warp_tot[w];
    tile_sums[blockIdx.x] = tot;
  }
}

template <typename T, bool Inclusive, typename Load, typename Store>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(Load load, Store store, const T *__restrict__ tile_off,
                                                             long long n)
{
  constexpr int kTile = scan_tile<T>(), kRows = scan_items<T>();
  __shared__ T warp_tot[kScanThreads / kWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long wbase = (long long)blockIdx.x * kTile + (long long)warp * kWarp * kRows;
  T v[kRows];
  T carry = zero_of<T>();
#pragma unroll
  for (int k = 0; k < kRows; k++)
  {
    const long long i = wbase + k * kWarp + lane;
    const T x = (i < n) ? load(i) : zero_of<T>();
    const T inc = warp_inclusive_scan(x, lane);
    T part = inc;
    if (!Inclusive)
    { // exclusive = the previous lane's inclusive value
      part = shfl_up(inc, 1);
      if (lane == 0)
        part = zero_of<T>();
    }
    v[k] = carry + part;
    carry = carry + shfl_idx(inc, 31);
  }
  if (lane == 0)
    warp_tot[warp] = carry;
  __syncthreads(); // every item of the tile is read before any is written (in == out allowed)
  T off = tile_off ? tile_off[blockIdx.x] : zero_of<T>();
  for (int w = 0; w < warp; w++)
    off = off + warp_tot[w];
#pragma unroll
  for (int k = 0; k < kRows; k++)
  {
    const long long i = wbase + k * kWarp + lane;
    if (i < n)
      store(i, off + v[k]);
  }
}

// Scratch needed by scan<T>(n): sum over recursion levels of the tile counts.
template <typename T>
inline size_t scan_scratch_elems(long long n)
{
  constexpr int kTile = scan_tile<T>();
  size_t tot = 0;
  while (n > kTile)
  {
    n = (n + kTile - 1) / kTile;
    tot += 2 * (size_t)n;
  }
  return tot + 2;
}

// Device-wide scan of the n items load(0..n-1), result i passed to store(i, .).
// `scratch` must hold scan_scratch_elems(n) items of T.
template <typename T, bool Inclusive, typename Load, typename Store>
void scan_load_store(Load load, Store store, long long n, T *scratch, cudaStream_t st, int64_t *launches)
{
  constexpr int kTile = scan_tile<T>();
  if (n <= 0)
    return;
  const long long tiles = (n + kTile - 1) / kTile;
  if (tiles == 1)
  {
    k_scan_apply<T, Inclusive, Load, Store><<<1, kScanThreads, 0, st>>>(load, store, nullptr, n);
    (*launches)++;
    return;
  }
  T *sums = scratch, *sums_scanned = scratch + tiles;
  k_scan_reduce<T, Load><<<(unsigned)tiles, kScanThreads, 0, st>>>(load, sums, n);
  scan_load_store<T, false>(ArrayLoad<T>{sums}, ArrayStore<T>{sums_scanned}, tiles, scratch + 2 * tiles, st,
                            launches);
  k_scan_apply<T, Inclusive, Load, Store><<<(unsigned)tiles, kScanThreads, 0, st>>>(load, store, sums_scanned, n);
  *launches += 2;
}

// Device-wide scan of the n items load(0..n-1) into out.
template <typename T, bool Inclusive, typename Load>
void scan_load(Load load, T *out, long long n, T *scratch, cudaStream_t st, int64_t *launches)
{
  scan_load_store<T, Inclusive>(load, ArrayStore<T>{out}, n, scratch, st, launches);
}

// Device-wide scan of n items (in may equal out).
template <typename T, bool Inclusive>
void scan(const T *in, T *out, long long n, T *scratch, cudaStream_t st, int64_t *launches)
{
  scan_load<T, Inclusive>(ArrayLoad<T>{in}, out, n, scratch, st, launches);
}

// ---------------------------------------------------------------------------
// LSD radix sort, 8-bit digits, stable.  Keys K = uint32_t or uint64_t,
// 32-bit values.
// ---------------------------------------------------------------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 8;
constexpr int kRadixTile = kRadixThreads * kRadixItems;

template <typename K>
__global__ void __launch_bounds__(kRadixThreads) k_radix_hist(const K *__restrict__ keys, long long n, int shift,
                                                              uint32_t mask, int *__restrict__ table, int tiles)
{
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRadixTile;
#pragma unroll
  for (int k = 0; k < kRadixItems; k++)
  {
    const long long i = base + k * kRadixThreads + threadIdx.x;
    if (i < n)
      atomicAdd(&cnt[(uint32_t)(keys[i] >> shift) & mask], 1);
  }
  __syncthreads();
  table[(long long)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Items of a scatter tile: warp w owns the contiguous items [w*256,
// (w+1)*256), read as 8 rows of 32 consecutive items.
// Stable scatter of one tile.  Each warp ranks its own items against a
// private per-digit count (match_any gives the equal-digit peers of a row),
// the per-digit counts are scanned across warps and digits, the items are
// placed into shared memory in digit order (input order within a digit) and
// written out so that consecutive threads store consecutive addresses of a
// digit's output run.
template <typename K>
__global__ void __launch_bounds__(kRadixThreads)
  k_radix_scatter(const K *__restrict__ kin, const uint32_t *__restrict__ vin, K *__restrict__ kout,
                  uint32_t *__restrict__ vout, long long n, int shift, uint32_t mask, const int *__restrict__ table,
                  int tiles)
{
  constexpr int kWarps = kRadixThreads / kWarp;
  __shared__ K s_key[kRadixTile];
  __shared__ uint32_t s_val[kRadixTile];
  __shared__ int s_off[256];         // this tile's first output slot per digit (scanned table)
  __shared__ int s_start[256];       // first shared-memory slot per digit
  __shared__ int s_wcnt[kWarps][256]; // per warp and digit: count, then the warp's offset within the digit
  __shared__ int s_wsum[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long tile0 = (long long)blockIdx.x * kRadixTile;
  const int count = (int)min((long long)kRadixTile, n - tile0);
  s_off[tid] = table[(long long)tid * tiles + blockIdx.x];
#pragma unroll
  for (int w = 0; w < kWarps; w++)
    s_wcnt[w][tid] = 0;
  __syncthreads();
  // 1. rank within the warp, row by row
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int wbase = warp * (kWarp * kRadixItems);
  K key[kRadixItems];
  uint32_t val[kRadixItems], dr[kRadixItems]; // digit (9 bits, 256 = no item) | rank in the warp << 9
#pragma unroll
  for (int r = 0; r < kRadixItems; r++)
  {
    const int k = wbase + r * kWarp + lane;
    const bool valid = k < count;
    key[r] = valid ? kin[tile0 + k] : K(0);
    val[r] = valid ? vin[tile0 + k] : 0u;
    const uint32_t d = valid ? ((uint32_t)(key[r] >> shift) & mask) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const int before = (d < 256u) ? s_wcnt[warp][d] : 0;
    dr[r] = d | ((uint32_t)(before + __popc(peers & lt_mask)) << 9);
    __syncwarp();
    if (d < 256u && lane == __ffs(peers) - 1)
      s_wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // 2. per digit (thread tid = digit): warp offsets within the digit, then
  // the digit's start in the tile (exclusive scan over digits)
  int run = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++)
  {
    const int c = s_wcnt[w][tid];
    s_wcnt[w][tid] = run;
    run += c;
  }
  int incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o)
      incl += y;
  }
  if (lane == 31)
    s_wsum[warp] = incl;
  __syncthreads();
  int woff = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++)
    woff += (w < warp) ? s_wsum[w] : 0;
  s_start[tid] = woff + incl - run;
  __syncthreads();
  // 3. place into shared memory in digit order
#pragma unroll
  for (int r = 0; r < kRadixItems; r++)
  {
    const uint32_t d = dr[r] & 511u;
    if (d < 256u)
    {
      const int pos = s_start[d] + s_wcnt[warp][d] + (int)(dr[r] >> 9);
      s_key[pos] = key[r];
      s_val[pos] = val[r];
    }
  }
  __syncthreads();
  // 4. write out
  for (int k = tid; k < count; k += kRadixThreads)
  {
    const K kk = s_key[k];
    const uint32_t d = (uint32_t)(kk >> shift) & mask;
    const int dst = s_off[d] + (k - s_start[d]);
    kout[dst] = kk;
    vout[dst] = s_val[k];
  }
}

// One-block LSD radix sort of n <= Threads * kRadixItems items: every pass
// runs in shared memory (the same per-warp ranking and digit scan as
// k_radix_scatter, with the whole input as one tile), and the sorted items
// are written back to (keys, vals).  It replaces three launches per pass for
// the small sorts of the late iterations, where launch latency, not memory
// traffic, is the cost.  Dynamic shared memory: radix_block_smem<K>(Threads).
template <typename K>
__host__ __device__ constexpr size_t radix_block_smem(int threads)
{
  return (size_t)threads * kRadixItems * (sizeof(K) + sizeof(uint32_t)) + sizeof(int) * (size_t)(threads / kWarp) * 256 +
         sizeof(int) * (256 + 8);
}

template <typename K, int Threads>
__global__ void __launch_bounds__(Threads)
  k_radix_sort_block(K *__restrict__ keys, uint32_t *__restrict__ vals, int n, int begin_bit, int end_bit)
{
  constexpr int kWarps = Threads / kWarp;
  constexpr int kN = Threads * kRadixItems;
  extern __shared__ __align__(16) unsigned char radix_smem[];
  K *s_key = reinterpret_cast<K *>(radix_smem);
  uint32_t *s_val = reinterpret_cast<uint32_t *>(s_key + kN);
  int *s_wcnt = reinterpret_cast<int *>(s_val + kN); // [kWarps][256]
  int *s_start = s_wcnt + kWarps * 256;               // [256]
  int *s_dsum = s_start + 256;                        // [8]: digit sums of the eight digit warps
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int wbase = warp * (kWarp * kRadixItems);
  K key[kRadixItems];
  uint32_t val[kRadixItems], dr[kRadixItems];
#pragma unroll
  for (int r = 0; r < kRadixItems; r++)
  {
    const int k = wbase + r * kWarp + lane;
    key[r] = k < n ? keys[k] : K(0);
    val[r] = k < n ? vals[k] : 0u;
  }
  for (int shift = begin_bit; shift < end_bit; shift += 8)
  {
    const int bits = (end_bit - shift) < 8 ? (end_bit - shift) : 8;
    const uint32_t mask = (1u << bits) - 1u;
    for (int i = tid; i < kWarps * 256; i += Threads)
      s_wcnt[i] = 0;
    __syncthreads();
    // 1. rank within the warp, row by row (rows in item order: stable)
#pragma unroll
    for (int r = 0; r < kRadixItems; r++)
    {
      const int k = wbase + r * kWarp + lane;
      const uint32_t d = k < n ? ((uint32_t)(key[r] >> shift) & mask) : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const int before = (d < 256u) ? s_wcnt[warp * 256 + d] : 0;
      dr[r] = d | ((uint32_t)(before + __popc(peers & lt_mask)) << 9);
      __syncwarp();
      if (d < 256u && lane == __ffs(peers) - 1)
        s_wcnt[warp * 256 + d] = before + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // 2. threads 0..255, one per digit: each warp's offset within the digit,
    // then the digit's first slot (exclusive scan over digits)
    int run = 0, incl = 0;
    if (tid < 256)
    {
      for (int w = 0; w < kWarps; w++)
      {
        const int c = s_wcnt[w * 256 + tid];
        s_wcnt[w * 256 + tid] = run;
        run += c;
      }
      incl = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
      {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
          incl += y;
      }
      if (lane == 31)
        s_dsum[warp] = incl;
    }
    __syncthreads();
    if (tid < 256)
    {
      int woff = 0;
      for (int w = 0; w < warp; w++)
        woff += s_dsum[w];
      s_start[tid] = woff + incl - run;
    }
    __syncthreads();
    // 3. place in digit order, then read back in item order for the next pass
#pragma unroll
    for (int r = 0; r < kRadixItems; r++)
    {
      const uint32_t d = dr[r] & 511u;
      if (d < 256u)
      {
        const int pos = s_start[d] + s_wcnt[warp * 256 + d] + (int)(dr[r] >> 9);
        s_key[pos] = key[r];
        s_val[pos] = val[r];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRadixItems; r++)
    {
      const int k = wbase + r * kWarp + lane;
      if (k < n)
      {
        key[r] = s_key[k];
        val[r] = s_val[k];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < kRadixItems; r++)
  {
    const int k = wbase + r * kWarp + lane;
    if (k < n)
    {
      keys[k] = key[r];
      vals[k] = val[r];
    }
  }
}

// Largest sort done by one block (k_radix_sort_block<K, 1024>).
constexpr int kRadixBlockMax = 1024 * kRadixItems;

inline size_t radix_table_elems(long long n)
{
  const long long tiles = (n + kRadixTile - 1) / kRadixTile;
  return (size_t)256 * tiles;
}

// Sorts (keys, vals) on bits [begin_bit, end_bit).  Ping-pongs between the
// two buffer pairs; returns true when the result lies in (k_alt, v_alt).
// `table` holds radix_table_elems(n) ints, `scan_scratch`
// scan_scratch_elems<int>(radix_table_elems(n)) ints.  Sorts of at most
// `block_max` items (<= kRadixBlockMax) run in one block; the result is the
// same either way (a stable sort).
template <typename K>
bool radix_sort_pairs(K *keys, uint32_t *vals, K *k_alt, uint32_t *v_alt, long long n, int begin_bit, int end_bit,
                      int *table, int *scan_scratch, cudaStream_t st, int64_t *launches,
                      int block_max = kRadixBlockMax)
{
  if (n <= 1 || end_bit <= begin_bit)
    return false;
  block_max = block_max < kRadixBlockMax ? block_max : kRadixBlockMax;
  if (n <= kRadixTile && n <= block_max)
  { // one block, every pass in shared memory; the result stays in (keys, vals)
    k_radix_sort_block<K, kRadixThreads><<<1, kRadixThreads, radix_block_smem<K>(kRadixThreads), st>>>(
      keys, vals, (int)n, begin_bit, end_bit);
    (*launches)++;
    return false;
  }
  if (n <= block_max)
  {
    const size_t smem = radix_block_smem<K>(1024);
    cudaFuncSetAttribute(k_radix_sort_block<K, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_radix_sort_block<K, 1024><<<1, 1024, smem, st>>>(keys, vals, (int)n, begin_bit, end_bit);
    (*launches)++;
    return false;
  }
  const int tiles = (int)((n + kRadixTile - 1) / kRadixTile);
  bool flipped = false;
  for (int shift = begin_bit; shift < end_bit; shift += 8)
  {
    const int bits = (end_bit - shift) < 8 ? (end_bit - shift) : 8;
    const uint32_t mask = (1u << bits) - 1u;
    const K *ki = flipped ? k_alt : keys;
    const uint32_t *vi = flipped ? v_alt : vals;
    K *ko = flipped ? keys : k_alt;
    uint32_t *vo = flipped ? vals : v_alt;
    k_radix_hist<K><<<tiles, kRadixThreads, 0, st>>>(ki, n, shift, mask, table, tiles);
    scan<int, false>(table, table, (long long)256 * tiles, scan_scratch, st, launches);
    k_radix_scatter<K><<<tiles, kRadixThreads, 0, st>>>(ki, vi, ko, vo, n, shift, mask, table, tiles);
    *launches += 2;
    flipped = !flipped;
  }
  return flipped;
}

} // namespace hbtg
