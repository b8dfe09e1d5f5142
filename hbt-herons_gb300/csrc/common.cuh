// common.cuh - shared device types and helpers of the GB300 unbinding library.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hbtg
{

constexpr int kWarp = 32;

// Float <-> order-preserving uint32 (used by min/max atomics and radix keys).
__device__ __forceinline__ uint32_t float_to_ordered(float f)
{
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(uint32_t u)
{
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Index of the segment holding packed item `idx`: the last s with off[s] <= idx,
// for a non-decreasing offset array of n+1 entries.
template <typename T>
__device__ __forceinline__ int find_segment(const T *__restrict__ off, int n, T idx)
{
  int lo = 0, hi = n; // answer in [lo, hi)
  while (hi - lo > 1)
  {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= idx)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// find_segment for a warp whose 32 lanes all call it with non-decreasing
// indices: a 32-ary search for the first and the last lane's segment (each
// step probes 32 evenly spaced offsets at once and counts them with a
// ballot), then each lane searches only between those two segments.
template <typename T>
__device__ __forceinline__ int find_segment_32ary(const T *__restrict__ off, int lo, int hi, T target)
{
  const int lane = threadIdx.x & 31;
  while (hi - lo > 1) // off[lo] <= target; answer in [lo, hi)
  {
    const int step = (hi - lo + 31) >> 5;
    const int pos = lo + (lane + 1) * step;
    const bool ok = pos < hi && __ldg(off + pos) <= target;
    const int c = __popc(__ballot_sync(0xffffffffu, ok));
    const int nlo = lo + c * step;
    hi = min(hi, nlo + step);
    lo = nlo;
  }
  return lo;
}

template <typename T>
__device__ __forceinline__ int find_segment_warp(const T *__restrict__ off, int n, T idx)
{
  const T first = __shfl_sync(0xffffffffu, idx, 0), last = __shfl_sync(0xffffffffu, idx, 31);
  const int s0 = find_segment_32ary(off, 0, n, first);
  const int s1 = (last == first) ? s0 : find_segment_32ary(off, s0, n, last);
  int lo = s0, hi = s1 + 1;
  while (hi - lo > 1)
  {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= idx)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Reference NEAREST macro (src/config_parser.h:218-219) in float.
__device__ __forceinline__ float nearest_f(float x, float half, float box)
{
  return x > half ? x - box : (x < -half ? x + box : x);
}
__device__ __forceinline__ double nearest_d(double x, double half, double box)
{
  return x > half ? x - box : (x < -half ? x + box : x);
}

// The octree is an array of 16-byte slots in depth-first preorder.
//   leaf (a particle): one slot  (x, y, z, m),             m >= 0 (sign bit clear)
//   cell:              two slots (x, y, z, -crit) (m, skip_bits, len, 0)
// The sign bit of w marks a cell; crit = len^2 / theta^2 (open when r^2 < crit);
// skip (an int stored in the float's bits) is the first slot after the
// subtree; len is the cell's side length.  A cell's first child starts two
// slots after it, and its children are the sibling subtrees up to its skip.
__device__ __forceinline__ bool slot_is_cell(float w) { return (__float_as_uint(w) & 0x80000000u) != 0; }

// Per-subhalo status while iterating.
enum SubState : int
{
  kActive = 0,
  kConverged = 1,
  kDisrupted = 2,
  kEmpty = 3,
  kMaxIter = 4
};

} // namespace hbtg
