// walk.cuh - the tree walk (GravityTree_t::EvaluatePotential,
// src/gravity_tree.cpp:82-166) for 32 targets at a time.
//
// One warp takes 32 neighbouring targets (key order) of one subhalo.  Each
// target's interaction list is exactly the reference's: the cells its own
// opening test accepts and the leaves it reaches.  The warp finds the union
// of those lists in one traversal and evaluates it in a second phase:
//
//   traversal   A stack in shared memory holds ranges of sibling subtrees
//               (first slot, end slot, the targets still walking them).  Each
//               step pops up to 32 ranges, one per lane; a lane reads its
//               range's first node and classifies it against the bounding
//               box of the targets: every target accepts it, every target
//               opens it, or (near the opening distance) each target decides
//               with its own test.  The node becomes an entry of the
//               interaction list with the mask of the targets that accept it;
//               the rest of the range and, if some targets open the node, its
//               children (with the mask of those targets) go back on the stack.
//               Nodes of the third kind wait in a pending list; once it holds
//               32 (or the stack is empty) each lane takes one and runs every
//               target's own test on it, two targets per packed FP32x2
//               operation, which gives its entry mask and its children's.
//   evaluation  Entries go to one of three lists: "far" entries, which every
//               target sees beyond the softening length (box distance), split
//               into those that every target takes (no selection at all) and
//               the rest, and "near" ones.  Whenever a list fills, every lane reads each
//               entry (a shared-memory broadcast) and adds the term of the
//               entries its mask bit selects: -m / r for the far list with no
//               branch, two entries at a time in packed FP32x2 arithmetic
//               (each half an IEEE FP32 operation, so the same values as
//               scalar code), and the cubic-spline softened kernel where
//               r < h for the near list.  Lists are padded to a multiple of
//               eight with massless entries; blocks of eight terms are summed
//               in FP32 and Kahan-added to the potential.
//
// Opening test.  The reference opens a cell when len^2 > r^2 theta^2, with
// len^2 in float and r^2 in double from the float coordinates
// (src/gravity_tree.cpp:137-145).  Here r^2 is FP32; outside a band of 1e-6
// relative around the stored threshold len^2 / theta^2 (far wider than the
// FP32 error of r^2 and of the threshold) the FP32 comparison decides as the
// reference does, and inside the band the reference's double arithmetic
// decides.  The bounding-box classifications use the same band, and the box
// distances are computed with the same monotonic FP32 operations as each
// target's own r^2, so "every target accepts" and "every target opens" never
// disagree with a target's own test.
//
// Bounds.  Stack pushes happen only in steps that start with at most
// kWalkDrain = kWalkStack - 64 ranges (a step pops k <= 32 ranges and pushes
// at most 2k, or resolves pending nodes and pushes at most 32); above that
// the warp drains the stack one range at a time, each target walking that
// range on its own with the reference's stackless walk (no pushes).  A list
// holding more than its capacity - 40 entries after a step (at most 32 added
// per step) is evaluated, so with its padding (at most 7) it never exceeds
// its capacity.  Pending nodes are added only by steps that start with fewer
// than 32 (at most 32 added), so at most 63 wait.  Every loop advances a slot
// index strictly or shrinks the pending list.
// A node's second slot is read for leaves too: the tree array carries one
// padding slot after its last slot.
#pragma once

#include "kernels.cuh"

namespace hbtg
{
namespace
{

// List and stack capacities (per warp); the defaults are the measured best on
// GB300 (overridable at build time for sweeps).  HBTG_WALK_MIN_BLOCKS, when
// defined, adds a minimum of resident blocks to the launch bounds (a register
// cap); by default the compiler's own allocation (72 registers, 7 blocks of 4
// warps per SM, limited equally by registers and shared memory) is kept.
#ifndef HBTG_WALK_FULL
#define HBTG_WALK_FULL 96
#endif
#ifndef HBTG_WALK_STACK
#define HBTG_WALK_STACK 256
#endif
constexpr int kWalkWarps = 4;   // warps per block
constexpr int kWalkFull = HBTG_WALK_FULL; // far-list entries that every target takes, per warp
constexpr int kWalkFar = 64;    // other far-list entries per warp
constexpr int kWalkNear = 64;   // near-list entries per warp
constexpr int kWalkStack = HBTG_WALK_STACK; // traversal ranges per warp
constexpr int kWalkDrain = kWalkStack - 64; // a deeper stack is drained (a step pushes at most 2 per lane)
constexpr int kWalkPending = 64; // cells waiting for the targets' own opening tests
constexpr int kWalkWarp2 = 16;  // target pairs per warp
constexpr int kFlushMargin = 40; // a list is evaluated once it holds more than capacity - this
constexpr float kBandLo = 1.f - 1e-6f, kBandHi = 1.f + 1e-6f;

// Per-lane walk counters (counted calls): see kWalkCounters.
struct WalkCount
{
  unsigned long long v[kWalkCounters];
};

// Lane 0 adds the clock cycles since t to counter q (counted calls only).
template <bool Count>
__device__ __forceinline__ void tick(WalkCount &cnt, int q, long long &t, int lane)
{
  if (!Count)
    return;
  const long long now = clock64();
  if (lane == 0)
    cnt.v[q] += (unsigned long long)(now - t);
  t = now;
}

struct WalkShared
{
  // far list, two entries per pair (packed FP32x2 evaluation): fa = (x0, x1,
  // y0, y1), fb = (z0, z1, m0, m1), fm = the two entries' target masks
  float4 fa[kWalkWarps][kWalkFar / 2];
  float4 fb[kWalkWarps][kWalkFar / 2];
  uint2 fm[kWalkWarps][kWalkFar / 2];
  // far list of entries that every target takes: ga = (x0, x1, y0, y1),
  // gb = (z0, z1, -m0, -m1)
  float4 ga[kWalkWarps][kWalkFull / 2];
  float4 gb[kWalkWarps][kWalkFull / 2];
  float4 near[kWalkWarps][kWalkNear];
  unsigned nmsk[kWalkWarps][kWalkNear];
  int ia[kWalkWarps][kWalkStack];       // range: first slot
  int ie[kWalkWarps][kWalkStack];       //        end slot
  unsigned im[kWalkWarps][kWalkStack];  //        targets still walking it
  int pa[kWalkWarps][kWalkPending];     // pending cell: slot
  unsigned pm[kWalkWarps][kWalkPending]; //              targets that reach it
  float4 txy[kWalkWarps][kWalkWarp2];   // targets, negated, in pairs: (x0, x1, y0, y1)
  float2 tz[kWalkWarps][kWalkWarp2];    //                             (z0, z1)
};

// a - b, with the periodic wrap of NEAREST (src/config_parser.h:218-219)
// formed without rounding the large intermediate a - b +- box: for a wrapped
// difference, a - box (or b - box) is exact (that operand is above half the
// box) and the result rounds once.
template <bool Wrap>
__device__ __forceinline__ float sep(float a, float b, const KParams &K)
{
  const float d = __fsub_rn(a, b);
  if (!Wrap)
    return d;
  return d > K.half ? __fsub_rn(__fsub_rn(a, K.box), b) : (d < -K.half ? __fsub_rn(a, __fsub_rn(b, K.box)) : d);
}

__device__ __forceinline__ float dist2(float dx, float dy, float dz)
{
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// The reference's opening decision in its own arithmetic: float len^2
// against r^2 theta^2 in double, r^2 from the float coordinates.
template <bool Wrap>
__device__ __noinline__ bool opens_exact(float cx, float cy, float cz, float lenf, float tx, float ty, float tz,
                                         const KParams &K)
{
  double d[3] = {(double)cx - (double)tx, (double)cy - (double)ty, (double)cz - (double)tz}; // exact
  if (K.periodic)
    for (int q = 0; q < 3; q++)
      d[q] = nearest_d(d[q], (double)K.half, (double)K.box);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
  return (double)__fmul_rn(lenf, lenf) > __dmul_rn(r2, (double)K.theta2);
}

// One target's test of a cell (centre c, threshold crit = len^2/theta^2).
template <bool Wrap>
__device__ __forceinline__ bool target_opens(float cx, float cy, float cz, float crit, float lenf, float tx, float ty,
                                             float tz, const KParams &K)
{
  const float r2 = dist2(sep<Wrap>(cx, tx, K), sep<Wrap>(cy, ty, K), sep<Wrap>(cz, tz, K));
  if (r2 < __fmul_rn(crit, kBandLo))
    return true;
  if (r2 > __fmul_rn(crit, kBandHi))
    return false;
  return opens_exact<Wrap>(cx, cy, cz, lenf, tx, ty, tz, K);
}

// Target t of the warp from the negated pairs.
__device__ __forceinline__ void target_at(const float4 *txy, const float2 *tz, int t, float &x, float &y, float &z)
{
  const float4 P = txy[t >> 1];
  const float2 Z = tz[t >> 1];
  const bool h = (t & 1) != 0;
  x = -(h ? P.y : P.x);
  y = -(h ? P.w : P.z);
  z = -(h ? Z.y : Z.x);
}

// Every target's own decision on one cell (centre c, threshold crit, side
// lenf): bit t set when target t (of the mask m) opens it.  Without the wrap,
// two targets per packed operation; each half is the FP32 operation of
// target_opens (c + (-t) is c - t exactly), so the decisions are the same.
template <bool Wrap>
__device__ __forceinline__ unsigned opens_mask(const float4 *txy, const float2 *tz, float cx, float cy, float cz,
                                               float crit, float lenf, unsigned m, const KParams &K)
{
  unsigned O = 0u;
  if (Wrap)
  {
    for (unsigned r = m; r; r &= r - 1u)
    {
      const int t = __ffs(r) - 1;
      float tx, ty, tzz;
      target_at(txy, tz, t, tx, ty, tzz);
      if (target_opens<true>(cx, cy, cz, crit, lenf, tx, ty, tzz, K))
        O |= 1u << t;
    }
    return O;
  }
  const float lo = __fmul_rn(crit, kBandLo), hi = __fmul_rn(crit, kBandHi);
  const float2 c_x = make_float2(cx, cx), c_y = make_float2(cy, cy), c_z = make_float2(cz, cz);
  unsigned B = 0u; // not beyond the band's far edge
#pragma unroll
  for (int q = 0; q < kWalkWarp2; q++)
  {
    const float4 P = txy[q];
    const float2 Z = tz[q];
    const float2 dx = __fadd2_rn(c_x, make_float2(P.x, P.y));
    const float2 dy = __fadd2_rn(c_y, make_float2(P.z, P.w));
    const float2 dz = __fadd2_rn(c_z, Z);
    float2 r2 = __fmul2_rn(dx, dx);
    r2 = __ffma2_rn(dy, dy, r2);
    r2 = __ffma2_rn(dz, dz, r2);
    O |= (r2.x < lo ? 1u : 0u) << (2 * q) | (r2.y < lo ? 2u : 0u) << (2 * q);
    B |= (r2.x > hi ? 0u : 1u) << (2 * q) | (r2.y > hi ? 0u : 2u) << (2 * q);
  }
  O &= m;
  // inside the band: the reference's double arithmetic
  for (unsigned r = B & m & ~O; r; r &= r - 1u)
  {
    const int t = __ffs(r) - 1;
    float tx, ty, tzz;
    target_at(txy, tz, t, tx, ty, tzz);
    if (opens_exact<false>(cx, cy, cz, lenf, tx, ty, tzz, K))
      O |= 1u << t;
  }
  return O;
}

// Squared distance from a point to the targets' bounding box.
__device__ __forceinline__ float box_gap2(const float *lo, const float *hi, float x, float y, float z)
{
  const float g[3] = {fmaxf(fmaxf(__fsub_rn(lo[0], x), __fsub_rn(x, hi[0])), 0.f),
                      fmaxf(fmaxf(__fsub_rn(lo[1], y), __fsub_rn(y, hi[1])), 0.f),
                      fmaxf(fmaxf(__fsub_rn(lo[2], z), __fsub_rn(z, hi[2])), 0.f)};
  return dist2(g[0], g[1], g[2]);
}

// The potential term of one entry for one target at squared distance r2.
__device__ __forceinline__ float softened_term(float m, float r2, const KParams &K, float h2)
{
  return r2 >= h2 ? -m * rsqrtf(r2) : m * K.h_inv * spline_w(sqrtf(r2) * K.h_inv);
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float v)
{
  const float y = v - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// A massless entry far from every target (finite terms, so the evaluation
// loops need no guard).
constexpr float kFarAway = 3e18f;

// Pads a list to a multiple of eight with massless entries; returns the
// padded length.  The caller leaves room for seven more entries.
__device__ __forceinline__ int pad8(float4 *ent, unsigned *msk, int n, int lane)
{
  const int padded = (n + 7) & ~7;
  if (n + lane < padded)
  {
    ent[n + lane] = make_float4(kFarAway, kFarAway, kFarAway, 0.f);
    msk[n + lane] = 0u;
  }
  __syncwarp();
  return padded;
}

// Writes far-list entry k (pair layout).
__device__ __forceinline__ void far_put(float4 *fa, float4 *fb, uint2 *fm, int k, float x, float y, float z, float m,
                                        unsigned mask)
{
  float *A = reinterpret_cast<float *>(fa + (k >> 1)), *B = reinterpret_cast<float *>(fb + (k >> 1));
  const int h = k & 1;
  A[h] = x;
  A[2 + h] = y;
  B[h] = z;
  B[2 + h] = m;
  reinterpret_cast<unsigned *>(fm + (k >> 1))[h] = mask;
}

__device__ __forceinline__ int pad8_far(float4 *fa, float4 *fb, uint2 *fm, int n, int lane)
{
  const int padded = (n + 7) & ~7;
  if (n + lane < padded)
    far_put(fa, fb, fm, n + lane, kFarAway, kFarAway, kFarAway, 0.f, 0u);
  __syncwarp();
  return padded;
}

// Far list: every target is at least one softening length from every entry
// (never used for wrapped subhaloes).  Two entries per packed operation.
__device__ __forceinline__ void eval_far(const float4 *fa, const float4 *fb, const uint2 *fm, int n, unsigned lanebit,
                                         float tx, float ty, float tz, float &sum, float &comp)
{
  const float2 ntx = make_float2(-tx, -tx), nty = make_float2(-ty, -ty), ntz = make_float2(-tz, -tz);
  for (int i = 0; i < n; i += 8)
  {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      const int pp = (i >> 1) + q;
      const float4 A = fa[pp], B = fb[pp];
      const uint2 mk = fm[pp];
      const float2 dx = __fadd2_rn(make_float2(A.x, A.y), ntx); // entry - target, exact as a subtraction
      const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nty);
      const float2 dz = __fadd2_rn(make_float2(B.x, B.y), ntz);
      float2 r2 = __fmul2_rn(dx, dx);
      r2 = __ffma2_rn(dy, dy, r2);
      r2 = __ffma2_rn(dz, dz, r2);
      const float2 rs = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
      const float2 nm = make_float2((mk.x & lanebit) ? -B.z : 0.f, (mk.y & lanebit) ? -B.w : 0.f);
      acc = __ffma2_rn(nm, rs, acc);
    }
    kahan_add(sum, comp, acc.x + acc.y);
  }
}

// Writes entry k of the far list that every target takes.
__device__ __forceinline__ void full_put(float4 *ga, float4 *gb, int k, float x, float y, float z, float m)
{
  float *A = reinterpret_cast<float *>(ga + (k >> 1)), *B = reinterpret_cast<float *>(gb + (k >> 1));
  const int h = k & 1;
  A[h] = x;
  A[2 + h] = y;
  B[h] = z;
  B[2 + h] = -m;
}

__device__ __forceinline__ int pad8_full(float4 *ga, float4 *gb, int n, int lane)
{
  const int padded = (n + 7) & ~7;
  if (n + lane < padded)
    full_put(ga, gb, n + lane, kFarAway, kFarAway, kFarAway, 0.f);
  __syncwarp();
  return padded;
}

// The far list that every target takes: no per-entry selection.
__device__ __forceinline__ void eval_full(const float4 *ga, const float4 *gb, int n, float tx, float ty, float tz,
                                          float &sum, float &comp)
{
  const float2 ntx = make_float2(-tx, -tx), nty = make_float2(-ty, -ty), ntz = make_float2(-tz, -tz);
  for (int i = 0; i < n; i += 8)
  {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      const int pp = (i >> 1) + q;
      const float4 A = ga[pp], B = gb[pp];
      const float2 dx = __fadd2_rn(make_float2(A.x, A.y), ntx);
      const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nty);
      const float2 dz = __fadd2_rn(make_float2(B.x, B.y), ntz);
      float2 r2 = __fmul2_rn(dx, dx);
      r2 = __ffma2_rn(dy, dy, r2);
      r2 = __ffma2_rn(dz, dz, r2);
      const float2 rs = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
      acc = __ffma2_rn(make_float2(B.z, B.w), rs, acc);
    }
    kahan_add(sum, comp, acc.x + acc.y);
  }
}

// Near list: the softened kernel where r < h (src/gravity_tree.cpp:150-162).
template <bool Wrap>
__device__ __forceinline__ void eval_near(const float4 *ent, const unsigned *msk, int n, unsigned lanebit, float tx,
                                          float ty, float tz, const KParams &K, float h2, float &sum, float &comp)
{
  const unsigned full = 0xffffffffu;
  for (int i = 0; i < n; i += 8)
  {
    float part = 0.f;
#pragma unroll 2
    for (int u = 0; u < 8; u++)
    {
      const float4 e = ent[i + u];
      const float m = (msk[i + u] & lanebit) ? e.w : 0.f;
      const float r2 = dist2(sep<Wrap>(e.x, tx, K), sep<Wrap>(e.y, ty, K), sep<Wrap>(e.z, tz, K));
      // the softened form only when some lane is inside the softening length
      // (its square root and polynomial are skipped otherwise)
      float t;
      if (__any_sync(full, r2 < h2))
        t = softened_term(m, r2, K, h2);
      else
        t = -m * rsqrtf(r2);
      part += t;
    }
    kahan_add(sum, comp, part);
  }
}

// The reference's stackless walk of one range [a, e) of sibling subtrees for
// one target (open: next slot; accept: interact and skip the subtree).
template <bool Wrap>
__device__ __forceinline__ void walk_range(const float4 *__restrict__ T, int a, int e, float tx, float ty, float tz,
                                           const KParams &K, float h2, float &sum, float &comp, WalkCount &cnt)
{
  int idx = a;
  while (idx < e)
  {
    const float4 n = __ldg(&T[idx]);
    float m;
    int next;
    if (slot_is_cell(n.w))
    {
      const float4 b = __ldg(&T[idx + 1]);
      const float crit = __uint_as_float(__float_as_uint(n.w) & 0x7fffffffu);
      if (target_opens<Wrap>(n.x, n.y, n.z, crit, b.z, tx, ty, tz, K))
      {
        idx += 2;
        continue;
      }
      m = b.x;
      next = __float_as_int(b.y);
    }
    else
    {
      m = n.w;
      next = idx + 1;
    }
    const float r2 = dist2(sep<Wrap>(n.x, tx, K), sep<Wrap>(n.y, ty, K), sep<Wrap>(n.z, tz, K));
    kahan_add(sum, comp, softened_term(m, r2, K, h2));
    cnt.v[0]++;
    idx = max(next, idx + 1);
  }
}

// Potentials of the (up to) 32 targets of chunk c.
template <bool Wrap, bool Count>
__device__ __forceinline__ void walk_group(const DevState &D, const KParams &K, int s, int root, int lane, bool valid,
                                           int p, float4 x, float self, WalkShared &sh, int w, WalkCount &cnt)
{
  const float4 *__restrict__ T = D.nodes;
  float4 *fa = sh.fa[w], *fb = sh.fb[w], *nea = sh.near[w], *ga = sh.ga[w], *gb = sh.gb[w];
  uint2 *fm = sh.fm[w];
  unsigned *nmsk = sh.nmsk[w];
  int *ia = sh.ia[w], *ie = sh.ie[w];
  unsigned *im = sh.im[w];
  const unsigned full = 0xffffffffu, lanebit = 1u << lane, below = lanebit - 1u;
  const float h2 = K.h * K.h;
  long long t_all = Count ? clock64() : 0, t = t_all;
  const unsigned vmask = __ballot_sync(full, valid);
  // bounding box of the targets
  float lo[3] = {valid ? x.x : INFINITY, valid ? x.y : INFINITY, valid ? x.z : INFINITY};
  float hi[3] = {valid ? x.x : -INFINITY, valid ? x.y : -INFINITY, valid ? x.z : -INFINITY};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      lo[d] = fminf(lo[d], __shfl_xor_sync(full, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(full, hi[d], o));
    }
  float sum = valid ? self / K.soft : 0.f, comp = 0.f;
  if (lane == 0)
  {
    ia[0] = root;
    ie[0] = __float_as_int(__ldg(&T[root + 1]).y);
    im[0] = vmask;
  }
  // the targets, negated, in pairs (the pending cells' tests read them)
  {
    float *X = reinterpret_cast<float *>(sh.txy[w]), *Z = reinterpret_cast<float *>(sh.tz[w]);
    const int q = lane >> 1, hh = lane & 1;
    X[4 * q + hh] = valid ? -x.x : 0.f;
    X[4 * q + 2 + hh] = valid ? -x.y : 0.f;
    Z[2 * q + hh] = valid ? -x.z : 0.f;
  }
  int *pa = sh.pa[w];
  unsigned *pmk = sh.pm[w];
  int sp = 1, np = 0, nf = 0, ng = 0, nn = 0;
  __syncwarp();
  tick<Count>(cnt, 8, t, lane);
  while (sp > 0 || np > 0)
  {
    if (sp > kWalkDrain)
    { // drain: each target walks the top range on its own
      sp--;
      const int a = ia[sp], e = ie[sp];
      const unsigned m = im[sp];
      __syncwarp();
      if (m & lanebit)
        walk_range<Wrap>(T, a, e, x.x, x.y, x.z, K, h2, sum, comp, cnt);
      if (Count && lane == 0)
        cnt.v[7]++;
      tick<Count>(cnt, 14, t, lane);
      continue;
    }
    bool act, cell = false, near = true;
    int a = 0, e = 0;
    unsigned m = 0u, A = 0u, O = 0u;
    float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = make_float4(0.f, 0.f, 0.f, 0.f);
    if (np >= kWarp || sp == 0)
    { // resolve up to 32 pending cells, one per lane, each against every target
      const int k = min(np, kWarp);
      act = lane < k;
      if (Count && lane == 0)
        cnt.v[3]++;
      if (act)
      {
        a = pa[np - k + lane];
        m = pmk[np - k + lane];
      }
      np -= k;
      __syncwarp();
      if (act)
      {
        na = __ldg(&T[a]);
        nb = __ldg(&T[a + 1]);
        cell = true;
        e = __float_as_int(nb.y); // the cell's siblings are on the stack already
        if (!Wrap)
          near = box_gap2(lo, hi, na.x, na.y, na.z) < h2;
        O = opens_mask<Wrap>(sh.txy[w], sh.tz[w], na.x, na.y, na.z,
                             __uint_as_float(__float_as_uint(na.w) & 0x7fffffffu), nb.z, m, K);
        A = m & ~O;
      }
      tick<Count>(cnt, 9, t, lane);
    }
    else
    { // the first nodes of up to 32 ranges, one per lane
      const int k = min(sp, kWarp);
      const int base = sp - k;
      act = lane < k;
      if (Count && lane == 0)
      {
        cnt.v[1]++;
        cnt.v[2] += k;
      }
      if (act)
      {
        a = ia[base + lane];
        e = ie[base + lane];
        m = im[base + lane];
      }
      sp = base;
      __syncwarp();
      int cls = 0; // 0: every target accepts, 1: every target opens, 2: each target decides
      if (act)
      {
        na = __ldg(&T[a]);
        nb = __ldg(&T[a + 1]); // a cell's mass, skip and side length (the tree has a padding slot)
        cell = slot_is_cell(na.w);
        if (Wrap)
          cls = cell ? 2 : 0;
        else
        {
          const float rmin2 = box_gap2(lo, hi, na.x, na.y, na.z);
          near = rmin2 < h2;
          if (cell)
          {
            const float crit = __uint_as_float(__float_as_uint(na.w) & 0x7fffffffu);
            if (!(rmin2 > __fmul_rn(crit, kBandHi)))
            {
              const float G[3] = {fmaxf(fabsf(__fsub_rn(na.x, lo[0])), fabsf(__fsub_rn(na.x, hi[0]))),
                                  fmaxf(fabsf(__fsub_rn(na.y, lo[1])), fabsf(__fsub_rn(na.y, hi[1]))),
                                  fmaxf(fabsf(__fsub_rn(na.z, lo[2])), fabsf(__fsub_rn(na.z, hi[2])))};
              cls = dist2(G[0], G[1], G[2]) < __fmul_rn(crit, kBandLo) ? 1 : 2;
            }
          }
        }
      }
      A = cls == 0 ? m : 0u;
      O = cls == 1 ? m : 0u;
      // cells near the targets' opening distance wait for a batch of their own
      const unsigned bp = __ballot_sync(full, act && cls == 2);
      if (act && cls == 2)
      {
        const int at = np + __popc(bp & below);
        pa[at] = a;
        pmk[at] = m;
      }
      np += __popc(bp);
      tick<Count>(cnt, 8, t, lane);
    }
    const bool has_e = act && A != 0u;
    const bool to_near = Wrap || near, every = A == vmask;
    const unsigned bg = __ballot_sync(full, has_e && !to_near && every),
                   bf = __ballot_sync(full, has_e && !to_near && !every), bn = __ballot_sync(full, has_e && to_near);
    if (has_e)
    {
      const float4 en = make_float4(na.x, na.y, na.z, cell ? nb.x : na.w);
      if (to_near)
      {
        const int at = nn + __popc(bn & below);
        nea[at] = en;
        nmsk[at] = A;
      }
      else if (every)
        full_put(ga, gb, ng + __popc(bg & below), en.x, en.y, en.z, en.w);
      else
        far_put(fa, fb, fm, nf + __popc(bf & below), en.x, en.y, en.z, en.w, A);
      if (Count)
        cnt.v[0] += __popc(A);
    }
    if (Count && lane == 0)
    {
      cnt.v[4] += __popc(bg);
      cnt.v[5] += __popc(bf);
      cnt.v[6] += __popc(bn);
    }
    ng += __popc(bg);
    nf += __popc(bf);
    nn += __popc(bn);
    // the rest of each range, then the children of opened cells (popped first: depth first)
    const int next = cell ? __float_as_int(nb.y) : a + 1;
    const bool has_sib = act && next < e, has_kid = act && O != 0u;
    const unsigned bs = __ballot_sync(full, has_sib), bk = __ballot_sync(full, has_kid);
    if (has_sib)
    {
      const int at = sp + __popc(bs & below);
      ia[at] = next;
      ie[at] = e;
      im[at] = m;
    }
    sp += __popc(bs);
    if (has_kid)
    {
      const int at = sp + __popc(bk & below);
      ia[at] = a + 2;
      ie[at] = next;
      im[at] = O;
    }
    sp += __popc(bk);
    __syncwarp();
    tick<Count>(cnt, 10, t, lane);
    if (ng > kWalkFull - kFlushMargin)
    {
      eval_full(ga, gb, pad8_full(ga, gb, ng, lane), x.x, x.y, x.z, sum, comp);
      ng = 0;
      __syncwarp();
      tick<Count>(cnt, 11, t, lane);
    }
    if (nf > kWalkFar - kFlushMargin)
    {
      eval_far(fa, fb, fm, pad8_far(fa, fb, fm, nf, lane), lanebit, x.x, x.y, x.z, sum, comp);
      nf = 0;
      __syncwarp();
      tick<Count>(cnt, 12, t, lane);
    }
    if (nn > kWalkNear - kFlushMargin)
    {
      eval_near<Wrap>(nea, nmsk, pad8(nea, nmsk, nn, lane), lanebit, x.x, x.y, x.z, K, h2, sum, comp);
      nn = 0;
      __syncwarp();
      tick<Count>(cnt, 13, t, lane);
    }
  }
  eval_full(ga, gb, pad8_full(ga, gb, ng, lane), x.x, x.y, x.z, sum, comp);
  tick<Count>(cnt, 11, t, lane);
  eval_far(fa, fb, fm, pad8_far(fa, fb, fm, nf, lane), lanebit, x.x, x.y, x.z, sum, comp);
  tick<Count>(cnt, 12, t, lane);
  eval_near<Wrap>(nea, nmsk, pad8(nea, nmsk, nn, lane), lanebit, x.x, x.y, x.z, K, h2, sum, comp);
  __syncwarp();
  tick<Count>(cnt, 13, t, lane);
  t = t_all;
  tick<Count>(cnt, 15, t, lane);
  if (valid)
    D.pot[p] = (sum - comp) * K.G_over_a;
}

// One 32-target chunk: its subhalo, targets and self terms (as the
// reference: a target that is a tree source starts from +m/soft, cancelling
// its own leaf, src/gravity_tree.cpp:98-101).
template <bool Count>
__device__ __forceinline__ void walk_chunk(const DevState &D, const KParams &K, int c, int lane, WalkShared &sh,
                                           int w, WalkCount &cnt)
{
  const int s = find_segment_warp(D.chunk_off, D.S, c); // c is the same on every lane
  const int t = (c - D.chunk_off[s]) * kWarp + lane;
  const bool valid = t < D.tgt_cnt[s];
  const bool corr = D.corr[s] != 0;
  const int ngrav = D.ngrav[s];
  int p = 0;
  if (valid) // correction: key-ordered bound set; subsampled: every candidate; else the sources
    p = corr ? D.tgt[D.off[s] + t] : (ngrav ? D.ord[D.off[s] + t] : (int)D.val[D.src_off[s] + t]);
  const float4 x = valid ? D.pm[p] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int nself = (corr && D.self_cnt) ? D.self_cnt[s] : 0;
  const float self =
    !valid ? 0.f : (corr ? (t < nself ? x.w : 0.f) : (ngrav ? (t < ngrav ? source_mass(D, s, p) : 0.f) : x.w));
  if (D.src_cnt[s] == 0)
  { // no sources this iteration: zero potential
    if (valid)
      D.pot[p] = 0.f;
    return;
  }
  const int root = D.src_off[s] + 2 * D.X[D.src_off[s]];
  if (D.wrap[s])
    walk_group<true, Count>(D, K, s, root, lane, valid, p, x, self, sh, w, cnt);
  else
    walk_group<false, Count>(D, K, s, root, lane, valid, p, x, self, sh, w, cnt);
}

// With walk counters, the chunks (key order) are split into `nranges`
// contiguous ranges of `per` chunks, one per SM (the host picks nranges so
// that every range holds a chunk): the warps resident on an SM take the
// chunks of their own range in order, so they walk neighbouring targets and
// share the tree slots in L1; a warp whose range is used up moves on to the
// next ranges (each tried once).  Without counters, a grid-stride loop.
template <bool Count>
#ifdef HBTG_WALK_MIN_BLOCKS
__global__ void __launch_bounds__(32 * kWalkWarps, HBTG_WALK_MIN_BLOCKS)
#else
__global__ void __launch_bounds__(32 * kWalkWarps)
#endif
  k_walk(DevState D, KParams K, int total_chunks, int nranges)
{
  __shared__ WalkShared sh;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WalkCount cnt = {};
  if (D.walk_ctr)
  {
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    const int per = (total_chunks + nranges - 1) / nranges;
    int r = (int)(smid % (unsigned)nranges);
    for (int tries = 0; tries < nranges;)
    {
      int got = 0;
      if (lane == 0)
        got = (int)atomicAdd(&D.walk_ctr[r], 1u);
      got = __shfl_sync(0xffffffffu, got, 0);
      const long long c = (long long)r * per + got;
      if (got >= per || c >= total_chunks)
      {
        r = (r + 1 == nranges) ? 0 : r + 1;
        tries++;
        continue;
      }
      walk_chunk<Count>(D, K, (int)c, lane, sh, w, cnt);
    }
  }
  else
  {
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int c = warp_global; c < total_chunks; c += nwarps)
      walk_chunk<Count>(D, K, c, lane, sh, w, cnt);
  }
  if (Count)
    for (int q = 0; q < kWalkCounters; q++)
    {
      unsigned long long v = cnt.v[q];
      for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0)
        atomicAdd(D.interactions + q, v);
    }
}

} // namespace
} // namespace hbtg
