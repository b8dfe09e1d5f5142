// kernels.cuh - device kernels of the batched unbinding iteration.
//
// Every subhalo of the batch is a segment of the particle arrays.  All
// subhaloes that are still iterating advance together: each lock-step
// iteration runs the same kernel sequence over the "active" segments, packed
// by device-side exclusive scans of per-subhalo counts (src_off, chunk_off,
// part_off, ...).  A packed item j is mapped back to its subhalo by a search
// over the packed offsets (warp-cooperative in the per-item kernels:
// find_segment_warp).  FP64 throughput is low on this GPU (about 1/64 of
// FP32, and 64-bit integer/float conversions issue to the same pipe), so the
// per-item kernels use FP32 and integer arithmetic, with error-free
// transforms or fixed point where the reference accumulates in double.
//
// Reference correspondence (HBT-HERONS):
//   k_bbox/k_root   bounding cube of the tree        src/oct_tree.tpp:27-47
//   k_keys          insertion descent, as key digits src/oct_tree.tpp:52-92
//   k_tree_*        octree + multipoles              src/oct_tree.tpp:52-136, src/gravity_tree.cpp:25-80
//   k_walk          EvaluatePotential                src/gravity_tree.cpp:82-166
//   k_energy        BindingEnergy + correction loop  src/gravity_tree.cpp:168-178, src/subhalo_unbind.cpp:563-621
//   k_part_*        RemoveUnboundParticles           src/subhalo_unbind.cpp:35-44, 626
//   k_after_part    tracer count, disruption, CorrectionLoop flag  src/subhalo_unbind.cpp:630-683
//   k_com/k_control CentreOfMassReferenceFrame, convergence        src/subhalo_unbind.cpp:151-198, 687-690
//   k_epilogue      AverageKinematics, CountParticleTypes, GetCorePhaseSpaceProperties,
//                   binding/potential energies      src/subhalo_unbind.cpp:200-249,764-802,
//                                                   src/subhalo.cpp:311-393, src/subhalo_merge.cpp:94-181
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "primitives.cuh"

namespace hbtg
{
// Internal linkage: each translation unit that launches these kernels gets its own copy.
namespace
{

// Values of HBTConfig / Cosmology as the reference stores them (HBTReal = float).
struct KParams
{
  float box, half;
  int periodic;
  float soft;     // GetCurrentSoftening(a)
  float h, h_inv; // 2.8 * soft and its inverse (spline support)
  float res;      // TreeNodeResolution
  float theta2;   // TreeNodeOpenAngleSquare
  float bmp;      // BoundMassPrecision
  int min_part, min_tracer;
  int tracer_mask;
  int dm_only, thermal;
  float G_over_a, a, hz;
  int max_iter;
  long long core_min;
  float core_factor;
  int count_interactions;
  int max_sample;       // MaxSampleSizeOfPotentialEstimate (0 = off)
  int nosub_mask;       // DoNotSubsampleParticleBitMask
  int upscale_per_type; // PotentialEstimateUpscaleMassesPerType
  int refine;           // RefineMostBoundParticle (with subsampling on)
  float refine_frac;    // BoundFractionCenterRefinement
};

// Device views of the batch state.
struct DevState
{
  int S;
  long long N;
  const long long *off; // [S+1]
  // particles
  float4 *pm; // x, y, z, mass
  float4 *vu; // vx, vy, vz, internal energy
  uint8_t *ty; // bits 0-2 type, bit 3 tracer
  int *seg_of; // subhalo of each particle
  int *ord, *ord_tmp; // current energy order: global particle index at each position
  int *sp;            // per subhalo: its particles in key order at the last full tree build
  int *tgt;           // per subhalo: correction-walk targets (bound particles in key order)
  uint8_t *bnd;       // 1 while a particle is in its subhalo's bound set
  float *Ep;  // binding energy per particle
  float *pot; // tree potential per particle (G/a applied)
  const long long *id;
  // subhaloes
  int *n_s, *nbound, *nlast, *state, *corr, *iter, *wrap, *tracers, *nb_new;
  float *ref_pos, *ref_vel, *old_pos, *old_vel, *mb_pos, *mb_vel, *mbound;
  long long *mb_id;
  // per-iteration plan
  int *src_begin, *src_cnt, *src_off, *tgt_cnt, *chunk_cnt, *chunk_off, *part_cnt, *part_off;
  int *tail_cnt, *tail_off, *fin_cnt, *fin_off;
  int *sp_cnt, *sp_off;    // correction subhaloes: key-order list lengths and packing
  int *sp_len;             // length of each subhalo's key-order list
  int *nunsample;          // leading particles exempt from subsampling (CountUnsampledParticles)
  int *ngrav;              // tree sources of a subsampled iteration (0 = not subsampled)
  float *factor;           // [6S] mass upscale factor per type of the current iteration
  unsigned *bb_lo, *bb_hi; // ordered-float bounding boxes [3S]
  double *root;            // [4S] centre xyz, side length
  float *keyp;             // [12S] per-axis origin hi/lo, 2^21/side, exact levels, halvings (see k_root)
  int *fb_list, *fb_count; // packed items whose key needs the exact double descent
  double *com;             // [7S] M, sum m dx, sum m v (epilogue: kinematics sums)
  double *com_part;        // [7 x blocks] per-block frame sums of single-subhalo k_com blocks
  int com_ipt = 16;        // items per thread of the k_com launch whose sums k_control / k_frame_flagged read
  // packed arrays
  unsigned long long *key, *key_alt;
  uint32_t *val, *val_alt, *k32, *k32_alt, *perm, *perm_alt;
  int *cnt, *X, *flags, *F;
  int *cell_list; // tree cells (first slot) grouped by level (k_tree_emit), for the bottom-up passes
  int *lvl;       // [2 kLevels]: cells per level (k_tree_count), fill cursors (k_tree_emit)
  float4 *nodes; // tree slots (see slot_is_cell)
  unsigned long long *interactions; // [kWalkCounters]: interactions, then the walk's traversal counters
  int *nb1 = nullptr; // Nbound after the first iteration (training traces), or null
  unsigned *walk_ctr = nullptr; // per-SM chunk counters of the walk (zeroed before each walk), or null
  // warm start (null on the plain path)
  int *warm = nullptr;       // 1 = started from a proposal, 2 = restarted cold, 3 = warm start verified
  int *nexcl = nullptr;      // particles the proposal excluded (parked at the end of the segment at the start)
  int *iter_extra = nullptr; // iterations spent before a cold restart
  int *flag_s = nullptr;     // per-subhalo scratch flag of the warm-start stages
  int *self_cnt = nullptr;   // leading targets of a correction-type walk that are also sources
  int *ntest = nullptr;      // particles the first test evaluates
  float *ref0 = nullptr;     // [6S] input frame, restored for a cold restart
};

// Tree levels: keys hold 21 digits, so cells sit at levels 0..21.
constexpr int kLevels = 32;
// walk counters (with counting on): interactions, traversal steps, nodes
// popped, pending-cell batches, entries of the three lists, drained ranges,
// then warp clock cycles spent in: popping and classifying, resolving
// pending cells, list and stack writes, the three list evaluations,
// draining, and whole target groups
constexpr int kWalkCounters = 16;

__device__ __forceinline__ int lcp_levels(unsigned long long a, unsigned long long b)
{
  // keys hold 21 levels of 3 bits in bits 62..0; bit 63 is zero
  return (a == b) ? 21 : (__clzll(a ^ b) - 1) / 3;
}

__device__ __forceinline__ bool is_tracer_bits(uint8_t t) { return (t & 8u) != 0; }
__device__ __forceinline__ bool is_nosub_bits(uint8_t t) { return (t & 16u) != 0; }

// EnergySnapshot_t::GetMass (src/subhalo_unbind.cpp:91-101): the particle mass
// times its type's upscale factor, except for types exempt from subsampling.
__device__ __forceinline__ float source_mass(const DevState &D, int s, int p)
{
  const float m = D.pm[p].w;
  const uint8_t t = D.ty[p];
  return is_nosub_bits(t) ? m : __fmul_rn(m, D.factor[6 * s + (t & 7)]);
}

// ---------------------------------------------------------------------------
// Set-up
// ---------------------------------------------------------------------------
__global__ void k_repack(DevState D, KParams K, const float *__restrict__ pos, const float *__restrict__ vel,
                         const float *__restrict__ mass, const float *__restrict__ u, const uint8_t *__restrict__ type)
{
  // one particle per thread (the grid covers N); the whole warp looks up the subhaloes
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp<long long>(D.off, D.S, min(i, D.N - 1));
  if (i < D.N)
  {
    D.pm[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], mass[i]);
    D.vu[i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], (K.thermal && u) ? u[i] : 0.f);
    int t = K.dm_only ? 1 : (type ? (int)type[i] : 1);
    t = t < 0 ? 0 : (t > 5 ? 5 : t);
    const bool tr = K.dm_only || ((1 << t) & K.tracer_mask);
    const bool ns = !K.dm_only && ((1 << t) & K.nosub_mask);
    D.ty[i] = (uint8_t)(t | (tr ? 8 : 0) | (ns ? 16 : 0));
    D.seg_of[i] = s;
    D.ord[i] = (int)i;
    D.bnd[i] = 1;
  }
}

__global__ void k_init_subs(DevState D, KParams K)
{
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < D.S; s += gridDim.x * blockDim.x)
  {
    const int n = (int)(D.off[s + 1] - D.off[s]);
    D.n_s[s] = n;
    D.nbound[s] = n;
    D.nlast[s] = n;
    D.state[s] = n > 0 ? kActive : kEmpty;
    D.corr[s] = 0;
    D.iter[s] = 0;
    D.wrap[s] = 0;
    D.tracers[s] = 0;
    D.mbound[s] = 0.f;
    D.ngrav[s] = 0;
    for (int t = 0; t < 6; t++)
      D.factor[6 * s + t] = 1.f;
    // PrepareParticlesForSubsampling put the exempt types first (done by the caller)
    int ns = 0;
    if (K.max_sample > 0 && n > K.max_sample)
      while (ns < n && is_nosub_bits(D.ty[D.off[s] + ns]))
        ns++;
    D.nunsample[s] = ns;
  }
}

// Per-iteration plan: ranges of tree sources, walk targets and partition.
__global__ void k_plan(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s > D.S)
    return;
  if (s == D.S)
  { // trailing zero so that the exclusive scans yield the totals
    D.src_cnt[s] = D.chunk_cnt[s] = D.part_cnt[s] = D.sp_cnt[s] = 0;
    return;
  }
  if (D.state[s] != kActive)
  {
    D.src_cnt[s] = D.chunk_cnt[s] = D.part_cnt[s] = D.tgt_cnt[s] = D.sp_cnt[s] = 0;
    return;
  }
  D.iter[s] += 1;
  int tgt;
  D.ngrav[s] = 0;
  for (int t = 0; t < 6; t++)
    D.factor[6 * s + t] = 1.f;
  if (!D.corr[s])
  {
    D.nlast[s] = D.nbound[s];
    D.src_begin[s] = 0;
    D.src_cnt[s] = D.nlast[s];
    tgt = D.nlast[s];
    // SetMassUpscaleFactor (src/subhalo_unbind.cpp:374-391): only the leading
    // MaxSample (+ exempt) particles are tree sources; k_upscale sets the factors
    if (K.max_sample > 0 && !(D.nlast[s] < K.max_sample + D.nunsample[s]))
    {
      D.ngrav[s] = K.max_sample + D.nunsample[s];
      D.src_cnt[s] = D.ngrav[s];
    }
  }
  else
  {
    D.src_begin[s] = D.nbound[s];
    D.src_cnt[s] = D.nlast[s] - D.nbound[s];
    tgt = D.nbound[s];
    D.nlast[s] = D.nbound[s];
  }
  D.tgt_cnt[s] = tgt;
  D.chunk_cnt[s] = (tgt + kWarp - 1) / kWarp;
  D.part_cnt[s] = D.nlast[s];
  // a full build records the key order (sp_len); a correction walk compacts it
  if (!D.corr[s])
  {
    D.sp_len[s] = D.nlast[s];
    D.sp_cnt[s] = 0;
  }
  else
    D.sp_cnt[s] = D.sp_len[s];
  D.bb_lo[3 * s] = D.bb_lo[3 * s + 1] = D.bb_lo[3 * s + 2] = 0xffffffffu;
  D.bb_hi[3 * s] = D.bb_hi[3 * s + 1] = D.bb_hi[3 * s + 2] = 0u;
  D.tracers[s] = 0;
}

// ---------------------------------------------------------------------------
// Tree build
// ---------------------------------------------------------------------------
__device__ __forceinline__ int src_particle(const DevState &D, int s, int j)
{
  const int k = D.src_begin[s] + (j - D.src_off[s]);
  return D.ord[D.off[s] + k];
}

// Per-subhalo bounding boxes of the sources (ordered-float min/max atomics).
// A block covers kBboxRows x 256 consecutive items; when they all belong to
// one subhalo (the common case for large subhaloes, whose atomics would
// otherwise all meet on the same six words) the block reduces them first and
// issues one set of atomics, else each warp reduces each row per subhalo.
constexpr int kBboxRows = 4;

__global__ void __launch_bounds__(256) k_bbox(DevState D, int total)
{
  __shared__ unsigned s_red[8][6];
  const long long tile0 = (long long)blockIdx.x * (256 * kBboxRows);
  const int jl = (int)min((long long)total - 1, tile0 + 256 * kBboxRows - 1);
  const int s_first = find_segment_warp(D.src_off, D.S, (int)tile0); // the same on every lane
  const int s_last = find_segment_warp(D.src_off, D.S, jl);
  unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  if (s_first == s_last)
  {
#pragma unroll
    for (int r = 0; r < kBboxRows; r++)
    {
      const long long j = tile0 + r * 256 + threadIdx.x;
      if (j < total)
      {
        const int p = src_particle(D, s_first, (int)j);
        const float4 x = D.pm[p];
        const unsigned v[3] = {float_to_ordered(x.x), float_to_ordered(x.y), float_to_ordered(x.z)};
#pragma unroll
        for (int d = 0; d < 3; d++)
        {
          lo[d] = min(lo[d], v[d]);
          hi[d] = max(hi[d], v[d]);
        }
      }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      lo[d] = __reduce_min_sync(0xffffffffu, lo[d]);
      hi[d] = __reduce_max_sync(0xffffffffu, hi[d]);
    }
    if (lane == 0)
    {
#pragma unroll
      for (int d = 0; d < 3; d++)
      {
        s_red[warp][d] = lo[d];
        s_red[warp][3 + d] = hi[d];
      }
    }
    __syncthreads();
    if (threadIdx.x < 6)
    {
      const int q = threadIdx.x;
      unsigned v = s_red[0][q];
      for (int w = 1; w < 8; w++)
        v = q < 3 ? min(v, s_red[w][q]) : max(v, s_red[w][q]);
      if (q < 3)
        atomicMin(&D.bb_lo[3 * s_first + q], v);
      else
        atomicMax(&D.bb_hi[3 * s_first + q - 3], v);
    }
    return;
  }
#pragma unroll 1
  for (int r = 0; r < kBboxRows; r++)
  {
    const long long jj = tile0 + r * 256 + threadIdx.x;
    const bool valid = jj < total;
    const int j = (int)jj;
    const int sw = find_segment_warp(D.src_off, D.S, min(j, total - 1));
    const int s = valid ? sw : -1;
    unsigned l[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, h[3] = {0u, 0u, 0u};
    if (valid)
    {
      const int p = src_particle(D, s, j);
      const float4 x = D.pm[p];
      l[0] = h[0] = float_to_ordered(x.x);
      l[1] = h[1] = float_to_ordered(x.y);
      l[2] = h[2] = float_to_ordered(x.z);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, s);
    const int leader = __ffs(peers) - 1;
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      l[d] = __reduce_min_sync(peers, l[d]);
      h[d] = __reduce_max_sync(peers, h[d]);
    }
    if (valid && (int)(threadIdx.x & 31) == leader)
    {
#pragma unroll
      for (int d = 0; d < 3; d++)
      {
        atomicMin(&D.bb_lo[3 * s + d], l[d]);
        atomicMax(&D.bb_hi[3 * s + d], h[d]);
      }
    }
  }
}

// Root cube (src/oct_tree.tpp:44-65): centre of the box, side = largest extent.
// Built for every subhalo with sources: the active ones, and the converged
// ones whose most-bound prefix gets its own tree (RefineBindingEnergyOrder).
__global__ void k_root(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S || D.src_cnt[s] == 0 || (D.state[s] != kActive && D.state[s] != kConverged))
    return;
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++)
  {
    lo[d] = ordered_to_float(D.bb_lo[3 * s + d]);
    hi[d] = ordered_to_float(D.bb_hi[3 * s + d]);
  }
  double len = hi[0] - lo[0];
  for (int d = 1; d < 3; d++)
    if (hi[d] - lo[d] > len)
      len = hi[d] - lo[d];
  for (int d = 0; d < 3; d++)
    D.root[4 * s + d] = 0.5 * (hi[d] + lo[d]);
  D.root[4 * s + 3] = len;
  // fast-descent constants: origin of the root cube per axis as a float pair,
  // 2^21 / side, and the number of levels that must match the reference
  // exactly (cells not smaller than TreeNodeResolution, plus one)
  float *kp = D.keyp + 12 * s;
  for (int d = 0; d < 3; d++)
  {
    const double o = 0.5 * (hi[d] + lo[d]) - 0.5 * len;
    kp[d] = (float)o;
    kp[3 + d] = (float)(o - (double)(float)o);
  }
  kp[6] = len > 0. ? (float)(2097152.0 / len) : 0.f;
  int exact_levels = 21;
  if (K.res > 0.f && len > 0.)
  {
    const double lv = floor(log2(len / (double)K.res)) + 2.;
    exact_levels = lv < 1. ? 1 : (lv > 21. ? 21 : (int)lv);
  }
  kp[7] = __int_as_float(exact_levels);
  // halvings until the side drops below TreeNodeResolution: a cell at level L
  // has side len * 2^-min(L, kstar) (src/gravity_tree.cpp:38-42)
  int kstar = 0;
  for (double l = len; l >= (double)K.res && kstar < 1000; l *= 0.5)
    kstar++;
  kp[8] = __int_as_float(kstar);
  kp[11] = (float)len;
  // first iteration: the sources are every particle (a warm start decides the
  // wrap from every particle before it starts)
  if (D.state[s] == kActive && D.iter[s] == 1 && !D.corr[s] && !(D.warm && D.warm[s] == 1))
    D.wrap[s] = K.periodic && (len > (double)K.half);
}

// The reference inserts each particle by descending from the root cube,
// halving the half-size and moving the centre by +-half per axis in double
// (src/oct_tree.tpp:70-92).  The 3-bit child indices of that descent, root
// first, form the key, so sorting by key orders particles as the reference
// walk visits them.
__device__ __forceinline__ unsigned long long descent_key(float4 x, const double *root, int levels = 21)
{
  double c0 = root[0], c1 = root[1], c2 = root[2];
  double half = 0.5 * root[3];
  const double x0 = x.x, x1 = x.y, x2 = x.z;
  unsigned long long key = 0;
#pragma unroll 1
  for (int l = 0; l < levels; l++)
  {
    half *= 0.5;
    unsigned dgt = 0;
    if (x0 > c0) { c0 += half; dgt |= 1u; } else c0 -= half;
    if (x1 > c1) { c1 += half; dgt |= 2u; } else c1 -= half;
    if (x2 > c2) { c2 += half; dgt |= 4u; } else c2 -= half;
    key = (key << 3) | dgt;
  }
  return key;
}

// Spreads the low 21 bits of v so that bit i lands on bit 3i.
__device__ __forceinline__ unsigned long long spread3(unsigned long long v)
{
  v &= 0x1fffffULL;
  v = (v | (v << 32)) & 0x1f00000000ffffULL;
  v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
  v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}

// The same key without FP64 arithmetic for almost every particle.  Per axis,
// the descent selects the 2^21-cell slab (cells left-open, right-closed)
// containing x: index = ceil(t) - 1 with t = (x - origin) * 2^21 / side.  The
// float estimate of t is within 0.75 slab widths of the exact value, so the
// first `exact_levels` digits are exact unless t lies within one slab of a
// boundary at those levels (or is not finite); then k_keys_fallback decides
// them exactly in double.  Digits below the exact levels only order particles inside
// cells smaller than the tree resolution, where the reference itself breaks
// ties at random (src/oct_tree.tpp:108-120).
// Returns false when the float estimate cannot guarantee the exact digits.
__device__ __forceinline__ bool descent_key_fast(float4 x, const float *kp, unsigned long long &key)
{
  key = 0;
  const float inv = kp[6];
  if (inv == 0.f) // zero-size cube: every digit is 0, as in the reference
    return true;
  const int lv = __float_as_int(kp[7]);
  const float unit = __int_as_float((127 + 21 - lv) << 23);     // 2^(21 - lv)
  const float inv_unit = __int_as_float((127 - 21 + lv) << 23); // 2^(lv - 21): t / unit exactly
  const float xs[3] = {x.x, x.y, x.z};
#pragma unroll
  for (int d = 0; d < 3; d++)
  {
    const float t = __fmul_rn(__fsub_rn(__fsub_rn(xs[d], kp[d]), kp[3 + d]), inv);
    if (!(t > -1e30f && t < 1e30f))
      return false;
    const float q = __fmul_rn(t, inv_unit);
    const float rem = (q - floorf(q)) * unit; // distance above the last exact-level boundary
    if (rem < 1.5f || unit - rem < 1.5f)
      return false;
    float c = floorf(t);
    c = c < 0.f ? 0.f : (c > 2097151.f ? 2097151.f : c);
    key |= spread3((unsigned long long)__float2uint_rz(c)) << d; // 32-bit conversion (c < 2^21)
  }
  return true;
}

// Keys by the fast descent; the few items it cannot decide are appended to
// fb_list and finished by k_keys_fallback, so no warp diverges into FP64.
__global__ void k_keys(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  const int s = find_segment_warp(D.src_off, D.S, min(j, total - 1));
  if (j < total)
  {
    const int p = src_particle(D, s, j);
    unsigned long long key;
    need = !descent_key_fast(D.pm[p], D.keyp + 12 * s, key);
    D.key[j] = key;
    D.val[j] = (uint32_t)p;
  }
  const unsigned m = __ballot_sync(0xffffffffu, need);
  if (m)
  {
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(m) - 1)
      base = atomicAdd(D.fb_count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (need)
      D.fb_list[base + __popc(m & ((1u << lane) - 1u))] = j;
  }
}

// Items the fast descent could not decide.  Per axis the exact-level slab
// index (slabs of width w = side 2^-lv, cells left-open, right-closed) lies
// within one of the float estimate's, so two exact comparisons in double
// settle it: x > o + m w with o the root cube's origin, the same dyadic
// boundaries that the reference's descent (src/oct_tree.tpp:70-92) computes
// without rounding.  The digits below the exact levels follow the float
// estimate, kept inside the decided cell.  A non-finite estimate takes the
// reference's descent level by level.
__global__ void k_keys_fallback(DevState D)
{
  const int n = *D.fb_count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const int j = D.fb_list[i];
    const int p = (int)D.val[j];
    const int s = D.seg_of[p];
    const float *kp = D.keyp + 12 * s;
    const double *r = D.root + 4 * s;
    const int lv = __float_as_int(kp[7]);
    const int low = 21 - lv;
    const float4 x = D.pm[p];
    const float xs[3] = {x.x, x.y, x.z};
    const double w = r[3] * __hiloint2double((1023 - lv) << 20, 0); // side 2^-lv, exact
    const float inv_unit = __int_as_float((127 - low) << 23);       // 2^-low
    const unsigned top = (1u << lv) - 1u;
    unsigned long long key = 0;
    bool finite = true;
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      const float t = __fmul_rn(__fsub_rn(__fsub_rn(xs[d], kp[d]), kp[3 + d]), kp[6]);
      if (!(t > -1e30f && t < 1e30f))
      {
        finite = false;
        break;
      }
      const float tl = floorf(__fmul_rn(t, inv_unit));
      const int m0 = (int)fminf(fmaxf(tl, -1.f), (float)top + 1.f);
      const double dx = (double)xs[d] - (r[d] - 0.5 * r[3]); // x - o
      int k = m0 - 1; // sign of dx - m w from one fused rounding: exact
      if (fma(-(double)m0, w, dx) > 0.)
        k = (fma(-(double)(m0 + 1), w, dx) > 0.) ? m0 + 1 : m0;
      k = k < 0 ? 0 : (k > (int)top ? (int)top : k);
      // digits below the exact levels: the float slab index, clamped into slab k
      float c = floorf(t);
      c = c < 0.f ? 0.f : (c > 2097151.f ? 2097151.f : c);
      unsigned c21 = __float2uint_rz(c);
      const unsigned lo21 = (unsigned)k << low, hi21 = lo21 | ((1u << low) - 1u);
      c21 = c21 < lo21 ? lo21 : (c21 > hi21 ? hi21 : c21);
      key |= spread3((unsigned long long)c21) << d;
    }
    if (!finite)
      key = descent_key(x, r);
    D.key[j] = key;
  }
}

// Segment keys of the key-sorted items, and the identity permutation that the
// stable sort on segments will carry.
__global__ void k_segkeys_iota(const uint32_t *__restrict__ val, const int *__restrict__ seg_of,
                               uint32_t *__restrict__ k32, uint32_t *__restrict__ perm, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < total)
  {
    k32[j] = (uint32_t)seg_of[val[j]];
    perm[j] = (uint32_t)j;
  }
}

__global__ void k_gather_keys(const unsigned long long *__restrict__ kin, const uint32_t *__restrict__ vin,
                              const uint32_t *__restrict__ perm, unsigned long long *__restrict__ kout,
                              uint32_t *__restrict__ vout, int total)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total)
  {
    const uint32_t j = perm[i];
    kout[i] = kin[j];
    vout[i] = vin[j];
  }
}

// After sorting on the key, a stable sort on the subhalo restores the packing.
__global__ void k_segkeys(const uint32_t *__restrict__ val, const int *__restrict__ seg_of, uint32_t *__restrict__ k32,
                          int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < total)
    k32[j] = (uint32_t)seg_of[val[j]];
}

// Subsampled subhaloes: the sources are not every candidate, so their
// correction targets come from the energy-list order instead (packed by part_off).
__global__ void k_record_candidates(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.part_off, D.S, min(j, total - 1));
  if (j >= total)
    return;
  if (!D.corr[s] && D.ngrav[s])
  {
    const long long g = D.off[s] + (j - D.part_off[s]);
    D.sp[g] = D.ord[g];
  }
}

// Mass upscale factors of the subsampled subhaloes, one block per subhalo
// (GetMassUpscaleFactor[PerParticleType], src/subhalo_unbind.cpp:290-361).
// Sums are in double; the factors follow the reference's float formulas.
__global__ void __launch_bounds__(256) k_upscale(DevState D, KParams K)
{
  __shared__ double sh[14][8];
  for (int s = blockIdx.x; s < D.S; s += gridDim.x)
  {
    if (D.state[s] != kActive || D.corr[s] || !D.ngrav[s])
      continue;
    const long long off = D.off[s];
    const int ns = D.nunsample[s], nl = D.nlast[s], ms = K.max_sample;
    double v[14] = {0.}; // sub[6], tot[6], unsampled, all
    for (int k = threadIdx.x; k < nl; k += blockDim.x)
    {
      const int p = D.ord[off + k];
      const double m = D.pm[p].w;
      const int t = D.ty[p] & 7;
      if (k < ns)
        v[12] += m;
      else if (k < ns + ms)
        v[t] += m;
      else
        v[6 + t] += m;
      v[13] += m;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 14; q++)
    {
      double x = v[q];
      for (int o = 16; o > 0; o >>= 1)
        x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0)
        sh[q][w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      double tot[14];
      for (int q = 0; q < 14; q++)
      {
        tot[q] = 0.;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++)
          tot[q] += sh[q][i];
      }
      float f[6];
      if (!K.dm_only && K.upscale_per_type)
      {
        float sub[6], all[6];
        for (int t = 0; t < 6; t++)
        {
          sub[t] = (float)tot[t];
          all[t] = (float)(tot[6 + t] + tot[t]);
        }
        for (int t = 0; t < 6; t++)
          f[t] = sub[t] != 0.f ? __fdiv_rn(all[t], sub[t]) : 0.f;
        float true_m = 0.f, scaled_m = 0.f;
        for (int t = 0; t < 6; t++)
        {
          true_m = __fadd_rn(true_m, all[t]);
          scaled_m = __fadd_rn(scaled_m, __fmul_rn(sub[t], f[t]));
        }
        const float r = __fdiv_rn(true_m, scaled_m);
        for (int t = 0; t < 6; t++)
          f[t] = __fmul_rn(f[t], r);
      }
      else
      {
        // Mlast: the bound mass of the previous iteration (the initial sum on the first)
        const float mlast = D.iter[s] == 1 ? (float)tot[13] : D.mbound[s];
        float msub = 0.f;
        for (int t = 0; t < 6; t++)
          msub = (float)((double)msub + tot[t]);
        const float fac = __fdiv_rn(__fsub_rn(mlast, (float)tot[12]), msub);
        for (int t = 0; t < 6; t++)
          f[t] = fac;
      }
      for (int t = 0; t < 6; t++)
        D.factor[6 * s + t] = f[t];
    }
    __syncthreads();
  }
}

// Correction walks: the bound particles in the key order of the last full
// build, so that a warp's 32 targets are neighbours (flag, scan, scatter).
__global__ void k_tgt_flags(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.sp_off, D.S, min(j, total - 1));
  if (j > total)
    return;
  if (j == total)
  {
    D.flags[j] = 0;
    return;
  }
  D.flags[j] = D.bnd[D.sp[D.off[s] + (j - D.sp_off[s])]];
}

__global__ void k_tgt_scatter(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.sp_off, D.S, min(j, total - 1));
  if (j >= total || !D.flags[j])
    return;
  D.tgt[D.off[s] + (D.F[j] - D.F[D.sp_off[s]])] = D.sp[D.off[s] + (j - D.sp_off[s])];
}

// Number of tree cells whose first particle (in key order) is item j:
// levels lo..hi, where lo is one past the common prefix with the previous key
// and hi the common prefix with the next key (a cell needs two particles).
__device__ __forceinline__ void cell_levels(const DevState &D, int j, int i, int m, int &lo, int &hi)
{
  const unsigned long long k = D.key[j];
  lo = (i == 0) ? 0 : lcp_levels(D.key[j - 1], k) + 1;
  if (i == m - 1)
    hi = (i == 0) ? 0 : -1; // a lone particle still gets the root cell
  else
    hi = lcp_levels(k, D.key[j + 1]);
}

// Also counts the cells of each level (block histogram, then one atomic per
// level and block) for the per-level lists of k_tree_emit.
__global__ void k_tree_count(DevState D, int total)
{
  __shared__ int hist[kLevels];
  if (threadIdx.x < kLevels)
    hist[threadIdx.x] = 0;
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.src_off, D.S, min(j, total - 1));
  if (j == total)
    D.cnt[j] = 0;
  else if (j < total)
  {
    const int i = j - D.src_off[s], m = D.src_cnt[s];
    int lo, hi;
    cell_levels(D, j, i, m, lo, hi);
    D.cnt[j] = hi >= lo ? hi - lo + 1 : 0;
    for (int L = lo; L <= hi; L++)
      atomicAdd(&hist[L], 1);
  }
  __syncthreads();
  if (threadIdx.x < kLevels && hist[threadIdx.x])
    atomicAdd(&D.lvl[threadIdx.x], hist[threadIdx.x]);
}

// 64-bit integer <-> float conversions by exponent and mantissa arithmetic
// (the hardware's 64-bit conversions issue to the FP64 pipe, whose
// throughput is low on this GPU).

// v = hi + lo: hi is v rounded to float (to nearest even), lo the remainder
// rounded to float.  |v| < 2^63.
__device__ __forceinline__ void ll_to_float2(long long v, float &hi, float &lo)
{
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  float h, l = 0.f;
  if (a < (1ull << 24))
    h = __uint2float_rn((unsigned)a);
  else
  {
    const int e = 63 - __clzll((long long)a);
    const int sh = e - 23;
    unsigned long long mant = a >> sh;
    const unsigned long long rem = a & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    long long r = (long long)rem;
    if (rem > half || (rem == half && (mant & 1ull)))
    {
      mant++;
      r -= (long long)(1ull << sh);
    }
    // a mantissa carried to 2^24 steps the exponent field by itself
    h = __uint_as_float((unsigned)((e + 127) << 23) + (unsigned)(mant - (1ull << 23)));
    const unsigned long long ar = r < 0 ? 0ull - (unsigned long long)r : (unsigned long long)r; // < 2^39
    l = __fmaf_rn(__uint2float_rn((unsigned)(ar >> 16)), 65536.f, __uint2float_rn((unsigned)(ar & 0xffffu)));
    if (r < 0)
      l = -l;
  }
  hi = v < 0 ? -h : h;
  lo = v < 0 ? -l : l;
}

// One cell: item j's cell at level L (slot `slot`), in segment s ending at
// seg_end.  Its last item b is found by galloping forward from j over the
// keys; that gives the slot after its subtree (its skip).  The cell's side
// length follows src/gravity_tree.cpp:38-42 (halved per level until below
// TreeNodeResolution) and its opening threshold is len^2 / theta^2, both in
// float as the reference stores them; mass and centre of mass are filled in
// by k_tree_moments.  Slots: (centre, -threshold), (mass, skip, side, 0).
__device__ __forceinline__ void emit_cell(const DevState &D, const KParams &K, int j, int s, int seg_end, int L,
                                          int slot)
{
  int b;
  if (L == 0)
    b = seg_end - 1;
  else
  {
    const int shift = 63 - 3 * L;
    const unsigned long long pref = D.key[j] >> shift;
    int a = j, e, step = 1; // key[a] has the prefix
    for (;;)
    {
      const int probe = a + step;
      if (probe >= seg_end || (D.key[probe] >> shift) != pref)
      {
        e = min(probe, seg_end);
        break;
      }
      a = probe;
      step <<= 1;
    }
    while (e - a > 1) // answer in [a, e)
    {
      const int mid = (a + e) >> 1;
      if ((D.key[mid] >> shift) == pref)
        a = mid;
      else
        e = mid;
    }
    b = a;
  }
  const float *kp = D.keyp + 12 * s;
  const int kstar = __float_as_int(kp[8]);
  const float lenf = ldexpf(kp[11], -min(L, kstar));
  const float crit = __fdiv_rn(__fmul_rn(lenf, lenf), K.theta2);
  const int skip = b + 2 * D.X[b] + 2 * D.cnt[b] + 1;
  D.nodes[slot] = make_float4(0.f, 0.f, 0.f, __uint_as_float(__float_as_uint(crit) | 0x80000000u));
  D.nodes[slot + 1] = make_float4(0.f, __int_as_float(skip), lenf, 0.f);
}

// Writes the tree slots in preorder.  Slot index: cell (j, level lo+t) =
// j + 2 X[j] + 2t; leaf of item j = j + 2 X[j] + 2 cnt[j].  A cell's subtree
// ends after its last particle's leaf.  Each thread writes its item's leaf;
// the warp then gathers the cells of its 32 items into one list (a shuffle
// scan of their counts) and emits them one per lane, so items with many
// cells do not hold the other lanes.
__global__ void k_tree_emit(DevState D, KParams K, int total)
{
  __shared__ int lvl_off[kLevels]; // first list position of each level's cells
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 32)
  {
    const int c = lane < kLevels ? D.lvl[lane] : 0;
    int incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
      const int o = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d)
        incl += o;
    }
    if (lane < kLevels)
      lvl_off[lane] = incl - c;
  }
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  int lo = 0, c = 0, seg_end = 0, base = 0;
  const int s = find_segment_warp(D.src_off, D.S, min(j, total - 1));
  if (j < total)
  {
    const int seg0 = D.src_off[s], m = D.src_cnt[s];
    seg_end = seg0 + m;
    int hi;
    cell_levels(D, j, j - seg0, m, lo, hi);
    c = hi >= lo ? hi - lo + 1 : 0;
    base = j + 2 * D.X[j];
    const int p = (int)D.val[j];
    const float4 x = D.pm[p];
    D.nodes[base + 2 * c] = make_float4(x.x, x.y, x.z, fabsf(source_mass(D, s, p)));
    // a full build records the subhalo's particles in key order (correction walks' targets)
    if (!D.corr[s] && !D.ngrav[s])
      D.sp[D.off[s] + (j - seg0)] = p;
  }
  int incl = c; // inclusive scan of the cell counts over the warp
#pragma unroll
  for (int d = 1; d < 32; d <<= 1)
  {
    const int o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d)
      incl += o;
  }
  const int cells = __shfl_sync(0xffffffffu, incl, 31);
  for (int q0 = 0; q0 < cells; q0 += 32)
  {
    const int q = q0 + lane;
    int owner = 0; // first lane whose inclusive count exceeds q
#pragma unroll
    for (int w = 16; w > 0; w >>= 1)
      if (__shfl_sync(0xffffffffu, incl, owner + w - 1) <= q)
        owner += w;
    const int o_incl = __shfl_sync(0xffffffffu, incl, owner), o_c = __shfl_sync(0xffffffffu, c, owner);
    const int o_s = __shfl_sync(0xffffffffu, s, owner), o_lo = __shfl_sync(0xffffffffu, lo, owner);
    const int o_end = __shfl_sync(0xffffffffu, seg_end, owner), o_base = __shfl_sync(0xffffffffu, base, owner);
    const int t = q - (o_incl - o_c);
    const int L = q < cells ? o_lo + t : -1;
    if (q < cells)
      emit_cell(D, K, j - lane + owner, o_s, o_end, L, o_base + 2 * t);
    // append the cell to its level's list (one atomic per level and warp)
    const unsigned peers = __match_any_sync(0xffffffffu, L);
    const int leader = __ffs(peers) - 1;
    int at = 0;
    if (L >= 0 && lane == leader)
      at = atomicAdd(&D.lvl[kLevels + L], __popc(peers));
    at = __shfl_sync(0xffffffffu, at, leader);
    if (L >= 0)
      D.cell_list[lvl_off[L] + at + __popc(peers & ((1u << lane) - 1u))] = o_base + 2 * t;
  }
}

// Mass and centre of mass of a cell from its children
// (GravityTree_t::UpdateInternalNodes / ProcessNode / FillNodeCenter,
// src/gravity_tree.cpp:18-80): children in octant order (their slot order),
// each child's float mass and float position (a leaf) or float centre (a
// cell) accumulated in double, then stored as float -- the reference's own
// rounding, so a cell's centre carries its children's roundings as in the
// reference.
// The multipoles of the cell at `slot` from its children.
__device__ __forceinline__ void cell_moments(const DevState &D, int slot)
{
  const int end = __float_as_int(D.nodes[slot + 1].y);
  double M = 0., X = 0., Y = 0., Z = 0.;
  float fx = 0.f, fy = 0.f, fz = 0.f; // first child's position (a massless cell)
  int ch = slot + 2;
  while (ch < end)
  {
    const float4 a = D.nodes[ch];
    float m;
    int nx;
    if (slot_is_cell(a.w))
    {
      const float4 b = D.nodes[ch + 1];
      m = b.x;
      nx = __float_as_int(b.y);
    }
    else
    {
      m = a.w;
      nx = ch + 1;
    }
    if (ch == slot + 2)
    {
      fx = a.x;
      fy = a.y;
      fz = a.z;
    }
    const double md = (double)m;
    M = __dadd_rn(M, md);
    X = __fma_rn((double)a.x, md, X); // the product is exact in double
    Y = __fma_rn((double)a.y, md, Y);
    Z = __fma_rn((double)a.z, md, Z);
    ch = max(nx, ch + 1); // strictly increasing
  }
  float *cs = reinterpret_cast<float *>(&D.nodes[slot]);
  if (M > 0.)
  {
    cs[0] = __double2float_rn(__ddiv_rn(X, M));
    cs[1] = __double2float_rn(__ddiv_rn(Y, M));
    cs[2] = __double2float_rn(__ddiv_rn(Z, M));
  }
  else
  {
    cs[0] = fx;
    cs[1] = fy;
    cs[2] = fz;
  }
  reinterpret_cast<float *>(&D.nodes[slot + 1])[0] = __double2float_rn(M);
}

// The cells of level L (deepest level first, one launch per level).
__global__ void k_tree_moments(DevState D, int L)
{
  int off = 0;
  for (int l = 0; l < L; l++)
    off += D.lvl[l];
  const int n = D.lvl[L];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    cell_moments(D, D.cell_list[off + c]);
}

// Geometric trees (neighbour searches): each cell's bounding box of its
// particles instead of its mass moments, from its children, deepest level
// first.  Slots of a cell: (lo.x, lo.y, lo.z, -threshold), (hi.x, skip,
// hi.y, hi.z); a leaf's w holds its source index (int bits) once
// k_tree_leaf_ids has run.
__global__ void k_tree_bounds(DevState D, int L)
{
  int off = 0;
  for (int l = 0; l < L; l++)
    off += D.lvl[l];
  const int n = D.lvl[L];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
  {
    const int slot = D.cell_list[off + c];
    const int end = __float_as_int(D.nodes[slot + 1].y);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    int ch = slot + 2;
    while (ch < end)
    {
      const float4 a = D.nodes[ch];
      int nx;
      if (slot_is_cell(a.w))
      {
        const float4 b = D.nodes[ch + 1];
        lo[0] = fminf(lo[0], a.x);
        lo[1] = fminf(lo[1], a.y);
        lo[2] = fminf(lo[2], a.z);
        hi[0] = fmaxf(hi[0], b.x);
        hi[1] = fmaxf(hi[1], b.z);
        hi[2] = fmaxf(hi[2], b.w);
        nx = __float_as_int(b.y);
      }
      else
      {
        lo[0] = fminf(lo[0], a.x);
        lo[1] = fminf(lo[1], a.y);
        lo[2] = fminf(lo[2], a.z);
        hi[0] = fmaxf(hi[0], a.x);
        hi[1] = fmaxf(hi[1], a.y);
        hi[2] = fmaxf(hi[2], a.z);
        nx = ch + 1;
      }
      ch = max(nx, ch + 1); // strictly increasing
    }
    float *c0 = reinterpret_cast<float *>(&D.nodes[slot]);
    float *c1 = reinterpret_cast<float *>(&D.nodes[slot + 1]);
    c0[0] = lo[0];
    c0[1] = lo[1];
    c0[2] = lo[2];
    c1[0] = hi[0];
    c1[2] = hi[1];
    c1[3] = hi[2];
  }
}

// Leaf slots of a geometric tree carry their source index in w.
__global__ void k_tree_leaf_ids(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total)
    return;
  const int slot = j + 2 * D.X[j] + 2 * D.cnt[j];
  reinterpret_cast<int *>(&D.nodes[slot])[3] = (int)D.val[j];
}

// ---------------------------------------------------------------------------
// Softened potential kernel of the tree walk (walk.cuh)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float spline_w(float u)
{
  // Gadget cubic-spline potential kernel, src/gravity_tree.cpp:154-160
  return (u < 0.5f) ? -2.8f + u * u * (5.333333333333f + u * u * (6.4f * u - 9.6f))
                    : -3.2f + 0.066666666667f / u +
                        u * u * (10.666666666667f + u * (-16.0f + u * (9.6f - 2.133333333333f * u)));
}

// ---------------------------------------------------------------------------
// Energies, partition, frame
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rel_vel(float3 x, float3 v, const float *rp, const float *rv, const KParams &K, float *dv)
{
  // Snapshot_t::RelativeVelocity (src/snapshot.h:135-148), float
  const float hz_a = K.hz * K.a;
  const float xs[3] = {x.x, x.y, x.z}, vs[3] = {v.x, v.y, v.z};
  for (int d = 0; d < 3; d++)
  {
    float dx = __fsub_rn(xs[d], rp[d]);
    if (K.periodic)
      dx = nearest_f(dx, K.half, K.box);
    dv[d] = __fadd_rn(__fsub_rn(vs[d], rv[d]), __fmul_rn(hz_a, dx));
  }
}
__device__ __forceinline__ float norm2_rn(const float *d)
{
  return __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
}

__global__ void k_energy(DevState D, KParams K, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.part_off, D.S, min(j, total - 1));
  if (j >= total)
    return;
  const int k = j - D.part_off[s];
  const int p = D.ord[D.off[s] + k];
  const float4 x = D.pm[p], v = D.vu[p];
  const float3 x3 = make_float3(x.x, x.y, x.z), v3 = make_float3(v.x, v.y, v.z);
  if (!D.corr[s])
  {
    float dv[3];
    rel_vel(x3, v3, D.ref_pos + 3 * s, D.ref_vel + 3 * s, K, dv);
    float e = __fadd_rn(__fmul_rn(0.5f, norm2_rn(dv)), D.pot[p]);
    if (K.thermal)
      e = __fadd_rn(e, v.w);
    D.Ep[p] = e;
  }
  else
  {
    float dV[3], ov[3];
    const float op[3] = {D.old_pos[3 * s], D.old_pos[3 * s + 1], D.old_pos[3 * s + 2]};
    const float ovl[3] = {D.old_vel[3 * s], D.old_vel[3 * s + 1], D.old_vel[3 * s + 2]};
    rel_vel(make_float3(op[0], op[1], op[2]), make_float3(ovl[0], ovl[1], ovl[2]), D.ref_pos + 3 * s,
            D.ref_vel + 3 * s, K, dV);
    const float dK = __fmul_rn(0.5f, norm2_rn(dV)); // halving is exact
    rel_vel(x3, v3, op, ovl, K, ov);
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(ov[0], dV[0]), __fmul_rn(ov[1], dV[1])), __fmul_rn(ov[2], dV[2]));
    D.Ep[p] = __fadd_rn(D.Ep[p], __fsub_rn(__fadd_rn(dot, dK), D.pot[p]));
  }
}

__global__ void k_part_flags(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.part_off, D.S, min(j, total - 1));
  if (j > total)
    return;
  if (j == total)
  {
    D.flags[j] = 0;
    return;
  }
  const int k = j - D.part_off[s];
  D.flags[j] = D.Ep[D.ord[D.off[s] + k]] < 0.f ? 1 : 0;
}

__global__ void k_part_count(DevState D)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S || D.part_cnt[s] == 0)
    return;
  D.nb_new[s] = D.F[D.part_off[s + 1]] - D.F[D.part_off[s]];
}

// Stable partition: bound particles first, each group in its previous order.
__global__ void k_part_scatter(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = j < total;
  int s = find_segment_warp(D.part_off, D.S, min(j, total - 1)), tracer = 0;
  if (!valid)
    s = -1;
  if (valid)
  {
    const int k = j - D.part_off[s];
    const int rb = D.F[j] - D.F[D.part_off[s]];
    const bool bound = D.flags[j] != 0;
    const int dest = bound ? rb : D.nb_new[s] + (k - rb);
    const int p = D.ord[D.off[s] + k];
    D.ord_tmp[D.off[s] + dest] = p;
    D.bnd[p] = bound ? 1 : 0;
    tracer = (bound && is_tracer_bits(D.ty[p])) ? 1 : 0;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, s);
  const int tot = __reduce_add_sync(peers, tracer);
  if (valid && (int)(threadIdx.x & 31) == __ffs(peers) - 1 && tot)
    atomicAdd(&D.tracers[s], tot);
}

__global__ void k_part_copy(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.part_off, D.S, min(j, total - 1));
  if (j >= total)
    return;
  const long long g = D.off[s] + (j - D.part_off[s]);
  D.ord[g] = D.ord_tmp[g];
}

// Disruption test and CorrectionLoop flag (src/subhalo_unbind.cpp:630-683).
__global__ void k_after_part(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s > D.S)
    return;
  if (s == D.S)
  {
    D.tail_cnt[s] = 0;
    return;
  }
  D.tail_cnt[s] = 0;
  if (D.state[s] != kActive)
    return;
  const int nb = D.nb_new[s];
  D.nbound[s] = nb;
  if (D.nb1 && D.iter[s] == 1)
    D.nb1[s] = nb;
  const int tracers = K.dm_only ? nb : D.tracers[s];
  if (nb < K.min_part || tracers < K.min_tracer)
  {
    for (int d = 0; d < 3; d++)
    {
      D.ref_pos[3 * s + d] = D.mb_pos[3 * s + d];
      D.ref_vel[3 * s + d] = D.mb_vel[3 * s + d];
    }
    D.nbound[s] = 0;
    D.mbound[s] = 0.f;
    D.state[s] = kDisrupted;
    return;
  }
  { // CountUnsampledParticles (src/subhalo_unbind.cpp:446-461)
    int k = 0;
    const int ns = D.nunsample[s];
    while (k < ns && is_nosub_bits(D.ty[D.ord[D.off[s] + k]]))
      k++;
    D.nunsample[s] = k;
  }
  const int ndiff = D.nlast[s] - nb;
  D.tail_cnt[s] = ndiff;
  if (ndiff < nb && (K.max_sample <= 0 || ndiff < K.max_sample))
  {
    D.corr[s] = 1;
    for (int d = 0; d < 3; d++)
    {
      D.old_pos[3 * s + d] = D.ref_pos[3 * s + d];
      D.old_vel[3 * s + d] = D.ref_vel[3 * s + d];
    }
  }
  for (int q = 0; q < 7; q++)
    D.com[7 * s + q] = 0.;
}

// RefineBindingEnergyOrder (src/subhalo_unbind.cpp:395-425, 712-738): for a
// converged subsampled subhalo, the leading max(MaxSample, fraction*Nbound)
// particles are re-ordered by their binding energy in the tree of just those
// particles.  The stored energies are left as they were (so, as in the
// reference, they are no longer in order there).
__global__ void k_plan_refine(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s > D.S)
    return;
  if (s == D.S)
  {
    D.src_cnt[s] = D.chunk_cnt[s] = 0;
    return;
  }
  D.src_cnt[s] = D.chunk_cnt[s] = D.tgt_cnt[s] = 0;
  const int nb = D.nbound[s];
  if (D.state[s] != kConverged || nb <= K.max_sample)
    return;
  const int size = max(K.max_sample, (int)(K.refine_frac * (float)nb));
  D.src_begin[s] = 0;
  D.src_cnt[s] = size;
  D.tgt_cnt[s] = size;
  D.chunk_cnt[s] = (size + kWarp - 1) / kWarp;
  D.corr[s] = 0;
  D.ngrav[s] = 0;
  for (int t = 0; t < 6; t++)
    D.factor[6 * s + t] = 1.f;
  // a fresh bounding box for the prefix's own tree (k_bbox, k_root)
  D.bb_lo[3 * s] = D.bb_lo[3 * s + 1] = D.bb_lo[3 * s + 2] = 0xffffffffu;
  D.bb_hi[3 * s] = D.bb_hi[3 * s + 1] = D.bb_hi[3 * s + 2] = 0u;
}

__global__ void k_refine_keys(DevState D, KParams K, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total)
    return;
  const int p = (int)D.val[j];
  const int s = D.seg_of[p];
  const float4 x = D.pm[p], v = D.vu[p];
  float dv[3];
  rel_vel(make_float3(x.x, x.y, x.z), make_float3(v.x, v.y, v.z), D.ref_pos + 3 * s, D.ref_vel + 3 * s, K, dv);
  D.k32[j] = float_to_ordered(__fadd_rn(__fmul_rn(0.5f, norm2_rn(dv)), D.pot[p]));
}

__global__ void k_refine_write(DevState D, const uint32_t *__restrict__ sorted_val, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.src_off, D.S, min(j, total - 1));
  if (j >= total)
    return;
  D.ord[D.off[s] + (j - D.src_off[s])] = (int)sorted_val[j];
}

// Keys for sorting ranges by energy: ordered float, value = particle.
// mode 0: the unbound tail [nbound, nbound + tail_cnt); mode 1: [0, nbound).
__global__ void k_energy_keys(DevState D, const int *__restrict__ offs, int total, int mode)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(offs, D.S, min(j, total - 1));
  if (j >= total)
    return;
  const int k = (mode == 0 ? D.nbound[s] : 0) + (j - offs[s]);
  const int p = D.ord[D.off[s] + k];
  D.k32[j] = float_to_ordered(D.Ep[p]);
  D.val[j] = (uint32_t)p;
}

__global__ void k_energy_write(DevState D, const uint32_t *__restrict__ sorted_val, const int *__restrict__ offs,
                               int total, int mode)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(offs, D.S, min(j, total - 1));
  if (j >= total)
    return;
  const int k = (mode == 0 ? D.nbound[s] : 0) + (j - offs[s]);
  D.ord[D.off[s] + k] = (int)sorted_val[j];
}

// Adds Q per-thread partial sums into out[Q*seg + q]: a warp-segmented
// reduction over lanes holding the same segment, then one atomic per segment.
template <int Q>
__device__ __forceinline__ void segmented_flush(double (&acc)[Q], int seg, double *out)
{
  const unsigned peers = __match_any_sync(0xffffffffu, seg);
  const int lane = threadIdx.x & 31;
  if (peers == 0xffffffffu)
  {
#pragma unroll
    for (int q = 0; q < Q; q++)
      for (int o = 16; o > 0; o >>= 1)
        acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
    if (lane == 0 && seg >= 0)
      for (int q = 0; q < Q; q++)
        atomicAdd(&out[Q * seg + q], acc[q]);
    return;
  }
  if (seg >= 0)
    for (int q = 0; q < Q; q++)
      if (acc[q] != 0.)
        atomicAdd(&out[Q * seg + q], acc[q]);
}

constexpr int kItemsPerThread = 16;

// k_com takes kItemsPerThread consecutive items per thread over large bound
// sets (bandwidth) and one item per thread over small ones (the late
// iterations: a thread's items are a chain of dependent loads, so fewer per
// thread means a shorter launch).
constexpr long long kComSmall = 65536;
__host__ __device__ inline int com_items_per_thread(long long total) { return total <= kComSmall ? 1 : kItemsPerThread; }
// Per-block partials that k_com can write over n bound particles.
__host__ __device__ inline long long com_part_blocks(long long n)
{
  return n / (256LL * kItemsPerThread) + kComSmall / 256 + 2;
}

// Kahan-compensated float accumulator.
struct KahanF
{
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v)
  {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Centre-of-mass sums over the bound set, wrapped about its first particle
// (src/subhalo_unbind.cpp:151-198).  Each thread sums 16 consecutive items
// with compensated float partials (FP64 is scarce on this GPU); the partials
// are added in double.  Offsets that need the periodic wrap are formed in
// double as the reference does.
__global__ void k_com(DevState D, KParams K, int total)
{
  const int ipt = D.com_ipt;
  const long long first = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * ipt;
  KahanF acc[7];
  double out[7] = {0., 0., 0., 0., 0., 0., 0.};
  int s = -1;
  auto flush = [&](int seg) {
    for (int q = 0; q < 7; q++)
    {
      const double v = acc[q].value();
      if (v != 0.)
        atomicAdd(&D.com[7 * seg + q], v);
      acc[q] = KahanF();
    }
  };
  // the whole warp looks up its threads' first subhaloes (first items ascend with the lane)
  const int s_first = find_segment_warp(D.fin_off, D.S, (int)min(first, (long long)total - 1));
  if (first < total)
  {
    s = s_first;
    const int last = (int)min((long long)total, first + ipt);
    float4 o = D.pm[D.ord[D.off[s]]];
    for (int j = (int)first; j < last; j++)
    {
      if (j >= D.fin_off[s + 1])
      { // next subhalo: flush the partial sums of this one
        flush(s);
        s = find_segment<int>(D.fin_off, D.S, j); // skips any run of empty segments
        o = D.pm[D.ord[D.off[s]]];
      }
      const int p = D.ord[D.off[s] + (j - D.fin_off[s])];
      const float4 x = D.pm[p], v = D.vu[p];
      const float m = x.w;
      acc[0].add(m);
      const float xs[3] = {x.x, x.y, x.z}, os[3] = {o.x, o.y, o.z};
#pragma unroll
      for (int d = 0; d < 3; d++)
      {
        if (K.periodic)
        {
          const float df = xs[d] - os[d];
          if (fabsf(df) < 0.25f * K.half) // no wrap possible; x - o is exact or nearly so
            acc[1 + d].add(__fmul_rn(df, m));
          else
            acc[1 + d].add((float)(nearest_d((double)xs[d] - (double)os[d], K.half, K.box) * m));
        }
        else
          acc[1 + d].add(__fmul_rn(xs[d], m));
      }
      acc[4].add(__fmul_rn(v.x, m));
      acc[5].add(__fmul_rn(v.y, m));
      acc[6].add(__fmul_rn(v.z, m));
    }
    for (int q = 0; q < 7; q++)
      out[q] = acc[q].value();
  }
  // A block whose items all belong to one subhalo writes a block-reduced
  // partial instead of contending atomics; k_control adds those partials.
  __shared__ int s_seg_lo, s_seg_hi;
  __shared__ double s_part[7][8];
  const long long b0 = (long long)blockIdx.x * blockDim.x * ipt;
  const long long b1 = min((long long)total, b0 + (long long)blockDim.x * ipt);
  if (threadIdx.x == 0)
  {
    s_seg_lo = find_segment<int>(D.fin_off, D.S, (int)b0);
    s_seg_hi = (b1 <= D.fin_off[s_seg_lo + 1]) ? s_seg_lo : -1;
  }
  __syncthreads();
  if (s_seg_hi >= 0)
  {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 7; q++)
    {
      double v = out[q];
      for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0)
        s_part[q][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < 7)
    {
      double v = 0.;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++)
        v += s_part[threadIdx.x][i];
      D.com_part[7LL * blockIdx.x + threadIdx.x] = v;
    }
    return;
  }
  segmented_flush<7>(out, s, D.com);
}

// Frame and bound mass from the k_com sums of subhalo s
// (CentreOfMassReferenceFrame, src/subhalo_unbind.cpp:151-198).
__device__ void frame_from_sums(DevState &D, const KParams &K, int s)
{
  double c[7];
  for (int q = 0; q < 7; q++)
    c[q] = D.com[7 * s + q];
  // add the partials of the k_com blocks lying entirely inside this subhalo
  // (same test as k_com: the block's item range [b0, b1) lies in [lo, hi))
  const long long per_block = 256LL * D.com_ipt;
  const long long lo = D.fin_off[s], hi = D.fin_off[s + 1], total = D.fin_off[D.S];
  for (long long b = (lo + per_block - 1) / per_block; b * per_block < hi; b++)
  {
    const long long b1 = min(total, (b + 1) * per_block);
    if (b1 <= hi)
      for (int q = 0; q < 7; q++)
        c[q] += D.com_part[7 * b + q];
  }
  const double M = c[0];
  const float4 o = D.pm[D.ord[D.off[s]]];
  const double org[3] = {o.x, o.y, o.z};
  for (int d = 0; d < 3; d++)
  {
    double px = c[1 + d] / M;
    if (K.periodic)
      px += org[d];
    D.ref_pos[3 * s + d] = (float)px;
    D.ref_vel[3 * s + d] = (float)(c[4 + d] / M);
  }
  D.mbound[s] = (float)M;
}

// New frame, bound mass and convergence test (src/subhalo_unbind.cpp:687-690).
__global__ void k_control(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S || D.state[s] != kActive)
    return;
  frame_from_sums(D, K, s);
  const int nb = D.nbound[s];
  if ((float)nb >= __fmul_rn((float)D.nlast[s], K.bmp))
    D.state[s] = kConverged;
  else if (D.iter[s] >= K.max_iter)
    D.state[s] = kMaxIter;
}

__global__ void k_plan_counts(DevState D, int mode)
{
  // mode 0: fin_cnt = nbound of active subhaloes (frame sums)
  // mode 1: fin_cnt = nbound of converged / stopped subhaloes (final sort)
  // mode 2: fin_cnt = nbound of the subhaloes flagged in flag_s (warm-start
  //         frames), whose frame sums are zeroed
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s > D.S)
    return;
  if (s == D.S)
  {
    D.fin_cnt[s] = 0;
    return;
  }
  const int st = D.state[s];
  bool take;
  if (mode >= 2)
  {
    take = D.flag_s[s] != 0;
    if (take)
      for (int q = 0; q < 7; q++)
        D.com[7 * s + q] = 0.;
  }
  else
    take = mode == 0 ? (st == kActive) : (st == kConverged || st == kMaxIter);
  D.fin_cnt[s] = take ? D.nbound[s] : 0;
}

// ---------------------------------------------------------------------------
// Epilogue: one block per subhalo.
// ---------------------------------------------------------------------------
struct OutPtrs
{
  long long *order, *nbound, *nbound_type, *tracer_index, *most_bound_id;
  float *mbound, *mbound_type, *kinematics, *core, *energy, *potential;
  int *iterations, *status;
};

// Zeroes the per-subhalo accumulators of the epilogue.
__global__ void k_epi_init(DevState D)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S)
    return;
  for (int q = 0; q < 7; q++)
    D.com[7 * s + q] = 0.;
  for (int t = 0; t < 6; t++)
  {
    reinterpret_cast<int *>(D.bb_lo)[6 * s + t] = 0;
  }
  D.nb_new[s] = 0x7fffffff;
}

// The output permutation: for resolved subhaloes the energy order, else the
// input order (the reference permutes Particles only on convergence,
// src/subhalo_unbind.cpp:744-750).
__global__ void k_epi_order(DevState D, OutPtrs O)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += (long long)gridDim.x * blockDim.x)
  {
    const int s = D.seg_of[i];
    const long long off = D.off[s];
    const int st = D.state[s];
    O.order[i] = (st == kConverged || st == kMaxIter) ? (long long)D.ord[i] - off : i - off;
  }
}

// Per-particle outputs of the bound sets (binding and potential energies) and
// the FP64 sums of AverageKinematics (src/subhalo_unbind.cpp:200-249), the
// per-type counts of CountParticleTypes (src/subhalo.cpp:311-393) and the
// first tracer position (the per-type masses are summed by k_epilogue).  Items are the bound particles of finished
// subhaloes packed by fin_off; each thread takes 16 consecutive items.
__global__ void k_epi_particles(DevState D, KParams K, OutPtrs O, int total)
{
  const long long first = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kItemsPerThread;
  // AverageKinematics sums (src/subhalo_unbind.cpp:200-249) in compensated
  // FP32 per thread (the per-particle terms the reference forms in double
  // carry one FP32 rounding each here), totals in double
  KahanF acc[6];
  int tn[6] = {0, 0, 0, 0, 0, 0};
  int ft = 0x7fffffff;
  int s = -1;
  auto flush_types = [&](int seg) {
    for (int t = 0; t < 6; t++)
      if (tn[t])
      {
        atomicAdd(&reinterpret_cast<int *>(D.bb_lo)[6 * seg + t], tn[t]);
        tn[t] = 0;
      }
    if (ft != 0x7fffffff)
      atomicMin(&D.nb_new[seg], ft);
    ft = 0x7fffffff;
  };
  if (first < total)
  {
    s = find_segment<int>(D.fin_off, D.S, (int)first);
    const int last = (int)min((long long)total, first + kItemsPerThread);
    for (int j = (int)first; j < last; j++)
    {
      if (j >= D.fin_off[s + 1])
      {
        for (int q = 0; q < 6; q++)
        {
          const double v = acc[q].value();
          if (v != 0.)
            atomicAdd(&D.com[7 * s + q], v);
          acc[q] = KahanF();
        }
        flush_types(s);
        s = find_segment<int>(D.fin_off, D.S, j); // skips any run of empty segments
      }
      const int k = j - D.fin_off[s];
      const long long off = D.off[s];
      const int p = D.ord[off + k];
      const float4 x = D.pm[p], v = D.vu[p];
      const float e = D.Ep[p];
      if (O.energy)
        O.energy[off + k] = e;
      const float m = x.w;
      acc[0].add(__fmul_rn(e, m));
      if (K.thermal)
        acc[0].add(-__fmul_rn(v.w, m));
      const float *rp = D.ref_pos + 3 * s, *rv = D.ref_vel + 3 * s;
      const float xs[3] = {x.x, x.y, x.z}, vs[3] = {v.x, v.y, v.z};
      float dx[3], dv[3];
      float pe = K.thermal ? __fsub_rn(e, v.w) : e;
#pragma unroll
      for (int d = 0; d < 3; d++)
      {
        dx[d] = __fsub_rn(xs[d], rp[d]);
        if (K.periodic)
          dx[d] = nearest_f(dx[d], K.half, K.box);
        dx[d] = __fmul_rn(dx[d], K.a);
        dv[d] = __fmaf_rn(K.hz, dx[d], __fsub_rn(vs[d], rv[d]));
        const float dv2 = __fmul_rn(dv[d], dv[d]);
        acc[1].add(__fmul_rn(dv2, m));
        if (O.potential)
          pe = __fsub_rn(pe, __fmul_rn(0.5f, dv2));
      }
      if (O.potential)
        O.potential[off + k] = pe;
      acc[2].add(__fmul_rn(__fmaf_rn(dx[1], dv[2], -__fmul_rn(dx[2], dv[1])), m));
      acc[3].add(__fmul_rn(__fmaf_rn(dx[2], dv[0], -__fmul_rn(dx[0], dv[2])), m));
      acc[4].add(__fmul_rn(__fmaf_rn(dx[0], dv[1], -__fmul_rn(dx[1], dv[0])), m));
      acc[5].add(m);
      const uint8_t t = D.ty[p];
#pragma unroll
      for (int q = 0; q < 6; q++)
        if ((t & 7) == q)
          tn[q]++;
      if (is_tracer_bits(t) && k < ft)
        ft = k;
    }
    flush_types(s);
  }
  double acc7[7] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value(), acc[4].value(),
                    acc[5].value(), 0.};
  segmented_flush<7>(acc7, s, D.com);
}

// MboundType as CountParticleTypes sums it (src/subhalo.cpp:311-393): per
// type, float additions in bound order.  One warp per subhalo: the lanes load
// 32 bound particles at a time (the next 32 while the current ones are
// added) and lane t replays the additions of type t in order, so the six
// sums are the reference's sequential ones.
__global__ void k_type_masses(DevState D, float *out)
{
  const int s = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= D.S) // whole warps
    return;
  const unsigned full = 0xffffffffu;
  const int st = D.state[s];
  const int nb = (st == kConverged || st == kMaxIter) ? D.nbound[s] : 0;
  const long long off = D.off[s];
  float acc = 0.f;
  int t = 7;
  float m = 0.f;
  if (lane < nb)
  {
    const int p = D.ord[off + lane];
    t = D.ty[p] & 7;
    m = D.pm[p].w;
  }
  for (int i0 = 0; i0 < nb; i0 += kWarp)
  {
    const int cur_t = t;
    const float cur_m = m;
    const int i = i0 + kWarp + lane;
    t = 7;
    m = 0.f;
    if (i < nb)
    {
      const int p = D.ord[off + i];
      t = D.ty[p] & 7;
      m = D.pm[p].w;
    }
    const int cnt = min(kWarp, nb - i0);
    for (int q = 0; q < cnt; q++)
    {
      const int tq = __shfl_sync(full, cur_t, q);
      const float mq = __shfl_sync(full, cur_m, q);
      if (tq == lane)
        acc = __fadd_rn(acc, mq);
    }
  }
  if (lane < 6)
    out[6 * s + lane] = acc;
}

// Scalar outputs of each subhalo (one thread per subhalo): kinematics, type
// counts, tracer index, most-bound particle and ID, core phase-space
// properties (src/subhalo_merge.cpp:94-181), status and iterations.
__global__ void k_epilogue(DevState D, KParams K, OutPtrs O)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S)
    return;
  const int st = D.state[s];
  const long long off = D.off[s];
  const bool resolved = (st == kConverged || st == kMaxIter);
  const int nb = resolved ? D.nbound[s] : 0;
  const double *c = D.com + 7 * s;
  float kin[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (nb > 1)
  {
    const double Ms = c[5];
    const double Et = c[0] / Ms;
    const double Kk = c[1] * (0.5 / Ms);
    kin[0] = (float)(Et - Kk);
    kin[1] = (float)Kk;
    kin[2] = (float)(c[2] / Ms);
    kin[3] = (float)(c[3] / Ms);
    kin[4] = (float)(c[4] / Ms);
  }
  if (O.kinematics)
    for (int q = 0; q < 5; q++)
      O.kinematics[5 * s + q] = kin[q];
  const int *tn = reinterpret_cast<const int *>(D.bb_lo) + 6 * s;
  if (O.nbound_type)
    for (int t = 0; t < 6; t++)
      O.nbound_type[6 * s + t] = resolved ? tn[t] : 0;
  const int first_tracer = D.nb_new[s];
  long long ti;
  if (st == kEmpty)
    ti = -1;
  else if (nb == 0 || K.dm_only || first_tracer == 0x7fffffff)
    ti = 0;
  else
    ti = first_tracer;
  O.tracer_index[s] = ti;
  O.nbound[s] = nb;
  O.mbound[s] = resolved ? D.mbound[s] : 0.f;
  O.iterations[s] = D.iter[s] + (D.iter_extra ? D.iter_extra[s] : 0);
  O.status[s] = st == kConverged ? 0 : st == kDisrupted ? 1 : st == kEmpty ? 2 : 3;
  float *mbp = D.mb_pos + 3 * s, *mbv = D.mb_vel + 3 * s;
  if (nb > 0)
  {
    const int p0 = D.ord[off];
    const float4 x0 = D.pm[p0], v0 = D.vu[p0];
    mbp[0] = x0.x;
    mbp[1] = x0.y;
    mbp[2] = x0.z;
    mbv[0] = v0.x;
    mbv[1] = v0.y;
    mbv[2] = v0.z;
    O.most_bound_id[s] = D.id[D.ord[off + ti]];
  }
  if (!O.core)
    return;
  float *cr = O.core + 8 * s;
  if (nb == 0)
  {
    for (int d = 0; d < 3; d++)
    {
      cr[d] = mbp[d];
      cr[3 + d] = mbv[d];
    }
    cr[6] = cr[7] = 0.f;
    return;
  }
  // first CoreSize tracers, then non-tracers
  const long long core_size = max((long long)((float)nb * K.core_factor), K.core_min);
  long long used = 0;
  double msum = 0., ps[3] = {0., 0., 0.}, ps2[3] = {0., 0., 0.}, vs[3] = {0., 0., 0.}, vs2[3] = {0., 0., 0.},
         org[3] = {0., 0., 0.};
  const float4 x0 = D.pm[D.ord[off]];
  if (K.periodic)
  {
    org[0] = x0.x;
    org[1] = x0.y;
    org[2] = x0.z;
  }
  for (int pass = 0; pass < 2 && used != core_size; pass++)
    for (int i = 0; i < nb; i++)
    {
      const int p = D.ord[off + i];
      const bool tr = is_tracer_bits(D.ty[p]);
      if ((tr && pass == 0) || (!tr && pass == 1))
      {
        used++;
        const float4 x = D.pm[p], v = D.vu[p];
        const float m = x.w;
        msum += m;
        const float xs[3] = {x.x, x.y, x.z}, vv[3] = {v.x, v.y, v.z};
        for (int d = 0; d < 3; d++)
        {
          double dx = xs[d];
          if (K.periodic)
            dx = nearest_d(dx - org[d], K.half, K.box);
          ps[d] += m * dx;
          ps2[d] += m * dx * dx;
          const double dvv = vv[d];
          vs[d] += m * dvv;
          vs2[d] += m * dvv * dvv;
        }
      }
      if (used == core_size)
        break;
    }
  for (int d = 0; d < 3; d++)
  {
    ps[d] /= msum;
    ps2[d] /= msum;
    float cp = (float)ps[d];
    if (K.periodic)
      cp = (float)((double)cp + org[d]);
    cr[d] = cp;
    ps2[d] -= ps[d] * ps[d];
    vs[d] /= msum;
    vs2[d] /= msum;
    cr[3 + d] = (float)vs[d];
    vs2[d] -= vs[d] * vs[d];
  }
  cr[6] = (float)sqrt(ps2[0] + ps2[1] + ps2[2]);
  cr[7] = (float)sqrt(vs2[0] + vs2[1] + vs2[2]);
}

} // namespace
} // namespace hbtg
