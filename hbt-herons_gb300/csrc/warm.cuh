// warm.cuh - warm start of the batched unbinding iteration from a proposed
// set, and the per-particle features of the learned proposer.
//
// No counterpart in the reference: Subhalo_t::Unbind always starts from every
// particle of the subhalo (src/subhalo_unbind.cpp:505-507), and its first
// iteration evaluates every particle against the tree of every particle, the
// most expensive step of the method.  A proposal predicts that iteration's
// survivors (E < 0 in the potential of every particle, in the input frame):
//
//   proposal     per particle: trusted (1: starts in the set), to test (0), or
//                left out (2: the proposer is sure the first iteration removes
//                it); each warm subhalo's particles are partitioned in that
//                order: trusted, tested, left out
//   first test   every particle to test gets the plain method's own first
//                test: its energy against the tree of every particle, in the
//                input frame; those with E < 0 join the set.  The targets walk
//                in the tree's key order, so a warp's 32 are neighbours
//   iteration    from that set, in its centre-of-mass frame (the frame the
//                plain method's second iteration uses), the unchanged exact
//                loop (driver.cuh) runs to its convergence test, so the path
//                is the plain method's own from its second iteration on
//   cold start   a subhalo whose first iteration would already have converged
//                (the test leaves fewer than 1 - BoundMassPrecision of its
//                particles out) is restarted cold from its inputs: the warm
//                start has nothing to save there
// Where the warm path can leave the plain one: a trusted particle that the
// first iteration would have removed (the exact loop still removes it, later),
// a left-out particle that it would have kept, and the second iteration, which the plain method usually computes as a
// correction (energies of the first minus the removed particles' potential,
// src/subhalo_unbind.cpp:563-621) and the warm path from a new tree of the
// same set: the two differ by the tree's approximation error, which moves
// particles with |E| that small across E = 0.
//
// Features (six per particle, about the input frame):
//   f0 log(1 + r / r_half)            r_half of the subhalo's radial mass profile
//   f1 min(|v - V| / v_c, 16)         v_c^2 = (G/a) (M/2) / r_half
//   f2 E_mono / v_c^2 (clamped 16)    first-iteration energy with the tree replaced by
//                                     the monopole of every particle: 1/2 |v - V|^2 + phi(r) (+ u)
//   f3 E_prev / v_c^2 (clamped 16)    previous-output binding energy, 0 if unknown
//   f4 +1 / -1 / 0                    bound / not bound at the previous output / unknown
//   f5 species code                   gas 1, DM 0, star -0.5, black hole -1, other 0.25/0.5
// The profile is 64 bins of a quarter octave below the largest radius,
// summed in fixed point so that the features are bit-reproducible.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "common.cuh"
#include "driver.cuh"
#include "kernels.cuh"
#include "primitives.cuh"

namespace hbtg
{
namespace
{

constexpr int kBins = 64;               // quarter-octave bins: 16 octaves below r_max
constexpr int kTab = 72;                // per subhalo: r_max, 1/r_half, 1/v_c^2, 1/v_c, phi at 65 edges
constexpr int kFeat = 6;                // features per particle
constexpr float kQScale = 1073741824.f; // 2^30: fixed-point mass unit = largest particle mass / 2^30

struct WarmBufs
{
  const long long *nb_prev; // [S] previous-output Nbound, or null
  const float *e_prev;      // [N] previous-output binding energies (first nb_prev of each subhalo), or null
  unsigned *rmax;           // [S] float bits of the largest radius (radii are >= 0)
  unsigned *mmax;           // [1] float bits of the largest particle mass
  unsigned *bb;             // [6S] ordered-float bounding box of every particle (lo xyz, hi xyz)
  unsigned long long *hist; // [64 S] fixed-point mass per radial bin
  float *tab;               // [kTab S]
  float *feat;              // [6 N]
  const uint8_t *prop;      // [N] proposal: 1 trusted, 0 uncertain, 2 left out
  long long min_n;          // subhaloes with fewer particles start cold
  int first_test;           // 1: the uncertain particles get the first test; 0: they join untested
};

__device__ __forceinline__ bool has_prior(const WarmBufs &W, int s) { return W.nb_prev && W.nb_prev[s] > 0; }

__device__ __forceinline__ float radius_about(float4 x, const float *c, const KParams &K)
{
  float d[3] = {__fsub_rn(x.x, c[0]), __fsub_rn(x.y, c[1]), __fsub_rn(x.z, c[2])};
  if (K.periodic)
    for (int q = 0; q < 3; q++)
      d[q] = nearest_f(d[q], K.half, K.box);
  return sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

__global__ void k_feat_reset(DevState D, WarmBufs W)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0)
    *W.mmax = 0u;
  if (s >= D.S)
    return;
  W.rmax[s] = 0u;
  for (int d = 0; d < 3; d++)
  {
    W.bb[6 * s + d] = 0xffffffffu;
    W.bb[6 * s + 3 + d] = 0u;
  }
}

// Largest radius about the input frame, bounding box, largest mass.  The
// block reduces first: to one set of atomics when all its particles belong
// to one subhalo (large subhaloes would otherwise send every warp's atomics
// to the same words), else per warp and subhalo; the largest mass always
// once per block.
__global__ void __launch_bounds__(256) k_feat_extent(DevState D, KParams K, WarmBufs W)
{
  __shared__ unsigned s_red[8][8];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < D.N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long b0 = (long long)blockIdx.x * blockDim.x;
  const long long b1 = min(D.N, b0 + (long long)blockDim.x) - 1;
  const bool uniform = b0 < D.N && D.seg_of[b0] == D.seg_of[b1];
  const int s = valid ? D.seg_of[i] : -1;
  unsigned r = 0u, m = 0u, lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  if (valid)
  {
    const float4 x = D.pm[i];
    r = __float_as_uint(radius_about(x, D.ref_pos + 3 * s, K));
    m = __float_as_uint(fmaxf(x.w, 0.f));
    lo[0] = hi[0] = float_to_ordered(x.x);
    lo[1] = hi[1] = float_to_ordered(x.y);
    lo[2] = hi[2] = float_to_ordered(x.z);
  }
  const unsigned peers = uniform ? 0xffffffffu : __match_any_sync(0xffffffffu, s);
  const unsigned mm = __reduce_max_sync(0xffffffffu, m);
  r = __reduce_max_sync(peers, r);
#pragma unroll
  for (int d = 0; d < 3; d++)
  {
    lo[d] = __reduce_min_sync(peers, lo[d]);
    hi[d] = __reduce_max_sync(peers, hi[d]);
  }
  if (lane == 0)
  {
    s_red[warp][0] = mm;
    s_red[warp][1] = r;
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      s_red[warp][2 + d] = lo[d];
      s_red[warp][5 + d] = hi[d];
    }
  }
  __syncthreads();
  if (threadIdx.x < 8)
  { // q = 0: largest mass; q = 1..7: the uniform subhalo's radius and box
    const int q = threadIdx.x;
    if (q == 0 || uniform)
    {
      unsigned v = s_red[0][q];
      for (int w = 1; w < 8; w++)
        v = (q >= 2 && q < 5) ? min(v, s_red[w][q]) : max(v, s_red[w][q]);
      const int su = uniform ? D.seg_of[b0] : 0;
      if (q == 0)
      {
        if (v)
          atomicMax(W.mmax, v);
      }
      else if (q == 1)
        atomicMax(&W.rmax[su], v);
      else if (q < 5)
        atomicMin(&W.bb[6 * su + (q - 2)], v);
      else
        atomicMax(&W.bb[6 * su + 3 + (q - 5)], v);
    }
  }
  if (!uniform && valid && lane == __ffs(peers) - 1)
  {
    atomicMax(&W.rmax[s], r);
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      atomicMin(&W.bb[6 * s + d], lo[d]);
      atomicMax(&W.bb[6 * s + 3 + d], hi[d]);
    }
  }
}

__device__ __forceinline__ int radial_bin(float r, float rmax)
{
  if (!(r > 0.f) || !(rmax > 0.f))
    return 0;
  const float t = 4.f * __log2f(r / rmax) + (float)kBins;
  const int b = (int)floorf(t);
  return b < 0 ? 0 : (b > kBins - 1 ? kBins - 1 : b);
}

// Fixed-point mass histogram of every particle about the input centre.  A
// block whose particles all belong to one subhalo sums in shared memory first.
constexpr int kHistItems = 8;
__global__ void __launch_bounds__(256) k_feat_hist(DevState D, KParams K, WarmBufs W)
{
  __shared__ unsigned long long sh[kBins];
  __shared__ int s_one;
  const long long b0 = (long long)blockIdx.x * blockDim.x * kHistItems;
  const long long b1 = min(D.N, b0 + (long long)blockDim.x * kHistItems);
  if (b0 >= D.N)
    return;
  if (threadIdx.x == 0)
    s_one = (D.seg_of[b0] == D.seg_of[b1 - 1]) ? D.seg_of[b0] : -1;
  if (threadIdx.x < kBins)
    sh[threadIdx.x] = 0ull;
  __syncthreads();
  const float mmax = __uint_as_float(*W.mmax);
  const int one = s_one;
  for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x)
  {
    const int s = D.seg_of[i];
    const float4 x = D.pm[i];
    if (!(x.w > 0.f) || !(mmax > 0.f))
      continue;
    const int b = radial_bin(radius_about(x, D.ref_pos + 3 * s, K), __uint_as_float(W.rmax[s]));
    // <= 2^30, so a 32-bit conversion (64-bit ones issue to the FP64 pipe)
    const unsigned long long q = (unsigned long long)__float2uint_rn(__fmul_rn(__fdiv_rn(x.w, mmax), kQScale));
    if (one >= 0)
      atomicAdd(&sh[b], q);
    else
      atomicAdd(&W.hist[(long long)kBins * s + b], q);
  }
  if (one >= 0)
  {
    __syncthreads();
    if (threadIdx.x < kBins && sh[threadIdx.x])
      atomicAdd(&W.hist[(long long)kBins * one + threadIdx.x], sh[threadIdx.x]);
  }
}

// Per-subhalo profile: half-mass radius, circular speed and the monopole
// potential at the 65 bin edges e_k = r_max 2^((k-64)/4):
//   phi(e_k) = -(G/a) [ M(<e_k) / e_k + sum_{b>=k} m_b / (e_b 2^(1/8)) ]
// One warp per subhalo, two bins per lane.
__global__ void __launch_bounds__(256) k_feat_profile(DevState D, KParams K, WarmBufs W)
{
  const int s = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= D.S)
    return;
  float *tab = W.tab + (long long)kTab * s;
  // FP32 throughout (FP64 throughput is low on this GPU; the features feed a
  // BF16 network); the 64-bit bin masses are converted by bit arithmetic
  const float unit = __fmul_rn(__uint_as_float(*W.mmax), 1.f / kQScale); // exact: kQScale is 2^30
  const float rmax = __uint_as_float(W.rmax[s]);
  float m0, m1, lo_unused;
  ll_to_float2((long long)W.hist[(long long)kBins * s + 2 * lane], m0, lo_unused);
  ll_to_float2((long long)W.hist[(long long)kBins * s + 2 * lane + 1], m1, lo_unused);
  m0 *= unit;
  m1 *= unit;
  const float e0 = rmax * exp2f((2 * lane - kBins) * 0.25f), e1 = rmax * exp2f((2 * lane + 1 - kBins) * 0.25f);
  const float w0 = m0 / (e0 * 1.0905077326652577f), w1 = m1 / (e1 * 1.0905077326652577f);
  // inclusive scans of the pair sums
  float cm = m0 + m1, cw = w0 + w1;
  for (int o = 1; o < 32; o <<= 1)
  {
    const float a = __shfl_up_sync(0xffffffffu, cm, o), b = __shfl_up_sync(0xffffffffu, cw, o);
    if (lane >= o)
    {
      cm += a;
      cw += b;
    }
  }
  const float M = __shfl_sync(0xffffffffu, cm, 31), Wt = __shfl_sync(0xffffffffu, cw, 31);
  const float C0 = cm - m0 - m1, C1 = C0 + m0;       // M(<e_2l), M(<e_2l+1)
  const float O0 = Wt - (cw - w0 - w1), O1 = O0 - w0; // outer sums from bins 2l and 2l+1
  const float g = K.G_over_a;
  if (rmax > 0.f)
  {
    tab[4 + 2 * lane] = -g * (C0 / e0 + O0);
    tab[4 + 2 * lane + 1] = -g * (C1 / e1 + O1);
    if (lane == 31)
      tab[4 + kBins] = -g * M / rmax;
  }
  else
  {
    tab[4 + 2 * lane] = tab[4 + 2 * lane + 1] = 0.f;
    if (lane == 31)
      tab[4 + kBins] = 0.f;
  }
  // half-mass radius: the bin where the cumulative mass crosses M/2, log-interpolated
  const float half = 0.5f * M;
  float rh = -1.f;
  if (M > 0.f)
  {
    if (C0 < half && half <= C1 && m0 > 0.f)
      rh = e0 * exp2f(0.25f * (half - C0) / m0);
    else if (C1 < half && half <= C1 + m1 && m1 > 0.f)
      rh = e1 * exp2f(0.25f * (half - C1) / m1);
  }
  const unsigned has = __ballot_sync(0xffffffffu, rh > 0.f);
  if (has)
    rh = __shfl_sync(0xffffffffu, rh, __ffs(has) - 1);
  if (lane == 0)
  {
    tab[0] = rmax;
    if (!(rh > 0.f))
      rh = rmax;
    const float vc2 = (rh > 0.f) ? g * half / rh : 0.f;
    tab[1] = rh > 0.f ? 1.f / rh : 0.f;
    tab[2] = vc2 > 0.f ? 1.f / vc2 : 0.f;
    tab[3] = vc2 > 0.f ? rsqrtf(vc2) : 0.f;
  }
}

__device__ __forceinline__ float clamp16(float v) { return fminf(fmaxf(v, -16.f), 16.f); }

// Monopole potential from a subhalo's table, linear in log radius between edges.
__device__ __forceinline__ float mono_phi(const float *tab, float r)
{
  const float rmax = tab[0];
  if (!(r > 0.f) || !(rmax > 0.f))
    return tab[4];
  const float t = 4.f * __log2f(r / rmax) + (float)kBins;
  if (t <= 0.f)
    return tab[4];
  if (t >= (float)kBins)
    return tab[4 + kBins];
  const int k = (int)t;
  const float f = t - (float)k;
  return tab[4 + k] + f * (tab[5 + k] - tab[4 + k]);
}

__device__ __forceinline__ float species_code(int t)
{
  switch (t)
  {
  case 0:
    return 1.f;
  case 1:
    return 0.f;
  case 4:
    return -0.5f;
  case 5:
    return -1.f;
  case 2:
    return 0.25f;
  default:
    return 0.5f;
  }
}

__global__ void k_features(DevState D, KParams K, WarmBufs W)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += (long long)gridDim.x * blockDim.x)
  {
    const int s = D.seg_of[i];
    const float *tab = W.tab + (long long)kTab * s;
    const float4 x = D.pm[i], v = D.vu[i];
    const float r = radius_about(x, D.ref_pos + 3 * s, K);
    float dv[3];
    rel_vel(make_float3(x.x, x.y, x.z), make_float3(v.x, v.y, v.z), D.ref_pos + 3 * s, D.ref_vel + 3 * s, K, dv);
    const float v2 = norm2_rn(dv);
    float e = 0.5f * v2 + mono_phi(tab, r);
    if (K.thermal)
      e += v.w;
    const long long k = i - D.off[s];
    const int prior = has_prior(W, s) ? (k < W.nb_prev[s] ? 1 : -1) : 0;
    float *f = W.feat + kFeat * i;
    f[0] = log1pf(r * tab[1]);
    f[1] = fminf(sqrtf(v2) * tab[3], 16.f);
    f[2] = clamp16(e * tab[2]);
    f[3] = (prior == 1 && W.e_prev) ? clamp16(W.e_prev[i] * tab[2]) : 0.f;
    f[4] = (float)prior;
    f[5] = species_code(D.ty[i] & 7);
  }
}

// ---------------------------------------------------------------------------
// Warm start from a proposal
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool warm_eligible(const DevState &D, const WarmBufs &W, int s)
{
  return D.state[s] == kActive && (long long)D.n_s[s] >= W.min_n;
}

// flags: trusted; cnt: to test (eligible subhaloes only; scanned into F and X)
__global__ void k_warm_flags(DevState D, WarmBufs W)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > D.N)
    return;
  if (i == D.N)
  {
    D.flags[i] = 0;
    D.cnt[i] = 0;
    return;
  }
  const bool ok = warm_eligible(D, W, D.seg_of[i]);
  const uint8_t q = W.prop[i];
  D.flags[i] = (ok && q == 1) ? 1 : 0;
  D.cnt[i] = (ok && q == 0) ? 1 : 0;
}

// Which subhaloes start warm (the proposal leaves more than 1 -
// BoundMassPrecision of the particles out: otherwise the first iteration
// would converge and a cold start costs no more); the input frame is kept for
// a cold restart.
__global__ void k_warm_setup(DevState D, KParams K, WarmBufs W)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S)
    return;
  for (int q = 0; q < 3; q++)
  {
    D.ref0[6 * s + q] = D.ref_pos[3 * s + q];
    D.ref0[6 * s + 3 + q] = D.ref_vel[3 * s + q];
  }
  D.iter_extra[s] = 0;
  const int n = D.n_s[s];
  const int npred = D.F[D.off[s + 1]] - D.F[D.off[s]];
  const int ntest = D.X[D.off[s + 1]] - D.X[D.off[s]];
  // without the first test the uncertain particles stay in the set
  const int nkept = W.first_test ? npred : npred + ntest;
  const bool warm = warm_eligible(D, W, s) && (float)nkept < __fmul_rn((float)n, K.bmp);
  D.warm[s] = warm ? 1 : 0;
  D.flag_s[s] = warm ? 1 : 0;
  D.nexcl[s] = warm ? n - npred : 0;
  D.ntest[s] = warm ? ntest : 0;
  if (!warm)
    return;
  D.nbound[s] = npred;
  D.nlast[s] = npred;
  // the periodic wrap as a cold start decides it: from every particle's box
  double len = 0.;
  for (int d = 0; d < 3; d++)
  {
    const double l = (double)ordered_to_float(W.bb[6 * s + 3 + d]) - (double)ordered_to_float(W.bb[6 * s + d]);
    len = l > len ? l : len;
  }
  D.wrap[s] = K.periodic && (len > (double)K.half);
}

// join_uncertain (no first test): the uncertain particles are set members from
// the start (bnd), though they are left out of the first frame (positions
// past nbound); the frame kernels read positions, not bnd.
__global__ void k_warm_scatter(DevState D, int join_uncertain)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N)
    return;
  const int s = D.seg_of[i];
  if (D.warm[s] != 1)
    return;
  const long long off = D.off[s];
  const int rt = D.F[i] - D.F[off], ru = D.X[i] - D.X[off];
  const int nt = D.nbound[s], nu = D.ntest[s];
  const int pos = D.flags[i] ? rt : (D.cnt[i] ? nt + ru : nt + nu + (int)(i - off) - rt - ru);
  D.ord[off + pos] = (int)i;
  D.bnd[i] = (uint8_t)(D.flags[i] | (join_uncertain ? D.cnt[i] : 0));
}

// Frame and mass of the flagged subhaloes from the k_com sums (no convergence
// test); `clear` resets the flags.
__global__ void k_frame_flagged(DevState D, KParams K, int clear)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S || !D.flag_s[s])
    return;
  if (D.fin_off[s + 1] > D.fin_off[s])
    frame_from_sums(D, K, s);
  if (clear)
    D.flag_s[s] = 0;
}

// Plan of the first test: for each warm subhalo, every particle is a tree
// source (positions [0, n)) and the particles to test (positions [nbound,
// nbound + ntest)) are the targets, each keeping its self term.  The walk
// treats it as a correction walk: targets from the tgt list.
__global__ void k_plan_first(DevState D)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s > D.S)
    return;
  if (s == D.S)
  {
    D.src_cnt[s] = D.chunk_cnt[s] = D.part_cnt[s] = D.tail_cnt[s] = 0;
    return;
  }
  if (D.warm[s] != 1)
  {
    D.src_cnt[s] = D.chunk_cnt[s] = D.part_cnt[s] = D.tail_cnt[s] = 0;
    return;
  }
  const int ne = D.ntest[s];
  D.corr[s] = 1;
  D.ngrav[s] = 0;
  D.src_begin[s] = 0;
  D.src_cnt[s] = ne > 0 ? D.n_s[s] : 0; // no tree where nothing is tested
  D.self_cnt[s] = ne;
  D.tgt_cnt[s] = ne;
  D.chunk_cnt[s] = (ne + kWarp - 1) / kWarp;
  D.part_cnt[s] = ne;
  D.tail_cnt[s] = ne;
  D.bb_lo[3 * s] = D.bb_lo[3 * s + 1] = D.bb_lo[3 * s + 2] = 0xffffffffu;
  D.bb_hi[3 * s] = D.bb_hi[3 * s + 1] = D.bb_hi[3 * s + 2] = 0u;
}

// Targets of the first test in the tree's key order: the sources (packed by
// src_off, key-sorted in val) that are to be tested (flag, scan, scatter).
__global__ void k_first_tgt_flags(DevState D, WarmBufs W, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > total)
    return;
  D.flags[j] = (j < total && W.prop[D.val[j]] == 0) ? 1 : 0;
}

__global__ void k_first_tgt_scatter(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.src_off, D.S, min(j, total - 1));
  if (j >= total || !D.flags[j])
    return;
  D.tgt[D.off[s] + (D.F[j] - D.F[D.src_off[s]])] = (int)D.val[j];
}

// First-iteration energy of each target (the potential of every particle,
// the input frame; src/subhalo_unbind.cpp:563-580).
__global__ void k_readmit_energy(DevState D, KParams K, int total)
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
  const int p = D.tgt[D.off[s] + (j - D.part_off[s])];
  const float4 x = D.pm[p], v = D.vu[p];
  float dv[3];
  rel_vel(make_float3(x.x, x.y, x.z), make_float3(v.x, v.y, v.z), D.ref_pos + 3 * s, D.ref_vel + 3 * s, K, dv);
  float e = __fadd_rn(__fmul_rn(0.5f, norm2_rn(dv)), D.pot[p]);
  if (K.thermal)
    e = __fadd_rn(e, v.w);
  D.Ep[p] = e;
  D.flags[j] = e < 0.f ? 1 : 0;
}

// New order of positions [nbound, nbound + ntest): the particles the test
// keeps, then the others, each group in its previous order.
__global__ void k_readmit_scatter(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.tail_off, D.S, min(j, total - 1));
  if (j >= total)
    return;
  const int q = j - D.tail_off[s];
  const int nb = D.nbound[s];
  const int base = D.part_off[s];
  const int r = D.F[D.part_off[s + 1]] - D.F[base];
  const int rank = D.F[base + q] - D.F[base];
  const int pos = D.flags[base + q] ? nb + rank : nb + r + (q - rank);
  const long long off = D.off[s];
  D.ord_tmp[off + pos] = D.ord[off + nb + q];
}

__global__ void k_readmit_copy(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.tail_off, D.S, min(j, total - 1));
  if (j >= total)
    return;
  const long long g = D.off[s] + D.nbound[s] + (j - D.tail_off[s]);
  D.ord[g] = D.ord_tmp[g];
}

// Outcome of the first test by position ([nbound, nbound + ntest), packed
// like the targets): flags the kept particles and marks them bound.
__global__ void k_first_flags(DevState D, int total)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(D.tail_off, D.S, min(j, total - 1));
  if (j > total)
    return;
  if (j == total)
  {
    D.flags[j] = 0;
    return;
  }
  const int p = D.ord[D.off[s] + D.nbound[s] + (j - D.tail_off[s])];
  const bool kept = D.Ep[p] < 0.f;
  D.flags[j] = kept ? 1 : 0;
  D.bnd[p] = kept ? 1 : 0;
}

// After the first test: the set is the trusted particles plus the r the test
// kept.  A subhalo whose first iteration would already have converged
// ((float)Nbound >= (float)N * BoundMassPrecision, src/subhalo_unbind.cpp:690)
// is marked for a cold restart; the others are flagged for their first frame.
__global__ void k_first_apply(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S)
    return;
  D.flag_s[s] = 0;
  if (D.warm[s] != 1)
    return;
  const int r = D.F[D.part_off[s + 1]] - D.F[D.part_off[s]];
  const int nb = D.nbound[s] + r;
  D.nbound[s] = nb;
  D.nlast[s] = nb;
  D.corr[s] = 0;
  D.self_cnt[s] = 0;
  D.nexcl[s] = D.n_s[s] - nb;
  D.iter_extra[s] = 1; // the first iteration, done by the proposal and the test
  if ((float)nb >= __fmul_rn((float)D.n_s[s], K.bmp))
    D.warm[s] = 4;
  else
    D.flag_s[s] = 1;
}

// The set after the proposal without the first test: trusted plus uncertain.
// As after the test, a subhalo whose first iteration would already have
// converged is marked for a cold restart (warm = 4).
__global__ void k_untested_apply(DevState D, KParams K)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S)
    return;
  D.flag_s[s] = 0;
  if (D.warm[s] != 1)
    return;
  const int nb = D.nbound[s] + D.ntest[s];
  D.nbound[s] = nb;
  D.nlast[s] = nb;
  D.corr[s] = 0;
  D.self_cnt[s] = 0;
  D.nexcl[s] = D.n_s[s] - nb;
  D.iter_extra[s] = 1; // the first iteration, done by the proposal
  if ((float)nb >= __fmul_rn((float)D.n_s[s], K.bmp))
    D.warm[s] = 4;
}

// Cold restart of the warm subhaloes marked for it (warm = 4).
__global__ void k_warm_fallback(DevState D)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.S)
    return;
  const bool restart = D.warm[s] == 4;
  D.flag_s[s] = restart ? 1 : 0;
  if (!restart)
    return;
  const int n = D.n_s[s];
  D.warm[s] = 2;
  D.iter_extra[s] += D.iter[s];
  D.iter[s] = 0;
  D.nbound[s] = n;
  D.nlast[s] = n;
  D.state[s] = kActive;
  D.corr[s] = 0;
  D.wrap[s] = 0;
  D.tracers[s] = 0;
  D.mbound[s] = 0.f;
  D.ngrav[s] = 0;
  for (int q = 0; q < 3; q++)
  {
    D.ref_pos[3 * s + q] = D.ref0[6 * s + q];
    D.ref_vel[3 * s + q] = D.ref0[6 * s + 3 + q];
  }
}

__global__ void k_warm_fallback_particles(DevState D)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N)
    return;
  if (D.flag_s[D.seg_of[i]])
  {
    D.ord[i] = (int)i;
    D.bnd[i] = 1;
  }
}

// Training trace, in input order: which = 1 marks the survivors of the first
// iteration (positions [0, Nbound after it): later iterations only reorder
// inside that range); which = 0 marks the set whose potential decided the
// final bound set (positions [0, Nlast) of the last iteration).
__global__ void k_trace_labels(DevState D, uint8_t *__restrict__ label, int which)
{
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < D.N; g += (long long)gridDim.x * blockDim.x)
  {
    const int s = D.seg_of[g];
    const long long k = g - D.off[s];
    const int st = D.state[s];
    label[D.ord[g]] = (st != kEmpty && k < (which == 1 ? D.nb1[s] : D.nlast[s])) ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// Host orchestration (templated on the driver's memory policy)
// ---------------------------------------------------------------------------
struct WarmCounters
{
  long long warm_subhaloes = 0, excluded = 0, readmitted = 0, restarts = 0, readmit_rounds = 0;
};

// Largest radius, bounding box of every particle and largest mass.
template <class Mem>
void compute_extent(IterationDriver<Mem> &R, const WarmBufs &W)
{
  DevState &D = R.D;
  k_feat_reset<<<grid_for(D.S, 256), 256, 0, R.st>>>(D, W);
  R.launches++;
  if (D.N > 0)
  {
    k_feat_extent<<<grid_for(D.N, 256), 256, 0, R.st>>>(D, R.K, W);
    R.launches++;
  }
  R.check();
}

template <class Mem>
void compute_features(IterationDriver<Mem> &R, const WarmBufs &W)
{
  DevState &D = R.D;
  cudaStream_t st = R.st;
  compute_extent(R, W);
  R.mem.check(cudaMemsetAsync(W.hist, 0, sizeof(unsigned long long) * kBins * (size_t)D.S, st));
  if (D.N > 0)
  {
    k_feat_hist<<<grid_for(D.N, 256 * kHistItems), 256, 0, st>>>(D, R.K, W);
    R.launches++;
  }
  k_feat_profile<<<grid_for((long long)D.S * 32, 256), 256, 0, st>>>(D, R.K, W);
  R.launches++;
  if (D.N > 0)
  {
    k_features<<<grid_for(D.N, 256), 256, 0, st>>>(D, R.K, W);
    R.launches++;
  }
  R.check();
}

// Frame and mass of the bound sets of the subhaloes flagged in flag_s (clears the flags).
template <class Mem>
void flagged_frames(IterationDriver<Mem> &R)
{
  DevState &D = R.D;
  cudaStream_t st = R.st;
  k_plan_counts<<<grid_for(D.S + 1, 256), 256, 0, st>>>(D, 2);
  R.launches++;
  const int total = R.scan_counts(D.fin_cnt, D.fin_off, D.S);
  if (total > 0)
  {
    D.com_ipt = com_items_per_thread(total); // k_frame_flagged reads the partials with the same blocking
    k_com<<<grid_for((total + D.com_ipt - 1) / D.com_ipt, 256), 256, 0, st>>>(D, R.K, total);
    R.launches++;
  }
  k_frame_flagged<<<grid_for(D.S, 256), 256, 0, st>>>(D, R.K, 1);
  R.launches++;
  R.check();
}

// The plain method's first test for the particles to test of the warm
// subhaloes (see k_plan_first); returns how many it keeps.
template <class Mem>
long long first_test(IterationDriver<Mem> &R, const WarmBufs &W)
{
  DevState &D = R.D;
  cudaStream_t st = R.st;
  const int S = D.S;
  k_plan_first<<<grid_for(S + 1, 256), 256, 0, st>>>(D);
  R.launches++;
  R.check();
  int tot[4];
  R.scan_counts4(D.src_cnt, D.src_off, D.chunk_cnt, D.chunk_off, D.part_cnt, D.part_off, D.tail_cnt, D.tail_off, S,
                 tot);
  const int src_total = tot[0], chunk_total = tot[1], part_total = tot[2], tail_total = tot[3];
  R.mem.mark(6);
  if (src_total > 0)
  {
    R.build_tree(src_total);
    k_first_tgt_flags<<<grid_for(src_total + 1, 256), 256, 0, st>>>(D, W, src_total);
    R.launches++;
    scan<int, false>(D.flags, D.F, src_total + 1, R.mem.scan_scratch(src_total + 1), st, &R.launches);
    k_first_tgt_scatter<<<grid_for(src_total, 256), 256, 0, st>>>(D, src_total);
    R.launches++;
    R.check();
  }
  R.mem.mark(2);
  R.walk(chunk_total);
  R.mem.mark(1);
  long long kept = 0;
  if (part_total > 0)
  {
    k_readmit_energy<<<grid_for(part_total + 1, 256), 256, 0, st>>>(D, R.K, part_total);
    k_first_flags<<<grid_for(tail_total + 1, 256), 256, 0, st>>>(D, tail_total);
    R.launches += 2;
    scan<int, false>(D.flags, D.F, tail_total + 1, R.mem.scan_scratch(tail_total + 1), st, &R.launches);
    R.check();
    kept = R.read_int(D.F + tail_total);
    k_readmit_scatter<<<grid_for(tail_total, 256), 256, 0, st>>>(D, tail_total);
    k_readmit_copy<<<grid_for(tail_total, 256), 256, 0, st>>>(D, tail_total);
    R.launches += 2;
  }
  else
    R.mem.check(cudaMemsetAsync(D.F, 0, sizeof(int), st)); // k_first_apply reads F[part_off[s]]
  k_first_apply<<<grid_for(S, 256), 256, 0, st>>>(D, R.K);
  R.launches++;
  R.check();
  return kept;
}

// Warm start from W.prop: partition, first test, cold restarts, first frame,
// exact iteration, final sort.  have_extent: compute_features ran.
template <class Mem>
void warm_run(IterationDriver<Mem> &R, const WarmBufs &W, WarmCounters &C, bool have_extent)
{
  DevState &D = R.D;
  cudaStream_t st = R.st;
  const int S = D.S;
  const unsigned sb = grid_for(S, 256);
  if (!have_extent)
    compute_extent(R, W); // the periodic-wrap decision of a cold start needs every particle's box
  if (D.N > 0)
  {
    k_warm_flags<<<grid_for(D.N + 1, 256), 256, 0, st>>>(D, W);
    R.launches++;
    scan<int, false>(D.flags, D.F, D.N + 1, R.mem.scan_scratch(D.N + 1), st, &R.launches);
    scan<int, false>(D.cnt, D.X, D.N + 1, R.mem.scan_scratch(D.N + 1), st, &R.launches);
    R.check();
  }
  else
  {
    R.mem.check(cudaMemsetAsync(D.F, 0, sizeof(int), st));
    R.mem.check(cudaMemsetAsync(D.X, 0, sizeof(int), st));
  }
  k_warm_setup<<<sb, 256, 0, st>>>(D, R.K, W);
  R.launches++;
  if (D.N > 0)
  {
    k_warm_scatter<<<grid_for(D.N, 256), 256, 0, st>>>(D, W.first_test ? 0 : 1);
    R.launches++;
  }
  R.check();
  if (W.first_test)
  {
    C.readmitted += first_test(R, W);
    C.readmit_rounds++;
  }
  else
  { // the first frame from the trusted particles alone (k_warm_setup flagged
    // the warm subhaloes), then the uncertain ones join the set
    R.mem.mark(6); // the proposal ends here
    flagged_frames(R);
    k_untested_apply<<<sb, 256, 0, st>>>(D, R.K);
    R.launches++;
    R.check();
  }
  long long restarts = 0;
  { // left-out counts and the subhaloes marked for a cold restart, in one host read
    std::vector<int> nex(S), wm(S);
    R.mem.check(cudaMemcpyAsync(nex.data(), D.nexcl, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
    R.mem.check(cudaMemcpyAsync(wm.data(), D.warm, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
    R.mem.check(cudaStreamSynchronize(st));
    R.host_syncs++;
    for (int v : nex)
      C.excluded += v;
    for (int v : wm)
      restarts += (v == 4);
  }
  if (W.first_test)
    flagged_frames(R); // the frame of the set the second iteration evaluates
  k_warm_fallback<<<sb, 256, 0, st>>>(D); // subhaloes whose first iteration converges run cold
  R.launches++;
  if (D.N > 0 && restarts > 0)
  {
    k_warm_fallback_particles<<<grid_for(D.N, 256), 256, 0, st>>>(D);
    R.launches++;
  }
  R.check();
  R.mem.mark(3);
  R.iterate();
  R.finish();
}

} // namespace
} // namespace hbtg
