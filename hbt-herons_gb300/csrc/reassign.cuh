// reassign.cuh - particle reassignment before unbinding
// (SubhaloSnapshot_t::ReassignParticles, src/subhalo_reassign_gas.cpp:65-197).
//
// Each FoF group's tracer particles form one geometric tree (the unbinding
// tree's build over the tracers, with cell bounding boxes; coordinates
// unwrapped about the group's first tracer, for the tree and its pruning
// only).  One thread per non-tracer particle finds its k nearest tracers by
// exact distance (double, from the float coordinates with the periodic wrap,
// as the reference's GeoTree_t::Search computes it) and then reads off what
// GeoTree_t::NearestNeighbours (src/geometric_tree.cpp:108-142) returns.
// That search widens its radius R_j (R_0 = SofteningHalo / 10 in float, each
// 1.26 times the last, rounded to float) until its collector holds
// min(tracers, k) entries; search j collects every tracer with
// |dx|, |dy|, |dz| <= R_j and r^2 < R_j * R_j (a float product), into the
// same collector, which keeps the k smallest r^2 it was given.  So a tracer
// first found by search jmin counts J - jmin + 1 times, J being the last
// search, and the list is the distinct tracers of those k entries, the
// nearest last.  Searches j < J collect fewer than k tracers, all among the
// k nearest, so the k nearest decide everything (up to ties in r^2, and to a
// tracer that the axis test rejects although r^2 < R_j * R_j: a rounding
// gap of one float ulp in R_j).
#pragma once

#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"

namespace hbtg
{
namespace
{

constexpr int kMaxNeighbours = 32;

struct ReState
{
  int S;                     // subhaloes
  int G;                     // FoF groups
  const long long *off;      // [S+1] particles of each subhalo
  const int *sub_group;      // [S] FoF group of each subhalo
  const long long *gpart;    // [G+1] particles of each group (contiguous)
  const float *pos;          // [3N] raw positions
  const uint8_t *type;       // [N]
  long long *dest;           // [N] out
  int *flags, *rank;         // [N+1] tracer flags and their exclusive scan
  int *tg;                   // [T] particle of each packed tracer
  int *tsub;                 // [T] subhalo of each packed tracer
  int tracer_mask;
  float box, half, r0, eps;
  int periodic, k;
};

__device__ __forceinline__ bool re_tracer(const ReState &R, long long g)
{
  return ((1 << (int)R.type[g]) & R.tracer_mask) != 0;
}

__global__ void k_re_flags(ReState R, long long n)
{
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g > n)
    return;
  R.flags[g] = (g < n && re_tracer(R, g)) ? 1 : 0;
}

// Packs the tracers by group (the reference's order: subhalo, then particle)
// into the tree state D: unwrapped position, unit mass, identity order.
__global__ void k_re_pack(ReState R, DevState D, long long n)
{
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n || !R.flags[g])
    return;
  const int s = find_segment<long long>(R.off, R.S, g);
  const int t = R.rank[g];
  R.tg[t] = (int)g;
  R.tsub[t] = s;
  D.seg_of[t] = R.sub_group[s];
  D.ord[t] = t;
  D.ty[t] = 0;
}

// The group's first tracer as the unwrapping point (positions as the
// reference's NEAREST sees them from it).
__device__ __forceinline__ float unwrap(float x, float ref, const ReState &R)
{
  const float d = __fsub_rn(x, ref);
  return R.periodic ? __fadd_rn(ref, nearest_f(d, R.half, R.box)) : x;
}

__global__ void k_re_unwrap(ReState R, DevState D, int total)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total)
    return;
  const int h = D.seg_of[t];
  const float *ref = R.pos + 3 * (long long)R.tg[D.off[h]];
  const float *x = R.pos + 3 * (long long)R.tg[t];
  D.pm[t] = make_float4(unwrap(x[0], ref[0], R), unwrap(x[1], ref[1], R), unwrap(x[2], ref[2], R), 1.f);
}

// First packed tracer of each group.
__global__ void k_re_goff(ReState R, long long *goff)
{
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h <= R.G)
    goff[h] = R.rank[R.gpart[h]];
}

// Per group: the tracers are the sources when the group has non-tracers.
__global__ void k_re_plan(ReState R, DevState D)
{
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h > D.S)
    return;
  if (h == D.S)
  {
    D.src_cnt[h] = 0;
    return;
  }
  const int nt = (int)(D.off[h + 1] - D.off[h]);
  const long long np = R.gpart[h + 1] - R.gpart[h];
  D.state[h] = kActive;
  D.iter[h] = 1;
  D.corr[h] = 1; // no key-order record
  D.wrap[h] = 0;
  D.ngrav[h] = 0;
  D.src_begin[h] = 0;
  D.src_cnt[h] = (nt > 0 && np > nt) ? nt : 0;
  for (int q = 0; q < 6; q++)
    D.factor[6 * h + q] = 1.f;
  for (int d = 0; d < 3; d++)
  {
    D.bb_lo[3 * h + d] = 0xffffffffu;
    D.bb_hi[3 * h + d] = 0u;
  }
}

// Exact squared distance and largest axis offset, as GeoTree_t::Search.
__device__ __forceinline__ double re_d2(const float *a, const float *q, const ReState &R, double &dmax)
{
  double d2 = 0.;
  dmax = 0.;
#pragma unroll
  for (int k = 0; k < 3; k++)
  {
    double d = (double)a[k] - (double)q[k];
    if (R.periodic)
      d = nearest_d(d, (double)R.half, (double)R.box);
    dmax = fmax(dmax, fabs(d));
    d2 = __dadd_rn(d2, __dmul_rn(d, d));
  }
  return d2;
}

// The first search that collects a tracer at (d2, dmax).
__device__ __forceinline__ int re_jmin(double d2, double dmax, float r0)
{
  int j = 0;
  for (float Rr = r0; j < 4096; Rr = __double2float_rn((double)Rr * 1.26), j++)
    if (dmax <= (double)Rr && d2 < (double)__fmul_rn(Rr, Rr))
      break;
  return j;
}

// One thread per particle: dest = the subhalo a non-tracer moves to, or -1.
__global__ void k_re_query(ReState R, DevState D, long long n)
{
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n)
    return;
  R.dest[g] = -1;
  if (re_tracer(R, g))
    return;
  const int s = find_segment<long long>(R.off, R.S, g);
  const int h = R.sub_group[s];
  const int nt = (int)(D.off[h + 1] - D.off[h]);
  if (nt == 0 || D.src_cnt[h] == 0)
    return;
  const int k = R.k;
  const float *q = R.pos + 3 * g;
  const float *ref = R.pos + 3 * (long long)R.tg[D.off[h]];
  const float uq[3] = {unwrap(q[0], ref[0], R), unwrap(q[1], ref[1], R), unwrap(q[2], ref[2], R)};
  double bd[kMaxNeighbours];
  int bi[kMaxNeighbours];
  int cnt = 0;
  const float4 *T = D.nodes;
  const int root = D.src_off[h] + 2 * D.X[D.src_off[h]];
  const int end = __float_as_int(T[root + 1].y);
  int idx = root;
  while (idx < end)
  {
    const float4 a = T[idx];
    if (slot_is_cell(a.w))
    {
      const float4 b = T[idx + 1];
      const int skip = __float_as_int(b.y);
      if (cnt == k)
      { // prune a box farther than the k-th distance (with a margin for the unwrapped floats)
        const float gx = fmaxf(fmaxf(a.x - uq[0], uq[0] - b.x), 0.f);
        const float gy = fmaxf(fmaxf(a.y - uq[1], uq[1] - b.z), 0.f);
        const float gz = fmaxf(fmaxf(a.z - uq[2], uq[2] - b.w), 0.f);
        const double dmin = sqrt((double)gx * gx + (double)gy * gy + (double)gz * gz) - (double)R.eps;
        if (dmin > 0. && dmin * dmin > bd[k - 1])
        {
          idx = max(skip, idx + 2);
          continue;
        }
      }
      idx += 2;
      continue;
    }
    const int t = __float_as_int(a.w); // the packed tracer (k_tree_leaf_ids)
    double dmax;
    const double d2 = re_d2(R.pos + 3 * (long long)R.tg[t], q, R, dmax);
    if (cnt < k || d2 < bd[cnt - 1])
    { // insertion into the sorted list (equal distances keep the earlier)
      int at = cnt < k ? cnt : k - 1;
      while (at > 0 && bd[at - 1] > d2)
      {
        bd[at] = bd[at - 1];
        bi[at] = bi[at - 1];
        at--;
      }
      bd[at] = d2;
      bi[at] = t;
      if (cnt < k)
        cnt++;
    }
    idx++;
  }
  // the widening searches, from the k nearest
  int jm[kMaxNeighbours];
  int jmax = 0;
  for (int i = 0; i < cnt; i++)
  {
    double dmax;
    const double d2 = re_d2(R.pos + 3 * (long long)R.tg[bi[i]], q, R, dmax);
    jm[i] = re_jmin(d2, dmax, R.r0);
    jmax = max(jmax, jm[i]);
  }
  const int to_find = min(nt, k);
  int J = jmax;
  long long cum = 0;
  for (int j = 0; j <= jmax; j++)
  {
    int nj = 0;
    for (int i = 0; i < cnt; i++)
      nj += jm[i] <= j;
    cum += nj;
    if (min(cum, (long long)k) >= to_find)
    {
      J = j;
      break;
    }
  }
  long long taken = 0;
  int first = -1;
  bool found = false;
  for (int i = 0; i < cnt; i++)
  {
    if (jm[i] > J)
      continue;
    if (taken >= k)
      break;
    if (first < 0)
      first = bi[i];
    if (R.tsub[bi[i]] == s)
      found = true;
    taken += J - jm[i] + 1;
  }
  if (!found && first >= 0)
  {
    const int to = R.tsub[first];
    if (to >= 0 && to != s)
      R.dest[g] = to;
  }
}

} // namespace
} // namespace hbtg
