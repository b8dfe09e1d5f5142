// props.cuh - properties of the unbound subhaloes from their bound sets:
//   Subhalo_t::CalculateProfileProperties  src/subhalo.cpp:175-243
//   Snapshot_t::SphericalOverdensitySize   src/snapshot.cpp:258-282
//   Subhalo_t::CalculateShape              src/subhalo.cpp:245-309
//   Subhalo_t::TruncateSource              src/subhalo_unbind.cpp:843-853
//
// The bound particles of every subhalo are packed (item j = bound position k
// of subhalo s).  One pass computes each item's distance from the most-bound
// particle and its shape terms (summed per subhalo in double); the items are
// then sorted by distance within their subhalo (radix sort by distance, then
// stably by subhalo), the cumulative masses come from one segmented scan in
// double, and the profile quantities from per-subhalo reductions over the
// sorted items.  Every per-item value is formed in the reference's float
// arithmetic (no fused multiply-adds); the double sums are exact for
// ordinary particle masses, so their order does not change the result.
// Ties in distance do not change any output: within a run of equal radii the
// cumulative mass, and so v = M(<r)/r and the overdensity test, are largest
// at the run's last rank whatever the order inside the run.
#pragma once

#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"
#include "primitives.cuh"

namespace hbtg
{
namespace
{

struct PropState
{
  int S;
  const long long *off;      // [S+1] particle offsets
  const float *pos, *mass;   // input particles
  const long long *order;    // bound order (local indices)
  const long long *nbound;   // [S]
  const float *mbound;       // [S]
  const float *mb_pos;       // [3S] most-bound positions (the profile's centre)
  int *cnt, *fin_off;        // [S+1] bound counts and their exclusive scan
  float *rr, *mm;            // [T] distance and mass of each item
  uint32_t *k32, *val, *k32_alt, *val_alt;
  double *mcum;              // [T] cumulative mass in sorted order
  unsigned long long *vkey;  // [S] packed (v, ~rank) of the largest v = M(<r)/r
  int *so_rank;              // [S] outermost rank inside the overdensity radius
  double *shape;             // [12 S] inertia sums, then the weighted ones
  float box, half;
  int periodic;
  float soft, velocity_unit, rho_vir, relax;
  int snapshot;
};

// PeriodicDistance (src/config_parser.h:220-231) in float.
__device__ __forceinline__ float periodic_distance_f(const float *a, const float *b, const PropState &P)
{
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
  {
    d[k] = __fsub_rn(a[k], b[k]);
    if (P.periodic)
      d[k] = nearest_f(d[k], P.half, P.box);
  }
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
}

__global__ void k_prop_init(PropState P)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s > P.S)
    return;
  // a count outside [0, particles of the subhalo] is clamped: reads stay in the segment
  P.cnt[s] = s < P.S ? (int)max(0ll, min(P.nbound[s], P.off[s + 1] - P.off[s])) : 0;
  if (s == P.S)
    return;
  P.vkey[s] = 0ull;
  P.so_rank[s] = -1;
  for (int q = 0; q < 12; q++)
    P.shape[12 * s + q] = 0.;
}

// Items: distances, masses, sort keys; shape sums (CalculateShape skips the
// first bound particle, the centre itself).  Each thread takes
// kItemsPerThread consecutive items and flushes its double sums per subhalo.
__global__ void k_prop_items(PropState P, int total)
{
  const long long first = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kItemsPerThread;
  if (first >= total)
    return;
  int s = find_segment<int>(P.fin_off, P.S, (int)first);
  double acc[12];
  for (int q = 0; q < 12; q++)
    acc[q] = 0.;
  auto flush = [&](int seg) {
    for (int q = 0; q < 12; q++)
      if (acc[q] != 0.)
      {
        atomicAdd(&P.shape[12 * seg + q], acc[q]);
        acc[q] = 0.;
      }
  };
  const int last = (int)min((long long)total, first + kItemsPerThread);
  for (int j = (int)first; j < last; j++)
  {
    if (j >= P.fin_off[s + 1])
    {
      flush(s);
      s = find_segment<int>(P.fin_off, P.S, j);
    }
    const int k = j - P.fin_off[s];
    const long long g = P.off[s] + P.order[P.off[s] + k];
    const float *x = P.pos + 3 * g, *c = P.mb_pos + 3 * s;
    const float m = P.mass[g];
    const float r = periodic_distance_f(c, x, P);
    P.rr[j] = r;
    P.mm[j] = m;
    P.k32[j] = __float_as_uint(r); // r >= 0: the bits order as the values
    P.val[j] = (uint32_t)j;
    if (k == 0)
      continue;
    float dx = __fsub_rn(x[0], c[0]), dy = __fsub_rn(x[1], c[1]), dz = __fsub_rn(x[2], c[2]);
    if (P.periodic)
    {
      dx = nearest_f(dx, P.half, P.box);
      dy = nearest_f(dy, P.half, P.box);
      dz = nearest_f(dz, P.half, P.box);
    }
    const float dx2 = __fmul_rn(dx, dx), dy2 = __fmul_rn(dy, dy), dz2 = __fmul_rn(dz, dz);
    acc[0] += (double)__fmul_rn(dx2, m);
    acc[1] += (double)__fmul_rn(__fmul_rn(dx, dy), m);
    acc[2] += (double)__fmul_rn(__fmul_rn(dx, dz), m);
    acc[3] += (double)__fmul_rn(dy2, m);
    acc[4] += (double)__fmul_rn(__fmul_rn(dy, dz), m);
    acc[5] += (double)__fmul_rn(dz2, m);
    const float dr2 = __fdiv_rn(__fadd_rn(__fadd_rn(dx2, dy2), dz2), m);
    acc[6] += (double)__fdiv_rn(dx2, dr2);
    acc[7] += (double)__fdiv_rn(__fmul_rn(dx, dy), dr2);
    acc[8] += (double)__fdiv_rn(__fmul_rn(dx, dz), dr2);
    acc[9] += (double)__fdiv_rn(dy2, dr2);
    acc[10] += (double)__fdiv_rn(__fmul_rn(dy, dz), dr2);
    acc[11] += (double)__fdiv_rn(dz2, dr2);
  }
  flush(s);
}

// Second sort key: the item's subhalo.
__global__ void k_prop_segkeys(PropState P, const uint32_t *__restrict__ v, uint32_t *__restrict__ k, int total)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total)
    k[i] = (uint32_t)find_segment<int>(P.fin_off, P.S, (int)v[i]);
}

struct PropMassLoad
{
  PropState P;
  const uint32_t *sorted;
  __device__ SegD operator()(long long i) const
  {
    const int s = find_segment<int>(P.fin_off, P.S, (int)i);
    return SegD{(double)P.mm[sorted[i]], i == P.fin_off[s] ? 1 : 0};
  }
};
struct PropMassStore
{
  double *out;
  __device__ void operator()(long long i, const SegD &v) const { out[i] = v.v; }
};

// Per sorted item (rank q of subhalo s): the clamped radius, v = M(<r)/r
// (the largest kept per subhalo, the first on ties) and the overdensity
// test (the outermost rank that passes it kept per subhalo).
__global__ void k_prop_profile(PropState P, const uint32_t *__restrict__ sorted, int total)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = find_segment_warp(P.fin_off, P.S, min(i, total - 1));
  if (i >= total)
    return;
  const int q = i - P.fin_off[s];
  const int nb = P.fin_off[s + 1] - P.fin_off[s];
  if (nb <= 1)
    return;
  float r = P.rr[sorted[i]];
  if (r < P.soft)
    r = P.soft; // resolution
  const float m = __double2float_rn(P.mcum[i]);
  const float v = __fdiv_rn(m, r);
  atomicMax(&P.vkey[s],
            ((unsigned long long)__float_as_uint(v) << 32) | (unsigned long long)(0xffffffffu - (unsigned)q));
  if (m > __fmul_rn(__fmul_rn(__fmul_rn(P.rho_vir, r), r), r))
    atomicMax(&P.so_rank[s], q);
}

struct PropOut
{
  float *rmax, *vmax, *rhalf, *renclose, *r200, *m200, *last_vmax, *rmax_last, *inertia, *inertia_w;
  int *snap_last;
  long long *nsource;
};

__device__ __forceinline__ float clamped_radius(const PropState &P, const uint32_t *sorted, int i)
{
  const float r = P.rr[sorted[i]];
  return r < P.soft ? P.soft : r;
}

// One thread per subhalo: the profile and shape outputs and the truncated
// source length.
__global__ void k_prop_finish(PropState P, const uint32_t *__restrict__ sorted, PropOut O)
{
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= P.S)
    return;
  const int nb = P.fin_off[s + 1] - P.fin_off[s];
  const long long n = P.off[s + 1] - P.off[s];
  if (O.nsource)
  {
    const long long ns = nb <= 1 ? nb : (long long)__fmul_rn((float)nb, P.relax);
    O.nsource[s] = ns > n ? n : ns;
  }
  if (nb <= 1)
  {
    O.rmax[s] = O.vmax[s] = O.rhalf[s] = O.renclose[s] = O.r200[s] = O.m200[s] = 0.f;
    for (int q = 0; q < 6; q++)
      O.inertia[6 * s + q] = O.inertia_w[6 * s + q] = 0.f;
    return;
  }
  const int base = P.fin_off[s];
  const unsigned long long key = P.vkey[s];
  const int qmax = (int)(0xffffffffu - (unsigned)(key & 0xffffffffull));
  const float v = __uint_as_float((unsigned)(key >> 32));
  const float rmax = clamped_radius(P, sorted, base + qmax);
  const float vmax = __fsqrt_rn(__fmul_rn(v, P.velocity_unit));
  O.rmax[s] = rmax;
  O.vmax[s] = vmax;
  O.rhalf[s] = clamped_radius(P, sorted, base + nb / 2);
  O.renclose[s] = clamped_radius(P, sorted, base + nb - 1);
  const int so = P.so_rank[s];
  if (so >= 0)
  {
    const float m = __double2float_rn(P.mcum[base + so]);
    O.m200[s] = m;
    O.r200[s] = __double2float_rn(pow((double)__fdiv_rn(m, P.rho_vir), 1.0 / 3));
  }
  if (vmax >= O.last_vmax[s])
  {
    O.snap_last[s] = P.snapshot;
    O.last_vmax[s] = vmax;
    O.rmax_last[s] = rmax;
  }
  const float mb = P.mbound[s];
  for (int q = 0; q < 6; q++)
  {
    O.inertia[6 * s + q] = __fdiv_rn(__double2float_rn(P.shape[12 * s + q]), mb);
    O.inertia_w[6 * s + q] = __fdiv_rn(__double2float_rn(P.shape[12 * s + 6 + q]), mb);
  }
}

} // namespace
} // namespace hbtg
