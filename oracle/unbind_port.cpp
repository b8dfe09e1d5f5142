/*
 * unbind_port.cpp — TEST INFRASTRUCTURE (oracle) and CPU baseline.
 *
 * The project's own CPU restatement of HBT-HERONS' iterative unbinding, used
 * (a) as the checker of the GPU path in tests, smoke() and bench.py, and
 * (b) as the timed CPU baseline on machines where the reference sources are
 * absent.  It is NOT part of the product: libhbtg.so never calls it.
 *
 * It restates, with the same float/double rounding so that its results are
 * bit-identical to the reference built with the same flags:
 *   Subhalo_t::Unbind                     src/subhalo_unbind.cpp:463-808
 *   EnergySnapshot_t (masses, CoM frame,  src/subhalo_unbind.cpp:46-393
 *     AverageKinematics, GetPotentialEnergy)
 *   RemoveUnboundParticles                src/subhalo_unbind.cpp:35-44
 *   OctTree_t::Build                      src/oct_tree.tpp:12-142
 *   GravityTree_t::UpdateInternalNodes    src/gravity_tree.cpp:18-80
 *   GravityTree_t::EvaluatePotential      src/gravity_tree.cpp:82-166
 *   GravityTree_t::BindingEnergy          src/gravity_tree.cpp:168-178
 *   Snapshot_t::RelativeVelocity          src/snapshot.h:135-148
 *   Subhalo_t::CountParticleTypes         src/subhalo.cpp:311-393
 *   Subhalo_t::GetCorePhaseSpaceProperties src/subhalo_merge.cpp:94-181
 *   Subhalo_t::CalculateProfileProperties src/subhalo.cpp:175-243 (with
 *     Snapshot_t::SphericalOverdensitySize src/snapshot.cpp:258-282)
 *   Subhalo_t::CalculateShape             src/subhalo.cpp:245-309
 *   Subhalo_t::TruncateSource             src/subhalo_unbind.cpp:843-853
 *   SubhaloSnapshot_t::ReassignParticles  src/subhalo_reassign_gas.cpp:65-197 (with
 *     GeoTree_t::NearestNeighbours        src/geometric_tree.cpp:108-142)
 * and potential subsampling (MaxSampleSizeOfPotentialEstimate > 0):
 *   PrepareParticlesForSubsampling        src/subhalo_unbind.cpp:430-443
 *   Get/SetMassUpscaleFactor[PerType]     src/subhalo_unbind.cpp:290-391
 *   CountUnsampledParticles               src/subhalo_unbind.cpp:446-461
 *   RefineBindingEnergyOrder              src/subhalo_unbind.cpp:395-425
 *
 * Build with -ffp-contract=off (oracle/build_oracle.py) so that no multiply-
 * add is fused: the reference is built the same way for comparison.
 */
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <omp.h>
#include <vector>

#include "hbt_unbind_gpu.h"

namespace
{

/* HBTConfig values as the reference stores them (HBTReal = float). */
struct Cfg
{
  float box, half;
  bool periodic;
  float soft;
  float res, res_half;
  float theta2;
  float bmp;
  int64_t min_part, min_tracer;
  int tracer_mask, nosub_mask;
  int64_t core_min;
  float core_factor;
  bool dm_only, thermal, want_energy, want_potential;
  float G, a, hz;
  int max_iter;
  int64_t max_sample;
  bool refine, upscale_per_type, prepare_inside;
  float refine_frac;
};

inline double wrap_d(double x, const Cfg &c)
{
  return x > (double)c.half ? x - (double)c.box : (x < -(double)c.half ? x + (double)c.box : x);
}
inline float wrap_f(float x, const Cfg &c)
{
  return x > c.half ? x - c.box : (x < -c.half ? x + c.box : x);
}

/* One particle of a subhalo, as the reference's Particle_t (src/snapshot.h:62-106). */
struct Part
{
  int64_t id;
  float x[3];
  float v[3];
  float m;
  float u;
  int type;
  int64_t input_index;
};

struct Entry /* ParticleEnergy_t, src/subhalo_unbind.cpp:12-16 */
{
  float E;
  int64_t p;
};

inline bool is_tracer(const Part &q, const Cfg &c) { return c.dm_only || (((1 << q.type) & c.tracer_mask) != 0); }
inline bool no_subsample(const Part &q, const Cfg &c) { return !c.dm_only && (((1 << q.type) & c.nosub_mask) != 0); }

/* RelativeVelocity (src/snapshot.h:135-148), all float. */
inline void rel_vel(const float *x, const float *v, const float *rx, const float *rv, const Cfg &c, float *dv)
{
  const float hz_a = c.hz * c.a;
  for (int j = 0; j < 3; j++)
  {
    float dx = x[j] - rx[j];
    if (c.periodic)
      dx = wrap_f(dx, c);
    dv[j] = v[j] - rv[j];
    dv[j] += hz_a * dx;
  }
}
inline float norm2_f(const float *d) { return d[0] * d[0] + d[1] * d[1] + d[2] * d[2]; }

/* ------------------------------------------------------------------------
 * Octree with the reference's insertion build and threaded walk.
 * Items 0..n-1 are the sources (particles), items >= n are cells.
 * ---------------------------------------------------------------------- */
class Tree
{
  /* One cell: its eight sons while the tree is built, then its multipole and
   * links, in the same 64 bytes, as the reference's TreeCell_t union
   * (src/oct_tree.h:30-45); finalize copies a cell's sons out before it
   * writes the multipole over them. */
  union Cell
  {
    int64_t son[8];
    struct
    {
      float s[3];
      float len, mass;
      int64_t sibling, nextnode;
    };
  };
  static_assert(sizeof(Cell) == 64, "cell size");
  std::vector<Cell> cells;
  std::vector<int64_t> next_of;
  const float *const *xs = nullptr; /* per source: pointer to float[3] */
  const float *ms = nullptr;        /* per source mass */
  int64_t n = 0;
  const Cfg *cfg = nullptr;

  Cell &cell(int64_t id) { return cells[id - n]; }

  void finalize(int64_t no, int64_t sib, double len)
  {
    int64_t sons[8];
    for (int j = 0; j < 8; j++)
      sons[j] = cell(no).son[j];
    cell(no).len = (float)len;
    cell(no).sibling = sib;
    int first = 0;
    while (sons[first] < 0)
      first++;
    cell(no).nextnode = sons[first];
    double mass = 0., com[3] = {0., 0., 0.};
    for (int j = first; j < 8; j++)
    {
      const int64_t it = sons[j];
      if (it < 0)
        continue;
      int64_t nxt = sib;
      for (int k = j + 1; k < 8; k++)
        if (sons[k] >= 0)
        {
          nxt = sons[k];
          break;
        }
      if (it < n)
      {
        const double mm = ms[it];
        mass += mm;
        for (int d = 0; d < 3; d++)
          com[d] += xs[it][d] * mm;
        next_of[it] = nxt;
      }
      else
      {
        finalize(it, nxt, len >= (double)cfg->res ? len / 2. : len);
        const double mm = cell(it).mass;
        mass += mm;
        for (int d = 0; d < 3; d++)
          com[d] += cell(it).s[d] * mm;
      }
    }
    cell(no).mass = (float)mass;
    for (int d = 0; d < 3; d++)
      cell(no).s[d] = (float)(com[d] / mass);
  }

public:
  /* OctTree_t::Build (src/oct_tree.tpp:12-142) followed by
   * UpdateInternalNodes (src/gravity_tree.cpp:50-80). */
  void build(int64_t np, const float *const *x, const float *m, const Cfg &c)
  {
    n = np;
    xs = x;
    ms = m;
    cfg = &c;
    cells.clear();
    cells.reserve(std::max<int64_t>(10, np));
    next_of.assign(np, -1);
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++)
      lo[d] = hi[d] = x[0][d];
    for (int64_t i = 1; i < np; i++)
      for (int d = 0; d < 3; d++)
      {
        const double v = x[i][d];
        if (v > hi[d])
          hi[d] = v;
        else if (v < lo[d])
          lo[d] = v;
      }
    double side = hi[0] - lo[0];
    for (int d = 1; d < 3; d++)
      if (hi[d] - lo[d] > side)
        side = hi[d] - lo[d];
    double centre0[3];
    for (int d = 0; d < 3; d++)
      centre0[d] = 0.5 * (hi[d] + lo[d]);
    const double half0 = 0.5 * side;
    auto new_cell = [&]() {
      Cell cc;
      for (int j = 0; j < 8; j++)
        cc.son[j] = -1;
      cells.push_back(cc);
      return n + (int64_t)cells.size() - 1;
    };
    new_cell(); /* root = n */
    for (int64_t i = 0; i < np; i++)
    {
      int64_t node = n;
      double half = half0, ctr[3] = {centre0[0], centre0[1], centre0[2]};
      for (;;)
      {
        half *= 0.5;
        int sub = 0;
        for (int d = 0; d < 3; d++)
        {
          if ((double)x[i][d] > ctr[d])
          {
            ctr[d] += half;
            sub += 1 << d;
          }
          else
            ctr[d] -= half;
        }
        const int64_t occ = cell(node).son[sub];
        if (occ < 0)
        {
          cell(node).son[sub] = i;
          break;
        }
        if (occ < n)
        {
          const int64_t fresh = new_cell();
          cell(node).son[sub] = fresh;
          node = fresh;
          int sub2;
          if (half < (double)c.res_half)
          {
            sub2 = (int)(8.0 * drand48());
            if (sub2 >= 8)
              sub2 = 7;
          }
          else
          {
            sub2 = 0;
            for (int d = 0; d < 3; d++)
              if ((double)x[occ][d] > ctr[d])
                sub2 += 1 << d;
          }
          cell(node).son[sub2] = occ;
        }
        else
          node = occ;
      }
    }
    finalize(n, -1, side);
  }

  int64_t num_cells() const { return (int64_t)cells.size(); }

  /* GravityTree_t::EvaluatePotential (src/gravity_tree.cpp:82-166). */
  double potential(const float *tp, float target_mass, int64_t *interactions) const
  {
    const Cfg &c = *cfg;
    const double h = 2.8 * (double)c.soft, h_inv = 1.0 / h;
    double pot = (double)(target_mass / c.soft);
    const double px = tp[0], py = tp[1], pz = tp[2];
    int64_t no = n, count = 0;
    while (no >= 0)
    {
      double dx, dy, dz, mass, r2;
      if (no < n)
      {
        dx = xs[no][0] - px;
        dy = xs[no][1] - py;
        dz = xs[no][2] - pz;
        if (c.periodic)
        {
          dx = wrap_d(dx, c);
          dy = wrap_d(dy, c);
          dz = wrap_d(dz, c);
        }
        mass = ms[no];
        no = next_of[no];
        r2 = dx * dx + dy * dy + dz * dz;
      }
      else
      {
        const Cell &q = cells[no - n];
        dx = q.s[0] - px;
        dy = q.s[1] - py;
        dz = q.s[2] - pz;
        if (c.periodic)
        {
          dx = wrap_d(dx, c);
          dy = wrap_d(dy, c);
          dz = wrap_d(dz, c);
        }
        mass = q.mass;
        r2 = dx * dx + dy * dy + dz * dz;
        const float len2 = q.len * q.len;
        if ((double)len2 > r2 * (double)c.theta2)
        {
          no = q.nextnode;
          continue;
        }
        no = q.sibling;
      }
      count++;
      const double r = std::sqrt(r2);
      if (r >= h)
        pot -= mass / r;
      else
      {
        const double u = r * h_inv;
        double wp;
        if (u < 0.5)
          wp = -2.8 + u * u * (5.333333333333 + u * u * (6.4 * u - 9.6));
        else
          wp = -3.2 + 0.066666666667 / u + u * u * (10.666666666667 + u * (-16.0 + u * (9.6 - 2.133333333333 * u)));
        pot += mass * h_inv * wp;
      }
    }
    if (interactions)
      *interactions += count;
    return pot * (double)c.G / (double)c.a;
  }
};

std::atomic<int64_t> g_interactions{0};
std::atomic<int64_t> g_cells{0};

/* Subhalo_t::Unbind restated for one subhalo of the batch. */
void unbind_one(const Cfg &c, const hbtg_batch *b, int64_t s, bool inner_parallel)
{
  const int64_t off = b->offsets[s], n = b->offsets[s + 1] - off;
  float ref_pos[3], ref_vel[3], mb_pos[3], mb_vel[3];
  for (int d = 0; d < 3; d++)
  {
    ref_pos[d] = b->ref_pos[3 * s + d];
    ref_vel[d] = b->ref_vel[3 * s + d];
    mb_pos[d] = b->mostbound_pos[3 * s + d];
    mb_vel[d] = b->mostbound_vel[3 * s + d];
  }
  int64_t most_bound_id = b->most_bound_id[s];
  int64_t nbound = 0, nbound_type[HBTG_TYPE_MAX] = {0};
  float mbound = 0.f, mbound_type[HBTG_TYPE_MAX] = {0.f};
  int64_t tracer_index = 0;
  float kin[HBTG_KIN_STRIDE] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float core[HBTG_CORE_STRIDE] = {0.f};
  int iterations = 0;
  int status = HBTG_SUB_CONVERGED;

  std::vector<Part> P(n);
  for (int64_t k = 0; k < n; k++)
  {
    const int64_t g = off + k;
    Part &q = P[k];
    q.id = b->id[g];
    for (int d = 0; d < 3; d++)
    {
      q.x[d] = b->pos[3 * g + d];
      q.v[d] = b->vel[3 * g + d];
    }
    q.m = b->mass[g];
    q.u = (c.thermal && b->u) ? b->u[g] : 0.f;
    q.type = c.dm_only ? 1 : (b->type ? b->type[g] : 1);
    q.input_index = k;
  }

  auto finish_core = [&](int64_t nb) {
    /* GetCorePhaseSpaceProperties (src/subhalo_merge.cpp:94-181) */
    if (nb == 0)
    {
      for (int d = 0; d < 3; d++)
      {
        core[d] = mb_pos[d];
        core[3 + d] = mb_vel[d];
      }
      core[6] = core[7] = 0.f;
      return;
    }
    int64_t used = 0;
    double msum = 0, ps[3] = {0, 0, 0}, ps2[3] = {0, 0, 0}, vs[3] = {0, 0, 0}, vs2[3] = {0, 0, 0};
    const int64_t core_size = std::max((int64_t)((float)nb * c.core_factor), c.core_min);
    double origin[3] = {0, 0, 0};
    if (c.periodic)
      for (int d = 0; d < 3; d++)
        origin[d] = P[0].x[d];
    for (int pass = 0; pass < 2 && used != core_size; pass++)
    {
      for (int i = 0; i < (int)nb; i++)
      {
        const bool t = is_tracer(P[i], c);
        if ((t && pass == 0) || (!t && pass == 1))
        {
          used++;
          const float m = P[i].m;
          msum += m;
          for (int d = 0; d < 3; d++)
          {
            double dx = P[i].x[d];
            if (c.periodic)
              dx = wrap_d(dx - origin[d], c);
            ps[d] += m * dx;
            ps2[d] += m * dx * dx;
            const double dv = P[i].v[d];
            vs[d] += m * dv;
            vs2[d] += m * dv * dv;
          }
        }
        if (used == core_size)
          break;
      }
    }
    for (int d = 0; d < 3; d++)
    {
      ps[d] /= msum;
      ps2[d] /= msum;
      float cp = (float)ps[d];
      if (c.periodic)
        cp += origin[d];
      core[d] = cp;
      ps2[d] -= ps[d] * ps[d];
      vs[d] /= msum;
      vs2[d] /= msum;
      core[3 + d] = (float)vs[d];
      vs2[d] -= vs[d] * vs[d];
    }
    core[6] = (float)std::sqrt(ps2[0] + ps2[1] + ps2[2]);
    core[7] = (float)std::sqrt(vs2[0] + vs2[1] + vs2[2]);
  };

  std::vector<Entry> E(n);
  int64_t interactions = 0;

  if (n == 0)
  {
    status = HBTG_SUB_EMPTY;
    tracer_index = -1; /* the reference returns before SetTracerIndex (src/subhalo_unbind.cpp:472-489) */
    finish_core(0);
  }
  else
  {
    /* PrepareParticlesForSubsampling (src/subhalo_unbind.cpp:430-443, 522-524) */
    int64_t nunsample = 0;
    if (c.max_sample > 0 && n > c.max_sample)
    {
      if (c.prepare_inside)
      {
        auto it = std::partition(P.begin(), P.end(), [&](const Part &q) { return no_subsample(q, c); });
        nunsample = it - P.begin();
        std::random_shuffle(P.begin() + nunsample, P.end());
      }
      else
        while (nunsample < n && no_subsample(P[nunsample], c))
          nunsample++;
    }
    for (int64_t i = 0; i < n; i++)
      E[i].p = i;
    nbound = n;
    /* initial AccumulateMass (src/subhalo_unbind.cpp:537-541) */
    {
      if (c.dm_only)
      {
        float m = 0.f;
        for (int64_t i = 0; i < n; i++)
          m += P[i].m;
        mbound = m;
      }
      else
      {
        float mt[HBTG_TYPE_MAX] = {0.f};
        for (int64_t i = 0; i < n; i++)
          mt[P[i].type] += P[i].m;
        float m = 0.f;
        for (int t = 0; t < HBTG_TYPE_MAX; t++)
          m += mt[t];
        mbound = m;
      }
    }
    int64_t nlast = n;
    bool correction = false;
    float old_pos[3] = {0, 0, 0}, old_vel[3] = {0, 0, 0};
    Tree tree;
    std::vector<const float *> src_x;
    std::vector<float> src_m;
    float factor[HBTG_TYPE_MAX] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
    /* EnergySnapshot_t::GetMass with the current upscale factors (src/subhalo_unbind.cpp:91-101) */
    auto scaled_mass = [&](const Part &q) -> float {
      if (c.dm_only)
        return q.m * factor[1];
      return no_subsample(q, c) ? q.m : q.m * factor[q.type];
    };
    auto gather_sources = [&](int64_t first, int64_t count) {
      src_x.resize(count);
      src_m.resize(count);
      for (int64_t i = 0; i < count; i++)
      {
        src_x[i] = P[E[first + i].p].x;
        src_m[i] = scaled_mass(P[E[first + i].p]);
      }
    };
    for (;;)
    {
      iterations++;
      if (correction)
      {
        float dV[3];
        rel_vel(old_pos, old_vel, ref_pos, ref_vel, c, dV);
        const float dK = (float)(0.5 * norm2_f(dV));
        gather_sources(nbound, nlast - nbound);
        tree.build(nlast - nbound, src_x.data(), src_m.data(), c);
        g_cells += tree.num_cells();
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : interactions) if (inner_parallel)
        for (int64_t i = 0; i < nbound; i++)
        {
          const Part &q = P[E[i].p];
          float ov[3];
          rel_vel(q.x, q.v, old_pos, old_vel, c, ov);
          const float dot = ov[0] * dV[0] + ov[1] * dV[1] + ov[2] * dV[2];
          const double phi = tree.potential(q.x, 0.f, &interactions);
          E[i].E = (float)((double)E[i].E + ((double)(dot + dK) - phi));
        }
        nlast = nbound;
      }
      else
      {
        nlast = nbound;
        const float mlast = mbound;
        /* SetMassUpscaleFactor (src/subhalo_unbind.cpp:374-391) */
        int64_t ngrav = nlast;
        if (c.max_sample > 0 && !(nlast < c.max_sample + nunsample))
        {
          ngrav = c.max_sample + nunsample;
          if (!c.dm_only && c.upscale_per_type)
          { /* GetMassUpscaleFactorPerParticleType (src/subhalo_unbind.cpp:323-361) */
            float sub[HBTG_TYPE_MAX] = {0.f}, tot[HBTG_TYPE_MAX] = {0.f};
            for (int64_t i = nunsample; i < nunsample + c.max_sample; i++)
              sub[P[E[i].p].type] += P[E[i].p].m;
            for (int64_t i = nunsample + c.max_sample; i < nlast; i++)
              tot[P[E[i].p].type] += P[E[i].p].m;
            for (int t = 0; t < HBTG_TYPE_MAX; t++)
              tot[t] += sub[t];
            for (int t = 0; t < HBTG_TYPE_MAX; t++)
              factor[t] = sub[t] ? tot[t] / sub[t] : 0.f;
            float true_m = 0.f, scaled_m = 0.f;
            for (int t = 0; t < HBTG_TYPE_MAX; t++)
            {
              true_m += tot[t];
              scaled_m += sub[t] * factor[t];
            }
            for (int t = 0; t < HBTG_TYPE_MAX; t++)
              factor[t] *= true_m / scaled_m;
          }
          else
          { /* GetMassUpscaleFactor (src/subhalo_unbind.cpp:290-317) */
            float munsampled = 0.f;
            for (int64_t i = 0; i < nunsample; i++)
              munsampled += P[E[i].p].m;
            const float mtrue = mlast - munsampled;
            float msub = 0.f;
            for (int64_t i = nunsample; i < nunsample + c.max_sample; i++)
              msub += P[E[i].p].m;
            for (int t = 0; t < HBTG_TYPE_MAX; t++)
              factor[t] = mtrue / msub;
          }
        }
        gather_sources(0, ngrav);
        tree.build(ngrav, src_x.data(), src_m.data(), c);
        g_cells += tree.num_cells();
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : interactions) if (inner_parallel)
        for (int64_t i = 0; i < nlast; i++)
        {
          const Part &q = P[E[i].p];
          const double phi = tree.potential(q.x, i < ngrav ? scaled_mass(q) : 0.f, &interactions);
          float dv[3];
          rel_vel(q.x, q.v, ref_pos, ref_vel, c, dv);
          float e = (float)((double)norm2_f(dv) * 0.5 + phi);
          if (c.thermal)
            e += q.u;
          E[i].E = e;
        }
        for (int t = 0; t < HBTG_TYPE_MAX; t++) /* ResetMassUpscaleFactor */
          factor[t] = 1.f;
      }
      /* RemoveUnboundParticles: stable partition on E < 0 */
      {
        std::vector<Entry> tmp;
        tmp.reserve(nlast);
        for (int64_t i = 0; i < nlast; i++)
          if (E[i].E < 0)
            tmp.push_back(E[i]);
        const int64_t nb = (int64_t)tmp.size();
        for (int64_t i = 0; i < nlast; i++)
          if (!(E[i].E < 0))
            tmp.push_back(E[i]);
        std::copy(tmp.begin(), tmp.end(), E.begin());
        nbound = nb;
      }
      { /* CountUnsampledParticles (src/subhalo_unbind.cpp:446-461) */
        int64_t k = 0;
        while (k < nunsample && no_subsample(P[E[k].p], c))
          k++;
        nunsample = k;
      }
      int64_t tracers = 0;
      if (c.dm_only)
        tracers = nbound;
      else
        for (int64_t i = 0; i < nbound; i++)
        {
          if (is_tracer(P[E[i].p], c))
            tracers++;
          if (tracers >= c.min_tracer)
            break;
        }
      if (nbound < c.min_part || tracers < c.min_tracer)
      {
        for (int d = 0; d < 3; d++)
        {
          ref_pos[d] = mb_pos[d];
          ref_vel[d] = mb_vel[d];
        }
        nbound = 0;
        mbound = 0.f;
        status = HBTG_SUB_DISRUPTED;
        break;
      }
      std::sort(E.begin() + nbound, E.begin() + nlast, [](const Entry &a, const Entry &q) { return a.E < q.E; });
      const int64_t ndiff = nlast - nbound;
      if (ndiff < nbound && (c.max_sample <= 0 || ndiff < c.max_sample))
      {
        correction = true;
        for (int d = 0; d < 3; d++)
        {
          old_pos[d] = ref_pos[d];
          old_vel[d] = ref_vel[d];
        }
      }
      /* CentreOfMassReferenceFrame (src/subhalo_unbind.cpp:151-198) */
      {
        double M = 0, wx[3] = {0, 0, 0}, wv[3] = {0, 0, 0}, origin[3] = {0, 0, 0};
        if (c.periodic)
          for (int d = 0; d < 3; d++)
            origin[d] = P[E[0].p].x[d];
        for (int64_t i = 0; i < nbound; i++)
        {
          const Part &q = P[E[i].p];
          const float m = q.m;
          M += m;
          for (int d = 0; d < 3; d++)
          {
            wx[d] += c.periodic ? wrap_d(q.x[d] - origin[d], c) * m : (double)(q.x[d] * m);
            wv[d] += q.v[d] * m;
          }
        }
        for (int d = 0; d < 3; d++)
        {
          wx[d] /= M;
          wv[d] /= M;
        }
        if (c.periodic)
          for (int d = 0; d < 3; d++)
            wx[d] += origin[d];
        for (int d = 0; d < 3; d++)
        {
          ref_pos[d] = (float)wx[d];
          ref_vel[d] = (float)wv[d];
        }
        mbound = (float)M;
      }
      if ((float)nbound >= (float)nlast * c.bmp)
      {
        std::sort(E.begin(), E.begin() + nbound, [](const Entry &a, const Entry &q) { return a.E < q.E; });
        if (c.max_sample > 0 && c.refine && nbound > c.max_sample)
        { /* RefineBindingEnergyOrder (src/subhalo_unbind.cpp:395-425, 715-738) */
          const int64_t size = std::max(c.max_sample, (int64_t)(c.refine_frac * (float)nbound));
          gather_sources(0, size);
          tree.build(size, src_x.data(), src_m.data(), c);
          g_cells += tree.num_cells();
          std::vector<Entry> inner(size);
          for (int64_t i = 0; i < size; i++)
          {
            const Part &q = P[E[i].p];
            const double phi = tree.potential(q.x, q.m, &interactions);
            float dv[3];
            rel_vel(q.x, q.v, ref_pos, ref_vel, c, dv);
            inner[i].p = i;
            inner[i].E = (float)((double)norm2_f(dv) * 0.5 + phi);
          }
          std::sort(inner.begin(), inner.end(), [](const Entry &a, const Entry &q) { return a.E < q.E; });
          std::vector<Entry> moved(size);
          for (int64_t i = 0; i < size; i++)
            moved[i] = E[inner[i].p];
          for (int64_t i = 0; i < size; i++)
            E[i] = moved[i];
        }
        std::vector<Part> Q(n);
        for (int64_t i = 0; i < n; i++)
        {
          Q[i] = P[E[i].p];
          E[i].p = i;
        }
        P.swap(Q);
        for (int d = 0; d < 3; d++)
        {
          mb_pos[d] = P[0].x[d];
          mb_vel[d] = P[0].v[d];
        }
        break;
      }
      if (iterations >= c.max_iter)
      {
        status = HBTG_SUB_MAX_ITER;
        break;
      }
    }
    /* AverageKinematics (src/subhalo_unbind.cpp:200-249) */
    if (nbound > 1)
    {
      double Et = 0, K = 0, L0 = 0, L1 = 0, L2 = 0, M = 0;
      for (int64_t i = 0; i < nbound; i++)
      {
        const Part &q = P[E[i].p];
        const float m = q.m;
        Et += E[i].E * m;
        if (c.thermal)
          Et -= q.u * m;
        double dx[3], dv[3];
        for (int j = 0; j < 3; j++)
        {
          dx[j] = q.x[j] - ref_pos[j];
          if (c.periodic)
            dx[j] = wrap_d(dx[j], c);
          dx[j] *= c.a;
          dv[j] = q.v[j] - ref_vel[j] + c.hz * dx[j];
          K += dv[j] * dv[j] * m;
        }
        L0 += (dx[1] * dv[2] - dx[2] * dv[1]) * m;
        L1 += (dx[2] * dv[0] - dx[0] * dv[2]) * m;
        L2 += (dx[0] * dv[1] - dx[1] * dv[0]) * m;
        M += m;
      }
      Et /= M;
      K *= 0.5 / M;
      kin[0] = (float)(Et - K);
      kin[1] = (float)K;
      kin[2] = (float)(L0 / M);
      kin[3] = (float)(L1 / M);
      kin[4] = (float)(L2 / M);
    }
    /* CountParticleTypes (src/subhalo.cpp:311-393) */
    int64_t first_tracer = -1;
    for (int64_t i = 0; i < nbound; i++)
    {
      const Part &q = P[i];
      nbound_type[q.type]++;
      mbound_type[q.type] += q.m;
      if (first_tracer < 0 && is_tracer(q, c))
        first_tracer = i;
    }
    tracer_index = (c.dm_only || first_tracer < 0) ? 0 : first_tracer;
    if (status == HBTG_SUB_CONVERGED || status == HBTG_SUB_MAX_ITER)
      most_bound_id = P[tracer_index].id;
    finish_core(nbound);
  }

  /* outputs */
  for (int64_t k = 0; k < n; k++)
    b->order[off + k] = P[k].input_index;
  b->nbound[s] = nbound;
  b->mbound[s] = mbound;
  for (int t = 0; t < HBTG_TYPE_MAX; t++)
  {
    if (b->nbound_type)
      b->nbound_type[HBTG_TYPE_MAX * s + t] = nbound_type[t];
    if (b->mbound_type)
      b->mbound_type[HBTG_TYPE_MAX * s + t] = c.dm_only ? 0.f : mbound_type[t];
  }
  b->tracer_index[s] = tracer_index;
  b->most_bound_id[s] = most_bound_id;
  for (int d = 0; d < 3; d++)
  {
    b->ref_pos[3 * s + d] = ref_pos[d];
    b->ref_vel[3 * s + d] = ref_vel[d];
    b->mostbound_pos[3 * s + d] = mb_pos[d];
    b->mostbound_vel[3 * s + d] = mb_vel[d];
  }
  if (b->kinematics)
    for (int j = 0; j < HBTG_KIN_STRIDE; j++)
      b->kinematics[HBTG_KIN_STRIDE * s + j] = kin[j];
  if (b->core)
    for (int j = 0; j < HBTG_CORE_STRIDE; j++)
      b->core[HBTG_CORE_STRIDE * s + j] = core[j];
  if (b->energy)
    for (int64_t k = 0; k < nbound; k++)
      b->energy[off + k] = E[k].E;
  if (b->potential)
    for (int64_t k = 0; k < nbound; k++)
    {
      /* GetPotentialEnergy (src/subhalo_unbind.cpp:114-135) */
      const Part &q = P[k];
      float e = E[k].E;
      if (c.thermal)
        e -= q.u;
      for (int j = 0; j < 3; j++)
      {
        double dx = q.x[j] - ref_pos[j];
        if (c.periodic)
          dx = wrap_d(dx, c);
        dx *= c.a;
        const double dv = q.v[j] - ref_vel[j] + c.hz * dx;
        e -= 0.5 * dv * dv;
      }
      b->potential[off + k] = e;
    }
  b->iterations[s] = iterations;
  b->status[s] = status;
  g_interactions += interactions;
}

Cfg make_cfg(const hbtg_params *p, const hbtg_batch *b)
{
  Cfg c;
  c.box = (float)p->box_size;
  c.half = (float)((double)c.box / 2.);
  c.periodic = p->periodic != 0;
  c.soft = (float)p->softening;
  c.res = (float)p->tree_node_resolution;
  c.res_half = (float)((double)c.res / 2.);
  const float theta = (float)p->open_angle;
  c.theta2 = theta * theta;
  c.bmp = (float)p->bound_mass_precision;
  c.min_part = (int)p->min_num_part;
  c.min_tracer = (int)p->min_num_tracer;
  c.tracer_mask = p->tracer_type_mask;
  c.nosub_mask = p->no_subsample_mask;
  c.core_min = p->sub_core_size_min;
  c.core_factor = (float)p->sub_core_size_factor;
  c.dm_only = p->dm_only != 0;
  c.thermal = p->thermal != 0;
  c.want_energy = b && b->energy;
  c.want_potential = b && b->potential;
  c.G = (float)p->G;
  c.a = (float)p->scale_factor;
  c.hz = (float)p->hubble;
  c.max_iter = p->max_iterations > 0 ? p->max_iterations : 1000000;
  c.max_sample = p->max_sample_size;
  c.refine = p->refine_most_bound != 0;
  c.refine_frac = (float)p->refine_fraction;
  c.upscale_per_type = p->upscale_per_type != 0;
  c.prepare_inside = p->prepared_subsample == 0;
  return c;
}

} // namespace

/* Batch entry with the library's contract.  nthreads <= 0 = all cores.
 * inner_parallel = 0: OpenMP dynamic,1 over subhaloes (RefineParticles);
 * inner_parallel = 1: subhaloes in turn, the energy loops parallel inside. */
extern "C" int oracle_unbind_batch(const hbtg_params *p, hbtg_batch *b, int nthreads, int inner_parallel)
{
  if (!p || !b || b->n_sub < 0 || (b->n_sub > 0 && !b->offsets))
    return HBTG_ERR_INVALID;
  for (int64_t s = 0; s < b->n_sub; s++)
    if (b->offsets[s + 1] < b->offsets[s])
      return HBTG_ERR_INVALID;
  const Cfg c = make_cfg(p, b);
  srand48(p->seed);
  srand((unsigned)p->seed);
  g_interactions = 0;
  g_cells = 0;
  if (nthreads <= 0)
    nthreads = omp_get_max_threads();
  if (inner_parallel)
  {
    omp_set_num_threads(nthreads);
    for (int64_t s = 0; s < b->n_sub; s++)
      unbind_one(c, b, s, true);
  }
  else
  {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t s = 0; s < b->n_sub; s++)
      unbind_one(c, b, s, false);
  }
  return HBTG_OK;
}

/* Interactions (accepted nodes + particles) evaluated by the last batch. */
extern "C" int64_t oracle_last_interactions() { return g_interactions.load(); }
extern "C" int64_t oracle_last_cells() { return g_cells.load(); }

/* Tree potential of `ns` sources at `nt` targets (specific, times G/a, as
 * EvaluatePotential).  target_mass may be NULL (no self term removed). */
extern "C" int oracle_tree_potential(const hbtg_params *p, int64_t ns, const float *src_pos, const float *src_mass,
                                     int64_t nt, const float *tgt_pos, const float *tgt_mass, double *out)
{
  if (ns <= 0)
    return HBTG_ERR_INVALID;
  const Cfg c = make_cfg(p, nullptr);
  std::vector<const float *> xs(ns);
  for (int64_t i = 0; i < ns; i++)
    xs[i] = src_pos + 3 * i;
  Tree t;
  srand48(p->seed);
  t.build(ns, xs.data(), src_mass, c);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < nt; i++)
    out[i] = t.potential(tgt_pos + 3 * i, tgt_mass ? tgt_mass[i] : 0.f, nullptr);
  return HBTG_OK;
}

/* FP64 direct-sum potential with the same softening kernel and periodic
 * wrap (no tree): the precision oracle for the FP32 walk. */
extern "C" int oracle_direct_potential(const hbtg_params *p, int64_t ns, const float *src_pos, const float *src_mass,
                                       int64_t nt, const float *tgt_pos, const float *tgt_mass, double *out)
{
  const Cfg c = make_cfg(p, nullptr);
  const double h = 2.8 * (double)c.soft, h_inv = 1.0 / h;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; i++)
  {
    double pot = tgt_mass ? (double)(tgt_mass[i] / c.soft) : 0.0;
    for (int64_t j = 0; j < ns; j++)
    {
      double d[3];
      for (int k = 0; k < 3; k++)
      {
        d[k] = (double)src_pos[3 * j + k] - (double)tgt_pos[3 * i + k];
        if (c.periodic)
          d[k] = wrap_d(d[k], c);
      }
      const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      const double m = src_mass[j];
      if (r >= h)
        pot -= m / r;
      else
      {
        const double u = r * h_inv;
        const double wp = u < 0.5 ? -2.8 + u * u * (5.333333333333 + u * u * (6.4 * u - 9.6))
                                  : -3.2 + 0.066666666667 / u +
                                      u * u * (10.666666666667 + u * (-16.0 + u * (9.6 - 2.133333333333 * u)));
        pot += m * h_inv * wp;
      }
    }
    out[i] = pot * (double)c.G / (double)c.a;
  }
  return HBTG_OK;
}

/* ------------------------------------------------------------------------
 * Properties of the bound sets of an unbinding call's outputs (see
 * hbtg_subhalo_properties in include/hbt_unbind_gpu.h), in the reference's
 * float/double arithmetic.
 * ------------------------------------------------------------------------ */
namespace
{
struct Prof
{
  float r, m, v;
};

/* PeriodicDistance (src/config_parser.h:220-231): float differences, NEAREST
 * in float, float sum of squares, correctly rounded square root. */
float periodic_distance(const float *a, const float *b, const Cfg &c)
{
  float d[3];
  for (int k = 0; k < 3; k++)
  {
    d[k] = a[k] - b[k];
    if (c.periodic)
      d[k] = wrap_f(d[k], c);
  }
  return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

void properties_one(const hbtg_batch *b, int64_t s, int snapshot_id, double source_relax, const Cfg &c,
                    hbtg_props *o)
{
  const int64_t off = b->offsets[s], n = b->offsets[s + 1] - off;
  const int64_t nb = b->nbound[s];
  const float *cen = b->mostbound_pos + 3 * s;
  auto pos_of = [&](int64_t k) { return b->pos + 3 * (off + b->order[off + k]); };
  auto mass_of = [&](int64_t k) { return b->mass[off + b->order[off + k]]; };
  /* CalculateProfileProperties (src/subhalo.cpp:175-243) */
  if (nb <= 1)
  {
    o->rmax[s] = o->vmax[s] = o->rhalf[s] = o->renclose[s] = 0.f;
    o->r200[s] = o->m200[s] = 0.f;
  }
  else
  {
    const float velocity_unit = c.G / c.a;
    std::vector<Prof> prof(nb);
    for (int64_t i = 0; i < nb; i++)
    {
      prof[i].r = periodic_distance(cen, pos_of(i), c);
      prof[i].m = mass_of(i);
    }
    std::stable_sort(prof.begin(), prof.end(), [](const Prof &x, const Prof &y) { return x.r < y.r; });
    double m_cum = 0.;
    for (auto &q : prof)
      q.m = (float)(m_cum += q.m);
    for (auto &q : prof)
    {
      if (q.r < c.soft)
        q.r = c.soft;
      q.v = q.m / q.r;
    }
    int64_t imax = 0;
    for (int64_t i = 1; i < nb; i++)
      if (prof[imax].v < prof[i].v)
        imax = i;
    o->rmax[s] = prof[imax].r;
    o->vmax[s] = std::sqrt(prof[imax].v * velocity_unit);
    o->rhalf[s] = prof[nb / 2].r;
    o->renclose[s] = prof[nb - 1].r;
    /* SphericalOverdensitySize (src/snapshot.cpp:258-282), VirialFactor 200 */
    const float rho = (float)((double)((200.f * c.hz) * c.hz) / 2.0 / (double)c.G * (double)c.a * (double)c.a *
                              (double)c.a);
    for (int64_t i = nb - 1; i >= 0; i--)
      if (prof[i].m > rho * prof[i].r * prof[i].r * prof[i].r)
      {
        o->m200[s] = prof[i].m;
        o->r200[s] = (float)std::pow((double)(prof[i].m / rho), 1.0 / 3);
        break;
      }
    if (o->vmax[s] >= o->last_vmax[s])
    {
      o->snap_last[s] = snapshot_id;
      o->last_vmax[s] = o->vmax[s];
      o->rmax_last[s] = o->rmax[s];
    }
  }
  /* CalculateShape (src/subhalo.cpp:245-309) */
  double I[6] = {0, 0, 0, 0, 0, 0}, W[6] = {0, 0, 0, 0, 0, 0};
  if (nb > 1)
  {
    for (int64_t i = 1; i < nb; i++)
    {
      const float m = mass_of(i);
      const float *x = pos_of(i);
      float dx = x[0] - cen[0], dy = x[1] - cen[1], dz = x[2] - cen[2];
      if (c.periodic)
      {
        dx = wrap_f(dx, c);
        dy = wrap_f(dy, c);
        dz = wrap_f(dz, c);
      }
      const float dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
      I[0] += dx2 * m;
      I[3] += dy2 * m;
      I[5] += dz2 * m;
      I[1] += dx * dy * m;
      I[2] += dx * dz * m;
      I[4] += dy * dz * m;
      float dr2 = dx2 + dy2 + dz2;
      dr2 /= m;
      W[0] += dx2 / dr2;
      W[3] += dy2 / dr2;
      W[5] += dz2 / dr2;
      W[1] += dx * dy / dr2;
      W[2] += dx * dz / dr2;
      W[4] += dy * dz / dr2;
    }
    for (int q = 0; q < 6; q++)
    {
      o->inertia[6 * s + q] = (float)I[q] / b->mbound[s];
      o->inertia_w[6 * s + q] = (float)W[q] / b->mbound[s];
    }
  }
  else
    for (int q = 0; q < 6; q++)
      o->inertia[6 * s + q] = o->inertia_w[6 * s + q] = 0.f;
  /* TruncateSource (src/subhalo_unbind.cpp:843-853) */
  if (o->nsource)
  {
    int64_t ns = nb <= 1 ? nb : (int64_t)((float)nb * (float)source_relax);
    o->nsource[s] = ns > n ? n : ns;
  }
}
} // namespace

extern "C" int oracle_subhalo_properties(const hbtg_params *p, const hbtg_batch *b, int snapshot_id,
                                         double source_relax, hbtg_props *o)
{
  if (!p || !b || !o || b->n_sub < 0)
    return HBTG_ERR_INVALID;
  const Cfg c = make_cfg(p, b);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < b->n_sub; s++)
    properties_one(b, s, snapshot_id, source_relax, c, o);
  return HBTG_OK;
}

/* ------------------------------------------------------------------------
 * ReassignParticles (src/subhalo_reassign_gas.cpp:65-197).  The neighbour
 * list of GeoTree_t::NearestNeighbours (src/geometric_tree.cpp:108-142)
 * follows from the distances alone: searches j = 0, 1, ... with radius R_j
 * (R_0 = SofteningHalo / 10 in float, each 1.26 times the last, rounded to
 * float) collect every tracer with |dx|, |dy|, |dz| <= R_j and
 * r^2 < R_j * R_j (float product) into one collector, until it holds
 * min(tracers, k); the collector keeps the k smallest r^2 of everything it
 * was given, so a tracer found by m searches counts m times.  The list is
 * the distinct tracers of those k, its last entry the nearest.
 * ------------------------------------------------------------------------ */
namespace
{
struct Cand
{
  double d2;
  int64_t i;
  int jmin;
};
} // namespace

extern "C" int oracle_reassign(const hbtg_params *p, hbtg_reassign *r, int k)
{
  if (!p || !r || r->n_groups < 0 || k <= 0)
    return HBTG_ERR_INVALID;
  const float boxf = (float)p->box_size, halff = (float)((double)boxf / 2.);
  const bool periodic = p->periodic != 0;
  const float r0 = (float)((double)(float)p->softening * 0.1);
  auto is_tracer = [&](int64_t g) { return ((1 << (int)r->type[g]) & p->tracer_type_mask) != 0; };
  auto nearest = [&](double x) {
    return x > (double)halff ? x - (double)boxf : (x < -(double)halff ? x + (double)boxf : x);
  };
  for (int64_t g = 0; g < r->offsets[r->n_sub]; g++)
    r->dest[g] = -1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t h = 0; h < r->n_groups; h++)
  {
    std::vector<int64_t> tr, tr_sub;
    int64_t non_tracers = 0;
    for (int64_t s = r->group_off[h]; s < r->group_off[h + 1]; s++)
      for (int64_t g = r->offsets[s]; g < r->offsets[s + 1]; g++)
        if (is_tracer(g))
        {
          tr.push_back(g);
          tr_sub.push_back(s);
        }
        else
          non_tracers++;
    if (non_tracers == 0 || tr.empty())
      continue;
    const int64_t nt = (int64_t)tr.size();
    const int64_t to_find = nt < k ? nt : k;
    std::vector<Cand> c(nt);
    for (int64_t s = r->group_off[h]; s < r->group_off[h + 1]; s++)
      for (int64_t g = r->offsets[s]; g < r->offsets[s + 1]; g++)
      {
        if (is_tracer(g))
          continue;
        for (int64_t i = 0; i < nt; i++)
        {
          double d[3];
          double dmax = 0.;
          for (int q = 0; q < 3; q++)
          {
            d[q] = (double)r->pos[3 * tr[i] + q] - (double)r->pos[3 * g + q];
            if (periodic)
              d[q] = nearest(d[q]);
            dmax = std::max(dmax, std::fabs(d[q]));
          }
          const double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          int j = 0;
          for (float R = r0;; R = (float)((double)R * 1.26), j++)
            if (dmax <= (double)R && d2 < (double)(R * R))
              break;
          c[i] = Cand{d2, i, j};
        }
        std::stable_sort(c.begin(), c.end(), [](const Cand &a, const Cand &b) { return a.d2 < b.d2; });
        /* the last search J: the first with sum over j <= J of N_j >= to_find,
           N_j = tracers that search j collects (jmin <= j) */
        int J = 0;
        for (int64_t cum = 0;; J++)
        {
          for (const Cand &q : c)
            if (q.jmin <= J)
              cum++;
          if (std::min<int64_t>(cum, k) >= to_find)
            break;
        }
        /* the k smallest r^2 of the collected multiset (a tracer counts J - jmin + 1 times) */
        int64_t taken = 0;
        bool found = false;
        int64_t first = -1;
        for (const Cand &q : c)
        {
          if (q.jmin > J)
            continue;
          if (taken >= k)
            break;
          if (first < 0)
            first = q.i;
          if (tr_sub[q.i] == s)
            found = true;
          taken += J - q.jmin + 1;
        }
        if (!found && first >= 0)
        {
          const int64_t to = tr_sub[first];
          if (to >= 0 && to != s)
            r->dest[g] = to;
        }
      }
  }
  return HBTG_OK;
}
