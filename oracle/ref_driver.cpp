/*
 * ref_driver.cpp — TEST INFRASTRUCTURE (oracle).  Runs the reference's own,
 * unmodified Subhalo_t::Unbind (src/subhalo_unbind.cpp:463-808) over a batch
 * described by the library's C ABI (include/hbt_unbind_gpu.h), so that the
 * reference itself can produce golden outputs and the CPU baseline.
 *
 * Built by oracle/build_oracle.py from the reference sources where they lie
 * (no source is copied) into oracle/_ref/libref_{dmo,hydro}.so, against the
 * single-rank stub headers in oracle/stub/.  Never linked into the product.
 *
 * The fake epoch follows the reference's own mocking idiom: a Snapshot_t
 * subclass that only carries Cosmology (unit_tests/test_neighbour_search.cpp:13-60).
 * Batching follows SubhaloSnapshot_t::RefineParticles (src/subhalo_unbind.cpp:888-903):
 * an OpenMP dynamic,1 loop over subhaloes with nested parallelism off
 * (HBT.cpp:26), so the per-particle loops inside Unbind run serially.
 * inner_parallel=1 instead calls Unbind serially over subhaloes with its inner
 * OpenMP loops enabled (the single-subhalo case).
 */
#include <cstdlib>
#include <omp.h>
#include <vector>

#include "config_parser.h"
#include "geometric_tree.h"
#include "snapshot.h"
#include "subhalo.h"

#include "hbt_unbind_gpu.h"

namespace
{
class EpochSnapshot_t : public Snapshot_t
{
  HBTxyz dummy{{0.f, 0.f, 0.f}};

public:
  EpochSnapshot_t(double a, double hz, int snapshot_id = 1)
  {
    Cosmology.ScaleFactor = a;
    Cosmology.Hz = hz;
    Cosmology.OmegaM0 = 0.3;
    Cosmology.OmegaLambda0 = 0.7;
    SnapshotIndex = snapshot_id;
    SnapshotId = snapshot_id;
  }
  HBTInt size() const override { return 0; }
  const HBTxyz &GetComovingPosition(const HBTInt) const override { return dummy; }
  const HBTxyz GetPhysicalVelocity(const HBTInt) const override { return dummy; }
  HBTReal GetMass(const HBTInt) const override { return 0; }
};

void set_config(const hbtg_params *p, const hbtg_batch *b)
{
  HBTConfig.BoxSize = p->box_size;
  HBTConfig.BoxHalf = HBTConfig.BoxSize / 2.;
  HBTConfig.PeriodicBoundaryOn = p->periodic != 0;
  HBTConfig.SofteningHalo = p->softening;
  HBTConfig.MaxPhysicalSofteningHalo = -1;
  HBTConfig.TreeNodeResolution = p->tree_node_resolution;
  HBTConfig.TreeNodeResolutionHalf = HBTConfig.TreeNodeResolution / 2.;
  HBTConfig.TreeNodeOpenAngle = p->open_angle;
  HBTConfig.TreeNodeOpenAngleSquare = HBTConfig.TreeNodeOpenAngle * HBTConfig.TreeNodeOpenAngle;
  HBTConfig.BoundMassPrecision = p->bound_mass_precision;
  HBTConfig.MinNumPartOfSub = (int)p->min_num_part;
  HBTConfig.MinNumTracerPartOfSub = (int)p->min_num_tracer;
  HBTConfig.TracerParticleBitMask = p->tracer_type_mask;
  HBTConfig.DoNotSubsampleParticleBitMask = p->no_subsample_mask;
  HBTConfig.MaxSampleSizeOfPotentialEstimate = p->max_sample_size;
  HBTConfig.RefineMostBoundParticle = p->refine_most_bound != 0;
  HBTConfig.BoundFractionCenterRefinement = p->refine_fraction;
  HBTConfig.PotentialEstimateUpscaleMassesPerType = p->upscale_per_type != 0;
  HBTConfig.SubCoreSizeMin = p->sub_core_size_min;
  HBTConfig.SubCoreSizeFactor = p->sub_core_size_factor;
  HBTConfig.SaveBoundParticleBindingEnergies = b->energy != nullptr;
  HBTConfig.SaveBoundParticlePotentialEnergies = b->potential != nullptr;
  PhysicalConst::G = p->G;
}

void load_subhalo(const hbtg_params *p, const hbtg_batch *b, int64_t s, Subhalo_t &sub)
{
  const int64_t off = b->offsets[s], n = b->offsets[s + 1] - off;
  sub.Particles.resize(n);
  for (int64_t k = 0; k < n; k++)
  {
    Particle_t &q = sub.Particles[k];
    const int64_t g = off + k;
    q.Id = b->id[g];
    for (int d = 0; d < 3; d++)
    {
      q.ComovingPosition[d] = b->pos[3 * g + d];
      q.PhysicalVelocity[d] = b->vel[3 * g + d];
    }
    q.Mass = b->mass[g];
#ifndef DM_ONLY
#ifdef HAS_THERMAL_ENERGY
    q.InternalEnergy = b->u ? b->u[g] : 0.f;
#endif
    q.Type = static_cast<ParticleType_t>(b->type ? b->type[g] : 1);
#endif
    q.HostId = k; /* carries the input index through the permutation */
  }
  sub.Nbound = n;
  for (int d = 0; d < 3; d++)
  {
    sub.ComovingAveragePosition[d] = b->ref_pos[3 * s + d];
    sub.PhysicalAverageVelocity[d] = b->ref_vel[3 * s + d];
    sub.ComovingMostBoundPosition[d] = b->mostbound_pos[3 * s + d];
    sub.PhysicalMostBoundVelocity[d] = b->mostbound_vel[3 * s + d];
  }
  sub.MostBoundParticleId = b->most_bound_id[s];
  /* members the empty-subhalo early return leaves untouched start at zero */
  sub.SpecificSelfPotentialEnergy = sub.SpecificSelfKineticEnergy = 0.f;
  for (int d = 0; d < 3; d++)
    sub.SpecificAngularMomentum[d] = 0.f;
  sub.SnapshotOfBirth = 0;
  sub.TrackId = s;
}

void store_subhalo(const hbtg_batch *b, int64_t s, Subhalo_t &sub)
{
  const int64_t off = b->offsets[s], n = b->offsets[s + 1] - off;
  for (int64_t k = 0; k < n; k++)
    b->order[off + k] = sub.Particles[k].HostId;
  b->nbound[s] = sub.Nbound;
  b->mbound[s] = sub.Mbound;
#ifndef DM_ONLY
  for (int t = 0; t < HBTG_TYPE_MAX; t++)
  {
    if (b->nbound_type)
      b->nbound_type[HBTG_TYPE_MAX * s + t] = sub.NboundType[t];
    if (b->mbound_type)
      b->mbound_type[HBTG_TYPE_MAX * s + t] = sub.MboundType[t];
  }
#else
  for (int t = 0; t < HBTG_TYPE_MAX; t++)
  {
    if (b->nbound_type)
      b->nbound_type[HBTG_TYPE_MAX * s + t] = (t == 1) ? sub.Nbound : 0;
    if (b->mbound_type)
      b->mbound_type[HBTG_TYPE_MAX * s + t] = 0.f;
  }
#endif
  b->tracer_index[s] = sub.TracerIndex;
  b->most_bound_id[s] = sub.MostBoundParticleId;
  for (int d = 0; d < 3; d++)
  {
    b->ref_pos[3 * s + d] = sub.ComovingAveragePosition[d];
    b->ref_vel[3 * s + d] = sub.PhysicalAverageVelocity[d];
    b->mostbound_pos[3 * s + d] = sub.ComovingMostBoundPosition[d];
    b->mostbound_vel[3 * s + d] = sub.PhysicalMostBoundVelocity[d];
  }
  if (b->kinematics)
  {
    float *k = b->kinematics + HBTG_KIN_STRIDE * s;
    k[0] = sub.SpecificSelfPotentialEnergy;
    k[1] = sub.SpecificSelfKineticEnergy;
    k[2] = sub.SpecificAngularMomentum[0];
    k[3] = sub.SpecificAngularMomentum[1];
    k[4] = sub.SpecificAngularMomentum[2];
  }
  if (b->core)
  {
    float *c = b->core + HBTG_CORE_STRIDE * s;
    for (int d = 0; d < 3; d++)
    {
      c[d] = sub.CoreComovingPosition[d];
      c[3 + d] = sub.CorePhysicalVelocity[d];
    }
    c[6] = sub.CoreComovingSigmaR;
    c[7] = sub.CorePhysicalSigmaV;
  }
  if (b->energy)
    for (int64_t k = 0; k < (int64_t)sub.ParticleBindingEnergies.size(); k++)
      b->energy[off + k] = sub.ParticleBindingEnergies[k];
  if (b->potential)
    for (int64_t k = 0; k < (int64_t)sub.ParticlePotentialEnergies.size(); k++)
      b->potential[off + k] = sub.ParticlePotentialEnergies[k];
#ifdef MEASURE_UNBINDING_TIME
  b->iterations[s] = sub.NumberUnbindingIterations;
#else
  b->iterations[s] = -1;
#endif
  if (n == 0)
    b->status[s] = HBTG_SUB_EMPTY;
  else if (sub.SnapshotOfDeath == 1)
    b->status[s] = HBTG_SUB_DISRUPTED;
  else
    b->status[s] = HBTG_SUB_CONVERGED;
}

void unbind_one(const hbtg_params *p, hbtg_batch *b, const EpochSnapshot_t &epoch, int64_t s)
{
  Subhalo_t sub;
  load_subhalo(p, b, s, sub);
  sub.Unbind(epoch);
  store_subhalo(b, s, sub);
}
} // namespace

extern "C" int ref_unbind_batch(const hbtg_params *p, hbtg_batch *b, int nthreads, int inner_parallel)
{
  if (!p || !b || b->n_sub < 0)
    return HBTG_ERR_INVALID;
  set_config(p, b);
  EpochSnapshot_t epoch(p->scale_factor, p->hubble);
  srand48(p->seed);
  srand((unsigned)p->seed);
  if (nthreads <= 0)
    nthreads = omp_get_max_threads();
  if (inner_parallel)
  {
    omp_set_max_active_levels(1);
    omp_set_num_threads(nthreads);
    for (int64_t s = 0; s < b->n_sub; s++)
      unbind_one(p, b, epoch, s);
  }
  else
  {
    omp_set_max_active_levels(1);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t s = 0; s < b->n_sub; s++)
    {
      omp_set_num_threads(1); /* the inner loops stay serial even when the team has one thread */
      unbind_one(p, b, epoch, s);
    }
  }
  return HBTG_OK;
}

/* The reference's own CalculateProfileProperties, CalculateShape and
 * TruncateSource on the bound sets of an unbinding call's outputs (see
 * hbtg_subhalo_properties in include/hbt_unbind_gpu.h). */
extern "C" int ref_subhalo_properties(const hbtg_params *p, const hbtg_batch *b, int snapshot_id, double source_relax,
                                      hbtg_props *o)
{
  if (!p || !b || !o || b->n_sub < 0)
    return HBTG_ERR_INVALID;
  set_config(p, b);
  HBTConfig.SourceSubRelaxFactor = source_relax;
  EpochSnapshot_t epoch(p->scale_factor, p->hubble, snapshot_id);
  omp_set_num_threads(1); /* the inner OpenMP reductions in a fixed order */
  for (int64_t s = 0; s < b->n_sub; s++)
  {
    const int64_t off = b->offsets[s], n = b->offsets[s + 1] - off;
    Subhalo_t sub;
    sub.Particles.resize(n);
    for (int64_t k = 0; k < n; k++)
    {
      const int64_t g = off + b->order[off + k];
      Particle_t &q = sub.Particles[k];
      q.Id = b->id ? b->id[g] : g;
      for (int d = 0; d < 3; d++)
      {
        q.ComovingPosition[d] = b->pos[3 * g + d];
        q.PhysicalVelocity[d] = b->vel ? b->vel[3 * g + d] : 0.f;
      }
      q.Mass = b->mass[g];
    }
    sub.Nbound = b->nbound[s];
    sub.Mbound = b->mbound[s];
    for (int d = 0; d < 3; d++)
      sub.ComovingMostBoundPosition[d] = b->mostbound_pos[3 * s + d];
    sub.BoundR200CritComoving = o->r200[s];
    sub.BoundM200Crit = o->m200[s];
    sub.LastMaxVmaxPhysical = o->last_vmax[s];
    sub.RmaxComovingOfLastMaxVmax = o->rmax_last[s];
    sub.SnapshotOfLastMaxVmax = o->snap_last[s];
    sub.CalculateProfileProperties(epoch);
    sub.CalculateShape();
    o->rmax[s] = sub.RmaxComoving;
    o->vmax[s] = sub.VmaxPhysical;
    o->rhalf[s] = sub.RHalfComoving;
    o->renclose[s] = sub.REncloseComoving;
    o->r200[s] = sub.BoundR200CritComoving;
    o->m200[s] = sub.BoundM200Crit;
    o->last_vmax[s] = sub.LastMaxVmaxPhysical;
    o->rmax_last[s] = sub.RmaxComovingOfLastMaxVmax;
    o->snap_last[s] = sub.SnapshotOfLastMaxVmax;
    for (int q = 0; q < 6; q++)
    {
      o->inertia[6 * s + q] = sub.InertialTensor[q];
      o->inertia_w[6 * s + q] = sub.InertialTensorWeighted[q];
    }
    if (o->nsource)
    {
      sub.TruncateSource();
      o->nsource[s] = (int64_t)sub.Particles.size();
    }
  }
  return HBTG_OK;
}

/* The reference's own Subhalo_t::RecursiveUnbind (src/subhalo_unbind.cpp:810-841,
 * with MergeRecursively and the second Unbind of MergeTrappedSubhalos,
 * src/subhalo_merge.cpp:46-92) from every root of a nesting forest.  Subhalo s
 * starts from its own particles (batch segment s) and frame; parent[s] is the
 * subhalo it is nested in (-1: a root), NestedSubhalos listing children in
 * ascending index; TrackId = s.  Outputs per subhalo: nbound, mbound, the IDs
 * of its final Particles (CSR: out_count[s], into out_ids from out_off[s],
 * capacity out_cap), SinkTrackId, SnapshotOfSink, SnapshotOfDeath and
 * MostBoundParticleId.  Returns HBTG_ERR_NOMEM when out_cap is too small. */
extern "C" int ref_recursive_unbind(const hbtg_params *p, hbtg_batch *b, const int64_t *parent, int merge_trapped,
                                    int snapshot_id, int64_t out_cap, int64_t *out_off, int64_t *out_count,
                                    int64_t *out_ids, int64_t *sink_track, int32_t *snap_sink,
                                    int32_t *snap_death)
{
  if (!p || !b || !parent || b->n_sub < 0)
    return HBTG_ERR_INVALID;
  set_config(p, b);
  HBTConfig.MergeTrappedSubhalos = merge_trapped != 0;
  EpochSnapshot_t epoch(p->scale_factor, p->hubble, snapshot_id);
  srand48(p->seed);
  srand((unsigned)p->seed);
  omp_set_num_threads(1);
  const int64_t S = b->n_sub;
  SubhaloList_t subs(S);
  for (int64_t s = 0; s < S; s++)
  {
    load_subhalo(p, b, s, subs[s]);
    subs[s].TrackId = s;
  }
  for (int64_t s = 0; s < S; s++)
    if (parent[s] >= 0)
      subs[parent[s]].NestedSubhalos.push_back(s);
  for (int64_t s = 0; s < S; s++)
    if (parent[s] < 0)
      subs[s].RecursiveUnbind(subs, epoch);
  int64_t at = 0;
  for (int64_t s = 0; s < S; s++)
  {
    const int64_t n = (int64_t)subs[s].Particles.size();
    if (at + n > out_cap)
      return HBTG_ERR_NOMEM;
    out_off[s] = at;
    out_count[s] = n;
    for (int64_t k = 0; k < n; k++)
      out_ids[at + k] = subs[s].Particles[k].Id;
    at += n;
    b->nbound[s] = subs[s].Nbound;
    b->mbound[s] = subs[s].Mbound;
    b->most_bound_id[s] = subs[s].MostBoundParticleId;
    sink_track[s] = subs[s].SinkTrackId;
    snap_sink[s] = subs[s].SnapshotOfSink;
    snap_death[s] = subs[s].SnapshotOfDeath;
  }
  return HBTG_OK;
}

namespace
{
/* Positions only: what GeoTree_t needs of a snapshot. */
class PositionSnapshot_t : public Snapshot_t
{
  HBTxyz zero{{0.f, 0.f, 0.f}};

public:
  std::vector<HBTxyz> x;
  HBTInt size() const override { return (HBTInt)x.size(); }
  const HBTxyz &GetComovingPosition(const HBTInt i) const override { return x[i]; }
  const HBTxyz GetPhysicalVelocity(const HBTInt) const override { return zero; }
  HBTReal GetMass(const HBTInt) const override { return 1.f; }
};
} // namespace

/* The moves of ReassignParticles (src/subhalo_reassign_gas.cpp:65-197) for a
 * batch of FoF groups, with the reference's own GeoTree_t::NearestNeighbours
 * (src/geometric_tree.cpp:108-142) over the tracers of each group. */
extern "C" int ref_reassign(const hbtg_params *p, hbtg_reassign *r, int num_neighbours)
{
  if (!p || !r || r->n_groups < 0)
    return HBTG_ERR_INVALID;
  HBTConfig.BoxSize = p->box_size;
  HBTConfig.BoxHalf = HBTConfig.BoxSize / 2.;
  HBTConfig.PeriodicBoundaryOn = p->periodic != 0;
  HBTConfig.SofteningHalo = p->softening;
  HBTConfig.TreeNodeResolution = p->tree_node_resolution;
  HBTConfig.TreeNodeResolutionHalf = HBTConfig.TreeNodeResolution / 2.;
  HBTConfig.TracerParticleBitMask = p->tracer_type_mask;
  srand48(p->seed);
  auto is_tracer = [&](int64_t g) { return ((1 << (int)r->type[g]) & p->tracer_type_mask) != 0; };
  for (int64_t g = 0; g < r->offsets[r->n_sub]; g++)
    r->dest[g] = -1;
  for (int64_t h = 0; h < r->n_groups; h++)
  {
    PositionSnapshot_t tracers;
    std::vector<int64_t> tracer_sub;
    int64_t non_tracers = 0;
    for (int64_t s = r->group_off[h]; s < r->group_off[h + 1]; s++)
      for (int64_t g = r->offsets[s]; g < r->offsets[s + 1]; g++)
        if (is_tracer(g))
        {
          tracers.x.push_back(HBTxyz{{r->pos[3 * g], r->pos[3 * g + 1], r->pos[3 * g + 2]}});
          tracer_sub.push_back(s);
        }
        else
          non_tracers++;
    if (non_tracers == 0 || tracers.x.empty())
      continue;
    GeoTree_t tree;
    tree.Build(tracers);
    for (int64_t s = r->group_off[h]; s < r->group_off[h + 1]; s++)
      for (int64_t g = r->offsets[s]; g < r->offsets[s + 1]; g++)
      {
        if (is_tracer(g))
          continue;
        const HBTxyz centre{{r->pos[3 * g], r->pos[3 * g + 1], r->pos[3 * g + 2]}};
        const std::vector<HBTInt> ngb = tree.NearestNeighbours(centre, num_neighbours, HBTConfig.SofteningHalo * 0.1);
        bool found = false;
        for (auto i : ngb)
          if (tracer_sub[i] == s)
          {
            found = true;
            break;
          }
        if (!found && !ngb.empty())
        {
          const int64_t to = tracer_sub[ngb.back()];
          if (to >= 0 && to != s)
            r->dest[g] = to;
        }
      }
  }
  return HBTG_OK;
}

extern "C" const char *ref_variant()
{
#ifdef DM_ONLY
  return "reference Subhalo_t::Unbind, DM_ONLY";
#elif defined(UNBIND_WITH_THERMAL_ENERGY)
  return "reference Subhalo_t::Unbind, hydro, UNBIND_WITH_THERMAL_ENERGY";
#else
  return "reference Subhalo_t::Unbind, hydro";
#endif
}
