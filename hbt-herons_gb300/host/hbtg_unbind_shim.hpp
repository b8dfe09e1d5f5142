// hbtg_unbind_shim.hpp - C++ host adapter between HBT-HERONS' Subhalo_t and
// the GPU unbinding library's C ABI (include/hbt_unbind_gpu.h).
//
// Header-only and templated on the caller's types, so a maintainer can use it
// from inside HBT-HERONS without this project depending on the reference's
// headers.  It mirrors
//   void Subhalo_t::Unbind(const Snapshot_t &epoch)        src/subhalo_unbind.cpp:463-808
//   the field / new-subhalo loops of RefineParticles       src/subhalo_unbind.cpp:888-903
// by marshalling Subhalo_t particle lists into one CSR batch, calling
// hbtg_unbind_batch once, and applying the results: permuting Particles by
// the returned order, and setting Nbound, Mbound, MboundType/NboundType,
// the frames, the most-bound particle, kinematics, core phase-space
// properties, binding energies and the death/sink bookkeeping exactly where
// Unbind sets them (src/subhalo_unbind.cpp:647-707, 754-802).
//
// recursive_unbind() is SubhaloSnapshot_t::RefineParticles' nested part,
//   Subhalo_t::RecursiveUnbind                             src/subhalo_unbind.cpp:810-841
//   Subhalo_t::MergeRecursively / MergeTo / phase space    src/subhalo_merge.cpp:14-92, 183-230
// run level-synchronously: the subhaloes of one nesting depth are one batch,
// deepest first; after a level's call each subhalo checks the subhaloes of
// its own subtree for phase-space overlap (and absorbs their bound sets when
// MergeTrappedSubhalos is on, then is unbound again), and every child's
// unbound tail is appended to its parent, children in NestedSubhalos order.
// Subhaloes at one depth never feed one another, so this is the reference's
// depth-first recursion batched.
//
// Requirements on the types (those of src/subhalo.h and src/snapshot.h):
//   Subhalo: Particles (vector of Particle), Nbound, Mbound, MboundType[6],
//            NboundType[6], TracerIndex, ComovingAveragePosition,
//            PhysicalAverageVelocity, ComovingMostBoundPosition,
//            PhysicalMostBoundVelocity, MostBoundParticleId,
//            SpecificSelfPotentialEnergy, SpecificSelfKineticEnergy,
//            SpecificAngularMomentum[3], CoreComovingPosition,
//            CorePhysicalVelocity, CoreComovingSigmaR, CorePhysicalSigmaV,
//            SnapshotOfDeath, SnapshotOfSink, DescendantTrackId, SinkTrackId,
//            ParticleBindingEnergies, ParticlePotentialEnergies
//   Particle: Id, ComovingPosition[3], PhysicalVelocity[3], Mass, Type
//            (InternalEnergy when thermal energy is used)
// and, for recursive_unbind: Subhalo::NestedSubhalos (indices into the
// subhalo list), TrackId.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "hbt_unbind_gpu.h"

namespace hbtg_shim
{

struct Options
{
  bool has_types = true;       // !DM_ONLY
  bool has_thermal = false;    // UNBIND_WITH_THERMAL_ENERGY
  bool save_binding = false;   // SaveBoundParticleBindingEnergies
  bool save_potential = false; // SaveBoundParticlePotentialEnergies
  int snapshot_id = 0;         // epoch.GetSnapshotId()
  int64_t null_snapshot = -1;  // SpecialConst::NullSnapshotId
  int64_t null_track = -1;     // SpecialConst::NullTrackId
  bool merge_trapped = false;  // MergeTrappedSubhalos (recursive_unbind)
};

class Unbinder
{
  hbtg_handle *h_ = nullptr;

public:
  explicit Unbinder(int device = 0)
  {
    const int rc = hbtg_create(&h_, device);
    if (rc != HBTG_OK)
      throw std::runtime_error(std::string("hbtg_create: ") + hbtg_status_string(rc));
  }
  ~Unbinder()
  {
    if (h_)
      hbtg_destroy(h_);
  }
  Unbinder(const Unbinder &) = delete;
  Unbinder &operator=(const Unbinder &) = delete;

  // Loads the learned warm start's proposer (weights of hbtg_mlp_forward's
  // layout); first_test as in hbtg_model.
  void set_model(const std::vector<float> &weights, float threshold, float exclude_below, int64_t min_particles,
                 int first_test = 1)
  {
    if (weights.size() != HBTG_MLP_PARAMS)
      throw std::runtime_error("hbtg_set_model: wrong number of weights");
    hbtg_model m{weights.data(), threshold, min_particles, exclude_below, (int32_t)first_test};
    const int rc = hbtg_set_model(h_, &m);
    if (rc != HBTG_OK)
      throw std::runtime_error(std::string("hbtg_set_model: ") + hbtg_status_string(rc));
  }

  // Unbinds every subhalo pointed to by `subs` in one GPU call.
  template <class Subhalo>
  void unbind(const hbtg_params &params_in, const std::vector<Subhalo *> &subs, const Options &opt)
  {
    run(params_in, subs, opt, false);
  }

  // The same with the learned warm start (set_model first).  The previous
  // output's knowledge comes from the Subhalo_t members as Unbind finds them:
  // Nbound (its bound particles lead Particles) and ParticleBindingEnergies
  // when the previous output saved them.  No potential subsampling.
  template <class Subhalo>
  void unbind_learned(const hbtg_params &params_in, const std::vector<Subhalo *> &subs, const Options &opt)
  {
    run(params_in, subs, opt, true);
  }

  // Subhalo_t::RecursiveUnbind from every root (src/subhalo_unbind.cpp:810-841)
  // over a subhalo list whose NestedSubhalos hold indices into it.  The
  // caller adds a FoF group's other heads to its central's NestedSubhalos
  // first, as RefineParticles does (src/subhalo_unbind.cpp:874-880).
  template <class SubhaloList>
  void recursive_unbind(const hbtg_params &params, SubhaloList &subs, const std::vector<int64_t> &roots,
                        const Options &opt)
  {
    using Subhalo = typename SubhaloList::value_type;
    const int64_t n = (int64_t)subs.size();
    std::vector<int> depth(n, -1);
    std::vector<int64_t> parent(n, -1);
    std::vector<std::vector<int64_t>> levels;
    std::vector<int64_t> stack;
    for (int64_t r : roots)
    {
      if (r < 0 || r >= n || depth[r] >= 0)
        throw std::runtime_error("recursive_unbind: bad or repeated root");
      depth[r] = 0;
      stack.push_back(r);
      while (!stack.empty())
      {
        const int64_t s = stack.back();
        stack.pop_back();
        if ((int64_t)levels.size() <= depth[s])
          levels.resize(depth[s] + 1);
        levels[depth[s]].push_back(s);
        for (auto c : subs[s].NestedSubhalos)
        {
          if (c < 0 || c >= n || depth[c] >= 0)
            throw std::runtime_error("recursive_unbind: a subhalo nested twice or in a cycle");
          depth[c] = depth[s] + 1;
          parent[c] = s;
          stack.push_back((int64_t)c);
        }
      }
    }
    for (int d = (int)levels.size() - 1; d >= 0; d--)
    {
      std::vector<int64_t> level = levels[d];
      std::sort(level.begin(), level.end());
      std::vector<Subhalo *> batch;
      for (int64_t s : level)
        batch.push_back(&subs[s]);
      run(params, batch, opt, false);
      // MergeRecursively after each Unbind; a host that absorbed a resolved
      // subhalo is unbound again when MergeTrappedSubhalos is on (:826-835)
      std::vector<Subhalo *> again;
      for (int64_t s : level)
        if (merge_recursively(params, subs, s, subs[s], opt) && opt.merge_trapped)
          again.push_back(&subs[s]);
      if (!again.empty())
        run(params, again, opt, false);
      // each child's unbound tail to its parent, children in NestedSubhalos order (:819-823)
      if (d == 0)
        continue;
      std::vector<int64_t> parents;
      for (int64_t s : level)
        parents.push_back(parent[s]);
      std::sort(parents.begin(), parents.end());
      parents.erase(std::unique(parents.begin(), parents.end()), parents.end());
      for (int64_t p : parents)
        for (auto c : subs[p].NestedSubhalos)
        {
          const Subhalo &child = subs[c];
          subs[p].Particles.insert(subs[p].Particles.end(), child.Particles.begin() + child.Nbound,
                                   child.Particles.end());
        }
    }
  }

  // Subhalo_t::CalculateProfileProperties and Subhalo_t::CalculateShape
  // (src/subhalo.cpp:175-309) for every subhalo of `subs` in one GPU call,
  // from the bound set that Unbind left (the first Nbound Particles, most
  // bound first, ComovingMostBoundPosition the centre); with `truncate`,
  // Subhalo_t::TruncateSource (src/subhalo_unbind.cpp:843-853) as well.
  // source_relax is SourceSubRelaxFactor.
  template <class Subhalo>
  void properties(const hbtg_params &params, const std::vector<Subhalo *> &subs, const Options &opt,
                  double source_relax, bool truncate)
  {
    const int64_t ns = (int64_t)subs.size();
    std::vector<int64_t> offsets(ns + 1, 0);
    for (int64_t s = 0; s < ns; s++)
      offsets[s + 1] = offsets[s] + (int64_t)subs[s]->Particles.size();
    const int64_t n = offsets[ns];
    std::vector<float> pos(3 * n), mass(n), mbound(ns), mb_pos(3 * ns);
    std::vector<int64_t> order(n), nbound(ns), nsource(ns);
    std::vector<float> rmax(ns), vmax(ns), rhalf(ns), renclose(ns), r200(ns), m200(ns), last_vmax(ns),
      rmax_last(ns), inertia(6 * ns), inertia_w(6 * ns);
    std::vector<int32_t> snap_last(ns);
    for (int64_t s = 0; s < ns; s++)
    {
      const Subhalo &sub = *subs[s];
      for (int64_t k = 0; k < (int64_t)sub.Particles.size(); k++)
      {
        const auto &p = sub.Particles[k];
        const int64_t g = offsets[s] + k;
        for (int d = 0; d < 3; d++)
          pos[3 * g + d] = p.ComovingPosition[d];
        mass[g] = p.Mass;
        order[g] = k;
      }
      nbound[s] = (int64_t)sub.Nbound;
      mbound[s] = sub.Mbound;
      for (int d = 0; d < 3; d++)
        mb_pos[3 * s + d] = sub.ComovingMostBoundPosition[d];
      r200[s] = sub.BoundR200CritComoving;
      m200[s] = sub.BoundM200Crit;
      last_vmax[s] = sub.LastMaxVmaxPhysical;
      rmax_last[s] = sub.RmaxComovingOfLastMaxVmax;
      snap_last[s] = sub.SnapshotOfLastMaxVmax;
    }
    hbtg_batch b{};
    b.n_sub = ns;
    b.offsets = offsets.data();
    b.pos = pos.data();
    b.mass = mass.data();
    b.mostbound_pos = mb_pos.data();
    b.order = order.data();
    b.nbound = nbound.data();
    b.mbound = mbound.data();
    hbtg_props pr{rmax.data(),      vmax.data(),      rhalf.data(),   renclose.data(),
                  r200.data(),      m200.data(),      last_vmax.data(), rmax_last.data(),
                  snap_last.data(), inertia.data(),   inertia_w.data(), nsource.data()};
    const int rc = hbtg_subhalo_properties(h_, &params, &b, opt.snapshot_id, source_relax, &pr);
    if (rc != HBTG_OK)
      throw std::runtime_error(std::string("hbtg_subhalo_properties: ") + hbtg_status_string(rc));
    for (int64_t s = 0; s < ns; s++)
    {
      Subhalo &sub = *subs[s];
      sub.RmaxComoving = rmax[s];
      sub.VmaxPhysical = vmax[s];
      sub.RHalfComoving = rhalf[s];
      sub.REncloseComoving = renclose[s];
      sub.BoundR200CritComoving = r200[s];
      sub.BoundM200Crit = m200[s];
      sub.LastMaxVmaxPhysical = last_vmax[s];
      sub.RmaxComovingOfLastMaxVmax = rmax_last[s];
      sub.SnapshotOfLastMaxVmax = snap_last[s];
      for (int q = 0; q < 6; q++)
      {
        sub.InertialTensor[q] = inertia[6 * s + q];
        sub.InertialTensorWeighted[q] = inertia_w[6 * s + q];
      }
      if (truncate)
        sub.Particles.resize((size_t)nsource[s]);
    }
  }

  // SubhaloSnapshot_t::ReassignParticles (src/subhalo_reassign_gas.cpp:65-197)
  // over a list of FoF groups, each the subhaloes of one
  // MemberTable.SubGroups entry in its order.  One GPU call decides every
  // move; each moved particle is then appended to its destination's
  // Particles (subhaloes in group order, particles in their order) and
  // dropped from its own; each subhalo's Nbound is clamped to its particle
  // count, the dropped particles are removed keeping the bound/unbound split
  // (Subhalo_t::KickNullParticles, src/subhalo.cpp:394-430) and NboundType,
  // MboundType and TracerIndex are counted again (Subhalo_t::CountParticleTypes,
  // src/subhalo.cpp:311-392).  num_neighbours is NumNeighboursForReassignment.
  // Returns the number of particles moved.
  template <class Subhalo>
  int64_t reassign(const hbtg_params &params, const std::vector<std::vector<Subhalo *>> &groups,
                   int num_neighbours)
  {
    std::vector<Subhalo *> subs;
    std::vector<int64_t> group_off(1, 0);
    for (const auto &g : groups)
    {
      subs.insert(subs.end(), g.begin(), g.end());
      group_off.push_back((int64_t)subs.size());
    }
    const int64_t ns = (int64_t)subs.size();
    std::vector<int64_t> offsets(ns + 1, 0);
    for (int64_t s = 0; s < ns; s++)
      offsets[s + 1] = offsets[s] + (int64_t)subs[s]->Particles.size();
    const int64_t n = offsets[ns];
    std::vector<float> pos(3 * n);
    std::vector<uint8_t> type(n, 0);
    std::vector<int64_t> dest(n, -1);
    Options with_types;
    for (int64_t s = 0; s < ns; s++)
      for (int64_t k = 0; k < (int64_t)subs[s]->Particles.size(); k++)
      {
        const auto &p = subs[s]->Particles[k];
        const int64_t g = offsets[s] + k;
        for (int d = 0; d < 3; d++)
          pos[3 * g + d] = p.ComovingPosition[d];
        set_type(type, g, p, with_types);
      }
    hbtg_reassign r{(int64_t)groups.size(), group_off.data(), ns, offsets.data(), pos.data(), type.data(),
                    dest.data()};
    const int rc = hbtg_reassign_particles(h_, &params, &r, num_neighbours);
    if (rc != HBTG_OK)
      throw std::runtime_error(std::string("hbtg_reassign_particles: ") + hbtg_status_string(rc));
    int64_t moved = 0;
    for (int64_t s = 0; s < ns; s++)
      for (int64_t k = 0; k < offsets[s + 1] - offsets[s]; k++)
        if (dest[offsets[s] + k] >= 0)
        {
          subs[dest[offsets[s] + k]]->Particles.push_back(subs[s]->Particles[k]);
          moved++;
        }
    // the tidy-up runs over every group that has a non-tracer particle
    std::vector<char> tidy(ns, 0);
    for (size_t h = 0; h + 1 < group_off.size(); h++)
    {
      bool any = false;
      for (int64_t g = offsets[group_off[h]]; g < offsets[group_off[h + 1]] && !any; g++)
        any = ((1 << (int)type[g]) & params.tracer_type_mask) == 0;
      for (int64_t s = group_off[h]; s < group_off[h + 1]; s++)
        tidy[s] = any;
    }
    for (int64_t s = 0; s < ns; s++)
    {
      if (!tidy[s])
        continue;
      Subhalo &sub = *subs[s];
      const int64_t len = offsets[s + 1] - offsets[s], np = (int64_t)sub.Particles.size();
      if ((int64_t)sub.Nbound > np)
        sub.Nbound = np;
      int64_t keep = 0, nb = 0;
      for (int64_t k = 0; k < np; k++)
      {
        if (k < len && dest[offsets[s] + k] >= 0)
          continue;
        if (k < (int64_t)sub.Nbound)
          nb++;
        if (keep != k)
          sub.Particles[keep] = std::move(sub.Particles[k]);
        keep++;
      }
      sub.Particles.resize((size_t)keep);
      sub.Nbound = nb;
      count_particle_types(sub, params, 0);
    }
    return moved;
  }

private:
  // Subhalo_t::CountParticleTypes (src/subhalo.cpp:311-392): per-type counts
  // and masses of the bound set (float sums in bound order) and the first
  // tracer's index (0 when there is none).
  template <class Subhalo>
  static auto count_particle_types(Subhalo &sub, const hbtg_params &params, int)
    -> decltype((void)sub.NboundType[0], (void)sub.Particles[0].Type)
  {
    for (int t = 0; t < HBTG_TYPE_MAX; t++)
    {
      sub.NboundType[t] = 0;
      sub.MboundType[t] = 0;
    }
    int64_t tracer = -1;
    for (int64_t k = 0; k < (int64_t)sub.Nbound; k++)
    {
      const auto &p = sub.Particles[k];
      sub.NboundType[p.Type]++;
      sub.MboundType[p.Type] += p.Mass;
      if (tracer < 0 && ((1 << (int)p.Type) & params.tracer_type_mask))
        tracer = k;
    }
    sub.TracerIndex = tracer < 0 ? 0 : tracer;
  }
  template <class Subhalo>
  static void count_particle_types(Subhalo &sub, const hbtg_params &, ...)
  {
    sub.TracerIndex = 0;
  }

  // Subhalo_t::MergeRecursively (src/subhalo_merge.cpp:46-92): the subtree of
  // subs[self], depth first, against `ref`.
  template <class SubhaloList, class Subhalo>
  bool merge_recursively(const hbtg_params &params, SubhaloList &subs, int64_t self, Subhalo &ref,
                         const Options &opt)
  {
    bool merged = false;
    if (ref.Nbound <= 1)
      return merged;
    Subhalo &me = subs[self];
    for (size_t i = 0; i < me.NestedSubhalos.size(); i++)
      merged = merge_recursively(params, subs, (int64_t)me.NestedSubhalos[i], ref, opt) | merged;
    if (me.SinkTrackId == opt.null_track && &me != &ref && phase_space_distance(params, me, ref) < 2.f)
    {
      // SetMergerInformation (src/subhalo_merge.cpp:30-41)
      me.SnapshotOfSink = opt.snapshot_id;
      me.SinkTrackId = ref.TrackId;
      if (me.SnapshotOfDeath == opt.null_snapshot)
        me.SnapshotOfDeath = opt.snapshot_id;
      merged = (me.Nbound > 1) | merged;
      if (opt.merge_trapped)
        merge_to(me, ref);
    }
    return merged;
  }

  // Subhalo_t::PhaseSpaceDistance (src/subhalo_merge.cpp:14-20) in float:
  // PeriodicDistance and Distance (src/config_parser.h:220-231, src/mymath.h:232-238).
  template <class Subhalo>
  static float phase_space_distance(const hbtg_params &params, const Subhalo &me, const Subhalo &ref)
  {
    const float box = (float)params.box_size, half = (float)((double)box / 2.);
    float dx[3], dv[3];
    for (int d = 0; d < 3; d++)
    {
      dx[d] = ref.CoreComovingPosition[d] - me.CoreComovingPosition[d];
      if (params.periodic)
        dx[d] = dx[d] > half ? dx[d] - box : (dx[d] < -half ? dx[d] + box : dx[d]);
      dv[d] = ref.CorePhysicalVelocity[d] - me.CorePhysicalVelocity[d];
    }
    const float pos = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    const float vel = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    return pos / ref.CoreComovingSigmaR + vel / ref.CorePhysicalSigmaV;
  }

  // Subhalo_t::MergeTo (src/subhalo_merge.cpp:183-230): the bound set moves
  // to the host; the subhalo keeps its most-bound tracer as an orphan.
  template <class Subhalo>
  static void merge_to(Subhalo &me, Subhalo &host)
  {
    if (me.Nbound <= 1)
      return;
    host.Particles.insert(host.Particles.end(), me.Particles.begin(), me.Particles.begin() + me.Nbound);
    const auto &t = me.Particles[me.TracerIndex];
    me.MostBoundParticleId = t.Id;
    for (int d = 0; d < 3; d++)
    {
      me.ComovingMostBoundPosition[d] = t.ComovingPosition[d];
      me.PhysicalMostBoundVelocity[d] = t.PhysicalVelocity[d];
      me.ComovingAveragePosition[d] = me.ComovingMostBoundPosition[d];
      me.PhysicalAverageVelocity[d] = me.PhysicalMostBoundVelocity[d];
    }
    me.Nbound = 0;
    me.Particles.resize(0);
    me.Mbound = 0; // CountParticles over no particles
    zero_types(me, 0);
  }
  template <class Subhalo>
  static auto zero_types(Subhalo &sub, int) -> decltype((void)sub.NboundType[0])
  {
    for (int t = 0; t < HBTG_TYPE_MAX; t++)
    {
      sub.NboundType[t] = 0;
      sub.MboundType[t] = 0;
    }
  }
  template <class Subhalo>
  static void zero_types(Subhalo &, ...)
  {
  }

  template <class Subhalo>
  void run(const hbtg_params &params_in, const std::vector<Subhalo *> &subs, const Options &opt, bool learned)
  {
    hbtg_params params = params_in;
    if (params.max_sample_size > 0 && !params.prepared_subsample)
    { // PrepareParticlesForSubsampling, as Unbind does it (src/subhalo_unbind.cpp:430-443, 522-524):
      // exempt types first, the rest shuffled with the process's rand() sequence
      for (Subhalo *sub : subs)
        if ((int64_t)sub->Particles.size() > params.max_sample_size)
        {
          auto it = std::partition(sub->Particles.begin(), sub->Particles.end(),
                                   [&](const auto &p) { return exempt(p, params, opt); });
          std::random_shuffle(it, sub->Particles.end());
        }
      params.prepared_subsample = 1;
    }
    const int64_t ns = (int64_t)subs.size();
    std::vector<int64_t> offsets(ns + 1, 0);
    for (int64_t s = 0; s < ns; s++)
      offsets[s + 1] = offsets[s] + (int64_t)subs[s]->Particles.size();
    const int64_t n = offsets[ns];
    std::vector<float> pos(3 * n), vel(3 * n), mass(n), u(opt.has_thermal ? n : 0);
    std::vector<int64_t> id(n), order(n), nbound(ns), nbound_type(6 * ns), tracer(ns), mbid(ns);
    std::vector<uint8_t> type(opt.has_types ? n : 0);
    std::vector<float> ref_pos(3 * ns), ref_vel(3 * ns), mb_pos(3 * ns), mb_vel(3 * ns), mbound(ns),
      mbound_type(6 * ns), kin(5 * ns), core(8 * ns), energy(n), potential(opt.save_potential ? n : 0);
    std::vector<int32_t> iters(ns), status(ns);
    for (int64_t s = 0; s < ns; s++)
    {
      const Subhalo &sub = *subs[s];
      for (int64_t k = 0; k < (int64_t)sub.Particles.size(); k++)
      {
        const auto &p = sub.Particles[k];
        const int64_t g = offsets[s] + k;
        for (int d = 0; d < 3; d++)
        {
          pos[3 * g + d] = p.ComovingPosition[d];
          vel[3 * g + d] = p.PhysicalVelocity[d];
        }
        mass[g] = p.Mass;
        id[g] = p.Id;
        set_type(type, g, p, opt);
        set_thermal(u, g, p, opt);
      }
      for (int d = 0; d < 3; d++)
      {
        ref_pos[3 * s + d] = sub.ComovingAveragePosition[d];
        ref_vel[3 * s + d] = sub.PhysicalAverageVelocity[d];
        mb_pos[3 * s + d] = sub.ComovingMostBoundPosition[d];
        mb_vel[3 * s + d] = sub.PhysicalMostBoundVelocity[d];
      }
      mbid[s] = sub.MostBoundParticleId;
    }
    hbtg_batch b{};
    b.n_sub = ns;
    b.offsets = offsets.data();
    b.pos = pos.data();
    b.vel = vel.data();
    b.mass = mass.data();
    b.u = opt.has_thermal ? u.data() : nullptr;
    b.id = id.data();
    b.type = opt.has_types ? type.data() : nullptr;
    b.ref_pos = ref_pos.data();
    b.ref_vel = ref_vel.data();
    b.mostbound_pos = mb_pos.data();
    b.mostbound_vel = mb_vel.data();
    b.most_bound_id = mbid.data();
    b.order = order.data();
    b.nbound = nbound.data();
    b.mbound = mbound.data();
    b.nbound_type = nbound_type.data();
    b.mbound_type = mbound_type.data();
    b.tracer_index = tracer.data();
    b.kinematics = kin.data();
    b.core = core.data();
    b.energy = energy.data();
    b.potential = opt.save_potential ? potential.data() : nullptr;
    b.iterations = iters.data();
    b.status = status.data();
    int rc;
    if (learned)
    {
      std::vector<int64_t> nb_prev(ns);
      std::vector<float> e_prev(n, 0.f);
      bool have_e = false;
      for (int64_t s = 0; s < ns; s++)
      {
        const Subhalo &sub = *subs[s];
        nb_prev[s] = std::min<int64_t>((int64_t)sub.Nbound, (int64_t)sub.Particles.size());
        const auto &E = sub.ParticleBindingEnergies;
        for (int64_t k = 0; k < nb_prev[s] && k < (int64_t)E.size(); k++)
        {
          e_prev[offsets[s] + k] = E[k];
          have_e = true;
        }
      }
      hbtg_prior prior{nb_prev.data(), have_e ? e_prev.data() : nullptr};
      rc = hbtg_unbind_batch_learned(h_, &params, &b, &prior);
    }
    else
      rc = hbtg_unbind_batch(h_, &params, &b);
    if (rc != HBTG_OK && rc != HBTG_ERR_MAX_ITER)
      throw std::runtime_error(std::string("hbtg_unbind_batch: ") + hbtg_status_string(rc));
    for (int64_t s = 0; s < ns; s++)
      apply(*subs[s], s, offsets, b, opt);
  }

  template <class P>
  static auto exempt(const P &p, const hbtg_params &prm, const Options &opt) -> decltype((void)p.Type, bool())
  {
    return opt.has_types && !prm.dm_only && (((1 << (int)p.Type) & prm.no_subsample_mask) != 0);
  }
  template <class P>
  static bool exempt(const P &, const hbtg_params &, ...)
  {
    return false;
  }
  template <class V, class P>
  static auto set_type(V &type, int64_t g, const P &p, const Options &opt) -> decltype((void)p.Type)
  {
    if (opt.has_types)
      type[g] = (uint8_t)p.Type;
  }
  template <class V, class P>
  static void set_type(V &, int64_t, const P &, ...)
  {
  }
  template <class V, class P>
  static auto set_thermal(V &u, int64_t g, const P &p, const Options &opt) -> decltype((void)p.InternalEnergy)
  {
    if (opt.has_thermal)
      u[g] = p.InternalEnergy;
  }
  template <class V, class P>
  static void set_thermal(V &, int64_t, const P &, ...)
  {
  }

  template <class Subhalo>
  static void apply(Subhalo &sub, int64_t s, const std::vector<int64_t> &offsets, const hbtg_batch &b,
                    const Options &opt)
  {
    const int64_t off = offsets[s], n = offsets[s + 1] - off;
    const int st = b.status[s];
    if (st == HBTG_SUB_EMPTY)
    {
      sub.Nbound = 0;
      sub.Mbound = 0;
      for (int d = 0; d < 3; d++)
      {
        sub.CoreComovingPosition[d] = b.core[8 * s + d];
        sub.CorePhysicalVelocity[d] = b.core[8 * s + 3 + d];
      }
      sub.CoreComovingSigmaR = sub.CorePhysicalSigmaV = 0;
      sub.ParticleBindingEnergies.clear();
      sub.ParticlePotentialEnergies.clear();
      return;
    }
    // permutation (identity for disrupted subhaloes)
    auto old = sub.Particles;
    for (int64_t k = 0; k < n; k++)
      sub.Particles[k] = old[b.order[off + k]];
    sub.Nbound = b.nbound[s];
    sub.Mbound = b.mbound[s];
    copy_types(sub, s, b, opt);
    sub.TracerIndex = b.tracer_index[s];
    for (int d = 0; d < 3; d++)
    {
      sub.ComovingAveragePosition[d] = b.ref_pos[3 * s + d];
      sub.PhysicalAverageVelocity[d] = b.ref_vel[3 * s + d];
      sub.ComovingMostBoundPosition[d] = b.mostbound_pos[3 * s + d];
      sub.PhysicalMostBoundVelocity[d] = b.mostbound_vel[3 * s + d];
      sub.CoreComovingPosition[d] = b.core[8 * s + d];
      sub.CorePhysicalVelocity[d] = b.core[8 * s + 3 + d];
    }
    sub.CoreComovingSigmaR = b.core[8 * s + 6];
    sub.CorePhysicalSigmaV = b.core[8 * s + 7];
    sub.SpecificSelfPotentialEnergy = b.kinematics[5 * s];
    sub.SpecificSelfKineticEnergy = b.kinematics[5 * s + 1];
    for (int d = 0; d < 3; d++)
      sub.SpecificAngularMomentum[d] = b.kinematics[5 * s + 2 + d];
    if (st == HBTG_SUB_DISRUPTED)
    {
      if (sub.SnapshotOfDeath == opt.null_snapshot) // IsAlive()
        sub.SnapshotOfDeath = opt.snapshot_id;
    }
    else
    {
      if (sub.SnapshotOfDeath != opt.null_snapshot)
      {
        sub.SnapshotOfDeath = opt.null_snapshot;
        sub.DescendantTrackId = opt.null_track;
      }
      if (sub.SinkTrackId != opt.null_track) // IsTrapped()
      {
        sub.SnapshotOfSink = opt.null_snapshot;
        sub.SinkTrackId = opt.null_track;
      }
      sub.MostBoundParticleId = b.most_bound_id[s];
    }
    if (opt.save_binding)
      sub.ParticleBindingEnergies.assign(b.energy + off, b.energy + off + sub.Nbound);
    if (opt.save_potential)
      sub.ParticlePotentialEnergies.assign(b.potential + off, b.potential + off + sub.Nbound);
  }

  template <class Subhalo>
  static auto copy_types(Subhalo &sub, int64_t s, const hbtg_batch &b, const Options &)
    -> decltype((void)sub.NboundType[0])
  {
    for (int t = 0; t < HBTG_TYPE_MAX; t++)
    {
      sub.NboundType[t] = b.nbound_type[6 * s + t];
      sub.MboundType[t] = b.mbound_type[6 * s + t];
    }
  }
  template <class Subhalo>
  static void copy_types(Subhalo &, int64_t, const hbtg_batch &, ...)
  {
  }
};

} // namespace hbtg_shim
