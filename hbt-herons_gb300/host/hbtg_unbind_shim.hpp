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
#pragma once

#include <algorithm>
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

  // Loads the learned warm start's proposer (weights of hbtg_mlp_forward's layout).
  void set_model(const std::vector<float> &weights, float threshold, float exclude_below, int64_t min_particles)
  {
    if (weights.size() != HBTG_MLP_PARAMS)
      throw std::runtime_error("hbtg_set_model: wrong number of weights");
    hbtg_model m{weights.data(), threshold, min_particles, exclude_below};
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

private:
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
