// shim_nested_driver.cpp - test program: runs the C++ host shim's
// recursive_unbind (hbt-herons_gb300/host/hbtg_unbind_shim.hpp) through
// libhbtg.so over a nesting forest read from a file, with types shaped like
// HBT-HERONS' Subhalo_t / Particle_t (src/subhalo.h, src/snapshot.h, DM_ONLY),
// and writes each subhalo's outcome.  Compiled and run by
// tests/test_shim_nested.py.
//
// Input (native-endian raw): hbtg_params; int64 P, S, merge_trapped,
// snapshot_id; float pos[3P], vel[3P], mass[P]; int64 id[P]; int64
// member_off[S+1], member_idx[member_off[S]], parent[S]; float ref_pos[3S],
// ref_vel[3S], mostbound_pos[3S], mostbound_vel[3S]; int64 most_bound_id[S].
// Output: per subhalo int64 nbound, most_bound_id, sink_track_id,
// snapshot_of_sink, snapshot_of_death, n_particles; float mbound; then the
// final Particles' IDs (int64 each).
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "hbtg_unbind_shim.hpp"

struct Particle
{
  int64_t Id;
  float ComovingPosition[3], PhysicalVelocity[3];
  float Mass;
};

struct Subhalo
{
  std::vector<Particle> Particles;
  int64_t Nbound = 0, TracerIndex = 0, MostBoundParticleId = -1, DescendantTrackId = -1, SinkTrackId = -1,
          TrackId = -1;
  float Mbound = 0.f;
  float ComovingAveragePosition[3], PhysicalAverageVelocity[3], ComovingMostBoundPosition[3],
    PhysicalMostBoundVelocity[3];
  float SpecificSelfPotentialEnergy = 0.f, SpecificSelfKineticEnergy = 0.f, SpecificAngularMomentum[3] = {};
  float CoreComovingPosition[3] = {}, CorePhysicalVelocity[3] = {}, CoreComovingSigmaR = 0.f,
        CorePhysicalSigmaV = 0.f;
  int SnapshotOfDeath = -1, SnapshotOfSink = -1;
  std::vector<float> ParticleBindingEnergies, ParticlePotentialEnergies;
  std::vector<int64_t> NestedSubhalos;
};

template <class T>
static void get(FILE *f, T *dst, size_t n)
{
  if (n && fread(dst, sizeof(T), n, f) != n)
    throw std::runtime_error("short input file");
}

int main(int argc, char **argv)
{
  if (argc != 3)
  {
    fprintf(stderr, "usage: %s input output\n", argv[0]);
    return 2;
  }
  try
  {
    FILE *f = fopen(argv[1], "rb");
    if (!f)
      throw std::runtime_error("cannot open input");
    hbtg_params params;
    get(f, &params, 1);
    int64_t hdr[4];
    get(f, hdr, 4);
    const int64_t P = hdr[0], S = hdr[1];
    std::vector<float> pos(3 * P), vel(3 * P), mass(P);
    std::vector<int64_t> id(P), member_off(S + 1), parent(S), mbid(S);
    get(f, pos.data(), pos.size());
    get(f, vel.data(), vel.size());
    get(f, mass.data(), mass.size());
    get(f, id.data(), id.size());
    get(f, member_off.data(), member_off.size());
    std::vector<int64_t> member_idx(member_off[S]);
    get(f, member_idx.data(), member_idx.size());
    get(f, parent.data(), parent.size());
    std::vector<float> frame(12 * S);
    get(f, frame.data(), frame.size());
    get(f, mbid.data(), mbid.size());
    fclose(f);

    std::vector<Subhalo> subs(S);
    std::vector<int64_t> roots;
    for (int64_t s = 0; s < S; s++)
    {
      Subhalo &sub = subs[s];
      sub.TrackId = s;
      for (int64_t k = member_off[s]; k < member_off[s + 1]; k++)
      {
        const int64_t g = member_idx[k];
        Particle p;
        p.Id = id[g];
        for (int d = 0; d < 3; d++)
        {
          p.ComovingPosition[d] = pos[3 * g + d];
          p.PhysicalVelocity[d] = vel[3 * g + d];
        }
        p.Mass = mass[g];
        sub.Particles.push_back(p);
      }
      sub.Nbound = (int64_t)sub.Particles.size();
      for (int d = 0; d < 3; d++)
      {
        sub.ComovingAveragePosition[d] = frame[3 * s + d];
        sub.PhysicalAverageVelocity[d] = frame[3 * S + 3 * s + d];
        sub.ComovingMostBoundPosition[d] = frame[6 * S + 3 * s + d];
        sub.PhysicalMostBoundVelocity[d] = frame[9 * S + 3 * s + d];
      }
      sub.MostBoundParticleId = mbid[s];
      if (parent[s] < 0)
        roots.push_back(s);
    }
    for (int64_t s = 0; s < S; s++)
      if (parent[s] >= 0)
        subs[parent[s]].NestedSubhalos.push_back(s);

    hbtg_shim::Unbinder gpu(0);
    hbtg_shim::Options opt;
    opt.has_types = false;
    opt.snapshot_id = (int)hdr[3];
    opt.merge_trapped = hdr[2] != 0;
    gpu.recursive_unbind(params, subs, roots, opt);

    FILE *o = fopen(argv[2], "wb");
    if (!o)
      throw std::runtime_error("cannot open output");
    for (const Subhalo &sub : subs)
    {
      const int64_t rec[6] = {sub.Nbound, sub.MostBoundParticleId, sub.SinkTrackId, sub.SnapshotOfSink,
                              sub.SnapshotOfDeath, (int64_t)sub.Particles.size()};
      fwrite(rec, sizeof(int64_t), 6, o);
      fwrite(&sub.Mbound, sizeof(float), 1, o);
      for (const Particle &p : sub.Particles)
        fwrite(&p.Id, sizeof(int64_t), 1, o);
    }
    fclose(o);
  }
  catch (const std::exception &e)
  {
    fprintf(stderr, "shim_nested_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
