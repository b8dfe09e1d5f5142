// shim_steps_driver.cpp - test program: runs the C++ host shim's properties()
// and reassign() (hbt-herons_gb300/host/hbtg_unbind_shim.hpp) through
// libhbtg.so on subhaloes read from a file, with types shaped like
// HBT-HERONS' Subhalo_t / Particle_t (src/subhalo.h, src/snapshot.h, hydro
// build), and writes each subhalo's outcome.  Compiled and run by
// tests/test_shim_steps.py.
//
// "props" input (native-endian raw): hbtg_params; int64 S, N, snapshot_id;
// double source_relax; int64 offsets[S+1]; float pos[3N], mass[N]; int64
// order[N] (the bound order: the file's particles are permuted by it first),
// nbound[S]; float mbound[S], mostbound_pos[3S], last_vmax[S], rmax_last[S];
// int32 snap_last[S]; float r200[S], m200[S].
// "props" output per subhalo: float rmax, vmax, rhalf, renclose, r200, m200,
// last_vmax, rmax_last; int32 snap_last; float inertia[6], inertia_w[6];
// int64 particles kept.
//
// "reassign" input: hbtg_params; int64 G, S, N, k; int64 group_off[G+1],
// offsets[S+1], nbound[S]; float pos[3N], mass[N]; uint8 type[N].  Particle
// IDs are the input positions 0..N-1.
// "reassign" output: int64 moved; per subhalo int64 nbound, tracer_index,
// n_particles, nbound_type[6]; float mbound_type[6]; int64 ids[n_particles].
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "hbtg_unbind_shim.hpp"

struct Particle
{
  int64_t Id;
  float ComovingPosition[3], PhysicalVelocity[3];
  float Mass, InternalEnergy;
  int Type;
};

struct Subhalo
{
  std::vector<Particle> Particles;
  int64_t Nbound = 0, NboundType[6] = {}, TracerIndex = 0, MostBoundParticleId = -1, DescendantTrackId = -1,
          SinkTrackId = -1, TrackId = -1;
  float Mbound = 0.f, MboundType[6] = {};
  float ComovingAveragePosition[3] = {}, PhysicalAverageVelocity[3] = {}, ComovingMostBoundPosition[3] = {},
        PhysicalMostBoundVelocity[3] = {};
  float SpecificSelfPotentialEnergy = 0.f, SpecificSelfKineticEnergy = 0.f, SpecificAngularMomentum[3] = {};
  float CoreComovingPosition[3] = {}, CorePhysicalVelocity[3] = {}, CoreComovingSigmaR = 0.f,
        CorePhysicalSigmaV = 0.f;
  int SnapshotOfDeath = -1, SnapshotOfSink = -1;
  std::vector<float> ParticleBindingEnergies, ParticlePotentialEnergies;
  std::vector<int64_t> NestedSubhalos;
  float RmaxComoving = 0.f, VmaxPhysical = 0.f, RHalfComoving = 0.f, REncloseComoving = 0.f,
        BoundR200CritComoving = 0.f, BoundM200Crit = 0.f, LastMaxVmaxPhysical = 0.f,
        RmaxComovingOfLastMaxVmax = 0.f, InertialTensor[6] = {}, InertialTensorWeighted[6] = {};
  int SnapshotOfLastMaxVmax = -1;
};

template <class T>
static void get(FILE *f, T *dst, size_t n)
{
  if (n && fread(dst, sizeof(T), n, f) != n)
    throw std::runtime_error("short input file");
}

template <class T>
static void put(FILE *f, const T *src, size_t n)
{
  if (n && fwrite(src, sizeof(T), n, f) != n)
    throw std::runtime_error("short write");
}

static void run_props(FILE *f, FILE *o)
{
  hbtg_params params;
  get(f, &params, 1);
  int64_t hdr[3];
  get(f, hdr, 3);
  const int64_t S = hdr[0], N = hdr[1];
  double relax;
  get(f, &relax, 1);
  std::vector<int64_t> off(S + 1), order(N), nbound(S);
  std::vector<float> pos(3 * N), mass(N), mbound(S), mbpos(3 * S), last_vmax(S), rmax_last(S), r200(S), m200(S);
  std::vector<int32_t> snap_last(S);
  get(f, off.data(), off.size());
  get(f, pos.data(), pos.size());
  get(f, mass.data(), mass.size());
  get(f, order.data(), order.size());
  get(f, nbound.data(), nbound.size());
  get(f, mbound.data(), mbound.size());
  get(f, mbpos.data(), mbpos.size());
  get(f, last_vmax.data(), S);
  get(f, rmax_last.data(), S);
  get(f, snap_last.data(), S);
  get(f, r200.data(), S);
  get(f, m200.data(), S);
  std::vector<Subhalo> subs(S);
  std::vector<Subhalo *> batch;
  for (int64_t s = 0; s < S; s++)
  {
    Subhalo &sub = subs[s];
    for (int64_t k = off[s]; k < off[s + 1]; k++)
    {
      const int64_t g = off[s] + order[k];
      Particle p{};
      p.Id = g;
      for (int d = 0; d < 3; d++)
        p.ComovingPosition[d] = pos[3 * g + d];
      p.Mass = mass[g];
      sub.Particles.push_back(p);
    }
    sub.Nbound = nbound[s];
    sub.Mbound = mbound[s];
    for (int d = 0; d < 3; d++)
      sub.ComovingMostBoundPosition[d] = mbpos[3 * s + d];
    sub.LastMaxVmaxPhysical = last_vmax[s];
    sub.RmaxComovingOfLastMaxVmax = rmax_last[s];
    sub.SnapshotOfLastMaxVmax = snap_last[s];
    sub.BoundR200CritComoving = r200[s];
    sub.BoundM200Crit = m200[s];
    batch.push_back(&sub);
  }
  hbtg_shim::Unbinder gpu(0);
  hbtg_shim::Options opt;
  opt.has_types = false;
  opt.snapshot_id = (int)hdr[2];
  gpu.properties(params, batch, opt, relax, true);
  for (const Subhalo &sub : subs)
  {
    const float a[8] = {sub.RmaxComoving,          sub.VmaxPhysical,  sub.RHalfComoving,
                        sub.REncloseComoving,      sub.BoundR200CritComoving, sub.BoundM200Crit,
                        sub.LastMaxVmaxPhysical,   sub.RmaxComovingOfLastMaxVmax};
    put(o, a, 8);
    const int32_t snap = sub.SnapshotOfLastMaxVmax;
    put(o, &snap, 1);
    put(o, sub.InertialTensor, 6);
    put(o, sub.InertialTensorWeighted, 6);
    const int64_t kept = (int64_t)sub.Particles.size();
    put(o, &kept, 1);
  }
}

static void run_reassign(FILE *f, FILE *o)
{
  hbtg_params params;
  get(f, &params, 1);
  int64_t hdr[4];
  get(f, hdr, 4);
  const int64_t G = hdr[0], S = hdr[1], N = hdr[2];
  std::vector<int64_t> goff(G + 1), off(S + 1), nbound(S);
  std::vector<float> pos(3 * N), mass(N);
  std::vector<uint8_t> type(N);
  get(f, goff.data(), goff.size());
  get(f, off.data(), off.size());
  get(f, nbound.data(), nbound.size());
  get(f, pos.data(), pos.size());
  get(f, mass.data(), mass.size());
  get(f, type.data(), type.size());
  std::vector<Subhalo> subs(S);
  for (int64_t s = 0; s < S; s++)
  {
    for (int64_t g = off[s]; g < off[s + 1]; g++)
    {
      Particle p{};
      p.Id = g;
      for (int d = 0; d < 3; d++)
        p.ComovingPosition[d] = pos[3 * g + d];
      p.Mass = mass[g];
      p.Type = type[g];
      subs[s].Particles.push_back(p);
    }
    subs[s].Nbound = nbound[s];
  }
  std::vector<std::vector<Subhalo *>> groups(G);
  for (int64_t h = 0; h < G; h++)
    for (int64_t s = goff[h]; s < goff[h + 1]; s++)
      groups[h].push_back(&subs[s]);
  hbtg_shim::Unbinder gpu(0);
  const int64_t moved = gpu.reassign(params, groups, (int)hdr[3]);
  put(o, &moved, 1);
  for (const Subhalo &sub : subs)
  {
    const int64_t rec[3] = {sub.Nbound, sub.TracerIndex, (int64_t)sub.Particles.size()};
    put(o, rec, 3);
    put(o, sub.NboundType, 6);
    put(o, sub.MboundType, 6);
    for (const Particle &p : sub.Particles)
      put(o, &p.Id, 1);
  }
}

int main(int argc, char **argv)
{
  if (argc != 4 || (strcmp(argv[1], "props") != 0 && strcmp(argv[1], "reassign") != 0))
  {
    fprintf(stderr, "usage: %s props|reassign input output\n", argv[0]);
    return 2;
  }
  try
  {
    FILE *f = fopen(argv[2], "rb");
    if (!f)
      throw std::runtime_error("cannot open input");
    FILE *o = fopen(argv[3], "wb");
    if (!o)
      throw std::runtime_error("cannot open output");
    if (strcmp(argv[1], "props") == 0)
      run_props(f, o);
    else
      run_reassign(f, o);
    fclose(f);
    fclose(o);
  }
  catch (const std::exception &e)
  {
    fprintf(stderr, "shim_steps_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
