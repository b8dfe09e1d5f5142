"""The C++ host shim (hbtg_unbind_shim.hpp) instantiates against types shaped
like HBT-HERONS' Subhalo_t / Particle_t (src/subhalo.h, src/snapshot.h): with
particle types and thermal energy (hydro build) and without them (DM_ONLY),
for both the plain and the learned call.  A syntax-only compile, no GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SOURCE = r"""
#include <cstdint>
#include <vector>
#include "hbtg_unbind_shim.hpp"

struct HydroParticle
{
  int64_t Id;
  float ComovingPosition[3], PhysicalVelocity[3];
  float Mass, InternalEnergy;
  int Type;
};
struct DmoParticle
{
  int64_t Id;
  float ComovingPosition[3], PhysicalVelocity[3];
  float Mass;
};
template <class P>
struct Subhalo
{
  std::vector<P> Particles;
  int64_t Nbound, NboundType[6], TracerIndex, MostBoundParticleId, DescendantTrackId, SinkTrackId;
  float Mbound, MboundType[6];
  float ComovingAveragePosition[3], PhysicalAverageVelocity[3];
  float ComovingMostBoundPosition[3], PhysicalMostBoundVelocity[3];
  float SpecificSelfPotentialEnergy, SpecificSelfKineticEnergy, SpecificAngularMomentum[3];
  float CoreComovingPosition[3], CorePhysicalVelocity[3], CoreComovingSigmaR, CorePhysicalSigmaV;
  int SnapshotOfDeath, SnapshotOfSink;
  std::vector<float> ParticleBindingEnergies, ParticlePotentialEnergies;
};

template <class P>
void use(hbtg_shim::Unbinder &u, std::vector<Subhalo<P> *> &subs, bool types)
{
  hbtg_params p;
  hbtg_default_params(&p);
  hbtg_shim::Options o;
  o.has_types = types;
  o.save_binding = true;
  u.unbind(p, subs, o);
  u.unbind_learned(p, subs, o);
}

void all(hbtg_shim::Unbinder &u, std::vector<Subhalo<HydroParticle> *> &h, std::vector<Subhalo<DmoParticle> *> &d)
{
  use(u, h, true);
  use(u, d, false);
  u.set_model(std::vector<float>(HBTG_MLP_PARAMS, 0.f), 0.5f, 0.f, 100);
}
"""


def test_shim_instantiates_for_hydro_and_dmo_types(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "use_shim.cpp"
    src.write_text(SOURCE)
    cmd = [cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wno-deprecated-declarations",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "hbt-herons_gb300", "host"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
