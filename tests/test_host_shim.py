"""The C++ host shim (hbtg_unbind_shim.hpp) instantiates against types shaped
like HBT-HERONS' Subhalo_t / Particle_t (src/subhalo.h, src/snapshot.h): with
particle types and thermal energy (hydro build) and without them (DM_ONLY),
for every entry: the plain and the learned call, the nested recursion, the
properties and the reassignment.  Syntax-only compiles, no GPU."""
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
  float RmaxComoving, VmaxPhysical, RHalfComoving, REncloseComoving, BoundR200CritComoving, BoundM200Crit;
  float LastMaxVmaxPhysical, RmaxComovingOfLastMaxVmax, InertialTensor[6], InertialTensorWeighted[6];
  int SnapshotOfLastMaxVmax;
  int64_t TrackId;
  std::vector<int64_t> NestedSubhalos;
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
  std::vector<Subhalo<P>> list(3);
  list[0].NestedSubhalos = {1, 2};
  u.recursive_unbind(p, list, std::vector<int64_t>{0}, o);
  u.properties(p, subs, o, 3.0, true);
  std::vector<std::vector<Subhalo<P> *>> groups{subs};
  u.reassign(p, groups, 10);
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


REAL_SOURCE = r"""
#include "subhalo.h"
#include "hbtg_unbind_shim.hpp"

// The reference's own Subhalo_t / Particle_t / SubhaloList_t through every
// entry of the shim.
void use_real(hbtg_shim::Unbinder &u, SubhaloList_t &subs, std::vector<Subhalo_t *> &batch)
{
  hbtg_params p;
  hbtg_default_params(&p);
  hbtg_shim::Options o;
#ifdef DM_ONLY
  o.has_types = false;
#endif
  o.save_binding = true;
  o.merge_trapped = true;
  u.unbind(p, batch, o);
  u.unbind_learned(p, batch, o);
  std::vector<int64_t> roots{0};
  u.recursive_unbind(p, subs, roots, o);
  u.properties(p, batch, o, HBTConfig.SourceSubRelaxFactor, true);
  std::vector<std::vector<Subhalo_t *>> groups{batch};
  u.reassign(p, groups, HBTConfig.NumNeighboursForReassignment);
}
"""


@pytest.mark.parametrize("variant", [["-DDM_ONLY"], ["-DUNBIND_WITH_THERMAL_ENERGY"]], ids=["dmo", "hydro"])
def test_shim_compiles_against_the_reference_headers(tmp_path, variant):
    """The shim instantiated with the reference's real types (src/subhalo.h,
    src/snapshot.h), against the oracle's single-rank MPI/HDF5 stub headers;
    skipped where the reference sources are absent."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle
    if not build_oracle.reference_available():
        pytest.skip("reference sources absent")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "use_real.cpp"
    src.write_text(REAL_SOURCE)
    ref = build_oracle.REF_ROOT
    cmd = [cxx, "-std=c++17", "-fsyntax-only", "-Wno-deprecated-declarations", "-DHBT_INT8", "-DINPUT_INT8",
           *variant, "-I", os.path.join(ROOT, "oracle", "stub"), "-I", os.path.join(ref, "src"), "-I", ref,
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "hbt-herons_gb300", "host"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.parametrize("program", ["shim_nested_driver.cpp", "shim_steps_driver.cpp"])
def test_driver_programs_build(tmp_path, program):
    """The shim's test programs (run on the GPU by tests/test_shim_nested.py
    and tests/test_shim_steps.py) compile and link against libhbtg.so."""
    from hbtg.build import LIB, build_library
    build_library()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "drv")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wno-deprecated-declarations", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "hbt-herons_gb300", "host"), os.path.join(ROOT, "tests", program),
           "-o", exe, "-L", os.path.dirname(LIB), "-lhbtg", "-Wl,-rpath," + os.path.dirname(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
