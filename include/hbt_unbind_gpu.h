/*
 * hbt_unbind_gpu.h — C ABI of the GB300 unbinding library (libhbtg.so).
 *
 * Drop-in for HBT-HERONS' iterative gravitational unbinding:
 *   void Subhalo_t::Unbind(const Snapshot_t &epoch)          src/subhalo.h:152,
 *                                                            src/subhalo_unbind.cpp:463-808
 *   void SubhaloSnapshot_t::RefineParticles(MpiWorker_t &)   src/subhalo.h:343,
 *                                                            src/subhalo_unbind.cpp:855-919
 * One call unbinds a batch of independent subhaloes (a batch of one is
 * Subhalo_t::Unbind; the field/new-subhalo loops of RefineParticles are a
 * batch of many).  Plain pointers and sizes only; no C++ types cross it.
 *
 * Conventions
 *  - Every function returns an hbtg_status (0 = OK).  Nothing throws across
 *    the ABI and the device never traps: per-subhalo problems are reported
 *    in batch->status.
 *  - The caller owns every array.  The handle owns the device arena.
 *  - One handle per host thread.  hbtg_unbind_batch is synchronous.
 */
#ifndef HBT_UNBIND_GPU_H
#define HBT_UNBIND_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HBTG_TYPE_MAX 6 /* ParticleType_t::TypeMax, src/datatypes.h:206-215 */
#define HBTG_KIN_STRIDE 5  /* SpecificSelfPotentialEnergy, SpecificSelfKineticEnergy, SpecificAngularMomentum[3] */
#define HBTG_CORE_STRIDE 8 /* CoreComovingPosition[3], CorePhysicalVelocity[3], CoreComovingSigmaR, CorePhysicalSigmaV */

/* Return codes of every entry point. */
enum hbtg_status
{
  HBTG_OK = 0,
  HBTG_ERR_INVALID = 1,     /* bad argument or inconsistent batch description */
  HBTG_ERR_NOMEM = 2,       /* device or pinned-host allocation failed */
  HBTG_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  HBTG_ERR_MAX_ITER = 4,    /* some subhalo reached params.max_iterations (see batch->status) */
  HBTG_ERR_UNSUPPORTED = 5, /* parameter combination not implemented on this path */
  HBTG_ERR_NO_DEVICE = 6    /* no CUDA device, or the device is not sm_103 */
};

/* Per-subhalo outcome written to hbtg_batch.status. */
enum hbtg_sub_status
{
  HBTG_SUB_CONVERGED = 0, /* Nbound >= Nlast*BoundMassPrecision reached (src/subhalo_unbind.cpp:690) */
  HBTG_SUB_DISRUPTED = 1, /* Nbound < MinNumPartOfSub or too few tracers (src/subhalo_unbind.cpp:647) */
  HBTG_SUB_EMPTY = 2,     /* no particles: the orphan early return (src/subhalo_unbind.cpp:472-489) */
  HBTG_SUB_MAX_ITER = 3   /* stopped at params.max_iterations; outputs hold the last iterate */
};

/* The HBTConfig / PhysicalConst / Cosmology values Subhalo_t::Unbind reads
 * (src/config_parser.h:22-201, src/snapshot.h:18-48).  Where the reference
 * stores a value as HBTReal (float), the library rounds it to float first. */
typedef struct hbtg_params
{
  double box_size;             /* BoxSize */
  int32_t periodic;            /* PeriodicBoundaryOn */
  double softening;            /* HBTConfig.GetCurrentSoftening(a) (src/config_parser.cpp:641-649) */
  double tree_node_resolution; /* TreeNodeResolution = 0.1*SofteningHalo (src/config_parser.cpp:210) */
  double open_angle;           /* TreeNodeOpenAngle (theta) */
  double bound_mass_precision; /* BoundMassPrecision */
  int64_t min_num_part;        /* MinNumPartOfSub */
  int64_t min_num_tracer;      /* MinNumTracerPartOfSub */
  int32_t tracer_type_mask;    /* TracerParticleBitMask */
  int32_t no_subsample_mask;   /* DoNotSubsampleParticleBitMask */
  int64_t max_sample_size;     /* MaxSampleSizeOfPotentialEstimate (0 = no subsampling) */
  int32_t refine_most_bound;   /* RefineMostBoundParticle */
  double refine_fraction;      /* BoundFractionCenterRefinement */
  int32_t upscale_per_type;    /* PotentialEstimateUpscaleMassesPerType */
  int64_t sub_core_size_min;   /* SubCoreSizeMin */
  double sub_core_size_factor; /* SubCoreSizeFactor */
  int32_t dm_only;             /* 1 = DM_ONLY build semantics: types ignored, every particle a tracer */
  int32_t thermal;             /* 1 = UNBIND_WITH_THERMAL_ENERGY: E += InternalEnergy */
  double G;                    /* PhysicalConst::G */
  double scale_factor;         /* epoch.Cosmology.ScaleFactor */
  double hubble;               /* epoch.Cosmology.Hz */
  int32_t max_iterations;      /* bound on the unbinding loop (no counterpart in the reference) */
  int32_t mode;                /* 0 = reference tree geometry (parity); other values reserved */
  int64_t seed;                /* seeds the tie-break of sub-resolution cells (reference: drand48) */
  int32_t prepared_subsample;  /* 1 = particles already prepared for subsampling: DoNotSubsample types
                                  first, the rest in random order (PrepareParticlesForSubsampling,
                                  src/subhalo_unbind.cpp:430-443).  The GPU path requires it when
                                  max_sample_size > 0; the subsample is the leading entries. */
} hbtg_params;

/* A batch of subhaloes in CSR layout: subhalo s owns particles
 * [offsets[s], offsets[s+1]) of every per-particle array.  Local index k of
 * subhalo s means global row offsets[s]+k.
 *
 * Inputs mirror Particle_t (src/snapshot.h:62-106) as structure-of-arrays;
 * in/out fields mirror the Subhalo_t members Unbind reads and writes
 * (src/subhalo.h:26-216). */
typedef struct hbtg_batch
{
  int64_t n_sub;
  const int64_t *offsets; /* [n_sub+1], offsets[0] = 0, non-decreasing */
  const float *pos;       /* [3N] ComovingPosition, xyz interleaved */
  const float *vel;       /* [3N] PhysicalVelocity */
  const float *mass;      /* [N]  Mass */
  const float *u;         /* [N]  InternalEnergy, or NULL (read only if params.thermal) */
  const int64_t *id;      /* [N]  Id */
  const uint8_t *type;    /* [N]  Type (0..5), or NULL = every particle TypeDM */

  float *ref_pos;       /* [3 n_sub] in: initial ComovingAveragePosition; out: final frame */
  float *ref_vel;       /* [3 n_sub] in: initial PhysicalAverageVelocity; out: final frame */
  float *mostbound_pos; /* [3 n_sub] in/out: ComovingMostBoundPosition */
  float *mostbound_vel; /* [3 n_sub] in/out: PhysicalMostBoundVelocity */
  int64_t *most_bound_id; /* [n_sub] in/out: MostBoundParticleId (kept when not resolved) */

  int64_t *order;       /* [N] out: order[offsets[s]+k] = input local index of the particle now at position k */
  int64_t *nbound;      /* [n_sub] out: Nbound */
  float *mbound;        /* [n_sub] out: Mbound */
  int64_t *nbound_type; /* [6 n_sub] out: NboundType, or NULL */
  float *mbound_type;   /* [6 n_sub] out: MboundType, or NULL */
  int64_t *tracer_index; /* [n_sub] out: TracerIndex */
  float *kinematics;    /* [5 n_sub] out, or NULL (HBTG_KIN_STRIDE) */
  float *core;          /* [8 n_sub] out, or NULL (HBTG_CORE_STRIDE) */
  float *energy;        /* [N] out, or NULL: ParticleBindingEnergies at positions k < nbound */
  float *potential;     /* [N] out, or NULL: ParticlePotentialEnergies at positions k < nbound */
  int32_t *iterations;  /* [n_sub] out: unbinding iterations (NumberUnbindingIterations) */
  int32_t *status;      /* [n_sub] out: enum hbtg_sub_status */
} hbtg_batch;

/* Counters of the last call, for measurement. */
typedef struct hbtg_stats
{
  int64_t n_sub;
  int64_t n_particles;
  int64_t total_bound;        /* sum of nbound */
  int64_t global_iterations;  /* lock-step iterations of the batch */
  int64_t interactions;       /* node/particle interactions evaluated by the tree walks (if counted) */
  int64_t tree_nodes;         /* internal nodes built, summed over iterations */
  double ms_total;            /* wall time of the device part of the last call (CUDA events) */
  double ms_walk;             /* summed tree-walk kernel time (CUDA events) */
  double ms_plan;             /* per-iteration planning: packing scans and host reads */
  double ms_tree;             /* tree builds: bounding cubes, keys, sorts, cells */
  double ms_part;             /* energies, partition, sort of the removed tails */
  double ms_frame;            /* centre-of-mass frames and convergence tests */
  double ms_final;            /* final energy sort and epilogue */
  int64_t walk_launches;
  int64_t kernel_launches;    /* kernels launched by the last call */
  int64_t h2d_bytes, d2h_bytes;
  /* warm-started calls only (zero otherwise) */
  double ms_propose;          /* features, network, partition and first frame */
  int64_t warm_subhaloes;     /* subhaloes started from a proposal */
  int64_t excluded;           /* particles left out after the first test */
  int64_t readmitted;         /* untrusted particles the first test kept */
  int64_t cold_restarts;      /* warm subhaloes restarted cold (their first iteration converges) */
  int64_t readmit_rounds;     /* first tests run (lock-step) */
  int64_t walk_blocks_per_sm; /* resident tree-walk blocks per SM of the last call's launches */
  double ms_h2d;              /* host-pointer calls: uploads on the call's stream before the first kernel */
  double ms_d2h;              /* host-pointer calls: downloads after the last kernel */
  /* tree-walk traversal counters (counted calls only, like interactions) */
  int64_t walk_steps;           /* warp traversal steps */
  int64_t walk_nodes;           /* nodes popped from the warps' range stacks */
  int64_t walk_pending_batches; /* batches of cells resolved by every target's own test */
  int64_t walk_entries_full;    /* far entries that every target of the warp takes */
  int64_t walk_entries_part;    /* far entries for part of the targets */
  int64_t walk_entries_near;    /* entries within a softening length of some target */
  int64_t walk_drained;         /* ranges walked target by target (deep stacks) */
  int64_t walk_cycles[8];       /* warp clock cycles: pop and classify, resolve pending cells, list and
                                   stack writes, evaluate the full / masked far / near lists, drain,
                                   whole target groups */
  int64_t host_syncs;           /* stream synchronisations for host reads of device totals */
} hbtg_stats;

typedef struct hbtg_handle hbtg_handle;

/* Creates a handle bound to CUDA device `device`.  Checks that the device is
 * compute capability 10.3.  Replaces nothing in the reference (its trees are
 * stack objects, src/subhalo_unbind.cpp:517-518). */
int hbtg_create(hbtg_handle **handle, int device);

/* Frees the device arena and the handle. */
int hbtg_destroy(hbtg_handle *handle);

/* Unbinds every subhalo of `batch`; all pointers are HOST pointers.  Copies
 * inputs to the device, runs, copies outputs back, synchronises.
 * Replaces: Subhalo_t::Unbind (src/subhalo_unbind.cpp:463) for n_sub = 1, and
 * the OpenMP loops of SubhaloSnapshot_t::RefineParticles
 * (src/subhalo_unbind.cpp:888-903) for a batch. */
int hbtg_unbind_batch(hbtg_handle *handle, const hbtg_params *params, hbtg_batch *batch);

/* Same as hbtg_unbind_batch but every array pointer in `batch` is a DEVICE
 * pointer, except `offsets`, which is a host array; work is queued on
 * `cuda_stream` (a cudaStream_t, NULL = legacy default stream) and the call
 * returns after the stream is synchronised. */
int hbtg_unbind_batch_device(hbtg_handle *handle, const hbtg_params *params, hbtg_batch *batch, void *cuda_stream);

/* Host-side PrepareParticlesForSubsampling (src/subhalo_unbind.cpp:430-443,
 * 522-524) for every subhalo of a batch (host arrays; no device work): for a
 * subhalo with more than max_sample_size particles, DoNotSubsample types first
 * (std::partition) and the rest shuffled (std::random_shuffle after
 * srand(seed), subhaloes in order), exactly as the reference reorders
 * Particles.  Writes perm[offsets[s]+k] = input local index to place at
 * position k (identity for the others).  Apply it to the particle arrays, call
 * hbtg_unbind_batch with prepared_subsample = 1, and compose the returned
 * order with perm.  Required before the GPU path when max_sample_size > 0. */
int hbtg_prepare_subsampling(const hbtg_params *params, const hbtg_batch *batch, int64_t *perm);

/* Fills `stats` with the counters of the last call on this handle. */
int hbtg_get_stats(const hbtg_handle *handle, hbtg_stats *stats);

/* Enables (1) or disables (0) the interaction counter of the tree walk
 * (slower; used to compute the roofline's algorithmic flops). */
int hbtg_set_count_interactions(hbtg_handle *handle, int enable);

/* Launch settings of the unbinding that leave every result unchanged: a
 * stable radix sort gives the same order whether one block or a chain of
 * passes runs it, the walk computes a 32-target chunk the same way whichever
 * warp takes it, and each tree cell is summed by one thread whatever the
 * grid.  No counterpart in the reference (they are choices of the GPU
 * schedule, not of the method). */
typedef struct hbtg_tuning
{
  int32_t block_sort_max;        /* sorts of at most this many items run in one block (0 = never; at most 8192) */
  int32_t walk_ranged_min;       /* walks of fewer 32-target chunks use a grid-stride loop, the others per-SM ranges */
  int32_t moments_blocks_per_sm; /* grid cap, in blocks per SM, of the per-level multipole passes (1-32) */
  double ms;                     /* hbtg_autotune: measured time of one call with these settings (0 = not measured) */
} hbtg_tuning;

/* The handle's launch settings (defaults: 8192, 0, 8). */
int hbtg_get_tuning(const hbtg_handle *handle, hbtg_tuning *tuning);
int hbtg_set_tuning(hbtg_handle *handle, const hbtg_tuning *tuning);

/* Autotuner: times hbtg_unbind_batch_device on `batch` (device arrays and
 * host offsets, as for that call) for each candidate setting
 * (block_sort_max in {0, 2048, 8192} x walk_ranged_min in {0, 1024} x
 * moments_blocks_per_sm in {4, 8}), two calls each with the second timed,
 * and keeps the fastest on the handle.  The batch's in/out frame arrays are
 * restored before every call and on return, so they hold their inputs again;
 * its outputs hold the results, which every candidate gives alike.  report
 * (may be NULL) receives up to max_report candidates with their times and
 * *n_report (may be NULL) their number.  No counterpart in the reference. */
int hbtg_autotune(hbtg_handle *handle, const hbtg_params *params, hbtg_batch *batch, void *cuda_stream,
                  hbtg_tuning *report, int max_report, int *n_report);

/* Static description of a return code. */
const char *hbtg_status_string(int status);

/* Fills `params` with the reference defaults (src/config_parser.h:98-172)
 * and a=1, Hz=0, G=43.0071 (src/config_parser.cpp:200 with default units). */
void hbtg_default_params(hbtg_params *params);

/* Unbinding for callers that cannot allocate GPU memory; no counterpart in
 * the reference.  Same contract as hbtg_unbind_batch_device (device arrays,
 * host offsets, work queued on `cuda_stream`, synchronised before return) but
 * it needs no handle and calls no allocator: its working memory is a fixed
 * reserve of about 17 MiB inside the library, held on every GPU that loads it
 * until the process exits.  Limits: at most 65,536 particles and 8,192
 * subhaloes per call (else HBTG_ERR_INVALID) and at most 196,608 tree records
 * in one tree (else HBTG_ERR_NOMEM).  On either of these two returns none
 * of the caller's arrays has been written: the iteration runs on copies of the
 * in/out frames inside the reserve, so the batch can be retried through an
 * allocating entry point.  Every call looks up the reserve's device address.
 * With lazy module loading (the CUDA default) the reserve itself is
 * allocated when the first call on a device loads the library's module: make
 * one warm-up call outside any region that must not allocate and before any
 * stream capture.  All calls share the reserve: calls that overlap on the GPU
 * race. */
int hbtg_unbind_batch_noalloc(const hbtg_params *params, hbtg_batch *batch, void *cuda_stream);

/* The tree potential of one particle set: GravityTree_t::Build over the n_src
 * sources (src/gravity_tree.cpp:25-80, src/oct_tree.tpp:12-142) and
 * EvaluatePotential (src/gravity_tree.cpp:82-166) at the sources listed in
 * tgt_index, each with its self term cancelled (as Unbind evaluates its
 * particles).  potential[t] = G/a * phi, in the geometry and FP32 arithmetic
 * of the unbinding walk.  Device arrays: pos [3 n_src], mass [n_src],
 * tgt_index [n_tgt] (int64 indices into the sources), potential [n_tgt]. */
int hbtg_tree_potential_device(hbtg_handle *handle, const hbtg_params *params, int64_t n_src, const float *pos,
                               const float *mass, int64_t n_tgt, const int64_t *tgt_index, float *potential,
                               void *cuda_stream);

/* ------------------------------------------------------------------------
 * Properties of the unbound subhaloes (the steps after Unbind that read the
 * bound set; the fields are Subhalo_t members, src/subhalo.h:55-77).
 * ------------------------------------------------------------------------ */
typedef struct hbtg_props
{
  float *rmax;        /* RmaxComoving */
  float *vmax;        /* VmaxPhysical */
  float *rhalf;       /* RHalfComoving */
  float *renclose;    /* REncloseComoving */
  float *r200;        /* BoundR200CritComoving (in/out: kept where no radius qualifies, as the reference) */
  float *m200;        /* BoundM200Crit (in/out, likewise) */
  float *last_vmax;   /* LastMaxVmaxPhysical (in/out) */
  float *rmax_last;   /* RmaxComovingOfLastMaxVmax (in/out) */
  int32_t *snap_last; /* SnapshotOfLastMaxVmax (in/out) */
  float *inertia;     /* InertialTensor, 6 per subhalo: xx, xy, xz, yy, yz, zz */
  float *inertia_w;   /* InertialTensorWeighted, 6 per subhalo */
  int64_t *nsource;   /* particles TruncateSource keeps (or NULL) */
} hbtg_props;

/* Subhalo_t::CalculateProfileProperties (src/subhalo.cpp:175-243, with
 * Snapshot_t::SphericalOverdensitySize, src/snapshot.cpp:258-282),
 * Subhalo_t::CalculateShape (src/subhalo.cpp:245-309) and
 * Subhalo_t::TruncateSource (src/subhalo_unbind.cpp:843-853) for every
 * subhalo of a batch, from the bound set an unbinding call returned: `batch`
 * holds the input particles (pos, mass; offsets on the host) and that call's
 * order, nbound, mbound and mostbound_pos.  Uses params' softening, box,
 * periodic flag, G, scale_factor and hubble; snapshot_id is the current
 * snapshot (SnapshotOfLastMaxVmax); source_relax is SourceSubRelaxFactor.
 * The _device form takes device arrays and queues on cuda_stream; the other
 * takes host arrays. */
int hbtg_subhalo_properties_device(hbtg_handle *handle, const hbtg_params *params, const hbtg_batch *batch,
                                   int32_t snapshot_id, double source_relax, hbtg_props *props, void *cuda_stream);
int hbtg_subhalo_properties(hbtg_handle *handle, const hbtg_params *params, const hbtg_batch *batch,
                            int32_t snapshot_id, double source_relax, hbtg_props *props);

/* ------------------------------------------------------------------------
 * Particle reassignment before unbinding (hydro runs): each non-tracer
 * particle looks up its NumNeighboursForReassignment nearest tracer particles
 * of its FoF group; if none of them belongs to its own subhalo, it moves to
 * the subhalo of the nearest one (SubhaloSnapshot_t::ReassignParticles,
 * src/subhalo_reassign_gas.cpp:65-197, with GeoTree_t::NearestNeighbours,
 * src/geometric_tree.cpp:108-142, whose widening searches count a particle
 * once per search that finds it).
 * ------------------------------------------------------------------------ */
typedef struct hbtg_reassign
{
  int64_t n_groups;         /* FoF groups */
  const int64_t *group_off; /* [n_groups+1] each group's subhaloes as a range of subhalo indices (host) */
  int64_t n_sub;
  const int64_t *offsets;   /* [n_sub+1] each subhalo's particles (host) */
  const float *pos;         /* [3N] comoving positions */
  const uint8_t *type;      /* [N] particle types (tracers: params.tracer_type_mask) */
  int64_t *dest;            /* [N] out: the subhalo the particle moves to, or -1 to stay */
} hbtg_reassign;

/* Decides every move of a batch of FoF groups (the caller appends each moved
 * particle to its destination's source, in subhalo then particle order, and
 * drops it from its own, as ReassignParticles does).  Uses params' box,
 * periodic flag, softening (SofteningHalo: the first search radius is a tenth
 * of it) and tracer_type_mask; num_neighbours is NumNeighboursForReassignment
 * (at most 32).  The _device form takes device pos, type and dest. */
int hbtg_reassign_particles_device(hbtg_handle *handle, const hbtg_params *params, const hbtg_reassign *batch,
                                   int num_neighbours, void *cuda_stream);
int hbtg_reassign_particles(hbtg_handle *handle, const hbtg_params *params, const hbtg_reassign *batch,
                            int num_neighbours);

/* Measurement utility, no counterpart in the reference: FP32 FMA throughput
 * of the device in TFLOP/s (the roofline denominator of the tree walk). */
int hbtg_measure_fp32_peak(int device, double *tflops);

/* ------------------------------------------------------------------------
 * Warm start (no counterpart in the reference, whose Unbind always starts
 * from every particle, src/subhalo_unbind.cpp:505-507, and spends most of its
 * time on that first iteration).  A proposal marks the particles predicted
 * to survive the first iteration (trusted), those it is sure the iteration
 * removes (left out), and the rest, which get the first iteration's own test
 * (their energy against the tree of every particle, in the input frame) and
 * join the trusted ones when bound.  From that set
 * the exact loop runs to its convergence test, the plain method's own path
 * from its second iteration on.  A subhalo whose first iteration would
 * already converge runs cold.  Outputs have the hbtg_unbind_batch layout;
 * `iterations` counts the first iteration.  Not combined with potential subsampling (max_sample_size
 * must be 0).
 * ------------------------------------------------------------------------ */
#define HBTG_MLP_PARAMS 4673 /* weights of the 6-64-64-1 proposer network (layout at hbtg_mlp_forward) */
#define HBTG_NUM_FEATURES 6  /* per-particle inputs of the proposer network */

/* What the previous output knew about each subhalo.  The reference keeps it in
 * Subhalo_t: the bound particles first in Particles, Nbound, and
 * ParticleBindingEnergies (src/subhalo.h:95, src/subhalo_unbind.cpp:787-793). */
typedef struct hbtg_prior
{
  const int64_t *nbound_prev; /* [n_sub] particles [0, nbound_prev[s]) were bound; NULL = unknown */
  const float *energy_prev;   /* [N] their binding energies (entries past nbound_prev ignored); NULL = unknown */
} hbtg_prior;

/* The learned proposer: a particle is trusted when the network's
 * probability is >= threshold, left out without the first test when it is
 * below exclude_below (0 = test every untrusted particle), uncertain
 * otherwise; subhaloes with fewer than min_particles particles start cold.
 * first_test = 1: every uncertain particle gets the plain method's first
 * test (its energy against the tree of every particle) and joins the set if
 * bound.  first_test = 0: the uncertain particles join the set untested (the
 * exact iteration removes those that are unbound) and the first frame is
 * that of the trusted particles alone; this skips the tree of every particle. */
typedef struct hbtg_model
{
  const float *weights; /* [HBTG_MLP_PARAMS] host array */
  float threshold;
  int64_t min_particles;
  float exclude_below;  /* <= threshold */
  int32_t first_test;   /* 1 or 0, see above */
} hbtg_model;

/* Copies the proposer network to the handle's device. */
int hbtg_set_model(hbtg_handle *handle, const hbtg_model *model);

/* Learned warm start: features, the network's proposal, then the
 * warm-started iteration.  Host pointers (prior may be NULL), like
 * hbtg_unbind_batch. */
int hbtg_unbind_batch_learned(hbtg_handle *handle, const hbtg_params *params, hbtg_batch *batch,
                              const hbtg_prior *prior);

/* The same with device pointers (offsets on the host, prior arrays on the
 * device), like hbtg_unbind_batch_device. */
int hbtg_unbind_batch_learned_device(hbtg_handle *handle, const hbtg_params *params, hbtg_batch *batch,
                                     const hbtg_prior *prior, void *cuda_stream);

/* Warm start from an explicit proposal ([N] device array: 1 = trusted,
 * 0 = to test, 2 = left out without the test) instead of the network;
 * subhaloes with fewer than min_particles particles start cold. */
int hbtg_unbind_batch_warm_device(hbtg_handle *handle, const hbtg_params *params, hbtg_batch *batch,
                                  const uint8_t *proposal, int64_t min_particles, void *cuda_stream);

/* The proposer's inputs, features[6i..6i+5] of particle i (device array),
 * computed exactly as the learned call computes them.  batch as for
 * hbtg_unbind_batch_device; nothing is unbound and no output is written. */
int hbtg_features_device(hbtg_handle *handle, const hbtg_params *params, const hbtg_batch *batch,
                         const hbtg_prior *prior, float *features, void *cuda_stream);

/* Training trace of the last unbinding call on this handle, labels[i] in
 * {0, 1} (device array, input order).  which = 1: particle i survived its
 * subhalo's first iteration (E < 0 in the potential of every particle; what
 * the learned proposer predicts).  which = 0: particle i belonged to the set
 * whose potential decided the final bound set (the tree sources of the last
 * iteration). */
int hbtg_trace_labels_device(hbtg_handle *handle, uint8_t *labels, int which, void *cuda_stream);

/* The proposer network on the tensor cores (tcgen05.mma, BF16 operands,
 * FP32 accumulators in tensor memory).  Weights (FP32, device): W1[6][64],
 * b1[64], W2[64][64], b2[64], w3[64], b3 (matrices in x out);
 * p = sigmoid(w3 . relu(W2^T relu(W1^T x + b1) + b2) + b3).
 * prob[i] for features[6i..6i+5]; all device arrays.  Should the tensor core
 * not signal completion within about a second, the rows it had not finished
 * get NaN (neither trusted nor left out by the learned call). */
int hbtg_mlp_forward(const float *weights, const float *features, float *prob, int64_t n, void *cuda_stream);

/* Gradient of sum_i w_i BCE(p_i, y_i) over n rows (sample_weights may be
 * NULL = 1): grad[HBTG_MLP_PARAMS] and loss[1] are overwritten (device). */
int hbtg_mlp_backward(const float *weights, const float *features, const float *labels,
                      const float *sample_weights, int64_t n, float *grad, float *loss, void *cuda_stream);

/* One Adam step on the device: g = grad * grad_scale, bias-corrected moments
 * at step `step` (>= 1). */
int hbtg_adam_step(float *weights, const float *grad, float *m, float *v, int n_params, float lr, float beta1,
                   float beta2, float eps, float grad_scale, int step, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* HBT_UNBIND_GPU_H */
