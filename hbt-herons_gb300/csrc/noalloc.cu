// noalloc.cu - hbtg_unbind_batch_noalloc: the batched unbinding for callers
// that cannot allocate GPU memory.
//
// Who needs this: code that runs where cudaMalloc is not allowed or not
// wanted -- inside a host callback or another library's allocation-free
// section, in a process whose device memory is owned by a pool it must not
// grow, or on a latency path where an allocation (which can synchronise the
// device) is unacceptable.  Such callers pass device inputs and outputs as
// for hbtg_unbind_batch_device; every working buffer (particle copies, keys,
// sort buffers, tree nodes, per-subhalo state) comes from one file-scope
// device array, g_noalloc_scratch, that the library reserves when it is
// loaded and keeps on every GPU that loads it until the process exits.
//
// Limits: at most kNoAllocMaxParticles particles and kNoAllocMaxSubhaloes
// subhaloes per call, and at most kNoAllocMaxRecords tree records (leaves
// plus cells) in one tree; larger calls are rejected with HBTG_ERR_INVALID
// (sizes, checked before any GPU work) or HBTG_ERR_NOMEM (a tree larger than
// the reserve, found mid-run).  The iteration runs on copies of the in/out
// frames (ref_pos, ref_vel, mostbound_pos, mostbound_vel) held in the
// reserve, and every caller array is written only after the last tree is
// built, so on HBTG_ERR_NOMEM none of the caller's arrays has changed and the
// same batch can be retried through an allocating entry point.
//
// Sharing: every call on a device uses the same array and leaves its contents
// behind; each call initialises what it reads before reading it.  Calls whose
// GPU work overlaps (two host threads, or two streams) race on the array and
// must be serialised by the caller.
//
// Set-up: every call looks up the array's device address with
// cudaGetSymbolAddress on the current device (host code cannot use the
// array's name as a device pointer); the lookup is not cached, so a device
// reset between calls is harmless.  With lazy module loading (the CUDA
// default) the array itself is allocated when this file's module is first
// loaded, which happens in the first call on each device: make one warm-up
// call outside any region where the device must not allocate, and before any
// stream capture begins.
#include <algorithm>
#include <cstring>

#include "../../include/hbt_unbind_gpu.h"
#include "common.cuh"
#include "driver.cuh"
#include "kernels.cuh"
#include "primitives.cuh"

using namespace hbtg;

namespace
{

constexpr long long kNoAllocMaxParticles = 1LL << 16; // 65,536
constexpr int kNoAllocMaxSubhaloes = 8192;
constexpr long long kNoAllocMaxRecords = 3 * kNoAllocMaxParticles;
constexpr int kMaxWalkRanges = 256; // walk ranges (one per SM) the counters cover

constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// Byte size of every carve-out, in carving order.
constexpr size_t kN1 = (size_t)kNoAllocMaxParticles + 1;
constexpr size_t kS1 = (size_t)kNoAllocMaxSubhaloes + 1;
constexpr size_t kTable = (size_t)256 * ((kNoAllocMaxParticles + kRadixTile - 1) / kRadixTile);
constexpr size_t kScanScr = 2 * (kN1 + kTable) / 64 + 4096; // > scan_scratch_elems<int> of any scan here
constexpr size_t kCells = (size_t)kNoAllocMaxRecords / 2 + 1; // cells of a tree within the record limit
constexpr size_t kScratchBytes =
  al(sizeof(long long) * kS1) +              // offsets
  2 * al(sizeof(float4) * kN1) +             // pm, vu
  al(kN1) +                                  // ty
  7 * al(sizeof(int) * kN1) +                // seg_of, ord, ord_tmp, sp, tgt + Ep, pot (4 bytes each)
  al(kN1) +                                  // bound flags
  26 * al(sizeof(int) * kS1) +               // per-subhalo ints
  al(sizeof(float) * 6 * kS1) +              // mass upscale factors
  al(sizeof(float) * 8 * kS1) +              // old frame, mbound
  al(sizeof(unsigned) * 7 * kS1) +           // bounding boxes, largest source masses
  al(sizeof(double) * 4 * kS1) +             // root cubes
  al(sizeof(float) * 12 * kS1) +             // fast key-descent constants
  al(sizeof(double) * 7 * kS1) +             // frame sums
  al(sizeof(double) * 7 * (kN1 / 4096 + kComSmall / 256 + 2)) + // per-block frame sums (com_part_blocks)
  2 * al(sizeof(unsigned long long) * kN1) + // key, key_alt
  6 * al(sizeof(uint32_t) * kN1) +           // val, val_alt, k32, k32_alt, perm, perm_alt
  al(sizeof(int) * kN1) + al(sizeof(int)) +  // key fallback list and its count
  4 * al(sizeof(int) * kN1) +                // cnt, X, flags, F
  al(sizeof(float4) * kNoAllocMaxRecords) +  // tree slots
  al(sizeof(int) * kTable) +                 // radix table
  al(sizeof(int) * kScanScr) +               // scan scratch
  al(sizeof(int) * kCells) +                 // per-level cell lists
  al(sizeof(int) * 2 * kLevels) +            // cells per level, list cursors
  al(sizeof(unsigned long long) * kWalkCounters) + // walk counters
  al(sizeof(float) * 12 * kS1) +             // working copies of the in/out frames
  al(sizeof(unsigned) * kMaxWalkRanges);     // per-SM walk chunk counters

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch on the current device.
int scratch_address(unsigned char **out)
{
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
  {
    cudaGetLastError();
    return HBTG_ERR_CUDA;
  }
  *out = static_cast<unsigned char *>(p);
  return HBTG_OK;
}

struct Carver
{
  unsigned char *base;
  size_t used = 0;
  bool overflow = false;
  template <typename T>
  T *take(size_t count)
  {
    const size_t bytes = al(sizeof(T) * std::max<size_t>(count, 1));
    if (used + bytes > kScratchBytes)
    {
      overflow = true;
      return nullptr;
    }
    T *p = reinterpret_cast<T *>(base + used);
    used += bytes;
    return p;
  }
};

struct Fail
{
  int code;
};

inline void ck(cudaError_t e)
{
  if (e != cudaSuccess)
    throw Fail{HBTG_ERR_CUDA};
}

inline unsigned nblocks(long long n, int threads)
{
  return (unsigned)std::max<long long>(1, (n + threads - 1) / threads);
}

// Memory policy of the no-allocation path: every buffer is a fixed carve-out
// of the static reserve; a request beyond its size fails the call.
struct StaticMem
{
  int *scan_scr = nullptr, *table = nullptr;
  int *cells = nullptr, *lvl = nullptr;
  float4 *slots = nullptr;

  void check(cudaError_t e) { ck(e); }
  int *scan_scratch(long long n)
  {
    if (scan_scratch_elems<int>(n) > kScanScr)
      throw Fail{HBTG_ERR_NOMEM};
    return scan_scr;
  }
  int *radix_table(long long n)
  {
    if (radix_table_elems(std::max<long long>(n, 1)) > kTable)
      throw Fail{HBTG_ERR_NOMEM};
    return table;
  }
  int *radix_scan_scratch(long long n) { return scan_scratch(radix_table_elems(std::max<long long>(n, 1)) + 1); }
  int *cell_list(long long n)
  {
    if (n > (long long)kCells)
      throw Fail{HBTG_ERR_NOMEM};
    return cells;
  }
  int *level_counts() { return lvl; }
  float4 *tree_slots(long long n)
  {
    if (n > kNoAllocMaxRecords)
      throw Fail{HBTG_ERR_NOMEM}; // tree larger than the reserve
    return slots;
  }
  void mark(int) {}
};

KParams noalloc_kparams(const hbtg_params *p)
{
  KParams K;
  K.box = (float)p->box_size;
  K.half = (float)((double)K.box / 2.);
  K.periodic = p->periodic != 0;
  K.soft = (float)p->softening;
  K.h = (float)(2.8 * (double)K.soft);
  K.h_inv = (float)(1.0 / (2.8 * (double)K.soft));
  K.res = (float)p->tree_node_resolution;
  const float theta = (float)p->open_angle;
  K.theta2 = theta * theta;
  K.bmp = (float)p->bound_mass_precision;
  K.min_part = (int)p->min_num_part;
  K.min_tracer = (int)p->min_num_tracer;
  K.tracer_mask = p->tracer_type_mask;
  K.dm_only = p->dm_only != 0;
  K.thermal = p->thermal != 0;
  K.G_over_a = (float)((double)(float)p->G / (double)(float)p->scale_factor);
  K.a = (float)p->scale_factor;
  K.hz = (float)p->hubble;
  K.max_iter = p->max_iterations > 0 ? p->max_iterations : 1000000;
  K.core_min = p->sub_core_size_min;
  K.core_factor = (float)p->sub_core_size_factor;
  K.max_sample = (int)std::min<int64_t>(p->max_sample_size, 1 << 30);
  K.nosub_mask = p->no_subsample_mask;
  K.upscale_per_type = p->upscale_per_type != 0;
  K.refine = p->refine_most_bound != 0;
  K.refine_frac = (float)p->refine_fraction;
  K.count_interactions = 0;
  return K;
}

int noalloc_call(const hbtg_params *p, hbtg_batch *b, cudaStream_t st)
{
  if (!p || !b || b->n_sub < 0 || (b->n_sub > 0 && !b->offsets))
    return HBTG_ERR_INVALID;
  if (p->max_sample_size > 0 && !p->prepared_subsample)
    return HBTG_ERR_UNSUPPORTED;
  if (!(p->softening > 0) || !(p->open_angle > 0) || !(p->box_size > 0))
    return HBTG_ERR_INVALID;
  const long long S = b->n_sub;
  if (S == 0)
    return HBTG_OK;
  if (S > kNoAllocMaxSubhaloes || b->offsets[0] != 0)
    return HBTG_ERR_INVALID;
  for (long long s = 0; s < S; s++)
    if (b->offsets[s + 1] < b->offsets[s])
      return HBTG_ERR_INVALID;
  const long long N = b->offsets[S];
  if (N > kNoAllocMaxParticles)
    return HBTG_ERR_INVALID; // larger than the static reserve
  if (N > 0 && (!b->pos || !b->vel || !b->mass || !b->id || !b->order))
    return HBTG_ERR_INVALID;
  if (!b->ref_pos || !b->ref_vel || !b->mostbound_pos || !b->mostbound_vel || !b->most_bound_id || !b->nbound ||
      !b->mbound || !b->tracer_index || !b->iterations || !b->status)
    return HBTG_ERR_INVALID;

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess)
    return HBTG_ERR_NO_DEVICE;
  unsigned char *base = nullptr;
  int rc = scratch_address(&base);
  if (rc != HBTG_OK)
    return rc;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
  {
    cudaGetLastError();
    return HBTG_ERR_CUDA;
  }

  StaticMem mem;
  IterationDriver<StaticMem> R(mem, st);
  R.K = noalloc_kparams(p);
  R.S = (int)S;
  R.sm_count = std::min(sms, kMaxWalkRanges);
  int bits = 0;
  while ((1LL << bits) < S)
    bits++;
  R.seg_bits = bits;
  Carver c{base};
  DevState &D = R.D;
  D.S = (int)S;
  D.N = N;
  long long *off = c.take<long long>(kS1);
  D.off = off;
  D.pm = c.take<float4>(kN1);
  D.vu = c.take<float4>(kN1);
  D.ty = c.take<uint8_t>(kN1);
  D.seg_of = c.take<int>(kN1);
  D.ord = c.take<int>(kN1);
  D.ord_tmp = c.take<int>(kN1);
  D.sp = c.take<int>(kN1);
  D.tgt = c.take<int>(kN1);
  D.bnd = c.take<uint8_t>(kN1);
  D.Ep = c.take<float>(kN1);
  D.pot = c.take<float>(kN1);
  int **ints[] = {&D.n_s, &D.nbound, &D.nlast, &D.state, &D.corr, &D.iter, &D.wrap, &D.tracers, &D.nb_new,
                  &D.src_begin, &D.src_cnt, &D.src_off, &D.tgt_cnt, &D.chunk_cnt, &D.chunk_off, &D.part_cnt,
                  &D.part_off, &D.tail_cnt, &D.tail_off, &D.fin_cnt, &D.fin_off, &D.sp_cnt, &D.sp_off, &D.sp_len, &D.nunsample, &D.ngrav};
  for (int **pp : ints)
    *pp = c.take<int>(kS1);
  float *subf = c.take<float>(8 * kS1);
  D.old_pos = subf;
  D.old_vel = subf + 3 * kS1;
  D.mbound = subf + 6 * kS1;
  unsigned *bb = c.take<unsigned>(7 * kS1);
  D.bb_lo = bb;
  D.bb_hi = bb ? bb + 3 * kS1 : nullptr;
  D.factor = c.take<float>(6 * kS1);
  D.root = c.take<double>(4 * kS1);
  D.keyp = c.take<float>(12 * kS1);
  D.com = c.take<double>(7 * kS1);
  D.com_part = c.take<double>(7 * (size_t)com_part_blocks((long long)kN1));
  D.key = c.take<unsigned long long>(kN1);
  D.key_alt = c.take<unsigned long long>(kN1);
  D.val = c.take<uint32_t>(kN1);
  D.val_alt = c.take<uint32_t>(kN1);
  D.k32 = c.take<uint32_t>(kN1);
  D.k32_alt = c.take<uint32_t>(kN1);
  D.perm = c.take<uint32_t>(kN1);
  D.perm_alt = c.take<uint32_t>(kN1);
  D.fb_list = c.take<int>(kN1);
  D.fb_count = c.take<int>(1);
  D.cnt = c.take<int>(kN1);
  D.X = c.take<int>(kN1);
  D.flags = c.take<int>(kN1);
  D.F = c.take<int>(kN1);
  mem.slots = c.take<float4>(kNoAllocMaxRecords);
  D.nodes = mem.slots;
  mem.table = c.take<int>(kTable);
  mem.scan_scr = c.take<int>(kScanScr);
  mem.cells = c.take<int>(kCells);
  mem.lvl = c.take<int>(2 * kLevels);
  D.interactions = c.take<unsigned long long>(kWalkCounters);
  float *frames = c.take<float>(12 * kS1);
  D.walk_ctr = c.take<unsigned>(kMaxWalkRanges);
  if (c.overflow || (size_t)scan_scratch_elems<int>(kN1 + kTable) > kScanScr)
    return HBTG_ERR_NOMEM; // layout does not fit the reserve (cannot happen with the constants above)
  // the iteration moves the frames: it works on copies in the reserve
  D.ref_pos = frames;
  D.ref_vel = frames + 3 * kS1;
  D.mb_pos = frames + 6 * kS1;
  D.mb_vel = frames + 9 * kS1;
  D.mb_id = reinterpret_cast<long long *>(b->most_bound_id);
  D.id = reinterpret_cast<const long long *>(b->id);
  const size_t fbytes = sizeof(float) * 3 * (size_t)S;

  try
  {
    ck(cudaMemcpyAsync(off, b->offsets, sizeof(long long) * (S + 1), cudaMemcpyHostToDevice, st));
    ck(cudaMemcpyAsync(D.ref_pos, b->ref_pos, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemcpyAsync(D.ref_vel, b->ref_vel, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemcpyAsync(D.mb_pos, b->mostbound_pos, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemcpyAsync(D.mb_vel, b->mostbound_vel, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemsetAsync(D.interactions, 0, sizeof(unsigned long long) * kWalkCounters, st));
    if (N > 0)
      k_repack<<<nblocks(N, 256), 256, 0, st>>>(D, R.K, b->pos, b->vel, b->mass, b->u, b->type);
    k_init_subs<<<nblocks(S, 256), 256, 0, st>>>(D, R.K);
    R.check();
    R.run();
    OutPtrs O;
    O.order = reinterpret_cast<long long *>(b->order);
    O.nbound = reinterpret_cast<long long *>(b->nbound);
    O.nbound_type = reinterpret_cast<long long *>(b->nbound_type);
    O.tracer_index = reinterpret_cast<long long *>(b->tracer_index);
    O.most_bound_id = reinterpret_cast<long long *>(b->most_bound_id);
    O.mbound = b->mbound;
    O.mbound_type = b->mbound_type;
    O.kinematics = b->kinematics;
    O.core = b->core;
    O.energy = b->energy;
    O.potential = b->potential;
    O.iterations = b->iterations;
    O.status = b->status;
    R.epilogue(O);
    ck(cudaMemcpyAsync(b->ref_pos, D.ref_pos, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemcpyAsync(b->ref_vel, D.ref_vel, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemcpyAsync(b->mostbound_pos, D.mb_pos, fbytes, cudaMemcpyDefault, st));
    ck(cudaMemcpyAsync(b->mostbound_vel, D.mb_vel, fbytes, cudaMemcpyDefault, st));
    ck(cudaStreamSynchronize(st));
  }
  catch (Fail &f)
  {
    cudaGetLastError();
    return f.code;
  }
  return HBTG_OK;
}

} // namespace

extern "C" int hbtg_unbind_batch_noalloc(const hbtg_params *params, hbtg_batch *batch, void *cuda_stream)
{
  return noalloc_call(params, batch, static_cast<cudaStream_t>(cuda_stream));
}
