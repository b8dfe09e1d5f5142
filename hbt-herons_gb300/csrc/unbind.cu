// unbind.cu - host orchestration and C ABI of libhbtg.so (include/hbt_unbind_gpu.h).
//
// One call unbinds a batch of subhaloes on one GPU.  All subhaloes still
// iterating advance in lock step: each global iteration is a fixed kernel
// sequence (plan, tree build, walk, energies, partition, sorts, frame,
// control) over the packed active segments; subhaloes leave the active set
// when they converge or disrupt, exactly where Subhalo_t::Unbind breaks out of
// its loop (src/subhalo_unbind.cpp:555-758).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/hbt_unbind_gpu.h"

// csrc/mlp.cu: the proposer's inference writing the proposal byte directly
int hbtg_mlp_propose(const float *weights, const float *features, uint8_t *prop, float trust, float leave_out,
                     int64_t n, cudaStream_t stream);
#include "common.cuh"
#include "driver.cuh"
#include "props.cuh"
#include "reassign.cuh"
#include "kernels.cuh"
#include "primitives.cuh"
#include "warm.cuh"

using namespace hbtg;

namespace hbtg
{
namespace
{
__global__ void k_pot_repack(DevState D, const float *__restrict__ pos, const float *__restrict__ mass)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += (long long)gridDim.x * blockDim.x)
  {
    D.pm[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], mass[i]);
    D.vu[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    D.ty[i] = 1;
    D.seg_of[i] = 0;
    D.ord[i] = (int)i;
  }
}

// One "subhalo" whose every particle is a source; the walk takes the
// requested particles as targets (tgt list) with their self terms.
__global__ void k_pot_plan(DevState D, int n_tgt, int phase)
{
  if (blockIdx.x != 0 || threadIdx.x != 0)
    return;
  const int n = (int)D.N;
  if (phase == 0)
  {
    D.state[0] = kActive;
    D.iter[0] = 1;
    D.corr[0] = 0; // the build decides the periodic wrap as a first iteration does
    D.wrap[0] = 0;
    D.ngrav[0] = 0;
    D.src_begin[0] = 0;
    D.src_cnt[0] = n;
    D.src_cnt[1] = 0;
    D.tgt_cnt[0] = n_tgt;
    D.chunk_cnt[0] = (n_tgt + kWarp - 1) / kWarp;
    D.chunk_cnt[1] = 0;
    D.sp_len[0] = n;
    for (int d = 0; d < 3; d++)
    {
      D.bb_lo[d] = 0xffffffffu;
      D.bb_hi[d] = 0u;
    }
    for (int t = 0; t < 6; t++)
      D.factor[t] = 1.f;
  }
  else
  {
    D.corr[0] = 1;
    D.self_cnt[0] = n_tgt;
  }
}

__global__ void k_pot_targets(DevState D, const long long *__restrict__ tgt, int n_tgt, int *__restrict__ bad)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tgt)
    return;
  const long long i = tgt[t];
  if (i < 0 || i >= D.N)
  {
    atomicExch(bad, 1);
    D.tgt[t] = 0;
    return;
  }
  D.tgt[t] = (int)i;
}

__global__ void k_pot_out(DevState D, int n_tgt, float *__restrict__ out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_tgt)
    out[t] = D.pot[D.tgt[t]];
}

} // namespace
} // namespace hbtg

namespace
{

struct CudaError
{
  cudaError_t err;
};
struct NoMem
{
};

#define HBTG_CUDA(call)                                                                                                \
  do                                                                                                                   \
  {                                                                                                                    \
    cudaError_t e_ = (call);                                                                                           \
    if (e_ != cudaSuccess)                                                                                             \
    {                                                                                                                  \
      if (e_ == cudaErrorMemoryAllocation)                                                                             \
        throw NoMem{};                                                                                                 \
      throw CudaError{e_};                                                                                             \
    }                                                                                                                  \
  } while (0)

// Grow-only device buffers, one per slot.
enum Slot
{
  S_POS, S_VEL, S_MASS, S_U, S_ID, S_TYPE, S_OFF,
  S_REFP, S_REFV, S_MBP, S_MBV, S_MBID,
  S_ORDER, S_NB, S_MB, S_NBT, S_MBT, S_TI, S_KIN, S_CORE, S_EN, S_POT, S_ITER, S_STAT,
  S_PM, S_VU, S_TY, S_SEG, S_ORD, S_ORDT, S_EP, S_PHI,
  S_SUBI, S_SUBF, S_BB, S_ROOT, S_KEYP, S_COM,
  S_KEY, S_KEYA, S_VAL, S_VALA, S_K32, S_K32A, S_CNT, S_X, S_FLAGS, S_F,
  S_NODES, S_TABLE, S_SCRATCH, S_CELLS, S_LVL, S_COUNTER, S_PERM, S_PERMA, S_FBL, S_FBC, S_TMASS, S_COMP, S_SP, S_TGT, S_BND, S_FACTOR,
  S_WARMI, S_REF0, S_RMAX, S_MMAX, S_WBB, S_HIST, S_TAB, S_FEAT, S_PROP, S_PNB, S_PEN, S_MODEL, S_NB1,
  S_POTI, S_WCTR, S_FRAMEW, S_TUNE,
  S_PR_OFF, S_PR_CNT, S_PR_FIN, S_PR_RR, S_PR_MM, S_PR_K, S_PR_V, S_PR_KA, S_PR_VA, S_PR_MC, S_PR_VK, S_PR_SO,
  S_PR_SH, S_PR_SCR, S_PR_POS, S_PR_MASS, S_PR_ORD, S_PR_NB, S_PR_MBND, S_PR_MBP, S_PR_OUTF, S_PR_OUTI, S_PR_OUTL,
  S_RE_OFF, S_RE_SG, S_RE_GP, S_RE_FL, S_RE_RK, S_RE_TG, S_RE_TS, S_RE_GO, S_RE_POS, S_RE_TY, S_RE_DEST,
  S_NUM
};

struct Pool
{
  void *ptr[S_NUM] = {};
  size_t cap[S_NUM] = {};
  void *get(int slot, size_t bytes)
  {
    if (bytes == 0)
      bytes = 16;
    if (cap[slot] >= bytes)
      return ptr[slot];
    if (ptr[slot])
      cudaFree(ptr[slot]);
    ptr[slot] = nullptr;
    cap[slot] = 0;
    const size_t want = bytes + bytes / 4;
    void *p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess)
    {
      cudaGetLastError();
      throw NoMem{};
    }
    ptr[slot] = p;
    cap[slot] = want;
    return p;
  }
  template <typename T>
  T *get(int slot, size_t count)
  {
    return static_cast<T *>(get(slot, count * sizeof(T)));
  }
  void release()
  {
    for (int i = 0; i < S_NUM; i++)
      if (ptr[i])
        cudaFree(ptr[i]);
    std::memset(ptr, 0, sizeof(ptr));
    std::memset(cap, 0, sizeof(cap));
  }
};

inline unsigned blocks_for(long long n, int threads)
{
  long long b = (n + threads - 1) / threads;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, 0x7fffffffLL));
}

} // namespace

struct hbtg_handle
{
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;              // uploads that only the epilogue needs (host-pointer calls)
  cudaStream_t side2 = nullptr;             // a second copy stream: velocities up, energies down
  cudaEvent_t copy_events[7] = {};          // host-pointer calls: copy phases and the side streams
  cudaEvent_t epilogue_wait = nullptr;      // set for one call: the epilogue waits for this event
  Pool pool;
  hbtg_stats stats{};
  bool count_interactions = false;
  std::vector<cudaEvent_t> walk_events;
  std::vector<cudaEvent_t> phase_events; // phase boundaries of the last call, in order
  // learned warm start (hbtg_set_model)
  bool has_model = false;
  float threshold = 0.5f;
  float exclude_below = 0.f;
  long long min_particles = 0;
  int first_test = 1;
  // launch settings (hbtg_set_tuning, hbtg_autotune)
  hbtg_tuning tune{kRadixBlockMax, 0, 8, 0.0};
  // state of the last unbinding call, for hbtg_trace_labels_device
  int last_S = 0;
  long long last_N = 0;
  int *last_ord = nullptr, *last_nlast = nullptr, *last_state = nullptr, *last_seg = nullptr, *last_nb1 = nullptr;
  long long *last_off = nullptr;
};

namespace
{

KParams make_kparams(const hbtg_params *p, bool count)
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
  const float G = (float)p->G, a = (float)p->scale_factor;
  K.G_over_a = (float)((double)G / (double)a);
  K.a = a;
  K.hz = (float)p->hubble;
  K.max_iter = p->max_iterations > 0 ? p->max_iterations : 1000000;
  K.core_min = p->sub_core_size_min;
  K.core_factor = (float)p->sub_core_size_factor;
  K.max_sample = (int)std::min<int64_t>(p->max_sample_size, 1 << 30);
  K.nosub_mask = p->no_subsample_mask;
  K.upscale_per_type = p->upscale_per_type != 0;
  K.refine = p->refine_most_bound != 0;
  K.refine_frac = (float)p->refine_fraction;
  K.count_interactions = count ? 1 : 0;
  return K;
}

// What a warm-started call adds to a plain one (device pointers).
struct WarmArgs
{
  const uint8_t *proposal = nullptr; // explicit proposal, or null to run the handle's model
  const long long *nb_prev = nullptr;
  const float *e_prev = nullptr;
  long long min_n = 0;
  int first_test = 1;             // 0: uncertain particles join the set untested
  float *features_only = nullptr; // compute the features into this [6N] array and stop
};

int validate(const hbtg_params *p, const hbtg_batch *b, long long &N)
{
  if (!p || !b || b->n_sub < 0 || (b->n_sub > 0 && !b->offsets))
    return HBTG_ERR_INVALID;
  if (p->max_sample_size > 0 && !p->prepared_subsample)
    return HBTG_ERR_UNSUPPORTED; // the caller must run PrepareParticlesForSubsampling first
  if (!(p->softening > 0) || !(p->open_angle > 0) || !(p->box_size > 0))
    return HBTG_ERR_INVALID;
  if (b->n_sub > 0 && b->offsets[0] != 0)
    return HBTG_ERR_INVALID;
  for (int64_t s = 0; s < b->n_sub; s++)
    if (b->offsets[s + 1] < b->offsets[s])
      return HBTG_ERR_INVALID;
  N = b->n_sub > 0 ? b->offsets[b->n_sub] : 0;
  if (N >= (1LL << 30) || b->n_sub >= (1LL << 30))
    return HBTG_ERR_INVALID;
  if (N > 0 && (!b->pos || !b->vel || !b->mass || !b->id || !b->order))
    return HBTG_ERR_INVALID;
  if (b->n_sub > 0 && (!b->ref_pos || !b->ref_vel || !b->mostbound_pos || !b->mostbound_vel ||
                       !b->most_bound_id || !b->nbound || !b->mbound || !b->tracer_index || !b->iterations ||
                       !b->status))
    return HBTG_ERR_INVALID;
  return HBTG_OK;
}

// Reads one int from device memory (synchronises the stream).
int read_int(const int *d, cudaStream_t st)
{
  int h = 0;
  HBTG_CUDA(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
  HBTG_CUDA(cudaStreamSynchronize(st));
  return h;
}

// Memory policy of the pooled entry points: grow-only buffers owned by the
// handle, CUDA events at phase boundaries for the per-phase times.
struct PoolMem
{
  hbtg_handle *H;
  cudaStream_t st;
  std::vector<int> mark_phase;

  void check(cudaError_t e) { HBTG_CUDA(e); }
  int *scan_scratch(long long n)
  {
    return H->pool.get<int>(S_SCRATCH, scan_scratch_elems<int>(std::max<long long>(n, 256LL * 4096)));
  }
  int *radix_table(long long n) { return H->pool.get<int>(S_TABLE, radix_table_elems(std::max<long long>(n, 1))); }
  int *radix_scan_scratch(long long n)
  {
    return H->pool.get<int>(S_SCRATCH, scan_scratch_elems<int>(
                                         std::max<long long>(radix_table_elems(std::max<long long>(n, 1)) + 1,
                                                             256LL * 4096)));
  }
  int *cell_list(long long cells) { return H->pool.get<int>(S_CELLS, (size_t)std::max<long long>(cells, 1)); }
  int *level_counts() { return H->pool.get<int>(S_LVL, 2 * kLevels); }
  float4 *tree_slots(long long slots)
  {
    if (slots >= (1LL << 31) - 64)
      throw NoMem{};
    return H->pool.get<float4>(S_NODES, (size_t)slots);
  }
  void mark(int phase)
  {
    const size_t k = mark_phase.size();
    if (k >= H->phase_events.size())
    {
      cudaEvent_t e;
      HBTG_CUDA(cudaEventCreate(&e));
      H->phase_events.push_back(e);
    }
    HBTG_CUDA(cudaEventRecord(H->phase_events[k], st));
    mark_phase.push_back(phase);
  }
  // Per-phase totals (ms): 0 plan, 1 walk, 2 tree, 3 partition, 4 frame, 5 final, 6 warm-start proposal.
  void phase_totals(double *ms)
  {
    for (size_t k = 1; k < mark_phase.size(); k++)
    {
      float t = 0.f;
      HBTG_CUDA(cudaEventElapsedTime(&t, H->phase_events[k - 1], H->phase_events[k]));
      if (mark_phase[k] >= 0)
        ms[mark_phase[k]] += t;
    }
  }
};

// The batch with every array on the device (offsets on the host).
int run_device(hbtg_handle *H, const hbtg_params *p, const hbtg_batch *b, cudaStream_t st,
               const WarmArgs *wa = nullptr)
{
  long long N = 0;
  int rc = validate(p, b, N);
  if (rc != HBTG_OK)
    return rc;
  if (wa && p->max_sample_size > 0)
    return HBTG_ERR_UNSUPPORTED; // the warm start does not combine with potential subsampling
  if (wa && !wa->proposal && !wa->features_only && !H->has_model)
    return HBTG_ERR_INVALID; // no model set on the handle
  const int S = (int)b->n_sub;
  H->stats = hbtg_stats{};
  H->stats.n_sub = S;
  H->stats.n_particles = N;
  if (S == 0)
    return HBTG_OK;
  cudaEvent_t t0, t1;
  HBTG_CUDA(cudaEventCreate(&t0));
  HBTG_CUDA(cudaEventCreate(&t1));
  HBTG_CUDA(cudaEventRecord(t0, st));

  PoolMem mem{H, st, {}};
  IterationDriver<PoolMem> R(mem, st);
  R.K = make_kparams(p, H->count_interactions);
  R.S = S;
  R.sm_count = H->sm_count;
  R.block_sort_max = H->tune.block_sort_max;
  R.walk_ranged_min = H->tune.walk_ranged_min;
  R.moments_blocks_per_sm = H->tune.moments_blocks_per_sm;
  int bits = 0;
  while ((1LL << bits) < S)
    bits++;
  R.seg_bits = bits;
  Pool &P = H->pool;
  DevState &D = R.D;
  D.S = S;
  D.N = N;
  long long *off = P.get<long long>(S_OFF, S + 1);
  HBTG_CUDA(cudaMemcpyAsync(off, b->offsets, sizeof(long long) * (S + 1), cudaMemcpyHostToDevice, st));
  D.off = off;
  const size_t n1 = (size_t)std::max<long long>(N, 1);
  D.pm = P.get<float4>(S_PM, n1);
  D.vu = P.get<float4>(S_VU, n1);
  D.ty = P.get<uint8_t>(S_TY, n1);
  D.seg_of = P.get<int>(S_SEG, n1);
  D.ord = P.get<int>(S_ORD, n1);
  D.ord_tmp = P.get<int>(S_ORDT, n1);
  D.sp = P.get<int>(S_SP, n1);
  D.tgt = P.get<int>(S_TGT, n1);
  D.bnd = P.get<uint8_t>(S_BND, n1);
  D.Ep = P.get<float>(S_EP, n1);
  D.pot = P.get<float>(S_PHI, n1);
  D.id = reinterpret_cast<const long long *>(b->id);
  int *subi = P.get<int>(S_SUBI, (size_t)(S + 1) * 28);
  int q = 0;
  auto nexti = [&]() { return subi + (size_t)(S + 1) * (q++); };
  D.n_s = nexti(); D.nbound = nexti(); D.nlast = nexti(); D.state = nexti(); D.corr = nexti(); D.iter = nexti();
  D.wrap = nexti(); D.tracers = nexti(); D.nb_new = nexti(); D.src_begin = nexti(); D.src_cnt = nexti();
  D.src_off = nexti(); D.tgt_cnt = nexti(); D.chunk_cnt = nexti(); D.chunk_off = nexti(); D.part_cnt = nexti();
  D.part_off = nexti(); D.tail_cnt = nexti(); D.tail_off = nexti(); D.fin_cnt = nexti(); D.fin_off = nexti();
  D.sp_cnt = nexti(); D.sp_off = nexti(); D.sp_len = nexti(); D.nunsample = nexti(); D.ngrav = nexti();
  D.nb1 = P.get<int>(S_NB1, (size_t)S + 1);
  D.walk_ctr = P.get<unsigned>(S_WCTR, (size_t)std::max(H->sm_count, 1));
  D.factor = P.get<float>(S_FACTOR, (size_t)S * 6);
  float *subf = P.get<float>(S_SUBF, (size_t)S * 8);
  D.old_pos = subf;
  D.old_vel = subf + 3 * (size_t)S;
  D.mbound = subf + 6 * (size_t)S;
  // The iteration moves the in/out frames: it works on copies and writes the
  // caller's arrays back after the epilogue, so a call that fails part-way
  // (HBTG_ERR_NOMEM when the pool cannot grow) leaves them as they were.
  float *framew = P.get<float>(S_FRAMEW, (size_t)S * 12);
  const size_t fbytes = sizeof(float) * 3 * (size_t)S;
  D.ref_pos = framew;
  D.ref_vel = framew + 3 * (size_t)S;
  D.mb_pos = framew + 6 * (size_t)S;
  D.mb_vel = framew + 9 * (size_t)S;
  HBTG_CUDA(cudaMemcpyAsync(D.ref_pos, b->ref_pos, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaMemcpyAsync(D.ref_vel, b->ref_vel, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaMemcpyAsync(D.mb_pos, b->mostbound_pos, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaMemcpyAsync(D.mb_vel, b->mostbound_vel, fbytes, cudaMemcpyDefault, st));
  D.mb_id = reinterpret_cast<long long *>(b->most_bound_id);
  unsigned *bb = P.get<unsigned>(S_BB, (size_t)S * 7);
  D.bb_lo = bb;
  D.bb_hi = bb + 3 * (size_t)S;
  D.root = P.get<double>(S_ROOT, (size_t)S * 4);
  D.keyp = P.get<float>(S_KEYP, (size_t)S * 12);
  D.com = P.get<double>(S_COM, (size_t)S * 7);
  D.com_part = P.get<double>(S_COMP, 7 * (size_t)com_part_blocks(N));
  D.key = P.get<unsigned long long>(S_KEY, n1);
  D.key_alt = P.get<unsigned long long>(S_KEYA, n1);
  D.val = P.get<uint32_t>(S_VAL, n1);
  D.val_alt = P.get<uint32_t>(S_VALA, n1);
  D.k32 = P.get<uint32_t>(S_K32, n1);
  D.k32_alt = P.get<uint32_t>(S_K32A, n1);
  D.perm = P.get<uint32_t>(S_PERM, n1);
  D.perm_alt = P.get<uint32_t>(S_PERMA, n1);
  D.fb_list = P.get<int>(S_FBL, n1);
  D.fb_count = P.get<int>(S_FBC, 1);
  D.cnt = P.get<int>(S_CNT, n1 + 1);
  D.X = P.get<int>(S_X, n1 + 1);
  D.flags = P.get<int>(S_FLAGS, n1 + 1);
  D.F = P.get<int>(S_F, n1 + 1);
  D.nodes = P.get<float4>(S_NODES, n1 * 3);
  D.interactions = P.get<unsigned long long>(S_COUNTER, kWalkCounters);
  HBTG_CUDA(cudaMemsetAsync(D.interactions, 0, sizeof(unsigned long long) * kWalkCounters, st));

  if (N > 0)
  {
    k_repack<<<blocks_for(N, 256), 256, 0, st>>>(D, R.K, b->pos, b->vel, b->mass, b->u, b->type);
    R.launches++;
  }
  k_init_subs<<<blocks_for(S, 256), 256, 0, st>>>(D, R.K);
  R.launches++;
  R.check();
  WarmCounters wc;
  if (!wa)
    R.run();
  else
  {
    int *wi = P.get<int>(S_WARMI, (size_t)(S + 1) * 6);
    D.warm = wi;
    D.nexcl = wi + (S + 1);
    D.iter_extra = wi + 2 * (size_t)(S + 1);
    D.flag_s = wi + 3 * (size_t)(S + 1);
    D.self_cnt = wi + 4 * (size_t)(S + 1);
    D.ntest = wi + 5 * (size_t)(S + 1);
    HBTG_CUDA(cudaMemsetAsync(D.self_cnt, 0, sizeof(int) * (S + 1), st));
    D.ref0 = P.get<float>(S_REF0, (size_t)S * 6);
    WarmBufs W;
    W.nb_prev = wa->nb_prev;
    W.e_prev = wa->e_prev;
    W.rmax = P.get<unsigned>(S_RMAX, S);
    W.mmax = P.get<unsigned>(S_MMAX, 1);
    W.bb = P.get<unsigned>(S_WBB, (size_t)S * 6);
    W.hist = P.get<unsigned long long>(S_HIST, (size_t)S * kBins);
    W.tab = P.get<float>(S_TAB, (size_t)S * kTab);
    W.feat = wa->features_only;
    W.prop = wa->proposal;
    W.min_n = wa->min_n;
    W.first_test = wa->first_test;
    mem.mark(-1);
    if (wa->features_only || !wa->proposal)
    {
      if (!W.feat)
        W.feat = P.get<float>(S_FEAT, n1 * kFeat);
      compute_features(R, W);
      if (wa->features_only)
      {
        HBTG_CUDA(cudaStreamSynchronize(st));
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        H->stats.kernel_launches = R.launches;
        return HBTG_OK;
      }
      uint8_t *prop = P.get<uint8_t>(S_PROP, n1);
      if (N > 0)
      { // the network's proposal (trusted / uncertain / left out) per particle
        const int mrc = hbtg_mlp_propose(P.get<float>(S_MODEL, HBTG_MLP_PARAMS), W.feat, prop, H->threshold,
                                         H->exclude_below, N, st);
        if (mrc != HBTG_OK)
          return mrc;
        R.launches++;
        R.check();
      }
      W.prop = prop;
    }
    warm_run(R, W, wc, !wa->proposal);
    std::vector<int> warm(S);
    HBTG_CUDA(cudaMemcpyAsync(warm.data(), D.warm, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
    HBTG_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < S; s++)
    {
      wc.warm_subhaloes += warm[s] != 0;
      wc.restarts += warm[s] == 2;
    }
  }

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
  if (H->epilogue_wait)
    HBTG_CUDA(cudaStreamWaitEvent(st, H->epilogue_wait, 0));
  R.epilogue(O);
  HBTG_CUDA(cudaMemcpyAsync(b->ref_pos, D.ref_pos, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaMemcpyAsync(b->ref_vel, D.ref_vel, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaMemcpyAsync(b->mostbound_pos, D.mb_pos, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaMemcpyAsync(b->mostbound_vel, D.mb_vel, fbytes, cudaMemcpyDefault, st));
  HBTG_CUDA(cudaEventRecord(t1, st));
  HBTG_CUDA(cudaEventSynchronize(t1));
  H->last_S = S;
  H->last_N = N;
  H->last_ord = D.ord;
  H->last_nlast = D.nlast;
  H->last_state = D.state;
  H->last_seg = D.seg_of;
  H->last_off = off;
  H->last_nb1 = D.nb1;
  double phase_ms[7] = {0, 0, 0, 0, 0, 0, 0};
  mem.phase_totals(phase_ms);
  H->stats.ms_propose = phase_ms[6];
  H->stats.warm_subhaloes = wc.warm_subhaloes;
  H->stats.excluded = wc.excluded;
  H->stats.readmitted = wc.readmitted;
  H->stats.cold_restarts = wc.restarts;
  H->stats.readmit_rounds = wc.readmit_rounds;
  H->stats.ms_plan = phase_ms[0];
  H->stats.ms_walk = phase_ms[1];
  H->stats.ms_tree = phase_ms[2];
  H->stats.ms_part = phase_ms[3];
  H->stats.ms_frame = phase_ms[4];
  H->stats.ms_final = phase_ms[5];
  float ms = 0.f;
  HBTG_CUDA(cudaEventElapsedTime(&ms, t0, t1));
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  H->stats.ms_total = ms;
  H->stats.kernel_launches = R.launches;
  H->stats.walk_launches = R.walk_launches;
  H->stats.host_syncs = R.host_syncs;
  H->stats.walk_blocks_per_sm = R.walk_blocks_per_sm;
  H->stats.global_iterations = R.global_iter;
  H->stats.tree_nodes = R.tree_nodes;
  if (H->count_interactions)
  {
    unsigned long long c[kWalkCounters] = {};
    HBTG_CUDA(cudaMemcpy(c, D.interactions, sizeof(c), cudaMemcpyDeviceToHost));
    H->stats.interactions = (int64_t)c[0];
    H->stats.walk_steps = (int64_t)c[1];
    H->stats.walk_nodes = (int64_t)c[2];
    H->stats.walk_pending_batches = (int64_t)c[3];
    H->stats.walk_entries_full = (int64_t)c[4];
    H->stats.walk_entries_part = (int64_t)c[5];
    H->stats.walk_entries_near = (int64_t)c[6];
    H->stats.walk_drained = (int64_t)c[7];
    for (int q = 0; q < 8; q++)
      H->stats.walk_cycles[q] = (int64_t)c[8 + q];
  }
  // summary counters
  std::vector<long long> nb(S);
  HBTG_CUDA(cudaMemcpy(nb.data(), b->nbound, sizeof(long long) * S, cudaMemcpyDeviceToHost));
  long long tot = 0;
  for (long long v : nb)
    tot += v;
  H->stats.total_bound = tot;
  int any_max = 0;
  std::vector<int> stv(S);
  HBTG_CUDA(cudaMemcpy(stv.data(), b->status, sizeof(int) * S, cudaMemcpyDeviceToHost));
  for (int v : stv)
    any_max |= (v == HBTG_SUB_MAX_ITER);
  return any_max ? HBTG_ERR_MAX_ITER : HBTG_OK;
}

template <typename T>
T *upload(Pool &P, int slot, const T *h, size_t n, cudaStream_t st, int64_t &bytes)
{
  if (!h)
    return nullptr;
  T *d = P.get<T>(slot, std::max<size_t>(n, 1));
  if (n)
    HBTG_CUDA(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, st));
  bytes += sizeof(T) * n;
  return d;
}
template <typename T>
T *alloc_out(Pool &P, int slot, const T *h, size_t n)
{
  return h ? P.get<T>(slot, std::max<size_t>(n, 1)) : nullptr;
}
template <typename T>
void download(T *h, const T *d, size_t n, cudaStream_t st, int64_t &bytes)
{
  if (h && d && n)
  {
    HBTG_CUDA(cudaMemcpyAsync(h, d, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    bytes += sizeof(T) * n;
  }
}

int guarded(int (*fn)(void *), void *arg)
{
  try
  {
    return fn(arg);
  }
  catch (NoMem &)
  {
    cudaGetLastError();
    return HBTG_ERR_NOMEM;
  }
  catch (CudaError &e)
  {
    (void)e;
    return HBTG_ERR_CUDA;
  }
  catch (std::bad_alloc &)
  {
    return HBTG_ERR_NOMEM;
  }
  catch (...)
  {
    return HBTG_ERR_CUDA;
  }
}

struct HostCall
{
  hbtg_handle *H;
  const hbtg_params *p;
  hbtg_batch *b;
  bool learned = false;
  const hbtg_prior *prior = nullptr; // host arrays
};

int host_call(void *arg)
{
  HostCall &c = *static_cast<HostCall *>(arg);
  hbtg_handle *H = c.H;
  hbtg_batch *b = c.b;
  long long N = 0;
  int rc = validate(c.p, b, N);
  if (rc != HBTG_OK)
    return rc;
  HBTG_CUDA(cudaSetDevice(H->device));
  cudaStream_t st = H->stream;
  const size_t S = (size_t)b->n_sub;
  Pool &P = H->pool;
  int64_t h2d = 0, d2h = 0;
  hbtg_batch d = *b;
  cudaEvent_t *ev = H->copy_events;
  HBTG_CUDA(cudaEventRecord(ev[0], st));
  // the particle IDs are read only by the epilogue: their upload overlaps the iteration
  d.id = upload(P, S_ID, b->id, N, H->side, h2d);
  HBTG_CUDA(cudaEventRecord(ev[4], H->side));
  // velocities (and thermal energies) on a second stream, concurrent with the positions
  HBTG_CUDA(cudaStreamWaitEvent(H->side2, ev[0], 0));
  d.vel = upload(P, S_VEL, b->vel, 3 * N, H->side2, h2d);
  d.u = (c.p->thermal && b->u) ? upload(P, S_U, b->u, N, H->side2, h2d) : nullptr;
  HBTG_CUDA(cudaEventRecord(ev[5], H->side2));
  d.pos = upload(P, S_POS, b->pos, 3 * N, st, h2d);
  d.mass = upload(P, S_MASS, b->mass, N, st, h2d);
  d.type = (c.p->dm_only || !b->type) ? nullptr : upload(P, S_TYPE, b->type, N, st, h2d);
  d.ref_pos = upload(P, S_REFP, b->ref_pos, 3 * S, st, h2d);
  d.ref_vel = upload(P, S_REFV, b->ref_vel, 3 * S, st, h2d);
  d.mostbound_pos = upload(P, S_MBP, b->mostbound_pos, 3 * S, st, h2d);
  d.mostbound_vel = upload(P, S_MBV, b->mostbound_vel, 3 * S, st, h2d);
  d.most_bound_id = upload(P, S_MBID, b->most_bound_id, S, st, h2d);
  d.order = alloc_out(P, S_ORDER, b->order, N);
  d.nbound = alloc_out(P, S_NB, b->nbound, S);
  d.mbound = alloc_out(P, S_MB, b->mbound, S);
  d.nbound_type = alloc_out(P, S_NBT, b->nbound_type, 6 * S);
  d.mbound_type = alloc_out(P, S_MBT, b->mbound_type, 6 * S);
  d.tracer_index = alloc_out(P, S_TI, b->tracer_index, S);
  d.kinematics = alloc_out(P, S_KIN, b->kinematics, 5 * S);
  d.core = alloc_out(P, S_CORE, b->core, 8 * S);
  d.energy = alloc_out(P, S_EN, b->energy, N);
  d.potential = alloc_out(P, S_POT, b->potential, N);
  d.iterations = alloc_out(P, S_ITER, b->iterations, S);
  d.status = alloc_out(P, S_STAT, b->status, S);
  WarmArgs wa;
  if (c.learned)
  {
    wa.min_n = H->min_particles;
    wa.first_test = H->first_test;
    if (c.prior && c.prior->nbound_prev)
    {
      wa.nb_prev = reinterpret_cast<const long long *>(upload(P, S_PNB, c.prior->nbound_prev, S, st, h2d));
      if (c.prior->energy_prev)
        wa.e_prev = upload(P, S_PEN, c.prior->energy_prev, N, st, h2d);
    }
  }
  HBTG_CUDA(cudaStreamWaitEvent(st, ev[5], 0));
  HBTG_CUDA(cudaEventRecord(ev[1], st));
  H->epilogue_wait = ev[4];
  rc = run_device(H, c.p, &d, st, c.learned ? &wa : nullptr);
  H->epilogue_wait = nullptr;
  if (rc != HBTG_OK && rc != HBTG_ERR_MAX_ITER)
  {
    cudaStreamSynchronize(H->side);
    cudaStreamSynchronize(H->side2);
    return rc;
  }
  HBTG_CUDA(cudaEventRecord(ev[2], st));
  // the per-particle energies on the second stream, concurrent with the order
  HBTG_CUDA(cudaStreamWaitEvent(H->side2, ev[2], 0));
  download(b->energy, d.energy, N, H->side2, d2h);
  download(b->potential, d.potential, N, H->side2, d2h);
  HBTG_CUDA(cudaEventRecord(ev[6], H->side2));
  download(b->order, d.order, N, st, d2h);
  download(b->nbound, d.nbound, S, st, d2h);
  download(b->mbound, d.mbound, S, st, d2h);
  download(b->nbound_type, d.nbound_type, 6 * S, st, d2h);
  download(b->mbound_type, d.mbound_type, 6 * S, st, d2h);
  download(b->tracer_index, d.tracer_index, S, st, d2h);
  download(b->kinematics, d.kinematics, 5 * S, st, d2h);
  download(b->core, d.core, 8 * S, st, d2h);
  download(b->iterations, d.iterations, S, st, d2h);
  download(b->status, d.status, S, st, d2h);
  download(b->ref_pos, d.ref_pos, 3 * S, st, d2h);
  download(b->ref_vel, d.ref_vel, 3 * S, st, d2h);
  download(b->mostbound_pos, d.mostbound_pos, 3 * S, st, d2h);
  download(b->mostbound_vel, d.mostbound_vel, 3 * S, st, d2h);
  download(b->most_bound_id, d.most_bound_id, S, st, d2h);
  HBTG_CUDA(cudaStreamWaitEvent(st, ev[6], 0));
  HBTG_CUDA(cudaEventRecord(ev[3], st));
  HBTG_CUDA(cudaStreamSynchronize(st));
  H->stats.h2d_bytes = h2d;
  H->stats.d2h_bytes = d2h;
  float t_up = 0.f, t_down = 0.f;
  HBTG_CUDA(cudaEventElapsedTime(&t_up, ev[0], ev[1]));
  HBTG_CUDA(cudaEventElapsedTime(&t_down, ev[2], ev[3]));
  H->stats.ms_h2d = t_up;
  H->stats.ms_d2h = t_down;
  return rc;
}

// ---------------------------------------------------------------------------
// Tree potential of one particle set (GravityTree_t::Build + EvaluatePotential)
// ---------------------------------------------------------------------------
struct PotCall
{
  hbtg_handle *H;
  const hbtg_params *p;
  long long ns, nt;
  const float *pos, *mass;
  const long long *tgt;
  float *out;
  cudaStream_t st;
};

int pot_call(void *arg)
{
  PotCall &c = *static_cast<PotCall *>(arg);
  hbtg_handle *H = c.H;
  HBTG_CUDA(cudaSetDevice(H->device));
  cudaStream_t st = c.st;
  Pool &P = H->pool;
  PoolMem mem{H, st, {}};
  IterationDriver<PoolMem> R(mem, st);
  R.K = make_kparams(c.p, false);
  R.S = 1;
  R.seg_bits = 0;
  R.sm_count = H->sm_count;
  DevState &D = R.D;
  D.S = 1;
  D.N = c.ns;
  const size_t n1 = (size_t)c.ns;
  long long *off = P.get<long long>(S_OFF, 2);
  const long long hoff[2] = {0, c.ns};
  HBTG_CUDA(cudaMemcpyAsync(off, hoff, sizeof(hoff), cudaMemcpyHostToDevice, st));
  D.off = off;
  D.pm = P.get<float4>(S_PM, n1);
  D.vu = P.get<float4>(S_VU, n1);
  D.ty = P.get<uint8_t>(S_TY, n1);
  D.seg_of = P.get<int>(S_SEG, n1);
  D.ord = P.get<int>(S_ORD, n1);
  D.sp = P.get<int>(S_SP, n1);
  D.tgt = P.get<int>(S_TGT, std::max<size_t>(n1, (size_t)c.nt));
  D.pot = P.get<float>(S_PHI, n1);
  int *subi = P.get<int>(S_SUBI, (size_t)2 * 28);
  int q = 0;
  auto nexti = [&]() { return subi + (size_t)2 * (q++); };
  D.n_s = nexti(); D.nbound = nexti(); D.nlast = nexti(); D.state = nexti(); D.corr = nexti(); D.iter = nexti();
  D.wrap = nexti(); D.tracers = nexti(); D.nb_new = nexti(); D.src_begin = nexti(); D.src_cnt = nexti();
  D.src_off = nexti(); D.tgt_cnt = nexti(); D.chunk_cnt = nexti(); D.chunk_off = nexti(); D.part_cnt = nexti();
  D.part_off = nexti(); D.tail_cnt = nexti(); D.tail_off = nexti(); D.fin_cnt = nexti(); D.fin_off = nexti();
  D.sp_cnt = nexti(); D.sp_off = nexti(); D.sp_len = nexti(); D.nunsample = nexti(); D.ngrav = nexti();
  D.self_cnt = nexti();
  int *bad = nexti();
  D.factor = P.get<float>(S_FACTOR, 6);
  unsigned *bb = P.get<unsigned>(S_BB, 7);
  D.bb_lo = bb;
  D.bb_hi = bb + 3;
  D.root = P.get<double>(S_ROOT, 4);
  D.keyp = P.get<float>(S_KEYP, 12);
  D.key = P.get<unsigned long long>(S_KEY, n1);
  D.key_alt = P.get<unsigned long long>(S_KEYA, n1);
  D.val = P.get<uint32_t>(S_VAL, n1);
  D.val_alt = P.get<uint32_t>(S_VALA, n1);
  D.k32 = P.get<uint32_t>(S_K32, n1);
  D.k32_alt = P.get<uint32_t>(S_K32A, n1);
  D.perm = P.get<uint32_t>(S_PERM, n1);
  D.perm_alt = P.get<uint32_t>(S_PERMA, n1);
  D.fb_list = P.get<int>(S_FBL, n1);
  D.fb_count = P.get<int>(S_FBC, 1);
  D.cnt = P.get<int>(S_CNT, n1 + 1);
  D.X = P.get<int>(S_X, n1 + 1);
  D.nodes = P.get<float4>(S_NODES, n1 * 3);
  D.interactions = P.get<unsigned long long>(S_COUNTER, kWalkCounters);
  D.walk_ctr = P.get<unsigned>(S_WCTR, (size_t)std::max(H->sm_count, 1));
  HBTG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
  k_pot_repack<<<blocks_for(c.ns, 256), 256, 0, st>>>(D, c.pos, c.mass);
  k_pot_plan<<<1, 32, 0, st>>>(D, (int)c.nt, 0);
  R.check();
  const int src_total = R.scan_counts(D.src_cnt, D.src_off, 1);
  const int chunk_total = R.scan_counts(D.chunk_cnt, D.chunk_off, 1);
  R.build_tree(src_total);
  k_pot_targets<<<blocks_for(c.nt, 256), 256, 0, st>>>(D, c.tgt, (int)c.nt, bad);
  k_pot_plan<<<1, 32, 0, st>>>(D, (int)c.nt, 1);
  R.check();
  R.walk(chunk_total);
  k_pot_out<<<blocks_for(c.nt, 256), 256, 0, st>>>(D, (int)c.nt, c.out);
  R.check();
  return read_int(bad, st) ? HBTG_ERR_INVALID : HBTG_OK;
}

struct DevCall
{
  hbtg_handle *H;
  const hbtg_params *p;
  hbtg_batch *b;
  cudaStream_t st;
  const WarmArgs *wa = nullptr;
};

int dev_call(void *arg)
{
  DevCall &c = *static_cast<DevCall *>(arg);
  HBTG_CUDA(cudaSetDevice(c.H->device));
  const int rc = run_device(c.H, c.p, c.b, c.st, c.wa);
  HBTG_CUDA(cudaStreamSynchronize(c.st));
  return rc;
}

// ---------------------------------------------------------------------------
// Autotuner of the launch settings (hbtg_autotune)
// ---------------------------------------------------------------------------
struct TuneCall
{
  hbtg_handle *H;
  const hbtg_params *p;
  hbtg_batch *b;
  cudaStream_t st;
  hbtg_tuning *report;
  int max_report;
  int *n_report;
};

int tune_call(void *arg)
{
  TuneCall &c = *static_cast<TuneCall *>(arg);
  hbtg_handle *H = c.H;
  hbtg_batch *b = c.b;
  long long N = 0;
  int rc = validate(c.p, b, N);
  if (rc != HBTG_OK)
    return rc;
  HBTG_CUDA(cudaSetDevice(H->device));
  cudaStream_t st = c.st;
  const size_t S = (size_t)b->n_sub;
  // the in/out frames, saved once and restored before every trial
  float *const fr[4] = {b->ref_pos, b->ref_vel, b->mostbound_pos, b->mostbound_vel};
  const size_t fbytes = sizeof(float) * 3 * S, ibytes = sizeof(int64_t) * S;
  unsigned char *save = H->pool.get<unsigned char>(S_TUNE, 4 * fbytes + ibytes);
  for (int k = 0; k < 4; k++)
    if (fr[k] && S)
      HBTG_CUDA(cudaMemcpyAsync(save + k * fbytes, fr[k], fbytes, cudaMemcpyDeviceToDevice, st));
  if (b->most_bound_id && S)
    HBTG_CUDA(cudaMemcpyAsync(save + 4 * fbytes, b->most_bound_id, ibytes, cudaMemcpyDeviceToDevice, st));
  auto restore = [&]() {
    for (int k = 0; k < 4; k++)
      if (fr[k] && S)
        HBTG_CUDA(cudaMemcpyAsync(fr[k], save + k * fbytes, fbytes, cudaMemcpyDeviceToDevice, st));
    if (b->most_bound_id && S)
      HBTG_CUDA(cudaMemcpyAsync(b->most_bound_id, save + 4 * fbytes, ibytes, cudaMemcpyDeviceToDevice, st));
  };
  const hbtg_tuning before = H->tune;
  cudaEvent_t e0, e1;
  HBTG_CUDA(cudaEventCreate(&e0));
  HBTG_CUDA(cudaEventCreate(&e1));
  std::vector<hbtg_tuning> tried;
  for (int bs : {0, 2048, kRadixBlockMax})
    for (int wr : {0, 1024})
      for (int mb : {4, 8})
      {
        H->tune = hbtg_tuning{bs, wr, mb, 0.0};
        float ms = 0.f;
        for (int rep = 0; rep < 2 && rc == HBTG_OK; rep++)
        {
          restore();
          HBTG_CUDA(cudaEventRecord(e0, st));
          rc = run_device(H, c.p, b, st);
          HBTG_CUDA(cudaEventRecord(e1, st));
          HBTG_CUDA(cudaStreamSynchronize(st));
          if (rc == HBTG_ERR_MAX_ITER)
            rc = HBTG_OK; // the same for every candidate; only the time matters here
          HBTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        }
        if (rc != HBTG_OK)
          break;
        tried.push_back(hbtg_tuning{bs, wr, mb, (double)ms});
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  restore();
  HBTG_CUDA(cudaStreamSynchronize(st));
  if (rc != HBTG_OK || tried.empty())
  {
    H->tune = before;
    return rc != HBTG_OK ? rc : HBTG_ERR_INVALID;
  }
  size_t best = 0;
  for (size_t i = 1; i < tried.size(); i++)
    if (tried[i].ms < tried[best].ms)
      best = i;
  H->tune = tried[best];
  for (size_t i = 0; i < tried.size() && (int)i < c.max_report; i++)
    c.report[i] = tried[i];
  if (c.n_report)
    *c.n_report = (int)tried.size();
  return HBTG_OK;
}

// ---------------------------------------------------------------------------
// Properties of the unbound subhaloes (props.cuh)
// ---------------------------------------------------------------------------
struct PropsCall
{
  hbtg_handle *H;
  const hbtg_params *p;
  const hbtg_batch *b;
  int snapshot;
  double relax;
  hbtg_props *o;
  cudaStream_t st;
  bool host = false;
};

// The property kernels over device arrays (b: positions, masses, order,
// nbound, mbound, mostbound_pos; offsets on the host), outputs into o.
int props_run(hbtg_handle *H, const hbtg_params *p, const hbtg_batch *b, int snapshot, double relax,
              const hbtg_props *o, cudaStream_t st, int64_t &launches)
{
  const int S = (int)b->n_sub;
  Pool &P = H->pool;
  PropState Q;
  Q.S = S;
  long long *off = P.get<long long>(S_PR_OFF, (size_t)S + 1);
  HBTG_CUDA(cudaMemcpyAsync(off, b->offsets, sizeof(long long) * (S + 1), cudaMemcpyHostToDevice, st));
  Q.off = off;
  Q.pos = b->pos;
  Q.mass = b->mass;
  Q.order = reinterpret_cast<const long long *>(b->order);
  Q.nbound = reinterpret_cast<const long long *>(b->nbound);
  Q.mbound = b->mbound;
  Q.mb_pos = b->mostbound_pos;
  Q.cnt = P.get<int>(S_PR_CNT, (size_t)S + 1);
  Q.fin_off = P.get<int>(S_PR_FIN, (size_t)S + 1);
  Q.vkey = P.get<unsigned long long>(S_PR_VK, (size_t)S);
  Q.so_rank = P.get<int>(S_PR_SO, (size_t)S);
  Q.shape = P.get<double>(S_PR_SH, (size_t)S * 12);
  Q.box = (float)p->box_size;
  Q.half = (float)((double)Q.box / 2.);
  Q.periodic = p->periodic != 0;
  Q.soft = (float)p->softening;
  const float G = (float)p->G, a = (float)p->scale_factor, hz = (float)p->hubble;
  Q.velocity_unit = G / a; // PhysicalConst::G / ScaleFactor in float
  // SphericalOverdensitySize's RhoVirial for VirialFactor 200, in the reference's mixed float/double order
  Q.rho_vir = (float)((double)((200.f * hz) * hz) / 2.0 / (double)G * (double)a * (double)a * (double)a);
  Q.relax = (float)relax;
  Q.snapshot = snapshot;
  k_prop_init<<<blocks_for(S + 1, 256), 256, 0, st>>>(Q);
  launches++;
  HBTG_CUDA(cudaGetLastError());
  scan<int, false>(Q.cnt, Q.fin_off, S + 1, P.get<int>(S_SCRATCH, scan_scratch_elems<int>(S + 1)), st, &launches);
  const int T = read_int(Q.fin_off + S, st);
  const size_t t1 = (size_t)std::max(T, 1);
  Q.rr = P.get<float>(S_PR_RR, t1);
  Q.mm = P.get<float>(S_PR_MM, t1);
  Q.k32 = P.get<uint32_t>(S_PR_K, t1);
  Q.val = P.get<uint32_t>(S_PR_V, t1);
  Q.k32_alt = P.get<uint32_t>(S_PR_KA, t1);
  Q.val_alt = P.get<uint32_t>(S_PR_VA, t1);
  Q.mcum = P.get<double>(S_PR_MC, t1);
  const uint32_t *sorted = Q.val;
  if (T > 0)
  {
    k_prop_items<<<blocks_for(((long long)T + kItemsPerThread - 1) / kItemsPerThread, 256), 256, 0, st>>>(Q, T);
    launches++;
    HBTG_CUDA(cudaGetLastError());
    // by distance, then stably by subhalo
    int *table = P.get<int>(S_TABLE, radix_table_elems(T));
    int *scr = P.get<int>(S_SCRATCH, scan_scratch_elems<int>(std::max<long long>(radix_table_elems(T) + 1,
                                                                                      256LL * 4096)));
    const bool f1 = radix_sort_pairs<uint32_t>(Q.k32, Q.val, Q.k32_alt, Q.val_alt, T, 0, 32, table, scr, st,
                                               &launches);
    uint32_t *v = f1 ? Q.val_alt : Q.val, *v_other = f1 ? Q.val : Q.val_alt;
    int bits = 0;
    while ((1LL << bits) < S)
      bits++;
    if (bits > 0)
    {
      k_prop_segkeys<<<blocks_for(T, 256), 256, 0, st>>>(Q, v, Q.k32, T);
      launches++;
      const bool f2 = radix_sort_pairs<uint32_t>(Q.k32, v, Q.k32_alt, v_other, T, 0, bits, table, scr, st,
                                                 &launches);
      v = f2 ? v_other : v;
    }
    sorted = v;
    SegD *sscr = P.get<SegD>(S_PR_SCR, scan_scratch_elems<SegD>(T));
    scan_load_store<SegD, true>(PropMassLoad{Q, sorted}, PropMassStore{Q.mcum}, T, sscr, st, &launches);
    k_prop_profile<<<blocks_for(T, 256), 256, 0, st>>>(Q, sorted, T);
    launches++;
    HBTG_CUDA(cudaGetLastError());
  }
  PropOut O;
  O.rmax = o->rmax;
  O.vmax = o->vmax;
  O.rhalf = o->rhalf;
  O.renclose = o->renclose;
  O.r200 = o->r200;
  O.m200 = o->m200;
  O.last_vmax = o->last_vmax;
  O.rmax_last = o->rmax_last;
  O.snap_last = o->snap_last;
  O.inertia = o->inertia;
  O.inertia_w = o->inertia_w;
  O.nsource = reinterpret_cast<long long *>(o->nsource);
  k_prop_finish<<<blocks_for(S, 256), 256, 0, st>>>(Q, sorted, O);
  launches++;
  HBTG_CUDA(cudaGetLastError());
  return HBTG_OK;
}

int props_call(void *arg)
{
  PropsCall &c = *static_cast<PropsCall *>(arg);
  hbtg_handle *H = c.H;
  const hbtg_batch *b = c.b;
  const hbtg_props *o = c.o;
  if (!c.p || !b || !o || b->n_sub < 0 || (b->n_sub > 0 && !b->offsets))
    return HBTG_ERR_INVALID;
  if (!o->rmax || !o->vmax || !o->rhalf || !o->renclose || !o->r200 || !o->m200 || !o->last_vmax ||
      !o->rmax_last || !o->snap_last || !o->inertia || !o->inertia_w)
    return HBTG_ERR_INVALID;
  const long long S = b->n_sub;
  if (S == 0)
    return HBTG_OK;
  if (S >= (1LL << 30) || b->offsets[0] != 0)
    return HBTG_ERR_INVALID;
  for (long long s = 0; s < S; s++)
    if (b->offsets[s + 1] < b->offsets[s])
      return HBTG_ERR_INVALID;
  const long long N = b->offsets[S];
  if (N >= (1LL << 30) || (N > 0 && (!b->pos || !b->mass || !b->order)) || !b->nbound || !b->mbound ||
      !b->mostbound_pos)
    return HBTG_ERR_INVALID;
  HBTG_CUDA(cudaSetDevice(H->device));
  cudaStream_t st = c.st;
  int64_t launches = 0, h2d = 0, d2h = 0;
  if (!c.host)
  {
    const int rc = props_run(H, c.p, b, c.snapshot, c.relax, o, st, launches);
    HBTG_CUDA(cudaStreamSynchronize(st));
    H->stats.kernel_launches = launches;
    return rc;
  }
  for (long long s = 0; s < S; s++)
    if (b->nbound[s] < 0 || b->nbound[s] > b->offsets[s + 1] - b->offsets[s])
      return HBTG_ERR_INVALID;
  Pool &P = H->pool;
  hbtg_batch d = *b;
  d.pos = upload(P, S_PR_POS, b->pos, 3 * (size_t)N, st, h2d);
  d.mass = upload(P, S_PR_MASS, b->mass, (size_t)N, st, h2d);
  d.order = upload(P, S_PR_ORD, b->order, (size_t)N, st, h2d);
  d.nbound = upload(P, S_PR_NB, b->nbound, (size_t)S, st, h2d);
  d.mbound = upload(P, S_PR_MBND, b->mbound, (size_t)S, st, h2d);
  d.mostbound_pos = upload(P, S_PR_MBP, b->mostbound_pos, 3 * (size_t)S, st, h2d);
  float *of = P.get<float>(S_PR_OUTF, 20 * (size_t)S);
  int32_t *oi = P.get<int32_t>(S_PR_OUTI, (size_t)S);
  int64_t *ol = P.get<int64_t>(S_PR_OUTL, (size_t)S);
  hbtg_props dp;
  dp.rmax = of;
  dp.vmax = of + S;
  dp.rhalf = of + 2 * S;
  dp.renclose = of + 3 * S;
  dp.r200 = of + 4 * S;
  dp.m200 = of + 5 * S;
  dp.last_vmax = of + 6 * S;
  dp.rmax_last = of + 7 * S;
  dp.inertia = of + 8 * S;
  dp.inertia_w = of + 14 * S;
  dp.snap_last = oi;
  dp.nsource = o->nsource ? ol : nullptr;
  const size_t fs = sizeof(float) * (size_t)S;
  // in/out members start from the caller's values
  HBTG_CUDA(cudaMemcpyAsync(dp.r200, o->r200, fs, cudaMemcpyHostToDevice, st));
  HBTG_CUDA(cudaMemcpyAsync(dp.m200, o->m200, fs, cudaMemcpyHostToDevice, st));
  HBTG_CUDA(cudaMemcpyAsync(dp.last_vmax, o->last_vmax, fs, cudaMemcpyHostToDevice, st));
  HBTG_CUDA(cudaMemcpyAsync(dp.rmax_last, o->rmax_last, fs, cudaMemcpyHostToDevice, st));
  HBTG_CUDA(cudaMemcpyAsync(dp.snap_last, o->snap_last, sizeof(int32_t) * (size_t)S, cudaMemcpyHostToDevice, st));
  const int rc = props_run(H, c.p, &d, c.snapshot, c.relax, &dp, st, launches);
  float *const hf[8] = {o->rmax, o->vmax, o->rhalf, o->renclose, o->r200, o->m200, o->last_vmax, o->rmax_last};
  for (int q = 0; q < 8; q++)
    download(hf[q], of + (size_t)q * S, (size_t)S, st, d2h);
  download(o->inertia, dp.inertia, 6 * (size_t)S, st, d2h);
  download(o->inertia_w, dp.inertia_w, 6 * (size_t)S, st, d2h);
  download(o->snap_last, dp.snap_last, (size_t)S, st, d2h);
  if (o->nsource)
    download(o->nsource, dp.nsource, (size_t)S, st, d2h);
  HBTG_CUDA(cudaStreamSynchronize(st));
  H->stats.kernel_launches = launches;
  H->stats.h2d_bytes = h2d;
  H->stats.d2h_bytes = d2h;
  return rc;
}

// ---------------------------------------------------------------------------
// Particle reassignment (reassign.cuh)
// ---------------------------------------------------------------------------
struct ReassignCall
{
  hbtg_handle *H;
  const hbtg_params *p;
  const hbtg_reassign *r;
  int k;
  cudaStream_t st;
  bool host = false;
};

int reassign_run(hbtg_handle *H, const hbtg_params *p, const hbtg_reassign *r, int k, cudaStream_t st,
                 int64_t &launches)
{
  const int S = (int)r->n_sub, G = (int)r->n_groups;
  const long long N = r->offsets[S];
  Pool &P = H->pool;
  std::vector<int> sub_group(std::max(S, 1));
  std::vector<long long> gpart(G + 1);
  for (int h = 0; h < G; h++)
    for (long long s = r->group_off[h]; s < r->group_off[h + 1]; s++)
      sub_group[s] = h;
  for (int h = 0; h <= G; h++)
    gpart[h] = r->offsets[r->group_off[h]];
  ReState Q;
  Q.S = S;
  Q.G = G;
  long long *off = P.get<long long>(S_RE_OFF, (size_t)S + 1);
  int *sg = P.get<int>(S_RE_SG, (size_t)std::max(S, 1));
  long long *gp = P.get<long long>(S_RE_GP, (size_t)G + 1);
  HBTG_CUDA(cudaMemcpyAsync(off, r->offsets, sizeof(long long) * (S + 1), cudaMemcpyHostToDevice, st));
  HBTG_CUDA(cudaMemcpyAsync(sg, sub_group.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  HBTG_CUDA(cudaMemcpyAsync(gp, gpart.data(), sizeof(long long) * (G + 1), cudaMemcpyHostToDevice, st));
  Q.off = off;
  Q.sub_group = sg;
  Q.gpart = gp;
  Q.pos = r->pos;
  Q.type = r->type;
  Q.dest = reinterpret_cast<long long *>(r->dest);
  Q.flags = P.get<int>(S_RE_FL, (size_t)N + 1);
  Q.rank = P.get<int>(S_RE_RK, (size_t)N + 1);
  Q.tracer_mask = p->tracer_type_mask;
  Q.box = (float)p->box_size;
  Q.half = (float)((double)Q.box / 2.);
  Q.periodic = p->periodic != 0;
  Q.r0 = (float)((double)(float)p->softening * 0.1); // HBTConfig.SofteningHalo * 0.1 as a float radius
  Q.eps = 16.f * std::ldexp(std::max(Q.box, 1.f), -23); // float rounding of unwrapped coordinates
  Q.k = k;
  k_re_flags<<<blocks_for(N + 1, 256), 256, 0, st>>>(Q, N);
  launches++;
  HBTG_CUDA(cudaGetLastError());
  scan<int, false>(Q.flags, Q.rank, N + 1, P.get<int>(S_SCRATCH, scan_scratch_elems<int>(N + 1)), st, &launches);
  const int T = read_int(Q.rank + N, st);
  const size_t t1 = (size_t)std::max(T, 1);
  Q.tg = P.get<int>(S_RE_TG, t1);
  Q.tsub = P.get<int>(S_RE_TS, t1);

  PoolMem mem{H, st, {}};
  IterationDriver<PoolMem> R(mem, st);
  R.K = make_kparams(p, false);
  R.S = G;
  int bits = 0;
  while ((1LL << bits) < G)
    bits++;
  R.seg_bits = bits;
  R.sm_count = H->sm_count;
  DevState &D = R.D;
  D.S = G;
  D.N = T;
  long long *goff = P.get<long long>(S_RE_GO, (size_t)G + 1);
  k_re_goff<<<blocks_for(G + 1, 256), 256, 0, st>>>(Q, goff);
  launches++;
  D.off = goff;
  D.pm = P.get<float4>(S_PM, t1);
  D.ty = P.get<uint8_t>(S_TY, t1);
  D.seg_of = P.get<int>(S_SEG, t1);
  D.ord = P.get<int>(S_ORD, t1);
  int *subi = P.get<int>(S_SUBI, (size_t)(G + 1) * 28);
  int q = 0;
  auto nexti = [&]() { return subi + (size_t)(G + 1) * (q++); };
  D.n_s = nexti(); D.nbound = nexti(); D.nlast = nexti(); D.state = nexti(); D.corr = nexti(); D.iter = nexti();
  D.wrap = nexti(); D.tracers = nexti(); D.nb_new = nexti(); D.src_begin = nexti(); D.src_cnt = nexti();
  D.src_off = nexti(); D.tgt_cnt = nexti(); D.chunk_cnt = nexti(); D.chunk_off = nexti(); D.part_cnt = nexti();
  D.part_off = nexti(); D.tail_cnt = nexti(); D.tail_off = nexti(); D.fin_cnt = nexti(); D.fin_off = nexti();
  D.sp_cnt = nexti(); D.sp_off = nexti(); D.sp_len = nexti(); D.nunsample = nexti(); D.ngrav = nexti();
  D.factor = P.get<float>(S_FACTOR, (size_t)G * 6 + 6);
  unsigned *bb = P.get<unsigned>(S_BB, (size_t)G * 7 + 7);
  D.bb_lo = bb;
  D.bb_hi = bb + 3 * (size_t)G;
  D.root = P.get<double>(S_ROOT, (size_t)G * 4 + 4);
  D.keyp = P.get<float>(S_KEYP, (size_t)G * 12 + 12);
  D.key = P.get<unsigned long long>(S_KEY, t1);
  D.key_alt = P.get<unsigned long long>(S_KEYA, t1);
  D.val = P.get<uint32_t>(S_VAL, t1);
  D.val_alt = P.get<uint32_t>(S_VALA, t1);
  D.k32 = P.get<uint32_t>(S_K32, t1);
  D.k32_alt = P.get<uint32_t>(S_K32A, t1);
  D.perm = P.get<uint32_t>(S_PERM, t1);
  D.perm_alt = P.get<uint32_t>(S_PERMA, t1);
  D.fb_list = P.get<int>(S_FBL, t1);
  D.fb_count = P.get<int>(S_FBC, 1);
  D.cnt = P.get<int>(S_CNT, t1 + 1);
  D.X = P.get<int>(S_X, t1 + 1);
  D.interactions = P.get<unsigned long long>(S_COUNTER, kWalkCounters);
  if (T > 0)
  {
    k_re_pack<<<blocks_for(N, 256), 256, 0, st>>>(Q, D, N);
    k_re_unwrap<<<blocks_for(T, 256), 256, 0, st>>>(Q, D, T);
    launches += 2;
  }
  k_re_plan<<<blocks_for(G + 1, 256), 256, 0, st>>>(Q, D);
  launches++;
  R.check();
  const int src_total = R.scan_counts(D.src_cnt, D.src_off, G);
  if (src_total > 0)
    R.build_tree(src_total, true);
  if (N > 0)
  {
    k_re_query<<<blocks_for(N, 128), 128, 0, st>>>(Q, D, N);
    launches++;
  }
  R.check();
  launches += R.launches;
  return HBTG_OK;
}

int reassign_call(void *arg)
{
  ReassignCall &c = *static_cast<ReassignCall *>(arg);
  hbtg_handle *H = c.H;
  const hbtg_reassign *r = c.r;
  if (!c.p || !r || r->n_groups < 0 || r->n_sub < 0 || !r->group_off || !r->offsets || c.k < 1 ||
      c.k > kMaxNeighbours)
    return HBTG_ERR_INVALID;
  const long long S = r->n_sub, G = r->n_groups;
  if (r->offsets[0] != 0 || r->group_off[0] != 0 || r->group_off[G] != S || S >= (1LL << 30))
    return HBTG_ERR_INVALID;
  for (long long s = 0; s < S; s++)
    if (r->offsets[s + 1] < r->offsets[s])
      return HBTG_ERR_INVALID;
  for (long long h = 0; h < G; h++)
    if (r->group_off[h + 1] < r->group_off[h])
      return HBTG_ERR_INVALID;
  const long long N = r->offsets[S];
  if (N >= (1LL << 30) || (N > 0 && (!r->pos || !r->type || !r->dest)))
    return HBTG_ERR_INVALID;
  if (N == 0)
    return HBTG_OK;
  HBTG_CUDA(cudaSetDevice(H->device));
  cudaStream_t st = c.st;
  int64_t launches = 0, h2d = 0, d2h = 0;
  int rc;
  if (!c.host)
    rc = reassign_run(H, c.p, r, c.k, st, launches);
  else
  {
    Pool &P = H->pool;
    hbtg_reassign d = *r;
    d.pos = upload(P, S_RE_POS, r->pos, 3 * (size_t)N, st, h2d);
    d.type = upload(P, S_RE_TY, r->type, (size_t)N, st, h2d);
    d.dest = P.get<int64_t>(S_RE_DEST, (size_t)N);
    rc = reassign_run(H, c.p, &d, c.k, st, launches);
    download(r->dest, d.dest, (size_t)N, st, d2h);
  }
  HBTG_CUDA(cudaStreamSynchronize(st));
  H->stats.kernel_launches = launches;
  H->stats.h2d_bytes = h2d;
  H->stats.d2h_bytes = d2h;
  return rc;
}

struct ModelCall
{
  hbtg_handle *H;
  const hbtg_model *m;
};

int model_call(void *arg)
{
  ModelCall &c = *static_cast<ModelCall *>(arg);
  HBTG_CUDA(cudaSetDevice(c.H->device));
  float *d = c.H->pool.get<float>(S_MODEL, HBTG_MLP_PARAMS);
  HBTG_CUDA(cudaMemcpy(d, c.m->weights, sizeof(float) * HBTG_MLP_PARAMS, cudaMemcpyHostToDevice));
  c.H->has_model = true;
  c.H->threshold = c.m->threshold;
  c.H->exclude_below = c.m->exclude_below;
  c.H->min_particles = c.m->min_particles;
  c.H->first_test = c.m->first_test;
  return HBTG_OK;
}

struct LabelCall
{
  hbtg_handle *H;
  uint8_t *labels;
  int which;
  cudaStream_t st;
};

int label_call(void *arg)
{
  LabelCall &c = *static_cast<LabelCall *>(arg);
  hbtg_handle *H = c.H;
  if (!H->last_ord)
    return HBTG_ERR_INVALID; // no unbinding call yet
  HBTG_CUDA(cudaSetDevice(H->device));
  DevState D;
  D.S = H->last_S;
  D.N = H->last_N;
  D.off = H->last_off;
  D.ord = H->last_ord;
  D.nlast = H->last_nlast;
  D.state = H->last_state;
  D.seg_of = H->last_seg;
  D.nb1 = H->last_nb1;
  if (D.N > 0)
    k_trace_labels<<<blocks_for(D.N, 256), 256, 0, c.st>>>(D, c.labels, c.which);
  HBTG_CUDA(cudaGetLastError());
  HBTG_CUDA(cudaStreamSynchronize(c.st));
  return HBTG_OK;
}

} // namespace

extern "C" {

int hbtg_create(hbtg_handle **handle, int device)
{
  if (!handle)
    return HBTG_ERR_INVALID;
  *handle = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0)
  {
    cudaGetLastError();
    return HBTG_ERR_NO_DEVICE;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
    return HBTG_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3)
    return HBTG_ERR_NO_DEVICE; // built for sm_103a only
  hbtg_handle *h = new (std::nothrow) hbtg_handle();
  if (!h)
    return HBTG_ERR_NOMEM;
  h->device = device;
  h->sm_count = prop.multiProcessorCount;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) !=
                                                  cudaSuccess)
  {
    delete h;
    return HBTG_ERR_CUDA;
  }
  h->walk_events.resize(2);
  for (auto &e : h->walk_events)
    if (cudaEventCreate(&e) != cudaSuccess)
    {
      delete h;
      return HBTG_ERR_CUDA;
    }
  if (cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->side2, cudaStreamNonBlocking) != cudaSuccess)
  {
    delete h;
    return HBTG_ERR_CUDA;
  }
  for (auto &e : h->copy_events)
    if (cudaEventCreate(&e) != cudaSuccess)
    {
      delete h;
      return HBTG_ERR_CUDA;
    }
  *handle = h;
  return HBTG_OK;
}

int hbtg_destroy(hbtg_handle *h)
{
  if (!h)
    return HBTG_ERR_INVALID;
  cudaSetDevice(h->device);
  h->pool.release();
  for (auto &e : h->walk_events)
    cudaEventDestroy(e);
  for (auto &e : h->phase_events)
    cudaEventDestroy(e);
  for (auto &e : h->copy_events)
    if (e)
      cudaEventDestroy(e);
  if (h->side)
    cudaStreamDestroy(h->side);
  if (h->side2)
    cudaStreamDestroy(h->side2);
  if (h->stream)
    cudaStreamDestroy(h->stream);
  delete h;
  return HBTG_OK;
}

int hbtg_subhalo_properties_device(hbtg_handle *h, const hbtg_params *p, const hbtg_batch *b, int32_t snapshot_id,
                                   double source_relax, hbtg_props *props, void *cuda_stream)
{
  if (!h)
    return HBTG_ERR_INVALID;
  PropsCall c{h, p, b, snapshot_id, source_relax, props, static_cast<cudaStream_t>(cuda_stream), false};
  return guarded(props_call, &c);
}

int hbtg_subhalo_properties(hbtg_handle *h, const hbtg_params *p, const hbtg_batch *b, int32_t snapshot_id,
                            double source_relax, hbtg_props *props)
{
  if (!h)
    return HBTG_ERR_INVALID;
  PropsCall c{h, p, b, snapshot_id, source_relax, props, h->stream, true};
  return guarded(props_call, &c);
}

int hbtg_reassign_particles_device(hbtg_handle *h, const hbtg_params *p, const hbtg_reassign *r, int num_neighbours,
                                   void *cuda_stream)
{
  if (!h)
    return HBTG_ERR_INVALID;
  ReassignCall c{h, p, r, num_neighbours, static_cast<cudaStream_t>(cuda_stream), false};
  return guarded(reassign_call, &c);
}

int hbtg_reassign_particles(hbtg_handle *h, const hbtg_params *p, const hbtg_reassign *r, int num_neighbours)
{
  if (!h)
    return HBTG_ERR_INVALID;
  ReassignCall c{h, p, r, num_neighbours, h->stream, true};
  return guarded(reassign_call, &c);
}

int hbtg_unbind_batch(hbtg_handle *h, const hbtg_params *p, hbtg_batch *b)
{
  if (!h)
    return HBTG_ERR_INVALID;
  HostCall c{h, p, b};
  return guarded(host_call, &c);
}

int hbtg_unbind_batch_device(hbtg_handle *h, const hbtg_params *p, hbtg_batch *b, void *cuda_stream)
{
  if (!h)
    return HBTG_ERR_INVALID;
  DevCall c{h, p, b, static_cast<cudaStream_t>(cuda_stream)};
  return guarded(dev_call, &c);
}

int hbtg_set_model(hbtg_handle *h, const hbtg_model *m)
{
  if (!h || !m || !m->weights || !(m->threshold == m->threshold) || !(m->exclude_below <= m->threshold) ||
      m->min_particles < 0 || (m->first_test != 0 && m->first_test != 1))
    return HBTG_ERR_INVALID;
  ModelCall c{h, m};
  return guarded(model_call, &c);
}

int hbtg_unbind_batch_learned(hbtg_handle *h, const hbtg_params *p, hbtg_batch *b, const hbtg_prior *prior)
{
  if (!h)
    return HBTG_ERR_INVALID;
  HostCall c{h, p, b, true, prior};
  return guarded(host_call, &c);
}

int hbtg_unbind_batch_learned_device(hbtg_handle *h, const hbtg_params *p, hbtg_batch *b, const hbtg_prior *prior,
                                     void *cuda_stream)
{
  if (!h)
    return HBTG_ERR_INVALID;
  WarmArgs wa;
  wa.min_n = h->min_particles;
  wa.first_test = h->first_test;
  if (prior && prior->nbound_prev)
  {
    wa.nb_prev = reinterpret_cast<const long long *>(prior->nbound_prev);
    wa.e_prev = prior->energy_prev;
  }
  DevCall c{h, p, b, static_cast<cudaStream_t>(cuda_stream), &wa};
  return guarded(dev_call, &c);
}

int hbtg_unbind_batch_warm_device(hbtg_handle *h, const hbtg_params *p, hbtg_batch *b, const uint8_t *proposal,
                                  int64_t min_particles, void *cuda_stream)
{
  if (!h || !b || min_particles < 0)
    return HBTG_ERR_INVALID;
  static const uint8_t none = 0;
  const bool empty = b->n_sub <= 0 || !b->offsets || b->offsets[b->n_sub] <= 0;
  if (!proposal && !empty)
    return HBTG_ERR_INVALID;
  WarmArgs wa;
  wa.proposal = proposal ? proposal : &none; // an empty batch never reads it
  wa.min_n = min_particles;
  DevCall c{h, p, b, static_cast<cudaStream_t>(cuda_stream), &wa};
  return guarded(dev_call, &c);
}

int hbtg_features_device(hbtg_handle *h, const hbtg_params *p, const hbtg_batch *b, const hbtg_prior *prior,
                         float *features, void *cuda_stream)
{
  if (!h || !b || !features)
    return HBTG_ERR_INVALID;
  WarmArgs wa;
  wa.features_only = features;
  if (prior && prior->nbound_prev)
  {
    wa.nb_prev = reinterpret_cast<const long long *>(prior->nbound_prev);
    wa.e_prev = prior->energy_prev;
  }
  hbtg_batch copy = *b; // a features-only call writes no output
  DevCall c{h, p, &copy, static_cast<cudaStream_t>(cuda_stream), &wa};
  return guarded(dev_call, &c);
}

int hbtg_tree_potential_device(hbtg_handle *h, const hbtg_params *p, int64_t n_src, const float *pos,
                               const float *mass, int64_t n_tgt, const int64_t *tgt_index, float *potential,
                               void *cuda_stream)
{
  if (!h || !p || n_src <= 0 || n_src >= (1LL << 30) || n_tgt < 0 || n_tgt >= (1LL << 30) || !pos || !mass ||
      (n_tgt > 0 && (!tgt_index || !potential)) || !(p->softening > 0) || !(p->open_angle > 0) ||
      !(p->box_size > 0))
    return HBTG_ERR_INVALID;
  if (n_tgt == 0)
    return HBTG_OK;
  PotCall c{h, p, n_src, n_tgt, pos, mass, reinterpret_cast<const long long *>(tgt_index), potential,
            static_cast<cudaStream_t>(cuda_stream)};
  return guarded(pot_call, &c);
}

int hbtg_trace_labels_device(hbtg_handle *h, uint8_t *labels, int which, void *cuda_stream)
{
  if (!h || !labels || which < 0 || which > 1)
    return HBTG_ERR_INVALID;
  LabelCall c{h, labels, which, static_cast<cudaStream_t>(cuda_stream)};
  return guarded(label_call, &c);
}

int hbtg_prepare_subsampling(const hbtg_params *p, const hbtg_batch *b, int64_t *perm)
{
  if (!p || !b || !perm || b->n_sub < 0 || (b->n_sub > 0 && !b->offsets))
    return HBTG_ERR_INVALID;
  for (int64_t s = 0; s < b->n_sub; s++)
    if (b->offsets[s + 1] < b->offsets[s])
      return HBTG_ERR_INVALID;
  std::srand((unsigned)p->seed);
  std::vector<int64_t> idx;
  for (int64_t s = 0; s < b->n_sub; s++)
  {
    const int64_t off = b->offsets[s], n = b->offsets[s + 1] - off;
    idx.resize(n);
    for (int64_t k = 0; k < n; k++)
      idx[k] = k;
    if (p->max_sample_size > 0 && n > p->max_sample_size)
    {
      auto exempt = [&](int64_t k) {
        if (p->dm_only || !b->type)
          return false;
        return ((1 << b->type[off + k]) & p->no_subsample_mask) != 0;
      };
      auto it = std::partition(idx.begin(), idx.end(), exempt);
      std::random_shuffle(it, idx.end());
    }
    for (int64_t k = 0; k < n; k++)
      perm[off + k] = idx[k];
  }
  return HBTG_OK;
}

int hbtg_get_stats(const hbtg_handle *h, hbtg_stats *s)
{
  if (!h || !s)
    return HBTG_ERR_INVALID;
  *s = h->stats;
  return HBTG_OK;
}

int hbtg_set_count_interactions(hbtg_handle *h, int enable)
{
  if (!h)
    return HBTG_ERR_INVALID;
  h->count_interactions = enable != 0;
  return HBTG_OK;
}

int hbtg_get_tuning(const hbtg_handle *h, hbtg_tuning *t)
{
  if (!h || !t)
    return HBTG_ERR_INVALID;
  *t = h->tune;
  return HBTG_OK;
}

int hbtg_set_tuning(hbtg_handle *h, const hbtg_tuning *t)
{
  if (!h || !t || t->block_sort_max < 0 || t->walk_ranged_min < 0 || t->moments_blocks_per_sm < 1 ||
      t->moments_blocks_per_sm > 32)
    return HBTG_ERR_INVALID;
  h->tune = *t;
  h->tune.block_sort_max = std::min(t->block_sort_max, kRadixBlockMax);
  return HBTG_OK;
}

int hbtg_autotune(hbtg_handle *h, const hbtg_params *p, hbtg_batch *b, void *cuda_stream, hbtg_tuning *report,
                  int max_report, int *n_report)
{
  if (!h || max_report < 0 || (max_report > 0 && !report))
    return HBTG_ERR_INVALID;
  TuneCall c{h, p, b, static_cast<cudaStream_t>(cuda_stream), report, max_report, n_report};
  return guarded(tune_call, &c);
}

const char *hbtg_status_string(int status)
{
  switch (status)
  {
  case HBTG_OK:
    return "ok";
  case HBTG_ERR_INVALID:
    return "invalid argument";
  case HBTG_ERR_NOMEM:
    return "out of memory";
  case HBTG_ERR_CUDA:
    return "CUDA error";
  case HBTG_ERR_MAX_ITER:
    return "a subhalo reached max_iterations";
  case HBTG_ERR_UNSUPPORTED:
    return "unsupported parameters";
  case HBTG_ERR_NO_DEVICE:
    return "no sm_103 CUDA device";
  default:
    return "unknown status";
  }
}

void hbtg_default_params(hbtg_params *p)
{
  if (!p)
    return;
  std::memset(p, 0, sizeof(*p));
  p->box_size = 100.0;
  p->periodic = 1;
  p->softening = 0.005;
  p->tree_node_resolution = 0.0005;
  p->open_angle = 0.45;
  p->bound_mass_precision = 0.995;
  p->min_num_part = 20;
  p->min_num_tracer = 10;
  p->tracer_type_mask = (1 << 1) | (1 << 4);
  p->no_subsample_mask = 1 << 5;
  p->max_sample_size = 1000;
  p->refine_most_bound = 1;
  p->refine_fraction = 0.1;
  p->upscale_per_type = 1;
  p->sub_core_size_min = 20;
  p->sub_core_size_factor = 0.0;
  p->dm_only = 0;
  p->thermal = 0;
  p->G = 43.0071;
  p->scale_factor = 1.0;
  p->hubble = 0.0;
  p->max_iterations = 1000;
  p->mode = 0;
  p->seed = 0;
}

} // extern "C"
