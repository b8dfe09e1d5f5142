// driver.cuh - the lock-step unbinding iteration shared by every entry point.
//
// Subhalo_t::Unbind's loop (src/subhalo_unbind.cpp:555-758) run for all
// subhaloes of a batch at once: each pass of the loop below is one iteration
// for every subhalo still active; subhaloes leave the active set where the
// reference breaks out of its loop.  The memory policy `Mem` supplies the
// working buffers (a grow-only pool, or a fixed static reserve) and turns CUDA
// errors into exceptions of its own type.
//
// Mem must provide:
//   void check(cudaError_t)                      throws on error
//   int *scan_scratch(long long n)               scratch for scan<int>(n)
//   int *radix_table(long long n)                table for radix_sort_pairs(n)
//   int *radix_scan_scratch(long long n)
//   int *cell_list(long long cells)              per-level cell lists of one tree (may throw)
//   int *level_counts()                          2 kLevels ints
//   float4 *tree_slots(long long slots)          tree storage (may throw when too large)
//   void mark(int phase)                         phase boundary for timing (may be a no-op)
#pragma once

#include <algorithm>
#include <cstdint>
#include <utility>

#include "common.cuh"
#include "kernels.cuh"
#include "primitives.cuh"
#include "walk.cuh"

namespace hbtg
{

inline unsigned grid_for(long long n, int threads)
{
  long long b = (n + threads - 1) / threads;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, 0x7fffffffLL));
}

template <class Mem>
struct IterationDriver
{
  Mem &mem;
  cudaStream_t st;
  KParams K;
  DevState D;
  int S = 0;
  int seg_bits = 0;
  int sm_count = 152;
  int walk_blocks_per_sm = 1; // resident k_walk blocks per SM (occupancy)
  // launch settings that leave every result unchanged (hbtg_tuning, hbtg_autotune)
  int block_sort_max = kRadixBlockMax; // largest sort done by one block
  int walk_ranged_min = 0;             // walks of fewer chunks use a grid-stride loop instead of per-SM ranges
  int moments_blocks_per_sm = 8;       // grid cap of the per-level multipole passes
  int64_t launches = 0;
  int64_t walk_launches = 0;
  int64_t tree_nodes = 0;
  int64_t host_syncs = 0; // stream synchronisations for host reads of device totals
  int global_iter = 0;

  IterationDriver(Mem &m, cudaStream_t s) : mem(m), st(s)
  {
    // the walk keeps its stacks and interaction lists in shared memory
    cudaFuncSetAttribute(k_walk<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_walk<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_walk<false>, 32 * kWalkWarps, 0) == cudaSuccess &&
        nb > 0)
      walk_blocks_per_sm = nb;
    cudaGetLastError();
  }

  void check() { mem.check(cudaGetLastError()); }

  int read_int(const int *d)
  {
    int h = 0;
    mem.check(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    mem.check(cudaStreamSynchronize(st));
    host_syncs++;
    return h;
  }

  // Up to four count arrays (null = none) read as one I4c item.
  struct Count4Load
  {
    const int *a, *b, *c, *d;
    __device__ I4c operator()(long long i) const
    {
      return I4c{a ? a[i] : 0, b ? b[i] : 0, c ? c[i] : 0, d ? d[i] : 0};
    }
  };
  struct Count4Store
  {
    int *a, *b, *c, *d;
    __device__ void operator()(long long i, const I4c &v) const
    {
      if (a)
        a[i] = v.a;
      if (b)
        b[i] = v.b;
      if (c)
        c[i] = v.c;
      if (d)
        d[i] = v.d;
    }
  };

  // Exclusive scans of up to four count arrays (n counts plus a trailing zero
  // each; null pairs are skipped) in one pass, with one host read of the totals.
  void scan_counts4(const int *c0, int *o0, const int *c1, int *o1, const int *c2, int *o2, const int *c3, int *o3,
                    long long n, int tot[4])
  {
    // an int scratch for 8 (n + 1) items covers scan_scratch_elems<I4c>(n + 1) I4cs
    I4c *scr = reinterpret_cast<I4c *>(mem.scan_scratch(8 * (n + 1)));
    scan_load_store<I4c, false>(Count4Load{c0, c1, c2, c3}, Count4Store{o0, o1, o2, o3}, n + 1, scr, st, &launches);
    check();
    int *outs[4] = {o0, o1, o2, o3};
    for (int k = 0; k < 4; k++)
    {
      tot[k] = 0;
      if (outs[k])
        mem.check(cudaMemcpyAsync(&tot[k], outs[k] + n, sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    mem.check(cudaStreamSynchronize(st));
    host_syncs++;
  }

  // Exclusive scan of n counts plus a trailing zero; returns the total.
  int scan_counts(const int *cnt, int *offs, long long n)
  {
    scan<int, false>(cnt, offs, n + 1, mem.scan_scratch(n + 1), st, &launches);
    check();
    return read_int(offs + n);
  }

  // Sorts (k32, val) of `total` packed items by energy key, then stably by
  // subhalo; returns the array holding the sorted particles.
  uint32_t *sort_energy_keys(int total)
  {
    int *table = mem.radix_table(total), *scr = mem.radix_scan_scratch(total);
    const bool flip =
      radix_sort_pairs<uint32_t>(D.k32, D.val, D.k32_alt, D.val_alt, total, 0, 32, table, scr, st, &launches,
                                 block_sort_max);
    uint32_t *v = flip ? D.val_alt : D.val;
    uint32_t *v_other = flip ? D.val : D.val_alt;
    if (S > 1 && seg_bits > 0)
    {
      k_segkeys<<<grid_for(total, 256), 256, 0, st>>>(v, D.seg_of, D.k32, total);
      launches++;
      const bool f2 =
        radix_sort_pairs<uint32_t>(D.k32, v, D.k32_alt, v_other, total, 0, seg_bits, table, scr, st, &launches,
                                   block_sort_max);
      v = f2 ? v_other : v;
    }
    check();
    return v;
  }

  // Sorts the tree keys by key, then stably by subhalo carrying the keys, and
  // leaves the result in D.key / D.val.
  void sort_tree_keys(int total)
  {
    int *table = mem.radix_table(total), *scr = mem.radix_scan_scratch(total);
    const bool flip =
      radix_sort_pairs<unsigned long long>(D.key, D.val, D.key_alt, D.val_alt, total, 0, 63, table, scr, st,
                                           &launches, block_sort_max);
    if (flip)
    {
      std::swap(D.key, D.key_alt);
      std::swap(D.val, D.val_alt);
    }
    if (S > 1 && seg_bits > 0)
    {
      k_segkeys_iota<<<grid_for(total, 256), 256, 0, st>>>(D.val, D.seg_of, D.k32, D.perm, total);
      launches++;
      const bool f2 = radix_sort_pairs<uint32_t>(D.k32, D.perm, D.k32_alt, D.perm_alt, total, 0, seg_bits, table,
                                                 scr, st, &launches, block_sort_max);
      const uint32_t *perm = f2 ? D.perm_alt : D.perm;
      k_gather_keys<<<grid_for(total, 256), 256, 0, st>>>(D.key, D.val, perm, D.key_alt, D.val_alt, total);
      launches++;
      std::swap(D.key, D.key_alt);
      std::swap(D.val, D.val_alt);
    }
    check();
  }

  // geometric: per-cell bounding boxes and leaf source indices (k_tree_bounds,
  // k_tree_leaf_ids) instead of mass moments.
  void build_tree(int src_total, bool geometric = false)
  {
    if (src_total <= 0)
      return;
    const unsigned sb = grid_for(S + 1, 256);
    mem.check(cudaMemsetAsync(D.fb_count, 0, sizeof(int), st));
    D.lvl = mem.level_counts();
    mem.check(cudaMemsetAsync(D.lvl, 0, sizeof(int) * 2 * kLevels, st));
    k_bbox<<<grid_for(src_total, 256 * kBboxRows), 256, 0, st>>>(D, src_total);
    k_root<<<sb, 256, 0, st>>>(D, K);
    k_keys<<<grid_for(src_total, 256), 256, 0, st>>>(D, src_total);
    k_keys_fallback<<<sm_count * 4, 256, 0, st>>>(D);
    launches += 4;
    check();
    sort_tree_keys(src_total);
    k_tree_count<<<grid_for(src_total + 1, 256), 256, 0, st>>>(D, src_total);
    launches++;
    check();
    // the cell total and the cells per level (k_tree_count's histogram) in one host read
    scan<int, false>(D.cnt, D.X, src_total + 1, mem.scan_scratch(src_total + 1), st, &launches);
    check();
    int counts[1 + kLevels];
    mem.check(cudaMemcpyAsync(&counts[0], D.X + src_total, sizeof(int), cudaMemcpyDeviceToHost, st));
    mem.check(cudaMemcpyAsync(&counts[1], D.lvl, sizeof(int) * kLevels, cudaMemcpyDeviceToHost, st));
    mem.check(cudaStreamSynchronize(st));
    host_syncs++;
    const int internal = counts[0];
    const int *per_level = counts + 1;
    // one padding slot after the last: the walk reads a node's second slot unconditionally
    D.nodes = mem.tree_slots((long long)src_total + 2LL * internal + 1);
    D.cell_list = mem.cell_list(internal);
    tree_nodes += internal;
    k_tree_emit<<<grid_for(src_total, 128), 128, 0, st>>>(D, K, src_total);
    launches++;
    // cell multipoles (or bounding boxes) bottom-up, one launch per non-empty
    // level, deepest first
    for (int L = 21; L >= 0; L--) // keys have 21 digits: no cell below level 21
    {
      if (per_level[L] <= 0)
        continue;
      const unsigned mg =
        std::max(1u, std::min(grid_for(per_level[L], 256), (unsigned)sm_count * (unsigned)moments_blocks_per_sm));
      if (geometric)
        k_tree_bounds<<<mg, 256, 0, st>>>(D, L);
      else
        k_tree_moments<<<mg, 256, 0, st>>>(D, L);
      launches++;
    }
    if (geometric)
    {
      k_tree_leaf_ids<<<grid_for(src_total, 256), 256, 0, st>>>(D, src_total);
      launches++;
    }
    check();
  }

  // Targets of the correction walks in key order (see k_tgt_flags); `total`
  // is the sum of sp_cnt, already scanned into sp_off.
  void correction_targets(int total)
  {
    if (total == 0)
      return;
    k_tgt_flags<<<grid_for(total + 1, 256), 256, 0, st>>>(D, total);
    launches++;
    scan<int, false>(D.flags, D.F, total + 1, mem.scan_scratch(total + 1), st, &launches);
    k_tgt_scatter<<<grid_for(total, 256), 256, 0, st>>>(D, total);
    launches++;
    check();
  }

  // One tree walk over `chunk_total` packed 32-target chunks.
  void walk(int chunk_total)
  {
    if (chunk_total <= 0)
      return;
    unsigned grid = grid_for(chunk_total, kWalkWarps);
    // ranges of `per` chunks, at most one per SM, none empty (a warp whose range is
    // done tries the following ranges one atomic each, so empty ranges cost time)
    const int per = (chunk_total + std::min(sm_count, chunk_total) - 1) / std::min(sm_count, chunk_total);
    const int nranges = (chunk_total + per - 1) / per;
    DevState Dw = D;
    if (chunk_total < walk_ranged_min)
      Dw.walk_ctr = nullptr; // a grid-stride loop, one warp per chunk
    if (Dw.walk_ctr)
    { // one resident wave over per-SM chunk ranges
      mem.check(cudaMemsetAsync(Dw.walk_ctr, 0, sizeof(unsigned) * (size_t)nranges, st));
      grid = std::min<unsigned>(grid, (unsigned)sm_count * (unsigned)walk_blocks_per_sm);
    }
    if (K.count_interactions)
      k_walk<true><<<grid, 32 * kWalkWarps, 0, st>>>(Dw, K, chunk_total, nranges);
    else
      k_walk<false><<<grid, 32 * kWalkWarps, 0, st>>>(Dw, K, chunk_total, nranges);
    launches++;
    walk_launches++;
    check();
  }

  void run()
  {
    mem.mark(-1);
    iterate();
    finish();
  }

  // The lock-step loop until no subhalo is active.
  void iterate()
  {
    const unsigned sb = grid_for(S + 1, 256);
    for (;;)
    {
      k_plan<<<sb, 256, 0, st>>>(D, K);
      launches++;
      check();
      int tot[4];
      scan_counts4(D.src_cnt, D.src_off, D.chunk_cnt, D.chunk_off, D.part_cnt, D.part_off, D.sp_cnt, D.sp_off, S, tot);
      const int src_total = tot[0], chunk_total = tot[1], part_total = tot[2], sp_total = tot[3];
      mem.mark(0);
      if (part_total == 0 && src_total == 0)
        break;
      global_iter++;
      if (K.max_sample > 0)
      { // upscale factors of the subsampled subhaloes
        k_upscale<<<(unsigned)std::min(S, 65535), 256, 0, st>>>(D, K);
        launches++;
        check();
      }
      if (src_total > 0)
        build_tree(src_total);
      if (K.max_sample > 0 && part_total > 0)
      {
        k_record_candidates<<<grid_for(part_total, 256), 256, 0, st>>>(D, part_total);
        launches++;
      }
      correction_targets(sp_total);
      mem.mark(2);
      walk(chunk_total);
      mem.mark(1);
      if (part_total > 0)
      {
        k_energy<<<grid_for(part_total, 256), 256, 0, st>>>(D, K, part_total);
        k_part_flags<<<grid_for(part_total + 1, 256), 256, 0, st>>>(D, part_total);
        launches += 2;
        check();
        scan<int, false>(D.flags, D.F, part_total + 1, mem.scan_scratch(part_total + 1), st, &launches);
        k_part_count<<<sb, 256, 0, st>>>(D);
        k_part_scatter<<<grid_for(part_total, 256), 256, 0, st>>>(D, part_total);
        k_part_copy<<<grid_for(part_total, 256), 256, 0, st>>>(D, part_total);
        k_after_part<<<sb, 256, 0, st>>>(D, K);
        k_plan_counts<<<sb, 256, 0, st>>>(D, 0); // the bound sets for the frame sums
        launches += 5;
        check();
        int tb[4];
        scan_counts4(D.tail_cnt, D.tail_off, D.fin_cnt, D.fin_off, nullptr, nullptr, nullptr, nullptr, S, tb);
        const int tail_total = tb[0], bound_total = tb[1];
        if (tail_total > 0)
        {
          k_energy_keys<<<grid_for(tail_total, 256), 256, 0, st>>>(D, D.tail_off, tail_total, 0);
          launches++;
          uint32_t *sorted = sort_energy_keys(tail_total);
          k_energy_write<<<grid_for(tail_total, 256), 256, 0, st>>>(D, sorted, D.tail_off, tail_total, 0);
          launches++;
          check();
        }
        mem.mark(3);
        if (bound_total > 0)
        {
          D.com_ipt = com_items_per_thread(bound_total); // k_control reads the partials with the same blocking
          k_com<<<grid_for((bound_total + D.com_ipt - 1) / D.com_ipt, 256), 256, 0, st>>>(D, K, bound_total);
          launches++;
        }
        k_control<<<sb, 256, 0, st>>>(D, K);
        launches++;
        check();
        mem.mark(4);
      }
    }
  }

  // Final sort of the bound sets by binding energy (and RefineBindingEnergyOrder).
  void finish()
  {
    const unsigned sb = grid_for(S + 1, 256);
    k_plan_counts<<<sb, 256, 0, st>>>(D, 1);
    launches++;
    const int fin_total = scan_counts(D.fin_cnt, D.fin_off, S);
    if (fin_total > 0)
    {
      k_energy_keys<<<grid_for(fin_total, 256), 256, 0, st>>>(D, D.fin_off, fin_total, 1);
      launches++;
      uint32_t *sorted = sort_energy_keys(fin_total);
      k_energy_write<<<grid_for(fin_total, 256), 256, 0, st>>>(D, sorted, D.fin_off, fin_total, 1);
      launches++;
      check();
    }
    if (K.max_sample > 0 && K.refine)
      refine_order();
  }

  // RefineBindingEnergyOrder for the converged subsampled subhaloes.
  void refine_order()
  {
    const unsigned sb = grid_for(S + 1, 256);
    k_plan_refine<<<sb, 256, 0, st>>>(D, K);
    launches++;
    check();
    int tot[4];
    scan_counts4(D.src_cnt, D.src_off, D.chunk_cnt, D.chunk_off, nullptr, nullptr, nullptr, nullptr, S, tot);
    const int src_total = tot[0], chunk_total = tot[1];
    if (src_total == 0)
      return;
    build_tree(src_total);
    walk(chunk_total);
    k_refine_keys<<<grid_for(src_total, 256), 256, 0, st>>>(D, K, src_total);
    launches++;
    check();
    uint32_t *sorted = sort_energy_keys(src_total);
    k_refine_write<<<grid_for(src_total, 256), 256, 0, st>>>(D, sorted, src_total);
    launches++;
    check();
  }

  // Outputs.  fin_off still packs the bound sets of the finished subhaloes.
  void epilogue(const OutPtrs &O)
  {
    const unsigned sb = grid_for(S, 256);
    k_epi_init<<<sb, 256, 0, st>>>(D);
    k_epi_order<<<grid_for(std::max<long long>(D.N, 1), 256), 256, 0, st>>>(D, O);
    launches += 2;
    const int fin_total = read_int(D.fin_off + S);
    if (fin_total > 0)
    {
      k_epi_particles<<<grid_for((fin_total + kItemsPerThread - 1) / kItemsPerThread, 256), 256, 0, st>>>(D, K, O,
                                                                                                        fin_total);
      launches++;
    }
    k_epilogue<<<sb, 256, 0, st>>>(D, K, O);
    if (O.mbound_type)
    {
      if (K.dm_only)
        mem.check(cudaMemsetAsync(O.mbound_type, 0, sizeof(float) * 6 * (size_t)S, st));
      else
      {
        k_type_masses<<<grid_for((long long)S * kWarp, 256), 256, 0, st>>>(D, O.mbound_type);
        launches++;
      }
    }
    launches++;
    check();
    mem.mark(5);
  }
};

} // namespace hbtg
