"""Benchmark: bound particles per second of batched iterative unbinding on GB300.

Workload (one "step" = one unbinding pass over one batch): the batched plain
method -- seeded synthetic NFW subhaloes with N_p ~ N^-1.9 on [20, 1e6],
c ~ logN(ln 8, 0.3), a fraction U(0, 0.5) of each heated to U(1.5, 4) v_esc,
in a 500-unit periodic box, drawn until the batch holds >= 5e7 particles.
All subhaloes are unbound in one call.  Inputs are far larger than L2.

Arms
  (default)          this library, learned warm start + batching.  `value`:
                     device-resident inputs (hbtg_unbind_batch_learned_device
                     with the shipped proposer); the plain batched GPU path
                     (hbtg_unbind_batch_device) is timed beside it on the same
                     batch ("plain", "learned_vs_plain") and judges its bound
                     mass ("dM_bound") and membership; `e2e`: the host-pointer
                     C-ABI call (hbtg_unbind_batch_learned) from pinned host
                     buffers, copies inside the timed region.
  --workload stripped  the learned warm start's evaluation set: held-out
                     tidally stripped subhaloes with a previous-output bound set.
  --impl reference   the reference CPU algorithm on the host cores: the
                     reference's own Unbind (oracle/_ref) where it was built,
                     else the project's bit-identical restatement (oracle/),
                     OpenMP over subhaloes as SubhaloSnapshot_t::RefineParticles.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "hbt-herons_gb300"))

METRIC = "bound particles/s on 1 GB300, learned+batched vs plain GPU at ΔM_bound≤1e-4"
UNIT = "bound particles/s"
FLOPS_PER_INTERACTION = 13  # 3 sub, 5 for r^2, 2 opening test, 1 rsqrt, 2 accumulate


WORKLOADS = {
    "batched": "batched method: NFW subhaloes N_p~N^-1.9 on [20,1e6] drawn to >=%.0e particles, "
               "f_unbound~U(0,0.5) heated to 1.5-4 v_esc, 500-unit periodic box",
    "stripped": "learned warm start evaluation: %d held-out tidally stripped NFW subhaloes (N_p~N^-1.9 on "
                "[20,1e6]) with a previous-output bound set, 500-unit periodic box",
    "hydro": "hydro mixed species: %.0e particles over subhaloes of N_p~N^-1.9 on [100,2e5] (55%% DM, 35%% gas with "
             "thermal energy and 0.3 v_circ rotation, 9.9%% Hernquist stars, 0.1%% BH m=50), 500-unit periodic box",
}


def workload(total, seed, kind="batched"):
    from hbtg import abi, synthetic
    if kind == "stripped":
        inp = synthetic.stripped(n_sub=int(total), seed=424242 + seed)  # seeds disjoint from the training traces
        prm = abi.parity_params(dm_only=1, box_size=500.0)
    elif kind == "hydro":
        inp = synthetic.hydro(total=total, seed=seed, nmin=100, nmax=200_000, box=500.0)
        prm = abi.parity_params(thermal=1, box_size=500.0)
    elif kind == "batched_n":  # a fixed count of 20,000 subhaloes
        inp = synthetic.batched(n_sub=20_000, seed=seed)
        prm = abi.parity_params(dm_only=1, box_size=500.0)
    else:
        inp = synthetic.batched(total=total, seed=seed)
        prm = abi.parity_params(dm_only=1, box_size=500.0)
    return inp, prm


def cpu_sample(inp, target_particles, seed=0, strict=False):
    """Particle-weighted stratified sample: the subhaloes are binned by size
    (decades of N_p); each bin gets a share of `target_particles` equal to its
    share of the batch's particles and contributes randomly chosen subhaloes
    until that share is reached (at least one per non-empty bin, so the
    largest decade is always represented; with `strict`, no bin exceeds 1.5x
    its share, so bins whose subhaloes are all larger are left out).  Returns
    (sample, picked indices)."""
    sizes = np.diff(inp.offsets)
    rng = np.random.default_rng(seed)
    dec = np.floor(np.log10(np.maximum(sizes, 1))).astype(int)
    total = max(1, int(sizes.sum()))
    pick = []
    for d in np.unique(dec):
        members = np.nonzero((dec == d) & (sizes > 0))[0]
        if not len(members):
            continue
        share = target_particles * sizes[members].sum() / total
        got = 0
        for s in rng.permutation(members):
            if got >= share and got > 0:
                break
            if (got > 0 or strict) and got + sizes[s] > 1.5 * share:
                continue
            pick.append(int(s))
            got += int(sizes[s])
    pick = np.sort(np.array(pick, np.int64))
    return inp.subset(pick), pick


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def sample_parity(sub, gpu_out, cpu_out, prm):
    """The plain GPU path's outputs on the sampled subhaloes (one call over
    the sample, potentials included) against the CPU leg's outputs on the
    same subhaloes: membership, raw bound mass, most-bound IDs, status, and
    every float output relative to its particle's potential (tests/parity.py)."""
    sys.path.insert(0, os.path.join(HERE, "tests"))
    from parity import compare, compare_full
    g = gpu_out
    m = compare(sub, g, cpu_out)
    mf, viol = compare_full(sub, g, cpu_out, prm)
    return {"subhaloes": int(sub.n_sub), "particles": int(sub.n_particles), "membership": m["membership"],
            "mass_rel": m["mass_rel"], "status_diff": len(m["status_diff"]), "mostbound_diff": len(m["mostbound_diff"]),
            "energy_rel_median": m["energy_rel_median"], "full_output_violations": len(viol),
            "violations_by_field": sorted({v[0] for v in viol}), "matched_subhaloes": mf["matched"],
            "float_outlier_fraction": mf["float_outliers"], "tail_moved": mf["tail_moved"],
            "tail_checked": mf["tail_checked"], "subresolution_exempt": mf["subres_exempt"],
            "violations": [[v[0], int(v[1]), str(v[2])[:160]] for v in viol[:6]]}


def run_cpu(inp, prm, threads, inner_parallel=False, want_potential=False):
    from hbtg import oracle
    ref = None
    try:
        lib = oracle.reference_lib("dmo" if prm.dm_only else "hydro")
        if lib is not None:
            ref = "reference"
    except Exception:
        ref = None
    t0 = time.perf_counter()
    if ref == "reference":
        out = oracle.run_reference(inp, prm, nthreads=threads, inner_parallel=inner_parallel,
                                   want_potential=want_potential)
    else:
        out = oracle.run_port(inp, prm, nthreads=threads, inner_parallel=inner_parallel, want_potential=want_potential)
    dt = time.perf_counter() - t0
    return out, dt, ref or "port"


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), "hbtg_bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        loaded = [s for s in sm if s > 0.5 * (max(sm) if sm else 1)]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(loaded)) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def bench_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    inp, prm = workload(args.total, args.seed, args.workload)
    threads = os.cpu_count() or 1
    sample, picked = cpu_sample(inp, args.ref_sample, seed=args.seed)
    for _ in range(args.warmup):
        run_cpu(sample, prm, threads)
    times, bounds, kind = [], [], "port"
    for _ in range(args.steps):
        out, dt, kind = run_cpu(sample, prm, threads, want_potential=True)
        times.append(dt)
        bounds.append(int(out.nbound.sum()))
    rate = float(np.sum(bounds) / np.sum(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload] % args.total,
                   "particles": inp.n_particles, "subhaloes": inp.n_sub},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": kind, "cpu_model": cpu_model(),
                         "sample": _sample_text(inp, sample, picked)},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "implementation": ("the reference's own Unbind, compiled from its sources (oracle/_ref)" if kind == "reference"
                           else "the oracle's restatement of the reference's Unbind (oracle/unbind_port.cpp), pinned "
                                "bit for bit to the reference's own outputs (tests/golden); the reference's own build "
                                "needs its sources, which this machine does not have"),
        "same_config": False,
        "why_sampled": "the whole batch would take hours on the host cores; each step times a particle-weighted "
                       "stratified sample of the same batch (same size distribution, largest decade included)",
    }
    print(json.dumps(line))
    return 0


def _sample_text(inp, sample, picked):
    sizes = np.diff(inp.offsets)
    return ("particle-weighted stratified sample (size decades, shares as in the batch): %d of %d subhaloes, "
            "%d of %d particles, mean N_p %.0f (batch %.0f), largest %d (batch %d); the reference's schedule "
            "(OpenMP dynamic over subhaloes)" %
            (sample.n_sub, inp.n_sub, sample.n_particles, inp.n_particles, sample.n_particles / max(1, sample.n_sub),
             inp.n_particles / max(1, inp.n_sub), int(sizes[picked].max()) if len(picked) else 0, int(sizes.max())))


def bench_gpu(args):
    import ctypes

    import torch

    from hbtg import learned
    from hbtg.abi import CallBuffers, CPrior, Inputs, _ptr
    from hbtg.build import build_library
    from hbtg.gpu import DeviceBatch, Unbinder, measure_fp32_peak

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    build_library()
    inp, prm = workload(args.total, args.seed + rank, args.workload)  # weak scaling: one full batch per GPU
    use_prior = inp.prior_nbound is not None
    model = learned.Model.load()
    u = Unbinder(local)
    model.install(u)
    db = DeviceBatch(inp, device="cuda:%d" % local)
    stream = torch.cuda.current_stream()

    def plain_step():
        db.reset_inout()
        u.unbind_device(prm, db.c, stream.cuda_stream)

    def learned_step():
        db.reset_inout()
        u.unbind_learned_device(prm, db, stream.cuda_stream, use_prior=use_prior)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def timed(step):
        """W warm-up steps, one untimed counted pass, K timed steps (CUDA events)."""
        for _ in range(max(3, args.warmup)):
            step()
        u.count_interactions(True)
        step()
        counted = u.stats()
        u.count_interactions(False)
        acc = dict(ms_walk=0.0, walk_launches=0, kernel_launches=0, total_bound=0)
        st = None
        with Clocks(local) as clk:
            barrier()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(args.steps):
                step()
                st = u.stats()
                for k in acc:
                    acc[k] += st[k]
            ev1.record(stream)
            barrier()
        ms = ev0.elapsed_time(ev1)
        t_max, bound_all = ms, acc["total_bound"]
        if world > 1:
            t_max = _max_over_ranks(ms)
            bound_all = _sum_over_ranks(bound_all)
        return dict(ms=ms, t_max=t_max, bound_all=bound_all, value=bound_all / (t_max * 1e-3), counted=counted,
                    clocks=clk.summary(), last=st, **acc)

    plain = timed(plain_step) if args.arm in ("both", "plain") else None
    plain_out = db.outputs() if plain else None
    if args.arm == "plain":  # profile the plain arm alone: report it as the line's value
        warm, warm_out = plain, plain_out
    else:
        warm = timed(learned_step)
        warm_out = db.outputs()
    dm = memb = None
    if plain and args.arm == "both":
        m_plain = float(np.sum(plain_out.mbound.astype(np.float64)))
        m_warm = float(np.sum(warm_out.mbound.astype(np.float64)))
        dm = abs(m_warm - m_plain) / max(m_plain, 1e-30)
        memb = _membership(inp, warm_out, plain_out)

    # end to end through the learned host-pointer C-ABI call: pinned host
    # buffers, host<->device copies inside the timed region
    pinned = {}

    def pin(a):
        if a is None:
            return None
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        arr = t.numpy()
        arr[...] = a
        pinned[id(arr)] = t
        return arr

    hin = Inputs(inp.offsets, pin(inp.pos), pin(inp.vel), pin(inp.mass), pin(inp.id), None, None,
                 pin(inp.ref_pos), pin(inp.ref_vel), pin(inp.mostbound_pos), pin(inp.mostbound_vel),
                 pin(inp.most_bound_id), {}, pin(inp.prior_nbound), pin(inp.prior_energy))
    buf = CallBuffers(hin, want_energy=True)
    # every host array the call reads or writes is pinned (the in/out frames
    # too: a pageable copy makes the driver stage it and can stall the stream)
    for name in ("order", "energy", "nbound", "mbound", "tracer_index", "iterations", "status", "kinematics", "core",
                 "nbound_type", "mbound_type", "ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel", "most_bound_id"):
        setattr(buf.out, name, pin(getattr(buf.out, name)))
    buf = _rebind(buf)
    prior = CPrior(_ptr(hin.prior_nbound), _ptr(hin.prior_energy))

    def e2e_call():
        rc = u.lib.hbtg_unbind_batch_learned(u.h, ctypes.byref(prm), ctypes.byref(buf.c), ctypes.byref(prior))
        assert rc in (0, 4), rc

    e2e_call()  # warm the host path once
    link = host_link_rates("cuda:%d" % local, u.stats()["h2d_bytes"], u.stats()["d2h_bytes"], args.steps)
    e2e_times, e2e_device, e2e_h2d, e2e_d2h, h2d, d2h = [], [], [], [], 0, 0
    for _ in range(args.steps):
        _reset_frames(buf, hin)
        barrier()
        t0 = time.perf_counter()
        e2e_call()
        e2e_times.append(time.perf_counter() - t0)
        st = u.stats()
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
        e2e_device.append(st["ms_total"])
        e2e_h2d.append(st["ms_h2d"])
        e2e_d2h.append(st["ms_d2h"])
    t_e2e = float(np.mean(e2e_times))
    if world > 1:
        t_e2e = _max_over_ranks(t_e2e)
    e2e_value = (warm["bound_all"] / args.steps) / t_e2e
    h2d_ms = float(np.mean([x for x in e2e_h2d])) if e2e_h2d else None
    d2h_ms = float(np.mean([x for x in e2e_d2h])) if e2e_d2h else None

    # the literal configuration of the workload's description: 20,000 subhaloes
    # (about 7e6 particles), both arms, device-resident inputs
    literal = None
    if args.workload == "batched" and not args.skip_literal and rank == 0:
        lit_inp, _ = workload(0, args.seed + 7, "batched_n")
        lit_db = DeviceBatch(lit_inp, device="cuda:%d" % local)
        lit = {}
        for arm in ("plain", "learned"):
            def lit_step(arm=arm):
                lit_db.reset_inout()
                if arm == "plain":
                    u.unbind_device(prm, lit_db.c, stream.cuda_stream)
                else:
                    u.unbind_learned_device(prm, lit_db, stream.cuda_stream, use_prior=False)
            for _ in range(max(3, args.warmup)):
                lit_step()
            bound = 0
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(args.steps):
                lit_step()
                bound += u.stats()["total_bound"]
            e1.record(stream)
            torch.cuda.synchronize()
            lit[arm] = bound / (e0.elapsed_time(e1) * 1e-3)
        literal = {"n_sub": int(lit_inp.n_sub), "particles": int(lit_inp.n_particles), "learned": lit["learned"],
                   "plain": lit["plain"], "learned_vs_plain": lit["learned"] / lit["plain"]}
        del lit_db

    # the other two workloads of the method at their own sizes (hydro mixed
    # species with thermal energy; held-out stripped subhaloes with a
    # previous-output prior), both arms, with parity against the CPU oracle
    # on a sample of each
    side = {}
    if args.workload == "batched" and not args.skip_side and rank == 0:
        for kind in ("hydro", "stripped"):
            side[kind] = side_workload(kind, u, args, local, stream)

    # roofline of the dominant kernel (the tree walk) in the learned arm
    peak = measure_fp32_peak(local)
    walk_ms_per_launch = warm["ms_walk"] / max(1, warm["walk_launches"])
    cw = warm["counted"]
    flops_per_launch = cw["interactions"] * FLOPS_PER_INTERACTION / max(1, cw["walk_launches"])
    achieved = flops_per_launch / (walk_ms_per_launch * 1e-3) / 1e12
    traffic = _walk_traffic(cw)
    issue = _walk_issue()

    cpu = parity = None
    if rank == 0 and not args.skip_cpu:
        sample, picked = cpu_sample(inp, args.cpu_sample, seed=args.seed)
        threads = os.cpu_count() or 1
        out, dt, kind = run_cpu(sample, prm, threads, want_potential=True)
        # one thread on about 1e5 particles (the same stratification; decades
        # whose subhaloes exceed their share are left out)
        small, _ = cpu_sample(inp, 100_000, seed=args.seed + 1, strict=True)
        out1, dt1, _ = run_cpu(small, prm, 1)
        cpu = {"value": float(out.nbound.sum() / dt), "unit": UNIT, "cores": threads, "kind": kind,
               "cpu_model": cpu_model(), "sample": _sample_text(inp, sample, picked) + ", %.1f s" % dt,
               "one_thread": {"value": float(out1.nbound.sum() / dt1), "particles": int(small.n_particles),
                              "subhaloes": int(small.n_sub), "largest": int(np.diff(small.offsets).max()),
                              "seconds": dt1}}
        if plain_out is not None:
            g = u.unbind(sample, prm, want_potential=True)
            parity = sample_parity(sample, g, out, prm)
            parity["against"] = "plain GPU path vs CPU %s on the sampled subhaloes" % kind

    if rank == 0:
        last = warm["last"]
        line = {
            "metric": METRIC, "value": warm["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": warm["t_max"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (walk) / f64 (reductions) / bf16 (proposer)",
            "data": "synthetic (seeded NFW subhaloes)",
            "config": {"workload": WORKLOADS[args.workload] % args.total,
                       "particles_per_gpu": inp.n_particles, "subhaloes_per_gpu": inp.n_sub,
                       "bound_per_gpu_step": warm["total_bound"] / args.steps, "open_angle": 0.45,
                       "softening": 0.005, "bound_mass_precision": 0.995, "max_sample_size": 0,
                       "l2": "inputs larger than L2 (%.1f GB of particle data)" % (inp.n_particles * 44 / 1e9),
                       "proposer": {"threshold": model.threshold, "exclude_below": model.exclude_below,
                                    "first_test": model.first_test, "min_particles": model.min_particles,
                                    "trained_on": {k: model.meta.get(k) for k in ("n_sub_stripped", "n_batched",
                                                                                  "rows", "steps")}},
                       "global_iterations": {"learned": cw["global_iterations"],
                                             "plain": plain and plain["counted"]["global_iterations"]},
                       "interactions_per_step": {"learned": cw["interactions"],
                                                 "plain": plain and plain["counted"]["interactions"]},
                       "walk_traversal_per_step": {k[5:]: cw[k] for k in (
                           "walk_steps", "walk_nodes", "walk_pending_batches", "walk_entries_full",
                           "walk_entries_part", "walk_entries_near", "walk_drained")},
                       "walk_cycles_per_step": dict(zip(("pop", "resolve", "write", "eval_full", "eval_far",
                                                         "eval_near", "drain", "groups"), cw["walk_cycles"])),
                       "arm": args.arm, "parallelism": "dp%d" % world},
            "plain": plain and {"value": plain["value"], "ms_per_step": plain["t_max"] / args.steps,
                                "bound_per_step": plain["total_bound"] / args.steps,
                                "ms_walk_per_step": plain["ms_walk"] / args.steps,
                                "gpu_launches": plain["kernel_launches"] // args.steps},
            "learned_vs_plain": (warm["value"] / plain["value"]) if plain and args.arm == "both" else None,
            "dM_bound": dm, "membership_vs_plain": memb,
            "warm_start": {k: last[k] for k in ("warm_subhaloes", "excluded", "readmitted", "cold_restarts",
                                                "ms_propose", "ms_walk", "ms_tree", "ms_part", "ms_frame",
                                                "ms_plan", "ms_final")},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "call": "hbtg_unbind_batch_learned (host pointers, pinned)",
                    "ms_per_call": 1e3 * float(np.mean(e2e_times)),
                    "ms_device_part": float(np.mean(e2e_device)), "ms_uploads": h2d_ms, "ms_downloads": d2h_ms,
                    "ms_uploads_each": [round(x, 2) for x in e2e_h2d],
                    "ms_downloads_each": [round(x, 2) for x in e2e_d2h],
                    "value_best_call": (warm["bound_all"] / args.steps) / float(np.min(e2e_times)),
                    "host_link": link},
            "gpu_launches": warm["kernel_launches"] // args.steps,
            "host_syncs_per_step": warm["last"].get("host_syncs"),
            "roofline": {"kernel": "k_walk", "bound": "fp32", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": "FP32 FMA throughput measured in-process (hbtg_measure_fp32_peak)",
                         "flops_per_launch": flops_per_launch, "ms_per_launch": walk_ms_per_launch,
                         "blocks_per_sm": warm["last"].get("walk_blocks_per_sm"),
                         "issue_active_ncu": issue,
                         "bound_note": "the walk is issue-bound (instruction issue slots, not the FP32 pipe): "
                                       "issue_active_ncu is its ncu issue-slot utilisation",
                         "walk_share_of_step": warm["ms_walk"] / max(warm["ms"], 1e-9)},
            "cpu_baseline": cpu,
            "parity": parity,
            "literal_20000": literal,
            "hydro": side.get("hydro"),
            "stripped": side.get("stripped"),
            "clocks": warm["clocks"],
            "clocks_plain": plain and plain["clocks"],
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    u.close()
    return 0


def side_workload(kind, u, args, local, stream):
    """Both GPU arms on one more workload at its own size (device-resident
    inputs, CUDA events over `args.steps` steps after 3 warm-up steps), the
    learned arm's bound-mass and membership error against the plain arm, and
    the plain arm's parity against the CPU oracle on a particle-weighted
    sample of about 2e5 particles."""
    import torch
    from hbtg.gpu import DeviceBatch
    total = {"stripped": 20000, "hydro": 4e6}[kind]
    inp, prm = workload(total, args.seed, kind)
    use_prior = inp.prior_nbound is not None
    db = DeviceBatch(inp, device="cuda:%d" % local)
    res = {"workload": WORKLOADS[kind] % total, "particles": int(inp.n_particles), "subhaloes": int(inp.n_sub)}
    outs = {}
    for arm in ("plain", "learned"):
        def step(arm=arm):
            db.reset_inout()
            if arm == "plain":
                u.unbind_device(prm, db.c, stream.cuda_stream)
            else:
                u.unbind_learned_device(prm, db, stream.cuda_stream, use_prior=use_prior)
        for _ in range(3):
            step()
        bound = 0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
            bound += u.stats()["total_bound"]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res[arm] = {"value": bound / args.steps / (ms * 1e-3), "ms_per_step": ms,
                    "global_iterations": u.stats()["global_iterations"]}
        outs[arm] = db.outputs()
    res["learned_vs_plain"] = res["learned"]["value"] / res["plain"]["value"]
    m_plain = float(np.sum(outs["plain"].mbound.astype(np.float64)))
    m_warm = float(np.sum(outs["learned"].mbound.astype(np.float64)))
    res["dM_bound"] = abs(m_warm - m_plain) / max(m_plain, 1e-30)
    res["membership_vs_plain"] = _membership(inp, outs["learned"], outs["plain"])
    del db
    if not args.skip_cpu:
        sample, picked = cpu_sample(inp, 200_000, seed=args.seed + 2)
        out, dt, kind_cpu = run_cpu(sample, prm, os.cpu_count() or 1, want_potential=True)
        g = u.unbind(sample, prm, want_potential=True)
        res["parity"] = sample_parity(sample, g, out, prm)
        res["parity"]["against"] = "plain GPU path vs CPU %s on the sampled subhaloes" % kind_cpu
        res["cpu"] = {"value": float(out.nbound.sum() / dt), "cores": os.cpu_count() or 1, "kind": kind_cpu,
                      "sample": _sample_text(inp, sample, picked)}
    return res


def host_link_rates(device, up_bytes, down_bytes, reps):
    """Plain pinned copies of the e2e call's byte counts (one cudaMemcpyAsync
    each way, CUDA events), repeated: the host link's own rate at the time of
    the e2e calls, which shares the link with the machine's other GPUs."""
    import torch
    up = torch.empty(int(up_bytes), dtype=torch.uint8, pin_memory=True)
    down = torch.empty(int(down_bytes), dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(int(max(up_bytes, down_bytes)), dtype=torch.uint8, device=device)
    up.fill_(1)
    ups, downs = [], []
    for _ in range(max(3, reps)):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record()
        dev[:up.numel()].copy_(up, non_blocking=True)
        e[1].record()
        down.copy_(dev[:down.numel()], non_blocking=True)
        e[2].record()
        torch.cuda.synchronize()
        ups.append(e[0].elapsed_time(e[1]))
        downs.append(e[1].elapsed_time(e[2]))
    del up, down, dev
    return {"h2d_GBs_each": [round(up_bytes / (t * 1e-3) / 1e9, 1) for t in ups],
            "d2h_GBs_each": [round(down_bytes / (t * 1e-3) / 1e9, 1) for t in downs],
            "note": "plain pinned copies of the same byte counts just before the e2e calls"}


def _membership(inp, got, ref):
    """Bound-membership mismatch sum_s |B xor B'| / sum_s |B'| (vectorised)."""
    seg = np.repeat(np.arange(inp.n_sub), np.diff(inp.offsets))
    local = np.arange(inp.n_particles) - inp.offsets[seg]

    def bound_mask(out):
        pos = np.empty(inp.n_particles, np.int64)
        pos[inp.offsets[seg] + out.order] = local  # position of each input particle
        return pos < out.nbound[seg]

    a, b = bound_mask(got), bound_mask(ref)
    return float(np.sum(a ^ b) / max(1, np.sum(b)))


def _rebind(buf):
    from hbtg.abi import _ptr
    o = buf.out
    c = buf.c
    c.order, c.energy, c.nbound, c.mbound = _ptr(o.order), _ptr(o.energy), _ptr(o.nbound), _ptr(o.mbound)
    c.tracer_index, c.iterations, c.status = _ptr(o.tracer_index), _ptr(o.iterations), _ptr(o.status)
    c.kinematics, c.core, c.nbound_type, c.mbound_type = _ptr(o.kinematics), _ptr(o.core), _ptr(o.nbound_type), \
        _ptr(o.mbound_type)
    c.ref_pos, c.ref_vel, c.mostbound_pos = _ptr(o.ref_pos), _ptr(o.ref_vel), _ptr(o.mostbound_pos)
    c.mostbound_vel, c.most_bound_id = _ptr(o.mostbound_vel), _ptr(o.most_bound_id)
    return buf


def _reset_frames(buf, hin):
    buf.out.ref_pos[...] = hin.ref_pos
    buf.out.ref_vel[...] = hin.ref_vel
    buf.out.mostbound_pos[...] = hin.mostbound_pos
    buf.out.mostbound_vel[...] = hin.mostbound_vel
    buf.out.most_bound_id[...] = hin.most_bound_id


def _reduce_device():
    """The device the process group reduces on: the GPU for NCCL, the host for gloo."""
    import torch.distributed as dist
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def _sum_over_ranks(x):
    """Sum of x over the ranks (weak scaling: every rank's bound particles)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=_reduce_device(), dtype=torch.float64)
    dist.all_reduce(t)
    return float(t.item())


def _max_over_ranks(x):
    """Max of x over the ranks (the slowest rank's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=_reduce_device(), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _walk_issue():
    """The walk's issue-slot utilisation (%) from the committed ncu summary, or None."""
    path = os.path.join(HERE, "profiles", "k_walk_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f).get("issue_active_pct")


def _walk_traffic(counted):
    """DRAM bytes per walk launch from the committed ncu summary of k_walk,
    scaled from the captured case to this one by interactions per launch."""
    path = os.path.join(HERE, "profiles", "k_walk_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    per_interaction = d["dram_bytes_per_launch"] / max(1.0, d["interactions_per_launch"])
    return per_interaction * counted["interactions"] / max(1, counted["walk_launches"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched", choices=sorted(WORKLOADS))
    ap.add_argument("--arm", default="both", choices=["both", "learned", "plain"],
                    help="time both GPU arms (default) or one alone (for profiling)")
    ap.add_argument("--total", type=float, default=None,
                    help="particles per batch (batched; default 5e7) or subhaloes (stripped; default 20000)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample", type=float, default=1e6, help="particles in the CPU baseline sample")
    ap.add_argument("--ref-sample", type=float, default=4e5, help="particles per reference-arm step")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-literal", action="store_true", help="skip the literal 20,000-subhalo timing")
    ap.add_argument("--skip-side", action="store_true", help="skip the hydro and stripped side workloads")
    ap.add_argument("--autotune", action="store_true",
                    help="only run the launch-settings autotuner (hbtg_autotune) on the workload and print its table")
    args = ap.parse_args()
    if args.total is None:
        args.total = {"stripped": 20000, "hydro": 4e6}.get(args.workload, 5e7)
    args.total = int(args.total)
    args.cpu_sample = int(args.cpu_sample)
    args.ref_sample = int(args.ref_sample)
    if args.impl == "reference":
        return bench_reference(args)
    if args.autotune:
        return autotune_table(args)
    return bench_gpu(args)


def autotune_table(args):
    """hbtg_autotune on the workload (plain path, device-resident inputs): one
    JSON line with every candidate's time and the setting it keeps."""
    import torch
    from hbtg.gpu import DeviceBatch, Unbinder
    inp, prm = workload(args.total, args.seed, args.workload)
    u = Unbinder(0)
    db = DeviceBatch(inp, device="cuda:0")
    db.reset_inout()
    report = u.autotune(prm, db.c, torch.cuda.current_stream().cuda_stream)
    print(json.dumps({"workload": WORKLOADS[args.workload] % args.total, "particles": int(inp.n_particles),
                      "candidates": report, "kept": u.tuning()}))
    u.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
