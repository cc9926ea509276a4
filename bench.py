"""Benchmark of the MLEM hot path on the full workload (one JSON line).

Workload ("full"): two 13x13-crystal heads 500 mm apart, 180 angles in 2
degree steps (5,140,980 channels), 52^3 voxels of 2 mm, 100 Monte-Carlo rays
per channel, 20 MLEM iterations; seeded synthetic phantom (cylinder + 3 hot
spheres) forward-projected with an independent ray seed, Poisson noise at
5e8 counts; measured rows = channels with counts > 0.

A step is one complete reconstruction through the library: the system
matrix of the measured rows built on the fly (rays -> walks -> CSR), its
column-major copy, and 20 MLEM iterations (forward product, ratio,
transpose product, update, normalisation).  The metric is MLEM iterations
per second of that step: 20 / step time, the matrix build included.  The
sensitivity image and the measurement are inputs (the reference reads them
from files).  Beside it the line carries:
  rebuild_per_iteration  the reference's own schedule (the matrix recomputed
                         in every iteration) on the GPU, matrix-free;
  parity_fp64            the image of every iteration of the FP32, BF16 and
                         FP16 forms against the FP64 oracle on the host;
  sm_build_steps         ray-voxel steps (grid cells crossed by all rays)
                         per second of the system-matrix build;
  forms, batched         the 16-bit value forms and batched reconstructions;
  cpu_baseline           the oracle on the host cores, same schedule.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With torchrun (N > 1) every rank reconstructs its own copy of the workload
(replicas): the step time is the max over ranks and the value counts all
ranks' iterations.  With --sharded the ranks share ONE reconstruction (its
measured rows split over the ranks, the correction image all-reduced over
NCCL in every iteration) and the value is that reconstruction's it/s.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLEM it/s (52^3 vox, 5.1M ch)"
UNIT = "it/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="full", choices=["full", "small"])
    ap.add_argument("--cpu-sample", type=int, default=4096,
                    help="channels in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=64, metavar="N",
                    help="problems of the batched-reconstruction measurement (0: skip)")
    ap.add_argument("--batch-gb", type=float, default=200.0,
                    help="device memory budget of the batched problems' matrices")
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched-reconstruction measurement")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the 16-bit value forms")
    ap.add_argument("--no-rebuild", action="store_true",
                    help="skip the matrix-free (rebuild every iteration) schedule")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the per-iteration image error against the FP64 oracle")
    ap.add_argument("--sharded", action="store_true",
                    help="with N > 1 ranks: ONE reconstruction whose measured rows are split "
                         "over the ranks (NCCL all-reduce of the correction image per "
                         "iteration; strong scaling) instead of N replicas")
    ap.add_argument("--profile", action="store_true",
                    help="one reconstruction with one iteration, nothing else (for ncu)")
    ap.add_argument("--profile-kernels", type=int, default=0, metavar="ROWS",
                    help="a reconstruction of the first ROWS channels of the workload (build, "
                         "column-major copy) and one MLEM iteration (small case for full ncu "
                         "captures)")
    ap.add_argument("--profile-16bit", action="store_true",
                    help="with --profile-kernels: also one iteration of the BF16 form")
    return ap.parse_args()


# --------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clocks/throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        # the raw samples (EPET_CLOCKS_DIR keeps them; the line carries the summary)
        import tempfile
        d = os.environ.get("EPET_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"epet_clocks_rank{index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------ CPU baseline

def cpu_baseline(cfg_name: str, sample: int, seed: int = 0):
    """The oracle (plain C restatement of the reference's work for the path,
    OpenMP over host cores) on a seeded sample of channels: the reference's
    dense candidate scan over all voxels plus the nrays-ray values of every
    candidate (the system-matrix build), and the forward and transpose
    products over those rows (replicated to a few tens of millions of
    non-zeros, beyond the caches).  Per-row costs are scaled to the measured
    rows (estimated from the sample) for two schedules: the matrix built
    once per step and iterated (the schedule of the GPU arm's `value`), and
    the reference's own loop, which rebuilds the matrix in every iteration
    (reco.cu:216-254)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    from epetreco_gb300.phantom import phantom_image
    from epetreco_gb300.problem import config
    cfg = config(cfg_name)
    p, nit = cfg["problem"], cfg["iterations"]
    o = Oracle()
    rng = np.random.default_rng(seed)
    rows = np.sort(rng.choice(p.nchannels, sample, replace=False)).astype(np.int32)
    rnd = rng.random((sample, p.nrays, 6)).astype(np.float32)
    rnd[rnd == 0] = 1.0
    x_true = phantom_image(p, 1)
    t0 = time.perf_counter()
    rp, col, val = o.sm_build_csr(p, rows, p.nrays, rnd, exact=False)
    t_build = time.perf_counter() - t0
    reps = max(1, int(2e7 // max(1, len(col))))
    lens = np.tile(np.diff(rp), reps)
    rpb = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    colb, valb = np.tile(col, reps), np.tile(val, reps)
    t0 = time.perf_counter()
    yb = o.csrmv(0, rpb, colb, valb, x_true, p.nvoxels)
    e = np.where(yb > 0, 1.0 / np.maximum(yb, 1e-30), 0).astype(np.float32)
    o.csrmv(1, rpb, colb, valb, e, p.nvoxels)
    t_prod = (time.perf_counter() - t0) / reps
    measured_frac = max(float((yb[:sample] > 0).mean()), 1.0 / sample)
    m_est = measured_frac * p.nchannels
    t_once = m_est / sample * (t_build + nit * t_prod)
    t_rebuild = m_est / sample * nit * (t_build + t_prod)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": nit / t_once, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"{sample} seeded channels of the {cfg_name} workload: candidate scan + "
                       f"{p.nrays}-ray values ({t_build:.1f} s), forward/transpose products "
                       f"({t_prod * 1e3:.1f} ms per pass over the sample, timed on {reps} "
                       f"copies); scaled to {m_est:.0f} measured rows, matrix built once and "
                       f"{nit} iterations"),
            "rebuild_per_iteration": nit / t_rebuild,
            "sample_seconds": t_build + reps * t_prod}


def aggregate_replicas(times, nit, world, dist, device, sharded=False):
    """Each time is the max over ranks.  Replicas (every rank ran the whole
    workload): the whole-job rate is world * nit / that time; one sharded
    reconstruction: nit / that time."""
    import torch
    vals = torch.tensor([float(t) for t in times], device=device, dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(vals, op=dist.ReduceOp.MAX)
    tmax = [float(v) for v in vals]
    k = 1 if sharded else world
    return tmax, [k * nit / t for t in tmax]


def workload_name(cfg_name: str) -> str:
    """The workload as both arms name it in `config`."""
    from epetreco_gb300.problem import config
    cfg = config(cfg_name)
    p = cfg["problem"]
    return (f"{cfg_name}: {p.grid.n[0]}^3 voxels x {p.nchannels} channels, {p.nrays} rays, "
            f"{cfg['iterations']} iterations per step")


SCHEDULE = ("a step = one reconstruction: the system matrix of the measured rows built once, "
            "then the workload's iterations")
REBUILD = ("the reference's own loop (reco.cu:216-254): the system matrix recomputed in every "
           "iteration")


def reference_arm(args):
    """--impl reference: the reference's CPU work for the path (oracle port;
    the reference's own sources are not available where the bench runs), on
    the same workload and schedule as the GB300 arm."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    per, reb = [], []
    if args.warmup > 0:
        cpu_baseline(args.config, max(4, args.cpu_sample // 16), seed=99)
    info = None
    for k in range(args.steps):
        info = cpu_baseline(args.config, args.cpu_sample, seed=k)
        per.append(info["value"])
        reb.append(info["rebuild_per_iteration"])
    v = sorted(per)[len(per) // 2]
    from epetreco_gb300.problem import config
    nit = config(args.config)["iterations"]
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1000.0 * nit / v if v else None, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": workload_name(args.config)},
           "schedule": SCHEDULE,
           "rebuild_per_iteration": {"value": sorted(reb)[len(reb) // 2], "unit": UNIT,
                                     "schedule": REBUILD},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"],
                            "kind": info["kind"], "sample": info["sample"]},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ GB300

def batch_measure(args, api, torch, st, nit: int = 10, grids=None, angles=None):
    """Batched form: args.batch seeded problems of uneven size (grids and
    angle counts drawn from the batched workload's sets), each with its own
    phantom and Poisson measurement.  Times nit iterations of all problems
    through the batched launches (one CUDA graph per iteration) against the
    same problems iterated one after another with the plain per-problem
    driver (its own graph per problem), on the same device arrays."""
    from epetreco_gb300.phantom import measurement, phantom_image
    from epetreco_gb300.problem import batch_members
    torch.cuda.empty_cache()
    api.trim_memory()
    t0 = time.perf_counter()
    from epetreco_gb300.problem import BATCH_ANGLES, BATCH_GRIDS
    grids = grids or BATCH_GRIDS
    angles = angles or BATCH_ANGLES
    members = batch_members(args.batch, grids=grids, angles=angles)
    # Problems are taken in draw order while their estimated matrix bytes fit
    # the budget: the grouped layout holds 6 bytes per non-zero (value and
    # group-local column rank; the CSR + column-major copy would need 16);
    # non-zeros per row from 512 sampled measured rows.
    free, _ = torch.cuda.mem_get_info()
    budget = min(args.batch_gb * 1e9, 0.75 * free)
    probs, used, skipped = [], 0.0, 0
    for b in members:
        q = b.problem
        rows, y, _ = measurement(q, b.counts, seed=b.poisson_seed,
                                 x_true=phantom_image(q, b.phantom_seed, b.n_spheres))
        m = rows.numel()
        smp = rows[torch.linspace(0, max(m - 1, 0), min(m, 512), device=rows.device).long()]
        est = 0.0
        if m:
            est = 6.0 * api.systemMatrixCalculation(q, smp).nnz / smp.numel() * m
        if used + est > budget:
            skipped += 1
            continue
        used += est
        probs.append((q, rows, y, api.sensitivity(q)))
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    B = api.MlemBatch(probs, use_graph=True, autotune=True)
    torch.cuda.synchronize()
    t_create = time.perf_counter() - t0
    stats = B.stats()
    views = [B.member(i) for i in range(len(probs))]
    B.iterate(1)
    for v in views:
        v.iterate(1)
    torch.cuda.synchronize()

    def timed(fn, reps=3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(reps):
            fn()
        b.record(st)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1000.0 / reps

    def seq():
        for v in views:
            v.iterate(nit)

    t_batch = timed(lambda: B.iterate(nit))
    t_seq = timed(seq)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    gbs = stats["bytes_per_iteration"] * nit / t_batch / 1e9
    out = {"problems": len(probs), "drawn": len(members), "skipped_for_memory": skipped,
           "iterations": nit,
           "workload": (f"{len(members)} seeded draws (grids {sorted(set(grids))}^3, angles "
                        f"{sorted(set(angles))}, 20-100 rays, 1e5-1e8 counts, FP32 values); "
                        f"the {len(probs)} whose matrices fit {budget / 1e9:.0f} GB, in draw "
                        f"order"),
           "layout": "grouped (6 bytes per non-zero)",
           "grids": [q.grid.n[0] for q, *_ in probs], "angles": [q.setup.na for q, *_ in probs],
           "measured_rows": int(sum(r.numel() for _, r, _, _ in probs)),
           "nnz": stats["nnz"], "plan": stats["plan"],
           "batched_ms": 1000 * t_batch, "sequential_plain_ms": 1000 * t_seq,
           "speedup_vs_plain": t_seq / t_batch,
           "problem_iterations_per_s": len(probs) * nit / t_batch,
           "gbs": gbs, "frac_of_hbm_peak": gbs / peak,
           "setup_s": {"data": t_data, "create": t_create}}
    del views
    B.close()
    return out


def gb300_arm(args):
    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from epetreco_gb300 import api, build, phantom
    from epetreco_gb300._lib import lib
    from epetreco_gb300.problem import config
    build.build()
    cfg = config(args.config)
    p, nit, counts = cfg["problem"], cfg["iterations"], cfg["counts"]
    L = lib()

    if args.profile_kernels:
        # the reconstruction's own products: rows in crystal-pair order, the
        # fused MLEM epilogues, the tuned launch plans; the iterations run in
        # the NVTX range "mlem_iteration" (ncu --nvtx-include skips the tuning)
        rows = torch.arange(args.profile_kernels, dtype=torch.int32, device="cuda")
        yk = torch.ones(rows.numel(), device="cuda")
        sk = torch.ones(p.nvoxels, device="cuda")
        R = api.Mlem(p, rows, yk, sk, use_graph=False, autotune=True)
        torch.cuda.nvtx.range_push("mlem_iteration")
        R.iterate(1)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        nnz = R.stats()["nnz"]
        R.close()
        if args.profile_16bit:
            R16 = api.Mlem(p, rows, yk, sk, use_graph=False, value_format=api.BF16)
            torch.cuda.nvtx.range_push("mlem_iteration")
            R16.iterate(1)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            R16.close()
        torch.cuda.synchronize()
        print(json.dumps({"profile_kernels": args.profile_kernels, "nnz": nnz}))
        return

    if args.batch_only:
        cs = torch.cuda.current_stream()
        print(json.dumps({"batched": batch_measure(args, api, torch, cs),
                          "batched_small": batch_measure(args, api, torch, cs, grids=(24, 32),
                                                         angles=(8,))}), flush=True)
        return

    # ---- inputs (not timed): measurement and sensitivity
    rows, y, _ = phantom.measurement(p, counts)
    s = api.sensitivity(p)
    torch.cuda.synchronize()
    m = rows.numel()
    rows_h = rows.cpu().pin_memory()
    y_h = y.cpu().pin_memory()
    s_h = s.cpu().pin_memory()
    x_h = torch.empty(p.nvoxels, dtype=torch.float32).pin_memory()
    st = torch.cuda.current_stream()

    it_events = []

    sharded = args.sharded and world > 1

    def step(r, yy, ss, record=False):
        if sharded:
            from epetreco_gb300.shard import ShardedMlem
            R = ShardedMlem(p, r, yy, ss, use_graph=True, autotune=True)
        else:
            R = api.Mlem(p, r, yy, ss, use_graph=True, autotune=True)
        if record:
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            R.iterate(nit)
            b.record(st)
            it_events.append((a, b))
        else:
            R.iterate(nit)
        return R

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    if args.profile:
        R = api.Mlem(p, rows, y, s, use_graph=False)
        R.iterate(1)
        torch.cuda.synchronize()
        print(json.dumps({"profile": True, "nnz": R.stats()["nnz"]}))
        R.close()
        return

    for _ in range(args.warmup):
        R = step(rows, y, s)
        R.close()
    barrier()

    # ---- timed: device-resident inputs
    clk = ClockSampler(local)
    clk.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    n0 = L.epet_launch_count()
    barrier()
    ev0.record(st)
    for _ in range(args.steps):
        R = step(rows, y, s, record=True)
        R.close()
    ev1.record(st)
    barrier()
    launches = (L.epet_launch_count() - n0) // args.steps
    t_step = ev0.elapsed_time(ev1) / 1000.0 / args.steps
    clocks = clk.stop()
    # MLEM iterations inside the timed steps (CUDA events on the launch stream)
    t_it_live = sum(a.elapsed_time(b) for a, b in it_events) / 1000.0 / (args.steps * nit)

    # ---- e2e: host buffers through the public API
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(st)
    for _ in range(args.steps):
        r_d = rows_h.to("cuda", non_blocking=True)
        y_d = y_h.to("cuda", non_blocking=True)
        s_d = s_h.to("cuda", non_blocking=True)
        R = step(r_d, y_d, s_d)
        x_h.copy_(R.image(), non_blocking=True)
        R.close()
    e1.record(st)
    barrier()
    t_e2e = e0.elapsed_time(e1) / 1000.0 / args.steps

    # ---- breakdown of the step's parts and the product kernels (after the
    # timed region, same stream)
    R = api.Mlem(p, rows, y, s, use_graph=True, autotune=True)
    stats = R.stats()
    plan = R.plan()
    nnz = stats["nnz"]
    bytes_it = stats["bytes_per_iteration"]
    A = api.systemMatrixCalculation(p, rows, cap=nnz)
    torch.cuda.synchronize()

    def timeit(fn, reps=3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        fn()
        torch.cuda.synchronize()
        a.record(st)
        for _ in range(reps):
            fn()
        b.record(st)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1000.0 / reps

    c0 = api.build_counters()
    t_build = timeit(lambda: api.systemMatrixCalculation(p, rows, cap=nnz), reps=1)
    c1 = api.build_counters()
    # rows of one build redone with their exact window size (timeit runs it twice)
    build_rows = {k: (c1[k] - c0[k]) // 2 for k in c0}
    steps = api.ray_steps(p, rows)
    t_csc = timeit(lambda: api.csr_to_csc(A), reps=1)
    At = api.csr_to_csc(A)
    x = torch.full((p.nvoxels,), 1.0 / p.nvoxels, device="cuda")
    e = torch.rand(m, device="cuda")
    t_fwd = timeit(lambda: api.CSRmv(0, A, x), reps=5)
    t_bwd = timeit(lambda: api.CSRmv(1, A, e, At=At), reps=5)
    t_iter = timeit(lambda: R.iterate(1), reps=5)
    del At
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    fwd_bytes = 8 * nnz + 8 * (m + 1) + 4 * p.nvoxels + 4 * m
    bwd_bytes = 8 * nnz + 8 * (p.nvoxels + 1) + 4 * m + 4 * p.nvoxels
    # roofline of the MLEM iteration (forward + transpose products with their
    # fused epilogues, image sum, normalisation): algorithmic bytes per
    # iteration over the iteration time measured inside the timed steps
    achieved = bytes_it / t_it_live / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic_full.json")
    if args.config == "full" and os.path.exists(tp):  # measured for the full workload
        try:
            traffic = json.load(open(tp)).get("mlem_iteration")
        except Exception:
            traffic = None

    # ---- the reference's schedule on the GPU: no matrix stored, the chords
    # recomputed in every iteration (one walk per row gives A x, the ratio
    # and the row's share of A^T e)
    rebuild = None
    if not args.no_rebuild:
        Rf = api.Mlem(p, rows, y, s, matrix_free=True)
        Rf.iterate(1)
        Rf.close()
        a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a_ev.record(st)
        Rf = api.Mlem(p, rows, y, s, matrix_free=True)
        Rf.iterate(nit)
        b_ev.record(st)
        torch.cuda.synchronize()
        Rf.close()
        t_rb = a_ev.elapsed_time(b_ev) / 1000.0
        rebuild = {"value": nit / t_rb, "unit": UNIT, "ms_per_step": 1000 * t_rb,
                   "ms_per_iteration": 1000 * t_rb / nit, "schedule": REBUILD,
                   "how": "matrix-free reconstruction object: one chord walk per row and "
                          "iteration (A x, e = y / A x, the row's A^T e)"}

    # ---- per-iteration images of the three value forms, for the FP64 oracle
    x0 = torch.full((p.nvoxels,), 1.0 / p.nvoxels, dtype=torch.float32, device="cuda")

    def trace(Rx):
        Rx.set_image(x0)
        imgs = []
        for _ in range(nit):
            Rx.iterate(1)
            imgs.append(Rx.image())
        return torch.stack(imgs).cpu().numpy()

    traces = {"fp32": trace(R)}
    forms = None
    if not args.no_forms:
        forms = {"fp32": {"iteration_ms": 1000 * t_iter, "it_per_s": 1.0 / t_iter,
                          "layout": "grouped (value + 2-byte group-local column rank)"},
                 "iterations": nit}
        labels = {api.LAYOUT_CSC: "CSR + column-major copy (16-bit chunks)",
                  api.LAYOUT_GROUPED: "grouped (16-bit value + 2-byte group-local column rank)"}
        for name, fmt in (("bf16", 1), ("fp16", 2)):
            # the library's default layout for 16-bit values; the other
            # layout's iteration timed beside it
            R16 = api.Mlem(p, rows, y, s, use_graph=True, value_format=fmt)
            t16 = timeit(lambda: R16.iterate(1), reps=5)
            traces[name] = trace(R16)
            st16 = R16.stats()
            lay = R16.layout
            R16.close()
            other = api.LAYOUT_CSC if lay == api.LAYOUT_GROUPED else api.LAYOUT_GROUPED
            O16 = api.Mlem(p, rows, y, s, use_graph=True, value_format=fmt, layout=other)
            t16o = timeit(lambda: O16.iterate(1), reps=5)
            O16.close()
            forms[name] = {"iteration_ms": 1000 * t16, "it_per_s": 1.0 / t16,
                           "layout": labels[lay],
                           "speedup_vs_fp32": t_iter / t16,
                           "bytes_per_iteration": st16["bytes_per_iteration"],
                           ("grouped_layout_iteration_ms" if other == api.LAYOUT_GROUPED else
                            "csc_layout_iteration_ms"): 1000 * t16o,
                           "image_rel_l2_vs_fp32": float(
                               np.linalg.norm(traces[name][-1] - traces["fp32"][-1]) /
                               np.linalg.norm(traces["fp32"][-1]))}
    R.close()
    parity = None
    if not args.no_parity and rank == 0:
        parity = fp64_parity(p, A, rows, y, s, traces, nit)
    del A
    torch.cuda.empty_cache()
    batched = batched_small = None
    if args.batch > 0 and world == 1:
        batched = batch_measure(args, api, torch, st)
        # the same form on small problems, where one launch per problem
        # leaves the GPU mostly idle
        batched_small = batch_measure(args, api, torch, st, grids=(24, 32), angles=(8,))

    # ---- aggregate over ranks
    (t_step, t_e2e), (value, value_e2e) = aggregate_replicas((t_step, t_e2e), nit, world, dist,
                                                            "cuda", sharded=sharded)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(args.config, args.cpu_sample)
        cpu.pop("sample_seconds", None)
    h2d = rows_h.numel() * 4 + y_h.numel() * 4 + s_h.numel() * 4
    d2h = x_h.numel() * 4
    # the walk's work: grid cells crossed by all rays, per second of the build
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_step, "higher_is_better": True,
        "scaling": "strong" if sharded else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": workload_name(args.config)},
        "schedule": SCHEDULE,
        "measured_rows": m, "nnz": nnz,
        "parallelism": f"rows{world}" if sharded else f"replicas{world}",
        "l2": "inputs larger than L2 (matrix streams of GBs per pass)",
        "e2e": {"value": value_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": "mlem_iteration (grouped layout: one pass giving "
                                               "A x, e = y / A x and the groups' A^T e; per-column "
                                               "slot sums fused with x*c/s; normalisation)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_src,
                     "algorithmic_bytes": bytes_it, "iteration_ms": 1000 * t_it_live},
        # the step's parts: the system-matrix build, the iterations, and the
        # rest of the reconstruction's set-up (row order, row move, grouped
        # layout); the drop-in operators on the list-order CSR beside them
        "breakdown_ms": {"sm_build": 1000 * t_build, "iteration": 1000 * t_iter,
                         "setup_rest": 1000 * (t_step - t_build - nit * t_it_live),
                         "dropin_csr_to_csc": 1000 * t_csc,
                         "dropin_csrmv_forward": 1000 * t_fwd,
                         "dropin_csrmv_transpose": 1000 * t_bwd},
        "plan": plan,
        "sm_build_nnz_per_s": nnz / t_build,
        "sm_build_steps": {"ray_voxel_steps": steps, "per_s": steps / t_build,
                           "per_sm_cycle": steps / t_build / (sms * 1e6 * (clocks.get("sm_mhz")
                                                                          or 2070.0))},
        "sm_build_rows_redone": build_rows,
        "spmv_gbs": {"forward": fwd_bytes / t_fwd / 1e9, "transpose": bwd_bytes / t_bwd / 1e9},
    }
    if rebuild is not None:
        out["rebuild_per_iteration"] = rebuild
    if parity is not None:
        out["parity_fp64"] = parity
    if forms is not None:
        out["forms"] = forms
    if batched is not None:
        out["batched"] = batched
    if batched_small is not None:
        out["batched_small"] = batched_small
    if cpu is not None:
        out["cpu_baseline"] = cpu
    print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def fp64_parity(p, A, rows, y, s, traces, nit):
    """Image error of every iteration of each value form against the FP64
    oracle (the plain C restatement, on the host cores) run on the same
    system matrix: the matrix of the measured rows copied to the host, the
    sensitivity as the FP64 column sums of that matrix when every channel is
    measured (else the library's FP64 sums), MLEM as reco.cu:209-281 in
    FP64."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    from epetreco_gb300 import api
    t0 = time.perf_counter()
    o = Oracle()
    rp = A.row_ptr.cpu().numpy()
    col = A.col.cpu().numpy()
    val = A.val.cpu().numpy()
    t_copy = time.perf_counter() - t0
    m = rows.numel()
    if m == p.nchannels:
        s64 = o.csrmv_f64(1, rp, col, val, np.ones(m), p.nvoxels)
        s_src = "FP64 column sums of the matrix on the host (every channel is measured)"
    else:
        s64 = api.sensitivity(p, return_f64=True)[1].cpu().numpy()
        s_src = "the library's FP64 column sums over all channels"
    x0 = np.full(p.nvoxels, 1.0 / p.nvoxels)
    tr = o.mlem_f64_trace(rp, col, val, y.cpu().numpy().astype(np.float64), s64 / s64.sum(), x0,
                          nit, p.nvoxels)
    out = {"oracle": "FP64 MLEM of the plain C restatement on the host cores, same matrix",
           "sensitivity": s_src, "iterations": nit, "nnz": int(len(col))}
    for name, t in traces.items():
        err = [float(np.linalg.norm(t[k] - tr[k]) / np.linalg.norm(tr[k])) for k in range(nit)]
        out[name] = {"image_rel_l2_per_iteration": err, "max": max(err), "last": err[-1]}
    out["seconds"] = {"copy": t_copy, "oracle": time.perf_counter() - t0 - t_copy}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
