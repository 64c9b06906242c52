#!/usr/bin/env python3
"""Benchmark of the voxelize -> seed -> flood -> perturb -> boundaries ->
count pipeline on one GB300.

Workload (one "step"): the mixed-256 batch -- 256 seeded synthetic vessels
with uneven grids (each axis log-uniform in [64, 384]), 5k-200k triangles,
2-32 fragments, metric and noise amplitude drawn per job (about 1.4 G
voxels, 2.8 GB of uint16 label grids).

Printed JSON line (rank 0):
  value     fragmented voxels/s of the batched path with the inputs already
            resident in HBM (vf_batch_prepare once, vf_batch_execute per
            step), CUDA events on the library's stream around K steps;
  e2e       the same metric through the public API with pinned host
            buffers: mesh upload, all stages, label-grid + count download
            per step, with two batches in flight (vf_pipeline_*: one batch's
            download overlaps the next batch's kernels); the one-batch-at-a-
            time vf_batch_run figure is reported beside it;
  plain     the reference-shaped per-job path (vf_plain_run) on a subset;
  serving   Poisson arrivals through vf_server (continuous batching):
            p50/p99 latency submit -> labels on host, sustained voxels/s;
  roofline  the flood relaxation kernel against the measured HBM peak;
  cpu_baseline the CPU oracle on a bounded sample of the same workload.

`--impl reference` times the reference algorithm's CPU restatement (the
reference itself is Windows/OpenGL-only and cannot run here) on a bounded
sample per step, with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fragmented voxels/s batched+served vs plain on 1 GB300; p50/p99 job latency"
WORKLOAD = ("mixed-256: 256 synthetic vessels, grid axes log-uniform in [64,384], "
            "5k-200k triangles, 2-32 fragments, per-job metric and noise amplitude 0-3 "
            "(period 16), flood + detectBoundaries(1)")


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "samples": len(sm), "reasons": sorted(reasons)}


def _oracle_params(job, O):
    from voxelfragmentml_gb300 import workloads as W
    import voxelfragmentml_gb300 as V  # enum values only
    kw = W.params_for(job, V)
    p = O.Params()
    base = dict(algorithm=1, distance=2, num_seeds=8, num_extra_seeds=0, merge_distance=0,
                seed_location=2, seed=80, noise_amplitude=0.0, noise_period=16, erode=0,
                erosion_type=1, erosion_size=3, erosion_iterations=3, erosion_probability=0.5,
                erosion_threshold=0.5, boundary_size=1)
    base.update(kw)
    for k, v in base.items():
        setattr(p, k, v)
    return p


def cpu_sample(jobs, stride=16, offset=0):
    return [j for j in jobs if j["index"] % stride == offset % stride]


def workload_config(jobs):
    """The `config` object of both arms: the workload and its size."""
    return {"workload": WORKLOAD, "jobs": len(jobs),
            "voxels_per_step": int(sum(int(np.prod(j["dims"])) for j in jobs)),
            "l2": "inputs larger than L2 (label grids 2.8 GB per step)"}


def run_cpu(jobs, meshes=None, check=None):
    """Oracle (CPU restatement of the reference algorithm) over `jobs`;
    returns (voxels, seconds, parity).  With `check` (job index -> JobSpec
    holding the GPU's labels and counts of that job) every oracle result is
    compared with the GPU's, outside the timed region; parity counts the
    jobs, the label voxels that differ and the jobs whose counts differ."""
    import oracle as O
    from voxelfragmentml_gb300 import vessel as Vs, workloads as W
    O.build()
    vox, secs = 0, 0.0
    par = {"jobs": 0, "voxels": 0, "label_mismatch_voxels": 0, "count_mismatches": 0}
    for j in jobs:
        v, f = meshes[j["index"]] if meshes else W.mesh_for(j)
        mn, mx = Vs.mesh_aabb(v)
        dims = j["dims"] or Vs.grid_dims(mn, mx, j["max_dim"])
        p = _oracle_params(j, O)
        t = time.perf_counter()
        lab, cnt, _ = O.run_job(v, f, dims, mn, mx, p, ncounts=256)
        secs += time.perf_counter() - t
        vox += int(np.prod(dims))
        if check is not None and j["index"] in check:
            spec = check[j["index"]]
            par["jobs"] += 1
            par["voxels"] += int(lab.size)
            par["label_mismatch_voxels"] += int(np.count_nonzero(spec.labels != lab))
            par["count_mismatches"] += int(not np.array_equal(spec.counts, cnt[:spec.counts.shape[0]]))
    return vox, secs, par


def reference_arm(args):
    """The reference's algorithm on the host cores: the CPU oracle over all
    jobs of the workload every timed step (the same jobs, metric and config
    as the GPU arm); warm-up steps take every 16th job."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from voxelfragmentml_gb300 import workloads as W
    jobs = W.mixed(args.jobs)
    sample = cpu_sample(jobs, args.ref_stride)
    meshes = {j["index"]: W.mesh_for(j) for j in sample}
    for w in range(args.warmup):
        run_cpu(cpu_sample(sample, 16, w), meshes)
    tot_v, tot_s = 0, 0.0
    for _ in range(args.steps):
        v, s, _ = run_cpu(sample, meshes)
        tot_v += v
        tot_s += s
    value = tot_v / tot_s
    cores = os.cpu_count()
    desc = (f"CPU oracle (restatement of the reference's voxelize/seed/flood/perturb/boundary/"
            f"count code; the reference itself is Windows+OpenGL only), OpenMP on {cores} threads, "
            f"{len(sample)} of {len(jobs)} mixed-256 jobs ({tot_v // args.steps} voxels) per step")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
            "config": workload_config(jobs),
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": cores, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# DRAM bytes per staged flood brick visit: dram__bytes_read.sum +
# dram__bytes_write.sum of one k_relax launch over the first 48 jobs of
# mixed-256 (ncu --set full, one GB300: 1.899087 GB + 184.804864 MB), divided
# by the 35370 visits of that launch that staged their brick (36922 visits,
# 1552 found nothing new).  The roofline's `traffic` is this figure times the
# staged visits of the timed launch.
K_RELAX_DRAM_BYTES_PER_VISIT = (1899086592 + 184804864) / 35370


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--jobs", type=int, default=256)
    ap.add_argument("--plain-jobs", type=int, default=32)
    ap.add_argument("--serve-rates", default="50,500,2000,4000,6000,8000",
                    help="Poisson arrival rates (jobs/s) of the serving sweep")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="seconds of arrivals per rate")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0,
                    help="HBM budget of the server (GiB) that admission control keeps to")
    ap.add_argument("--configs", action="store_true",
                    help="single-instance configurations 1-3 (128^3, 256^3, 512^3 vessels): "
                         "one JSON line each with batched, plain and CPU times and a parity check")
    ap.add_argument("--mesh", action="store_true",
                    help="fragment meshes (RegularGrid::toTriangleMesh) of one fractured vessel: "
                         "one JSON line")
    ap.add_argument("--mesh-dim", type=int, default=512, choices=[128, 256, 512],
                    help="--mesh workload: the 128^3 / 256^3 / 512^3 vessel of --configs")
    ap.add_argument("--impact", action="store_true",
                    help="impact path (ray entry voxels, nearSeeds) on the voxelized vessel of "
                         "--mesh-dim: one JSON line")
    ap.add_argument("--rays", type=int, default=1 << 20, help="--impact: rays per step")
    ap.add_argument("--cpu-stride", type=int, default=2,
                    help="cpu_baseline sample: every n-th job of the workload (2: about 10-15 s)")
    ap.add_argument("--ref-stride", type=int, default=1,
                    help="--impl reference: every n-th job per step (1: the whole workload)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default settings)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.configs:
        return single_configs(args)
    if args.mesh:
        return mesh_bench(args)
    if args.impact:
        return impact_bench(args)

    from voxelfragmentml_gb300 import replicas as R
    # replicas: every rank runs the whole workload on its own GPU; no collective on
    # the data path (jobs are independent), timings max-reduced over gloo
    world = R.init()
    rank = R.rank()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    from voxelfragmentml_gb300 import build as B
    B.build()
    import voxelfragmentml_gb300 as V
    from voxelfragmentml_gb300 import workloads as W

    ctx = V.Context(local)
    jobs = W.mixed(args.jobs)
    specs = [W.to_spec(j, V, want_labels=True, ncounts=256, pinned=True) for j in jobs]
    voxels = sum(int(np.prod(s.dims)) for s in specs)
    h2d = sum(s.verts.nbytes + s.faces.nbytes for s in specs)
    d2h = sum(s.labels.nbytes + s.counts.nbytes for s in specs)

    # ---- launch settings from the autotuner (a 64-job sample) -------------
    tuning = ctx.autotune(specs[:min(64, len(specs))]) if not args.no_tune else ctx.tuning()

    # ---- value: inputs resident in HBM ------------------------------------
    rb = V.ResidentBatch(specs, ctx)
    for _ in range(args.warmup):
        res = rb.execute(download=False)
    bad = [r.status for r in res if r.status]
    if bad:
        raise SystemExit(f"batch failed: {bad[:4]} {V.lib().vf_last_error()}")
    L = V.lib()
    clocks = Clocks()
    clocks.start()
    R.barrier()
    ctx.synchronize()
    L.vf_ctx_event_record(ctx.h, 0)
    launches, flood_ms, flood_bytes, visits, passes, sweeps, maxit = 0, 0.0, 0, 0, 0, 0, 0
    act_rows, key_changes, busy_warps, empty = 0, 0, 0, 0
    phase = {}
    stage_tot = {}
    for _ in range(args.steps):
        rb.execute(download=False)
        st = ctx.last_stats()
        launches += st["launches"]
        flood_ms += st["flood_ms"]
        flood_bytes += st["flood_bytes"]
        visits += st["flood_visits"]
        empty += st["flood_empty_visits"]
        passes += st["flood_passes"]
        sweeps += st["flood_sweeps"]
        maxit += st["flood_maxit_hits"]
        act_rows += st["flood_active_row_sweeps"]
        key_changes += st["flood_key_changes"]
        busy_warps += st["flood_busy_warp_sweeps"]
        pass_sizes = ctx.flood_pass_sizes()
        for k, v in st["flood_phase_cycles"].items():
            phase[k] = phase.get(k, 0) + v
        for k, v in ctx.stage_ms().items():
            stage_tot[k] = stage_tot.get(k, 0.0) + v
    L.vf_ctx_event_record(ctx.h, 1)
    ctx.synchronize()
    import ctypes as C
    msv = C.c_float()
    L.vf_ctx_event_elapsed(ctx.h, 0, 1, C.byref(msv))
    dev_ms = msv.value
    dev_ms = R.max_over_ranks(dev_ms)
    ms_per_step = dev_ms / args.steps
    value = voxels * args.steps * world / (dev_ms / 1000.0)

    # ---- e2e: host buffers, copies inside the timed region ----------------
    # Headline: vf_pipeline_* with two batches in flight and two sets of
    # pinned host buffers used in turn.  Every step's mesh upload, stages and
    # label + count download are inside the timed region; the download of
    # step k (copy engine) runs while step k+1 computes.  Host wall clock,
    # from an idle device to the last step's results on the host.
    specs2 = [W.to_spec(j, V, want_labels=True, ncounts=256, pinned=True) for j in jobs]
    sets = (specs, specs2)
    pipe = V.Pipeline(ctx, depth=2)
    for w in range(max(2, min(args.warmup, 4))):  # warms both slots
        if len(pipe._inflight) == 2:
            pipe.collect()
        pipe.submit(sets[w % 2])
    while pipe._inflight:
        pipe.collect()
    ctx.synchronize()
    R.barrier()
    t0 = time.perf_counter()
    res = []
    submit_s, collect_s = 0.0, 0.0
    for k in range(args.steps):
        if len(pipe._inflight) == 2:
            tc = time.perf_counter()
            res += pipe.collect()
            collect_s += time.perf_counter() - tc
        ts = time.perf_counter()
        pipe.submit(sets[k % 2])
        submit_s += time.perf_counter() - ts
    while pipe._inflight:
        tc = time.perf_counter()
        res += pipe.collect()
        collect_s += time.perf_counter() - tc
    wall_pipe = time.perf_counter() - t0
    pipe.close()
    e2e_ms = R.max_over_ranks(1000.0 * wall_pipe)
    e2e_stages = ctx.stage_ms()  # the last collected step, per stage
    e2e_value = voxels * args.steps * world / (e2e_ms / 1000.0)
    assert all(r.status == 0 for r in res)

    # One batch at a time through vf_batch_run (download by the pack kernel
    # straight into the pinned buffers), CUDA events on the library's stream.
    for _ in range(1):
        V.batch_run(specs, ctx)
    ctx.synchronize()
    L.vf_ctx_event_record(ctx.h, 2)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = V.batch_run(specs, ctx)
    L.vf_ctx_event_record(ctx.h, 3)
    ctx.synchronize()
    wall_sync = time.perf_counter() - t0
    L.vf_ctx_event_elapsed(ctx.h, 2, 3, C.byref(msv))
    sync_ms = R.max_over_ranks(max(msv.value, 1e-6))
    sync_value = voxels * args.steps * world / (sync_ms / 1000.0)
    assert all(r.status == 0 for r in res)
    clk = clocks.stop()
    assert all(r.status == 0 for r in res)

    # host link and placement of the pinned buffers (explains e2e - value)
    h2d_gbs, d2h_gbs = ctx.copy_bandwidth(256 << 20)
    L = V.lib()
    buf_nodes = sorted({L.vf_host_numa_node(s.labels.ctypes.data) for s in specs[::16]})
    host_link = {"h2d_gbs": h2d_gbs, "d2h_gbs": d2h_gbs,
                 "probe": "best of 3 copies of 256 MB, pinned host <-> device, CUDA events",
                 "gpu_host_numa_node": ctx.host_numa(), "label_buffer_numa_nodes": buf_nodes,
                 "host_cpus": os.cpu_count()}

    # ---- CPU baseline (oracle) on a bounded sample, and parity ----------
    # The GPU's labels and counts of the sample's jobs (in `specs` from the
    # last vf_batch_run above) are compared with the oracle's, job by job.
    cpu, parity = None, None
    if not args.no_cpu and rank == 0:
        sample = cpu_sample(jobs, args.cpu_stride)
        cv, cs, parity = run_cpu(sample, check={s.tag: s for s in specs})
        cpu = {"value": cv / cs, "unit": "voxels/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"CPU oracle on every {args.cpu_stride}th job of mixed-256 "
                         f"({len(sample)} jobs, {cv} voxels, {cs:.1f} s)"}
        parity["compared"] = ("labels and per-fragment counts of the headline batch "
                              "(vf_batch_run) against the oracle on the cpu_baseline jobs")
        if parity["label_mismatch_voxels"] or parity["count_mismatches"]:
            print(json.dumps({"parity": parity}), file=sys.stderr, flush=True)
            raise SystemExit("GPU labels or counts differ from the oracle on the headline batch")
    del specs2, sets

    # ---- plain per-job path (reference-shaped) on a subset ---------------
    plain = None
    if args.plain_jobs > 0:
        sub = specs[:args.plain_jobs]
        sub_vox = sum(int(np.prod(s.dims)) for s in sub)
        V.plain_run(sub[:2], ctx)
        ctx.synchronize()
        t0 = time.perf_counter()
        pr = V.plain_run(sub, ctx)
        ctx.synchronize()
        pt = time.perf_counter() - t0
        waves = [r.flood_passes for r in pr]
        plain = {"value": sub_vox / pt, "unit": "voxels/s", "jobs": len(sub),
                 "ms_per_job": 1000.0 * pt / len(sub), "mean_bfs_waves": float(np.mean(waves)),
                 "batched_over_plain": e2e_value / (sub_vox / pt),
                 "resident_batched_over_plain": value / (sub_vox / pt),
                 "timing": "wall clock, synchronised; includes mesh upload and label download"}

    # ---- serving: Poisson arrivals, continuous batching -----------------
    serving = None
    if not args.no_serve and args.serve_seconds > 0:
        rates = [float(r) for r in args.serve_rates.split(",") if r]
        budget = int(args.serve_budget_gb * (1 << 30))
        sweep = serve_sweep(V, ctx, jobs, rates, args.serve_seconds, budget)
        serving = {"sweep": sweep, "hbm_budget_bytes": budget,
                   "note": f"Poisson arrivals drawn from the {len(jobs)} mixed-256 jobs through "
                           "vf_server_* (continuous batching; one server for the sweep, warmed "
                           "by one untimed pass over the jobs; 3 slots, micro-batches of up to "
                           "128 jobs): latency = submit to labels in host memory; sustained = "
                           "voxels of completed jobs / (last completion - first arrival)"}

    peak, peak_kind = _peaks()
    flood_launch_ms = flood_ms / args.steps
    flood_launch_bytes = flood_bytes / args.steps
    achieved = (flood_launch_bytes / 1e9) / (flood_launch_ms / 1000.0) if flood_launch_ms else 0.0
    roof = {"kernel": "k_relax (flood brick relaxation, one cooperative launch per step)",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": f"{peak_kind} copy bandwidth",
            "algorithmic_bytes_per_launch": flood_launch_bytes,
            "bytes_rule": "4 B (u16 label read + write) per voxel of every brick visit",
            "brick_visits_per_launch": visits / args.steps,
            "empty_visits_per_launch": empty / args.steps,
            "passes_per_launch": passes / args.steps,
            "sweeps_per_visit": sweeps / max(visits, 1),
            "visits_at_sweep_cap": maxit / args.steps,
            "active_rows_per_sweep": act_rows / max(sweeps, 1),
            "busy_warps_per_sweep": busy_warps / max(sweeps, 1),
            "key_changes_per_visit": key_changes / max(visits, 1),
            "bricks_per_pass_last_step": pass_sizes,
            "phase_share": {k: round(v / max(sum(phase.values()), 1), 4) for k, v in phase.items()},
            "phase_kcycles_per_visit": {k: round(v / max(visits, 1) / 1000.0, 2) for k, v in phase.items()},
            "launch_ms": flood_launch_ms,
            "traffic": K_RELAX_DRAM_BYTES_PER_VISIT * (visits - empty) / args.steps,
            "traffic_source": "ncu DRAM bytes per brick visit (48-job capture) x visits of this launch"}
    line = {"metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic",
            "config": workload_config(jobs),
            "setup": {"parallelism": "replicas" if world > 1 else "single GPU",
                      "path": "batched (one persistent brick-queue kernel per stage)",
                      "cuda_graph": bool(getattr(rb, "graph", False)),
                      "tuning": tuning},
            "e2e": {"value": e2e_value, "unit": "voxels/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms / args.steps,
                    "path": "vf_pipeline_submit / vf_pipeline_collect, 2 batches in flight",
                    "timing": "host wall clock over the K steps, device idle at the start",
                    "stages_ms_last_step": {k: round(v, 3) for k, v in e2e_stages.items()},
                    "host_ms_per_step": {"submit": 1000.0 * submit_s / args.steps,
                                         "collect_wait": 1000.0 * collect_s / args.steps},
                    "host_link": host_link,
                    "one_batch_at_a_time": {"path": "vf_batch_run", "value": sync_value,
                                            "ms_per_step": sync_ms / args.steps,
                                            "wall_ms_per_step": 1000.0 * wall_sync / args.steps}},
            "roofline": roof, "cpu_baseline": cpu, "parity": parity, "clocks": clk,
            "gpu_launches": launches, "plain": plain, "serving": serving,
            "stages_ms_per_step": {k: v / args.steps for k, v in stage_tot.items()}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    R.finalize()
    return 0


def serve_sweep(V, ctx, jobs, rates, seconds, budget, copies=2):
    """Poisson arrivals at each rate (jobs/s) for `seconds`; each arrival is
    a job drawn uniformly from `jobs`.  Every job has `copies` pinned label
    buffers used in turn, so a job that is in flight twice writes to two
    buffers.  One server takes the whole sweep, as a deployed server runs
    through changes of load; before the first rate it serves every job
    `copies` times (untimed warm-up, which sizes the arenas of its slots), and
    each rate starts after the previous one has drained."""
    from voxelfragmentml_gb300 import workloads as W
    base = [W.to_spec(j, V, want_labels=False, ncounts=256, pinned=True) for j in jobs]
    outs = {}
    for k in range(copies):
        for i, s in enumerate(base):
            outs[(i, k)] = V.pinned_array(s.dims, np.uint16)
    sweep = []
    srv = V.Server(ctx, hbm_budget=budget, max_inflight=3, max_batch=128)
    nwarm = 0
    for k in range(copies):  # every slot takes a warm-up batch
        for i, s in enumerate(base):
            s.labels = outs[(i, k)]
            s.tag = nwarm
            srv.submit(s)
            nwarm += 1
    got, deadline = 0, time.perf_counter() + 300
    while got < nwarm and time.perf_counter() < deadline:
        got += len(srv.poll(256, 50))
    for rate in rates:
        rng = np.random.default_rng(7)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * seconds * 1.5) + 64))
        arrivals = arrivals[arrivals < seconds]
        pick = rng.integers(0, len(base), size=len(arrivals))
        uses = np.zeros(len(base), np.int64)
        results = []
        vox_of = {}
        t0 = time.perf_counter()
        for n, at in enumerate(arrivals):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            i = int(pick[n])
            s = base[i]
            s.labels = outs[(i, int(uses[i]) % copies)]
            uses[i] += 1
            s.tag = n
            vox_of[n] = int(np.prod(s.dims))
            srv.submit(s)
            results += srv.poll(256, 0)
        offered = time.perf_counter() - t0
        deadline = time.perf_counter() + 300
        while len(results) < len(arrivals) and time.perf_counter() < deadline:
            results += srv.poll(256, 50)
        lat = np.array(sorted(r.done_ms - r.submit_ms for r in results))
        ok = [r for r in results if r.status == 0]
        done_vox = sum(vox_of[int(r.user_tag)] for r in ok)
        span_ms = max(r.done_ms for r in results) - min(r.submit_ms for r in results) \
            if results else 0.0
        offered_vox = sum(vox_of.values()) / max(offered, 1e-9)
        sweep.append({"rate_jobs_per_s": rate, "seconds": seconds, "submitted": int(len(arrivals)),
                      "achieved_arrival_rate": len(arrivals) / max(offered, 1e-9),
                      "completed_ok": len(ok),
                      "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                      "p90_ms": float(np.percentile(lat, 90)) if len(lat) else None,
                      "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                      "offered_voxels_per_s": offered_vox,
                      "sustained_voxels_per_s": done_vox / max(span_ms / 1000.0, 1e-9),
                      "sustained_over_offered": (done_vox / max(span_ms / 1000.0, 1e-9)) /
                      max(offered_vox, 1e-9)})
    srv.close()
    return sweep


def single_configs(args):
    """Configurations 1-3 as single jobs: device time with resident inputs,
    end-to-end vf_batch_run, the plain per-job path, the CPU oracle, and the
    labels checked against the oracle's."""
    import oracle as O
    import voxelfragmentml_gb300 as V
    from voxelfragmentml_gb300 import build as B, workloads as W
    B.build()
    O.build()
    cfgs = [
        ("1: 128x96 vessel, 128^3, 8 fragments, Manhattan",
         W.single(128, 128, 96, 8, 1, 0.0, 16, False, 42, 42)),
        ("2: 256x192 vessel, 256^3, 16 fragments, Euclidean, noise A=2 P=16, one 3x3x3 erosion",
         W.single(256, 256, 192, 16, 0, 2.0, 16, True, 42, 42)),
        ("3: 512x384 vessel, 512^3, 64 fragments, Chebyshev, noise A=2 P=16",
         W.single(512, 512, 384, 64, 2, 2.0, 16, False, 42, 42)),
    ]
    ctx = V.Context(0)
    L = V.lib()
    import ctypes as C
    for name, job in cfgs:
        spec = W.to_spec(job, V, want_labels=True, ncounts=256, pinned=True)
        vox = int(np.prod(spec.dims))
        rb = V.ResidentBatch([spec], ctx)
        for _ in range(2):
            rb.execute(download=False)
        ctx.synchronize()
        reps = 5
        L.vf_ctx_event_record(ctx.h, 0)
        for _ in range(reps):
            rb.execute(download=False)
        L.vf_ctx_event_record(ctx.h, 1)
        ctx.synchronize()
        ms = C.c_float()
        L.vf_ctx_event_elapsed(ctx.h, 0, 1, C.byref(ms))
        dev_ms = ms.value / reps
        stages = ctx.stage_ms()
        st = ctx.last_stats()
        V.batch_run([spec], ctx)
        t = time.perf_counter()
        for _ in range(reps):
            (r,) = V.batch_run([spec], ctx)
        e2e_ms = 1000.0 * (time.perf_counter() - t) / reps
        got = spec.labels.copy()
        plain = W.to_spec(job, V, want_labels=True, ncounts=256, pinned=True)
        V.plain_run([plain], ctx)
        t = time.perf_counter()
        (pr,) = V.plain_run([plain], ctx)
        plain_ms = 1000.0 * (time.perf_counter() - t)
        v, f = W.mesh_for(job)
        q = O.Params()
        base = dict(algorithm=1, distance=2, num_seeds=8, num_extra_seeds=0, merge_distance=0,
                    seed_location=2, seed=80, noise_amplitude=0.0, noise_period=16, erode=0,
                    erosion_type=1, erosion_size=3, erosion_iterations=3, erosion_probability=0.5,
                    erosion_threshold=0.5, boundary_size=1)
        base.update(W.params_for(job, V))
        for k, val in base.items():
            setattr(q, k, val)
        t = time.perf_counter()
        lab, cnt, _ = O.run_job(v, f, spec.dims, spec.aabb[0], spec.aabb[1], q)
        cpu_ms = 1000.0 * (time.perf_counter() - t)
        flood_bytes = 4.0 * 8192 * st["flood_visits"]
        print(json.dumps({
            "config": name, "dims": list(spec.dims), "voxels": vox, "triangles": int(spec.faces.shape[0]),
            "batched_device_ms": dev_ms, "batched_voxels_per_s": vox / (dev_ms / 1e3),
            "e2e_ms": e2e_ms, "e2e_voxels_per_s": vox / (e2e_ms / 1e3),
            "plain_ms": plain_ms, "plain_voxels_per_s": vox / (plain_ms / 1e3),
            "plain_bfs_waves": int(pr.flood_passes),
            "cpu_oracle_ms": cpu_ms, "cpu_voxels_per_s": vox / (cpu_ms / 1e3), "cpu_cores": os.cpu_count(),
            "stages_ms": stages,
            "flood": {"k_relax_ms": st["flood_ms"], "brick_visits": st["flood_visits"],
                      "passes": st["flood_passes"],
                      "hbm_frac": (flood_bytes / (st["flood_ms"] / 1e3) / 1e9) / _peaks()[0]
                      if st["flood_ms"] else None},
            "labels_equal_oracle": bool(np.array_equal(got, lab)),
            "plain_equals_batched": bool(np.array_equal(plain.labels, got)),
            "counts_equal_oracle": bool(np.array_equal(spec.counts, cnt[:spec.counts.shape[0]])
                                        and not cnt[spec.counts.shape[0]:].any())}), flush=True)
    ctx.close()
    return 0


# ncu DRAM bytes (read + write) of one non-boundary k_lap_gather launch on the
# 512^3 mesh workload (one GB300, --clock-control none)
K_LAP_GATHER_NB_DRAM_BYTES_512 = 125.624576e6 + 17.66e6

MESH_JOBS = {
    128: ("128x96 vessel, 128^3, 8 fragments, Manhattan", (128, 128, 96, 8, 1, 0.0, 16, False, 42, 42)),
    256: ("256x192 vessel, 256^3, 16 fragments, Euclidean, noise A=2 P=16, one 3x3x3 erosion",
          (256, 256, 192, 16, 0, 2.0, 16, True, 42, 42)),
    512: ("512x384 vessel, 512^3, 64 fragments, Chebyshev, noise A=2 P=16",
          (512, 512, 384, 64, 2, 2.0, 16, False, 42, 42)),
}


def mesh_bench(args):
    """Fragment meshes: RegularGrid::toTriangleMesh of one fractured vessel
    (the --configs vessel of --mesh-dim, fractured on the GPU before timing),
    every fragment's marching-cubes mesh with the reference's default
    smoothing (max_dim * 0.048 iterations per vertex class).

    value: grid voxels meshed per second, vf_grid_triangulate with the label
           grid resident (wall clock per call: two size read-backs included);
    e2e:   the same with the labels uploaded from pinned host memory and the
           meshes (vec4 vertices, uvec4 faces) downloaded to pinned memory;
    roofline: the smoothing gather kernel (k_lap_gather, CUDA events around
              its iterations) against the measured HBM peak;
    cpu_baseline: the oracle (OpenMP over fragments) on the same grid."""
    import ctypes as C
    import oracle as O
    import voxelfragmentml_gb300 as V
    from voxelfragmentml_gb300 import build as B, vessel as Vs, workloads as W
    B.build()
    O.build()
    name, a = MESH_JOBS[args.mesh_dim]
    job = W.single(*a)
    v, f = W.mesh_for(job)
    mn, mx = Vs.mesh_aabb(v)
    dims = Vs.grid_dims(mn, mx, job["max_dim"])
    ctx = V.Context(0)
    g = V.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    V.fracture_model(g, V.Params.default(**W.params_for(job, V)))
    labels = V.pinned_array(dims, np.uint16)
    labels[...] = g.data()
    p = V.MCParams.default(max(dims))
    nvox = int(np.prod(dims))
    for _ in range(max(args.warmup, 1)):
        sizes = g.triangulate(p)
    F, NV, NT = sizes
    clocks = Clocks()
    clocks.start()
    wall, phases = [], []
    for _ in range(args.steps):
        t = time.perf_counter()
        g.triangulate(p)
        wall.append(time.perf_counter() - t)
        phases.append(g.mesh_phase_ms())
    L = V.lib()
    hvals = np.zeros(max(F, 1), np.uint16)
    hvo = V.pinned_array((F + 1,), np.uint64)
    hfo = V.pinned_array((F + 1,), np.uint64)
    hv = V.pinned_array((NV, 4), np.float32)
    hf = V.pinned_array((NT, 4), np.uint32)
    e2e = []
    for _ in range(args.steps):
        t = time.perf_counter()
        g.upload(labels)
        g.triangulate(p)
        V._check(L.vf_grid_meshes(g.h, V._p(hvals), V._p(hvo), V._p(hfo), V._p(hv), V._p(hf)))
        e2e.append(time.perf_counter() - t)
    # point clouds of every fragment mesh (CADModel::sampleCPU, 1024 points: the
    # reference's default _targetPoints)
    pc_wall = []
    for i in range(args.steps + 1):
        t = time.perf_counter()
        clouds = g.samplePointClouds(1024, 80)
        if i:
            pc_wall.append(time.perf_counter() - t)
    # RegularGrid::exportRLE of the same labels (the dataset's grid format)
    rle_wall = []
    for i in range(args.steps + 1):
        t = time.perf_counter()
        rle = g.exportRLE()
        if i:
            rle_wall.append(time.perf_counter() - t)
    clk = clocks.stop()
    st = g.mesh_phase_ms()
    cnt = g.mesh_counters()
    t = time.perf_counter()
    e = O.triangulate(labels, mn, mx, p.nonboundary_iterations, p.nonboundary_weight,
                      p.boundary_iterations, p.boundary_weight)
    cpu_s = time.perf_counter() - t
    t = time.perf_counter()
    e_pc = [O.sample_mesh(e[3][e[1][i]:e[1][i + 1]], e[4][e[2][i]:e[2][i + 1]], 1024, 80, int(v))
            for i, v in enumerate(e[0])]
    cpu_pc_s = time.perf_counter() - t
    pc_parity = len(e_pc) == len(clouds) and all(
        np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(clouds, e_pc))
    t = time.perf_counter()
    e_rle = O.rle_encode(labels)
    cpu_rle_s = time.perf_counter() - t
    rle_parity = bytes(e_rle) == rle
    parity = (np.array_equal(hvals[:F], e[0]) and np.array_equal(hvo, e[1]) and
              np.array_equal(hfo, e[2]) and np.array_equal(hf, e[4]) and
              np.array_equal(hv.view(np.uint32), e[3].view(np.uint32)))
    step_s = statistics.median(wall)
    e2e_s = statistics.median(e2e)
    dev_ms = [sum(ph) - ph[1] for ph in phases]
    peak, src = _peaks()
    sm = statistics.median(ph[4] for ph in phases)
    # k_lap_gather, per launch: every vertex reads its 8-byte meta word; each
    # vertex of the pass's type reads and writes its 16-byte position and
    # reads its 4-byte neighbour entries (neighbour positions come from L2)
    nv, _, vb, _, ne, neb = cnt
    per_nb = 8 * nv + 32 * (nv - vb) + 4 * (ne - neb)
    per_b = 8 * nv + 32 * vb + 4 * neb
    alg = p.nonboundary_iterations * per_nb + p.boundary_iterations * per_b
    print(json.dumps({
        "metric": "fragment-mesh grid voxels/s (RegularGrid::toTriangleMesh, all fragments)",
        "value": nvox / step_s, "unit": "voxels/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": name, "dims": list(dims), "fragments": F, "vertices": NV,
                   "faces": NT, "smoothing_iterations": [p.nonboundary_iterations,
                                                          p.boundary_iterations],
                   "l2": "label grid and mesh arrays larger than L2" if nvox * 2 > 129e6
                   else "label grid smaller than L2"},
        "faces_per_s": NT / step_s,
        "device_ms": statistics.median(dev_ms), "phase_ms": dict(zip(
            ["counts", "size_readback", "records_split_outputs", "smoothing_lists",
             "smoothing_iterations", "local_indices"], [round(x, 3) for x in st])),
        "counters": dict(zip(["vertices", "faces", "boundary_vertices", "face_incidences",
                              "neighbour_entries", "boundary_neighbour_entries"], cnt)),
        "e2e": {"value": nvox / e2e_s, "unit": "voxels/s", "ms": 1e3 * e2e_s,
                "h2d_bytes_per_step": int(labels.nbytes),
                "d2h_bytes_per_step": int(hv.nbytes + hf.nbytes + hvo.nbytes + hfo.nbytes)},
        "roofline": {"bound": "hbm", "kernel": "k_lap_gather (smoothing iterations)",
                     "launches": p.nonboundary_iterations + p.boundary_iterations,
                     "bytes_per_launch": [per_nb, per_b],
                     "achieved": (alg / (sm / 1e3) / 1e9) if sm else None, "peak": peak,
                     "unit": "GB/s", "frac": (alg / (sm / 1e3) / 1e9 / peak) if sm else None,
                     "peak_source": src,
                     "traffic": K_LAP_GATHER_NB_DRAM_BYTES_512 if args.mesh_dim == 512 else None,
                     "traffic_note": "ncu DRAM bytes of one non-boundary launch (its algorithmic "
                                     "bytes: bytes_per_launch[0])"},
        "cpu_baseline": {"value": nvox / cpu_s, "unit": "voxels/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": "the same grid, once"},
        "parity_with_oracle": bool(parity),
        "point_clouds": {"points_per_mesh": 1024, "meshes": F,
                         "ms": 1e3 * statistics.median(pc_wall),
                         "cpu_oracle_ms": 1e3 * cpu_pc_s, "parity_with_oracle": bool(pc_parity)},
        "rle_export": {"bytes": len(rle), "ms": 1e3 * statistics.median(rle_wall),
                       "note": "vf_grid_export_rle: size query + records to host",
                       "cpu_oracle_ms": 1e3 * cpu_rle_s, "parity_with_oracle": bool(rle_parity)},
        "clocks": clk,
    }), flush=True)
    g.close()
    ctx.close()
    return 0 if (parity and pc_parity and rle_parity) else 1


def impact_rays(mn, mx, n, seed=5):
    """n rays from a sphere around the box towards random points inside it."""
    rng = np.random.default_rng(seed)
    mn, mx = np.asarray(mn, np.float64), np.asarray(mx, np.float64)
    c, r = (mn + mx) / 2, np.linalg.norm(mx - mn)
    u = rng.normal(size=(n, 3))
    o = c + r * u / np.linalg.norm(u, axis=1, keepdims=True)
    t = mn + rng.random((n, 3)) * (mx - mn)
    return np.concatenate([o, t - o], axis=1).astype(np.float32)


def impact_bench(args):
    """Impact path on the voxelized vessel of --mesh-dim (CADScene::hit +
    Seeder::nearSeeds): a batch of rays through vf_ray_entry_voxels (host
    rays in, entry voxels out, per step), and nearSeeds calls with the
    reference's defaults (32 seeds, spreading 5) around 6 uniform seeds."""
    import oracle as O
    import voxelfragmentml_gb300 as V
    from voxelfragmentml_gb300 import build as B, vessel as Vs, workloads as W
    B.build()
    O.build()
    name, a = MESH_JOBS[args.mesh_dim]
    job = W.single(*a)
    v, f = W.mesh_for(job)
    mn, mx = Vs.mesh_aabb(v)
    dims = Vs.grid_dims(mn, mx, job["max_dim"])
    ctx = V.Context(0)
    g = V.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    occ = g.data()
    rays = V.pinned_array((args.rays, 6), np.float32)
    rays[...] = impact_rays(mn, mx, args.rays)
    out = V.pinned_array((args.rays, 3), np.uint32)
    L = V.lib()
    for _ in range(max(args.warmup, 1)):
        V._check(L.vf_ray_entry_voxels(g.h, V._p(rays), args.rays, V._p(out)))
    clocks = Clocks()
    clocks.start()
    wall = []
    for _ in range(args.steps):
        t = time.perf_counter()
        V._check(L.vf_ray_entry_voxels(g.h, V._p(rays), args.rays, V._p(out)))
        wall.append(time.perf_counter() - t)
    frags = V.Seeder.uniform(g, 6, 80, V.OUTER)
    near = []
    for i in range(args.steps + args.warmup):
        t = time.perf_counter()
        seeds = V.Seeder.nearSeeds(g, frags, 1, 32, 5, 80 + i)
        if i >= args.warmup:
            near.append(time.perf_counter() - t)
    clk = clocks.stop()
    step_s = statistics.median(wall)
    sample = min(args.rays, 1 << 18)
    t = time.perf_counter()
    e = O.ray_entry_batch(occ, mn, mx, rays[:sample])
    cpu_s = time.perf_counter() - t
    te = time.perf_counter()
    es = O.near_seeds(occ, frags, 1, 32, 5, 80 + args.warmup + args.steps - 1)
    cpu_near_s = time.perf_counter() - te
    parity = bool(np.array_equal(out[:sample], e) and np.array_equal(seeds, es))
    print(json.dumps({
        "metric": "ray entry voxels/s (RegularGrid::getClosestEntryVoxel, batched), host rays in "
                  "and voxels out per step; nearSeeds latency",
        "value": args.rays / step_s, "unit": "rays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "voxelized " + name.split(",")[0], "dims": list(dims),
                   "rays": args.rays, "hits": int((out[:, 0] != 0xFFFFFFFF).sum()),
                   "near_seeds": {"impacts": 1, "seeds": 32, "spreading": 5, "given": 6}},
        "e2e": {"value": args.rays / step_s, "unit": "rays/s",
                "h2d_bytes_per_step": int(rays.nbytes), "d2h_bytes_per_step": int(out.nbytes)},
        "near_seeds_ms": {"p50": 1e3 * statistics.median(near), "max": 1e3 * max(near)},
        "cpu_baseline": {"value": sample / cpu_s, "unit": "rays/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": f"the first {sample} rays",
                         "near_seeds_ms": 1e3 * cpu_near_s},
        "parity_with_oracle": parity,
        "clocks": clk,
    }), flush=True)
    g.close()
    ctx.close()
    return 0 if parity else 1


if __name__ == "__main__":
    sys.exit(main())
