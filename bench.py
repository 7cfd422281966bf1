#!/usr/bin/env python3
"""Cut candidates evaluated per second by the lookahead tree on GB300.

Workload (the staircase configuration): the closed union of 8 boxes (1.0 x
0.25 x k * 0.125, k = 1..8), welded without T-junctions, its side-wall
triangles split at their centroids: 188 triangles over 96 vertices,
normalised to a largest extent of 2 as decompose() does, cut with width 6, width2 3,
depth 3, 16 concave edges (64 plane slots), threshold 0.1 (minEdgeDist
0.015) and 2 refinement rounds of 8 probes. One step is one GpuTree.run over
a batch of maxNCutting = 160 such seeds: the tree, its evaluate kernel and
both probe rounds. A candidate cut is a job that is valid after plan (all
levels and rounds); the count comes from the device.

value: candidates per second of device time, seeds resident on the device
  (one CUDA-graph replay per step, CUDA events on the library's stream, L2
  flushed by a 256 MiB write between steps, outside the timed events).
e2e: the same metric through the public C call cuacd_tree_run with host
  buffers: seed upload, the run and the result readback in the timed region.

--impl reference: the CPU restatement of the same path (the oracle port of
the reference's kernels) on all host threads, on the same 160-seed batch.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

THRESHOLD = 0.1
TREE = dict(width=6, width2=3, depth=3, nConcaveEdges=16, minEdgeDist=min(THRESHOLD / 4, 0.015))
POOLS = dict(vertexCap=64 << 20, triCap=64 << 20, edgeCap=4 << 20, scratchWords=64 << 20,
             hullBudgetBytes=6 << 30, hullMaxVerts=4096)
REFINE_ROUNDS, REFINE_PROBES = 2, 8
METRIC = "cut candidates evaluated/s"
UNIT = "candidates/s"
L2_FLUSH_BYTES = 256 << 20


def workload(n_seeds):
    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    mesh = importlib.import_module("cuacd-web_gb300.mesh")
    conc = importlib.import_module("cuacd-web_gb300.concave")
    seed, _, _ = mesh.normalize(gen.staircase(8, wall_centroids=True))
    planes = conc.concave_edge_planes(seed, TREE["nConcaveEdges"])
    spacing = conc.refine_spacing([seed], THRESHOLD, TREE["width"])[0]
    seeds = [seed] * n_seeds
    refine = dict(rounds=REFINE_ROUNDS, probes=REFINE_PROBES, spacing=[spacing] * n_seeds)
    return seeds, [planes] * n_seeds, refine


def config_dict(n_seeds):
    return {"workload": f"staircase-8 lookahead tree, {n_seeds} seeds per step", "mesh": "staircase-8 (188 tris, 96 verts: side-wall triangles split at their centroids)",
            "seeds": n_seeds, "width": TREE["width"], "width2": TREE["width2"], "depth": TREE["depth"],
            "nConcaveEdges": TREE["nConcaveEdges"], "threshold": THRESHOLD, "refineRounds": REFINE_ROUNDS,
            "refineProbes": REFINE_PROBES, "l2": "flushed between timed steps (256 MiB write)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        if self.gpu is None:  # no sampling
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        mhz, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                mhz.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(mhz)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_figures(kernel):
    """Figures of a kernel at this workload from its committed ncu summary
    (lines `name: value`): traffic_bytes_per_launch (dram read + write per
    launch), issue_active_pct, warps_active_pct."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_staircase160.md")
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        k, sep, v = line.partition(":")
        if sep and k.strip() in ("traffic_bytes_per_launch", "issue_active_pct", "warps_active_pct"):
            try:
                out[k.strip()] = float(v)
            except ValueError:
                pass
    return out


def cpu_tree_rate(seeds, planes, refine, threads):
    """Oracle restatement of the tree (the CPU port) on host threads: seeds
    are split over the threads, each with its own tree. Returns (candidates,
    seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness

    harness.lib()
    threads = max(1, min(threads, len(seeds)))
    chunks = [list(range(i, len(seeds), threads)) for i in range(threads)]
    results = [None] * threads
    cfg = dict(TREE, **POOLS)
    cfg.update(vertexCap=32 << 20, triCap=32 << 20, edgeCap=4 << 20, scratchWords=32 << 20)
    trees = [harness.OracleTree(**cfg) for _ in range(threads)]

    def work(k):
        idx = chunks[k]
        r = trees[k].run([seeds[i] for i in idx], [planes[i] for i in idx],
                         refine=dict(rounds=refine["rounds"], probes=refine["probes"],
                                     spacing=[refine["spacing"][i] for i in idx]))
        results[k] = r["validJobs"]

    t0 = time.perf_counter()
    th = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    dt = time.perf_counter() - t0
    return sum(results), dt


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device="cuda") -> float:
    """The largest of every rank's x (each rank runs its own replica; the
    job's time is the slowest rank's)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    world, rank, local = dist_setup(args)
    if rank != 0:
        return
    n = host_threads()
    sample = args.seeds  # the engine arm's batch: 160 seeds per step
    seeds, planes, refine = workload(sample)
    for _ in range(args.warmup):
        cpu_tree_rate(seeds[:n], planes[:n], refine, n)
    cands, secs = 0, 0.0
    for _ in range(args.steps):
        c, s = cpu_tree_rate(seeds, planes, refine, n)
        cands += c
        secs += s
    value = cands / secs
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(sample),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": n, "kind": "port",
                             "sample": f"{sample} staircase seeds per step (the oracle's restatement of the reference "
                                       f"kernels; the reference's own path is WebGPU, unavailable on this box)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_engine(args):
    import numpy as np
    import torch

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    tree_mod = importlib.import_module("cuacd-web_gb300.tree")
    seeds, planes, refine = workload(args.seeds)
    g = tree_mod.GpuTree(**TREE, **POOLS)
    g.set_profile(True)  # per-kernel CUDA events recorded as graph nodes
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # the autotuner's trials for this distribution of part sizes (one run per
    # schedule), untimed; the runs below use the schedule it kept
    for _ in range(4):
        g.run(seeds, planes, refine=refine)
    # ---- value: seeds resident on the device ----
    g.prepare(seeds, planes, refine=refine)
    schedule = g.schedule()
    for _ in range(args.warmup):
        g.launch()
        r = g.collect()
        # a run that overflowed a pool evaluated fewer candidates: not a valid step
        assert not r["overflow"] and not r["npOverflow"], "pool overflow: raise the pool capacities"
    barrier()
    dev_ms, cands = 0.0, 0
    kms = {k: 0.0 for k in g.KERNELS}
    kbytes = np.zeros(3, np.float64)
    lib = tree_mod.load_library()
    import ctypes as C

    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            g.launch()
            r = g.collect()
            dev_ms += r["gpuMs"]
            cands += r["validJobs"]
            for k, v in g.kernel_ms().items():
                kms[k] += v
            b = (C.c_uint64 * 3)()
            lib.cuacd_tree_kernel_bytes(g.h, b)
            kbytes += np.array(list(b), np.float64)
    barrier()
    t_max = max_over_ranks(dev_ms, world)
    value = world * cands / (t_max / 1000.0)

    # ---- e2e: public C call with host buffers ----
    g.set_profile(False)
    for _ in range(args.warmup):
        g.run(seeds, planes, refine=refine)
    barrier()
    e2e_s = 0.0
    e2e_c = 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = g.run(seeds, planes, refine=refine)
        e2e_s += time.perf_counter() - t0
        e2e_c += r["validJobs"]
    barrier()
    e2e_s = max_over_ranks(e2e_s, world)
    n = len(seeds)
    ps = g.plane_slots
    h2d = sum(s.verts.nbytes + s.tris.nbytes for s in seeds) + n * ps * 16 \
        + n * 64 + n * 80 + (16 + 1032) * 4 + n * ps * 16 + (16 + 4 * n) * 16
    d2h = (16 + 4 * n) * 16 + 64

    if rank != 0:
        return
    # ---- roofline of the dominant kernel ----
    dom = max((k for k in kms if k in ("plan", "emit", "hull", "scan", "record")), key=lambda k: kms[k])
    depth, stages = TREE["depth"], 1 + REFINE_ROUNDS
    # a level's hull step is two launches (warp and 256-thread groups), timed
    # together; on the staircase only the warp launch has parts
    launches_per_step = {"plan": depth * stages, "scan": depth * stages, "emit": depth * stages,
                         "hull": depth * stages, "record": depth * stages}
    byte_idx = {"plan": 0, "emit": 1, "hull": 2}
    peak, peak_kind = peaks()

    def kernel_roof(k):
        """HBM fraction of kernel class k from its algorithmic bytes (counted
        by the kernels) over its average launch time in the timed steps, with
        the issue figures of its committed ncu summary at this workload."""
        nl = launches_per_step[k] * args.steps
        per_launch = kbytes[byte_idx[k]] / nl
        avg_s = kms[k] / 1000.0 / nl
        achieved = per_launch / avg_s / 1e9
        prof = profile_figures(f"k_{k}")
        r = {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
             "algorithmic_bytes_per_launch": per_launch, "avg_launch_us": avg_s * 1e6,
             "traffic": prof.get("traffic_bytes_per_launch")}
        if "issue_active_pct" in prof:
            r["issue_active"] = prof["issue_active_pct"] / 100.0
        if "warps_active_pct" in prof:
            r["warps_active"] = prof["warps_active_pct"] / 100.0
        return r

    roof = None
    if dom in byte_idx:
        # the hull is bound by instruction issue and latency (integer
        # predicates, shared memory, dependent L2 round trips): its bound is
        # issue, reported as the issue-active fraction beside its HBM fraction
        roof = dict(bound="issue" if dom == "hull" else "hbm", kernel=f"k_{dom}", **kernel_roof(dom))
        if dom == "hull" and "issue_active" in roof:
            roof["issue_frac"] = roof["issue_active"]
        roof["kernels"] = {f"k_{k}": kernel_roof(k) for k in byte_idx if k != dom}
        roof["kernel_ms_per_step"] = {k: v / args.steps for k, v in kms.items()}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args.seeds),
            "e2e": {"value": world * e2e_c / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1000 * e2e_s / args.steps},
            "roofline": roof, "clocks": clk.summary(),
            # per level: plan, scan sums, scan, emit, two hull widths,
            # record; per stage the last level's seed bound and one evaluate
            "gpu_launches": args.steps * stages * (depth * 7 + 2),
            "schedule": {"warp_max_nv": schedule["warpMaxNv"], "big_job_nv": schedule["bigJobNv"],
                         "autotuned": not schedule["trial"] and schedule["tuned"] > 0},
            "candidates_per_step": cands / args.steps}
    if world == 1 and not args.no_cpu_baseline:
        nthr = host_threads()
        sample = 64 * nthr  # several seconds of CPU work on the host's cores
        s2, p2, r2 = workload(sample)
        c, s = cpu_tree_rate(s2, p2, r2, nthr)
        line["cpu_baseline"] = {"value": c / s, "unit": UNIT, "cores": nthr, "kind": "port",
                                "sample": f"{sample} staircase seeds, one tree run with {REFINE_ROUNDS} refinement "
                                          f"rounds on the oracle's CPU restatement ({c} candidates, {s:.1f} s)"}
    if world == 1 and not args.no_cpu_baseline:
        # the icosphere configuration against the reference's CPU helpers
        line["cpu_helpers"] = cut_eval_measure()
    if world == 1 and not args.no_decompose:
        # the metric's second half: whole decompositions per second, the
        # uneven batch decomposed together against one mesh at a time
        line["decompose"] = decompose_measure(args.meshes)
    if world == 1 and not args.no_serve:
        # the serving configuration: 60 s of Poisson arrivals at 200 req/s
        # under the device-memory budget, p50 / p99 latency beside the rate
        line["serving"] = serve_measure(args.rate, args.duration, args.pool, args.admit_bytes, args.slots, args.max_queue)
    print(json.dumps(line), flush=True)


def cut_eval_measure(steps=5, warmup=2):
    """The icosphere configuration: a level-4 icosphere (2,562 vertices,
    5,120 triangles) with radial noise U[-0.15, 0.15] of the radius,
    normalised to the unit cube, cut by 96 seeded planes; every half gets a
    capped cut, an exact hull, its volumes and rv cost and its sampled
    Hausdorff distance to its hull. On the GPU through the public call
    cuacd_tree_eval_cuts (mesh and planes from host memory, results back to
    host memory, in the timed region); beside it the oracle's restatement of
    the reference's CPU helpers on 1 host thread and on every host thread."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import harness

    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    tree_mod = importlib.import_module("cuacd-web_gb300.tree")
    m = gen.noisy_icosphere(4, noise=0.15, seed=0)
    planes = gen.random_planes(m, 96, seed=0).astype(np.float64)
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096, scratchWords=64 << 20)
    for _ in range(warmup):
        g.eval_cuts(m, planes)
    wall, dev = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        got = g.eval_cuts(m, planes)
        wall.append(time.perf_counter() - t0)
        dev.append(g.last_eval_ms / 1000.0)
    g.destroy()
    harness.lib()
    nthr = host_threads()
    t0 = time.perf_counter()
    ref = harness.eval_candidates(m, planes, threads=1, with_hd=True, use_ref=False)
    t1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    harness.eval_candidates(m, planes, threads=nthr, with_hd=True, use_ref=False)
    tn = time.perf_counter() - t0
    ok = (got[:, 0] == 1) & (ref[:, 0] == 1)
    rel = lambda a, b: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-12))) if a.size else 0.0  # noqa: E731
    hd_err = np.abs(got[ok, 7] - ref[ok, 7]) / (1e-4 + 1e-3 * ref[ok, 7])
    n = len(planes)
    return {"metric": "cut candidates evaluated/s (capped cut, hull, volumes, rv, Hausdorff per half)",
            "workload": "noisy icosphere L4 (2,562 verts, 5,120 tris) x 96 seeded planes, samples "
                        "max(1000, floor(2000 area)) per mesh side",
            "gpu": {"value": n / statistics.median(dev), "unit": "candidates/s", "ms": 1000 * statistics.median(dev)},
            "gpu_e2e": {"value": n / statistics.median(wall), "unit": "candidates/s",
                        "ms": 1000 * statistics.median(wall), "h2d_bytes_per_step": m.verts.nbytes + m.tris.nbytes + planes.nbytes,
                        "d2h_bytes_per_step": got.nbytes},
            "cpu_1thread": {"value": n / t1, "unit": "candidates/s", "cores": 1, "kind": "port", "ms": 1000 * t1},
            "cpu_all_threads": {"value": n / tn, "unit": "candidates/s", "cores": nthr, "kind": "port", "ms": 1000 * tn},
            "match": {"split_equal": bool(np.array_equal(got[:, 0], ref[:, 0])), "splits": int(ok.sum()),
                      "max_rel_volume": rel(got[ok, 1:3], ref[ok, 1:3]), "max_rel_hull": rel(got[ok, 3:5], ref[ok, 3:5]),
                      "max_abs_rv": float(np.max(np.abs(got[ok, 5:7] - ref[ok, 5:7]))) if ok.any() else 0.0,
                      "max_hausdorff_err_over_tolerance": float(hd_err.max()) if ok.any() else 0.0}}


def sample_counts(m):
    """Samples per mesh by the reference's rule (hausdorff_shader.ts:57-78)."""
    import numpy as np

    v = m.verts.astype(np.float32)
    a, b, c = v[m.tris[:, 0]], v[m.tris[:, 1]], v[m.tris[:, 2]]
    ar = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1).astype(np.float32)
    total = np.float32(ar.astype(np.float64).sum())
    res = max(np.float32(1000.0), np.floor(np.float32(2000.0) * total))
    cnt = np.floor((res / total) * ar).astype(np.int64)
    nt = len(ar)
    if nt > res:
        step = max(nt // int(res), 1)
        fill = (np.arange(nt) % step) == 0
    else:
        fill = (np.arange(nt) % 2) == 0
    cnt = np.where(cnt > 0, cnt, fill.astype(np.int64))
    return int(cnt.sum())


def run_secondary(args):
    """Hausdorff or hull batches (the merge pass's GPU work) on one GPU."""
    import numpy as np
    import torch

    tree_mod = importlib.import_module("cuacd-web_gb300.tree")
    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    mesh = importlib.import_module("cuacd-web_gb300.mesh")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    if args.workload == "bighulls":
        # the large-part hulls of a decomposition's first cuts: the 56k-triangle
        # blob mesh (28,152 points) cut by 64 seeded planes through its middle
        dec = importlib.import_module("cuacd-web_gb300.decompose")
        big = mesh.normalize(gen.blob_mesh(24, 71, seed=0))[0]
        rng = np.random.default_rng(0)
        parts = []
        for _ in range(64):
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            parts += list(dec.plane_cut(big, [nrm[0], nrm[1], nrm[2], rng.uniform(-0.2, 0.2)]))
        g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=32768,
                             hullBudgetBytes=16 << 30, scratchWords=64 << 20)
        n = len(parts)
        call = lambda: g.hull_meshes(parts, no_export=True)  # noqa: E731
        metric, unit, units = "convex hulls/s", "hulls/s", n
        cfg = {"workload": f"hulls of the {n} halves of the 56,300-triangle blob mesh cut by 64 seeded planes "
                           f"(mean {np.mean([m.nv for m in parts]):.0f} points)", "l2": "flushed between steps"}
    else:
        g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096,
                             hullBudgetBytes=6 << 30, scratchWords=256 << 20)
        n = args.pairs
        parts = [gen.noisy_icosphere(3, noise=0.15, seed=s) for s in range(n)]
        hulls, _ = g.hull_meshes(parts)
    if args.workload == "bighulls":
        pass
    elif args.workload == "hausdorff":
        pairs = [(m, mesh.Mesh(m.verts, h["tris"])) for m, h in zip(parts, hulls)]
        evals = sum(sample_counts(a) * b.nt + sample_counts(b) * a.nt for a, b in pairs)
        call = lambda: g.hausdorff(pairs)  # noqa: E731
        metric, unit, units = "point-triangle distance evaluations/s", "evals/s", evals
        cfg = {"workload": f"Hausdorff of {n} (noisy icosphere L3, its hull) pairs", "tris_per_mesh": parts[0].nt,
               "samples": "max(1000, floor(2000 area)) per mesh"}
    else:
        pts = [mesh.Mesh(m.verts, np.zeros((0, 3), np.uint32)) for m in parts]
        call = lambda: g.hull_meshes(pts)  # noqa: E731
        metric, unit, units = "convex hulls/s", "hulls/s", n
        cfg = {"workload": f"hulls of {n} point sets of {parts[0].nv} points (noisy icosphere L3)"}
    for _ in range(args.warmup):
        call()
    ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        call()
        ms += g.last_gpu_ms
    value = units * args.steps / (ms / 1000.0)
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "dtype": "f32", "data": "synthetic", "config": cfg}
    if args.workload == "hausdorff":
        # the tensor-core screen: sample-triangle pairs screened (one K = 16
        # bf16 MMA column each, 2 x 16 flops) and exact distances left
        st = g.hd_stats()
        secs = ms / args.steps / 1000.0
        tflops = 2 * 16 * st["screened"] / secs / 1e12
        bf16_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] \
            if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
        line["screen"] = {"screened_pairs": st["screened"], "exact_distances": st["exact"],
                          "exact_fraction": st["exact"] / max(st["screened"], 1), "timeout": st["timeout"],
                          "tensor_tflops": tflops, "bf16_peak_tflops": bf16_peak, "tensor_frac": tflops / bf16_peak}
        # the same batch through the exhaustive search alone
        g2 = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096,
                              hullBudgetBytes=6 << 30, scratchWords=256 << 20, hdScreenMinTris=-1)
        a = g.hausdorff(pairs)
        for _ in range(args.warmup):
            b = g2.hausdorff(pairs)
        ms2 = 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            b = g2.hausdorff(pairs)
            ms2 += g2.last_gpu_ms
        line["exhaustive"] = {"value": units * args.steps / (ms2 / 1000.0), "unit": unit,
                              "ms_per_step": ms2 / args.steps,
                              "same_results": bool((a.view(np.uint32) == b.view(np.uint32)).all())}
        # float32 operations counted from hd_tri_sq's source: 67 on the face
        # interior branch, 150 through the three edge tests; nominal FP32 peak
        # 152 SMs x 128 lanes x 2 x 2.07 GHz
        peak = 152 * 128 * 2 * 2.07e9 / 1e12
        ex_value = line["exhaustive"]["value"]
        for c, name in ((67, "flops_face_interior"), (150, "flops_edge_tests")):
            line.setdefault("fp32_exhaustive", {})[name] = c * ex_value / 1e12
        line["fp32_exhaustive"]["peak_tflops_nominal"] = peak
    if args.workload == "bighulls":
        # one hull alone: the whole mesh's point set, its latency
        one = [big]
        for _ in range(args.warmup):
            g.hull_meshes(one, no_export=True)
        t = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            g.hull_meshes(one, no_export=True)
            t.append(g.last_gpu_ms)
        line["single"] = {"points": big.nv, "ms": statistics.median(t)}
    print(json.dumps(line), flush=True)


# The uneven-batch decomposition: blob meshes (2..32 Gaussian blobs, marching
# tetrahedra, triangle counts log-uniform in 500..60k) at threshold 0.05,
# width 6, depth 2; the hull bound covers every part, so no GPU hull fails.
DEC_TREE = dict(vertexCap=256 << 20, triCap=256 << 20, edgeCap=16 << 20, scratchWords=256 << 20,
                hullBudgetBytes=16 << 30, hullMaxVerts=32768)
DEC_OPTS = dict(threshold=0.05, width=6, width2=3, depth=2, tree=DEC_TREE)
# the single large organic mesh: 24 blobs, about 56k triangles, threshold
# 0.1, width 9, depth 3
BIG_OPTS = dict(threshold=0.1, width=9, width2=3, depth=3, maxNCutting=160, tree=DEC_TREE)


def _parts_equal(ra, rb):
    if len(ra.parts) != len(rb.parts):
        return False
    return all(a.mesh.nv == b.mesh.nv and a.meshVol == b.meshVol and a.hullVol == b.hullVol
               and a.hausdorff == b.hausdorff for a, b in zip(ra.parts, rb.parts))


def decompose_measure(n_meshes, big_steps=2, max_iters=0):
    """meshes/s of the uneven batch decomposed together and one at a time
    (same decomposer, same parts), and the large mesh's latency. max_iters
    > 0 caps the iterations per mesh (the 256-mesh batch holds two meshes
    that never reach the threshold at 100)."""
    dec = importlib.import_module("cuacd-web_gb300.decompose")
    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    meshes = gen.blob_batch(n_meshes, seed=0)
    opts = dict(DEC_OPTS, **({"maxIters": max_iters} if max_iters > 0 else {}))
    d = dec.Decomposer(**opts)
    try:
        small = sorted(meshes, key=lambda m: m.nt)[:2]
        d.decompose_many(small, batched=True)  # warm-up: tree buffers and graphs
        t0 = time.perf_counter()
        rb = d.decompose_many(meshes, batched=True)
        tb = time.perf_counter() - t0
        t0 = time.perf_counter()
        rp = d.decompose_many(meshes, batched=False)
        tp = time.perf_counter() - t0
    finally:
        d.destroy()
    same = all(_parts_equal(a, b) for a, b in zip(rb, rp))
    big = gen.blob_mesh(24, 71, seed=0)
    d = dec.Decomposer(**BIG_OPTS)
    try:
        d.decompose(big)
        ms = []
        for _ in range(big_steps):
            t0 = time.perf_counter()
            rbig = d.decompose(big)
            ms.append(1000 * (time.perf_counter() - t0))
    finally:
        d.destroy()
    h2d = sum(m.verts.nbytes + m.tris.nbytes for m in meshes)
    d2h = sum(p.mesh.verts.nbytes + p.mesh.tris.nbytes + p.hull.verts.nbytes + p.hull.tris.nbytes
              for r in rb for p in r.parts)
    return {
        "metric": "meshes decomposed/s, batched vs one at a time",
        "batched": {"value": n_meshes / tb, "unit": "meshes/s", "seconds": tb},
        "plain": {"value": n_meshes / tp, "unit": "meshes/s", "seconds": tp},
        "speedup": tp / tb,
        "parts_equal": same,
        "parts": sum(len(r.parts) for r in rb),
        "stuck": sum(p.stuck for r in rb for p in r.parts),
        "config": {"workload": f"{n_meshes} blob meshes (2..32 Gaussian blobs, marching tetrahedra, triangles "
                               f"log-uniform in 500..60k, seed 0)", "tris": sum(m.nt for m in meshes),
                   "maxIters": opts.get("maxIters", 100),
                   "threshold": 0.05, "width": 6, "width2": 3, "depth": 2, "maxNCutting": 16, "nConcaveEdges": 16,
                   "refineRounds": 2, "mergeHulls": True, "hullMaxVerts": DEC_TREE["hullMaxVerts"]},
        "e2e_bytes": {"h2d": h2d, "d2h": d2h},
        "large_mesh": {"tris": big.nt, "ms": statistics.median(ms), "parts": len(rbig.parts),
                       "iterations": rbig.iterations, "config": "24 blobs, 71^3 grid, threshold 0.1, width 9, depth 3"},
    }


def serve_session(dec, pool, rate, duration, admit_bytes=0, max_active=0, max_queue=0, seed=1, clocks=False):
    """One serving session: Poisson arrivals at `rate` for `duration`
    seconds into a fresh server (device budget admit_bytes, 0 = 80 % of the
    GPU's memory; max_active slots; at most max_queue waiting requests, 0 =
    no bound), then
    drained. Returns a dict: latencies in ms (completion minus arrival,
    queueing included) overall and per mesh kind, wall seconds, requests
    offered, submissions refused with a full queue, the server's memory
    figures and the clock summary."""
    import numpy as np

    rng = np.random.default_rng(seed)
    arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 2) + 16))
    arr = arr[arr < duration]
    pick = rng.integers(0, len(pool), size=len(arr))
    srv = dec.Server(admit_bytes=admit_bytes, max_active=max_active, max_queue=max_queue, threshold=0.05, width=6,
                     width2=3, depth=2, tree=DEC_TREE)
    clk_summary = None
    try:
        # warm-up: the two trees (one per threshold) and their buffers
        for k, (_, m, thr) in enumerate(sorted(pool, key=lambda x: x[1].nt)[:4]):
            t = srv.submit(m, thr)
            while srv.take(t) is None:
                srv.step()
        t0 = time.perf_counter()
        i, out, lat, kinds, refused, most_active = 0, {}, [], {}, 0, 0
        with ClockSampler(0 if clocks else None) as clk:
            while i < len(arr) or srv.pending:
                now = time.perf_counter() - t0
                while i < len(arr) and arr[i] <= now:
                    kind, m, thr = pool[pick[i]]
                    try:
                        out[srv.submit(m, thr)] = (arr[i], kind)
                    except dec.CuacdError as e:
                        if e.code != dec.Server.E_BUSY:
                            raise
                        refused += 1
                    i += 1
                if srv.pending:
                    srv.step()
                    most_active = max(most_active, srv.stats()["active"])
                elif i < len(arr):
                    time.sleep(max(0.0, arr[i] - (time.perf_counter() - t0)))
                for t in list(out):
                    r = srv.take(t)
                    if r is not None:
                        a, kind = out.pop(t)
                        ms = 1000 * (time.perf_counter() - t0 - a)
                        lat.append(ms)
                        kinds.setdefault(kind, []).append(ms)
        wall = time.perf_counter() - t0
        if clocks:
            clk_summary = clk.summary()
        st = srv.stats()
    finally:
        srv.destroy()
    return {"lat": np.array(lat), "kinds": kinds, "wall": wall, "offered": len(arr), "refused": refused,
            "most_active": most_active, "memory": {"budget_bytes": st["budgetBytes"],
                                                   "peak_device_bytes": st["peakDeviceBytes"],
                                                   "device_bytes_at_end": st["deviceBytes"]},
            "clocks": clk_summary}


def _lat_summary(lat, kinds):
    import numpy as np

    return ({"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
            {k: {"p50": float(np.percentile(v, 50)), "p99": float(np.percentile(v, 99)), "n": len(v)}
             for k, v in kinds.items()})


SERVE_MIX = "40% staircases 4..16 steps, 40% blobs 2k..60k tris, 20% carved icospheres L3..5"


def serve_measure(rate=200.0, duration=60.0, pool_size=48, admit_bytes=0, max_active=32, max_queue=64, low_rate=2.0,
                  low_duration=15.0, clocks=False):
    """The serving configuration: Poisson arrivals of decomposition
    requests (40% staircases of 4..16 steps, 40% blobs of 2k..60k triangles,
    20% carved icospheres of level 3..5; thresholds 0.05 or 0.1) into the
    continuous-batching server for `duration` seconds under a device budget
    (0 = 80 % of the GPU's memory) and max_active slots, with at most
    max_queue waiting requests,
    then drained. A second session at low_rate (below the server's
    capacity) reports the latency without a standing queue."""
    dec = importlib.import_module("cuacd-web_gb300.decompose")
    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    pool = gen.serving_mix(pool_size, seed=0)
    hi = serve_session(dec, pool, rate, duration, admit_bytes, max_active, max_queue, clocks=clocks)
    p, pk = _lat_summary(hi["lat"], hi["kinds"])
    out = {"metric": "decomposition requests served/s", "value": len(hi["lat"]) / hi["wall"], "unit": "requests/s",
           "seconds": hi["wall"], "offered_rate": rate, "offered": hi["offered"], "served": len(hi["lat"]),
           "refused_queue_full": hi["refused"], "most_running": hi["most_active"], "latency_ms": p,
           "latency_ms_by_kind": pk, "memory": hi["memory"],
           "config": {"workload": f"Poisson arrivals at {rate} req/s for {duration} s ({hi['offered']} requests "
                                  f"from {pool_size} distinct meshes), then drained",
                      "mix": SERVE_MIX, "thresholds": [0.05, 0.1], "width": 6, "width2": 3, "depth": 2,
                      "admission": "device memory: 80 % of the GPU's" if admit_bytes == 0 else f"{admit_bytes} bytes",
                      "slots": max_active, "max_queue": max_queue}}
    if clocks:
        out["clocks"] = hi["clocks"]
    if low_rate and low_rate < rate:
        lo = serve_session(dec, pool, low_rate, low_duration, admit_bytes, max_active, max_queue, seed=2)
        p2, pk2 = _lat_summary(lo["lat"], lo["kinds"])
        out["below_capacity"] = {"offered_rate": low_rate, "duration_s": low_duration, "offered": lo["offered"],
                                 "served": len(lo["lat"]), "refused_queue_full": lo["refused"],
                                 "served_per_s": len(lo["lat"]) / lo["wall"], "latency_ms": p2,
                                 "latency_ms_by_kind": pk2, "memory": lo["memory"]}
    return out


def run_serve(args):
    m = serve_measure(args.rate, args.duration, args.pool, args.admit_bytes, args.slots, args.max_queue, clocks=True)
    line = {"metric": m["metric"], "value": m["value"], "unit": m["unit"], "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1000 * m["seconds"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": m.pop("config"), "clocks": m.pop("clocks", None)}
    line.update({k: v for k, v in m.items() if k not in ("metric", "value", "unit")})
    print(json.dumps(line), flush=True)


# the reference's own meshes at its README's comparison settings (width 30,
# nConcaveEdges 16, threshold 0.05, merging on; README.md:151-157), with the
# parts and wall times it reports on an RTX 4090
REF_MESHES = [("49160.stl", 142, 0.77), ("teapot_vox64.stl.gz", 16, 0.69), ("bunny_vox64.stl.gz", 246, 2.3)]


def refmeshes_measure(steps=1):
    import gzip

    dec = importlib.import_module("cuacd-web_gb300.decompose")
    io = importlib.import_module("cuacd-web_gb300.meshio")
    mesh_mod = importlib.import_module("cuacd-web_gb300.mesh")
    out = {}
    d = dec.Decomposer(threshold=0.05, width=30, nConcaveEdges=16, mergeHulls=True, tree=DEC_TREE)
    try:
        for name, ref_parts, ref_s in REF_MESHES:
            with open(os.path.join(ROOT, "tests", "golden", name), "rb") as f:
                buf = f.read()
            m = io.parse_stl(gzip.decompress(buf) if name.endswith(".gz") else buf)
            d.decompose(m)  # warm-up
            ms = []
            for _ in range(max(steps, 1)):
                t0 = time.perf_counter()
                r = d.decompose(m)
                ms.append(1000 * (time.perf_counter() - t0))
            vol = sum(mesh_mod.volume(p.mesh) for p in r.parts)
            out[name] = {"tris": m.nt, "parts": len(r.parts), "ms": statistics.median(ms), "iterations": r.iterations,
                         "volume_rel_err": abs(vol - mesh_mod.volume(m)) / mesh_mod.volume(m),
                         "reference_rtx4090": {"parts": ref_parts, "ms": 1000 * ref_s}}
    finally:
        d.destroy()
    return out


def run_refmeshes(args):
    res = refmeshes_measure(args.steps)
    total = sum(v["ms"] for v in res.values())
    line = {"metric": "reference meshes decomposed (README settings)", "value": 1000 * len(res) / total,
            "unit": "meshes/s", "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": total,
            "higher_is_better": True, "dtype": "f32", "data": "the reference's test meshes",
            "config": {"workload": "49160.stl, teapot_vox64, bunny_vox64 at width 30, nConcaveEdges 16, threshold 0.05, "
                                   "merging on"}, "meshes": res}
    print(json.dumps(line), flush=True)


def run_cuts(args):
    """The capped winning cut on the GPU (cuacd_tree_plane_cuts): the
    icosphere configuration's mesh (level 4, 2,562 vertices, 5,120
    triangles, radial noise) cut by its 96 seeded planes in one batch, the
    halves read back to host memory. value: cuts/s of device time; e2e: the
    public call with host buffers (mesh and planes in, every half out).
    Roofline: per cut the mesh is read once and both halves written once
    (12 bytes per vertex and per triangle each way), over the batch's
    device time."""
    import ctypes as C

    import numpy as np

    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    tree_mod = importlib.import_module("cuacd-web_gb300.tree")
    A = importlib.import_module("cuacd-web_gb300._abi")
    m = gen.noisy_icosphere(4, noise=0.15, seed=0)
    planes = np.ascontiguousarray(gen.random_planes(m, 96, seed=0).astype(np.float64))
    n = planes.shape[0]
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    L = tree_mod.load_library()
    ma = A.MeshArray([A.as_mesh(m)])
    idx = np.zeros(n, np.int32)

    def batch():
        h = C.c_void_p()
        t0 = time.perf_counter()
        rc = L.cuacd_tree_plane_cuts(g.h, ma.arr, 1, idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                     planes.ctypes.data_as(C.POINTER(C.c_double)), n, 1, C.byref(h))
        wall = time.perf_counter() - t0
        assert rc == 0, L.cuacd_last_error().decode()
        ms = float(L.cuacd_cuts_gpu_ms(h))
        sizes = []
        for k in range(n):
            for side in (0, 1):
                v, t = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
                nv, nt = C.c_uint32(), C.c_uint32()
                if L.cuacd_cuts_half(h, k, side, C.byref(v), C.byref(nv), C.byref(t), C.byref(nt)) == 0:
                    sizes.append((nv.value, nt.value))
        L.cuacd_cuts_free(h)
        return wall, ms, sizes

    for _ in range(args.warmup):
        batch()
    walls, devs, sizes = [], [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            w, ms, sizes = batch()
            walls.append(w)
            devs.append(ms)
    dev = statistics.median(devs) / 1000.0
    wall = statistics.median(walls)
    out_bytes = sum(12 * (nv + nt) for nv, nt in sizes)
    alg = n * 12 * (m.nv + m.nt) + out_bytes
    peak, peak_kind = peaks()
    achieved = alg / dev / 1e9
    line = {"metric": "capped plane cuts/s", "value": n / dev, "unit": "cuts/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dev, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "noisy icosphere L4 (2,562 verts, 5,120 tris) cut by 96 seeded planes in one batch",
                       "halves": len(sizes), "closed": True},
            "e2e": {"value": n / wall, "unit": "cuts/s", "h2d_bytes_per_step": m.verts.nbytes + m.tris.nbytes +
                    planes.nbytes, "d2h_bytes_per_step": out_bytes},
            "roofline": {"bound": "latency", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes_per_step": alg},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_decompose(args):
    m = decompose_measure(args.meshes, big_steps=max(args.steps, 1), max_iters=args.max_iters)
    line = {"metric": m["metric"], "value": m["batched"]["value"], "unit": "meshes/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "ms_per_step": 1000 * m["batched"]["seconds"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": m["config"],
            "e2e": {"value": m["batched"]["value"], "unit": "meshes/s", "h2d_bytes_per_step": m["e2e_bytes"]["h2d"],
                    "d2h_bytes_per_step": m["e2e_bytes"]["d2h"]},
            "plain": m["plain"], "speedup": m["speedup"], "parts_equal": m["parts_equal"], "parts": m["parts"],
            "large_mesh": m["large_mesh"]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--seeds", type=int, default=160)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="tree",
                    choices=["tree", "hausdorff", "hulls", "bighulls", "decompose", "serve", "refmeshes", "cuts"])
    ap.add_argument("--pairs", type=int, default=256)
    ap.add_argument("--meshes", type=int, default=32, help="meshes of the uneven decomposition batch")
    ap.add_argument("--no-decompose", action="store_true", help="leave the decomposition summary out of the tree line")
    ap.add_argument("--max-iters", type=int, default=0, help="decompose workload: iterations per mesh at most (0: 100)")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serving: seconds of arrivals")
    ap.add_argument("--pool", type=int, default=48, help="serving: distinct request meshes")
    ap.add_argument("--admit-bytes", type=int, default=0, help="serving: device budget in bytes (0: 80%% of the GPU's)")
    ap.add_argument("--slots", type=int, default=32, help="serving: decompositions running at once (0: no bound)")
    ap.add_argument("--max-queue", type=int, default=64, help="serving: waiting requests at most (0: no bound)")
    ap.add_argument("--no-serve", action="store_true", help="leave the serving session out of the tree line")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "decompose":
        run_decompose(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "refmeshes":
        run_refmeshes(args)
    elif args.workload == "cuts":
        run_cuts(args)
    elif args.workload != "tree":
        run_secondary(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
