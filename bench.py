"""Benchmark of the matchScene hot path on GB300.

Workload (the large single-scene configuration): a 24-tooth gear model (20k points with
exact normals, trained at sampling distance 0.03 of its diameter) and a seeded scene of 10
gears at random SO(3) poses in a 400x400x200 mm box with 30% clutter of random boxes and
spheres, sigma 0.3 mm noise, viewpoint-culled (about 0.9-1M points, no normals: they are
estimated). One step = one matchScene(scene, 0.03, 0.2, 0.2, MatchParam(numMatches=16)).

value: scenes/s with the scene already resident in HBM (device pointers passed through
the C ABI), timed with CUDA events on the library's stream, L2 flushed (256 MB write)
between steps outside the timed windows. e2e: the same call with pinned host buffers
(host->device copy of the scene and device->host read of the results inside the timed
region). cpu_baseline: the CPU restatement of the reference (k-d tree order, OpenMP over
8 threads as the reference caps it) on one scene of the same workload.

--impl reference: times that CPU restatement (all host threads) as the reference arm.
Multi-GPU: replicas (scenes are independent); each rank matches its own scene, max time
over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# Hardware work queues of the CUDA context (read when it is created, before torch loads):
# the batching workload's worker streams (up to 24) would otherwise share 8 queues, and
# kernels of unrelated scenes queued behind each other (measured: 64-scene batch 50 ->
# 44 ms). A deployment setting of the process, as sm_match_batch's callers would use it.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = ("scenes/sec and votes/sec on 1 GB300, batched vs plain GPU vs host CPU; "
          "p50/p99 ms")
SD = 0.03
KP = 0.2
MS = 0.2
NUM_MATCHES = 16


WORKLOADS = {
    # name: (scene builder, sampling distance, keypoint fraction, description)
    "large": ("scene_large", 0.03, 0.2,
              "large single scene: 10 gears, 30% box/sphere clutter, sigma 0.3 mm, "
              "viewpoint-culled, normals estimated; trainModel(gear 20k pts, 0.03), "
              "matchScene(0.03, 0.2, 0.2, numMatches=16)"),
    "batch": (None, 0.04, 0.2,
              "batching: 64 scenes, points log-uniform in [50k, 2M], 1-12 instances each of a "
              "gear, L-bracket or torus (models 20k-40k points), sigma U(0.2, 0.5) mm, clutter "
              "U(10%, 40%) boxes/spheres; matchScene(0.04, 0.2, 0.2, numMatches=16) per scene"),
    "serve": (None, 0.04, 0.2,
              "serving: Poisson arrivals of scenes (100k-3M points, log-uniform) against 8 "
              "resident models; rates 10..2000 scenes/s; matchScene(0.04, 0.2, 0.2, 16)"),
    "precision": (None, 0.04, 0.2,
                  "precision: scenes of 2M points with gears and L-brackets, sigma 0.5 mm, "
                  "normals estimated (k=10), dense ICP 30 iterations; GPU FP32 + Kahan vs "
                  "the CPU restatement with FP64 accumulation, same search orders"),
    "small": ("scene_small", 0.04, 0.1,
              "small scene: 3 gears over a 400x400 mm plane, 10% uniform clutter, sigma 0.2 mm, "
              "normals estimated; trainModel(gear 20k pts, 0.04), "
              "matchScene(0.04, 0.1, 0.2, numMatches=16)"),
}
WL = "large"


def workload(seed_offset=0):
    from surface_match_gb300 import synth
    model = synth.gear_model(20000, seed=7)
    builder = getattr(synth, WORKLOADS[WL][0])
    scene = builder(seed=(2 if WL == "large" else 1) + seed_offset, model=model)
    return model[0], scene


def workload_config(n_points):
    return {"workload": WORKLOADS[WL][3],
            "scene_points": int(n_points), "model_points": 20000,
            "l2": "flushed between steps (256 MB device write outside the timed window)"}


def start_clock_sampler(path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        return subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader",
                                 "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL), f
    except Exception:
        return None, None


def read_clocks(path, device_index):
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    try:
        for line in open(path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9 or p[0] != str(device_index):
                continue
            try:
                sm.append(float(p[1].split()[0]))
                mx.append(float(p[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
    except FileNotFoundError:
        pass
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons)}


def cpu_match(model_xyz, model_nrm, scene, threads, reps=1):
    """Median wall time of `reps` matchScene calls of the CPU restatement in reference
    order (trained once), and the last call's result."""
    from oracle import MODE_REF, MatchParam, Oracle
    o = Oracle(mode=MODE_REF, threads=threads)
    m = o.train(model_xyz, model_nrm, SD)
    times = []
    for _ in range(reps):
        t = time.perf_counter()
        r = o.match(m, scene.cloud.xyz, None, scene.viewpoint, SD, KP, MS,
                    MatchParam(numMatches=NUM_MATCHES))
        times.append(time.perf_counter() - t)
    return statistics.median(times), r


def job_totals(totals_ms, dist=None, device="cpu"):
    """The job's timed totals (ms): each the maximum over ranks (the job ends with its
    slowest rank); `dist` is torch.distributed when several ranks run, else None."""
    if dist is None:
        return [float(t) for t in totals_ms]
    import torch
    t = torch.tensor([float(x) for x in totals_ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_rate(world, steps, total_ms):
    """Whole-job scenes/s: every rank matched `steps` scenes (replicas, weak scaling)."""
    return world * steps / (total_ms / 1000.0)


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    model, scene = workload()
    times, votes = [], []
    for i in range(args.warmup + args.steps):
        dt, r = cpu_match(model.xyz, model.normal, scene, threads)
        if i >= args.warmup:
            times.append(dt)
            votes.append(int(r.kp_stats[:, 3].sum()))
    total = sum(times)
    v = args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "scenes/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(len(scene.cloud.xyz)),
            "votes_per_s": sum(votes) / total,
            "cpu_baseline": {"value": v, "unit": "scenes/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} matchScene calls of the workload scene, "
                                       "CPU restatement in reference (k-d tree) order"},
            "e2e": {"value": v, "unit": "scenes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_batch(n_scenes, steps, warmup, sd=0.04, kp=0.2):
    """The batching workload (64 seeded scenes of 50k-2M points, 1-12 instances of a gear,
    an L-bracket or a torus each): matchScene of every scene through sm_match_batch
    (concurrency picked by measurement among 4/8/12/16/24/32) against the same scenes one by one
    through sm_match. Wall clock around the synchronous calls; scenes resident in HBM for
    `value`, pinned host buffers (copies inside the call) for `e2e`."""
    import torch
    from surface_match_gb300 import Detector, MatchParam, PointCloud, match_batch, synth
    models = synth.batch_models()
    dets = {}
    for name, (cloud, _, _) in models.items():
        d = Detector()
        d.trainModel(PointCloud(cloud.xyz, cloud.normal), sd)
        dets[name] = d
    t = time.time()
    scenes = synth.batch_scenes(n_scenes, models=models)
    gen_s = time.time() - t
    param = MatchParam(numMatches=NUM_MATCHES)
    dev = [(dets[nm], PointCloud(torch.from_numpy(sc.cloud.xyz).cuda(), None, sc.viewpoint))
           for nm, sc in scenes]
    host = [(dets[nm], PointCloud(torch.from_numpy(sc.cloud.xyz).pin_memory().numpy(), None,
                                  sc.viewpoint)) for nm, sc in scenes]
    total_pts = sum(len(sc.cloud.xyz) for _, sc in scenes)

    def plain(jobs):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for d, pc in jobs:
            d.matchScene(pc, sd, kp, MS, param)
        return time.perf_counter() - t0

    def batched(jobs, conc):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out, st = match_batch(jobs, sd, kp, MS, param, concurrency=conc)
        return time.perf_counter() - t0, st

    for _ in range(max(1, warmup)):
        match_batch(dev, sd, kp, MS, param, concurrency=4)
    plain(dev[:4])
    tune = {}
    for conc in (4, 8, 12, 16, 24, 32):  # concurrency picked by measurement
        tune[conc] = batched(dev, conc)[0]
    best = min(tune, key=tune.get)
    times, votes = [], 0
    for _ in range(steps):
        dt, st = batched(dev, best)
        times.append(dt)
        votes = sum(x["n_votes"] for x in st)
    e2e_times = [batched(host, best)[0] for _ in range(max(1, steps // 2))]
    t_plain = [plain(dev) for _ in range(max(1, steps // 2))]
    n = len(scenes)
    return {"workload": WORKLOADS["batch"][3], "scenes": n, "total_points": int(total_pts),
            "generation_s": round(gen_s, 1), "steps": steps,
            "timing": "wall clock around the synchronous batch call (median of steps)",
            "value": n / statistics.median(times), "unit": "scenes/s",
            "ms_per_batch": 1000 * statistics.median(times),
            "plain_value": n / statistics.median(t_plain),
            "batched_over_plain": statistics.median(t_plain) / statistics.median(times),
            "votes_per_s": votes / statistics.median(times),
            "concurrency": best,
            "concurrency_sweep_ms": {str(k): round(1000 * x, 2) for k, x in tune.items()},
            "e2e": {"value": n / statistics.median(e2e_times), "unit": "scenes/s",
                    "h2d_bytes_per_step": int(total_pts * 12),
                    "d2h_bytes_per_step": int(n * NUM_MATCHES * 68)}}


def run_profile(args):
    """warmup + steps matchScene calls of the workload scene (scene resident in HBM) in the
    chosen search order, nothing else: the command that profiler captures run."""
    import torch
    from surface_match_gb300 import Detector, MatchParam, PointCloud
    model, scene = workload()
    det = Detector(search_order=args.search_order)
    det.trainModel(PointCloud(model.xyz, model.normal), SD)
    xyz = torch.from_numpy(scene.cloud.xyz).cuda()
    for _ in range(args.warmup + args.steps):
        det.matchScene(PointCloud(xyz, None, scene.viewpoint), SD, KP, MS,
                       MatchParam(numMatches=NUM_MATCHES))
    torch.cuda.synchronize()


def run_batch(args):
    """The batching workload as the headline line."""
    b = measure_batch(args.batch_scenes, args.steps, args.warmup, SD, KP)
    line = {"metric": METRIC, "value": b["value"], "unit": "scenes/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": b["ms_per_batch"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural gear / L-bracket / torus scenes)",
            "config": {k: b[k] for k in ("workload", "scenes", "total_points", "generation_s",
                                         "timing", "concurrency", "concurrency_sweep_ms")},
            "plain_value": b["plain_value"], "batched_over_plain": b["batched_over_plain"],
            "votes_per_s": b["votes_per_s"], "e2e": b["e2e"]}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Poisson arrival sweep against the serving loop: p50/p99 latency and throughput."""
    import numpy as np
    from surface_match_gb300 import Detector, MatchParam, PointCloud, Server, synth
    models = synth.serving_models()
    dets = {}
    for name, (cloud, _, _) in models.items():
        d = Detector()
        d.trainModel(PointCloud(cloud.xyz, cloud.normal), SD)
        dets[name] = d
    rng = np.random.default_rng(77)
    names = sorted(models)
    pool = []
    for i in range(args.serve_pool):
        nm = names[int(rng.integers(len(names)))]
        n = int(np.exp(rng.uniform(np.log(100_000), np.log(3_000_000))))
        sc = synth.scene_random(int(rng.integers(1 << 30)), n, {nm: models[nm][1]},
                                {nm: models[nm][2]}, float(rng.uniform(0.2, 0.5)),
                                float(rng.uniform(0.1, 0.4)), int(rng.integers(1, 13)))
        pool.append((nm, PointCloud(sc.cloud.xyz, None, sc.viewpoint)))
    param = MatchParam(numMatches=NUM_MATCHES)
    srv = Server(slots=args.serve_slots, hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)))
    # warm-up as a server would at start: every slot matches the pool's largest scene once
    # (its workspace grows to that size), so the rates below see no first-use allocation
    big = max(range(len(pool)), key=lambda i: len(pool[i][1].point))
    n_warm = 2 * args.serve_slots
    for _ in range(n_warm):
        nm, pc = pool[big]
        srv.submit(dets[nm], pc, SD, KP, MS, param)
    got = 0
    while got < n_warm:
        got += len(srv.poll(wait_ms=500))
    rates = []
    for rate in args.serve_rates:
        nreq = int(min(args.serve_requests, max(20, rate * 3)))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
        order = rng.integers(len(pool), size=nreq)
        done = []
        t0 = time.perf_counter()
        k = 0
        while len(done) < nreq:
            now = time.perf_counter() - t0
            while k < nreq and arrivals[k] <= now:
                nm, pc = pool[order[k]]
                srv.submit(dets[nm], pc, SD, KP, MS, param)
                k += 1
            wait = 0 if k < nreq else 50
            if k < nreq:
                wait = max(0, int(1000 * (arrivals[k] - (time.perf_counter() - t0))))
                wait = min(wait, 50)
            done.extend(srv.poll(max_requests=256, wait_ms=wait))
        span = time.perf_counter() - t0
        lat = np.array([d["total_ms"] for d in done])
        rates.append({"rate_per_s": rate, "requests": nreq, "throughput_scenes_per_s": nreq / span,
                      "p50_ms": float(np.percentile(lat, 50)),
                      "p99_ms": float(np.percentile(lat, 99)),
                      "p50_service_ms": float(np.percentile([d["service_ms"] for d in done], 50)),
                      "peak_bytes_in_flight": srv.status()["peak_bytes"]})
    srv.close()
    best = max(r["throughput_scenes_per_s"] for r in rates)
    line = {"metric": METRIC, "value": best, "unit": "scenes/s", "n_gpus": 1,
            "steps": sum(r["requests"] for r in rates), "warmup": n_warm,
            "ms_per_step": 1000.0 / best, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scenes, 8 resident models)",
            "config": {"workload": WORKLOADS["serve"][3], "slots": args.serve_slots,
                       "hbm_budget_gb": args.serve_budget_gb, "scene_pool": len(pool),
                       "pool_points": int(sum(len(pc.point) for _, pc in pool))},
            "rates": rates}
    print(json.dumps(line), flush=True)


def _rot_err_deg(A, B):
    import numpy as np
    R = A[:3, :3].astype(np.float64).T @ B[:3, :3].astype(np.float64)
    return float(np.degrees(np.arccos(np.clip((np.trace(R) - 1) / 2, -1, 1))))


def _precision_scene(o64, models, name, seed, npts, noise, n_inst):
    """One scene of the precision study: GPU (FP32 + Kahan) against the oracle with FP64
    accumulation, both with the GPU's search orders, so that only the accumulation differs."""
    import numpy as np
    from oracle import MatchParam as OMP
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    cloud, surf, ctr = models[name]
    sc = synth.scene_random(seed, npts, {name: surf}, {name: ctr}, noise, 0.2, n_inst)
    det = Detector()
    det.trainModel(PointCloud(cloud.xyz, cloud.normal), SD)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), SD, KP, MS,
                                   MatchParam(numMatches=NUM_MATCHES, poseRefNumSteps=30))
    nrm32, sampled = det.debug(4), det.debug(0)
    m64 = o64.train(cloud.xyz, cloud.normal, SD)
    r64 = o64.match(m64, sc.cloud.xyz, None, sc.viewpoint, SD, KP, MS,
                    OMP(numMatches=NUM_MATCHES, poseRefNumSteps=30))
    common = np.intersect1d(sampled, r64.sampled)
    a, b = nrm32[common].astype(np.float64), r64.normals[common].astype(np.float64)
    cosang = np.abs(np.sum(a * b, 1)) / np.maximum(np.linalg.norm(a, axis=1) *
                                                   np.linalg.norm(b, axis=1), 1e-30)
    nerr = np.degrees(np.arccos(np.clip(cosang, -1, 1)))
    diam = float(np.linalg.norm(np.ptp(cloud.xyz.astype(np.float64), axis=0)))
    inst, used = [], set()
    for P, s in zip(poses, scores):
        best = None
        for j, Q in enumerate(r64.poses):
            if j in used:
                continue
            dt = float(np.linalg.norm(P[:3, 3].astype(np.float64) - Q[:, 3]))
            if best is None or dt < best[1]:
                best = (j, dt)
        if best is None or best[1] > 0.1 * diam:
            continue
        used.add(best[0])
        Q = np.vstack([r64.poses[best[0]], [0, 0, 0, 1]])
        inst.append({"rot_err_deg": _rot_err_deg(P, Q), "trans_err_mm": best[1],
                     "score_fp32": float(s), "score_fp64": float(r64.scores[best[0]])})
    return {"model": name, "noise_mm": noise, "points": int(len(sc.cloud.xyz)),
            "sampled": int(len(common)),
            "instances_fp32": int(len(scores)), "instances_fp64": int(len(r64.scores)),
            "normal_err_deg": {"median": float(np.median(nerr)) if len(nerr) else None,
                               "p99": float(np.percentile(nerr, 99)) if len(nerr) else None,
                               "max": float(nerr.max()) if len(nerr) else None,
                               "bit_equal_frac": float(np.mean(
                                   (nrm32[common] == r64.normals[common]).all(1)))},
            "instances": inst}


def run_precision(args):
    """FP32 + Kahan accumulation (GPU) against FP64 accumulation (oracle, GPU search
    orders): normal angle error of every sampled scene point, and rotation / translation
    error of every matched instance. The study's scenes (2M points, noise 0.5 mm) are
    followed by a supplement of sparser, less noisy scenes, where instances are found and
    poses compared."""
    import numpy as np
    from oracle import MODE_GRID, Oracle
    from surface_match_gb300 import synth
    models = {name: synth.model_cloud(name, 20000, 50 + k)
              for k, name in enumerate(["gear", "bracket"])}
    rng = np.random.default_rng(91)
    o64 = Oracle(mode=MODE_GRID, threads=os.cpu_count() or 8, fp64=True)
    plan = [(0.5, args.precision_points, i) for i in range(args.precision_scenes)]
    plan += [(args.precision_supplement_noise, args.precision_supplement_points, i)
             for i in range(args.precision_supplement)]
    rows = []
    for noise, npts, i in plan:
        r = _precision_scene(o64, models, ["gear", "bracket"][i % 2],
                             int(rng.integers(1 << 30)), npts, noise, int(rng.integers(3, 9)))
        rows.append(r)
        print(json.dumps({"scene": len(rows) - 1, **{k: v for k, v in r.items()
                                                      if k != "instances"},
                          "n_inst_compared": len(r["instances"])}), file=sys.stderr, flush=True)
    allr = [x["rot_err_deg"] for r in rows for x in r["instances"]]
    allt = [x["trans_err_mm"] for r in rows for x in r["instances"]]
    nmax = [r["normal_err_deg"]["max"] for r in rows if r["normal_err_deg"]["max"] is not None]
    line = {"metric": "precision: FP32+Kahan vs FP64 accumulation", "workload": "precision",
            "config": {"workload": WORKLOADS["precision"][3],
                       "scenes": args.precision_scenes,
                       "supplement": {"scenes": args.precision_supplement,
                                      "noise_mm": args.precision_supplement_noise,
                                      "points_per_scene": args.precision_supplement_points},
                       "points_per_scene": args.precision_points, "sd_rel": SD, "kp": KP},
            "same_instance_count": all(r["instances_fp32"] == r["instances_fp64"]
                                       for r in rows),
            "instances_compared": len(allr),
            "max_rot_err_deg": max(allr) if allr else None,
            "max_trans_err_mm": max(allt) if allt else None,
            "max_normal_err_deg": max(nmax) if nmax else None,
            "median_normal_err_deg": float(np.median([r["normal_err_deg"]["median"]
                                                      for r in rows])),
            "scenes": rows}
    print(json.dumps(line), flush=True)


def _lib_tuned_shape(device):
    import ctypes as C
    from surface_match_gb300 import _lib
    t, p = C.c_int(0), C.c_int(0)
    _lib.load().sm_vote_tuned_shape(int(device), C.byref(t), C.byref(p))
    return {"threads_per_cta": t.value, "persistent": bool(p.value)}


def vote_traffic():
    """DRAM bytes (read + write) of one k_vote_acc launch of this workload, from the ncu capture
    summarised in profiles/k_vote_acc_<workload>.md (its line "dram_bytes_per_launch = N");
    None when no capture of this workload exists."""
    import re
    try:
        txt = open(os.path.join(ROOT, "profiles", f"k_vote_acc_{WL}.md")).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch\s*=\s*([0-9]+)", txt)
    return int(m.group(1)) if m else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-threads", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS))
    ap.add_argument("--profile", action="store_true",
                    help="only run warmup + steps matchScene calls of the workload in the given "
                         "search order (for profiler captures); prints no result line")
    ap.add_argument("--search-order", default="grid", choices=["grid", "reference"],
                    help="search order of the headline measurement; the other order is "
                         "measured beside it")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--serve-pool", type=int, default=12)
    ap.add_argument("--serve-slots", type=int, default=12)
    ap.add_argument("--serve-budget-gb", type=float, default=32.0)
    ap.add_argument("--serve-requests", type=int, default=120)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[10, 50, 200, 1000, 2000])
    ap.add_argument("--precision-scenes", type=int, default=16)
    ap.add_argument("--precision-points", type=int, default=2_000_000)
    ap.add_argument("--precision-supplement", type=int, default=6)
    ap.add_argument("--precision-supplement-noise", type=float, default=0.2)
    ap.add_argument("--precision-supplement-points", type=int, default=300_000)
    args = ap.parse_args()
    global WL, SD, KP
    WL = args.workload
    SD, KP = WORKLOADS[WL][1], WORKLOADS[WL][2]
    if WL == "batch" and args.impl != "reference":
        return run_batch(args)
    if WL == "serve" and args.impl != "reference":
        return run_serve(args)
    if WL == "precision":
        return run_precision(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.profile:
        return run_profile(args)

    import numpy as np
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from surface_match_gb300 import Context, Detector, MatchParam, PointCloud, _lib
    L = _lib.load()
    model, scene = workload(seed_offset=rank)
    n = len(scene.cloud.xyz)
    order = args.search_order
    other = "reference" if order == "grid" else "grid"
    det = Detector(Context(local), search_order=order)
    det.trainModel(PointCloud(model.xyz, model.normal), SD)
    param = MatchParam(numMatches=NUM_MATCHES)
    ext = torch.cuda.ExternalStream(det.ctx.stream)
    xyz_dev = torch.from_numpy(scene.cloud.xyz).cuda()
    xyz_pin = torch.from_numpy(scene.cloud.xyz).pin_memory()
    xyz_host = xyz_pin.numpy()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    vp = scene.viewpoint

    def step(src):
        return det.matchScene(PointCloud(src, None, vp), SD, KP, MS, param)

    ppf_ms = []

    def timed(src, steps, vote_ms=None):
        ms, launches = [], []
        for i in range(steps):
            with torch.cuda.stream(ext):
                flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = L.sm_launch_count()
            a.record(ext)
            step(src)
            b.record(ext)
            launches.append(L.sm_launch_count() - l0)
            b.synchronize()
            ms.append(a.elapsed_time(b))
            if vote_ms is not None:
                vote_ms.append(det.last_stats["vote_ms"][1])
                ppf_ms.append(det.last_stats["vote_ms"][0])
        return ms, launches

    for _ in range(args.warmup):
        step(xyz_dev)
        step(xyz_host)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    import tempfile
    clk_dir = os.environ.get("SM_CLOCKS_DIR") or tempfile.gettempdir()
    sampler, sf = start_clock_sampler(os.path.join(clk_dir, f"sm_clocks_r{rank}.csv"))
    clk_path = sf.name if sf else None
    torch.cuda.synchronize()
    vote_ms = []
    dev_ms, launches = timed(xyz_dev, args.steps, vote_ms)
    stats = det.last_stats
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e2e_ms, _ = timed(xyz_host, args.steps)
    torch.cuda.synchronize()
    if sampler:
        sampler.terminate()
        sampler.wait()
        sf.close()
    clocks = read_clocks(clk_path, local) if clk_path else {"sm_mhz": None}
    # the other search order on the same scene, measured the same way after the headline
    det2 = Detector(Context(local), search_order=other)
    det2.trainModel(PointCloud(model.xyz, model.normal), SD)
    ext2 = torch.cuda.ExternalStream(det2.ctx.stream)

    def timed_other(src, steps):
        ms = []
        for i in range(steps):
            with torch.cuda.stream(ext2):
                flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(ext2)
            det2.matchScene(PointCloud(src, None, vp), SD, KP, MS, param)
            b.record(ext2)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return ms

    for _ in range(args.warmup):
        det2.matchScene(PointCloud(xyz_dev, None, vp), SD, KP, MS, param)
    o_dev = timed_other(xyz_dev, args.steps)
    o_stats = det2.last_stats
    o_e2e = timed_other(xyz_host, args.steps)
    tot, tot_e2e = job_totals([sum(dev_ms), sum(e2e_ms)], dist, "cuda")
    o_tot, o_tot_e2e = job_totals([sum(o_dev), sum(o_e2e)], dist, "cuda")
    value = job_rate(world, args.steps, tot)
    e2e = job_rate(world, args.steps, tot_e2e)
    votes = stats["n_votes"]
    pairs = stats["n_pairs"]
    vk = statistics.mean(vote_ms)  # k_vote_acc: mean launch time, CUDA events on its stream
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    hits = stats["n_hits"]
    # k_vote_acc reads every matched bucket entry (8 B) and every hit record (16 B) once
    alg_bytes = 8 * votes + 16 * hits
    achieved = alg_bytes / (vk / 1000.0) / 1e9
    traffic = vote_traffic()
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    vote_rate = votes / (vk / 1000.0)
    # the vote kernel's bounding operation, measured on this GPU after the timed steps
    from surface_match_gb300 import probe_vote_atomics
    atomic_peak = probe_vote_atomics(torch.cuda.current_device())
    n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    # The same launch with nothing beside it: in the timed steps matchScene prepares the dense
    # refinement scene on a second stream while it votes, so the vote kernel shares the SMs;
    # a one-job batch runs the same matchScene without that overlap (after the timed steps).
    from surface_match_gb300 import match_batch
    iso_ms = []
    for i in range(4):
        _, st = match_batch([(det, PointCloud(xyz_dev, None, vp))], SD, KP, MS, param,
                            concurrency=1)
        if i:
            iso_ms.append(st[0]["vote_ms"][1])
    vk_iso = statistics.mean(iso_ms)
    # The latency-bound kernels of the path, timed per launch by the library's opt-in clock
    # (a CUDA event pair around each launch on its stream) over 3 matchScene calls after the
    # timed steps, against their algorithmic bytes.
    det.ctx.kernel_clock(True)
    for _ in range(3):
        det.matchScene(PointCloud(xyz_dev, None, vp), SD, KP, MS, param)
    clock_rep = det.ctx.kernel_report()
    det.ctx.kernel_clock(False)
    per_unit = {"k_sample_phase": "20 B per point of a sampling (position read, kept flag "
                                  "written), spread over its 8 phase launches",
                "k_scan_lookback": "8 B per scanned value (read, written)",
                "k_corr": "88 B per searched (candidate, model point): point and normal "
                          "read, moved point and normal, 3 indices written, winner atomic"}
    kernel_rooflines = []
    for name, r in clock_rep.items():
        if name in per_unit and r["launches"] and r["ms"] > 0:
            ach = r["bytes"] / (r["ms"] / 1000.0) / 1e9
            kernel_rooflines.append({
                "kernel": name, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "launch_ms": r["ms"] / r["launches"],
                "launches_per_call": r["launches"] / 3.0,
                "alg_bytes_per_launch": r["bytes"] / r["launches"],
                "alg_bytes": per_unit[name], "traffic": None,
                "how": "CUDA events around each launch (sm_context_kernel_clock), 3 "
                       "matchScene calls after the timed steps"})
    line = {"metric": METRIC, "value": value, "unit": "scenes/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural gears, clutter, noise)",
            "config": workload_config(n),
            "votes_per_s": world * votes * args.steps / (tot / 1000.0),
            "p50_ms": statistics.median(dev_ms),
            "p99_ms": float(np.percentile(dev_ms, 99)),
            "stage_ms": {k: round(v, 4) for k, v in zip(
                ["prep", "sample_normals", "keypoints", "voting", "cluster", "icp_prep",
                 "icp", "total"], stats["ms"])},
            "sizes": {k: stats[k] for k in ("n_valid", "n_sampled", "n_keypoints",
                                            "n_resampled", "n_poses", "n_clusters", "n_pairs",
                                            "n_hits", "n_votes")},
            "e2e": {"value": e2e, "unit": "scenes/s", "h2d_bytes_per_step": int(n * 12),
                    "d2h_bytes_per_step": int(NUM_MATCHES * 68)},
            "gpu_launches": int(sum(launches)),
            "roofline": {"kernel": "k_vote_acc", "bound": "hbm", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
                         "launch_ms": vk,
                         "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                         "note": "bucket entries and hit records are L2-resident (traffic is "
                                 "DRAM bytes per launch); the kernel's own limit is the "
                                 "shared-memory vote atomics, see shared_atomics",
                         "shared_atomics": {
                             "votes_per_s": vote_rate,
                             "per_sm_per_clk": vote_rate / n_sm / (sm_mhz * 1e6),
                             "probe_peak_per_s": atomic_peak,
                             "probe_peak_per_sm_per_clk": atomic_peak / n_sm / (sm_mhz * 1e6),
                             "frac_of_probe_peak": vote_rate / atomic_peak,
                             "probe": "sm_probe_vote_atomics: 16-bit shared counters at "
                                      "pseudo-random cells of a 48 KB accumulator, 512-thread "
                                      "CTAs, 2 per SM (one vote = one increment)"},
                         "isolated": {
                             "launch_ms": vk_iso,
                             "achieved": alg_bytes / (vk_iso / 1000.0) / 1e9,
                             "frac": alg_bytes / (vk_iso / 1000.0) / 1e9 / hbm,
                             "frac_of_probe_peak": votes / (vk_iso / 1000.0) / atomic_peak,
                             "how": "mean of 3 launches in one-job batches after the timed "
                                    "steps: the same matchScene without the dense preparation "
                                    "running beside the vote kernel (launch_ms above is "
                                    "measured in the timed, overlapped steps)"}},
            "kernel_rooflines": kernel_rooflines,
            "vote_launch_tuning": {
                "chosen": _lib_tuned_shape(local),
                "candidates": "256/512/1024 threads per CTA x (a CTA per keypoint | a "
                              "persistent grid taking keypoints from a device work counter)",
                "how": "the library's launch tuner: the first call on the device with at least "
                       "512 keypoints times each shape twice on its own data (CUDA events) and "
                       "keeps the fastest for the process"},
            "vote_stage_ms": {"pairs_probe_k_ppf": statistics.mean(ppf_ms),
                              "accumulate_k_vote_acc": vk,
                              "stage": stats["ms"][3]},
            "clocks": clocks,
            "search_order": order,
            "other_order": {
                "search_order": other,
                "value": job_rate(world, args.steps, o_tot),
                "e2e": job_rate(world, args.steps, o_tot_e2e),
                "ms_per_step": o_tot / args.steps,
                "p50_ms": statistics.median(o_dev),
                "stage_ms": {k: round(v, 4) for k, v in zip(
                    ["prep", "sample_normals", "keypoints", "voting", "cluster", "icp_prep",
                     "icp", "total"], o_stats["ms"])},
                "sizes": {k: o_stats[k] for k in ("n_sampled", "n_keypoints", "n_resampled",
                                                  "n_votes")},
                "note": "reference: the reference's k-d tree orders and search pruning, "
                        "results bit-identical to the reference-order restatement (see "
                        "reference_order_parity); grid: the same rules in uniform-grid "
                        "orders (faster, another sample)"}}
    if rank == 0 and args.batch_scenes > 0:
        line["batched"] = measure_batch(args.batch_scenes, max(2, min(args.steps, 4)), 1)
    if rank == 0 and not args.no_cpu_baseline:
        dt, r = cpu_match(model.xyz, model.normal, scene, args.cpu_threads, reps=3)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "scenes/s",
                                "cores": args.cpu_threads, "kind": "port",
                                "sample": "median of 3 matchScene calls of the workload scene: "
                                          "the reference's algorithm restated in C++ (oracle/, "
                                          "g++ -O3 with the compiler's auto-vectorisation for "
                                          "the host's baseline SIMD, no hand-written SIMD, "
                                          "transcendentals from the shared Cephes header) in "
                                          "reference (k-d tree) order, OpenMP 8 threads (the "
                                          "reference's cap, ppf.cpp:23); the reference itself "
                                          "(Eigen, xsimd, gtl absent) is not built",
                                "votes_per_s": float(r.kp_stats[:, 3].sum()) / dt}
        # end-to-end agreement at full size with that run (reference search order): same
        # instances, poses within the tolerance modulo the gear's symmetries
        from surface_match_gb300 import synth
        ref_det, grid_det = (det2, det) if order == "grid" else (det, det2)
        gpu_poses, gpu_scores = ref_det.matchScene(PointCloud(xyz_host, None, vp), SD, KP, MS,
                                                   param)
        grid_poses, _ = grid_det.matchScene(PointCloud(xyz_host, None, vp), SD, KP, MS, param)
        ref = [np.vstack([Q, [0, 0, 0, 1]]) for Q in r.poses]
        err = synth.match_poses(gpu_poses, ref, synth.gear_symmetries())
        diam = float(np.linalg.norm(model.xyz.max(0) - model.xyz.min(0)))
        # both against the synthetic ground truth: where the search orders disagree, which
        # one found the instances
        truth = [np.vstack([np.c_[i.R, i.t], [0, 0, 0, 1]]) for i in scene.instances]

        def vs_truth(poses):
            e = synth.match_poses(poses, truth, synth.gear_symmetries())
            return {"instances": int(len(poses)),
                    "within_tolerance": int(sum(a < 0.1 and b < 1e-3 * diam for a, b in e)),
                    "rotation_deg": [round(float(a), 4) for a, _ in e],
                    "translation_mm": [round(float(b), 4) for _, b in e]}

        same = (len(gpu_poses) == len(r.poses) and np.array_equal(
            gpu_poses[:, :3, :].reshape(len(gpu_poses), -1),
            np.asarray(r.poses).reshape(len(r.poses), -1)) and
            np.array_equal(gpu_scores, r.scores))
        line["reference_order_parity"] = {
            "gpu_search_order": "reference",
            "instances_gpu": int(len(gpu_poses)), "instances_reference_order": int(len(ref)),
            "bit_identical_poses_and_scores": bool(same),
            "max_rotation_deg": max((e[0] for e in err), default=0.0),
            "max_translation_mm": max((e[1] for e in err), default=0.0),
            "tolerance": {"rotation_deg": 0.1, "translation_mm": 1e-3 * diam},
            "vs_truth": {"instances": len(truth), "gpu_reference_order": vs_truth(gpu_poses),
                         "gpu_grid_order": vs_truth(grid_poses),
                         "cpu_reference_order": vs_truth(ref)}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
