#!/usr/bin/env python
"""PPM-APA pass throughput on GB300 (the 1080p at-scale workload).

Workload (one step = one render pass): 1920x1080, a noise-displaced geodesic
sphere of 873,620 triangles (frequency 209) over a ground quad, lit by a
seeded 2048x1024 FP32 equirect sky (gradient + 0.5 degree sun lobe of peak
5e4 + lognormal texel noise sigma 0.3), materials 60/20/20 Lambertian /
mirror / dielectric per surface cluster, 4M photons per pass, alpha 0.7,
photon and eye depth 12. Data are synthetic (seeded); nothing is downloaded.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--mode canonical|compat]

--impl gb300 (default) times the hand-written sm_103a kernels through the C
ABI: `value` is device time of K passes with every input resident in HBM;
`e2e` is the same passes through pppm_render_pass + pppm_render_read into
pinned host memory (the reference writes an image every pass). --impl
reference times the reference algorithm on the host cores instead (the
oracle port of oracle/pppm_port.cc, built from the reference's own algorithm
and pinned bit-exact to it; the reference sources do not travel to the GPU
machine) on a bounded sample of the workload. Multi-GPU runs are replicas
(passes shard with no exchange until an image reduction, not timed here).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "tatsy-pppm_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

METRIC = "Mphotons/s + equal-time relMSE, learned vs plain PPM-APA, 1080p, 1 GB300"
UNIT = "Mphotons/s"
# the headline workload and the subsurface one (measured on request)
WORKLOADS = {
    "config2": dict(photons=4_000_000, depth=12, width=1920, height=1080, triangles=873_622,
                    desc="ppm-apa pass, 1920x1080, displaced icosphere 873,620 tris + ground, 2048x1024 sky env, "
                         "4M photons/pass, depth 12"),
    "config4": dict(photons=0, depth=8, width=0, height=0, triangles=0,
                    desc="64 independent ppm-apa renders (canonical), each its own scene: displaced icosphere or "
                         "torus of log-uniform 5k-500k tris + ground, own sky, image sides log-uniform 128-1024, "
                         "photons log-uniform 100k-2M, alpha in {0.6, 0.7, 0.8}, 16 passes, depth 8; up to 8 jobs "
                         "in flight, autotuned launch shapes"),
    "config3": dict(photons=2_000_000, depth=12, width=1280, height=720, triangles=200_002,
                    desc="ppm-apa pass with dipole subsurface scattering, 1280x720, displaced torus 200,000 tris "
                         "(refractive + BSSRDF) + ground, 1024x512 sky env, 2M photons/pass, depth 12, Poisson "
                         "irradiance points + octree rebuilt every pass"),
}
PHOTONS = WORKLOADS["config2"]["photons"]
DEPTH = WORKLOADS["config2"]["depth"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="canonical", choices=["canonical", "compat"])
    ap.add_argument("--cell-factor", type=float, default=1.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-study", action="store_true", help="skip the equal-time learned-vs-plain relMSE study")
    ap.add_argument("--no-graph", action="store_true", help="config4: run every pass through pppm_render_pass")
    ap.add_argument("--graph-lanes", type=int, default=0, help="config4: jobs at once inside the graph")
    args = ap.parse_args()
    global PHOTONS, DEPTH
    PHOTONS = WORKLOADS[args.workload]["photons"]
    DEPTH = WORKLOADS[args.workload]["depth"]
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_config(mode, cell_factor, workload="config2"):
    w = WORKLOADS[workload]
    return {"workload": w["desc"], "mode": mode, "width": w["width"], "height": w["height"],
            "triangles": w["triangles"], "photons_per_pass": w["photons"], "max_depth": w["depth"], "alpha": 0.7,
            "radius_scale": (1 / 64) if mode == "canonical" else 0.1, "cell_factor": cell_factor,
            "parallelism": "replicas",
            "l2": "inputs larger than L2 (photon map, path queues and BVH ~1.5 GB per pass)"}


class ClockSampler:
    """nvidia-smi samples every 50 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start (NVML initialisation) can stall the driver:
            # the timed region begins once the first sample has arrived
            t0 = time.perf_counter()
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
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
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_scene(workload="config2"):
    import scenes as S

    return S.config3() if workload == "config3" else S.config2()


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(scene, sample_scale=16, threads=None):
    """The reference algorithm (oracle port, compat semantics) on the host
    cores over a bounded sample: photons and pixels divided by sample_scale."""
    import port
    import pppm_gb300 as P

    threads = threads or os.cpu_count() or 1
    w, h = 1920 // int(sample_scale ** 0.5), 1080 // int(sample_scale ** 0.5)
    cam = P.Context.make_camera(scene.camera)
    cam.width, cam.height = w, h
    photons = PHOTONS // sample_scale
    par = P.Context.make_params(mode=P.MODE_COMPAT, photons=photons, num_streams=threads, max_bounce_photon=DEPTH,
                                max_bounce_eye=DEPTH)
    ps = port.PortScene(scene)
    out = ps.render(cam, par, 1)
    st = out["stats"][0]
    sec = (st["ms_photon"] + st["ms_eye"]) / 1e3
    return {"value": photons / sec / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"1 pass of {photons} photons at {w}x{h} on the same scene (1/{sample_scale} of the photons "
                      f"and pixels), reference semantics, {threads} OpenMP threads; scene setup untimed"}


def equal_time_study(ctx, scene, common, ref_passes=4096, budget_passes=64):
    """relMSE of plain and learned-proposal renders against a ref_passes plain
    render (relMSE = mean over pixels and channels of (x - r)^2 / (r^2 + 0.01)).
    Plain renders budget_passes passes; their wall time is the budget. The
    learned render runs whole passes until the budget is spent. Both images
    are read at checkpoints (the reads are not counted in the wall times),
    which gives the learned render's relMSE at equal time and the first
    checkpoint at which it is at or below plain's final relMSE."""
    import pppm_gb300 as P

    checkpoints = {2, 4, 6, 8, 10, 12, 14, 16, 20, 24, 28, 32, 40, 48, 56, 64, 80, 96, 128}
    ref = None

    def rel(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    def render(flags, seed, passes=None, budget=None, curve=None):
        ctx.render_begin(scene.camera, P.Context.make_params(**dict(common, seed=seed, flags=flags)))
        el = 0.0
        t = 0
        while True:
            t += 1
            t0 = time.perf_counter()
            ctx.render_pass(t)
            el += time.perf_counter() - t0
            done = (passes is not None and t >= passes) or (budget is not None and el >= budget)
            if curve is not None and (t in checkpoints or done):
                curve.append({"passes": t, "seconds": round(el, 4), "relmse": rel(ctx.render_read() / t)})
            if done:
                break
        return ctx.render_read() / t, t, el

    ref, _, ref_s = render(0, 1000, passes=ref_passes)
    cp, cl = [], []
    plain, n_plain, budget = render(0, 7, passes=budget_passes, curve=cp)
    e_plain = rel(plain)
    ctx.learned_config(retrain_every=2, steps=2, batch=65536, lr=4e-3, floor_bsdf=0.3, max_log_kappa=7.0,
                       guide_bounces=0)
    learned, n_learned, el = render(P.FLAG_LEARNED, 7, budget=budget, curve=cl)
    match = next((c for c in cl if c["relmse"] <= e_plain), None)
    return {"reference_passes": ref_passes, "reference_s": ref_s, "budget_s": budget,
            "plain": {"passes": n_plain, "relmse": e_plain, "curve": cp},
            "learned": {"passes": n_learned, "seconds": el, "relmse": rel(learned), "curve": cl},
            "relmse_learned_over_plain": rel(learned) / e_plain,
            "learned_reaches_plain_relmse_at_s": match["seconds"] if match else None,
            "time_ratio_plain_over_learned": budget / match["seconds"] if match else None,
            "relmse": "mean((x - r)^2 / (r^2 + 0.01)) over pixels and channels",
            "learned_settings": "environment direction proposed by the network (8 vMF lobes at the emission input), "
                                "one-sample MIS with the reference's cell sampling at floor 0.3; retrain every 2 "
                                "passes, 2 Adam steps x 65536 records, lr 4e-3, max log kappa 7; bounces not "
                                "guided"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import port
    import pppm_gb300 as P

    scene = build_scene()
    threads = os.cpu_count() or 1
    scale = 16
    w, h = 1920 // 4, 1080 // 4
    photons = PHOTONS // scale
    cam = P.Context.make_camera(scene.camera)
    cam.width, cam.height = w, h
    par = P.Context.make_params(mode=P.MODE_COMPAT, photons=photons, num_streams=threads, max_bounce_photon=DEPTH,
                                max_bounce_eye=DEPTH)
    ps = port.PortScene(scene)
    out = ps.render(cam, par, args.warmup + args.steps)
    timed = out["stats"][args.warmup:]
    sec = sum((s["ms_photon"] + s["ms_eye"]) / 1e3 for s in timed)
    value = photons * args.steps / sec / 1e6
    sample = (f"each step: 1 pass of {photons} photons at {w}x{h} (1/{scale} of the photons and pixels of the "
              f"workload), reference semantics (kNN gather, growing radius), {threads} OpenMP threads")
    # n_gpus: the launch's N (rank 0 alone runs the CPU port)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config("compat", 1.0),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch

    import pppm_gb300 as P

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    scene = build_scene(args.workload)
    ctx = P.Context(local)
    ctx.set_scene(scene)
    compat = args.mode == "compat"
    common = dict(mode=P.MODE_COMPAT if compat else P.MODE_CANONICAL, photons=PHOTONS, num_streams=16,
                  max_bounce_photon=DEPTH, max_bounce_eye=DEPTH, radius_scale=0.1 if compat else 1 / 64,
                  seed=1 + rank, cell_factor=args.cell_factor)

    # one untimed pass with traversal counting: algorithmic bytes per ray
    ctx.render_begin(scene.camera, P.Context.make_params(**common, flags=P.FLAG_COUNT_TRAVERSAL))
    cnt = ctx.render_pass(1)

    ctx.render_begin(scene.camera, P.Context.make_params(**common))
    t = 1
    for _ in range(args.warmup):
        ctx.render_pass(t)
        t += 1
    stream = torch.cuda.ExternalStream(ctx.stream_ptr())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    stats = []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            stats.append(ctx.render_pass(t).as_dict())
            t += 1
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    value = world * args.steps * PHOTONS / (ms / 1e3) / 1e6

    # end to end through the C ABI: pass + image readback into pinned memory
    host = torch.empty((scene.camera.height, scene.camera.width, 3), dtype=torch.float32, pin_memory=True)
    hp = host.numpy()
    barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.render_pass(t)
        t += 1
        ctx.render_read(hp)
    e2e_s = time.perf_counter() - w0
    if world > 1:
        tt = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e = world * args.steps * PHOTONS / e2e_s / 1e6
    h2d = (16 * 16) if compat else 0  # per-pass stream states (compat only)
    d2h = host.numel() * 4 + 2 * 112  # image + two counter readbacks

    # roofline of the photon bounce kernels (traversal dominated): the
    # algorithmic bytes of a traversal, 32 B ray + 16 B hit + 128 B per node
    # visited + 48 B per triangle tested
    ms_bounce = sum(s["ms_bounce"] for s in stats) / len(stats)
    alg = cnt.photon_rays * 48 + cnt.photon_node_visits * 128 + cnt.photon_tri_tests * 48
    peak, peak_kind = measured_peak()
    achieved = alg / (ms_bounce / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "photon_bounce_traffic.json"
    if tf.exists():
        d = json.loads(tf.read_text())
        traffic = d.get("dram_bytes_per_pass")

    line = None
    if rank == 0:
        cfg = workload_config(args.mode, args.cell_factor, args.workload)
        clocks = clk.summary()
        per = {k: statistics.mean(s[k] for s in stats) for k in ("ms_photon", "ms_bounce", "ms_grid", "ms_eye",
                                                                   "ms_gather", "ms_subsurface",
                                                                   "ms_subsurface_host")}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (f64 triangle test, exact)", "data": "synthetic (seeded)",
                "config": cfg,
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "kernel": "kPhotonPersistent (all photon bounces)",
                             "peak_kind": peak_kind,
                             "algorithmic_bytes_per_pass": alg},
                "clocks": clocks,
                "stage_ms": per,
                "per_pass": {"photon_rays": cnt.photon_rays, "eye_rays": cnt.eye_rays,
                             "stored": int(stats[-1]["photons_stored"]), "queries": int(stats[-1]["gather_queries"]),
                             "node_visits_per_photon_ray": cnt.photon_node_visits / max(cnt.photon_rays, 1),
                             "tri_tests_per_photon_ray": cnt.photon_tri_tests / max(cnt.photon_rays, 1),
                             "gather_pairs_per_query": cnt.gather_pairs / max(cnt.gather_queries, 1),
                             "gather_inside_per_query": cnt.gather_inside / max(cnt.gather_queries, 1),
                             "sss_points": int(stats[-1]["sss_points"]), "sss_photons": int(stats[-1]["sss_photons"])}}
        if world == 1 and not args.no_cpu_baseline and args.workload == "config2":
            line["cpu_baseline"] = cpu_baseline(scene)
        if world == 1 and not args.no_study and args.workload == "config2" and args.mode == "canonical":
            line["equal_time_relmse"] = equal_time_study(ctx, scene, common)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batch(args):
    """Batched uneven jobs: aggregate Mrays/s over the whole batch and per-job
    pass latency p50/p99 (wall time of each pppm_render_pass)."""
    import pppm_gb300 as P
    import scenes as S

    rank, world, local = dist_env()
    if rank != 0:
        return 0
    jobs = S.config4_jobs(seed=4 + args.warmup)
    b = P.Batch(local)
    b.config(use_graph=not args.no_graph, graph_lanes=args.graph_lanes)
    ids = []
    for sc, alpha in jobs:
        par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=8,
                                    max_bounce_eye=8, alpha=alpha, radius_scale=1 / 64, seed=len(ids) + 1)
        ids.append(b.submit(sc, par, 16))
    with ClockSampler(local) as clk:
        b.run(autotune=True, max_concurrent=8)
    stats = [b.result(i, image=False)[1] for i in ids]
    wall = stats[0]["batch_wall_ms"] / 1e3
    rays = sum(s["rays"] for s in stats)
    shapes = {}
    for s in stats:
        k = f'cell {s["cell_factor"]:.2f} bounce {s["bounce_blocks_per_sm"]} eye {s["eye_blocks_per_sm"]}'
        shapes[k] = shapes.get(k, 0) + 1
    line = {"metric": "aggregate Mrays/s over 64 batched uneven jobs (config 4)", "value": rays / wall / 1e6,
            "unit": "Mrays/s", "n_gpus": 1, "steps": 16, "warmup": 0, "ms_per_step": wall * 1e3 / 16,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 triangle test)",
            "data": "synthetic (seeded)", "config": workload_config("canonical", 1.0, "config4"),
            "batch": {"jobs": len(ids), "wall_s": wall, "rays": rays,
                      "pass_ms_p50_median_over_jobs": statistics.median(s["ms_pass_p50"] for s in stats),
                      "pass_ms_p99_max_over_jobs": max(s["ms_pass_p99"] for s in stats),
                      "graph_passes": sum(s["graph_passes"] for s in stats),
                      "graph_s": stats[0]["batch_graph_ms"] / 1e3,
                      "graph_capture_s": stats[0]["batch_graph_capture_ms"] / 1e3,
                      "graph_instantiate_s": stats[0]["batch_graph_instantiate_ms"] / 1e3,
                      "autotuned_shapes": shapes},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    b.close()
    return 0


def main():
    args = parse()
    if args.workload == "config4" and args.impl == "gb300":
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
