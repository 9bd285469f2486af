#!/usr/bin/env python
"""PPM-APA pass throughput on GB300 (the 1080p at-scale workload).

Workload (one step = one render pass): 1920x1080, a noise-displaced geodesic
sphere of 873,620 triangles (frequency 209) over a ground quad, lit by a
seeded 2048x1024 FP32 equirect sky (gradient + 0.5 degree sun lobe of peak
5e4 + lognormal texel noise sigma 0.3), materials 60/20/20 Lambertian /
mirror / dielectric per surface cluster, 4M photons per pass, alpha 0.7,
r1 = diag/64, photon and eye depth 12, canonical Knaus-Zwicker mode. Data
are synthetic (seeded); nothing is downloaded.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--mode canonical|compat] [--workload config2|config3|config4]
                  [--case mlp_forward|mlp_train|render|subsurface|classic ...]

--impl gb300 (default) times the hand-written sm_103a kernels through the C
ABI: `value` is the device time of passes W+1..W+K with every input resident
in HBM; `e2e` replays the same passes (same indices, same radii) through
pppm_render_pass + pppm_render_read into pinned host memory, wall clock.
--impl reference times the CPU restatement of the same workload (the oracle
port, oracle/pppm_port.cc: the reference's algorithm pinned bit-exact to the
compiled reference in compat mode, with the same canonical gather as the GPU
arm) on all host cores, passes W+1..W+K of the identical configuration.
The default gb300 run also carries, as extra keys: the CPU baseline, a
full-size compat-mode figure for both GPU and port, the subsurface (config3)
and batched-jobs (config4) workloads, and the equal-time learned-vs-plain
relMSE study. --case runs one small profiling case (kernel timings only).
Multi-GPU runs are replicas (passes shard with no exchange until one image
reduction, not timed here).
"""
from __future__ import annotations

import argparse
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
# issue slots: 4 warp schedulers per SM, one warp instruction each per cycle
SMS, SCHEDULERS_PER_SM = 152, 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="canonical", choices=["canonical", "compat"])
    ap.add_argument("--cell-factor", type=float, default=1.0)
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-study", action="store_true", help="skip the equal-time learned-vs-plain relMSE study")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the compat, config3, config4 and cold end-to-end extra keys")
    ap.add_argument("--study-seeds", type=int, default=3)
    ap.add_argument("--no-graph", action="store_true", help="config4: run every pass through pppm_render_pass")
    ap.add_argument("--graph-lanes", type=int, default=0, help="config4: jobs at once inside the graph")
    ap.add_argument("--case", default=None, choices=["mlp_forward", "mlp_train", "render", "subsurface", "classic"],
                    help="one small profiling case instead of the bench")
    ap.add_argument("--photons", type=int, default=1_000_000, help="--case render/classic: photons per pass")
    ap.add_argument("--width", type=int, default=960, help="--case render/classic: image width")
    ap.add_argument("--height", type=int, default=540, help="--case render/classic: image height")
    ap.add_argument("--passes", type=int, default=3, help="--case: passes per render")
    ap.add_argument("--rows", type=int, default=4_000_000, help="--case mlp_forward: network rows")
    ap.add_argument("--records", type=int, default=65536, help="--case mlp_train: training records")
    ap.add_argument("--full", action="store_true", help="--case subsurface: the config3 sizes")
    ap.add_argument("--count", action="store_true", help="--case render: a first render with traversal counting")
    return ap.parse_args()


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
            "l2": "inputs larger than L2 (photon map, path queues and BVH ~1.5 GB per pass), no flush"}


def params_for(P, mode, workload, seed, threads, cell_factor=1.0, flags=0):
    w = WORKLOADS[workload]
    compat = mode == "compat"
    return P.Context.make_params(mode=P.MODE_COMPAT if compat else P.MODE_CANONICAL, photons=w["photons"],
                                 num_streams=threads, max_bounce_photon=w["depth"], max_bounce_eye=w["depth"],
                                 radius_scale=0.1 if compat else 1 / 64, seed=seed, cell_factor=cell_factor,
                                 flags=flags)


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
        return float(d["hbm_gbs"]), "measured", float(d.get("sm_max_mhz", 2070.0))
    return 6800.0, "fallback", 2070.0


def profile_json(name):
    p = ROOT / "profiles" / name
    return json.loads(p.read_text()) if p.exists() else {}


def port_passes(scene, mode, passes, threads, warm):
    """Passes 1..passes of the oracle port on the host cores; returns the
    wall time of passes warm+1..passes (photon trace + map build + eye paths
    and gather, as the reference's pass loop times them) and the radii."""
    import port
    import pppm_gb300 as P

    cam = P.Context.make_camera(scene.camera)
    par = params_for(P, mode, "config2", 1, threads)
    ps = port.PortScene(scene)
    out = ps.render(cam, par, passes)
    st = out["stats"][warm:]
    return sum((s["ms_photon"] + s["ms_eye"]) / 1e3 for s in st), [s["radius"] for s in out["stats"]]


def cpu_baseline(scene, threads):
    """The port on the host cores: passes 2-3 of the full workload (pass 1
    untimed), canonical mode, all threads."""
    sec, _ = port_passes(scene, "canonical", 3, threads, 1)
    photons = WORKLOADS["config2"]["photons"]
    return {"value": 2 * photons / sec / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"passes 2-3 (pass 1 untimed) of the full workload: 1920x1080, 4M photons, canonical, "
                      f"r1 = diag/64, depth 12; oracle port on {threads} OpenMP threads; scene set-up untimed"}


def compat_full_size(ctx, scene, threads):
    """Full-size compat mode (the reference's semantics: kNN gather with
    k = (int)r, growing radius, phantom photons, per-stream tapes) on the GPU
    and on the port, passes 2-3 of the same render (pass 1 untimed)."""
    import torch

    import pppm_gb300 as P

    photons = WORKLOADS["config2"]["photons"]
    ctx.render_begin(scene.camera, params_for(P, "compat", "config2", 1, threads))
    ctx.render_pass(1)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for t in (2, 3):
        ctx.render_pass(t)
    e1.record(stream)
    torch.cuda.synchronize()
    gpu = 2 * photons / (e0.elapsed_time(e1) / 1e3) / 1e6
    sec, radii = port_passes(scene, "compat", 3, threads, 1)
    cpu = 2 * photons / sec / 1e6
    return {"gpu": gpu, "port": cpu, "unit": UNIT, "gpu_over_port": gpu / cpu, "passes_timed": [2, 3],
            "port_threads": threads, "num_streams": threads, "radii": radii,
            "what": "compat mode at the full size (1920x1080, 4M photons, r1 = 0.1 diag, depth 12): the reference's "
                    "own semantics; GPU device time vs the oracle port on all host cores, same passes"}


def counted_passes(ctx, scene, common, warm, steps):
    """Traversal and gather counters of passes warm+1..warm+steps (the timed
    passes) from a separate counting render: canonical passes depend only on
    their index, so the counting render skips to them."""
    import pppm_gb300 as P

    par = P.Context.make_params(**dict(common, flags=P.FLAG_COUNT_TRAVERSAL))
    ctx.render_begin(scene.camera, par)
    if warm:
        ctx.render_skip(warm)
    keys = ("photon_rays", "photon_node_visits", "photon_tri_tests", "gather_pairs", "gather_inside",
            "gather_queries", "eye_rays", "node_visits", "tri_tests")
    tot = dict.fromkeys(keys, 0)
    for t in range(warm + 1, warm + steps + 1):
        st = ctx.render_pass(t)
        for k in keys:
            tot[k] += getattr(st, k)
    return {k: v / steps for k, v in tot.items()}


def rooflines(cnt, stats, clocks):
    """Photon-pass roofline (the pass's byte model against the measured HBM copy
    bandwidth, plus the DRAM fraction the ncu capture gives) and the gather's
    issue-rate roofline (warp instructions per second against the SMs' issue
    slots)."""
    peak, peak_kind, sm_max = measured_peak()
    ms_bounce = statistics.mean(s["ms_bounce"] for s in stats)
    alg = cnt["photon_rays"] * 48 + cnt["photon_node_visits"] * 128 + cnt["photon_tri_tests"] * 48
    achieved = alg / (ms_bounce / 1e3) / 1e9
    traf = profile_json("photon_bounce_traffic.json")
    traffic = traf.get("dram_bytes_per_pass")
    photon = {"bound": "latency/divergence", "ceiling": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
              "frac": achieved / peak, "traffic": traffic, "kernel": "kPhotonPersistent (all photon bounces)",
              "peak_kind": peak_kind, "algorithmic_bytes_per_pass": alg,
              "model": "photon-pass byte model: 48 B per ray + 128 B per BVH node visited + 48 B per triangle tested "
                       "(counted live over the timed passes); most of these bytes are L1/L2 hits"}
    if traffic:
        photon["dram_achieved"] = traffic / (ms_bounce / 1e3) / 1e9
        photon["dram_frac"] = photon["dram_achieved"] / peak
    if "threads_per_inst" in traf:
        photon["lanes_per_instruction"] = traf["threads_per_inst"]
        photon["lanes_source"] = "smsp__thread_inst_executed / smsp__inst_executed of the committed capture"
    gat = profile_json("gather_tiled_issue.json")
    ms_gather = statistics.mean(s["ms_gather"] for s in stats)
    mhz = (clocks or {}).get("sm_mhz") or sm_max
    issue_peak = SMS * SCHEDULERS_PER_SM * mhz * 1e6 / 1e9
    gather = {"bound": "issue", "kernel": "kGatherTiled (canonical gather, incl. its small set-up launches)",
              "unit": "G warp-instructions/s", "peak": issue_peak,
              "peak_model": f"{SMS} SMs x {SCHEDULERS_PER_SM} schedulers x 1 warp instruction per cycle at the "
                            f"sampled SM clock {mhz:.0f} MHz",
              "pairs_per_query": cnt["gather_pairs"] / max(cnt["gather_queries"], 1),
              "inside_per_query": cnt["gather_inside"] / max(cnt["gather_queries"], 1),
              "pair_tests_per_s": cnt["gather_pairs"] / (ms_gather / 1e3)}
    if "warp_inst_per_pair" in gat:
        ach = gat["warp_inst_per_pair"] * cnt["gather_pairs"] / (ms_gather / 1e3) / 1e9
        gather.update({"achieved": ach, "frac": ach / issue_peak, "warp_inst_per_pair": gat["warp_inst_per_pair"],
                       "traffic": gat.get("dram_bytes_per_launch")})
    return photon, gather


def run_gb300(args):
    import torch

    import pppm_gb300 as P

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    W = WORKLOADS[args.workload]
    photons = W["photons"]
    threads = os.cpu_count() or 1
    scene = build_scene(args.workload)
    ctx = P.Context(local)
    ctx.set_scene(scene)
    compat = args.mode == "compat"
    common = dict(mode=P.MODE_COMPAT if compat else P.MODE_CANONICAL, photons=photons, num_streams=16,
                  max_bounce_photon=W["depth"], max_bounce_eye=W["depth"], radius_scale=0.1 if compat else 1 / 64,
                  seed=1 + rank, cell_factor=args.cell_factor)

    # counters of the timed passes (untimed counting render)
    cnt = counted_passes(ctx, scene, common, args.warmup, args.steps) if not compat else None

    ctx.render_begin(scene.camera, P.Context.make_params(**common))
    t = 1
    for _ in range(args.warmup):
        ctx.render_pass(t)
        t += 1
    stream = torch.cuda.ExternalStream(ctx.stream_ptr())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    raw = []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            raw.append(ctx.render_pass(t))
            t += 1
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    # the per-pass statistics as dicts, outside the timed region
    stats = [s.as_dict() for s in raw]
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    value = world * args.steps * photons / (ms / 1e3) / 1e6

    # end to end through the C ABI on the same passes: a fresh render, the
    # warm-up passes untimed, then passes W+1..W+K each followed by the read
    # of the accumulator into pinned host memory (the reference writes an
    # image after every pass)
    host = torch.empty((scene.camera.height, scene.camera.width, 3), dtype=torch.float32, pin_memory=True)
    hp = host.numpy()
    ctx.render_begin(scene.camera, P.Context.make_params(**common))
    for t in range(1, args.warmup + 1):
        ctx.render_pass(t)
    barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for t in range(args.warmup + 1, args.warmup + args.steps + 1):
        ctx.render_pass(t)
        ctx.render_read(hp)
    e2e_s = time.perf_counter() - w0
    if world > 1:
        tt = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e = world * args.steps * photons / e2e_s / 1e6
    h2d = (16 * 16) if compat else 0  # per-pass stream states (compat only)
    d2h = host.numel() * 4 + 2 * 112  # image + two counter readbacks

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
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "passes": [args.warmup + 1, args.warmup + args.steps],
                        "note": "scene resident (uploaded once by pppm_scene_set / pppm_env_set before the timed "
                                "region); per-pass upload = pass parameters only (by value); per-pass download = "
                                "the W x H x 3 FP32 accumulator + pass counters; same pass indices as value"},
                "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
                "clocks": clocks,
                "stage_ms": per}
        if cnt is not None:
            photon_roof, gather_roof = rooflines(cnt, stats, clocks)
            line["roofline"] = photon_roof
            line["roofline_gather"] = gather_roof
            line["per_pass"] = {"photon_rays": cnt["photon_rays"], "eye_rays": cnt["eye_rays"],
                                "stored": int(stats[-1]["photons_stored"]),
                                "queries": int(stats[-1]["gather_queries"]),
                                "node_visits_per_photon_ray": cnt["photon_node_visits"] / max(cnt["photon_rays"], 1),
                                "tri_tests_per_photon_ray": cnt["photon_tri_tests"] / max(cnt["photon_rays"], 1),
                                "mrays_per_s": (cnt["photon_rays"] + cnt["eye_rays"]) / (ms / args.steps / 1e3) / 1e6,
                                "counters": "means over the timed passes (separate counting render)"}
        full = world == 1 and args.workload == "config2" and not compat
        if full and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(scene, threads)
            line["passes_per_s"] = {"gpu": 1e3 / (ms / args.steps),
                                    "cpu_port_all_cores": line["cpu_baseline"]["value"] / (photons / 1e6),
                                    "what": "passes per second at the full workload; the target is >= 50x"}
            line["passes_per_s"]["gpu_over_cpu"] = line["passes_per_s"]["gpu"] / line["passes_per_s"]["cpu_port_all_cores"]
        if full and not args.no_extra:
            line["e2e_cold"] = e2e_cold(ctx, scene, common, args.steps)
            line["compat_full_size"] = compat_full_size(ctx, scene, threads)
        if full and not args.no_study:
            line["equal_time_relmse"] = equal_time_study(ctx, scene, common, seeds=args.study_seeds)
        ctx.close()
        if full and not args.no_extra:
            line["config3"] = config3_line(local, args)
            line["config4"] = run_batch(args, as_extra=True)
        print(json.dumps(line), flush=True)
    else:
        ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def e2e_cold(ctx, scene, common, steps):
    """The reference's render() call as a user makes it, from host buffers:
    scene and env upload, BVH build, env tables, render set-up, `steps`
    passes and the accumulator read, all inside the wall-clock region."""
    import torch

    import pppm_gb300 as P

    host = torch.empty((scene.camera.height, scene.camera.width, 3), dtype=torch.float32, pin_memory=True)
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    ctx.set_scene(scene)
    ctx.render_begin(scene.camera, P.Context.make_params(**common))
    for t in range(1, steps + 1):
        ctx.render_pass(t)
    ctx.render_read(host.numpy())
    sec = time.perf_counter() - w0
    h2d = scene.tris.nbytes + scene.mat_id.nbytes + scene.mats.nbytes + scene.env.nbytes
    return {"value": steps * common["photons"] / sec / 1e6, "unit": UNIT, "seconds": sec, "passes": [1, steps],
            "h2d_bytes": int(h2d), "d2h_bytes": int(host.numel() * 4),
            "what": "one pppm_scene_set + pppm_env_set (upload, host BVH build, env tables) + render_begin + "
                    f"{steps} passes + one accumulator read, wall clock"}


def config3_line(local, args):
    """The subsurface workload (config 3): device time per pass."""
    import torch

    import pppm_gb300 as P

    sc = build_scene("config3")
    ctx = P.Context(local)
    try:
        ctx.set_scene(sc)
        par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=12,
                                    max_bounce_eye=12, radius_scale=1 / 64, seed=1)
        ctx.render_begin(sc.camera, par)
        warm, steps = 2, 8
        for t in range(1, warm + 1):
            ctx.render_pass(t)
        stream = torch.cuda.ExternalStream(ctx.stream_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        raw = [ctx.render_pass(t) for t in range(warm + 1, warm + steps + 1)]
        e1.record(stream)
        torch.cuda.synchronize()
        stats = [s.as_dict() for s in raw]
        ms = e0.elapsed_time(e1) / steps
    finally:
        ctx.close()
    keys = ("ms_subsurface", "ms_photon", "ms_eye", "ms_gather", "ms_grid")
    return {"value": sc.photons / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_pass": ms, "passes": [warm + 1, warm + steps],
            "config": workload_config("canonical", 1.0, "config3"),
            "sss_points": int(stats[-1]["sss_points"]), "sss_photons": int(stats[-1]["sss_photons"]),
            "stage_ms": {k: statistics.mean(s[k] for s in stats) for k in keys},
            "note": "irradiance points follow the reference's areaRadius rule (ppm_probabilistic.cc:35-46)"}


def run_reference(args):
    """The CPU restatement (oracle port) of the identical workload and
    configuration on all host cores: passes W+1..W+K timed, as the GPU arm."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    scene = build_scene()
    sec, _ = port_passes(scene, args.mode, args.warmup + args.steps, threads, args.warmup)
    photons = WORKLOADS["config2"]["photons"]
    value = photons * args.steps / sec / 1e6
    sample = (f"passes {args.warmup + 1}-{args.warmup + args.steps} of the full workload (warm-up passes untimed), "
              f"{args.mode} mode, oracle port on {threads} OpenMP threads; per pass: photon trace + photon map "
              f"build + eye paths and gather")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": workload_config(args.mode, args.cell_factor),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- learned vs plain
def _stays_below(curve, target):
    """Earliest checkpoint after which the curve never rises above target."""
    at = None
    for c in curve:
        if c["relmse"] <= target:
            if at is None:
                at = c
        else:
            at = None
    return at


def _first_below(curve, target):
    return next((c for c in curve if c["relmse"] <= target), None)


def equal_time_study(ctx, scene, common, seeds=3, ref_passes=4096, budget_passes=64):
    """relMSE of several samplers against a ref_passes plain render
    (relMSE = mean over pixels and channels of (x - r)^2 / (r^2 + 0.01)),
    at equal wall time. For each seed the plain render's budget_passes
    passes set the time budget and the target (its final relMSE); every arm
    runs whole passes until the budget is spent. One rule on every curve:
    the time to the target is the earliest checkpoint after which the curve
    stays at or below it (the first checkpoint at or below it is reported
    too). Checkpoint reads are not counted in the wall times."""
    import torch

    import pppm_gb300 as P

    checkpoints = set(range(2, 65, 2)) | {80, 96, 128}
    H, Wd = scene.camera.height, scene.camera.width
    img = torch.empty((H, Wd, 3), dtype=torch.float32, device="cuda")
    ref = None

    def read():
        ctx.render_read(img)
        ctx.sync()
        return img

    def rel(x, t):
        y = x / t
        return float(((y - ref) ** 2 / (ref ** 2 + 1e-2)).mean().item())

    def render(flags, seed, passes=None, budget=None, curve=None):
        ctx.render_begin(scene.camera, P.Context.make_params(**dict(common, seed=seed, flags=flags)))
        el, t, train = 0.0, 0, 0.0
        while True:
            t += 1
            t0 = time.perf_counter()
            st = ctx.render_pass(t)
            el += time.perf_counter() - t0
            train += st.ms_train
            done = (passes is not None and t >= passes) or (budget is not None and el >= budget)
            if curve is not None and (t in checkpoints or done):
                curve.append({"passes": t, "seconds": round(el, 4), "relmse": rel(read(), t)})
            if done:
                break
        return t, el, train

    render(0, 1000, passes=ref_passes)
    ref = read().clone() / ref_passes
    arms = {
        "luminance": dict(exponent=1.0, learned=None),
        "learned_config5": dict(exponent=2.0, learned=dict(retrain_every=4, steps=8, batch=65536, lr=1e-3,
                                                             floor_bsdf=0.3, max_log_kappa=7.0, guide_bounces=0)),
        "learned_tuned": dict(exponent=2.0, learned=dict(retrain_every=2, steps=2, batch=65536, lr=4e-3,
                                                           floor_bsdf=0.3, max_log_kappa=7.0, guide_bounces=0)),
        "learned_tuned_guided_bounces": dict(exponent=2.0, learned=dict(retrain_every=2, steps=2, batch=65536,
                                                                          lr=4e-3, floor_bsdf=0.3, max_log_kappa=7.0,
                                                                          guide_bounces=1)),
        "learned_tuned_over_luminance": dict(exponent=1.0, learned=dict(retrain_every=2, steps=2, batch=65536,
                                                                          lr=4e-3, floor_bsdf=0.3,
                                                                          max_log_kappa=7.0, guide_bounces=0)),
    }
    per_seed = []
    for s in range(seeds):
        seed = 7 + s
        cp = []
        ctx.env_importance(2.0)
        n_plain, budget, _ = render(0, seed, passes=budget_passes, curve=cp)
        target = cp[-1]["relmse"]
        row = {"seed": seed, "budget_s": budget, "target_relmse": target,
               "plain": {"passes": n_plain, "relmse": target, "curve": cp,
                         "stays_below_s": _stays_below(cp, target)["seconds"],
                         "first_below_s": _first_below(cp, target)["seconds"]}}
        for name, arm in arms.items():
            ctx.env_importance(arm["exponent"])
            flags = 0
            if arm["learned"]:
                ctx.learned_config(**arm["learned"])
                flags = P.FLAG_LEARNED
            cv = []
            n, el, train = render(flags, seed, budget=budget, curve=cv)
            sb, fb = _stays_below(cv, target), _first_below(cv, target)
            row[name] = {"passes": n, "seconds": el, "train_ms": train, "relmse": cv[-1]["relmse"], "curve": cv,
                         "stays_below_s": sb["seconds"] if sb else None,
                         "first_below_s": fb["seconds"] if fb else None}
        ctx.env_importance(2.0)
        per_seed.append(row)

    def ratio(num, den, key):
        vals = [r[num][key] / r[den][key] for r in per_seed if r[num][key] and r[den][key]]
        return {"mean": statistics.mean(vals) if vals else None, "per_seed": vals,
                "seeds_reaching": len(vals)}

    def rel_ratio(a, b):
        vals = [r[a]["relmse"] / r[b]["relmse"] for r in per_seed]
        return {"mean": statistics.mean(vals), "per_seed": vals}

    summary = {}
    for name in ["luminance", *[a for a in arms if a != "luminance"]]:
        summary[name] = {"time_ratio_plain_over_arm": ratio("plain", name, "stays_below_s"),
                         "time_ratio_plain_over_arm_first_below": ratio("plain", name, "first_below_s"),
                         "relmse_arm_over_plain_at_equal_time": rel_ratio(name, "plain")}
    summary["learned_config5_vs_luminance"] = {
        "time_ratio_luminance_over_learned": ratio("luminance", "learned_config5", "stays_below_s"),
        "relmse_learned_over_luminance_at_equal_time": rel_ratio("learned_config5", "luminance")}
    summary["learned_tuned_vs_luminance"] = {
        "time_ratio_luminance_over_learned": ratio("luminance", "learned_tuned", "stays_below_s"),
        "relmse_learned_over_luminance_at_equal_time": rel_ratio("learned_tuned", "luminance")}
    head = summary["learned_config5"]["time_ratio_plain_over_arm"]["mean"]
    return {"reference_passes": ref_passes, "budget_passes_plain": budget_passes, "seeds": [r["seed"] for r in per_seed],
            "time_ratio_plain_over_learned": head,
            "headline": "learned_config5 (retrain every 4 passes, 8 Adam steps x 65,536 records, lr 1e-3, MIS floor "
                        "0.3): mean over seeds of plain's time to its own final relMSE over the learned arm's, "
                        "both by the stays-below rule",
            "rule": "time to target = earliest checkpoint after which the curve stays <= target (the plain "
                    "render's relMSE after 64 passes, per seed); first_below = first checkpoint <= target",
            "relmse": "mean((x - r)^2 / (r^2 + 0.01)) over pixels and channels",
            "arms": {"plain": "the reference's environment sampling (cell pdf ~ luminance^2)",
                     "luminance": "plain with the cell pdf ~ luminance (pppm_env_importance(1)), no network",
                     "learned_config5": "network proposes the environment direction (8 vMF lobes at the emission "
                                        "input), one-sample MIS with the reference's cell draw at floor 0.3; "
                                        "retrain every 4 passes, 8 steps, lr 1e-3",
                     "learned_tuned": "same, retrain every 2 passes, 2 steps, lr 4e-3",
                     "learned_tuned_guided_bounces": "learned_tuned + the network evaluated per photon at its "
                                                     "Lambertian hit position and normal, proposing the bounce "
                                                     "direction (MIS with the cosine lobe at floor 0.3)",
                     "learned_tuned_over_luminance": "learned_tuned with the luminance cell pdf as the MIS "
                                                     "defensive component"},
            "summary": summary, "per_seed": per_seed}


# ---------------------------------------------------------------- config 4
def run_batch(args, as_extra=False):
    """Batched uneven jobs: aggregate Mrays/s over the whole batch and per-job
    pass latency p50/p99 (device time of each pass inside the batch graphs;
    wall time of the eager first pass)."""
    import pppm_gb300 as P
    import scenes as S

    rank, world, local = dist_env()
    if rank != 0:
        return 0
    jobs = S.config4_jobs(seed=4 + (3 if as_extra else args.warmup))
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
        k = (f'candidate {s["tune_candidate"]}: cell {s["cell_factor"]:.2f} bounce {s["bounce_blocks_per_sm"]} '
             f'eye {s["eye_blocks_per_sm"]} refill {s["refill"]} exact {s["exact_batch"]} '
             f'stage {s["gather_stage"]} sub {s["query_sub_bits"]}')
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
                      "autotuned_shapes": shapes,
                      "tuning": (f"{stats[0]['tune_passes']} of 16 passes per job: {stats[0]['tune_passes'] // 3} "
                                 "candidate settings of every pppm_tune knob, 3 interleaved passes each, captured "
                                 "in the first batch graph; the rest of the job runs the lowest median")},
            "clocks": clk.summary()}
    b.close()
    if as_extra:
        return line
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- profiling cases
def run_case(args):
    """Small, seeded cases for kernel profiling (ncu) and timing: each builds
    its inputs, runs the kernels a few times and prints one line of timings.
    Inputs exceed the 129 MB L2 where the kernel streams memory and stay far
    below the device capacity, so a capture of one or two launches ends
    within seconds."""
    import torch

    import pppm_gb300 as P
    import scenes as S

    ctx = P.Context(0)
    out = {"case": args.case}
    if args.case == "mlp_forward":
        rows = args.rows
        rng = np.random.default_rng(0)
        pos = torch.tensor(rng.uniform(-30, 30, (rows, 3)).astype(np.float32), device="cuda")
        nrm = torch.nn.functional.normalize(torch.tensor(rng.normal(size=(rows, 3)).astype(np.float32), device="cuda"))
        res = torch.empty((rows, 40), device="cuda")
        params = torch.tensor(rng.normal(size=P.MLP_PARAMS).astype(np.float32) * 0.1, device="cuda")
        bb = np.array([-50.0, -50.0, -50.0, 50.0, 50.0, 50.0])

        def call():
            return ctx.lib.pppm_mlp_forward(ctx.h, params.data_ptr(), pos.data_ptr(), nrm.data_ptr(), rows,
                                            bb.ctypes.data, res.data_ptr())
        for _ in range(3):
            assert call() == P.OK
        stream = torch.cuda.ExternalStream(ctx.stream_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(10):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 10
        out.update(rows=rows, ms_per_call=ms, tflops=rows * 31.7e3 / (ms / 1e3) / 1e12)
    elif args.case == "mlp_train":
        rng = np.random.default_rng(1)
        n = args.records
        pos = rng.uniform(-30, 30, (n, 3))
        nr = rng.normal(size=(n, 3))
        nr /= np.linalg.norm(nr, axis=1, keepdims=True)
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        w = rng.lognormal(size=(n, 1))
        rec = np.concatenate([pos, nr, d, w], 1).astype(np.float32)
        params = rng.normal(size=P.MLP_PARAMS).astype(np.float32) * 0.1
        bb = np.array([-50.0, -50.0, -50.0, 50.0, 50.0, 50.0])
        for _ in range(2):
            ctx.mlp_grad(params, rec, bb)
        t0 = time.perf_counter()
        for _ in range(5):
            loss, _g = ctx.mlp_grad(params, rec, bb)
        out.update(records=n, ms_per_step_incl_host=(time.perf_counter() - t0) / 5 * 1e3, loss=loss)
    elif args.case in ("render", "subsurface", "classic"):
        if args.case == "render":
            sc = S.config2(width=args.width, height=args.height)
            par = dict(mode=P.MODE_CANONICAL, photons=args.photons, max_bounce_photon=12, max_bounce_eye=12,
                       radius_scale=1 / 64, seed=1)
        elif args.case == "subsurface":
            sc = S.config3() if args.full else S.config3(width=640, height=360, photons=1_000_000, nu=250, nv=100)
            par = dict(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=12, max_bounce_eye=12,
                       radius_scale=1 / 64, seed=1)
        else:
            sc = S.config2(width=args.width, height=args.height, freq=96)
            par = dict(mode=P.MODE_CLASSIC, photons=args.photons, num_streams=16, max_bounce_photon=12,
                       max_bounce_eye=12)
        ctx.set_scene(sc)
        if args.count and args.case == "render":
            ctx.render_begin(sc.camera, P.Context.make_params(**par, flags=P.FLAG_COUNT_TRAVERSAL))
            keys = ("photon_rays", "photon_node_visits", "photon_tri_tests", "gather_pairs", "gather_inside",
                    "gather_queries")
            counted = [ctx.render_pass(t + 1) for t in range(args.passes)]
            out["counted"] = [{k: getattr(st, k) for k in keys} for st in counted]
        ctx.render_begin(sc.camera, P.Context.make_params(**par))
        res = [ctx.render_pass(t + 1).as_dict() for t in range(args.passes)]
        keys = ("ms_subsurface", "ms_photon", "ms_bounce", "ms_grid", "ms_eye", "ms_gather", "photon_rays",
                "eye_rays", "photons_stored", "sss_points")
        out.update({k: res[-1][k] for k in keys}, photons=par["photons"], w=sc.camera.width, h=sc.camera.height)
    ctx.close()
    print(json.dumps(out), flush=True)
    return 0


def main():
    args = parse()
    if args.case:
        return run_case(args)
    if args.workload == "config4" and args.impl == "gb300":
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
