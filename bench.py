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
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="canonical", choices=["canonical", "compat"])
    ap.add_argument("--cell-factor", type=float, default=1.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
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
    """nvidia-smi samples every 200 ms while the timed region runs."""

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
                                          "-i", str(self.device), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
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
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
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
    # traversal bytes per ray of the survey's byte model, 32 B ray + 16 B hit
    # + 128 B per node visited + 48 B per triangle tested
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
                             "frac": achieved / peak, "traffic": traffic, "kernel": "kPhotonBounce (all bounces)",
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
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
