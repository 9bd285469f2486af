#!/usr/bin/env python
"""Small, self-contained GPU cases for kernel profiling (ncu) and timing.

  python tatsy-pppm_gb300/profile_cases.py mlp_forward [rows]
  python tatsy-pppm_gb300/profile_cases.py mlp_train [records]
  python tatsy-pppm_gb300/profile_cases.py render [photons] [width] [height]
  python tatsy-pppm_gb300/profile_cases.py subsurface [passes] [full]
  python tatsy-pppm_gb300/profile_cases.py classic

Each case builds its inputs from seeded synthetic data, runs the kernels a
few times and prints one line of timings (CUDA events on the context
stream). Inputs are sized above the 129 MB L2 where the kernel streams
memory, and far below the device capacity, so a profiler capture of one or
two launches ends within seconds.
"""
from __future__ import annotations

import ctypes
import json
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import pppm_gb300 as P  # noqa: E402
import scenes as S  # noqa: E402


def _events(ctx):
    import torch

    st = torch.cuda.ExternalStream(ctx.stream_ptr())
    return st, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def mlp_forward(rows=4_000_000):
    import torch

    ctx = P.Context(0)
    rng = np.random.default_rng(0)
    pos = torch.tensor(rng.uniform(-30, 30, (rows, 3)).astype(np.float32), device="cuda")
    nrm = torch.nn.functional.normalize(torch.tensor(rng.normal(size=(rows, 3)).astype(np.float32), device="cuda"))
    out = torch.empty((rows, 40), device="cuda")
    params = torch.tensor(rng.normal(size=P.MLP_PARAMS).astype(np.float32) * 0.1, device="cuda")
    bb = np.array([-50.0, -50.0, -50.0, 50.0, 50.0, 50.0])
    call = lambda: ctx.lib.pppm_mlp_forward(ctx.h, params.data_ptr(), pos.data_ptr(), nrm.data_ptr(), rows,  # noqa
                                            bb.ctypes.data, out.data_ptr())
    for _ in range(3):
        assert call() == P.OK
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        call()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / 10 * 1e3
    print(json.dumps({"case": "mlp_forward", "rows": rows, "ms_per_call": ms,
                      "tflops_incl_pack": rows * 31.7e3 / (ms / 1e3) / 1e12}))


def mlp_train(records=65536):
    ctx = P.Context(0)
    rng = np.random.default_rng(1)
    pos = rng.uniform(-30, 30, (records, 3))
    n = rng.normal(size=(records, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    d = rng.normal(size=(records, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.lognormal(size=(records, 1))
    rec = np.concatenate([pos, n, d, w], 1).astype(np.float32)
    params = rng.normal(size=P.MLP_PARAMS).astype(np.float32) * 0.1
    bb = np.array([-50.0, -50.0, -50.0, 50.0, 50.0, 50.0])
    for _ in range(2):
        ctx.mlp_grad(params, rec, bb)
    t0 = time.perf_counter()
    for _ in range(5):
        loss, g = ctx.mlp_grad(params, rec, bb)
    ms = (time.perf_counter() - t0) / 5 * 1e3
    print(json.dumps({"case": "mlp_train", "records": records, "ms_per_step_incl_host": ms, "loss": loss}))


def render(photons=1_000_000, width=960, height=540, passes=3):
    sc = S.config2(width=int(width), height=int(height))
    ctx = P.Context(0)
    ctx.set_scene(sc)
    par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=int(photons), max_bounce_photon=12,
                                max_bounce_eye=12, radius_scale=1 / 64, seed=1)
    ctx.render_begin(sc.camera, par)
    out = [ctx.render_pass(t + 1).as_dict() for t in range(passes)]
    keys = ("ms_photon", "ms_bounce", "ms_grid", "ms_eye", "ms_gather", "photon_rays", "eye_rays", "photons_stored")
    print(json.dumps({"case": "render", "photons": photons, "w": width, "h": height,
                      **{k: out[k2][k] for k2 in (-1,) for k in keys}, "photon_rays_per_pass": [o["photon_rays"] for o in out]}))


def subsurface(passes=3, full=0):
    """full=1: the subsurface workload's own sizes (1280x720, 2M photons,
    200k-triangle torus); else a quarter-size case."""
    sc = S.config3() if full else S.config3(width=640, height=360, photons=1_000_000, nu=250, nv=100)
    ctx = P.Context(0)
    ctx.set_scene(sc)
    par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=12,
                                max_bounce_eye=12, radius_scale=1 / 64, seed=1)
    ctx.render_begin(sc.camera, par)
    out = [ctx.render_pass(t + 1).as_dict() for t in range(passes)]
    keys = ("ms_subsurface", "ms_subsurface_host", "ms_photon", "ms_eye", "ms_gather", "sss_points", "sss_photons")
    print(json.dumps({"case": "subsurface", **{k: out[-1][k] for k in keys}}))


def classic(passes=3):
    sc = S.config2(width=480, height=270, freq=96)
    ctx = P.Context(0)
    ctx.set_scene(sc)
    par = P.Context.make_params(mode=P.MODE_CLASSIC, photons=1_000_000, num_streams=16, max_bounce_photon=12,
                                max_bounce_eye=12)
    ctx.render_begin(sc.camera, par)
    out = [ctx.render_pass(t + 1).as_dict() for t in range(passes)]
    keys = ("ms_eye", "ms_grid", "ms_photon", "ms_gather", "photons_stored")
    print(json.dumps({"case": "classic", **{k: out[-1][k] for k in keys}}))


if __name__ == "__main__":
    case = sys.argv[1]
    args = [float(a) if "." in a else int(a) for a in sys.argv[2:]]
    {"mlp_forward": mlp_forward, "mlp_train": mlp_train, "render": render, "subsurface": subsurface,
     "classic": classic}[case](*args)
