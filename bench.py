#!/usr/bin/env python3
"""Throughput of the icosahedral global orientation search at box 256.

Workload (the production-size plain-method configuration): 256x256 particles at
1.5 A/px, band 1/50 - 1/6 A^-1 (minR 7, maxR 64), 1-degree asymmetric-unit grid
(Nomega 360), 20 templates, CTF 300 kV / 2.7 mm / 0.07 with defocus 0.8-3.5 um and
astigmatism up to 0.1 um, SNR 0.05, origins within +-6 px.  Synthetic, seeded
(phantom: Gaussian blobs placed by the 60 icosahedral rotations plus a shell; random-
init inputs with the workload's shapes and value distributions).

A step is one call of the reference-facing search (cryoim_globesearch*, the
replacement of ort_globesearch.f90) over one batch of particles.  `value` is
particles/s with the images already resident in HBM; `e2e` is the same call with host
(pinned) images, host->device copies inside the timed region.  The L2 is flushed
(256 MiB write) before every timed step.

--impl reference times the reference algorithm's CPU restatement (the oracle port,
FP32 in the Fortran's operation order) on all host cores over a bounded sample of
views of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(nx=256, apix=1.5, min_res=50.0, max_res=6.0, searchstep=1.0, ntemplates=20,
                df=(0.8, 3.5), astig=0.1, snr=0.05, origin=6.0, ampwg=0.07, seed=20261205)
METRIC = "particles/s (box 256), FP32 cross-common-line PR global search, 1-deg ASU grid"
FP32_PEAK_TFLOPS_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12  # FMA lanes x 2 flop x max SM clock
FLOPS_PER_TERM = 30.0


def rank_env():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


def make_params(ci):
    w = WORKLOAD
    return ci.default_params(w["nx"], apix=w["apix"], minRes=w["min_res"], maxRes=w["max_res"],
                             searchstep=w["searchstep"], ampwg=w["ampwg"],
                             imgmask=(w["nx"] // 2 - 2) * w["apix"])


def make_data(ci, ctx, params, nparticles: int, projector):
    from cryoim_gb300 import synth
    w = WORKLOAD
    rng = np.random.default_rng(w["seed"])
    vol = synth.phantom(w["nx"], w["seed"])
    te = synth.random_asu_orientations(w["ntemplates"], rng)
    tmpl = ci.templates(w["ntemplates"])
    tmpl["particle_id"] = np.arange(1, w["ntemplates"] + 1)
    tmpl["theta"], tmpl["phi"], tmpl["omega"] = te[:, 0], te[:, 1], te[:, 2]
    timgs = projector(vol, tmpl)
    imgs, parts, truth = synth.make_particles(
        vol, nparticles, w["seed"] + 1,
        lambda v, e: projector(v, _as_tmpl(ci, e)), w["apix"], df_range=w["df"],
        astig_max=w["astig"], origin_max=w["origin"], snr=w["snr"], ampwg=w["ampwg"])
    return tmpl, timgs, imgs, parts, truth


def _as_tmpl(ci, e):
    t = ci.templates(len(e))
    t["theta"], t["phi"], t["omega"] = e[:, 0], e[:, 1], e[:, 2]
    return t


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def asu_views(step: float):
    """The (theta, phi) views of ort_globesearch.f90:68-101 (FP32 test)."""
    f = np.float32
    d2r = f(np.arctan2(f(1), f(1))) / f(45)
    c31, s31 = np.cos(f(31.717) * d2r), np.sin(f(31.717) * d2r)
    c69, s69 = np.cos(f(69.09) * d2r), np.sin(f(69.09) * d2r)
    A1, B1, C1 = -s31 * c69, -c31 * c69, s31 * s69
    A2, B2, C2 = -s31 * c69, c31 * c69, s31 * s69
    out = []
    for it in range(int(f(21.0) / f(step)) + 1):
        th = f(69.0) + f(step) * f(it)
        z, z0 = np.cos(th * d2r), np.sin(th * d2r)
        for ip in range(int(f(32.0) / f(step)) + 1):
            ph = f(step) * f(ip)
            x, y = z0 * np.cos(ph * d2r), z0 * np.sin(ph * d2r)
            if z >= 0 and z <= -(A1 * x + B1 * y) / C1 and z <= -(A2 * x + B2 * y) / C2:
                out.append((th, -ph))
                if ip > 0:
                    out.append((th, ph))
    return np.array(out, np.float32)


def cpu_sample(ci, params, tmpl, timgs, img, part, seconds: float = 15.0):
    """Time the oracle port (FP32) on all host cores over a bounded sample of views of
    one particle; return particles/s extrapolated to the full view set."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    tm, tf = pyoracle.load_templates(timgs, tmpl, params, "f32")
    views = asu_views(params.searchstep)
    nthr = pyoracle.num_threads()
    t0 = time.perf_counter()
    pyoracle.search_views(params, tm, tf, tmpl, img, part, views[:nthr], nthreads=nthr, fp="f32")
    t1 = time.perf_counter() - t0
    nv = int(min(len(views), max(nthr, nthr * max(1, int(seconds / max(t1, 1e-3))))))
    t0 = time.perf_counter()
    pyoracle.search_views(params, tm, tf, tmpl, img, part, views[:nv], nthreads=nthr, fp="f32")
    dt = time.perf_counter() - t0
    pps = (nv / len(views)) / dt
    return pps, {"cores": nthr, "kind": "port", "views": nv, "views_total": len(views), "seconds": dt,
                 "sample": f"1 particle x {nv}/{len(views)} ASU views (x {len(tmpl)} templates, "
                           f"Nomega {int(360 / params.searchstep)}), oracle FP32 port, OpenMP over views, "
                           f"extrapolated to the full grid"}


def run_reference(args):
    r, w, _ = rank_env()
    if r != 0:
        return 0
    import cryoim_gb300 as ci
    from cryoim_gb300 import synth
    params = make_params(ci)
    tmpl, timgs, imgs, parts, truth = make_data(ci, None, params, 1, lambda v, t: synth.project_numpy(
        v, np.stack([t["theta"], t["phi"], t["omega"]], 1)))
    vals = []
    info = None
    for k in range(args.warmup + args.steps):
        pps, info = cpu_sample(ci, params, tmpl, timgs, imgs[0], parts[0], seconds=args.ref_seconds)
        if k >= args.warmup:
            vals.append(pps)
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particles/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_dict(params, 1),
            "cpu_baseline": {"value": v, "unit": "particles/s", "cores": info["cores"], "kind": info["kind"],
                             "sample": info["sample"]},
            "e2e": {"value": v, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def config_dict(params, batch):
    w = WORKLOAD
    return {"workload": "icos global search, box 256 (10k-particle production config shapes)",
            "box": w["nx"], "apix": w["apix"], "band_A": [w["min_res"], w["max_res"]],
            "minR": params.min_r, "maxR": params.max_r, "searchstep_deg": w["searchstep"],
            "templates": w["ntemplates"], "particles_per_step": batch, "snr": w["snr"],
            "l2": "flushed (256 MiB write) before every timed step"}


def run_ours(args):
    import torch
    import cryoim_gb300 as ci
    r, world, lr = rank_env()
    dev = lr if torch.cuda.device_count() > 1 else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    params = make_params(ci)
    ctx = ci.Context(dev, params)
    B = args.batch
    ctx.set_batch(B)
    proj = lambda v, t: ctx.project_templates(v, t)
    tmpl, timgs, imgs, parts, truth = make_data(ci, ctx, params, B, proj)
    ctx.load_templates(timgs, tmpl)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    d_imgs = torch.from_numpy(imgs).to(f"cuda:{dev}")
    h_imgs = torch.from_numpy(imgs).pin_memory()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    terms = ctx.search_terms()
    nth, nph, nom, nviews = ctx.search_grid()

    def step(dev_ptr=True):
        q = parts.copy()
        with torch.cuda.stream(stream):
            flush.zero_()
        if dev_ptr:
            ctx.globesearch(d_imgs.data_ptr(), q)
        else:
            ctx.globesearch(h_imgs.numpy(), q)
        return q

    for _ in range(args.warmup):
        q = step()
    ctx.set_profiling(True)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            q = step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kms, klaunch = ctx.kernel_time()
    ctx.set_profiling(False)
    if world > 1:
        t = torch.tensor([ms], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * B * args.steps / (ms / 1000.0)
    # end to end: host images through the same call
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k2 = max(1, args.steps // 2)
    e2.record(stream)
    for _ in range(k2):
        q = step(dev_ptr=False)
    e3.record(stream)
    torch.cuda.synchronize()
    e2e = world * B * k2 / (e2.elapsed_time(e3) / 1000.0)
    # accuracy against the generating orientations (informational)
    from cryoim_gb300 import synth
    errs = [synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i]) for i in range(B)]
    if r != 0:
        return 0
    avg_launch_ms = kms / max(klaunch, 1)
    achieved = terms * B * FLOPS_PER_TERM / (avg_launch_ms / 1000.0) / 1e12
    line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded phantom, CTF, noise; see bench.py docstring)",
            "config": config_dict(params, B),
            "e2e": {"value": e2e, "unit": "particles/s", "h2d_bytes_per_step": int(imgs.nbytes + B * 8 * 4),
                    "d2h_bytes_per_step": int(B * 8)},
            "gpu_launches": 5 * args.steps,
            "roofline": {"bound": "fp32", "kernel": "k_pr_omega", "achieved": achieved,
                         "peak": FP32_PEAK_TFLOPS_NOMINAL, "unit": "TFLOP/s", "frac": achieved / FP32_PEAK_TFLOPS_NOMINAL,
                         "traffic": None, "terms_per_particle": terms, "flops_per_term": FLOPS_PER_TERM,
                         "terms_per_s": terms * B / (avg_launch_ms / 1000.0),
                         "avg_launch_ms": avg_launch_ms, "launches": klaunch,
                         "peak_source": "nominal FP32 FMA rate at 2.07 GHz (MEASURED_PEAKS.json has no "
                                        "non-tensor FP32 figure); the kernel is ALU/SFU-bound, not HBM or tensor"},
            "clocks": clk.summary(),
            "grid": {"ntheta": nth, "nphi": nph, "nomega": nom, "views": nviews},
            "orientation_error_deg_median": float(np.median(errs))}
    if not args.no_cpu_baseline:
        pps, info = cpu_sample(ci, params, tmpl, timgs, imgs[0], parts[0], seconds=args.ref_seconds)
        line["cpu_baseline"] = {"value": pps, "unit": "particles/s", "cores": info["cores"],
                                "kind": info["kind"], "sample": info["sample"]}
    print(json.dumps(line))
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ref-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
