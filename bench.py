#!/usr/bin/env python3
"""Global orientation search throughput at box 256: the BF16 tensor-core contraction
form against the plain FP32 (reference-parity) form.

Workload (the production-size configuration): 256x256 particles at 1.5 A/px, band
1/50 - 1/6 A^-1 (minR 7, maxR 64), 1-degree asymmetric-unit grid (664 views x 360
omega = 239,040 orientations), origins +-6 px at 0.5 px (625), 20 templates, CTF 300 kV
/ 2.7 mm / 0.07 with defocus 0.8-3.5 um and astigmatism up to 0.1 um, SNR 0.05.
Synthetic and seeded: a phantom of Gaussian blobs placed by the 60 icosahedral
rotations plus a shell (the reference map), projected at random orientations; the
reference names no public dataset.

A step is one call of cryoim_contract_search_device over a batch of 1,024 particles in
the headline form: particle transforms, CTF and origin ramps, the learned proposer's 24
best cells per particle, the BF16 contraction of their +-1-step grid neighbourhoods
(section rows read by index from the bank) with a fused argmax, the top-16 distinct
orientations and the grid neighbours of the best 4 rescored by phase residual.  The
central sections (operand B) are built once per map and the proposer is trained once per
map; each step is charged its pro-rata share of both for a 10,000-particle cycle.
`value` = particles/s with images resident in HBM; `e2e` = the same call with pinned host
images, host->device copies in the timed region.  The L2 is flushed (256 MiB write)
before every timed step.  The FP32 form (cryoim_globesearch_device, the drop-in
replacement of ort_globesearch.f90) is timed on 384 particles of the same set, the
exhaustive BF16 and FP8 contraction forms and the other proposal forms on smaller
batches (--side-batch), and every form's chosen orientations are compared with the FP32
form's on those 384 particles.

--impl reference times the reference algorithm's CPU restatement (the oracle port of
the phase-residual search, FP32 in the Fortran's operation order) on every usable host
core: each step is the complete search of one particle of the same workload (every
grid view and omega), measured, not extrapolated.  That arm loads no code of this
package.
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
                df=(0.8, 3.5), astig=0.1, snr=0.05, origin=6.0, origin_step=0.5, topk=16,
                ampwg=0.07, seed=20261205, cycle_particles=10000, learned=24, nbr_best=4, learn_lr=4e-3,
                proposal_nbr=1)
METRIC = "particles/s (box 256), BF16+learned vs plain FP32 GPU at >=99% same orientation"
FP32_PEAK_TFLOPS_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12  # FMA lanes x 2 flop x max SM clock
FLOPS_PER_TERM = 30.0
# this library's kernels launched per 64-particle pass of the headline form (ncu launch
# list, cuFFT's own kernels not counted): prep, FFT post-processing, CTF, template cuts,
# templates x CTF, particle norms, features, 4 convolutions, 3 poolings, mix, head (2
# forward real transforms, the product, 1 inverse), cell top-k, operand A, grouped
# contraction, distinct selection, and two rounds (candidates, neighbours of the best
# four) of band shift and phase residual (the line angles come from the grid's view
# table, built once per template set; the FP64 correlation is not computed for a
# phase-residual pick without candidate output)
LAUNCHES_PER_PASS = 27
# DRAM bytes (read + write) of one GEMM launch (3 particles x 625 origins) from an ncu
# capture at the 2-degree grid (1.483 GB for 31,320 orientations), scaled to the
# orientation count: operand B streams once per launch.
GEMM_TRAFFIC_PER_ORIENT = 1.483e9 / 31320
LANES = 6  # pass lanes of the contraction search (the library's default)
# the L2's peak rate of float4 reductions (one sector per cycle per slice): ncu's
# lts__t_sectors_srcunit_tex_op_red at 56.5 % of peak sustained = 2.136e11 / s in the
# k_insert capture of profiles/k_insert_box256.md
L2_RED_PEAK = 3.779e11
# sm__pipe_tensor_cycles_active of the FP8 contraction (profiles/k_gemm_argmax_e4m3_box256.md)
TENSOR_PIPE_ACTIVE_E4M3 = 0.781
# dram__bytes_read.sum + dram__bytes_write.sum of one grouped fine-contraction launch over
# a 64-particle pass of the box-256 workload (ncu capture of --profile-case learned: rows
# copied from the section bank by index, +-1-step proposal neighbourhoods)
GROUPED_GEMM_TRAFFIC_PER_PASS = 1.783445e9 + 4.284416e6
# the same for the phase-residual rescoring (mean of the two launches of a pass,
# profiles/k_pr_rescore_s_box256.md)
RESCORE_TRAFFIC_PER_LAUNCH = 0.5 * (585.458432e6 + 3.246592e6 + 769.335296e6 + 3.527936e6)
# l1tex__throughput (pct of peak, active) of the same capture: the rescoring's limiter
RESCORE_L1_ACTIVE = 0.5 * (0.806 + 0.824)



def grouped_algorithmic_bytes(g, origins, particles=64):
    """Algorithmic bytes of one grouped-contraction launch from the library's counters
    (cryoim_contract_stats): operand A of the pass (particles x origins BF16 rows) plus
    each listed bank row once, the listed rows from the counted FLOPs
    (2 x origins x rows x K per particle).  None without a launch."""
    if not g.get("gemm_launches") or not g.get("kpad"):
        return None
    rows = g["gemm_flops"] / g["gemm_launches"] / (2.0 * origins * g["kpad"])
    return (float(particles) * origins + rows) * g["kpad"] * 2.0


def rank_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def measured_peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["bf16_tflops_sustained"]), float(d["bf16_tflops"]), float(d["hbm_gbs"]), "measured"
    except Exception:
        return 1700.0, 1900.0, 6800.0, "fallback"


def make_params(ci, searchstep=None):
    w = WORKLOAD
    return ci.default_params(w["nx"], apix=w["apix"], minRes=w["min_res"], maxRes=w["max_res"],
                             searchstep=searchstep or w["searchstep"], ampwg=w["ampwg"],
                             imgmask=(w["nx"] // 2 - 2) * w["apix"])


def _as_tmpl(ci, e):
    t = ci.templates(len(e))
    t["theta"], t["phi"], t["omega"] = e[:, 0], e[:, 1], e[:, 2]
    return t


def make_data(ci, nparticles: int, projector):
    """projector(map, template_records) -> images."""
    import synth
    w = WORKLOAD
    rng = np.random.default_rng(w["seed"])
    vol = synth.phantom(w["nx"], w["seed"])
    te = synth.random_asu_orientations(w["ntemplates"], rng)
    tmpl = _as_tmpl(ci, te)
    tmpl["particle_id"] = np.arange(1, w["ntemplates"] + 1)
    timgs = projector(vol, tmpl)
    imgs, parts, truth = synth.make_particles(
        vol, nparticles, w["seed"] + 1, lambda v, e: projector(v, _as_tmpl(ci, e)), w["apix"],
        df_range=w["df"], astig_max=w["astig"], origin_max=w["origin"], snr=w["snr"], ampwg=w["ampwg"])
    return vol, tmpl, timgs, imgs, parts, truth


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms.  The sampler is started
    ahead of the timed region (nvidia-smi takes a moment to come up) and summary() keeps
    the samples that arrived between begin() and end(): the timed region itself."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, cmd=None):
        self.index, self.rows, self.proc = index, [], None
        self.cmd = cmd or ["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                           "--format=csv,noheader,nounits", "-lms", "100"]
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(self.cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append((time.perf_counter(), parts))

    def begin(self):
        self.t0 = time.perf_counter()

    def end(self):
        self.t1 = time.perf_counter()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=5)

    def summary(self):
        t0 = self.t0 if self.t0 is not None else -float("inf")
        t1 = self.t1 if self.t1 is not None else float("inf")
        rows = [r for (t, r) in self.rows if t0 <= t <= t1]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        num = lambda s: s.replace(".", "", 1).isdigit()
        sm = [float(r[0]) for r in rows if num(r[0])]
        mx = [float(r[1]) for r in rows if num(r[1])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


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


def host_cpu() -> dict:
    """Host cores this process may run on, the machine's count and the CPU model."""
    try:
        usable = len(os.sched_getaffinity(0))
    except Exception:
        usable = os.cpu_count() or 1
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            model = "unknown"
    return {"threads": usable, "nproc": os.cpu_count(), "cpu_model": model}


class CpuSearch:
    """The reference's global search (ort_globesearch.f90) restated on the CPU: the oracle
    port in FP32, the Fortran's operation order, one whole particle at a time over every
    asymmetric-unit view of the grid with OpenMP over views on `threads` host threads,
    then minloc.  Templates are prepared once (load_template.f90), outside the timing."""

    def __init__(self, pyoracle, params, tmpl, timgs, threads: int):
        self.orc, self.p, self.tmpl, self.threads = pyoracle, params, tmpl, threads
        self.tm, self.tf = pyoracle.load_templates(timgs, tmpl, params, "f32")
        self.views = asu_views(params.searchstep)

    def particle(self, img, part) -> tuple[float, float, float, float]:
        pr = self.orc.search_views(self.p, self.tm, self.tf, self.tmpl, img, part, self.views,
                                   nthreads=self.threads, fp="f32")
        k = int(np.argmin(pr))
        v, iom = divmod(k, pr.shape[1])
        return (float(self.views[v, 0]), float(self.views[v, 1]), float(self.p.searchstep * iom),
                float(pr.flat[k]))


def cpu_sample(params, tmpl, timgs, imgs, parts, particles: int = 2):
    """cpu_baseline of the GPU arm: `particles` whole particles of the same workload
    searched by the oracle port on every usable host core (about 10-20 s), and one
    particle on one thread (the reference's own single-threaded execution model)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    host = host_cpu()
    cs = CpuSearch(pyoracle, params, tmpl, timgs, host["threads"])
    n = min(particles, len(parts))
    t0 = time.perf_counter()
    for i in range(n):
        cs.particle(imgs[i], parts[i])
    dt = time.perf_counter() - t0
    cs1 = CpuSearch(pyoracle, params, tmpl, timgs, 1)
    t0 = time.perf_counter()
    cs1.particle(imgs[0], parts[0])
    dt1 = time.perf_counter() - t0
    return n / dt, {"cores": host["threads"], "kind": "port", "nproc": host["nproc"],
                    "cpu_model": host["cpu_model"], "seconds": dt, "value_1thread": 1.0 / dt1,
                    "sample": f"{n} whole particles of the workload ({len(cs.views)} ASU views x "
                              f"{int(round(360 / params.searchstep))} omega x {len(tmpl)} templates each), "
                              f"the oracle's FP32 port of ort_globesearch, OpenMP over views on "
                              f"{host['threads']} host threads; value_1thread: one particle on one thread"}


def config_dict(params):
    """The workload (identical in both arms): sizes of the box-256 global search."""
    w = WORKLOAD
    return {"workload": "icos global search, box 256, 1-deg ASU grid x 625 origins (10k-particle "
                        "production configuration shapes)",
            "box": w["nx"], "apix": w["apix"], "band_A": [w["min_res"], w["max_res"]],
            "minR": params.min_r, "maxR": params.max_r, "searchstep_deg": w["searchstep"],
            "origins": f"+-{w['origin']} px @ {w['origin_step']} px", "templates": w["ntemplates"],
            "snr": w["snr"], "defocus_um": list(w["df"]), "astigmatism_um": w["astig"]}


def form_dict(batch, learn_samples):
    w = WORKLOAD
    return {"form": f"BF16 contraction over the neighbourhoods (+-{w['proposal_nbr']} steps) of the learned proposer's "
                    f"{w['learned']} cells per particle, top-{w['topk']} rescored (FP64 CC, phase residual)",
            "particles_per_step": batch,
            "section_build": f"per map, charged pro rata per particle of a {w['cycle_particles']}-particle cycle",
            "learned_proposer": (f"trained on {learn_samples} rendered projections per map, the training time "
                                 f"charged pro rata per particle of a {w['cycle_particles']}-particle cycle"),
            "pass_lanes": LANES, "l2": "flushed (256 MiB write) before every timed step"}


def run_reference(args):
    """The reference's CPU path on this host: each step searches one whole particle of
    the box-256 workload (every grid view and omega, 20 templates) with the oracle's FP32
    port of ort_globesearch.f90 on every usable host core.  Nothing of this package is
    imported: parameters and records come from the oracle's restatement, the synthetic
    data from synth (numpy)."""
    r, w, _ = rank_env()
    if r != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    import synth
    wl = WORKLOAD
    params = pyoracle.default_params(wl["nx"], apix=wl["apix"], minRes=wl["min_res"], maxRes=wl["max_res"],
                                     searchstep=wl["searchstep"], ampwg=wl["ampwg"],
                                     imgmask=(wl["nx"] // 2 - 2) * wl["apix"])
    ops = pyoracle.icos_ops("f32")
    nsteps = args.warmup + args.steps
    rng = np.random.default_rng(wl["seed"])
    vol = synth.phantom(wl["nx"], wl["seed"], ops)
    te = synth.random_asu_orientations(wl["ntemplates"], rng)
    tmpl = np.zeros(wl["ntemplates"], pyoracle.TEMPLATE_DTYPE)
    tmpl["particle_id"] = np.arange(1, wl["ntemplates"] + 1)
    tmpl["theta"], tmpl["phi"], tmpl["omega"] = te[:, 0], te[:, 1], te[:, 2]
    timgs = synth.project_fourier(vol, te)
    imgs, parts, truth = synth.make_particles(
        vol, nsteps, wl["seed"] + 1, synth.project_fourier, wl["apix"], dtype=pyoracle.PARTICLE_DTYPE,
        df_range=wl["df"], astig_max=wl["astig"], origin_max=wl["origin"], snr=wl["snr"], ampwg=wl["ampwg"])
    host = host_cpu()
    cs = CpuSearch(pyoracle, params, tmpl, timgs, host["threads"])
    times = []
    for k in range(nsteps):
        t0 = time.perf_counter()
        cs.particle(imgs[k], parts[k])
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = 1000.0 * float(np.mean(times))
    v = 1000.0 / ms
    sample = (f"1 whole particle per step ({len(cs.views)} ASU views x {int(round(360 / params.searchstep))} "
              f"omega x {wl['ntemplates']} templates), {args.steps} timed particles, the oracle's FP32 port "
              f"of ort_globesearch, OpenMP over views on {host['threads']} host threads")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particles/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded phantom, CTF, noise)", "config": config_dict(params),
            "particles_per_step": 1, "form": "the reference's phase-residual global search (CPU)",
            "cpu_baseline": {"value": v, "unit": "particles/s", "cores": host["threads"], "kind": "port",
                             "nproc": host["nproc"], "cpu_model": host["cpu_model"], "sample": sample},
            "e2e": {"value": v, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "product_modules_loaded": sorted(m for m in sys.modules if m.startswith("cryoim_gb300"))}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import cryoim_gb300 as ci
    import synth
    r, world, lr = rank_env()
    dev = lr if torch.cuda.device_count() > 1 else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    w = WORKLOAD
    params = make_params(ci)
    ctx = ci.Context(dev, params)
    ctx.set_lanes(LANES)
    B = args.batch
    npr = args.pr_particles
    P = max(B, npr)
    vol, tmpl, timgs, imgs, parts, truth = make_data(ci, P, lambda v, t: ctx.project_templates(v, t))
    ctx.load_templates(timgs, tmpl)
    ctx.set_reference_map(vol)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    d_imgs = torch.from_numpy(imgs).to(f"cuda:{dev}")
    h_imgs = torch.from_numpy(imgs[:B]).pin_memory()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    copts = dict(origin_max=w["origin"], origin_step=w["origin_step"], topk=w["topk"], pick=0)
    lopts = dict(copts, learned=w["learned"], nbr_best=w["nbr_best"], proposal_nbr=w["proposal_nbr"])
    cyc = w["cycle_particles"]

    def timed_steps(fn, steps, sampler=None):
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if sampler is not None:
            sampler.begin()
        e0.record(stream)
        out = None
        for _ in range(steps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler is not None:
            sampler.end()
        return e0.elapsed_time(e1), out

    def search_step(dev_ptr=True, n=B, **kw):
        q = parts[:n].copy()
        with torch.cuda.stream(stream):
            flush.zero_()
        ctx.contract_search(d_imgs.data_ptr() if dev_ptr else h_imgs.numpy(), q, **kw)
        return q

    # ---- the learned proposer, trained on projections the library renders from the map ----
    torch.cuda.nvtx.range_push("training")
    lst = ctx.learn_train(vol, samples=args.learn_samples, batch=256, lr=w["learn_lr"], seed=w["seed"],
                          snr=w["snr"], df_min=w["df"][0], df_max=w["df"][1], astig_max=w["astig"],
                          origin_max=w["origin"])
    torch.cuda.nvtx.range_pop()
    train_ms = lst["seconds"] * 1000.0

    # ---- headline: BF16 contraction on the learned proposer's neighbourhoods ----
    clk = ClockSampler(dev).start()  # running before the timed region begins
    for _ in range(args.warmup):
        search_step(**lopts)
    st0 = ctx.contract_stats()  # section build time (first call) and reset
    ctx.set_profiling(True)
    torch.cuda.nvtx.range_push("headline")
    ms, _ = timed_steps(lambda: search_step(**lopts), args.steps, clk)
    torch.cuda.nvtx.range_pop()
    clk.stop()
    gst_lanes = ctx.contract_stats()
    ctx.rescore_stats()  # reset: the rescoring is timed with one lane below
    ctx.set_profiling(False)
    # The timed steps run LANES pass lanes whose kernels overlap, so a launch's event-timed
    # duration there includes other lanes' work: the contraction's roofline is taken from
    # two more steps with one lane (the kernel alone, same workload).
    ctx.set_lanes(1)
    ctx.set_profiling(True)
    for _ in range(2):
        search_step(**lopts)
    torch.cuda.synchronize()
    gst = ctx.contract_stats()
    rst = ctx.rescore_stats()
    ctx.set_profiling(False)
    ctx.set_lanes(LANES)
    # per-cycle costs charged pro rata: the section build and the proposer's training
    share = B * args.steps / cyc
    ms_eff = ms + (st0["slice_ms"] + train_ms) * share
    if world > 1:
        t = torch.tensor([ms_eff], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_eff = float(t.item())
    value = world * B * args.steps / (ms_eff / 1000.0)
    search_only = world * B * args.steps / (ms / 1000.0)
    k2 = max(1, args.steps // 2)
    e2e_ms, _ = timed_steps(lambda: search_step(dev_ptr=False, **lopts), k2)
    e2e = world * B * k2 / ((e2e_ms + (st0["slice_ms"] + train_ms) * B * k2 / cyc) / 1000.0)

    # ---- the FP32 exhaustive phase-residual form (the drop-in) on npr particles ----
    ctx.globesearch(d_imgs.data_ptr(), parts[:4].copy())
    ctx.set_profiling(True)
    q_pr = parts[:npr].copy()
    pr_ms, _ = timed_steps(lambda: ctx.globesearch(d_imgs.data_ptr(), q_pr), 1)
    kms, klaunch = ctx.kernel_time()
    ctx.set_profiling(False)
    fp32_pps = world * npr / (pr_ms / 1000.0)
    terms = ctx.search_terms()

    def agree(qa, n=npr):
        return sum(int(np.allclose((qa["theta"][i], qa["phi"][i], qa["omega"][i]),
                                   (q_pr["theta"][i], q_pr["phi"][i], q_pr["omega"][i]), atol=1e-3))
                   for i in range(n)) / n

    def on_npr(**kw):
        q = parts[:npr].copy()
        ctx.contract_search(d_imgs.data_ptr(), q, **kw)
        return q
    q_learn = on_npr(**lopts)

    # ---- the exhaustive contraction forms (every grid orientation), BF16 and FP8, on
    # steps of Bs particles ----
    Bs = min(B, args.side_batch)
    share_s = Bs * args.steps / cyc
    forms = {}
    for form in ("bf16", "fp8"):
        kw = dict(copts, precision=form)
        for _ in range(args.warmup):
            search_step(n=Bs, **kw)
        stf = ctx.contract_stats()
        ctx.set_profiling(True)
        msf, _ = timed_steps(lambda: search_step(n=Bs, **kw), args.steps)
        gf = ctx.contract_stats()
        ctx.set_profiling(False)
        vf = world * Bs * args.steps / ((msf + stf["slice_ms"] * share_s) / 1000.0)
        forms[form] = (vf, stf, gf, on_npr(**kw))

    # ---- the other proposal forms: learned with FP8 operands, coarse contraction ----
    extra = {}
    for name, kw in (("learned_fp8", dict(lopts, precision="fp8")),
                     ("coarse_bf16", dict(copts, coarse=32, nbr_best=w["nbr_best"])),
                     ("coarse_fp8", dict(copts, coarse=32, nbr_best=w["nbr_best"], precision="fp8"))):
        for _ in range(args.warmup):
            search_step(n=Bs, **kw)
        mse, _ = timed_steps(lambda: search_step(n=Bs, **kw), args.steps)
        charge = st0["slice_ms"] + (train_ms if name.startswith("learned") else 0.0)
        extra[name] = (world * Bs * args.steps / ((mse + charge * share_s) / 1000.0), on_npr(**kw))

    # ---- the other stages of a refinement cycle: local refinement and insertion ----
    def timed(fn, reps=2):
        fn()
        t_ms, _ = timed_steps(fn, reps)
        return t_ms / reps

    q_ref = q_learn[:Bs].copy()
    ref_ms = timed(lambda: ctx.refine(d_imgs.data_ptr(), q_ref.copy()))
    q_ins = q_learn[:Bs].copy()
    q_ins["pr"] = 0.0

    def insert_all():
        ctx.rec_begin()
        ctx.rec_insert(d_imgs.data_ptr(), q_ins)
    ins_ms = timed(insert_all)
    fin0 = time.perf_counter()
    ctx.rec_finish()
    fin_ms = (time.perf_counter() - fin0) * 1000.0

    # ---- localized refinement at the sub-particle configuration's shapes: 512^2 whole
    # images, 128^3 C5 local map, 12 descent cycles (local_refine's refine_PR) ----
    lrng = np.random.default_rng(w["seed"] + 7)
    lp = ci.local_params(128, 512, apix=1.0, max_res=4.0, nsym=5, ncycle=12, apply_ctf=1)
    lmap = synth.phantom(128, w["seed"] + 7)
    nloc = 64
    limgs = lrng.normal(size=(nloc, 512, 512)).astype(np.float32)
    lq = ci.local_particles(nloc)
    lq["local_hx0"], lq["local_ky0"] = lrng.integers(64, 448, (2, nloc))
    lq["local_theta0"], lq["local_phi0"], lq["local_omega0"] = lrng.uniform(0, 180, (3, nloc))
    lq["local_x0"], lq["local_y0"] = lrng.uniform(0, 1, (2, nloc))
    lq["df1"] = lq["df2"] = 15000.0
    ctx.local_refine(lp, lmap, limgs, lq.copy())
    torch.cuda.synchronize()
    l0 = time.perf_counter()
    for _ in range(2):
        ctx.local_refine(lp, lmap, limgs, lq.copy())
    loc_s = (time.perf_counter() - l0) / 2

    # ---- local form of the contraction at the sub-particle shapes: 128^2 sub-particles of
    # a 128^3 map at 1 A/px (band 1/50-1/4 A^-1), each searched over its own grid of
    # +-3 degrees at 0.25 degrees (15,625 orientations) x origins +-4 px at 0.5 px (289),
    # BF16 on the tensor cores, the top 16 rescored in FP64 ----
    lcp = ci.default_params(128, apix=1.0, minRes=50.0, maxRes=4.0, searchstep=1.0, ampwg=w["ampwg"],
                            imgmask=62.0)
    lctx = ci.Context(dev, lcp)
    # one pass lane: each grid's row-line slicer CTAs share texture-cache lines between
    # neighbouring omegas, which other lanes' grids on the same SMs would evict (measured
    # 3,295 sub-particles/s with one lane, 2,480-2,704 with six)
    lctx.set_lanes(1)
    lvol = synth.phantom(128, w["seed"] + 11)
    nlc = 128
    limg_c, lparts_c, ltruth_c = synth.make_particles(
        lvol, nlc, w["seed"] + 12, lambda v, e: lctx.project_templates(v, _as_tmpl(ci, e)), 1.0,
        df_range=w["df"], astig_max=w["astig"], origin_max=3.0, snr=w["snr"], ampwg=w["ampwg"])
    lrng2 = np.random.default_rng(w["seed"] + 13)
    lparts_c["theta"] = ltruth_c[:, 0] + lrng2.uniform(-2.5, 2.5, nlc)
    lparts_c["phi"] = ltruth_c[:, 1] + lrng2.uniform(-2.5, 2.5, nlc)
    lparts_c["omega"] = ltruth_c[:, 2] + lrng2.uniform(-2.5, 2.5, nlc)
    lctx.set_reference_map(lvol)
    lctx.set_interpolation("oversampled")
    d_limg = torch.from_numpy(limg_c).to(f"cuda:{dev}")
    lcopts = dict(origin_max=4.0, origin_step=0.5, topk=16, pick=1, local_range=3.0, local_step=0.25)
    lctx.contract_search(d_limg.data_ptr(), lparts_c[:64].copy(), **lcopts)
    torch.cuda.synchronize()
    def local_step():
        qq = lparts_c.copy()
        lctx.contract_search(d_limg.data_ptr(), qq, **lcopts)
        return qq
    lc_ms, q_lc = timed_steps(local_step, 2)
    lctx.set_lanes(1)
    lctx.set_profiling(True)
    lctx.contract_search(d_limg.data_ptr(), lparts_c[:64].copy(), **lcopts)
    lc_g = lctx.contract_stats()
    lctx.set_profiling(False)
    lc_err = [synth.orientation_error(tuple(float(q_lc[f][i]) for f in ("theta", "phi", "omega")), ltruth_c[i])
              for i in range(nlc)]
    lc_err0 = [synth.orientation_error(tuple(float(lparts_c[f][i]) for f in ("theta", "phi", "omega")), ltruth_c[i])
               for i in range(nlc)]
    lctx.close()
    del d_limg

    # ---- map agreement: FSC between reconstructions from the two forms' orientations ----
    def tnf_from(qq):
        qq = qq.copy()
        qq["pr"] = 0.0
        ctx.rec_begin_half(parts["x"][0], parts["y"][0])
        ctx.rec_insert(d_imgs.data_ptr(), qq)
        return ctx.rec_get_partial()
    fsc_forms, _ = ctx.fsc_combine(tnf_from(q_learn), tnf_from(q_pr), want_map=False)

    # ---- agreement and accuracy of the headline form ----
    same1 = 0
    e_l, e_p = [], []
    for i in range(npr):
        ol = (q_learn["theta"][i], q_learn["phi"][i], q_learn["omega"][i])
        op = (q_pr["theta"][i], q_pr["phi"][i], q_pr["omega"][i])
        same1 += int(synth.orientation_error(ol, op) <= 1.5 * w["searchstep"])
        e_l.append(synth.orientation_error(ol, truth[i]))
        e_p.append(synth.orientation_error(op, truth[i]))
    if r != 0:
        return 0
    peak_s, peak_b, hbm, src = measured_peaks()
    R = params.max_r
    s_ins = sum(1 for ky in range(-R, R + 1) for hx in range(R + 1) if hx * hx + ky * ky <= R * R)
    slice_bytes = st0["orientations"] * st0["kpad"] * 2 + (2 * R + 3) ** 3 * 8 if st0["orientations"] else 0
    ach = gst["gemm_flops"] / max(gst["gemm_ms"], 1e-9) / 1e9  # TFLOP/s of the grouped fine contraction
    # k_pr_omega: every launch of the npr-particle call summed (a launch covers a batch of
    # up to 64 particles), so the FLOPs are those of all npr particles
    pr_avg = kms / max(klaunch, 1)
    pr_terms_per_s = terms * npr / (kms / 1000.0)
    pr_achieved = pr_terms_per_s * FLOPS_PER_TERM / 1e12

    # the phase-residual rescoring (k_pr_rescore_s): one term = one (candidate, template,
    # line, radius) sample pair; a candidate carries the grid's mean terms per orientation
    # (the FP32 form's exact count over the 1-degree grid / its orientations)
    terms_per_orient = terms / max(st0["orientations"], 1)
    rs_terms_per_s = rst["candidates"] * terms_per_orient / max(rst["ms"] / 1000.0, 1e-12)
    rs_achieved = rs_terms_per_s * FLOPS_PER_TERM / 1e12
    rescore_roofline = {"bound": "fp32", "kernel": "k_pr_rescore_s", "achieved": rs_achieved,
                        "peak": FP32_PEAK_TFLOPS_NOMINAL, "unit": "TFLOP/s",
                        "frac": rs_achieved / FP32_PEAK_TFLOPS_NOMINAL, "terms_per_s": rs_terms_per_s,
                        "terms_per_candidate": terms_per_orient,
                        "avg_launch_ms": rst["ms"] / max(rst["launches"], 1), "launches": rst["launches"],
                        "candidates": rst["candidates"],
                        "timing": "CUDA events around each launch in 2 one-lane steps of the same workload",
                        "peak_source": "nominal FP32 FMA rate (no measured non-tensor FP32 peak)",
                        "traffic": RESCORE_TRAFFIC_PER_LAUNCH,
                        "traffic_note": "DRAM bytes per launch, ncu capture of --profile-case learned "
                                        "(mean of the two launches of a 64-particle pass)",
                        "limiter": {"unit": "l1tex__throughput (L1 / shared-memory data pipe)",
                                    "active_frac": RESCORE_L1_ACTIVE,
                                    "note": "ncu, profiles/k_pr_rescore_s_box256.md: the four shared-memory "
                                            "taps of each term and the template pairs from L1 keep the "
                                            "data pipe busy; the FP32 pipe is not the bound"}}

    def gemm_roofline(g, peak, kernel, src_note):
        a = g["gemm_flops"] / max(g["gemm_ms"], 1e-9) / 1e9
        return {"bound": "tensor", "kernel": kernel, "achieved": a, "peak": peak, "unit": "TFLOP/s",
                "frac": a / peak, "avg_launch_ms": g["gemm_ms"] / max(g["gemm_launches"], 1),
                "launches": g["gemm_launches"], "orientations": g["orientations"], "kpad": g["kpad"],
                "peak_source": src_note}
    contraction_roofline = dict(gemm_roofline(gst, peak_s, "k_gemm_argmax<bf16> (grouped, rows by index)",
                                f"{src} bf16_tflops_sustained"),
                                timing="CUDA events around each launch in 2 one-lane steps of the same "
                                "workload (the kernel alone)",
                                achieved_in_timed_steps=gst_lanes["gemm_flops"] / max(gst_lanes["gemm_ms"], 1e-9) / 1e9,
                                achieved_in_timed_steps_note=f"{LANES} lanes: each launch's event time includes the "
                                "overlapping kernels of the other lanes",
                                traffic=GROUPED_GEMM_TRAFFIC_PER_PASS * min(1.0, B / 64.0),
                                traffic_note="DRAM bytes of one launch (64-particle pass) from an ncu capture of "
                                "--profile-case learned with 16 learned cells, whose lists hold fewer rows "
                                "than this run's 24-cell lists (algorithmic_bytes_per_launch is this run's)",
                                algorithmic_bytes_per_launch=grouped_algorithmic_bytes(
                                    gst, (int(round(2 * w["origin"] / w["origin_step"])) + 1) ** 2),
                                note="the grouped fine contraction of the headline form; its launches are "
                                "small (each particle's 625 origins x its few hundred listed "
                                "orientations, copied from the section bank by index), and the step is "
                                "shared with the rescoring kernels (profiles/ has the launch list)")
    bf_v, bf_st, bf_g, bf_q = forms["bf16"]
    f8_v, f8_st, f8_g, f8_q = forms["fp8"]
    passes = (B + 63) // 64
    line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_eff / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic (seeded phantom, CTF, noise; see bench.py docstring)",
            "config": config_dict(params), **form_dict(B, args.learn_samples),
            "e2e": {"value": e2e, "unit": "particles/s", "h2d_bytes_per_step": int(imgs[:B].nbytes + B * 32),
                    "d2h_bytes_per_step": int(B * (w["topk"] * 16 + 8))},
            "gpu_launches": LAUNCHES_PER_PASS * passes * args.steps,
            "search_only_value": search_only,
            "charged_per_cycle_ms": {"proposer_training": train_ms, "section_build": st0["slice_ms"],
                                     "cycle_particles": cyc},
            "proposer": {"training_samples": args.learn_samples, "training_s": lst["seconds"],
                         "final_loss": lst["loss"], "views": lst["views"], "cells_per_particle": w["learned"],
                         "rescoring": f"top-{w['topk']} distinct orientations (FP64 CC), phase residual of "
                                      f"those and of the grid neighbours of the best {w['nbr_best']}"},
            # the kernel that takes most of the step's GPU time (one lane, kernels alone)
            "roofline": rescore_roofline if rst["ms"] > gst["gemm_ms"] else contraction_roofline,
            "roofline_contraction": contraction_roofline,
            "roofline_rescoring": rescore_roofline,
            "step_gpu_ms_one_lane": {"contraction": gst["gemm_ms"] / 2, "rescoring": rst["ms"] / 2},
            "section_build_ms": st0["slice_ms"],
            "fp32_form": {"value": fp32_pps, "unit": "particles/s", "particles": npr,
                          "speedup_of_headline": value / fp32_pps,
                          "roofline": {"bound": "fp32", "kernel": "k_pr_omega", "achieved": pr_achieved,
                                       "peak": FP32_PEAK_TFLOPS_NOMINAL, "unit": "TFLOP/s",
                                       "frac": pr_achieved / FP32_PEAK_TFLOPS_NOMINAL,
                                       "terms_per_particle": terms, "terms_per_s": pr_terms_per_s,
                                       "avg_launch_ms": pr_avg, "launches": klaunch,
                                       "kernel_ms_total": kms,
                                       "peak_source": "nominal FP32 FMA rate (no measured non-tensor FP32 peak)"}},
            "bf16_exhaustive_form": {"value": bf_v, "unit": "particles/s",
                                     "identical_orientation_vs_fp32_form": agree(bf_q),
                                     "section_build_ms": bf_st["slice_ms"],
                                     "roofline": dict(gemm_roofline(bf_g, peak_s, "k_gemm_argmax<bf16>",
                                                                    f"{src} bf16_tflops_sustained"),
                                                      traffic=GEMM_TRAFFIC_PER_ORIENT * bf_g["orientations"],
                                                      traffic_note="bytes per launch, ncu capture at the 2-degree "
                                                                   "grid scaled by orientations")},
            "fp8_exhaustive_form": {"value": f8_v, "unit": "particles/s",
                                    "identical_orientation_vs_fp32_form": agree(f8_q),
                                    "section_build_ms": f8_st["slice_ms"],
                                    "roofline": dict(gemm_roofline(f8_g, float("nan"), "k_gemm_argmax<e4m3>",
                                                                   "no measured FP8 peak exists: the fraction is the "
                                                                   "tensor pipe's active share from ncu"),
                                                     peak=None, frac=TENSOR_PIPE_ACTIVE_E4M3,
                                                     frac_kind="sm__pipe_tensor_cycles_active, fraction of active "
                                                               "cycles (ncu, profiles/k_gemm_argmax_e4m3_box256.md)")},
            "other_proposal_forms": {k: {"value": v[0], "unit": "particles/s",
                                         "identical_orientation_vs_fp32_form": agree(v[1])}
                                     for k, v in extra.items()},
            "refinement": {"value": Bs / (ref_ms / 1000.0), "unit": "particles/s",
                           "ncycle": int(params.ncycle), "entry": "cryoim_refine_device"},
            "reconstruction": {"insert_value": Bs / (ins_ms / 1000.0), "unit": "particles/s",
                               "samples_x_operators_per_particle": "r <= maxR half plane x 60",
                               "finish_ms": fin_ms, "entry": "cryoim_rec_insert_device / cryoim_rec_finish",
                               "roofline": {"bound": "l2_reductions", "kernel": "k_insert",
                                            "achieved": s_ins * 60 * 8 * Bs / (ins_ms / 1000.0),
                                            "peak": L2_RED_PEAK, "unit": "float4 reductions/s",
                                            "frac": s_ins * 60 * 8 * Bs / (ins_ms / 1000.0) / L2_RED_PEAK,
                                            "hbm_bytes_per_s": s_ins * 12 * Bs / (ins_ms / 1000.0),
                                            "note": "S_ins x 60 operators x 8 corners float4 reductions per "
                                                    "particle into the L2-resident accumulator; peak = the L2's "
                                                    "reduction sector rate from ncu (profiles/k_insert_box256.md); "
                                                    "the insertion call's time includes the H2D-free device path"}},
            "local_refine": {"value": nloc / loc_s, "unit": "sub-particles/s", "sub_particles": nloc,
                             "config": "512^2 whole images, 128^3 C5 local map, maxRes 4 A at 1 A/px, "
                                       "5 equivalents + 12 cycles x 11 candidates",
                             "entry": "cryoim_local_refine (host images and map: H2D, map transform and "
                                      "soft mask inside the timing)"},
            "local_contraction": {
                "value": 2 * nlc / (lc_ms / 1000.0), "unit": "sub-particles/s", "sub_particles": nlc,
                "config": "128^2 sub-particles of a 128^3 map at 1 A/px, band 1/50-1/4 A^-1, local grid "
                          "+-3 deg at 0.25 deg (15,625 orientations) x origins +-4 px at 0.5 px (289), "
                          "top 16 rescored in FP64, sections from the twice-oversampled transform, SNR %g, "
                          "starting orientations within 2.5 deg per Euler angle of the truth" % w["snr"],
                "entry": "cryoim_contract_search_device with local_range 3, local_step 0.25",
                "pass_lanes": 1,
                "median_error_vs_truth_deg": {"after": float(np.median(lc_err)), "before": float(np.median(lc_err0))},
                "roofline": dict(gemm_roofline(lc_g, peak_s, "k_gemm_argmax<bf16> (grouped, local grids)",
                                               f"{src} bf16_tflops_sustained; one-lane call, kernel alone"),
                                 orientations=15625)},
            "slicing": {"kernel": "k_slice_bf16", "ms_per_map": st0["slice_ms"],
                        "roofline": {"bound": "hbm",
                                     "achieved": slice_bytes / (st0["slice_ms"] / 1000.0) / 1e9 if slice_bytes else None,
                                     "peak": hbm, "unit": "GB/s",
                                     "frac": slice_bytes / (st0["slice_ms"] / 1000.0) / 1e9 / hbm if slice_bytes else None,
                                     "traffic_algorithmic": slice_bytes,
                                     "note": "BF16 rows written + band cube read once; the kernel is bound by "
                                             "its trilinear texture fetches (one per sample, hardware "
                                             "filtering of the cube), and runs once per map"}},
            "agreement": {"identical_orientation": agree(q_learn), "within_1_step": same1 / npr, "particles": npr,
                          "form": "headline (BF16 + learned proposals) against the FP32 form",
                          "map_fsc_min": float(fsc_forms[1:].min()),
                          "map_fsc_note": "FSC (shells 1..maxR) between the maps reconstructed from the "
                                          "headline form's and the FP32 form's orientations of the same particles",
                          "median_error_vs_truth_deg": {"headline_form": float(np.median(e_l)),
                                                        "fp32_form": float(np.median(e_p))}},
            "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        pps, info = cpu_sample(params, tmpl, timgs, imgs, parts)
        line["cpu_baseline"] = {"value": pps, "unit": "particles/s", "cores": info["cores"],
                                "kind": info["kind"], "sample": info["sample"], "nproc": info["nproc"],
                                "cpu_model": info["cpu_model"], "value_1thread": info["value_1thread"]}
    print(json.dumps(line))
    ctx.close()
    return 0


def run_profile_case(args):
    """Small cases for profiler captures (a few GB on the device, seconds of GPU time):
    learned: 64 particles of the box-256 workload, the headline form with a proposer
    trained on 2,560 projections, 2 calls; exhaustive-bf16 / exhaustive-fp8: 12
    particles at a 2-degree grid (31,320 orientations, the section bank built once), 2
    calls; fp32: 4 particles of the FP32 phase-residual form, 2 calls; insert: 64
    particles inserted into a fresh reconstruction, 2 calls; local: 16 sub-particles of
    the local contraction form (128^2 at 1 A/px, +-3 degrees at 0.25 degrees x origins
    +-4 px at 0.5 px, oversampled sections), 2 calls."""
    import torch
    import cryoim_gb300 as ci
    w = WORKLOAD
    case = args.profile_case
    if case == "local":
        import synth
        lcp = ci.default_params(128, apix=1.0, minRes=50.0, maxRes=4.0, searchstep=1.0, ampwg=w["ampwg"],
                                imgmask=62.0)
        lctx = ci.Context(0, lcp)
        lvol = synth.phantom(128, w["seed"] + 11)
        nlc = 16
        limg_c, lparts_c, ltruth_c = synth.make_particles(
            lvol, nlc, w["seed"] + 12, lambda v, e: lctx.project_templates(v, _as_tmpl(ci, e)), 1.0,
            df_range=w["df"], astig_max=w["astig"], origin_max=3.0, snr=w["snr"], ampwg=w["ampwg"])
        lrng2 = np.random.default_rng(w["seed"] + 13)
        for k, f in enumerate(("theta", "phi", "omega")):
            lparts_c[f] = ltruth_c[:, k] + lrng2.uniform(-2.5, 2.5, nlc)
        lctx.set_reference_map(lvol)
        lctx.set_interpolation("oversampled")
        d_limg = torch.from_numpy(limg_c).cuda()
        for _ in range(2):
            lctx.contract_search(d_limg.data_ptr(), lparts_c.copy(), origin_max=4.0, origin_step=0.5, topk=16,
                                 pick=1, local_range=3.0, local_step=0.25)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": case, "particles": nlc, "ok": True}))
        lctx.close()
        return 0
    step = 2.0 if case.startswith("exhaustive") else w["searchstep"]
    params = make_params(ci, searchstep=step)
    ctx = ci.Context(0, params)
    P = {"learned": 64, "exhaustive-bf16": 12, "exhaustive-fp8": 12, "fp32": 4, "insert": 64}[case]
    vol, tmpl, timgs, imgs, parts, truth = make_data(ci, P, lambda v, t: ctx.project_templates(v, t))
    ctx.load_templates(timgs, tmpl)
    ctx.set_reference_map(vol)
    d = torch.from_numpy(imgs).cuda()
    copts = dict(origin_max=w["origin"], origin_step=w["origin_step"], topk=w["topk"], pick=0)
    if case == "learned":
        ctx.learn_train(vol, samples=2560, batch=256, lr=w["learn_lr"], seed=w["seed"], snr=w["snr"],
                        df_min=w["df"][0], df_max=w["df"][1], astig_max=w["astig"], origin_max=w["origin"])
        copts.update(learned=w["learned"], nbr_best=w["nbr_best"], proposal_nbr=w["proposal_nbr"])
    elif case == "exhaustive-fp8":
        copts.update(precision="fp8")
    for _ in range(2):
        if case == "fp32":
            ctx.globesearch(d.data_ptr(), parts.copy())
        elif case == "insert":
            q = parts.copy()
            q["pr"] = 0.0
            ctx.rec_begin()
            ctx.rec_insert(d.data_ptr(), q)
        else:
            ctx.contract_search(d.data_ptr(), parts.copy(), **copts)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": case, "particles": P, "ok": True}))
    ctx.close()
    return 0


def run_precision_report(args):
    """Precision form on the CPU-runnable configuration's data: box 128, 2.0 A/px, band
    1/60-1/10 A^-1, defocus 1.0-3.0 um without astigmatism, SNR 0.1, origins within
    +-3 px; global 0.5-degree grid with origins +-6 px at 0.5 px; the contraction in BF16
    and in FP8-e4m3 (per-band scales, FP32 accumulation, FP64 rescoring of the top 16).
    Reports, per form, the contraction score error against the FP64 CC of the same
    candidates, orientation agreement with the exhaustive FP32 phase-residual search (the
    drop-in form, itself held to the FP64 oracle by the parity tests) and throughput."""
    import torch
    import cryoim_gb300 as ci
    import synth
    r, world, lr = rank_env()
    if r != 0:
        return 0
    n, P = 128, args.precision_report
    seed = 20261204
    params = ci.default_params(n, apix=2.0, minRes=60.0, maxRes=10.0, searchstep=0.5, ampwg=0.07,
                               imgmask=(n // 2 - 2) * 2.0)
    ctx = ci.Context(0, params)
    rng = np.random.default_rng(seed)
    vol = synth.phantom(n, seed)
    te = synth.random_asu_orientations(20, rng)
    tmpl = _as_tmpl(ci, te)
    tmpl["particle_id"] = np.arange(1, 21)
    timgs = ctx.project_templates(vol, tmpl)
    imgs, parts, truth = synth.make_particles(
        vol, P, seed + 1, lambda v, e: ctx.project_templates(v, _as_tmpl(ci, e)), 2.0, df_range=(1.0, 3.0),
        astig_max=0.0, origin_max=3.0, snr=0.1, ampwg=0.07)
    ctx.load_templates(timgs, tmpl)
    ctx.set_reference_map(vol)
    d_imgs = torch.from_numpy(imgs).to("cuda:0")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q_pr = parts.copy()
    ctx.globesearch(d_imgs.data_ptr(), q_pr)
    torch.cuda.synchronize()
    t_pr = time.perf_counter() - t0
    out = {"report": "precision form", "config": {"box": n, "apix": 2.0, "band_A": [60.0, 10.0],
                                                  "minR": params.min_r, "maxR": params.max_r,
                                                  "searchstep_deg": 0.5, "origins": "+-6 px @ 0.5 px",
                                                  "particles": P, "snr": 0.1, "topk_rescored": 16,
                                                  "data": "synthetic, seeded"},
           "fp32_form": {"particles_per_s": P / t_pr}}
    forms = [(f, k, b, 0) for f in ("bf16", "fp8") for k, b in ((16, 1), (16, 2), (32, 2))]
    forms += [(f, 32, 2, kc) for f in ("bf16", "fp8") for kc in (16, 32)]
    for form, topk, nbr, kc in forms:
        q = parts.copy()
        ctx.contract_search(d_imgs.data_ptr(), q[:1].copy(), origin_max=6.0, origin_step=0.5, topk=topk,
                            precision=form, nbr=nbr, coarse=kc)  # section build outside the timing
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c = ctx.contract_search(d_imgs.data_ptr(), q, origin_max=6.0, origin_step=0.5, topk=topk,
                                want_cands=True, precision=form, nbr=nbr, coarse=kc)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        err = np.abs(c[:, :, 5].astype(np.float64) - c[:, :, 6])
        rel = err / np.maximum(np.abs(c[:, :, 6]), 1e-12)
        same = np.array([np.allclose((q["theta"][i], q["phi"][i], q["omega"][i]),
                                     (q_pr["theta"][i], q_pr["phi"][i], q_pr["omega"][i]), atol=1e-3)
                         for i in range(P)])
        errs = [synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i]) for i in range(P)]
        apart = [synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]),
                                         (q_pr["theta"][i], q_pr["phi"][i], q_pr["omega"][i]))
                 for i in range(P) if not same[i]]
        out[f"{form}_form_top{topk}_nbr{nbr}" + (f"_coarse{kc}" if kc else "")] = {
            "particles_per_s": P / dt,
            "disagreement_angle_deg": {"median": float(np.median(apart)) if apart else 0.0,
                                       "max": float(np.max(apart)) if apart else 0.0},
            "exhaustive_pick_closer_to_truth": float(np.mean(
                [synth.orientation_error((q_pr["theta"][i], q_pr["phi"][i], q_pr["omega"][i]), truth[i]) <
                 synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i])
                 for i in range(P) if not same[i]])) if apart else 0.0,
            "cc_abs_error_vs_fp64": {"median": float(np.median(err)), "p99": float(np.quantile(err, 0.99)),
                                     "max": float(err.max())},
            "cc_rel_error_vs_fp64": {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99))},
            "identical_orientation_vs_fp32_form": float(same.mean()),
            "pr_gap_on_disagreement": float(np.max(np.abs(q["pr"][~same] - q_pr["pr"][~same]) /
                                                   q_pr["pr"][~same])) if (~same).any() else 0.0,
            "median_error_vs_truth_deg": float(np.median(errs))}
    out["fp32_form"]["median_error_vs_truth_deg"] = float(np.median(
        [synth.orientation_error((q_pr["theta"][i], q_pr["phi"][i], q_pr["omega"][i]), truth[i]) for i in range(P)]))
    print(json.dumps(out))
    ctx.close()
    return 0


def run_learned_report(args):
    """The learned-proposal form evaluated the way its configuration states it, on P
    particles of the CPU-runnable configuration's generator (box 128, 2.0 A/px, band
    1/60-1/10 A^-1, defocus 1.0-3.0 um, SNR 0.1, origins within +-3 px; 1-degree grid,
    origins +-4 px at 0.5 px):
      * the proposer trained on `--learn-samples` projections the library renders from
        the map (noisy and noise-free halves are not separated: every render carries
        noise at the stated SNR);
      * its cells seed the BF16 fine contraction (pick = 1: best FP64 cross-correlation);
      * each seed is refined by a local search of +-2 degrees at 0.2 degrees and +-1.5 px
        at 0.25 px around the particle's own origin (the local form with centred origins);
      * the judge is the exhaustive BF16 contraction (every grid orientation, pick = 1);
        a particle whose refined FP64 CC is below the judge's by more than 1e-3 counts as
        a fallback (the configuration's rule), and the run-time fallback rule of the
        library (phase residual more than 3 robust standard deviations above the median)
        is reported beside it, with the agreement of its picks with the exhaustive
        phase-residual search."""
    import torch
    import cryoim_gb300 as ci
    import synth
    r, world, lr = rank_env()
    if r != 0:
        return 0
    n, P = 128, args.learned_report
    seed = 20261204
    params = ci.default_params(n, apix=2.0, minRes=60.0, maxRes=10.0, searchstep=1.0, ampwg=0.07,
                               imgmask=(n // 2 - 2) * 2.0)
    ctx = ci.Context(0, params)
    rng = np.random.default_rng(seed)
    vol = synth.phantom(n, seed)
    te = synth.random_asu_orientations(20, rng)
    tmpl = _as_tmpl(ci, te)
    tmpl["particle_id"] = np.arange(1, 21)
    timgs = ctx.project_templates(vol, tmpl)
    imgs, parts, truth = synth.make_particles(
        vol, P, seed + 101, lambda v, e: ctx.project_templates(v, _as_tmpl(ci, e)), 2.0, df_range=(1.0, 3.0),
        astig_max=0.0, origin_max=3.0, snr=0.1, ampwg=0.07)
    ctx.load_templates(timgs, tmpl)
    ctx.set_reference_map(vol)
    d = torch.from_numpy(imgs).to("cuda:0")
    g = dict(origin_max=4.0, origin_step=0.5, topk=16)
    ctx.contract_search(d.data_ptr(), parts[:64].copy(), **g)  # section bank outside the timing

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    st, t_train = timed(lambda: ctx.learn_train(vol, samples=args.learn_samples, batch=256, lr=4e-3, seed=seed,
                                                snr=0.1, df_min=1.0, df_max=3.0, astig_max=0.0, origin_max=3.0))
    # judge: the exhaustive contraction, best FP64 CC
    qj = parts.copy()
    _, t_judge = timed(lambda: ctx.contract_search(d.data_ptr(), qj, pick=1, **g))
    # the learned form, best FP64 CC among its candidates, then the local search
    ql = parts.copy()
    _, t_learn = timed(lambda: ctx.contract_search(d.data_ptr(), ql, pick=1, learned=16, **g))
    # the local search on sections of the twice-oversampled transform (the local form's
    # setting), then back to plain trilinear sections for the global forms below
    ctx.set_interpolation("oversampled")
    ctx.contract_search(d.data_ptr(), ql[:64].copy(), pick=1, origin_max=1.5, origin_step=0.25, topk=16,
                        local_range=2.0, local_step=0.2, centred_origins=True)  # the cube outside the timing
    qloc = ql.copy()
    _, t_local = timed(lambda: ctx.contract_search(d.data_ptr(), qloc, pick=1, origin_max=1.5, origin_step=0.25,
                                                   topk=16, local_range=2.0, local_step=0.2, centred_origins=True))
    # the local form scores by the unbiased correlation (particle against the CTF-modulated
    # section, both norms), the global judge by its bank's: the judge's pick is rescored
    # by the local form on its own 3^3 neighbourhood (0.2 degrees, origins within 0.25 px)
    # so that the two are compared on one score
    qjl = qj.copy()
    ctx.contract_search(d.data_ptr(), qjl, pick=1, origin_max=0.25, origin_step=0.25, topk=4, local_range=0.2,
                        local_step=0.2, centred_origins=True)
    off = qloc["pr"] < qjl["pr"] - 1e-3
    ctx.set_interpolation("trilinear")
    # the phase-residual forms: exhaustive PR search on the GPU (the drop-in), the learned
    # form with and without its run-time fallback
    qpr = parts.copy()
    _, t_pr = timed(lambda: ctx.globesearch(d.data_ptr(), qpr))
    qa = parts.copy()
    _, t_a = timed(lambda: ctx.contract_search(d.data_ptr(), qa, learned=16, nbr_best=4, **g))
    # cells and neighbourhood widths of the proposal lists at this configuration
    variants = []
    for kl, pn, tk in ((16, 1, 16), (16, 2, 16), (32, 1, 16), (32, 2, 16), (64, 2, 32)):
        qv = parts.copy()
        gv = dict(g, topk=tk)
        _, tv = timed(lambda: ctx.contract_search(d.data_ptr(), qv, learned=kl, nbr_best=4, proposal_nbr=pn, **gv))
        variants.append({"learned": kl, "proposal_nbr": pn, "topk": tk, "particles_per_s": P / tv,
                         "identical_to_fp32_exhaustive": None, "_q": qv})
    qf = parts.copy()
    _, t_f = timed(lambda: ctx.contract_search(d.data_ptr(), qf, learned=16, nbr_best=4, fallback=3.0, **g))
    nfb = ctx.contract_fallbacks()

    def same(q1, q2):
        return np.all(np.abs(np.stack([q1["theta"] - q2["theta"], q1["phi"] - q2["phi"],
                                       q1["omega"] - q2["omega"]], 1)) < 1e-3, axis=1)

    def err(q):
        return float(np.median([synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i])
                                for i in range(P)]))

    def oerr(q):  # the generated origins are the records' input (x, y)
        return float(np.median(np.hypot(q["x"] - parts["x"], q["y"] - parts["y"])))
    out = {"report": "learned-proposal form", "particles": P,
           "config": {"box": n, "apix": 2.0, "band_A": [60.0, 10.0], "searchstep_deg": 1.0,
                      "origins": "+-4 px @ 0.5 px", "snr": 0.1, "data": "synthetic, seeded"},
           "proposer": {"training_samples": args.learn_samples, "training_s": t_train, "views": st["views"],
                        "final_loss": st["loss"]},
           "cc_form": {"judge": "exhaustive BF16 contraction, best FP64 CC (pick 1)",
                       "judge_particles_per_s": P / t_judge,
                       "learned_particles_per_s": P / t_learn,
                       "local_search": "+-2 deg @ 0.2 deg x +-1.5 px @ 0.25 px around each seed, centred origins, "
                                       "sections of the twice-oversampled transform",
                       "local_particles_per_s": P / t_local,
                       "learned_plus_local_particles_per_s": P / (t_learn + t_local),
                       "fallbacks_by_the_1e-3_rule": int(off.sum()), "fallback_rate": float(off.mean()),
                       "fallback_rule": "learned + local scores more than 1e-3 below the judge's pick, both by "
                                        "the local form's unbiased correlation",
                       "learned_identical_to_judge_grid_pick": float(same(ql, qj).mean()),
                       "cc_gain_of_local_search_median_vs_judge": float(np.median(qloc["pr"] - qjl["pr"])),
                       "median_error_vs_truth_deg": {"judge": err(qj), "learned": err(ql), "learned_plus_local": err(qloc)},
                       "median_origin_error_px": {"judge": oerr(qj), "learned": oerr(ql),
                                                  "learned_plus_local": oerr(qloc),
                                                  "note": "origins are not proposed: every proposed orientation is "
                                                          "correlated at every origin of the grid (289 here)"}},
           "pr_form": {"fp32_exhaustive_particles_per_s": P / t_pr,
                       "learned_particles_per_s": P / t_a,
                       "learned_identical_to_fp32_exhaustive": float(same(qa, qpr).mean()),
                       "learned_with_fallback_particles_per_s": P / t_f,
                       "runtime_fallback_rule": "PR above median + 3 x 1.4826 x MAD -> exhaustive contraction",
                       "runtime_fallbacks": nfb, "runtime_fallback_rate": nfb / P,
                       "learned_with_fallback_identical_to_fp32_exhaustive": float(same(qf, qpr).mean()),
                       "variants": variants}}
    for v in variants:
        v["identical_to_fp32_exhaustive"] = float(same(v.pop("_q"), qpr).mean())
    print(json.dumps(out))
    ctx.close()
    return 0


def run_cycle_report(args):
    """Three refinement cycles of the production configuration as one unit, each map
    feeding the next: P particles of the box-256 workload; the starting reference is the
    phantom low-pass filtered to 20 A.  Per cycle: 20 templates projected from the current
    map (load_template.f90), the proposer trained on the current map, the headline search
    (BF16 contraction over learned proposals, phase-residual rescoring; mode 4), the
    phase-residual refinement (6 cycles of the 11-point descent; mode 5), the 60-fold
    insertion and finish (mode 1) -> the next cycle's map.  Reported per cycle: wall time
    of each stage and of the cycle (synchronised), median orientation error, and the FSC
    of the new map against the phantom (shells 1..maxR)."""
    import torch
    import cryoim_gb300 as ci
    import synth
    r, world, lr = rank_env()
    if r != 0:
        return 0
    w = WORKLOAD
    P = args.cycle_report
    params = make_params(ci)
    ctx = ci.Context(0, params)
    ctx.set_lanes(LANES)
    vol = synth.phantom(w["nx"], w["seed"])
    rng = np.random.default_rng(w["seed"])
    te = synth.random_asu_orientations(w["ntemplates"], rng)
    tmpl = _as_tmpl(ci, te)
    tmpl["particle_id"] = np.arange(1, w["ntemplates"] + 1)
    imgs, parts, truth = synth.make_particles(
        vol, P, w["seed"] + 21, lambda v, e: ctx.project_templates(v, _as_tmpl(ci, e)), w["apix"],
        df_range=w["df"], astig_max=w["astig"], origin_max=w["origin"], snr=w["snr"], ampwg=w["ampwg"])
    d_imgs = torch.from_numpy(imgs).to("cuda:0")
    n, R = w["nx"], params.max_r
    h = np.arange(n) - n // 2
    kz, ky, kx = np.meshgrid(h, h, h, indexing="ij")
    kr = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    F = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(vol.astype(np.float64))))
    cut = n * w["apix"] / 20.0  # 20 A
    ref = np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(F * np.exp(-(kr / cut) ** 2 / 2)))).real.astype(np.float32)
    shell = np.rint(kr).astype(int)

    def fsc_vs_phantom(m):
        G = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(m.astype(np.float64))))
        out = []
        for sh in range(1, R + 1):
            k = shell == sh
            num = np.real(np.vdot(F[k], G[k]))
            out.append(num / np.sqrt(np.vdot(F[k], F[k]).real * np.vdot(G[k], G[k]).real))
        return np.array(out)

    def sync_time(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    q = parts.copy()
    cycles = []
    m = ref
    for cyc in range(3):
        st = {}
        timgs, st["templates_s"] = sync_time(lambda: ctx.project_templates(m, tmpl))
        _, st["load_templates_s"] = sync_time(lambda: ctx.load_templates(timgs, tmpl))
        _, st["reference_map_s"] = sync_time(lambda: ctx.set_reference_map(m))
        _, st["proposer_training_s"] = sync_time(lambda: ctx.learn_train(
            m, samples=args.learn_samples, batch=256, lr=w["learn_lr"], seed=w["seed"] + cyc, snr=w["snr"],
            df_min=w["df"][0], df_max=w["df"][1], astig_max=w["astig"], origin_max=w["origin"]))
        _, st["search_s"] = sync_time(lambda: ctx.contract_search(
            d_imgs.data_ptr(), q, origin_max=w["origin"], origin_step=w["origin_step"], topk=w["topk"],
            learned=w["learned"], nbr_best=w["nbr_best"], proposal_nbr=w["proposal_nbr"]))
        _, st["refine_s"] = sync_time(lambda: ctx.refine(d_imgs.data_ptr(), q))

        def insert():
            qq = q.copy()
            qq["pr"] = 0.0
            ctx.rec_begin()
            ctx.rec_insert(d_imgs.data_ptr(), qq)
            return ctx.rec_finish()
        m, st["insert_finish_s"] = sync_time(insert)
        st["cycle_s"] = sum(v for k, v in st.items() if k.endswith("_s"))
        err = [synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i]) for i in range(P)]
        f = fsc_vs_phantom(m)
        st["median_error_vs_truth_deg"] = float(np.median(err))
        st["fsc_vs_phantom"] = {"shell_16": float(f[15]), "shell_32": float(f[31]), "shell_48": float(f[47]),
                                "shell_64": float(f[R - 1]),
                                "first_below_0.5": int(np.argmax(f < 0.5) + 1) if (f < 0.5).any() else None}
        st["particles_per_s"] = P / st["cycle_s"]
        cycles.append(st)
    print(json.dumps({"report": "three refinement cycles (search, refine, insert), each map the next reference",
                      "particles": P, "config": config_dict(params),
                      "start": "phantom low-pass filtered (Gaussian, 20 A)", "cycles": cycles}))
    ctx.close()
    return 0


def _rot_angle(Ra, Rb):
    c = np.clip((np.trace(Ra.T @ Rb) - 1) / 2, -1, 1)
    return float(np.degrees(np.arccos(c)))


def run_local_report(args):
    """Batched localized refinement from whole particles, the sub-particle configuration's
    pipeline: P particles of 512^2 at 1.0 A/px projected from a 512^3 phantom (the
    generator's radii x4) in the icosprocess 2-fold frame, CTF 1.0-3.0 um, noise-free and at
    SNR 0.1 (the same particles); orientations taken to the 5-fold frame (proc_icos
    transform, Ry(v) R); the 12 vertex sub-particles of 128^2 per particle cut by
    local_box's stack mode on the GPU (cryoim_local_box_extract: one rotation of the 5-fold
    frame's icosahedral set per vertex, vertex at (0, 0, 184 px)); the 128^3 C5 local map
    cut from the phantom around that vertex; then the contraction search's local form (BF16
    on the tensor cores, +-3 degrees at 0.25 degrees x origins +-4 px at 0.5 px around each
    sub-particle's own origin, top 16 rescored in FP64).  Starting orientations are the
    truth perturbed by up to 1 degree per Euler angle; errors are measured modulo the
    local map's C5.

    Signal subtraction, as localized reconstruction does before it cuts a sub-particle:
    the image a vertex's sub-particle is cut from keeps that vertex's region (a sphere of
    radius 56 px) and the particle's noise, the projections of the rest of the particle
    subtracted.  Without it (all 12 vertex regions kept in one image) other vertices that
    project into the sub-particle's box, and the CTF's delocalisation of their signal, move
    the correlation's maximum away from the truth; that case is reported beside it."""
    import torch
    import cryoim_gb300 as ci
    import synth
    from scipy.ndimage import map_coordinates
    r, world, lr = rank_env()
    if r != 0:
        return 0
    P, n0, n, zv, rmask = args.local_report, 512, 128, 184.0, 56.0
    seed = 20261208
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    vol = synth.phantom(n0, seed)
    t_phantom = time.perf_counter() - t0
    # the 5-fold frame: E5 = Ry(v) E, the map M5(X) = M2(Ry(v)^T X)
    v = np.arccos(np.cos(np.radians(60.0)) / np.sin(np.radians(36.0)))
    Ry = np.array([[np.cos(v), 0, np.sin(v)], [0, 1, 0], [-np.sin(v), 0, np.cos(v)]])
    # 12 vertices: the first rotation of the 5-fold frame's icosahedral set for each
    # distinct image S^T z of the 5-fold axis
    s60 = ci.local_sym_matrices("i5").astype(np.float64)
    sym, seen = [], []
    for S in s60:
        u = S.T @ np.array([0.0, 0.0, 1.0])
        if all(np.linalg.norm(u - w) > 1e-3 for w in seen):
            seen.append(u)
            sym.append(S)
    sym = np.array(sym, np.float32)
    assert len(sym) == 12
    # the vertex regions: spheres of radius rmask around the vertices, in the map's 2-fold
    # frame Ry^T S^T (0, 0, zv)
    g0 = np.arange(n0, dtype=np.float32) - n0 // 2

    def region(S):
        cv = Ry.T @ (S.astype(np.float64).T @ np.array([0.0, 0.0, zv]))
        lo = np.maximum(np.floor(cv - rmask).astype(int) + n0 // 2, 0)
        hi = np.minimum(np.ceil(cv + rmask).astype(int) + n0 // 2 + 1, n0)
        zs, ys, xs = g0[lo[2]:hi[2]], g0[lo[1]:hi[1]], g0[lo[0]:hi[0]]
        d2 = ((zs[:, None, None] - cv[2]) ** 2 + (ys[None, :, None] - cv[1]) ** 2 + (xs[None, None, :] - cv[0]) ** 2)
        return (slice(lo[2], hi[2]), slice(lo[1], hi[1]), slice(lo[0], hi[0])), d2 <= rmask * rmask

    regions = [region(S) for S in sym]
    keep = np.zeros((n0, n0, n0), bool)
    for sl, m in regions:
        keep[sl] |= m
    vol12 = np.where(keep, vol, np.float32(0.0))
    del keep
    p0 = ci.default_params(n0, apix=1.0, minRes=50.0, maxRes=4.0, searchstep=1.0, ampwg=0.07)
    c0 = ci.Context(0, p0)

    def particles(V, snr):  # the same orientations, CTF, origins and noise draws for every V
        return synth.make_particles(V, P, seed + 1, lambda v_, e: c0.project_templates(v_, _as_tmpl(ci, e)), 1.0,
                                    df_range=(1.0, 3.0), astig_max=0.0, origin_max=2.0, snr=snr, ampwg=0.07)

    full0, parts, truth = particles(vol12, 0.0)
    full1 = particles(vol12, 0.1)[0]
    noise = full1 - full0
    # per vertex: that vertex's signal alone (+ the particle's noise)
    vert0 = []
    for sl, m in regions:
        vk = np.zeros_like(vol)
        vk[sl] = np.where(m, vol[sl], np.float32(0.0))
        vert0.append(particles(vk, 0.0)[0])
        del vk
    c0.close()
    t5, p5, o5 = ci.transform_ort(5, truth[:, 0], truth[:, 1], truth[:, 2])
    # the local map: 128^3 around (0, 0, zv) in the 5-fold frame, C5 about z
    g = np.arange(n) - n // 2
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    X = np.stack([xx.ravel(), yy.ravel(), zz.ravel() + zv]).astype(np.float64)
    Xm = Ry.T @ X + n0 // 2
    lmap = map_coordinates(vol, [Xm[2], Xm[1], Xm[0]], order=1, mode="constant").reshape(n, n, n)
    # the local map holds the vertex region the sub-particles keep (a map reconstructed
    # from the subtracted sub-particles holds no more)
    lmap = np.where(zz ** 2 + yy ** 2 + xx ** 2 <= rmask * rmask, lmap, 0.0).astype(np.float32)
    # starting orientations in the 5-fold frame, up to 1 degree off per Euler angle
    q = parts.copy()
    q["theta"] = t5 + rng.uniform(-1, 1, P)
    q["phi"] = p5 + rng.uniform(-1, 1, P)
    q["omega"] = o5 + rng.uniform(-1, 1, P)
    q["pr"] = 10.0
    lp = ci.default_params(n, apix=1.0, minRes=50.0, maxRes=4.0, searchstep=1.0, ampwg=0.07,
                           imgmask=(n // 2 - 2) * 1.0)
    lctx = ci.Context(0, lp)
    lctx.set_lanes(LANES)
    lctx.set_reference_map(lmap)
    lctx.set_interpolation("oversampled")
    # the noisy set also searched at a band to 8 A (the resolution such data support)
    lp8 = ci.default_params(n, apix=1.0, minRes=50.0, maxRes=8.0, searchstep=1.0, ampwg=0.07,
                            imgmask=(n // 2 - 2) * 1.0)
    lctx8 = ci.Context(0, lp8)
    lctx8.set_lanes(LANES)
    lctx8.set_reference_map(lmap)
    lctx8.set_interpolation("oversampled")
    c5 = [np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
          for a in np.radians(72.0 * np.arange(5))]

    def err(th, ph, om, i, k):  # against the sub-particle's true orientation S E5, modulo C5
        Rt = sym[k].astype(np.float64) @ synth.euler_mat(t5[i], p5[i], o5[i])
        R = synth.euler_mat(th, ph, om)
        return min(_rot_angle(R, Z @ Rt) for Z in c5)

    kw = dict(origin_max=4.0, origin_step=0.5, topk=16, pick=1, local_range=3.0, local_step=0.25,
              centred_origins=True)
    d_sub = torch.empty((P * 12, n, n), device="cuda:0")

    def run(images_of_vertex, sctx=None):
        """Extraction (one call per vertex image set, or one call for all 12 vertices) and
        the local search of every sub-particle (by sctx, else lctx); records in the order
        (vertex, particle)."""
        sctx = sctx or lctx
        recs, t_extract = [], 0.0
        for k, imgs in images_of_vertex:
            d_imgs = torch.from_numpy(imgs).to("cuda:0")
            syms = sym if k is None else sym[k:k + 1]
            off = sum(len(r_) for r_ in recs)
            torch.cuda.synchronize()
            te = time.perf_counter()
            _, rec = lctx.local_box_extract(d_imgs.data_ptr(), q, syms, (0.0, 0.0, zv), 1.0, n,
                                            d_out=d_sub.data_ptr() + off * n * n * 4, fftsize=n0)
            torch.cuda.synchronize()
            t_extract += time.perf_counter() - te
            recs.append(rec)
            del d_imgs
        rec = np.concatenate(recs)
        K = len(rec)
        assert K == 12 * P, K  # every particle selected, every vertex inside its image
        sp = ci.particles(K)
        sp["particle_id"] = np.arange(1, K + 1)
        sp["img_id"] = np.arange(1, K + 1)
        sp["img_particle_id"] = np.arange(1, K + 1)
        sp["theta"], sp["phi"], sp["omega"] = rec["local_theta0"], rec["local_phi0"], rec["local_omega0"]
        sp["x"], sp["y"] = rec["local_x0"], rec["local_y0"]
        sp["df1"], sp["df2"], sp["astigang"] = rec["df1"], rec["df2"], rec["astigang"]
        sctx.contract_search(d_sub.data_ptr(), sp[:64].copy(), **kw)  # warm-up (sample lists, texture)
        torch.cuda.synchronize()
        ts = time.perf_counter()
        out = sp.copy()
        sctx.contract_search(d_sub.data_ptr(), out, **kw)
        torch.cuda.synchronize()
        t_search = time.perf_counter() - ts
        # (particle, vertex) of each record: per-vertex calls give P records per vertex;
        # the all-vertex call gives 12 per particle
        if len(images_of_vertex) == 1:
            pi, kk = np.arange(K) // 12, np.arange(K) % 12
        else:
            pi, kk = np.tile(np.arange(P), 12), np.repeat(np.arange(12), P)
        before = np.array([err(sp["theta"][j], sp["phi"][j], sp["omega"][j], pi[j], kk[j]) for j in range(K)])
        after = np.array([err(out["theta"][j], out["phi"][j], out["omega"][j], pi[j], kk[j]) for j in range(K)])
        return {"extraction": {"entry": "cryoim_local_box_extract_device", "seconds": t_extract,
                               "sub_particles_per_s": K / t_extract},
                "local_search": {"entry": "cryoim_contract_search_device (local form, centred origins)",
                                 "seconds": t_search, "sub_particles_per_s": K / t_search},
                "pipeline_sub_particles_per_s": K / (t_extract + t_search),
                "median_error_deg_c5": {"before": float(np.median(before)), "after": float(np.median(after))},
                "fraction_improved": float(np.mean(after < before)),
                "fraction_within_0.5_deg_after": float(np.mean(after < 0.5))}

    per_snr = {}
    for name, nz in (("noise-free", None), ("snr 0.1", noise)):
        sub = [(k, vert0[k] + (nz if nz is not None else 0.0)) for k in range(12)]
        kept = [(None, full0 + (nz if nz is not None else 0.0))]
        per_snr[name] = {"per-vertex subtraction": run(sub), "12 vertices kept": run(kept)}
        if nz is not None:
            per_snr[name]["per-vertex subtraction, band to 8 A"] = run(sub, lctx8)
    res = {"report": "batched localized refinement from whole particles", "particles": P, "sub_particles": P * 12,
           "config": {"particle_box": n0, "apix": 1.0, "sub_box": n, "vertex_z_px": zv, "vertices": 12,
                      "signal": (f"per sub-particle: its vertex region (sphere of radius {rmask:g} px) and the "
                                 "particle's noise, the rest of the particle subtracted; beside it all 12 vertex "
                                 "regions kept in one image"),
                      "local_map": "128^3 around the vertex, 5-fold frame (C5 about z), the vertex region "
                                   f"(radius {rmask:g} px) only",
                      "search": "+-3 deg @ 0.25 deg (15,625 orientations) x origins +-4 px @ 0.5 px (289), "
                                "centred on each sub-particle's own origin, top 16 rescored in FP64; sections "
                                "from the twice-oversampled transform; score sum Re(P conj(CTF S)) / "
                                "(|P| |CTF S|)",
                      "ctf": "defocus U(1.0, 3.0) um", "start": "truth + U(+-1 deg) per Euler angle"},
           "phantom_s": t_phantom, "results": per_snr}
    print(json.dumps(res))
    lctx.close()
    lctx8.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=1024, help="particles per headline step")
    ap.add_argument("--side-batch", type=int, default=64, help="particles per step of the other forms")
    ap.add_argument("--pr-particles", type=int, default=384,
                    help="particles of the agreement check against the FP32 form")
    ap.add_argument("--learn-samples", type=int, default=16384,
                    help="projections the learned proposer is trained on")
    ap.add_argument("--searchstep", type=float, default=None,
                    help="override the 1-degree grid (small cases for profiler captures only)")
    ap.add_argument("--origin-step", type=float, default=None,
                    help="override the 0.5 px origin step (small cases for profiler captures only)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", choices=["learned", "exhaustive-bf16", "exhaustive-fp8", "fp32", "insert", "local"],
                    default=None, help="instead of the bench line: a small case for profiler captures")
    ap.add_argument("--precision-report", type=int, default=0, metavar="P",
                    help="instead of the bench line: BF16 and FP8 contraction against FP64 scores and the "
                         "exhaustive FP32 search on P particles of the box-128 configuration (0.5-degree grid)")
    ap.add_argument("--cycle-report", type=int, default=0, metavar="P",
                    help="instead of the bench line: three refinement cycles (search, refine, insert) of P box-256 "
                         "particles, each map the next cycle's reference")
    ap.add_argument("--local-report", type=int, default=0, metavar="P",
                    help="instead of the bench line: 12 vertex sub-particles of P whole 512^2 particles cut on the "
                         "GPU and refined by the local contraction form against a 128^3 C5 local map")
    ap.add_argument("--learned-report", type=int, default=0, metavar="P",
                    help="instead of the bench line: the learned-proposal form with local search, judged by the "
                         "exhaustive contraction on P particles of the box-128 configuration")
    args = ap.parse_args()
    if args.cycle_report:
        return run_cycle_report(args)
    if args.local_report:
        return run_local_report(args)
    if args.learned_report:
        return run_learned_report(args)
    if args.precision_report:
        return run_precision_report(args)
    if args.profile_case:
        return run_profile_case(args)
    if args.searchstep:
        WORKLOAD["searchstep"] = args.searchstep
    if args.origin_step:
        WORKLOAD["origin_step"] = args.origin_step
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
