"""Benchmark: gradient shots/s of the batched native path on the C2 workload.

One step = one gradient evaluation of the whole batch (32 shots of the
601 x 301, nt = 3000 C2 workload): forward with image storage, residual and
FP64 misfit, adjoint + imaging, on-device shot reduction.  Inputs (observed
data) and outputs (gradients) are resident in HBM for `value`; `e2e` passes
pinned host buffers through the public C-ABI (fwi_gradient), so the
host-to-device copy of the observed data and the device-to-host copy of the
gradients and misfit are inside its timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

Multi-GPU (torchrun): every rank runs its own C2 batch on its own GPU (weak
scaling, no collective on the data path); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "gradient shots/s & Gpt-updates/s, batched+ckpt vs plain GPU, grad rel-err≤1e-4"
ALG_BYTES_FWD = 36   # B per point update: P,F now and previous, P,F next, three models
ALG_BYTES_ADJ = 68   # adjoint 36 + forward image 8 + three gradient read-modify-writes 24


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_workload(args):
    """The named seeded workload; --shots and --nt replace its shot count and step count
    where it has them (C4 draws each shot's steps; its --shots takes the first shots of the set)."""
    from fwi_gb300 import synth
    kw = {}
    if args.shots is not None and args.workload != "C1":
        kw["shots"] = args.shots
    if args.nt is not None and args.workload in ("C2", "C3", "C5"):
        kw["nt"] = args.nt
    return synth.WORKLOADS[args.workload](**kw)


def traffic_from_profile(name):
    path = os.path.join(ROOT, "profiles", name)
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    def __init__(self):
        self.p = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self, gpu_index=0):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9 or f[0] != str(gpu_index):
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        load = [s for s in sm if mx and s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    n = int(os.environ.get("WORLD_SIZE", "1"))
    if n <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, n, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------- CPU (oracle) timing

def cpu_sample(w, seconds=15.0, threads=None):
    """Time the oracle's reference-arithmetic gradient (src/main.c:408-495 sequence) of one
    shot over a bounded number of steps; returns (shots/s extrapolated, threads, sample)."""
    from oracle import pyoracle as po
    po.build()
    threads = threads or os.cpu_count() or 1
    po.set_threads(threads)
    vh, vp, vn = w.squared(initial=True)
    s = w.shots[0]
    probe_nt = 40
    ax, bx, az, bz = po.cpml_profiles(w.nx, w.nz, w.cpml, w.dh, w.dt, w.f)
    def run(nt):
        p = dict(nx=w.nx, nz=w.nz, nt=nt, cpml=w.cpml, dh=w.dh, dt=w.dt, ax=ax, bx=bx, az=az, bz=bz,
                 source=po.ricker(nt, w.dt, w.f), vh=vh, vp=vp, vn=vn)
        obs = np.zeros((nt, w.nx), np.float32)
        t0 = time.perf_counter()
        po.gradient_shot(p, s["sx"] + 1, s["sz"] + 1, obs)
        return time.perf_counter() - t0
    t_probe = run(probe_nt)
    nt = int(max(probe_nt, min(s["nt"], probe_nt * seconds / max(t_probe, 1e-3))))
    t = run(nt)
    per_step = t / nt
    shots_per_s = 1.0 / (per_step * s["nt"])
    return shots_per_s, threads, (f"one {w.nx}x{w.nz} shot, {nt} forward + {nt} adjoint steps of "
                                  f"{s['nt']}, extrapolated to the full shot; {t:.1f} s")


# ----------------------------------------------------------------- GPU timing

def image_bytes(store):
    """Adjoint algorithmic bytes per point: 68 with FP32 images, 64 with 16-bit images
    (the forward state the imaging reads is one FP16 / BF16 image pair, 4 B, not 8)."""
    return ALG_BYTES_ADJ - (4 if store in ("fp16", "bf16") else 0)


def config_of(args, w):
    """The workload's `config` object, the same in both arms."""
    nrec = max(s["rx1"] - s["rx0"] for s in w.shots)
    ntr = sum(s["nt"] * (s["rx1"] - s["rx0"]) for s in w.shots)
    return {"workload": w.name, "nx": w.nx, "nz": w.nz, "dh": w.dh, "dt": w.dt, "nt": w.nt,
            "shots": len(w.shots), "receivers_per_shot": nrec, "ricker_hz": w.f, "cpml": w.cpml,
            "mode": args.mode, "image_store": f"{args.storage}, {args.store}", "batch": args.batch,
            **({"ckpt_every": args.ckpt_every} if args.ckpt_every > 0 else {}),
            "l2": f"inputs larger than L2 (observed data {ntr * 4 / 1e6:.0f} MB; the per-step state of "
                  f"all shots {6 * 4 * w.nz * w.nx * len(w.shots) / 1e6:.0f} MB; images or rings streamed "
                  f"through HBM)"}


def native_arm(args, rank, world, dist):
    import torch

    import fwi_gb300

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    w = make_workload(args)
    shots = fwi_gb300.make_shots(w.shots)
    mode = fwi_gb300.MODE_EXACT if args.mode == "exact" else fwi_gb300.MODE_REF_COMPAT
    sprec = {"fp32": fwi_gb300.SPREC_NATIVE, "fp16": fwi_gb300.SPREC_FP16, "bf16": fwi_gb300.SPREC_BF16}[args.store]
    nrec = max(s["rx1"] - s["rx0"] for s in w.shots)
    store_of = {"full": fwi_gb300.STORE_FULL, "checkpoint": fwi_gb300.STORE_CHECKPOINT,
                "boundary": fwi_gb300.STORE_BOUNDARY}

    # widest shot aperture (per-shot windows): per-shot arrays are sized by it, not by the model
    max_window = max((s["nxw"] or w.nx) for s in w.shots)

    def context(max_shots, precision=fwi_gb300.PREC_FP32, store_prec=sprec, store=args.storage):
        c = fwi_gb300.Context(nx=w.nx, nz=w.nz, dh=w.dh, dt=w.dt, cpml=w.cpml, f_cpml=w.f, nt_max=w.nt,
                              max_shots=max_shots, max_receivers=nrec, max_window=max_window, mode=mode,
                              precision=precision, store_prec=store_prec, store=store_of[store],
                              ckpt_every=args.ckpt_every, device=dev)
        c.set_ricker(w.f, w.nt)
        return c

    # observed data from the true model (FP32, on the GPU); the runs then start from the initial model
    ntr = sum(s["nt"] * (s["rx1"] - s["rx0"]) for s in w.shots)
    obs_d = torch.zeros(ntr, dtype=torch.float32, device="cuda")
    c0 = context(min(args.batch, len(w.shots)))
    c0.set_model(*w.squared())
    c0.forward(shots, out=obs_d)
    del c0
    hbm, peak_kind = peaks()
    nshots = len(w.shots)
    upd = w.physical_point_updates()
    pts = sum(((s["nxw"] or w.nx) - 8) * (w.nz - 8) * s["nt"] for s in w.shots)  # updated points per phase
    adj_bytes = image_bytes(args.store)

    def measure(storage, clocks_too):
        """Gradient shots/s of the whole batch with `storage`: device-resident `value`, then e2e through
        fwi_gradient with pinned host buffers."""
        ctx = context(min(args.batch, len(w.shots)), store=storage)
        # device memory of the context by fwi_config_bytes (the storage mode's figure)
        device_gb = round(fwi_gb300.native.lib().fwi_config_bytes(ctypes.byref(ctx.cfg)) / 1e9, 2)
        ctx.set_model(*w.squared(initial=True))
        g_d = [torch.zeros((w.nz, w.nx), dtype=torch.float32, device="cuda") for _ in range(3)]
        # launch choice: measured by the autotuner (before the warm-up, untimed) or the built-in one
        tuning = ctx.autotune(shots, steps=args.autotune) if args.autotune > 0 else None

        def step():
            J, *_ = ctx.gradient(shots, obs_d, w.mask, out=g_d)
            return J

        ctx.set_tile_timing(True)  # events around the interior tile launches of sampled steps
        for _ in range(args.warmup):
            step()
        clocks = Clocks() if clocks_too else None
        barrier(dist)
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches = 0
        t_fwd = t_adj = t_tot = 0.0
        tile = np.zeros(4)
        rec = np.zeros(3)
        e0.record()
        for _ in range(args.steps):
            J = step()
            t = ctx.last_timing()
            t_tot += float(t[0])
            t_fwd += float(t[1])
            t_adj += float(t[2])
            tile += ctx.last_tile_timing() / args.steps
            rec += ctx.last_recompute_timing() / args.steps
            launches += ctx.last_launches()
        e1.record()
        torch.cuda.synchronize()
        barrier(dist)
        clk = clocks.stop(dev) if clocks else None
        ms = max_over_ranks(dist, e0.elapsed_time(e1) / args.steps)

        # end to end: pinned host observed data in, host gradients and misfit out
        obs_h = obs_d.cpu().pin_memory()
        g_h = [torch.zeros((w.nz, w.nx), dtype=torch.float32).pin_memory() for _ in range(3)]
        for _ in range(2):
            ctx.gradient(shots, obs_h, w.mask, out=g_h)
        barrier(dist)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.gradient(shots, obs_h, w.mask, out=g_h)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks(dist, (time.perf_counter() - t0) * 1e3 / args.steps)
        barrier(dist)
        del ctx
        # dominant kernel: of the two interior tile passes, the one with the larger live total (mean
        # sampled launch duration x launches): the adjoint's with full storage; the forward's with
        # checkpoint storage, where it runs twice (the forward, and each segment's recompute beside the
        # adjoint).  Per launch: algorithmic bytes of the interior points it updates / its mean duration,
        # from CUDA events on its stream around sampled launches
        adj_ms, adj_pts = float(tile[2]), float(tile[3])
        fwd_ms, fwd_pts = float(tile[0]), float(tile[1])
        rec_ms, rec_pts, rec_steps = float(rec[0]), float(rec[1]), float(rec[2])
        batches = [w.shots[i:i + args.batch] for i in range(0, nshots, args.batch)]
        steps_fwd = sum(max(s["nt"] for s in bt) for bt in batches)  # interior launches of a phase
        fwd_launches = steps_fwd + rec_steps
        fwd_mean = (fwd_ms * steps_fwd + rec_ms * rec_steps) / fwd_launches if fwd_launches else 0.0
        kern_gbs = adj_bytes * adj_pts / (adj_ms / 1e3) / 1e9 if adj_ms > 0 else None
        fwd_kern_gbs = ALG_BYTES_FWD * fwd_pts / (fwd_mean / 1e3) / 1e9 if fwd_mean > 0 else None
        fwd_dominant = fwd_mean * fwd_launches > adj_ms * steps_fwd
        img_write = adj_bytes - (ALG_BYTES_ADJ - 8)  # the two images of a point: 4 B in FP16, 8 B in FP32
        rec_bytes = (ALG_BYTES_FWD + img_write) * rec_pts * rec_steps
        r = {
            "value": round(world * nshots / (ms / 1e3), 4), "ms_per_step": round(ms, 3), "misfit": J,
            "device_gb": device_gb,
            "gpt_updates_per_s": round(world * upd / (ms / 1e3) / 1e9, 3),
            "e2e": {"value": round(world * nshots / (ms_e2e / 1e3), 4), "unit": "shots/s",
                    "h2d_bytes_per_step": int(ntr * 4), "d2h_bytes_per_step": int(3 * w.nx * w.nz * 4 + 8)},
            "roofline": ({"bound": "hbm", "kernel": "k_fwd_tma interior tiles (forward step; with checkpoint "
                                                              "storage also each segment's recompute)",
                          "achieved": round(fwd_kern_gbs, 1) if fwd_kern_gbs else None, "peak": hbm, "unit": "GB/s",
                          "frac": round(fwd_kern_gbs / hbm, 4) if fwd_kern_gbs else None, "peak_kind": peak_kind,
                          "traffic": traffic_from_profile(f"k_fwd_tma_interior_{args.workload}.txt"),
                          "launch_ms": round(fwd_mean, 4), "points_per_launch": int(fwd_pts),
                          "bytes_per_point": ALG_BYTES_FWD,
                          "launches_per_gradient": int(fwd_launches),
                          "forward_pass_launch_ms": round(fwd_ms, 4), "recompute_launch_ms": round(rec_ms, 4),
                          "adjoint_interior": {"achieved": round(kern_gbs, 1) if kern_gbs else None,
                                               "frac": round(kern_gbs / hbm, 4) if kern_gbs else None,
                                               "launch_ms": round(adj_ms, 4), "points_per_launch": int(adj_pts),
                                               "bytes_per_point": adj_bytes}}
                         if fwd_dominant else
                         {"bound": "hbm", "kernel": "k_adj_tma interior tiles (adjoint step + imaging)",
                          "achieved": round(kern_gbs, 1) if kern_gbs else None, "peak": hbm, "unit": "GB/s",
                          "frac": round(kern_gbs / hbm, 4) if kern_gbs else None, "peak_kind": peak_kind,
                          "traffic": traffic_from_profile(f"k_adj_tma_interior_{args.workload}.txt"),
                          "launch_ms": round(adj_ms, 4), "points_per_launch": int(adj_pts),
                          "bytes_per_point": adj_bytes, "launches_per_gradient": int(steps_fwd),
                          "forward_interior": {"achieved": round(fwd_kern_gbs, 1) if fwd_kern_gbs else None,
                                               "frac": round(fwd_kern_gbs / hbm, 4) if fwd_kern_gbs else None,
                                               "launch_ms": round(fwd_mean, 4), "points_per_launch": int(fwd_pts),
                                               "bytes_per_point": ALG_BYTES_FWD}}) | {
                         # whole phases (all kernels of a step, every updated point), on the context stream;
                         # the adjoint phase with checkpoint storage also carries the segment recompute
                         "adjoint_step_frac": round(adj_bytes * pts / (t_adj / args.steps / 1e3) / 1e9 / hbm, 4),
                         "adjoint_phase_frac_with_recompute": round((adj_bytes * pts + rec_bytes)
                                                                    / (t_adj / args.steps / 1e3) / 1e9 / hbm, 4),
                         "forward_step_frac": round(ALG_BYTES_FWD * pts / (t_fwd / args.steps / 1e3) / 1e9 / hbm, 4),
                         # the point-update basis: useful updates x 52 B (36 forward + 68 adjoint, two updates)
                         "gradient_frac": round(world * upd / (ms / 1e3) * (ALG_BYTES_FWD + ALG_BYTES_ADJ) / 2
                                                / 1e9 / hbm, 4)},
            "gpu_launches": int(launches),
            "phase_ms": {"forward": round(t_fwd / args.steps, 3), "adjoint": round(t_adj / args.steps, 3),
                         "other": round((t_tot - t_fwd - t_adj) / args.steps, 3)},
            "launch_choice": ({k: (round(v, 2) if isinstance(v, float) else v) for k, v in tuning.items()}
                              | {"by": f"fwi_autotune, {args.autotune} steps per candidate"}
                              if tuning else "built-in"),
        }
        if clk:
            r["clocks"] = clk
        return r

    if args.only_accuracy:  # the FP64 comparison alone (any storage, large workloads)
        return {"metric": METRIC, "workload": w.name, "shots": nshots, "storage": args.storage,
                "accuracy_vs_fp64": accuracy(args, w, context, obs_d, fwi_gb300)} if rank == 0 else None
    if args.only_inversion:  # the inversion loop alone (large workloads)
        return {"metric": METRIC, "workload": w.name, "shots": nshots, "storage": args.storage,
                "inversion": inversion(args, w, context, obs_d, shots, torch)} if rank == 0 else None
    head = measure(args.storage, True)
    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": head["value"], "unit": "shots/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": f"synthetic (seeded {args.workload} model, observed data modelled on the GPU from the true model)",
            "config": config_of(args, w), "launch_choice": head["launch_choice"],
            "gpt_updates_per_s": head["gpt_updates_per_s"],
            "gpt_updates_counted_on": f"updated points: {w.nx - 8} x {w.nz - 8} per shot and step, forward and "
                                      f"adjoint (the 4-point frame excluded)",
            "e2e": head["e2e"], "roofline": head["roofline"], "gpu_launches": head["gpu_launches"],
            "phase_ms": head["phase_ms"], "misfit": head["misfit"], "device_gb": head["device_gb"],
        }
        if "clocks" in head:
            out["clocks"] = head["clocks"]

    if not args.skip_extras:
        # the other image stores, same workload and timing rules
        for other in [s for s in ("checkpoint", "full") if s != args.storage]:
            o = measure(other, False)
            if rank == 0:
                out.setdefault("other_storage", {})[other] = {
                    k: o[k] for k in ("value", "ms_per_step", "gpt_updates_per_s", "phase_ms", "launch_choice",
                                      "device_gb")
                } | {"e2e": o["e2e"]["value"], "roofline_frac": o["roofline"]["frac"],
                     "gradient_frac": o["roofline"]["gradient_frac"]}

    if rank == 0 and not args.skip_extras:
        # plain per-shot FP32 path (one shot per launch sequence, FP32 images, every step's kernels
        # launched from the host as the reference does), on a subset; the same with the batch
        # sections replayed as CUDA graphs beside it
        sub = fwi_gb300.make_shots(w.shots[: args.plain_shots])
        nsub = sum(s["nt"] * (s["rx1"] - s["rx0"]) for s in w.shots[: args.plain_shots])
        plain = {}
        os.environ["FWI_CLUSTER"] = "0"  # the per-step tile launches, whatever the window
        for graphs in (False, True):
            c1 = context(1, store_prec=fwi_gb300.SPREC_NATIVE, store="full")
            c1.set_graphs(graphs)
            c1.set_model(*w.squared(initial=True))
            for _ in range(2):
                c1.gradient(sub, obs_d[:nsub])
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            c1.gradient(sub, obs_d[:nsub])
            torch.cuda.synchronize()
            plain[graphs] = args.plain_shots / (time.perf_counter() - t0)
            del c1
        os.environ.pop("FWI_CLUSTER", None)
        value = out["value"] / world
        out["plain_gpu"] = {"value": round(plain[False], 4), "unit": "shots/s",
                            "how": f"max_shots=1, FP32 images, full storage, kernels launched from the host "
                                   f"every step, {args.plain_shots} shots timed",
                            "speedup": round(value / plain[False], 2),
                            "with_graph_replay": {"value": round(plain[True], 4),
                                                  "speedup": round(value / plain[True], 2)}}
        for k, o in out.get("other_storage", {}).items():
            o["plain_gpu_speedup"] = round(o["value"] / world / plain[False], 2)
        out["accuracy_vs_fp64"] = accuracy(args, w, context, obs_d, fwi_gb300)
        out["single_shot_c1"] = single_shot_c1(args, fwi_gb300, torch, dev)
        # L-BFGS two-loop (m = 5) on this grid, FP64 dots
        cl = context(1)
        cl.set_model(*w.squared(initial=True))
        rng = np.random.default_rng(0)
        g0 = [rng.standard_normal((w.nz, w.nx)).astype(np.float32) for _ in range(3)]
        cl.set_gradient(*g0)
        cl.first_step(3e5, 2e5, 2.5e5)
        for it in range(6):
            cl.set_gradient(*(a * (1 + 0.01 * it) + rng.standard_normal(a.shape).astype(np.float32) * 1e-3
                              for a in g0))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cl.lbfgs_direction(5)
            tl = time.perf_counter() - t0
            cl.lbfgs_update(1e-3, 1e-3, 1e-3)
        out["lbfgs_direction_ms"] = round(tl * 1e3, 3)
        del cl
        if args.invert_iters > 0:
            out["inversion"] = inversion(args, w, context, obs_d, shots, torch)
    if rank == 0 and not args.skip_cpu:
        v, thr, sample = cpu_sample(w, seconds=args.cpu_seconds)
        out["cpu_baseline"] = {"value": round(v, 6), "unit": "shots/s", "cores": thr, "kind": "port",
                               "sample": sample}
        v1, _, sample1 = cpu_sample(w, seconds=args.cpu_seconds, threads=1)
        out["cpu_baseline_single_thread"] = {"value": round(v1, 6), "unit": "shots/s", "cores": 1, "kind": "port",
                                             "sample": sample1}
    return out


def single_shot_c1(args, fwi_gb300, torch, dev, steps=10, warmup=3):
    """The plain single-shot gradient (C1: 209 x 209, nt 2000, one shot, full image storage) on the
    small-shot cluster path (one 16-CTA cluster takes the shot through every step in one launch per
    phase) and, beside it, on the per-step tile passes (FWI_CLUSTER=0); device-resident inputs,
    CUDA events over `steps` gradients after `warmup`."""
    from fwi_gb300 import synth
    w = synth.WORKLOADS["C1"]()
    shots = fwi_gb300.make_shots(w.shots)
    sprec = {"fp32": fwi_gb300.SPREC_NATIVE, "fp16": fwi_gb300.SPREC_FP16, "bf16": fwi_gb300.SPREC_BF16}[args.store]
    out = {"workload": w.name, "storage": "full", "image_store": args.store, "steps": steps}
    obs = None
    for name, flag in (("cluster", "1"), ("tile_passes", "0")):
        os.environ["FWI_CLUSTER"] = flag
        c = fwi_gb300.Context(nx=w.nx, nz=w.nz, dh=w.dh, dt=w.dt, cpml=w.cpml, f_cpml=w.f, nt_max=w.nt,
                              max_shots=1, max_receivers=w.nx, mode=fwi_gb300.MODE_EXACT,
                              precision=fwi_gb300.PREC_FP32, store_prec=sprec, store=fwi_gb300.STORE_FULL,
                              device=dev)
        c.set_ricker(w.f, w.nt)
        if obs is None:
            c.set_model(*w.squared())
            obs = torch.zeros(w.nt * (w.shots[0]["rx1"] - w.shots[0]["rx0"]), dtype=torch.float32, device="cuda")
            c.forward(shots, out=obs)
        c.set_model(*w.squared(initial=True))
        g = [torch.zeros((w.nz, w.nx), dtype=torch.float32, device="cuda") for _ in range(3)]
        for _ in range(warmup):
            c.gradient(shots, obs, out=g)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        t_fwd = t_adj = 0.0
        launches = 0
        for _ in range(steps):
            c.gradient(shots, obs, out=g)
            t = c.last_timing()
            t_fwd += float(t[1])
            t_adj += float(t[2])
            launches += c.last_launches()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"value": round(1e3 / ms, 3), "unit": "shots/s", "ms_per_gradient": round(ms, 3),
                     "phase_ms": {"forward": round(t_fwd / steps, 3), "adjoint": round(t_adj / steps, 3)},
                     "launches_per_gradient": launches // steps,
                     "gpt_updates_per_s": round(w.physical_point_updates() / (ms / 1e3) / 1e9, 3)}
        del c
    os.environ.pop("FWI_CLUSTER", None)
    out["cluster_speedup_over_tile_passes"] = round(out["cluster"]["value"] / out["tile_passes"]["value"], 3)
    # the same small shots in a batch: one cluster per shot, the clusters side by side on the GPU
    nb = 8
    base = w.shots[0]
    many = [dict(base, sx=int(8 + (w.nx - 16) * (k + 0.5) / nb)) for k in range(nb)]
    sh8 = fwi_gb300.make_shots(many)
    for name, flag in (("cluster_batch_of_8", "1"), ("tile_passes_batch_of_8", "0")):
        os.environ["FWI_CLUSTER"] = flag
        c = fwi_gb300.Context(nx=w.nx, nz=w.nz, dh=w.dh, dt=w.dt, cpml=w.cpml, f_cpml=w.f, nt_max=w.nt,
                              max_shots=nb, max_receivers=w.nx, mode=fwi_gb300.MODE_EXACT,
                              precision=fwi_gb300.PREC_FP32, store_prec=sprec, store=fwi_gb300.STORE_FULL,
                              device=dev)
        c.set_ricker(w.f, w.nt)
        c.set_model(*w.squared())
        obs8 = torch.zeros(nb * w.nt * (base["rx1"] - base["rx0"]), dtype=torch.float32, device="cuda")
        c.forward(sh8, out=obs8)
        c.set_model(*w.squared(initial=True))
        g = [torch.zeros((w.nz, w.nx), dtype=torch.float32, device="cuda") for _ in range(3)]
        for _ in range(warmup):
            c.gradient(sh8, obs8, out=g)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            c.gradient(sh8, obs8, out=g)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"value": round(nb * 1e3 / ms, 3), "unit": "shots/s", "shots": nb, "ms_per_gradient": round(ms, 3)}
        del c
    os.environ.pop("FWI_CLUSTER", None)
    return out


def accuracy(args, w, context, obs_d, fwi_gb300):
    """Residual, misfit and gradient errors of this configuration (storage, image type) against the FP64 GPU
    path on the first shots, same observed data.  Gradients compare over the whole grid and over the rows
    the model update changes (below the near-surface layer of 15 rows, src/parallelcalls.cu:343-404)."""
    n = args.accuracy_shots
    sub = fwi_gb300.make_shots(w.shots[:n])
    nsub = sum(s["nt"] * (s["rx1"] - s["rx0"]) for s in w.shots[:n])
    obs32 = obs_d[:nsub].cpu().numpy()
    mask = None if w.mask is None else w.mask[: sum(s["rx1"] - s["rx0"] for s in w.shots[:n])]
    # every step's images kept where they fit (60 GB), else checkpoints (the same images, recomputed)
    nb = min(n, args.batch)
    win = max((s["nxw"] or w.nx) for s in w.shots[:n])
    full_bytes = lambda elem: nb * w.nt * 2 * w.nz * (-(-win // 32) * 32) * elem
    ref_store = "full" if full_bytes(8) <= 60e9 else "checkpoint"
    c64 = context(nb, precision=fwi_gb300.PREC_FP64, store_prec=fwi_gb300.SPREC_NATIVE, store=ref_store)
    c64.set_model(*(a.astype(np.float64) for a in w.squared(initial=True)))
    r64 = c64.gradient(sub, obs32.astype(np.float64), mask)
    syn64 = c64.forward(sub)
    del c64
    out = {"shots": n, "order": "v_hor, v_po, v_nmo", "update_rows": "iz > 15", "fp64_storage": ref_store}
    rel = lambda a, b, z=0: float(np.linalg.norm((a - b)[z:]) / np.linalg.norm(b[z:]))
    res64 = syn64 - obs32.astype(np.float64)
    exact32 = "full" if full_bytes(4) <= 60e9 else "checkpoint"
    for label, store, sp in ((f"{args.storage}_{args.store}", args.storage, None),
                             (f"{exact32}_fp32_images", exact32, fwi_gb300.SPREC_NATIVE)):
        cx = context(min(n, args.batch), store=store, **({} if sp is None else {"store_prec": sp}))
        cx.set_model(*w.squared(initial=True))
        rx = cx.gradient(sub, obs32, mask)
        syn32 = cx.forward(sub)
        del cx
        out[label] = {
            "gradient": [round(rel(a, b), 7) for a, b in zip(rx[1:], r64[1:])],
            "gradient_update_rows": [round(rel(a, b, 16), 7) for a, b in zip(rx[1:], r64[1:])],
            "residual": round(float(np.linalg.norm(syn32 - obs32 - res64) / np.linalg.norm(res64)), 9),
            "traces": round(float(np.linalg.norm(syn32 - syn64) / np.linalg.norm(syn64)), 9),
            "misfit": abs(rx[0] - r64[0]) / abs(r64[0])}
    g = r64[1:]
    out["gradient_norm_share_in_rows_0_15"] = [round(float(np.sum(a[:16] ** 2) / np.sum(a ** 2)), 4) for a in g]
    return out


def inversion(args, w, context, obs_d, shots, torch):
    """The workload's inversion loop through the C driver (fwi_invert: steepest first step, then L-BFGS
    with the backtracking line search, src/main.c:396-801) from the initial model, timed end to end:
    the reference's policy as it is, and with the curvature safeguard (pairs with y.s <= 0 skipped)
    and the step length reset to 1 at each iteration."""
    out = {}
    for name, opts in (("reference_policy", {}), ("curvature_guard", {"curvature_guard": 1, "reset_alpha": 1})):
        ctx = context(min(args.batch, len(w.shots)))
        ctx.set_model(*w.squared(initial=True))
        if args.autotune > 0:
            ctx.autotune(shots, steps=args.autotune)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if w.bands:
            # multiscale (src/main.c:274-806): per band, the records re-modelled on the device from the
            # true model at the band's frequency into the context's store (no host copy)
            true = w.squared()

            def band_obs(band, f):
                ctx.model_observed(shots, *true)
                return None
            hist = ctx.invert_bands(shots, band_obs, w.bands[0], w.bands[1] - w.bands[0], len(w.bands), w.nt,
                                    mask=w.mask, iterations=args.invert_iters, lbfgs_m=5, **opts)
            hist = np.concatenate(hist)
        else:
            hist = ctx.invert(shots, obs_d, w.mask, iterations=args.invert_iters, lbfgs_m=5, **opts)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        del ctx
        out[name] = {"options": opts, "iterations": len(hist), "requested": args.invert_iters, "lbfgs_m": 5,
                     "bands_hz": list(w.bands) or None,
                     "storage": args.storage, "wall_s": round(dt, 3),
                     "s_per_iteration": round(dt / max(1, len(hist)), 4),
                     "misfit_first": float(hist[0]) if len(hist) else None,
                     "misfit_last": float(hist[-1]) if len(hist) else None,
                     "misfit_history": [round(float(x), 3) for x in hist]}
    return out


def reference_arm(args, rank, world, dist):
    """The reference's CPU arithmetic (oracle restatement; the reference has no CPU
    path of its own), all host threads, bounded samples of the same workload."""
    if rank != 0:
        return None
    w = make_workload(args)
    secs = max(2.0, args.cpu_seconds / max(1, args.steps))
    vals = []
    for _ in range(args.warmup):  # untimed, short samples
        cpu_sample(w, seconds=1.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, thr, sample = cpu_sample(w, seconds=secs)
        vals.append(v)
    dt = time.perf_counter() - t0
    v = statistics.median(vals)
    out = {"metric": METRIC, "value": round(v, 6), "unit": "shots/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "impl": "reference",
            "data": f"synthetic (seeded {args.workload} model)", "config": config_of(args, w),
            "cpu_baseline": {"value": round(v, 6), "unit": "shots/s", "cores": thr, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 6), "unit": "shots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    ref_gpu = reference_gpu_kernels(w)
    if ref_gpu:
        out["reference_gpu_kernels"] = ref_gpu
    return out


def reference_gpu_kernels(w):
    """The reference's own CUDA kernels (compiled unchanged for sm_103a into oracle/_ref where the
    reference checkout was present at build time) on one GPU, one shot at a time as src/main.c runs
    them (per-step snapshot through pinned host memory, host misfit sum): gradient shots/s of the
    workload's first shot, for context beside the CPU figure.  None where they were not built."""
    from oracle import pyoracle as po
    if not po.ref_gpu_available():
        return None
    s = w.shots[0]
    if s["nxw"]:
        return None  # the reference has no shot windows
    obs = np.zeros((s["nt"], w.nx), np.float32)  # the work does not depend on the data
    try:
        secs, _, _, _ = po.ref_gpu_shot(w.vel0, w.eps0, w.delta0, obs, w.nx, w.nz, s["nt"], w.cpml, w.dh, w.dt, w.f,
                                        s["sx"] + 1, s["sz"] + 1, runs=3)
    except Exception as e:  # noqa: BLE001 - reported, not fatal to the CPU arm
        return {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    best = min(secs[1:])
    return {"value": round(1.0 / best, 4), "unit": "shots/s", "seconds_per_shot": [round(x, 4) for x in secs],
            "how": "src/parallelcalls.cu compiled for sm_103a with nvcc's defaults, one shot sequenced as "
                   "src/main.c:318-495 (per-step snapshot via pinned host memory, residual summed on the host); "
                   "best of the runs after the first; zero observed data (the work does not depend on it)",
            "gpt_updates_per_s": round(2 * (w.nx - 8) * (w.nz - 8) * s["nt"] / best / 1e9, 3)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="C2")
    ap.add_argument("--shots", type=int, default=None, help="shots (default: the workload's own)")
    ap.add_argument("--nt", type=int, default=None, help="time steps (default: the workload's own)")
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--mode", default="exact", choices=["exact", "ref"])
    ap.add_argument("--store", default="fp16", choices=["fp32", "fp16", "bf16"])
    ap.add_argument("--storage", default="checkpoint", choices=["full", "checkpoint", "boundary"],
                    help="how the forward images are kept (FWI_STORE_*) in the headline run")
    ap.add_argument("--ckpt-every", type=int, default=0,
                    help="checkpoint interval in steps (0: automatic, the one that needs the least memory)")
    ap.add_argument("--plain-shots", type=int, default=4)
    ap.add_argument("--accuracy-shots", type=int, default=8, help="shots of the FP64 comparison")
    ap.add_argument("--invert-iters", type=int, default=20,
                    help="L-BFGS iterations of the timed inversion loop (per band for multiscale workloads; 0: none)")
    ap.add_argument("--only-accuracy", action="store_true",
                    help="only the FP64 comparison of --storage / --store on --accuracy-shots shots")
    ap.add_argument("--only-inversion", action="store_true",
                    help="time the inversion loop only (no gradient benchmark), e.g. C5's bands on a shot subset")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-extras", action="store_true")
    ap.add_argument("--autotune", type=int, default=48,
                    help="fwi_autotune with this many steps per candidate before the warm-up (0: built-in choice)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, dist = dist_setup()
    if args.impl == "reference":
        out = reference_arm(args, rank, world, dist)
    else:
        out = native_arm(args, rank, world, dist)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
