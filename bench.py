#!/usr/bin/env python
"""Benchmark: Mpoints/s of the plain per-pair GPU path on the 5 MP workload.

Workload (one step = one stereo pair): 2448x2048 per camera, hierarchical
1/8/64-fringe phase shift, 4 steps each (12 frames), 12-bit values in u16,
seeded synthetic scene (Gaussian bumps over a plane at 900 mm plus box
occluders), f = 2400 px, baseline 200 mm, k1 = -0.05, k2 = 0.01; decode ->
rectify -> match -> 5x5 median -> Q reprojection -> SOR (k = 30) -> MLS
(radius 2 mm, order 2) -> Gaussian (sigma 0.5 mm).  Inputs (240 MB per pair)
exceed the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--width W --height H]   (the same workload scaled; profiling runs)

N > 1 runs under torchrun: independent replicas, one pair per rank per step
(weak scaling, no collective on the data path); the time is the max over ranks.
--impl reference times the CPU restatement of the path (oracle/, all host
threads; the CPU suite pins it to the reference's own code) on the same
workload: each timed step is one whole pair (warm-up steps are one band of
rows each, to warm the caches and the thread pool only).
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpoints/s at 5 MP (plain per-pair GPU path)"
UNIT = "Mpoints/s"
WORKLOAD = "5MP pair: 2448x2048 x2 cams, hierarchical 1/8/64 x 4 steps, u16 12-bit; decode+rectify+match+median+reproject+SOR(k30)+MLS(r2mm,o2)+Gaussian(0.5mm)"


def workload_name(W, H):
    if (W, H) == (2448, 2048):
        return WORKLOAD
    return WORKLOAD.replace("5MP pair: 2448x2048", f"{W}x{H} pair (5 MP workload scaled)")


def workload_config(W, H, F, rect_w, rect_h, input_bytes):
    """The `config` object, identical for both arms (same workload, same keys)."""
    return {"workload": workload_name(W, H), "width": W, "height": H, "rect": [rect_w, rect_h],
            "frames_per_camera": F, "parallelism": "one pair per step per GPU (replicas)",
            "l2": (f"inputs {input_bytes / 1e6:.0f} MB per pair > 129 MB L2 (no flush)"
                   if input_bytes > 129e6 else "inputs smaller than L2: profiling size only")}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


# DRAM bytes per launch (read + write) of a stage's kernel on the 5 MP
# workload, from one ncu capture each (profiles/*_5mp_dram.md): the
# roofline's `traffic` for that kernel when it dominates the step.
MEASURED_TRAFFIC = {("mls", 2448, 2048): (68118016 + 26156032, "profiles/mls_smem_kernel_5mp.md")}
# Warp instructions per launch and the FMA pipe's busy fraction of a stage's
# kernel on the 5 MP workload, from one ncu capture (profiles/*_5mp.md): the
# issue-slot side of the roofline for kernels bound by instruction issue.
# timed blocks of the end-to-end measurement (the median is reported)
E2E_BLOCKS = 3
MEASURED_ISSUE = {("mls", 2448, 2048): (1079920613, 0.6405, "profiles/mls_smem_kernel_5mp.md")}


def issue_roofline(stage, W, H, ms_per_launch, sm_mhz):
    """Achieved warp instructions per second against the issue peak (one warp
    instruction per scheduler per cycle: 4 x SMs x SM clock), or None."""
    m = MEASURED_ISSUE.get((stage, W, H))
    if not m:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    inst, fma, src = m
    ach = inst / (ms_per_launch * 1e-3) / 1e9
    pk = 4 * sms * sm_mhz * 1e6 / 1e9
    return {"warp_inst_per_launch": inst, "achieved_ginst_s": round(ach, 1), "peak_ginst_s": round(pk, 1),
            "frac": round(ach / pk, 4), "fma_pipe_frac": fma, "source": src,
            "note": "peak: one warp instruction per scheduler per cycle at the median SM clock of the timed region"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled every 20 ms from before
    the warm-up to after the timed regions; the summary keeps the samples
    taken inside the windows passed to mark()."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int, period_ms: int = 20):
        self.gpu, self.rows, self.proc, self.period = gpu, [], None, period_ms
        self.windows = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0:  # sampler running before any timing
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def mark(self, t0, t1):
        """A timed window (perf_counter seconds)."""
        self.windows.append((t0, t1))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        inside = [r for t, r in self.rows if any(a <= t <= b for a, b in self.windows)]
        rows = inside or [r for _, r in self.rows]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "in_timed_windows": bool(inside),
                "samples_total": len(self.rows),
                "period_ms": self.period}


def config1_recon(api):
    return api.recon_config(use_px_gaussian=0, use_ror=0, use_sor=1, sor_mean_k=30, sor_std_mul=1.0, use_mls=1,
                            mls_window_size=7, mls_spatial_sigma=2.0 / math.sqrt(2.0), mls_polynomial_order=2,
                            mls_max_radius=2.0, mls_iterations=1, use_metric_gaussian=1, metric_gaussian_sigma=0.5)


def stage_breakdown(api, ctx, dcfg, rcfg, spec, dL, dR, steps):
    """Per-stage device time (CUDA events on the launching stream), ms per launch.

    The stages are called one by one from Python, so each step starts with a
    bounded spin kernel (about 2 ms) queued ahead of the first event: the host
    enqueues the stages while the device is still busy, and each event pair
    brackets device work only, not the Python call between two stages."""
    import torch
    H, W = dL.shape[1:]
    st = torch.cuda.current_stream()
    names = ["decode", "rectify_match", "median_reproject", "sor", "mls", "metric_gaussian"]
    acc = {n: 0.0 for n in names}
    cnt = {n: 0 for n in names}
    ev = lambda: torch.cuda.Event(enable_timing=True)
    hold = getattr(torch.cuda, "_sleep", None)
    stage_breakdown.hold_ran = hold is not None
    for _ in range(steps):
        e = [ev() for _ in range(12)]
        if hold is not None:
            hold(4_000_000)  # clock cycles
        e[0].record(st)
        dl = api.decode(ctx, dcfg, dL, want_mod=False, want_valid=False)
        e[1].record(st)
        dr = api.decode(ctx, dcfg, dR, want_mod=False, want_valid=False)
        e[2].record(st)
        disp = api.rectify_match(ctx, (dl["order"], dl["residual"]), (dr["order"], dr["residual"]), spec.pha_f)
        e[3].record(st)
        e[4].record(st)
        _, xyz, mask = api.median_reproject(ctx, rcfg, disp)
        e[5].record(st)
        m2, _ = api.filter_sor(ctx, xyz, mask, 30, 1.0)
        e[6].record(st)
        x2 = api.filter_mls(ctx, xyz, m2, 7, 2.0 / math.sqrt(2.0), 2, 2.0, 1)
        e[7].record(st)
        api.filter_metric_gaussian(ctx, x2, m2, 0.5)
        e[8].record(st)
        torch.cuda.synchronize()
        acc["decode"] += e[0].elapsed_time(e[1]) + e[1].elapsed_time(e[2]); cnt["decode"] += 2
        acc["rectify_match"] += e[2].elapsed_time(e[4]); cnt["rectify_match"] += 1
        acc["median_reproject"] += e[4].elapsed_time(e[5]); cnt["median_reproject"] += 1
        acc["sor"] += e[5].elapsed_time(e[6]); cnt["sor"] += 1
        acc["mls"] += e[6].elapsed_time(e[7]); cnt["mls"] += 1
        acc["metric_gaussian"] += e[7].elapsed_time(e[8]); cnt["metric_gaussian"] += 1
    per_step = {n: acc[n] / steps for n in names}
    per_launch = {n: acc[n] / cnt[n] for n in names}
    return per_step, per_launch


def run_ours(args):
    import numpy as np
    import torch
    from zim_gb300 import api, synth

    rank, local, world = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    spec = synth.config1(seed=1 + rank, width=args.width, height=args.height)
    L, R = spec.render(0), spec.render(1)
    F, H, W = L.shape
    # `inflight` pairs in flight: one context (scratch) and one stream each,
    # pairs assigned round-robin; the timed region spans all of them
    nf = max(1, args.inflight)
    ctxs = [api.Context(local) for _ in range(nf)]
    for c in ctxs:
        c.set_calibration(spec.rig.as_dict(), True)
    ctx = ctxs[0]
    dcfg = api.decode_config(**spec.decode_kwargs())
    rcfg = config1_recon(api)
    dL, dR = torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda()
    outs = [(torch.empty((ctx.rect_h, ctx.rect_w, 3), dtype=torch.float32, device="cuda"),
             torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8, device="cuda"), None) for _ in range(nf)]
    streams = [torch.cuda.Stream() for _ in range(nf)]
    st = torch.cuda.current_stream()
    for i in range(args.warmup):
        with torch.cuda.stream(streams[i % nf]):
            api.reconstruct_pair(ctxs[i % nf], dcfg, rcfg, dL, dR, out=outs[i % nf])
    torch.cuda.synchronize()
    n_pts = int(outs[0][1].sum().item())

    def barrier():
        if dist:
            dist.barrier()

    def fork(ev):
        ev.record(st)
        for s in streams:
            s.wait_event(ev)

    def join():
        for s in streams:
            ev = torch.cuda.Event()
            ev.record(s)
            st.wait_event(ev)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # end to end through the host entry: pinned frames in, xyz + mask out, copies timed
    hL = torch.from_numpy(L).pin_memory()
    hR = torch.from_numpy(R).pin_memory()
    houts = [(torch.empty((ctx.rect_h, ctx.rect_w, 3), dtype=torch.float32).pin_memory(),
              torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8).pin_memory()) for _ in range(nf)]
    hx, hm = houts[0]

    def host_pairs(steps):
        for i in range(steps):
            api.reconstruct_pair_host(ctxs[i % nf], dcfg, rcfg, hL, hR, xyz=houts[i % nf][0], mask=houts[i % nf][1],
                                      stream=streams[i % nf], asynchronous=True)

    host_pairs(max(nf, args.warmup // 2))
    torch.cuda.synchronize()
    gc.collect()
    gc.disable()  # no collector pause inside the timed regions
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        l0 = sum(c.launch_count() for c in ctxs)
        t0 = time.perf_counter()
        fork(e0)
        for i in range(args.steps):
            with torch.cuda.stream(streams[i % nf]):
                api.reconstruct_pair(ctxs[i % nf], dcfg, rcfg, dL, dR, out=outs[i % nf])
        join()
        e1.record(st)
        torch.cuda.synchronize()
        clk.mark(t0, time.perf_counter())
        barrier()
        launches = sum(c.launch_count() for c in ctxs) - l0
        ms = e0.elapsed_time(e1) / args.steps

        # end to end: E2E_BLOCKS timed blocks of `steps` pairs each, every
        # pair's frames up and cloud down inside its block; the median block
        # is reported (one stalled host thread otherwise decides the figure)
        block_ms = []
        for _ in range(E2E_BLOCKS):
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fork(e0)
            host_pairs(args.steps)
            join()
            e1.record(st)
            torch.cuda.synchronize()
            wall = (time.perf_counter() - t0) / args.steps
            clk.mark(t0, time.perf_counter())
            barrier()
            block_ms.append(max(e0.elapsed_time(e1) / args.steps, wall * 1e3))
    gc.enable()
    e2e_ms = statistics.median(block_ms)
    pts_total = n_pts
    if dist:
        t = torch.tensor([ms, e2e_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, e2e_ms = float(t[0].item()), float(t[1].item())
        p = torch.tensor([n_pts], device="cuda", dtype=torch.float64)
        dist.all_reduce(p, op=dist.ReduceOp.SUM)
        pts_total = int(p.item())
    value = pts_total / (ms * 1e-3) / 1e6
    e2e = pts_total / (e2e_ms * 1e-3) / 1e6
    h2d = 2 * L.nbytes
    d2h = hx.numel() * 4 + hm.numel()

    result = None
    if rank == 0:
        per_step, per_launch = stage_breakdown(api, ctx, dcfg, rcfg, spec, dL, dR, max(3, min(args.steps, 10)))
        dom = max(per_step, key=per_step.get)
        peak, src = peaks()
        npx, rpx = H * W, ctx.rect_h * ctx.rect_w
        # algorithmic bytes per launch: each stage's compulsory reads + writes per source pixel (npx)
        # or rectified pixel (rpx), e.g. decode reads F u16 frames and writes an int32 fringe order
        # and an f32 residual phase (8 B)
        # rectify_match: both cameras' decoded maps read (8 B per source pixel each; the post-smooth's
        # taps are an intermediate) and the raw disparity written (4 B per rectified pixel)
        alg = {"decode": npx * (F * 2 + 8), "rectify_match": 2 * npx * 8 + rpx * 4,
               "median_reproject": rpx * (4 + 13), "sor": rpx * (13 + 13), "mls": rpx * (13 + 12),
               "metric_gaussian": rpx * (13 + 12)}
        # decode + rectify + match + median + reprojection against the HBM roofline:
        # the pair's compulsory bytes (both frame stacks in, cloud + mask out)
        # over the stages' summed one-stream times
        pix_ms = per_step["decode"] + per_step["rectify_match"] + per_step["median_reproject"]
        pix_bytes = 2 * npx * F * 2 + rpx * 13
        pixel_stages = {"ms_per_pair": round(pix_ms, 4), "compulsory_bytes": pix_bytes,
                        "achieved_gbs": round(pix_bytes / (pix_ms * 1e-3) / 1e9, 1),
                        "frac": round(pix_bytes / (pix_ms * 1e-3) / 1e9 / peaks()[0], 4)}
        stages = {n: {"ms_per_step": round(per_step[n], 4), "ms_per_launch": round(per_launch[n], 4),
                      "gbs": round(alg[n] / (per_launch[n] * 1e-3) / 1e9, 1)} for n in per_step}
        achieved = alg[dom] / (per_launch[dom] * 1e-3) / 1e9
        dec_achieved = alg["decode"] / (per_launch["decode"] * 1e-3) / 1e9
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            cpu = cpu_baseline(spec, L, R)
        result = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (u16 samples; FP64 only for near-zero-disparity divides)",
            "data": "synthetic (seeded scene renderer, zim_gb300/synth)",
            "config": workload_config(W, H, F, ctx.rect_w, ctx.rect_h, 2 * L.nbytes),
            "points_per_pair": n_pts, "replicas": world, "pairs_in_flight": nf,
            "pixel_pairs_per_s": round(world * npx / (ms * 1e-3), 1),
            "pixel_stages": pixel_stages,
            "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "blocks_ms_per_step": [round(b, 4) for b in block_ms],
                    "ms_per_step": round(e2e_ms, 4)},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "peak_source": src, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": MEASURED_TRAFFIC.get((dom, W, H), (None, None))[0],
                         "traffic_source": MEASURED_TRAFFIC.get((dom, W, H), (None, None))[1],
                         "algorithmic_bytes": alg[dom],
                         "decode_kernel": {"achieved": round(dec_achieved, 1),
                                           "frac": round(dec_achieved / peak, 4)}},
            "stages": stages,
            "stages_hold": bool(getattr(stage_breakdown, "hold_ran", False)),
            "clocks": clk.summary(),
        }
        iss = issue_roofline(dom, W, H, per_launch[dom], result["clocks"].get("sm_mhz") or 2070.0)
        if iss:
            result["roofline"]["issue"] = iss
        if cpu:
            result["cpu_baseline"] = cpu
        if not args.no_batch:
            result["batch"] = run_batch(api, local, steps=5, warmup=3)
        if not args.no_diff:
            result["diff"] = run_diff(api, local, steps=5, warmup=3,
                                      want_cpu=world == 1 and not args.no_cpu_baseline)
        if not args.no_refine:
            result["refine"] = run_refine(api, local, args.refine_poses, args.refine_iters)
        print(json.dumps(result))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return result


def cpu_band_step(spec, L, R, rect, y0, y1):
    from oracle import pipeline as P
    t = time.perf_counter()
    xyz, mask = P.run_band(spec.decode_kwargs(), spec.pha_f, L, R, rect, y0, y1, P.CONFIG1_FILTERS)
    return time.perf_counter() - t, int(mask.sum())


def cpu_pair_step(spec, L, R, rect):
    """The whole pair on the CPU restatement (every stage, SOR statistics over
    the whole cloud): seconds and points."""
    from oracle import pipeline as P
    t = time.perf_counter()
    xyz, mask = P.run_pair(spec.decode_kwargs(), spec.pha_f, L, R, rect, P.CONFIG1_FILTERS)
    return time.perf_counter() - t, int(mask.sum())


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


def cpu_baseline(spec, L, R):
    """The CPU restatement on one whole pair of the same workload (all host threads)."""
    from oracle import pipeline as P
    rect = P.Rectification(spec.rig.as_dict(), True)
    cpu_band_step(spec, L, R, rect, rect.h // 2, rect.h // 2 + 16)  # warm caches / OpenMP pool
    dt, n = cpu_pair_step(spec, L, R, rect)
    return {"value": round(n / dt / 1e6, 4), "unit": UNIT, "cores": cpu_threads(), "kind": "port",
            "sample": f"one whole pair of the same workload ({n} points), every stage incl. SOR/MLS/Gaussian, "
                      f"{dt:.2f} s; the restatement is pinned to the reference's own code by the CPU tests"}


DIFF_WORKLOAD = ("planar target at 8 seeded poses (tilt +-30 deg, depth 600-1200 mm), 2448x2048 x2 cams, "
                 "config-1 rig; forward + adjoint of sub-pixel matching + reprojection w.r.t. 16 calibration "
                 "parameters and per-pixel phase, point-to-plane loss, evaluated at the perturbed calibration "
                 "(baseline +0.5%, cx0 +3 px, k1_0 +0.02)")


def perturbed_theta(theta):
    import numpy as np
    th = np.array(theta, np.float64)
    th[12] *= 1.005
    th[2] += 3.0
    th[4] += 0.02
    return th


def diff_poses(api, local, n_poses, seed=3):
    """Renders n_poses planar-target poses, decodes them on the GPU (phase stays
    resident) under the true calibration."""
    from zim_gb300 import calib_refine as CR, synth
    specs = [synth.pose_plane(seed=seed, pose=p) for p in range(n_poses)]
    ctx = api.Context(local)
    ctx.set_calibration(specs[0].rig.as_dict(), True)
    dcfg = api.decode_config(**specs[0].decode_kwargs())
    poses = []
    for s in specs:
        poses += CR.decode_views(ctx, dcfg, [(s.render(0), s.render(1))], [(s.plane_n, s.plane_d)])
    return specs, ctx, poses


def cpu_diff_baseline(spec, ctx, pose, theta):
    """FP64 CPU forward + adjoint of one pose (the oracle restatement), timed;
    its gradient is the reference the GPU gradient is checked against."""
    import numpy as np
    from oracle import oracle as O
    rig = spec.rig
    calib = O.make_calib(rig.K, rig.D, rig.R, rig.t, rig.width, rig.height)
    R1, R2, P1, P2, Q, rw, rh = O.rectification(calib)
    ir = [np.linalg.inv(P1[:, :3] @ R1), np.linalg.inv(P2[:, :3] @ R2)]
    dist = [(rig.D[c][2], rig.D[c][3], rig.D[c][4]) for c in range(2)]
    geom = O.diff_geom(ir, dist, Q, float(np.linalg.norm(rig.t)), rw, rh, rig.width, rig.height)
    order = [o.cpu().numpy() for o in pose.order]
    res = [r.cpu().numpy().astype(np.float64) for r in pose.residual]
    t = time.perf_counter()
    o = O.diff_eval(geom, theta, order[0], res[0], order[1], res[1], pose.best.cpu().numpy(), pose.plane,
                    want_grad_abs=True)
    dt = time.perf_counter() - t
    # the same gradient with only the sample positions rounded to FP32: the
    # floor FP32 positions put under an FP32 implementation
    O.diff_round_positions(True)
    try:
        o["grad_fp32_positions"] = O.diff_eval(geom, theta, order[0], res[0], order[1], res[1],
                                               pose.best.cpu().numpy(), pose.plane)["grad"]
    finally:
        O.diff_round_positions(False)
    return o, dt


def run_diff(api, local, steps, warmup, want_cpu=True):
    """Config 3: batched forward/adjoint over 8 poses at 5 MP."""
    import numpy as np
    import torch
    from zim_gb300 import calib_refine as CR, diff
    specs, ctx, poses = diff_poses(api, local, 8)
    th = perturbed_theta(diff.nominal(ctx))
    pha_f = specs[0].pha_f
    CR.update_matches(ctx, th, poses, pha_f)
    views = CR.views_of(poses)
    for _ in range(warmup):
        r = diff.backward(ctx, th, views)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(st)
    for _ in range(steps):
        r = diff.backward(ctx, th, views)
    e1.record(st)
    torch.cuda.synchronize()
    bwd_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3) / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        f = diff.forward(ctx, th, views)
    fwd_ms = (time.perf_counter() - t0) * 1e3 / steps
    t0 = time.perf_counter()
    for _ in range(max(1, steps // 2)):
        CR.update_matches(ctx, th, poses, pha_f)
    torch.cuda.synchronize()
    match_ms = (time.perf_counter() - t0) * 1e3 / max(1, steps // 2)
    out = {"workload": DIFF_WORKLOAD, "poses": len(poses), "points": int(r["n_points"]),
           "forward_ms": round(fwd_ms, 3), "forward_adjoint_ms": round(bwd_ms, 3),
           "rematch_ms": round(match_ms, 3),
           "forward_adjoint_mpoints_s": round(r["n_points"] / (bwd_ms * 1e-3) / 1e6, 2),
           "reductions": "FP64, fixed order (bit-reproducible)"}
    if want_cpu:
        one = diff.backward(ctx, th, views[:1])
        o, dt = cpu_diff_baseline(specs[0], ctx, poses[0], th)
        g, go = one["grad"], o["grad"]
        out["grad_err_vs_fp64"] = {"normwise_rel": float(np.linalg.norm(g - go) / np.linalg.norm(go)),
                                   "worst_component_rel": float(np.max(np.abs(g - go) / np.abs(go))),
                                   "loss_rel": float(abs(one["loss"] - o["loss"]) / o["loss"])}
        # per component: the error against the FP64 oracle, the cancellation
        # factor sum|term| / |sum term|, and the floor of FP32 sample
        # positions (the FP64 oracle's own change when only its positions are
        # rounded to FP32)
        from zim_gb300 import diff as D
        canc = o["grad_abs"] / np.maximum(np.abs(go), 1e-300)
        gp = o["grad_fp32_positions"]
        out["grad_components"] = {
            D.PARAM_NAMES[k]: {"rel_err": float(abs(g[k] - go[k]) / abs(go[k])), "cancellation": float(canc[k]),
                               "fp32_position_floor": float(abs(gp[k] - go[k]) / abs(go[k]))}
            for k in range(len(go))}
        out["grad_err_vs_fp64"]["fp32_position_floor_normwise"] = float(np.linalg.norm(gp - go) /
                                                                         np.linalg.norm(go))
        out["cpu_baseline"] = {"value": round(o["n_points"] / dt / 1e6, 4), "unit": "Mpoints/s (forward+adjoint)",
                               "cores": 1, "kind": "port", "sample": "pose 0 of 8, FP64 oracle, one thread",
                               "seconds": round(dt, 3)}
    return out


def run_refine(api, local, n_poses=8, iterations=60):
    """Config 4 (scaled: n_poses of its 32 planar-target poses, `iterations`
    of its 200 Levenberg-Marquardt steps; --refine-poses 32 --refine-iters 200
    runs it in full): calibration refinement from the perturbed calibration,
    with every parameter's final error against the true calibration."""
    import numpy as np
    import torch
    from zim_gb300 import calib_refine as CR, diff, synth
    specs = [synth.pose_plane(seed=3, pose=p) for p in range(n_poses)]
    rig = specs[0].rig.as_dict()
    truth_ctx = api.Context(local)
    truth_ctx.set_calibration(rig, True)
    theta_true = diff.nominal(truth_ctx)
    # start: the calibration perturbed as config 4 states; its rectified frame
    # defines the virtual cameras, the truth is theta_true in that frame
    pert = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in rig.items()}
    pert["K"] = [k.copy() for k in rig["K"]]
    pert["D"] = [d.copy() for d in rig["D"]]
    pert["K"][0][0, 2] += 3.0
    pert["D"][0][0] += 0.02
    pert["t"] = rig["t"] * 1.005
    ctx = api.Context(local)
    ctx.set_calibration(pert, True)
    dcfg = api.decode_config(**specs[0].decode_kwargs())
    t_r = time.perf_counter()
    poses = []
    for s in specs:
        poses += CR.decode_views(ctx, dcfg, [(s.render(0), s.render(1))], [(s.plane_n, s.plane_d)])
    prep_s = time.perf_counter() - t_r
    th0 = diff.nominal(ctx)
    th, log = CR.refine(ctx, poses, th0, specs[0].pha_f, iterations=iterations)
    names = diff.PARAM_NAMES
    err0 = th0 - theta_true
    err1 = th - theta_true
    return {"workload": f"{n_poses} of config 4's 32 planar-target poses at 2448x2048, {iterations} of its 200 "
                        "Levenberg-Marquardt iterations, from baseline +0.5%, cx0 +3 px, k1_0 +0.02",
            "poses": n_poses, "iterations": iterations, "seconds": round(log.seconds, 3),
            "iterations_per_s": round(iterations / log.seconds, 3), "prepare_s": round(prep_s, 1),
            "start_error": {names[k]: float(err0[k]) for k in (2, 4, 12)},
            "final_error": {n: float(e) for n, e in zip(names, err1)},
            "loss_start": log.losses[0] if log.losses else None, "loss_final": log.losses[-1] if log.losses else None}


BATCH_WORKLOAD = ("64 seeded stereo pairs, sizes drawn from {640x480, 1280x1024, 2448x2048, 4096x3000}, each "
                  "4-step + 5-bit Gray + complementary (config-0 scene/rig, u8; then SOR k=50) or three-frequency "
                  "1/8/64 x 4 steps (config-1 scene/rig, 12-bit u16; then SOR k=30 + MLS r2mm o2 + Gaussian 0.5mm); "
                  "decode+rectify+match+median+reproject+filters; 8 distinct calibrations; plain = the whole-pair "
                  "path pair after pair on one stream")


def run_batch(api, local, steps, warmup, n_pairs=64):
    """Config 2: the batched persistent path against the plain per-pair path
    on the same pairs, same stages, same outputs (checked equal)."""
    import numpy as np
    import torch
    from zim_gb300 import synth
    from zim_gb300.batch import Batch, BatchPair
    specs, keys = synth.config2(n_pairs=n_pairs)
    t0 = time.perf_counter()
    dev = []
    for s in specs:
        dev.append((torch.from_numpy(s.render(0)).cuda(), torch.from_numpy(s.render(1)).cuda()))
    render_s = time.perf_counter() - t0
    uniq = []
    for k in keys:
        if k not in uniq:
            uniq.append(k)
    cidx = [uniq.index(k) for k in keys]
    rigs = [specs[keys.index(k)].rig.as_dict() for k in uniq]
    # per pair the pipeline of its kind: config 0's SOR (k = 50) after the
    # 4-step + Gray pairs, config 1's SOR (k = 30) + MLS + metric Gaussian
    # after the 1/8/64 pairs; no pixel-window filters (neither config has them)
    rcfg = api.recon_config(use_px_gaussian=0, use_ror=0)
    gray_cfg = api.recon_config(use_px_gaussian=0, use_ror=0, use_sor=1, sor_mean_k=50, sor_std_mul=1.0)
    freq_cfg = config1_recon(api)
    pcfg = [gray_cfg if k[0] == "gray" else freq_cfg for k in keys]
    dcfgs = [api.decode_config(**s.decode_kwargs()) for s in specs]
    st = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    # plain per-pair path: one context per calibration (set up untimed), pairs in turn
    ctxs = []
    for r in rigs:
        c = api.Context(local)
        c.set_calibration(r, True)
        ctxs.append(c)
    outs = []
    for i in range(n_pairs):
        c = ctxs[cidx[i]]
        outs.append((torch.empty((c.rect_h, c.rect_w, 3), dtype=torch.float32, device="cuda"),
                     torch.empty((c.rect_h, c.rect_w), dtype=torch.uint8, device="cuda"), None))

    def plain_pass():
        for i in range(n_pairs):
            api.reconstruct_pair(ctxs[cidx[i]], dcfgs[i], pcfg[i], dev[i][0], dev[i][1], out=outs[i])

    for _ in range(warmup):
        plain_pass()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record(st)
    for _ in range(steps):
        plain_pass()
    e1.record(st)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / steps
    n_points = int(sum(int(m.sum().item()) for _, m, _ in outs))

    # batched path
    ctx = api.Context(local)
    b = Batch(ctx, rigs)
    pairs = [BatchPair(dcfgs[i], dev[i][0], dev[i][1], calib=cidx[i], filters=pcfg[i]) for i in range(n_pairs)]
    b.submit(pairs, rcfg)
    tuning, tune_ms = b.autotune()
    for _ in range(warmup):
        b.run()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    e0.record(st)
    for _ in range(steps):
        b.run()
    e1.record(st)
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / steps
    launches = (ctx.launch_count() - l0) // steps
    same = all(torch.equal(p.mask, o[1]) and torch.equal(p.xyz, o[0]) for p, o in zip(pairs, outs))
    alg = 0
    for s, (L, _), i in zip(specs, dev, range(n_pairs)):
        c = ctxs[cidx[i]]
        alg += 2 * L.numel() * L.element_size() + 13 * c.rect_h * c.rect_w
    peak, src = peaks()
    ach = alg / (batch_ms * 1e-3) / 1e9
    sizes = {}
    for k in keys:
        sizes[f"{k[1]}x{k[2]}"] = sizes.get(f"{k[1]}x{k[2]}", 0) + 1
    return {"workload": BATCH_WORKLOAD, "pairs": n_pairs, "points": n_points, "size_mix": sizes,
            "megapixels": round(sum(s.rig.width * s.rig.height for s in specs) / 1e6, 1),
            "batched_mpoints_s": round(n_points / (batch_ms * 1e-3) / 1e6, 2), "batched_ms": round(batch_ms, 3),
            "plain_mpoints_s": round(n_points / (plain_ms * 1e-3) / 1e6, 2), "plain_ms": round(plain_ms, 3),
            "speedup_vs_plain": round(plain_ms / batch_ms, 3), "outputs_identical": bool(same),
            "tuning": tuning, "autotune_best_ms": round(tune_ms, 3), "gpu_launches_per_run": int(launches),
            "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "peak_source": src,
                         "unit": "GB/s", "frac": round(ach / peak, 4),
                         "algorithmic_bytes": int(alg)},
            "render_s": round(render_s, 1)}


def run_reference(args):
    """The reference arm: the CPU restatement of the path (oracle/, all host
    threads), which the CPU suite pins to the reference's own code; each timed
    step is one whole pair of the same workload.  Warm-up steps are one band of
    rows each (they warm the caches and the thread pool; they are not timed)."""
    rank, local, world = env_rank()
    if rank != 0:
        return None
    from oracle import pipeline as P
    from zim_gb300 import synth
    spec = synth.config1(seed=1, width=args.width, height=args.height)
    L, R = spec.render(0), spec.render(1)
    F, H, W = L.shape
    rect = P.Rectification(spec.rig.as_dict(), True)
    band = 64
    for i in range(args.warmup):
        y0 = (rect.h // 2 + 97 * i) % max(1, rect.h - band)
        cpu_band_step(spec, L, R, rect, y0, y0 + band)
    tot_t, tot_n = 0.0, 0
    for _ in range(args.steps):
        dt, n = cpu_pair_step(spec, L, R, rect)
        tot_t += dt
        tot_n += n
    value = tot_n / tot_t / 1e6
    cores = cpu_threads()
    res = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(tot_t / args.steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene renderer)",
           "config": workload_config(W, H, F, rect.w, rect.h, 2 * L.nbytes), "impl": "reference",
           "points_per_pair": tot_n // max(1, args.steps),
           "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": "each timed step: one whole pair, every stage incl. SOR/MLS/Gaussian "
                                      "(warm-up steps: one 64-row band each); the restatement is pinned to the "
                                      "reference's own code by the CPU tests"},
           "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(res))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--inflight", type=int, default=6,
                    help="pairs in flight: one context and one stream each, round-robin (1: one stream)")
    ap.add_argument("--no-diff", action="store_true", help="skip the forward/adjoint leg (8 planar poses)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched leg (64 mixed pairs)")
    ap.add_argument("--no-refine", action="store_true", help="skip the calibration-refinement leg")
    ap.add_argument("--refine", action="store_true", help="(the refinement leg runs by default)")
    ap.add_argument("--refine-poses", type=int, default=8)
    ap.add_argument("--refine-iters", type=int, default=60)
    ap.add_argument("--width", type=int, default=2448, help="camera width (default: the 5 MP workload)")
    ap.add_argument("--height", type=int, default=2048)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
