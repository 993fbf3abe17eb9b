"""Benchmark: forward + adjoint events/s on one GB300 (batched FP32).

Workload (one "step" = one misfit + gradient evaluation): 256 events on one
128 x 128 x 64 grid, h = 0.5 km, velocity rising linearly 4 -> 8 km/s with
depth times a +-5% checkerboard of 8-cell blocks; sources uniform in the
volume, 100 stations uniform on the top surface; observed times from a
+2%-noise velocity model.  Inputs are seeded synthetic data (the reference
ships no dataset).  Each step: FP32 forward sweeps for all events, trilinear
sampling + weighted misfit, FP32 adjoint sweeps, FP64 gradient summed over
events.

  value : events/s with inputs resident in HBM (CUDA events on the plan's
          stream around K graph launches)
  e2e   : events/s through adt_batch_run with host buffers (H2D of the
          slowness and picks, D2H of misfit, predicted times, gradient and
          status inside the timed region)
  --impl reference : the reference's CPU algorithm (the oracle port of
          Eikonal3D.cpp, all host threads) on a bounded sample of events.

Under torchrun each rank runs the full 256-event workload on its own GPU
(weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "adtomo.jl_gb300"))
sys.path.insert(0, ROOT)

METRIC = "fwd+adjoint events/s on 1 GB300: batched FP32 vs plain FP64, ≤1e-4 rel error"
M, N, L, H = 128, 128, 64, 0.5
N_EVENTS, N_STA = 256, 100
SEED = 0
BYTES_PER_FWD_UPDATE = 12  # FP32: read u, read f, write u per cell-update
BYTES_PER_ADJ_UPDATE = 14  # FP32: read u, read code (2 B), read and write lambda


def workload():
    from adtomo_gb300 import synth
    rng = np.random.default_rng(SEED)
    f = synth.layered_checkerboard(M, N, L, block=8)
    sta = synth.surface_stations(M, N, N_STA, rng)
    src = synth.volume_sources(M, N, L, N_EVENTS, rng)
    f_obs = f / (1.0 + 0.02 * rng.standard_normal(f.shape))
    w = np.ones(N_EVENTS * N_STA)
    return f, f_obs, sta, src, w


def sample_weights(sta, m=M, n=N, l=L):
    """Node indices and trilinear weights of each station (scripts/inversion.jl:64-95:
    floor/ceil per axis, weight 1 on an axis where they agree), for the host-side
    misfit of the plain single-event path."""
    idx = np.zeros((len(sta), 8), np.int64)
    wt = np.zeros((len(sta), 8))
    for q, (x, y, z) in enumerate(sta):
        xi = (int(np.floor(x)), int(np.ceil(x)))
        yi = (int(np.floor(y)), int(np.ceil(y)))
        zi = (int(np.floor(z)), int(np.ceil(z)))
        xw = (1.0, 0.0) if xi[0] == xi[1] else (xi[1] - x, x - xi[0])
        yw = (1.0, 0.0) if yi[0] == yi[1] else (yi[1] - y, y - yi[0])
        zw = (1.0, 0.0) if zi[0] == zi[1] else (zi[1] - z, z - zi[0])
        c = 0
        for a in range(2):
            for b in range(2):
                for d in range(2):
                    idx[q, c] = (xi[a] * n + yi[b]) * l + zi[d]
                    wt[q, c] = xw[a] * yw[b] * zw[d]
                    c += 1
    return idx, wt


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 7:
                    continue
                try:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        finally:
            os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons)}


def oracle_picks(k):
    """Observed times of the first k events: the reference's FP64 op (the
    oracle port, tol 1e-6, 20-iteration cap) on the +2%-noise model, sampled at
    the stations.  The same bits as the GPU arm's picks, which come from the
    library's FP64 plan with the reference stopping rule (bit-exact to the
    oracle).  Untimed setup of the CPU legs."""
    from oracle import oracle as O
    f, f_obs, sta, src, w = workload()
    threads = os.cpu_count() or 1
    _, tp, _, _ = O.batch_misfit_grad([(f_obs, H)], [sta], np.zeros(k, np.int32), src[:k],
                                      np.full(k * N_STA, 1.0), w[:k * N_STA], tol=1e-6,
                                      max_iter=20, nthreads=threads)
    return tp


def cpu_events_per_s(sample_events, threads, t_obs):
    """The oracle port of the reference's CPU op on a bounded sample, with the
    given picks (t_obs of the first sample_events events).  Returns
    (events/s, seconds, (misfit, t_pred, grad))."""
    from oracle import oracle as O
    f, f_obs, sta, src, w = workload()
    k = sample_events
    t0 = time.perf_counter()
    mis, tp, (g,), _ = O.batch_misfit_grad([(f, H)], [sta], np.zeros(k, np.int32), src[:k],
                                           t_obs[:k * N_STA], w[:k * N_STA], tol=1e-6,
                                           max_iter=20, nthreads=threads)
    dt = time.perf_counter() - t0
    return k / dt, dt, (mis, tp, g)


def plain_fp64_events_per_s(k, t_obs):
    """The plain FP64 single-event GPU path on the same workload: one event
    per call (adt_eikonal_three_d, then adt_eikonal_three_d_grad), no
    batching, no graph.  u0 (scripts/gene_obs.jl:42-51's near-source rule, in
    NumPy) and the stations' trilinear weights are built before the timer;
    inside it only the two library calls and the host-side misfit seeds (a
    NumPy gather and scatter).  Picks t_obs as in the batched legs."""
    import adtomo_gb300 as A
    f, f_obs, sta, src, w = workload()
    idx, wt = sample_weights(sta)
    u0s = []
    for e in range(k):
        u0 = np.full(M * N * L, 1000.0)
        xs = (int(np.ceil(src[e, 0])), int(np.floor(src[e, 0])))
        ys = (int(np.ceil(src[e, 1])), int(np.floor(src[e, 1])))
        zs = (int(np.ceil(src[e, 2])), int(np.floor(src[e, 2])))
        fcol = f[xs[0], ys[0]]
        for a in xs:
            for b in ys:
                for c in zs:
                    r = np.sqrt((src[e, 0] - a) ** 2 + (src[e, 1] - b) ** 2 + (src[e, 2] - c) ** 2)
                    u0[(a * N + b) * L + c] = r * fcol[c] * H
        u0s.append(u0.reshape(M, N, L))
    t0 = time.perf_counter()
    for e in range(k):
        u = A.eikonal3d(u0s[e], f, H, M, N, L, 1e-6)
        t = (u.ravel()[idx] * wt).sum(axis=1)
        dt = -2.0 * w[e * N_STA:(e + 1) * N_STA] * (t_obs[e * N_STA:(e + 1) * N_STA] - t)
        gu = np.bincount(idx.ravel(), weights=(dt[:, None] * wt).ravel(), minlength=M * N * L)
        A.eikonal3d_grad(gu.reshape(M, N, L), u, u0s[e], f, H, M, N, L)
    dt = time.perf_counter() - t0
    return k / dt, dt


def gpu_picks(A):
    """Observed times of all events on the GPU: the library's FP64 plan with
    the reference stopping rule (tol 1e-6, 20 iterations; bit-exact to the
    reference's op) on the +2%-noise model.  Untimed setup."""
    f, f_obs, sta, src, w = workload()
    P = A.Batch3D([(M, N, L, H)], [sta], np.zeros(N_EVENTS, np.int32), src, precision=A.ADT_F64,
                  tol=1e-6, ref_compat=True)
    _, tp, _, _ = P.run([f_obs], np.full(N_EVENTS * N_STA, 1.0), w)
    P.close()
    return tp


def fp64_batched_events_per_s(A, t_obs, steps=1, adj_solver="auto"):
    """The same batched plan in FP64 (exact brick skipping, tol 1e-6, the same
    adjoint solver): the yardstick the FP32 path is measured against.  CUDA
    events around `steps` evaluations after one warm-up."""
    import torch
    f, f_obs, sta, src, w = workload()
    P = A.Batch3D([(M, N, L, H)], [sta], np.zeros(N_EVENTS, np.int32), src, precision=A.ADT_F64,
                  tol=1e-6, adj_solver=adj_solver)
    P.upload([f], t_obs, w)
    P.run_resident()
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(P.stream())
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(steps):
            P.run_resident()
        end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / steps
    st = P.stats()
    P.close()
    return N_EVENTS / (ms / 1000.0), ms, st


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = max(threads, 16)
    t_obs = oracle_picks(sample)  # untimed setup: the same picks as the GPU arm's
    for _ in range(args.warmup):
        cpu_events_per_s(min(sample, threads), threads, t_obs)
    vals, total = [], 0.0
    for _ in range(args.steps):
        v, dt, _ = cpu_events_per_s(sample, threads, t_obs)
        vals.append(v)
        total += dt
    value = sample * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "C3: 256 events on 128x128x64, h=0.5 km, layered+checkerboard, "
                               "100 surface stations", "sample_events_per_step": sample,
                   "picks": "FP64 travel times on the +2%-noise model (reference stopping rule), "
                            "the same bits as the GPU arm's"},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of the 256 events per step (oracle/eikonal_oracle.c, "
                                   f"FP64, tol 1e-6, 20-iteration cap, {threads} threads)"},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import torch
    import adtomo_gb300 as A

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    f, f_obs, sta, src, w = workload()
    sf = np.zeros(N_EVENTS, np.int32)
    # observed times: FP64 on the +2% noise model, reference stopping rule (setup, untimed)
    t_obs = gpu_picks(A)
    B = A.Batch3D([(M, N, L, H)], [sta], sf, src, precision=A.ADT_F32, tol=args.tol, bk=args.bk,
                  warps=args.warps, groups=args.groups, wake_tol=args.wake_tol,
                  adj_wake_tol=args.adj_wake_tol, fwd_order_filter=bool(args.fwd_order_filter),
                  adj_warps=args.adj_warps, adj_groups=args.adj_groups,
                  adj_solver=args.adj_solver)
    B.upload([f], t_obs, w)
    if args.autotune and not (args.warps or args.groups or args.adj_warps or args.adj_groups):
        B.autotune(reps=2)  # launch shapes (and adjoint solver) timed on this workload, untimed
    solver_used = "causal" if B.stats().adj_solver == A.ADT_ADJ_CAUSAL else "sweeps"
    stream = torch.cuda.ExternalStream(B.stream())
    for _ in range(args.warmup):
        B.run_resident()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fwd_ms, adj_ms, upd_f, upd_a = [], [], [], []
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(args.steps):
                B.run_resident()
            end.record(stream)
        torch.cuda.synchronize()
        ms = start.elapsed_time(end)
        st = B.stats()  # in-graph events of the last step
        fwd_ms.append(st.fwd_ms)
        adj_ms.append(st.adj_ms)
        upd_f.append(st.fwd_cell_updates)
        upd_a.append(st.adj_cell_updates)
        # end to end through the C ABI with host buffers in pinned memory
        def pinned(a):
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        f_h, tobs_h, w_h = pinned(f), pinned(t_obs), pinned(w)
        out_h = (torch.empty(N_EVENTS * N_STA, dtype=torch.float64, pin_memory=True).numpy(),
                 torch.empty(M * N * L, dtype=torch.float64, pin_memory=True).numpy())
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            mis, tp, grads, status = B.run([f_h], tobs_h, w_h, out=out_h)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
    clocks = clk.summary()
    vs_exact = None
    if rank == 0 and (args.wake_tol > 0 or args.adj_wake_tol > 0):
        # untimed: the same evaluation with exact brick skipping, as the yardstick of
        # what the wake tolerances changed
        E = A.Batch3D([(M, N, L, H)], [sta], sf, src, precision=A.ADT_F32, tol=1e-6,
                      adj_solver=solver_used)
        _, tp_x, g_x, _ = E.run([f], t_obs, w)
        E.close()
        vs_exact = {"t_pred_max_rel": float(np.max(np.abs(tp - tp_x) / np.abs(tp_x))),
                    "grad_rel_l2": float(np.linalg.norm(grads[0] - g_x[0]) /
                                         np.linalg.norm(g_x[0]))}
    t = torch.tensor([ms, e2e_s * 1000.0], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms, e2e_ms = float(t[0]), float(t[1])
    if rank != 0:
        return
    ms_step = ms / args.steps
    value = N_EVENTS * world / (ms_step / 1000.0)
    e2e_val = N_EVENTS * world / (e2e_ms / 1000.0 / args.steps)
    peak, peak_kind = peaks()
    traffic = {}
    prof = os.path.join(ROOT, "profiles", "k_batch_sweeps_c3_dram_traffic.json")
    if os.path.exists(prof) and N_EVENTS == 256:
        try:
            d = json.load(open(prof))
            traffic = {k: d[k]["traffic_bytes_per_launch"] for k in d if k.startswith("k_batch_")}
        except (OSError, ValueError, KeyError):
            traffic = {}
    kern = {
        "k_batch_fwd": {"launch_ms": fwd_ms[-1], "cell_updates": int(upd_f[-1]),
                        "bytes_per_update": BYTES_PER_FWD_UPDATE},
        ("k_batch_adj_causal" if solver_used == "causal" else "k_batch_adj"): {
            "launch_ms": adj_ms[-1], "cell_updates": int(upd_a[-1]),
            "bytes_per_update": BYTES_PER_ADJ_UPDATE},
    }
    for k, v in kern.items():
        v["achieved_GBs"] = v["cell_updates"] * v["bytes_per_update"] / (v["launch_ms"] / 1e3) / 1e9
        v["traffic"] = traffic.get(k)
    dom = max(kern, key=lambda k: kern[k]["launch_ms"])
    other = [k for k in kern if k != dom][0]
    achieved = kern[dom]["achieved_GBs"]
    n_obs = N_EVENTS * N_STA
    h2d = M * N * L * 8 + 2 * n_obs * 8
    d2h = 8 + n_obs * 8 + M * N * L * 8 + N_EVENTS * 24
    threads = os.cpu_count() or 1
    cpu_sample = max(threads, 16) if args.cpu_sample is None else args.cpu_sample
    cpu_sample = min(cpu_sample, N_EVENTS)
    cpu_val, cpu_dt, cpu_out = (cpu_events_per_s(cpu_sample, threads, t_obs) if cpu_sample > 0
                                else (None, 0.0, None))
    err64 = None
    if cpu_out is not None:
        # FP32 error against the reference's FP64 op on the CPU sample: the same
        # events, picks and options as the headline plan (untimed)
        k = cpu_sample
        E = A.Batch3D([(M, N, L, H)], [sta], np.zeros(k, np.int32), src[:k], precision=A.ADT_F32,
                      tol=args.tol, wake_tol=args.wake_tol, adj_wake_tol=args.adj_wake_tol,
                      fwd_order_filter=bool(args.fwd_order_filter), adj_solver=solver_used)
        mis_k, tp_k, (g_k,), _ = E.run([f], t_obs[:k * N_STA], w[:k * N_STA])
        E.close()
        mo, tpo, go = cpu_out
        err64 = {"sample": f"first {k} events, all {N_STA} stations",
                 "reference": "oracle port of Eikonal3D.cpp (FP64, tol 1e-6, 20-iteration cap, "
                              "exact causal adjoint)",
                 "t_pred_max_rel": float(np.max(np.abs(tp_k - tpo) / np.abs(tpo))),
                 "t_pred_max_rel_in_headline_run": float(np.max(np.abs(tp[:k * N_STA] - tpo) /
                                                               np.abs(tpo))),
                 "misfit_rel": float(abs(mis_k - mo) / abs(mo)),
                 "grad_rel_l2": float(np.linalg.norm(g_k - go) / np.linalg.norm(go)),
                 "grad_max_abs_rel": float(np.max(np.abs(g_k - go)) / np.max(np.abs(go))),
                 "tolerances": {"t_pred": 1e-4, "grad": 1e-3}}
    iters = [s.iters for s in status]
    plain_val, plain_dt = (plain_fp64_events_per_s(args.plain_sample, t_obs)
                           if args.plain_sample > 0 else (None, 0.0))
    f64b = None
    if args.fp64_batched:
        v64, ms64, st64 = fp64_batched_events_per_s(A, t_obs, adj_solver=args.adj_solver)
        f64b = {"value": v64, "unit": "events/s", "ms_per_evaluation": ms64,
                "fwd_ms": st64.fwd_ms, "adj_ms": st64.adj_ms,
                "cell_updates": int(st64.fwd_cell_updates + st64.adj_cell_updates),
                "fp32_over_fp64": value / world / v64,
                "what": "the same batched plan in FP64 (tol 1e-6, exact brick skipping in "
                        f"the forward, adjoint solver '{args.adj_solver}': causal order in FP64 "
                        "unless 'sweeps'), 256 events, one evaluation after a warm-up, "
                        "CUDA events"}
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered+checkerboard model)",
        "config": {"workload": "C3: 256 events on 128x128x64, h=0.5 km, layered 4-8 km/s x "
                               "(1+-5%) 8-cell checkerboard, 100 surface stations, misfit + "
                               "summed slowness gradient",
                   "events_per_gpu": N_EVENTS, "grid": [M, N, L], "l2": "inputs larger than L2 "
                   "(1 GB of travel times + 1 GB of adjoint variables per step)",
                   "bk": st.bk, "warps_per_solve": st.warps, "solves_per_cta": st.groups,
                   "adjoint_warps_per_solve": st.adj_warps, "adjoint_solves_per_cta": st.adj_groups,
                   "shapes": "autotuned" if args.autotune and not (args.warps or args.groups or
                                                                args.adj_warps or args.adj_groups)
                   else "fixed",
                   "ctas": st.ctas,
                   "fwd_iters_mean": float(np.mean(iters)),
                   "adj_iters_mean": float(np.mean([s.adj_iters for s in status])),
                   "tol": args.tol, "wake_tol": args.wake_tol, "adj_wake_tol": args.adj_wake_tol,
                   "fwd_order_filter": args.fwd_order_filter, "adj_solver": args.adj_solver,
                   "adj_solver_used": solver_used,
                   "picks": "FP64 travel times on the +2%-noise model (reference stopping rule)",
                   "vs_exact_skipping": vs_exact, "error_vs_fp64": err64},
        "e2e": {"value": e2e_val, "unit": "events/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": kern[dom]["traffic"], "kernel": dom,
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "bytes_per_update": kern[dom]["bytes_per_update"],
                     "cell_updates_per_launch": kern[dom]["cell_updates"],
                     "launch_ms": kern[dom]["launch_ms"], other: kern[other]},
        "cell_updates_per_s": (upd_f[-1] + upd_a[-1]) / (ms_step / 1000.0),
        "cpu_baseline": ({"value": cpu_val, "unit": "events/s", "cores": threads, "kind": "port",
                          "sample": f"{cpu_sample} of the 256 events (oracle port of "
                                    f"Eikonal3D.cpp, FP64, tol 1e-6, 20-iteration cap), "
                                    f"{cpu_dt:.1f} s"} if cpu_val else None),
        "plain_fp64": ({"value": plain_val, "unit": "events/s",
                        "sample": f"{args.plain_sample} events, one per call through "
                                  f"adt_eikonal_three_d + adt_eikonal_three_d_grad (FP64, "
                                  f"host buffers), {plain_dt:.2f} s"} if plain_val else None),
        "fp64_batched": f64b,
        "clocks": clocks,
        # per evaluation of the one-field, one-chunk plan: k_to_t_f32, k_src_init,
        # k_batch_fwd, k_batch_misfit, k_batch_adj or k_batch_adj_causal, k_batch_grad, k_grad_scale,
        # k_misfit_sum, k_order_by_cost
        "gpu_launches": 9 * args.steps,
    }
    B.close()
    if args.secondary:
        line["secondary"] = secondary_results(args)
    print(json.dumps(line), flush=True)


def secondary_results(args):
    """The other configurations, measured after the headline (outside its
    timed region) so that one default run covers them: C1 and C2 (the plain
    FP64 ops, one event, host buffers, against the oracle port on one core,
    with parity), C4 (the uneven P/S batch, adjoint solver chosen by the
    autotuner) and one C5 evaluation (2000 events in 128-event chunks, the
    shapes the autotuner picks there).  The inversions take minutes:
    --workload c5inv / inversion."""
    import copy
    out = {}
    for wl, steps, warmup in (("c1", 10, 2), ("c2", 3, 1)):
        a = copy.copy(args)
        a.workload, a.steps, a.warmup = wl, steps, warmup
        r = run_single(a, emit=False)
        out[wl] = {"workload": r["config"]["workload"], "gpu_ms_per_event": r["value"],
                   "cpu_ms_per_event": r["cpu_baseline"]["value"], "parity": r["parity"]}
    for wl, steps, shapes in (("c4", 3, None), ("c5", 1, (12, 1, 32))):
        a = copy.copy(args)
        a.workload, a.steps, a.warmup = wl, steps, 1
        if shapes:  # C5: the shapes the autotuner picks there (forward 12 x 1, causal 32)
            a.autotune = 0
            a.warps, a.groups, a.adj_warps, a.adj_groups = shapes[0], shapes[1], shapes[2], 0
        r = run_large(a, emit=False)
        c = r["config"]
        out[wl] = {"workload": c["workload"], "solves_per_s": r["value"],
                   "ms_per_evaluation": r["ms_per_step"], "fwd_ms": c["fwd_ms"],
                   "adj_ms": c["adj_ms"], "adj_solver_used": c["adj_solver_used"],
                   "shapes": c["shapes"], "autotuned": bool(a.autotune),
                   "all_converged": c["all_converged"]}
    return out


def large_workload(name, rng):
    """The uneven P/S batch (C4) and the inversion-scale grid (C5)."""
    from adtomo_gb300 import synth
    if name == "c4":
        fields, stations, slow, sf, src = [], [], [], [], []
        for gi, (m, n, l) in enumerate([(64, 64, 32), (96, 96, 48), (128, 128, 64), (160, 160, 80)]):
            vp = synth.layered_smooth(m, n, l, rng)
            sta = synth.surface_stations(m, n, 150, rng)
            for v in (vp, vp / 1.73):
                fields.append((m, n, l, 0.5))
                slow.append(1.0 / v)
                stations.append(sta)
            for e in synth.volume_sources(m, n, l, 128, rng):
                for ph in range(2):
                    sf.append(2 * gi + ph)
                    src.append(e)
        desc = ("C4: 512 events on grids 64x64x32, 96x96x48, 128x128x64, 160x160x80 (h=0.5 km), "
                "P and S fields each (Vp layered 4-8 km/s x (1+-5%) smooth, Vs = Vp/1.73), "
                "1024 solves, 150 surface stations per grid, gradients wrt all 8 slownesses")
        return fields, stations, slow, np.array(sf, np.int32), np.array(src), 0, desc
    m, n, l = 256, 256, 128
    f = synth.layered_checkerboard(m, n, l, block=8)
    sta = synth.surface_stations(m, n, 300, rng)
    src = synth.volume_sources(m, n, l, 2000, rng)
    desc = ("C5: 2000 events on 256x256x128, h=0.25 km, layered+checkerboard, 300 surface "
            "stations, forward fields recomputed per 128-event chunk")
    return [(m, n, l, 0.25)], [sta], [f], np.zeros(2000, np.int32), src, 128, desc


def run_large(args, emit=True):
    """Secondary lines for the larger configurations (not the headline);
    returns the line (printed when emit)."""
    import torch
    import adtomo_gb300 as A
    rng = np.random.default_rng(SEED)
    fields, stations, slow, sf, src, chunk, desc = large_workload(args.workload, rng)
    B = A.Batch3D(fields, stations, sf, src, precision=A.ADT_F32, tol=1e-6, chunk=chunk,
                  wake_tol=args.wake_tol, adj_wake_tol=args.adj_wake_tol,
                  overlap_chunks=bool(args.overlap_chunks), warps=args.warps, groups=args.groups,
                  adj_warps=args.adj_warps, adj_groups=args.adj_groups,
                  adj_solver=args.adj_solver)
    n_obs = sum(len(stations[f]) for f in sf)
    B.upload(slow, np.full(n_obs, 1.0), np.ones(n_obs))
    B.run_resident()
    _, tp, _, _ = B.download()  # picks from the model itself, then a 2% slower model
    B.upload([s * 1.02 for s in slow], tp, np.ones(n_obs))
    if args.autotune:
        B.autotune(reps=1)
    for _ in range(args.warmup):
        B.run_resident()
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(B.stream())
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(args.steps):
            B.run_resident()
        end.record(stream)
    torch.cuda.synchronize()
    ms_step = start.elapsed_time(end) / args.steps
    mis, tp, grads, status = B.download()
    st = B.stats()
    line = {
        "metric": METRIC, "value": len(sf) / (ms_step / 1000.0), "unit": "solves/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": desc, "solves": int(len(sf)), "chunk": chunk,
                   "overlap_chunks": args.overlap_chunks if chunk else 0,
                   "shapes": {"warps": st.warps, "groups": st.groups, "adj_warps": st.adj_warps,
                              "adj_groups": st.adj_groups},
                   "wake_tol": args.wake_tol, "adj_wake_tol": args.adj_wake_tol,
                   "adj_solver": args.adj_solver,
                   "adj_solver_used": "causal" if st.adj_solver == A.ADT_ADJ_CAUSAL else "sweeps",
                   "fwd_ms": st.fwd_ms, "adj_ms": st.adj_ms,
                   "cell_updates_per_s": (st.fwd_cell_updates + st.adj_cell_updates) /
                   (ms_step / 1000.0),
                   "fwd_iters_mean": float(np.mean([x.iters for x in status])),
                   "adj_iters_mean": float(np.mean([x.adj_iters for x in status])),
                   "all_converged": bool(all(x.converged and x.adj_converged for x in status))},
    }
    if emit:
        print(json.dumps(line), flush=True)
    B.close()
    return line


def run_single(args, emit=True):
    """Secondary lines for the plain FP64 configurations (one event, no
    batching), GPU through the host-pointer API against the oracle port of the
    reference's CPU op on one core, with parity:
      c1: 2D 101x101, h = 1 km, 6 km/s + 3 Gaussian anomalies (+-10%, sigma 8
          cells), 1 interior source, 20 receivers at random nodes, misfit
          against times from a +2%-noise model; 2D stopping rule (1e-8);
      c2: 3D 64x64x32, h = 1 km, layered 4-8 km/s x (1+-5%) checkerboard of
          8-cell blocks, 1 interior source, 50 surface receivers, tol 1e-6,
          20-iteration cap."""
    import adtomo_gb300 as A
    from adtomo_gb300 import synth
    from oracle import oracle as O
    rng = np.random.default_rng(SEED)
    if args.workload == "c1":
        n1 = m1 = 101
        f = 1.0 / synth.gaussian_anomalies_2d(n1, m1, rng)
        f_obs = f / (1.0 + 0.02 * rng.standard_normal(f.shape))
        ix, jx = (int(x) for x in rng.integers(1, m1 - 1, 2))  # 0-based source node
        rx, ry = rng.integers(0, m1, 20), rng.integers(0, n1, 20)
        t_obs = A.eikonal(f_obs, ix + 1, jx + 1, 1.0)[ry, rx]

        def gpu():
            u = A.eikonal(f, ix + 1, jx + 1, 1.0)
            gu = np.zeros_like(u)
            np.add.at(gu, (ry, rx), -2.0 * (t_obs - u[ry, rx]))
            return u, A.eikonal_grad(gu, u, f, ix + 1, jx + 1, 1.0), gu

        def cpu(gu):
            u, _, _ = O.eik2d_forward(f, ix, jx, 1.0)
            return u, O.eik2d_backward(gu, u, f, ix, jx, 1.0)
        desc = ("C1: 2D 101x101, h=1 km, 6 km/s + 3 Gaussian anomalies (+-10%, sigma 8 cells), "
                "1 interior source, 20 receivers, +2%-noise picks, stopping rule 1e-8")
    else:
        m, n, l, h = 64, 64, 32, 1.0
        f = synth.layered_checkerboard(m, n, l, block=8)
        src = synth.volume_sources(m, n, l, 1, rng)[0]
        sta = synth.surface_stations(m, n, 50, rng)
        idx, wt = sample_weights(sta, m, n, l)
        f_obs = f * (1 + 0.02 * rng.standard_normal(f.shape))
        u0 = O.src_u0(f, h, src)
        uo = A.eikonal3d(O.src_u0(f_obs, h, src), f_obs, h, m, n, l, 1e-6)
        t_obs = (uo.ravel()[idx] * wt).sum(axis=1)

        def seeds(u):
            t = (u.ravel()[idx] * wt).sum(axis=1)
            dt = -2.0 * (t_obs - t)
            return np.bincount(idx.ravel(), weights=(dt[:, None] * wt).ravel(),
                               minlength=m * n * l).reshape(m, n, l)

        def gpu():
            u = A.eikonal3d(u0, f, h, m, n, l, 1e-6)
            gu = seeds(u)
            return u, A.eikonal3d_grad(gu, u, u0, f, h, m, n, l)[1], gu

        def cpu(gu):
            u, _, _ = O.eik3d_forward(u0, f, h, 1e-6)
            return u, O.eik3d_backward(gu, u, u0, f, h)[1]
        desc = ("C2: 3D 64x64x32, h=1 km, layered 4-8 km/s x (1+-5%) checkerboard, 1 interior "
                "source, 50 surface receivers, +2%-noise picks, tol 1e-6, 20-iteration cap")
    for _ in range(args.warmup):
        gpu()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        u, gf, gu = gpu()
    gpu_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    reps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(reps):
        ur, rf = cpu(gu)
    cpu_ms = (time.perf_counter() - t0) * 1000.0 / reps
    line = {
        "metric": "plain FP64 forward + adjoint, time per event (host buffers)",
        "value": gpu_ms, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": desc},
        "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": 1, "kind": "port",
                         "sample": f"the same event, {reps} repetitions (oracle port, FP64)"},
        "parity": {"forward_bit_identical": bool(np.array_equal(u, ur)),
                   "grad_max_rel": float(np.max(np.abs(gf - rf)) / np.max(np.abs(rf)))},
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_inversion(args):
    """10 L-BFGS iterations of the inversion driver in FP32 and in FP64 on the
    C3 grid, stations as sources (scripts/inversion.jl): time per iteration
    and the FP32 model's distance from the FP64 one (secondary line)."""
    import torch  # noqa: F401  (CUDA context through the library)
    import adtomo_gb300 as A
    from adtomo_gb300 import synth
    from adtomo_gb300.inversion import TravelTimeInversion
    rng = np.random.default_rng(SEED)
    f_true = synth.layered_checkerboard(M, N, L, block=8)
    v_true = 1.0 / f_true
    vel0 = np.broadcast_to(v_true.mean(axis=(0, 1), keepdims=True), v_true.shape).copy()
    sta = synth.surface_stations(M, N, N_STA, rng)
    eve = synth.volume_sources(M, N, L, N_EVENTS, rng)
    P = A.Batch3D([(M, N, L, H)], [eve], np.zeros(N_STA, np.int32), sta, precision=A.ADT_F64,
                  tol=1e-9, max_iter=200)
    _, tp, _, _ = P.run([f_true], np.full(N_STA * N_EVENTS, 1.0), np.ones(N_STA * N_EVENTS))
    P.close()
    uobs = tp.reshape(N_STA, N_EVENTS)
    qua = np.ones_like(uobs)
    out = {}
    for name, prec in (("f32", A.ADT_F32), ("f64", A.ADT_F64)):
        inv = TravelTimeInversion((M, N, L, H), vel0, sta, eve, uobs, qua, lambda_p=0.0,
                                  tol=1e-6, max_iter=200, precision=prec)
        t0 = time.perf_counter()
        x, loss, hist = inv.optimize(iterations=args.steps)
        dt = time.perf_counter() - t0
        out[name] = {"x": x, "loss": loss, "hist": hist, "s_per_iter": dt / max(len(hist), 1),
                     "evaluations": inv.evaluations, "v": inv.velocity(x)}
        inv.close()
    dv64 = np.linalg.norm(out["f64"]["v"] - vel0)
    line = {
        "metric": "L-BFGS time per iteration (s) and FP32-vs-FP64 model difference",
        "value": out["f32"]["s_per_iter"], "unit": "s/iteration", "n_gpus": 1,
        "steps": args.steps, "higher_is_better": False, "dtype": "f32",
        "data": "synthetic (seeded): true layered+checkerboard, start = its depth average",
        "config": {"workload": f"inversion: 128x128x64, h=0.5 km, {N_STA} stations as sources, "
                               f"{N_EVENTS} events as receivers, {args.steps} L-BFGS iterations",
                   "f32_s_per_iteration": out["f32"]["s_per_iter"],
                   "f64_s_per_iteration": out["f64"]["s_per_iter"],
                   "f32_evaluations": out["f32"]["evaluations"],
                   "f64_evaluations": out["f64"]["evaluations"],
                   "f32_loss": out["f32"]["hist"], "f64_loss": out["f64"]["hist"],
                   "model_update_rel_diff": float(np.linalg.norm(out["f32"]["v"] - out["f64"]["v"])
                                                  / max(dv64, 1e-300)),
                   "model_error_f32": float(np.linalg.norm(out["f32"]["v"] - v_true) /
                                            np.linalg.norm(vel0 - v_true)),
                   "model_error_f64": float(np.linalg.norm(out["f64"]["v"] - v_true) /
                                            np.linalg.norm(vel0 - v_true))},
    }
    print(json.dumps(line), flush=True)


def run_c5_inversion(args):
    """The inversion-scale configuration as specified: 10 L-BFGS iterations of
    the inversion driver (scripts/inversion.jl around src/mpi_optimize.jl) on
    256x256x128, h = 0.25 km, 2000 events uniform in the volume and 300
    surface stations on the layered+checkerboard model, FP32, forward fields
    recomputed per 128-event chunk.  By reciprocity the events are the sources
    (2000 solves in chunks of 128) and the stations the receivers.  Picks come
    from the true model through the same plan (gene_obs.jl's near-source rule);
    the inversion starts from the true model's depth average and builds u0
    from it (inversion.jl's rule).  Reported: seconds per L-BFGS iteration,
    the loss history and the model error against the true model; then the
    FP32 run against the FP64 run on a stated reduction (the first
    --c5-fp64-events events, --c5-fp64-iters iterations): relative difference
    of the model updates."""
    import torch  # noqa: F401  (CUDA context through the library)
    import adtomo_gb300 as A
    from adtomo_gb300 import synth
    from adtomo_gb300.inversion import TravelTimeInversion
    rng = np.random.default_rng(SEED)
    m, n, l, h = 256, 256, 128, 0.25
    n_eve, n_sta, chunk = 2000, 300, 128
    f_true = synth.layered_checkerboard(m, n, l, block=8)
    v_true = 1.0 / f_true
    vel0 = np.broadcast_to(v_true.mean(axis=(0, 1), keepdims=True), v_true.shape).copy()
    sta = synth.surface_stations(m, n, n_sta, rng)
    eve = synth.volume_sources(m, n, l, n_eve, rng)
    opts = dict(tol=1e-6, max_iter=200, wake_tol=args.wake_tol, adj_wake_tol=args.adj_wake_tol,
                chunk=chunk, overlap_chunks=bool(args.overlap_chunks), adj_solver=args.adj_solver)
    t0 = time.perf_counter()
    P = A.Batch3D([(m, n, l, h)], [sta], np.zeros(n_eve, np.int32), eve, precision=A.ADT_F32,
                  **opts)
    _, tp, _, _ = P.run([f_true], np.full(n_eve * n_sta, 1.0), np.ones(n_eve * n_sta))
    P.close()
    picks_s = time.perf_counter() - t0
    uobs = tp.reshape(n_eve, n_sta)
    qua = np.ones_like(uobs)

    def invert(k_eve, iters, prec):
        inv = TravelTimeInversion((m, n, l, h), vel0, eve[:k_eve], sta, uobs[:k_eve], qua[:k_eve],
                                  lambda_p=0.0, precision=prec, autotune=1 if args.autotune else 0,
                                  **opts)
        t1 = time.perf_counter()
        x, loss, hist = inv.optimize(iterations=iters)
        dt = time.perf_counter() - t1
        v = inv.velocity(x)
        out = {"s": dt, "hist": hist, "evaluations": inv.evaluations, "v": v}
        inv.close()
        return out

    full = invert(n_eve, args.steps, A.ADT_F32)
    k64, it64 = args.c5_fp64_events, args.c5_fp64_iters
    r32 = invert(k64, it64, A.ADT_F32) if k64 > 0 else None
    r64 = invert(k64, it64, A.ADT_F64) if k64 > 0 else None
    err0 = np.linalg.norm(vel0 - v_true)
    line = {
        "metric": "C5 L-BFGS time per iteration (s), FP32, 2000 events in 128-event chunks",
        "value": full["s"] / max(len(full["hist"]), 1), "unit": "s/iteration", "n_gpus": 1,
        "steps": args.steps, "higher_is_better": False, "dtype": "f32",
        "data": "synthetic (seeded): true layered+checkerboard, start = its depth average",
        "config": {"workload": "C5: 256x256x128, h=0.25 km, 2000 events (sources, 128-event "
                               "chunks, forward recomputed per chunk) and 300 surface stations, "
                               f"{args.steps} L-BFGS iterations of the inversion driver",
                   "iterations": len(full["hist"]), "evaluations": full["evaluations"],
                   "seconds_total": full["s"], "picks_setup_s": picks_s,
                   "loss_history": full["hist"],
                   "model_error_rel": float(np.linalg.norm(full["v"] - v_true) / err0),
                   "tol": 1e-6, "wake_tol": args.wake_tol, "adj_wake_tol": args.adj_wake_tol,
                   "adj_solver": args.adj_solver},
    }
    if r64 is not None:
        dv64 = np.linalg.norm(r64["v"] - vel0)
        line["config"]["vs_fp64"] = {
            "reduction": f"first {k64} events, {it64} L-BFGS iterations (FP64 plan with the "
                         "same options; wake tolerances apply to FP32 only)",
            "model_update_rel_diff": float(np.linalg.norm(r32["v"] - r64["v"]) / max(dv64, 1e-300)),
            "f32_loss": r32["hist"], "f64_loss": r64["hist"],
            "f32_s_per_iteration": r32["s"] / max(len(r32["hist"]), 1),
            "f64_s_per_iteration": r64["s"] / max(len(r64["hist"]), 1)}
    print(json.dumps(line), flush=True)


def main():
    global N_EVENTS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--events", type=int, default=N_EVENTS,
                    help="events per GPU (default 256, the workload; smaller for profiling)")
    ap.add_argument("--bk", type=int, default=0, help="brick depth (0 = library default)")
    ap.add_argument("--warps", type=int, default=0, help="warps per solve (0 = default)")
    ap.add_argument("--groups", type=int, default=0, help="solves per CTA (0 = as many as fit)")
    ap.add_argument("--adj-warps", type=int, default=0, help="adjoint warps per solve (0 = --warps)")
    ap.add_argument("--adj-groups", type=int, default=0,
                    help="adjoint solves per CTA (0 = --groups)")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: time candidate launch shapes on the workload first (untimed setup)")
    ap.add_argument("--workload", default="c3",
                    choices=["c1", "c2", "c3", "c4", "c5", "c5inv", "inversion"],
                    help="c3 (default): the headline; c1, c2: the plain FP64 single-event "
                         "configurations; c4, c5: secondary lines for the larger "
                         "configurations; c5inv: C5's 10 L-BFGS iterations; inversion: the "
                         "inversion driver on the C3 grid, FP32 against FP64")
    ap.add_argument("--tol", type=float, default=1e-6,
                    help="forward stopping tolerance of the FP32 plan (s; default 1e-6)")
    ap.add_argument("--wake-tol", type=float, default=1e-6,
                    help="forward: a brick that moved by at most this (s) wakes no neighbour "
                         "(default 1e-6, the stopping tolerance; 0 = exact skipping)")
    ap.add_argument("--adj-wake-tol", type=float, default=1e-4,
                    help="adjoint: the same for relative changes (default 1e-4; 0 = exact)")
    ap.add_argument("--adj-solver", default="auto", choices=["auto", "sweeps", "causal"],
                    help="adjoint: reverse sweeps until nothing changes, one evaluation per "
                         "cell in reverse causal order, or auto (the library default: causal, "
                         "and in FP32 the autotuner keeps the faster of the two)")
    ap.add_argument("--fwd-order-filter", type=int, default=1,
                    help="1 (library default): FP32 forward sweeps each brick only in the "
                         "orderings that follow its learned upwind directions; 0: all")
    ap.add_argument("--plain-sample", type=int, default=4,
                    help="events timed through the plain FP64 single-event path (0 skips)")
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="events timed for the cpu_baseline and compared for error_vs_fp64 "
                         "(0 skips both)")
    ap.add_argument("--overlap-chunks", type=int, default=1,
                    help="c5, c5inv: 1 keeps two 128-event chunks resident, the next chunk's "
                         "forward beside this chunk's adjoint (0: one chunk at a time)")
    ap.add_argument("--c5-fp64-events", type=int, default=128,
                    help="c5inv: events of the FP32-vs-FP64 comparison (0 skips it)")
    ap.add_argument("--c5-fp64-iters", type=int, default=2,
                    help="c5inv: L-BFGS iterations of the FP32-vs-FP64 comparison")
    ap.add_argument("--secondary", type=int, default=1,
                    help="c3: also measure C1, C2, C4 and C5 after the headline (0 skips)")
    ap.add_argument("--fp64-batched", type=int, default=1,
                    help="1: time the same batched plan in FP64 as a yardstick (untimed leg)")
    args = ap.parse_args()
    N_EVENTS = args.events
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "inversion":
        if rank == 0:
            run_inversion(args)
        return
    if args.workload == "c5inv":
        if rank == 0:
            run_c5_inversion(args)
        return
    if args.workload in ("c1", "c2"):
        if rank == 0:
            run_single(args)
        return
    if args.workload != "c3":
        if rank == 0:
            run_large(args)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    run_ours(args, rank, world)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
