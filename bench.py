"""Benchmark: Biot-Savart node-evals/s of the velocity path on one GB300.

Workload (the reference's FP64 velocity-evaluation configuration): a
65,536-node tangle of 256 closed random-walk loops x 256 nodes (step
0.001 cm, Gaussian turning angle sigma 0.3 rad, seeded Philox), wrapped into
a periodic cube D = 0.1 cm with all 26 periodic images; one step = one
update_tangle (tangents/normals + octree build + fused LIA / Barnes-Hut at
theta 0.4 / mutual friction with alpha 0.098, alpha' 0.016, v_n 0.5 x).

  value  node-evals/s with the tangle resident in HBM (CUDA events per step,
         L2 flushed with a 256 MiB write between steps)
  e2e    node-evals/s through the host C ABI: positions + topology uploaded
         from pinned host memory, velocities downloaded, every step
  mixed  the same workload in the mixed-precision path, with its relative L2
         error against the FP64 tree

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Multi-GPU (torchrun): every rank runs an independent replica (the path does
not shard); value is the sum over ranks of nodes / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "biot_savart_node_evals_per_s"
# DRAM bytes (read + write) of one FP64 traversal launch on this workload, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum of k_vel_fp64, two launches: 9.87 and 9.92 MB)
K_VEL_FP64_DRAM_BYTES = 15.108e6   # k_vel_split: 14.63 MB read + 0.48 MB written (ncu)
UNIT = "node-evals/s"
WORKLOAD = dict(workload="random-walk tangle, 256 loops x 256 nodes (65,536), D=0.1 cm, periodic_26, "
                         "theta=0.4, one update_tangle per step",
                n_loops=256, per_loop=256, D=0.1, delta=1e-3, sigma=0.3, seed=1, theta=0.4, n_images=26)


def make_tangle():
    from openvort_gb300 import workloads as W
    return W.random_walk_tangle(WORKLOAD["n_loops"], WORKLOAD["per_loop"], D=WORKLOAD["D"],
                                delta=WORKLOAD["delta"], sigma=WORKLOAD["sigma"], seed=WORKLOAD["seed"])


def make_params(threads=1):
    from openvort_gb300 import workloads as W
    p = W.config_params("rw", bh_resolution=WORKLOAD["theta"])
    p.num_threads = threads
    return p


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_eval_time(kind: str, threads: int, reps: int, tangle=None, params=None):
    """Seconds per full update_tangle of the workload in the CPU checker."""
    from oracle.pyoracle import Checker
    c = Checker(kind, fast=(kind == "port"))
    if params is None:
        params = make_params(threads)
    params.num_threads = threads
    c.set_params(params)
    ht = tangle or make_tangle()
    times = []
    for _ in range(reps):
        t = c.tangle(ht)
        t0 = time.perf_counter()
        c.update_tangle(t, 0.0)
        times.append(time.perf_counter() - t0)
        t.free()
    return times


def cpu_kind():
    from oracle import pyoracle
    return "reference" if pyoracle.reference_available() else "port"


def port_vs_reference():
    """The restatement's speed over OpenVort's own build at equal threads,
    measured where OpenVort's sources exist (oracle/port_vs_reference.py)."""
    path = os.path.join(ROOT, "oracle", "port_vs_reference.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def cpu_line(value, threads, kind, sample):
    """A cpu_baseline object; for the restatement, with its measured speed
    ratio to OpenVort's own build and the reference rate that implies."""
    out = {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample}
    pvr = port_vs_reference() if kind == "port" else None
    if pvr:
        out["port_over_reference"] = pvr["port_over_reference"]
        out["reference_estimate"] = value / pvr["port_over_reference"]
        out["port_over_reference_measured"] = (f"{pvr['machine']}, {pvr['threads']} threads each: "
                                               f"{pvr['workload']}")
        out["note"] = ("OpenVort's sources are not on this host, so the C restatement runs (bit-identical results); "
                       "it is port_over_reference times faster than OpenVort's own build, so ratios against this "
                       "value understate the speed-up over the reference")
    return out


def run_reference(args):
    world, rank, local, dist = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    kind = cpu_kind()
    ht = make_tangle()
    for _ in range(args.warmup):
        cpu_eval_time(kind, threads, 1, ht)
    times = cpu_eval_time(kind, threads, args.steps, ht)
    n = ht.n
    per = statistics.mean(times)
    value = n / per
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference", "config": WORKLOAD,
        "l2": "inputs rebuilt per step on the host (CPU run)", "parallelism": "host threads",
        "cpu_baseline": cpu_line(value, threads, kind, f"{args.steps} full update_tangle of the 65,536-node tangle"),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


ENSEMBLE = dict(workload="ensemble of 48 independent random-walk tangles, 256-node loops, node counts "
                         "log-uniform in [2048, 131072], D=0.1 cm, periodic_26, theta=0.4; per-member "
                         "alpha~U(0.03,0.3), alpha'~U(0,0.02), v_n~U(0.2,2) x (seeded)",
                n_tangles=48, min_nodes=2048, max_nodes=131072, per_loop=256, D=0.1, seed=11, dt=5e-5)


def run_ensemble(args, device=0):
    """The batching form: every member in one context, one persistent
    traversal launch per evaluation, RK4 as one graph, topology passes per
    member; mixed precision after the autotuner picked the launch shape."""
    from openvort_gb300 import abi, gpu, workloads as W
    E = ENSEMBLE
    ms = W.ensemble(E["n_tangles"], E["min_nodes"], E["max_nodes"], E["per_loop"], D=E["D"], seed=E["seed"])
    hosts = [m.tangle for m in ms]
    params = [W.member_params(m) for m in ms]
    n = sum(h.n for h in hosts)
    ctx = gpu.Context(device, params=params[0], precision=abi.OV_PREC_FP64)
    ctx.upload_ensemble(hosts, params, headroom=2.0)

    def timed_evals(reps):
        ts = []
        for _ in range(reps):
            ctx.flush_l2(256 << 20)
            ctx.timer_start()
            ctx.update_tangle(0.0)
            ts.append(ctx.timer_stop())
        return statistics.mean(ts)

    # FP64 reference evaluation (same launch shape rules, untuned)
    ctx.update_tangle(0.0)
    fp64_ms = timed_evals(2)
    ref = [ctx.download_member(i, W.HostTangle(h.pos.copy(), h.conn[:, 0].copy(), h.conn[:, 1].copy(),
                                               h.box_lo, h.box_hi, n_images=h.n_images)).vels.copy()
           for i, h in enumerate(hosts)]
    # mixed precision, autotuned
    ctx.set_precision(abi.OV_PREC_MIXED)
    tune, tune_ms = ctx.autotune(0.0)
    for _ in range(max(1, args.warmup)):
        ctx.update_tangle(0.0)
    l0 = ctx.kernel_launches
    mixed_ms = timed_evals(max(3, args.steps))
    launches_per_eval = (ctx.kernel_launches - l0 - max(3, args.steps)) / max(3, args.steps)
    st = ctx.stats()
    num = den = 0.0
    for i, h in enumerate(hosts):
        v = ctx.download_member(i, W.HostTangle(h.pos.copy(), h.conn[:, 0].copy(), h.conn[:, 1].copy(),
                                                h.box_lo, h.box_hi, n_images=h.n_images)).vels
        num += float(np.sum((v[:len(ref[i])] - ref[i]) ** 2))
        den += float(np.sum(ref[i] ** 2))
    # RK4 steps/s (update_tangle + rk4_step, all members in one graph)
    dt = E["dt"]
    for w in range(2):
        ctx.update_tangle(w * dt)
        ctx.rk4_step(w * dt, dt)
    ts = []
    for k in range(max(2, args.steps // 2)):
        ctx.timer_start()
        ctx.update_tangle(k * dt)
        ctx.rk4_step(k * dt, dt)
        ts.append(ctx.timer_stop())
    rk4_ms = statistics.mean(ts)
    # full time steps with reconnection and remeshing (host wall clock)
    ctx.upload_ensemble(hosts, params, headroom=2.0)
    K = args.ensemble_steps
    recs = added = 0
    passes = {}
    rstat = {"reconnect_candidates": 0, "reconnect_evaluated": 0, "reconnect_fp64_pairs": 0,
             "reconnect_exact_pairs": 0, "reconnect_lazy_evals": 0}
    t0 = time.perf_counter()
    for k in range(K):
        ctx.step(k * dt, dt)
        s2 = ctx.stats()
        recs += s2["reconnections"]
        added += s2["remesh_added"]
        for key in rstat:
            rstat[key] += s2[key]
        for name, v in ctx.step_times().items():
            passes[name] = passes.get(name, 0.0) + v / K
    ctx.synchronize()
    full_ms = (time.perf_counter() - t0) * 1e3 / max(1, K)
    n_end = sum(ctx.member_info(i)[0] - ctx.member_info(i)[2] for i in range(len(hosts)))
    ctx.close()
    cpu = None
    if args.cpu_sections:
        threads = os.cpu_count() or 1
        cpu_s = sum(min(cpu_eval_time(cpu_kind(), threads, 1, h, p)) for h, p in zip(hosts, params))
        cpu = cpu_line(n / cpu_s, threads, cpu_kind(),
                       "one full update_tangle of every member, members one after another")
    return {
        "cpu_baseline": cpu,
        "config": E, "members": len(hosts), "nodes": n, "nodes_per_member_min_max": [min(h.n for h in hosts),
                                                                                  max(h.n for h in hosts)],
        "tuning": tune, "tuned_eval_ms": tune_ms,
        "mixed": {"value": n / (mixed_ms * 1e-3), "unit": UNIT, "ms_per_eval": mixed_ms,
                  "rel_l2_vs_fp64_tree": (num / den) ** 0.5 if den > 0 else None,
                  "fp64_guard_band_decisions": st["fp64_fallbacks"], "fp64_near_field": st["near_field_fp64"],
                  "kernel_launches_per_eval": launches_per_eval},
        "fp64": {"value": n / (fp64_ms * 1e-3), "unit": UNIT, "ms_per_eval": fp64_ms},
        "mixed_speedup_vs_fp64": fp64_ms / mixed_ms,
        "rk4_mixed": {"steps_per_s": 1e3 / rk4_ms, "ms_per_step": rk4_ms,
                      "node_evals_per_s": 4 * n / (rk4_ms * 1e-3)},
        "full_steps_mixed": {"steps": K, "ms_per_step_wall": full_ms, "steps_per_s": 1e3 / full_ms,
                             "reconnections": recs, "remesh_added": added, "live_nodes_end": n_end,
                             "pass_ms": passes, "reconnect_counts": rstat,
                             "includes": "small loops x3, reconnect, periodic wrap, remesh, update_tangle, "
                                         "rk4_step (graph), per step; host wall clock"},
    }


PRECISION_FORM = dict(workload="random-walk tangle, 1,024 loops x 256 nodes (262,144), D=0.1 cm, periodic_26, "
                               "theta in {0.3, 0.5}", n_loops=1024, per_loop=256, D=0.1, seed=3, thetas=[0.3, 0.5],
                      direct_subsample=8192)
LARGE = dict(workload="random-walk tangle, 4,096 loops x 256 nodes (1,048,576), D=0.2 cm, periodic_26, theta=0.4, "
                      "alpha=0.098, alpha'=0.016, v_n=1.0 x, dt=2e-5, reconnect + remesh + smoothing (cutoff 0.8)",
             n_loops=4096, per_loop=256, D=0.2, seed=5, theta=0.4, dt=2e-5)


def direct_subsample(n, count, seed=0):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(count, n), replace=False))


def eval_ms(ctx, reps):
    ts = []
    for _ in range(reps):
        ctx.flush_l2(256 << 20)
        ctx.timer_start()
        ctx.update_tangle(0.0)
        ts.append(ctx.timer_stop())
    return statistics.mean(ts)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_precision_form(args, device=0):
    """262,144 nodes at theta 0.3 and 0.5: mixed vs FP64 tree, both against
    FP64 direct sums on a node subsample."""
    from openvort_gb300 import abi, gpu, workloads as W
    P = PRECISION_FORM
    ht = W.random_walk_tangle(P["n_loops"], P["per_loop"], D=P["D"], seed=P["seed"])
    n = ht.n
    sub = direct_subsample(n, P["direct_subsample"], 1)
    out = {"config": P, "nodes": n, "by_theta": {}}
    direct = None
    for theta in P["thetas"]:
        ctx = gpu.Context(device, params=W.config_params("rw", bh_resolution=theta), precision=abi.OV_PREC_FP64)
        ctx.upload(ht)
        ctx.update_tangle(0.0)
        if direct is None:
            direct, _ = ctx.direct_velocities(sub)   # FP64 direct sums (tree == NULL branch), tangents current
        fp64_ms = eval_ms(ctx, 2)
        v64 = ctx.download(ht, abi.OV_F_VELS).vels.copy()
        st64 = ctx.stats()
        ctx.set_precision(abi.OV_PREC_MIXED)
        ctx.update_tangle(0.0)
        mixed_ms = eval_ms(ctx, max(3, args.steps))
        v32 = ctx.download(ht, abi.OV_F_VELS).vels.copy()
        st32 = ctx.stats()
        ctx.close()
        cpu_s = None
        if args.cpu_sections:
            threads = os.cpu_count() or 1
            cpu_s = min(cpu_eval_time(cpu_kind(), threads, 1, ht, W.config_params("rw", bh_resolution=theta)))
        out["by_theta"][str(theta)] = {
            "cpu_baseline": None if cpu_s is None else cpu_line(
                n / cpu_s, os.cpu_count() or 1, cpu_kind(), "one full update_tangle of the 262,144-node tangle"),
            "fp64": {"value": n / (fp64_ms * 1e-3), "unit": UNIT, "ms_per_eval": fp64_ms,
                     "rel_l2_vs_direct_subsample": rel_l2(v64[sub], direct)},
            "mixed": {"value": n / (mixed_ms * 1e-3), "unit": UNIT, "ms_per_eval": mixed_ms,
                      "rel_l2_vs_fp64_tree": rel_l2(v32, v64),
                      "rel_l2_vs_direct_subsample": rel_l2(v32[sub], direct),
                      "same_decisions_as_fp64": bool(st32["accepts"] == st64["accepts"]
                                                     and st32["visits"] == st64["visits"])},
            "mixed_speedup_vs_fp64": fp64_ms / mixed_ms,
        }
    return out


def run_large(args, device=0):
    """1,048,576 nodes: mixed-precision RK4 and full time steps with
    reconnection, remeshing and smoothing; FP64 evaluation beside it."""
    from openvort_gb300 import abi, gpu, workloads as W
    E = LARGE
    ht = W.random_walk_tangle(E["n_loops"], E["per_loop"], D=E["D"], seed=E["seed"])
    n = ht.n
    p = W.config_params("large", bh_resolution=E["theta"])
    ctx = gpu.Context(device, params=p, precision=abi.OV_PREC_FP64)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    fp64_ms = eval_ms(ctx, 1)
    v64 = ctx.download(ht, abi.OV_F_VELS).vels.copy()
    ctx.set_precision(abi.OV_PREC_MIXED)
    ctx.upload(ht)
    tune, _ = ctx.autotune(0.0)
    ctx.update_tangle(0.0)
    mixed_ms = eval_ms(ctx, max(3, args.steps))
    v32 = ctx.download(ht, abi.OV_F_VELS).vels.copy()
    ctx.set_phase_timing(True)
    ph = []
    for _ in range(3):
        ctx.flush_l2(256 << 20)
        ctx.update_tangle(0.0)
        ph.append(ctx.phase_times())
    ctx.set_phase_timing(False)
    ph = np.median(np.array(ph), axis=0).tolist()
    dt = E["dt"]
    ctx.upload(ht)
    for w in range(2):
        ctx.update_tangle(w * dt)
        ctx.rk4_step(w * dt, dt)
    ts = []
    for k in range(max(2, args.steps // 2)):
        ctx.timer_start()
        ctx.update_tangle(k * dt)
        ctx.rk4_step(k * dt, dt)
        ts.append(ctx.timer_stop())
    rk4_ms = statistics.mean(ts)
    ctx.upload(ht)
    K = args.large_steps
    passes, recs, added = {}, 0, 0
    rstat = {"reconnect_candidates": 0, "reconnect_evaluated": 0, "reconnect_fp64_pairs": 0,
             "reconnect_exact_pairs": 0, "reconnect_lazy_evals": 0}
    t0 = time.perf_counter()
    for k in range(K):
        ctx.step(k * dt, dt)
        s2 = ctx.stats()
        recs += s2["reconnections"]
        added += s2["remesh_added"]
        for key in rstat:
            rstat[key] += s2[key]
        for name, v in ctx.step_times().items():
            passes[name] = passes.get(name, 0.0) + v / max(1, K)
    ctx.synchronize()
    full_ms = (time.perf_counter() - t0) * 1e3 / max(1, K)
    ctx.close()
    cpu = None
    if args.cpu_sections:
        threads = os.cpu_count() or 1
        cpu_s = min(cpu_eval_time(cpu_kind(), threads, 1, ht, W.config_params("large", bh_resolution=E["theta"])))
        cpu = cpu_line(n / cpu_s, threads, cpu_kind(),
                       "one full update_tangle of the 1,048,576-node tangle (a full step is reconnect-dominated "
                       "and not run on the CPU)")
    return {
        "config": E, "nodes": n, "tuning": tune, "cpu_baseline": cpu,
        "fp64": {"value": n / (fp64_ms * 1e-3), "unit": UNIT, "ms_per_eval": fp64_ms},
        "mixed": {"value": n / (mixed_ms * 1e-3), "unit": UNIT, "ms_per_eval": mixed_ms,
                  "rel_l2_vs_fp64_tree": rel_l2(v32, v64),
                  "phases_ms": {"tangents": ph[0], "tree_build": ph[1], "traversal": ph[2]}},
        "mixed_speedup_vs_fp64": fp64_ms / mixed_ms,
        "rk4_mixed": {"steps_per_s": 1e3 / rk4_ms, "ms_per_step": rk4_ms, "node_evals_per_s": 4 * n / (rk4_ms * 1e-3)},
        "full_steps_mixed": {"steps": K, "ms_per_step_wall": full_ms, "steps_per_s": 1e3 / full_ms if K else None,
                             "reconnections": recs, "remesh_added": added, "pass_ms": passes,
                             "reconnect_counts": rstat},
    }


CONFIG_A = dict(workload="8 vortex rings of radius 0.02 cm (add_loop placement, 62 nodes each, 496 nodes), centres "
                         "uniform and axes uniform on the sphere (seeded), D=0.1 cm, periodic_26, dl_min 1e-3, "
                         "dl_max 3e-3, rec_dist 8e-4, alpha 0.098, alpha' 0.016, v_n 0.5 x, theta 0.4, dt 5e-5, "
                         "200 main-loop steps (small loops, reconnect, periodic wrap, remesh, update_tangle, "
                         "rk4_step); FP64",
                steps=200, dt=5e-5,
                crossing="the same step on 8 pairs of crossing rings (992 nodes; 12 reconnections in 200 steps)")


def run_config_a(args, device=0):
    """The small configuration's full 200-step run: GPU (FP64 path through
    ov_step) and the CPU path on all host cores, steps/s; and the same for
    crossing ring pairs, whose steps reconnect."""
    from openvort_gb300 import abi, gpu, workloads as W
    from oracle.pyoracle import Checker
    A = CONFIG_A
    out = {"config": A}
    for name, ht in (("rings8", W.ring_tangle()), ("crossing_rings", W.crossing_rings())):
        p = W.config_params("rings8")
        ctx = gpu.Context(device, params=p, precision=abi.OV_PREC_FP64)
        ctx.upload(ht)
        tune, _ = ctx.autotune(0.0)              # launch shape for this size (query groups, block shape)
        ctx.upload(ht)
        for w in range(3):                       # warm-up on a copy of the run (graph capture, buffers)
            ctx.step(w * A["dt"], A["dt"])
        ctx.upload(ht)
        recs = 0
        ctx.synchronize()
        t0 = time.perf_counter()
        for k in range(A["steps"]):
            ctx.step(k * A["dt"], A["dt"])
            recs += ctx.stats()["reconnections"]
        ctx.synchronize()
        g_s = time.perf_counter() - t0
        ctx.close()
        sec = {"nodes": ht.n, "steps": A["steps"], "reconnections": recs, "tuning": tune,
               "gpu": {"steps_per_s": A["steps"] / g_s, "ms_per_step": g_s * 1e3 / A["steps"],
                       "timing": "host wall clock around the 200 ov_step calls"}}
        if args.cpu_sections:
            threads = os.cpu_count() or 1
            port = Checker("port", fast=True)
            p.num_threads = threads
            port.set_params(p)
            t = port.tangle(ht)
            t0 = time.perf_counter()
            crecs = sum(port.step(t, k * A["dt"], A["dt"]) for k in range(A["steps"]))
            c_s = time.perf_counter() - t0
            t.free()
            pvr = port_vs_reference()
            sec["cpu_baseline"] = {"steps_per_s": A["steps"] / c_s, "cores": threads, "kind": "port",
                                   "reconnections": crecs, "sample": "the full 200 steps"}
            if pvr:
                sec["cpu_baseline"]["port_over_reference"] = pvr["port_over_reference"]
            sec["gpu_over_cpu"] = c_s / g_s
        out[name] = sec
    return out


def run_next_rows(args, device=0):
    """The rows beside the benchmarked path: mirror walls (wall_2_4) on the
    headline tangle, frame files, injection, and the spherical fork's
    velocity path."""
    import tempfile
    from openvort_gb300 import abi, gpu, workloads as W
    out = {}
    base = make_tangle()
    n = base.n
    hw = W.HostTangle(base.pos.copy(), base.conn[:, 0].copy(), base.conn[:, 1].copy(), base.box_lo, base.box_hi,
                      image_set="wall_2_4")
    ctx = gpu.Context(device, params=make_params(1))
    ctx.upload(hw)
    walls = {"config": "the 65,536-node tangle with mirror walls in z (wall_2_4: 4 periodic images, "
                       "4 reflected; theta 0.4)"}
    res = {}
    for name, prec in (("fp64", abi.OV_PREC_FP64), ("mixed", abi.OV_PREC_MIXED)):
        ctx.set_precision(prec)
        ctx.upload(hw)
        ctx.update_tangle(0.0)
        ms = eval_ms(ctx, max(3, args.steps // 2))
        res[name] = (ms, np.array(ctx.download(hw, abi.OV_F_VELS).vels))
        walls[name] = {"value": n / (ms * 1e-3), "unit": UNIT, "ms_per_eval": ms}
    walls["mixed"]["rel_l2_vs_fp64_tree"] = rel_l2(res["mixed"][1], res["fp64"][1])
    if args.cpu_sections:
        threads = os.cpu_count() or 1
        kind = cpu_kind()
        t = min(cpu_eval_time(kind, threads, 1, hw))
        walls["cpu_baseline"] = cpu_line(n / t, threads, kind, "1 full update_tangle of the wall tangle")
    out["walls"] = walls
    # frames: the reference's text format, host code
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "frame.dat")
        t0 = time.perf_counter()
        gpu.write_frame(base, path, 15)
        tw = time.perf_counter() - t0
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        gpu.read_frame(path, n0=1)
        tr = time.perf_counter() - t0
    out["frames"] = {"nodes": n, "bytes": size, "write_ms": tw * 1e3, "read_ms": tr * 1e3,
                     "write_mb_per_s": size / tw / 1e6, "read_mb_per_s": size / tr / 1e6}
    # injection: one loop and one pinned line pair into the resident wall tangle
    ctx.set_precision(abi.OV_PREC_FP64)
    ctx.upload(hw)
    ctx.set_injection(abi.make_injection(seed=5, loop_frequency=1.0, line_n=1, line_frequency=1.0,
                                         line_polarized=True))
    t0 = time.perf_counter()
    ctx.inject_vortices(2.0)
    ti = time.perf_counter() - t0
    out["injection"] = {"nodes_added": ctx.stats()["injected_nodes"], "ms": ti * 1e3,
                        "includes": "draws, slot allocation with pool growth, push of positions and topology"}
    ctx.close()
    # the spherical fork's update_tangle (tangents + velocities, temperature model on)
    sph = W.spherical_tangle(n_rings=640)
    p = gpu.sph_params_default()
    ctx = gpu.Context(device)
    for _ in range(2):
        ctx.sph_update(sph, p, 0.0)
    ts = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        ctx.sph_update(sph, p, 0.0)
        ts.append(time.perf_counter() - t0)
    st = ctx.stats()
    v64 = sph.vels.copy()
    # the same call in mixed precision
    ctx.set_precision(abi.OV_PREC_MIXED)
    ctx.sph_update(sph, p, 0.0)
    tm = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        ctx.sph_update(sph, p, 0.0)
        tm.append(time.perf_counter() - t0)
    ctx.close()
    live = int((sph.stat[:, 0] != abi.OV_EMPTY).sum())
    free = (sph.stat[:, 0] != abi.OV_EMPTY) & (sph.stat[:, 0] != abi.OV_PINNED)
    sph_cpu = None
    if args.cpu_sections:
        from oracle.pyoracle import sph_update_tangle
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        sph_update_tangle(W.spherical_tangle(n_rings=640), p, threads=threads, fast=True)
        tc = time.perf_counter() - t0
        sph_cpu = {"value": live / tc, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": "one update_tangle of the same tangle in the C restatement of the fork "
                             "(bit-identical to the fork on the committed golden vectors)"}
    ms = statistics.mean(ts) * 1e3
    ms32 = statistics.mean(tm) * 1e3
    out["spherical"] = {
        "config": f"spherical fork's default section (r 0.02..0.1 cm, +-15 deg), {live} nodes: 640 rings + a "
                  "pinned radial line; temperature model on; one update_tangle (tangents, both trees, 18 "
                  "queries per node) per call, through the C ABI with host buffers",
        "value": live / (ms * 1e-3), "unit": UNIT, "ms_per_call": ms, "visits": st["visits"],
        "accepts": st["accepts"],
        "mixed": {"value": live / (ms32 * 1e-3), "unit": UNIT, "ms_per_call": ms32,
                  "rel_l2_vs_fp64_tree": rel_l2(sph.vels[free], v64[free])},
        "cpu_baseline": sph_cpu}
    return out


def run_ours(args):
    from openvort_gb300 import abi, gpu
    world, rank, local, dist = dist_setup()
    device = local if world > 1 else 0
    peaks, peak_src = load_peaks()
    ht = make_tangle()
    n = ht.n
    p = make_params(1)
    ctx = gpu.Context(device, params=p)
    ctx.upload(ht)
    ctx.set_phase_timing(True)

    # ---- value: resident in HBM, CUDA events per step, L2 flushed between steps
    for _ in range(args.warmup):
        ctx.update_tangle(0.0)
    step_ms, trav_ms = [], []
    l0 = ctx.kernel_launches
    barrier(dist)
    ctx.synchronize()
    clk = ClockSampler(device).__enter__()
    for _ in range(args.steps):
        ctx.flush_l2(256 << 20)
        ctx.timer_start()
        ctx.update_tangle(0.0)
        step_ms.append(ctx.timer_stop())
        trav_ms.append(ctx.phase_times())
    ctx.synchronize()
    launches = ctx.kernel_launches - l0 - args.steps     # minus the flush memsets (not kernels of ours)
    barrier(dist)
    st = ctx.stats()
    mean_ms = statistics.mean(step_ms)
    mean_ms = dist_max(dist, mean_ms)
    value = world * n / (mean_ms * 1e-3)
    phases = np.mean(np.array(trav_ms), axis=0).tolist()

    # ---- roofline of the dominant kernel (the FP64 traversal: FMA-pipe bound)
    acc, vis = st["accepts"], st["visits"]
    flops = 42 * acc + 9 * vis   # algorithmic flops per launch (fixed convention, whatever pipe runs them)
    trav_s = phases[2] * 1e-3
    achieved = flops / trav_s / 1e12
    fp64_peak = ctx.fma_peak_tflops(abi.OV_PREC_FP64)
    fp32_peak = ctx.fma_peak_tflops(abi.OV_PREC_MIXED)

    # ---- e2e: host buffers through the C ABI every step
    e2e_ms = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        ctx.upload_fields(ht, abi.OV_F_POS | abi.OV_F_TOPOLOGY)
        ctx.update_tangle(0.0)
        ctx.download(ht, abi.OV_F_VELS)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_mean = dist_max(dist, statistics.mean(e2e_ms))
    h2d = n * (3 * 8 + 4 * 4)
    d2h = n * 3 * 8

    fp64_vels = np.array(ht.vels)   # the FP64 tree's velocities (accuracy check at the end)

    # ---- the FP64 path with every walk test in FP64 (OV_WALK_FP64), for comparison
    walk64 = None
    try:
        ctx.set_walk(abi.OV_WALK_FP64)
        ctx.upload(ht)
        for _ in range(args.warmup):
            ctx.update_tangle(0.0)
        wt, wp = [], []
        for _ in range(args.steps):
            ctx.flush_l2(256 << 20)
            ctx.timer_start()
            ctx.update_tangle(0.0)
            wt.append(ctx.timer_stop())
            wp.append(ctx.phase_times()[2])
        ctx.download(ht, abi.OV_F_VELS)
        wst = ctx.stats()
        per_node = np.linalg.norm(ht.vels - fp64_vels, axis=1) / np.linalg.norm(fp64_vels, axis=1)
        walk64 = {"value": world * n / (statistics.mean(wt) * 1e-3), "unit": UNIT, "ms_per_step": statistics.mean(wt),
                  "traversal_ms": statistics.mean(wp),
                  "split_walk_speedup": statistics.mean(wt) / mean_ms,
                  "same_decisions": bool(wst["accepts"] == st["accepts"] and wst["visits"] == st["visits"]),
                  "max_node_rel_diff": float(per_node.max()),
                  "arithmetic": "every distance and opening test in FP64 with the reference's rounding, each "
                                "accepted cell evaluated where the walk meets it"}
        ctx.set_walk(abi.OV_WALK_SPLIT)
        ctx.upload(ht)
        ctx.update_tangle(0.0)
    except Exception as e:
        walk64 = {"unavailable": str(e)[:200]}

    # ---- mixed precision on the same workload (reported beside FP64)
    mixed = None
    try:
        ctx.set_precision(abi.OV_PREC_MIXED)
        ref_v = np.array(ht.vels)
        ctx.upload(ht)
        for _ in range(args.warmup):
            ctx.update_tangle(0.0)
        mt, mph = [], []
        for _ in range(args.steps):
            ctx.flush_l2(256 << 20)
            ctx.timer_start()
            ctx.update_tangle(0.0)
            mt.append(ctx.timer_stop())
            mph.append(ctx.phase_times()[2])
        ctx.download(ht, abi.OV_F_VELS)
        mst = ctx.stats()
        # the same flop convention on the FP32 pipe (the walk's tests are FP32 here)
        m_achieved = (42 * mst["accepts"] + 9 * mst["visits"]) / (statistics.mean(mph) * 1e-3) / 1e12
        err = float(np.linalg.norm(ht.vels - ref_v) / np.linalg.norm(ref_v))
        mixed_vels = np.array(ht.vels)
        mixed = {"value": world * n / (statistics.mean(mt) * 1e-3), "unit": UNIT,
                 "rel_l2_vs_fp64_tree": err, "ms_per_step": statistics.mean(mt),
                 "speedup_vs_fp64": mean_ms / statistics.mean(mt),
                 "same_decisions_as_fp64": bool(mst["accepts"] == acc and mst["visits"] == vis),
                 "fp64_guard_band_decisions": mst["fp64_fallbacks"], "fp64_near_field": mst["near_field_fp64"],
                 "warp_efficiency": mst["visits"] / max(1, 32 * mst["warp_steps"]),
                 "roofline": {"bound": "issue", "pipe": "fp32", "achieved": m_achieved, "peak": fp32_peak,
                              "unit": "TFLOP/s", "frac": m_achieved / fp32_peak,
                              "traversal_ms": statistics.mean(mph),
                              "work": "42 flops per accepted interaction + 9 per visited cell",
                              "note": "instruction issue and latency bound (the walk), not the FMA pipe"}}
        ctx.set_precision(abi.OV_PREC_FP64)
    except Exception as e:  # mixed path not built yet
        mixed = {"unavailable": str(e)[:200]}

    # ---- double-single interactions (OV_PREC_DD) on the same workload
    dd = None
    try:
        ctx.set_precision(abi.OV_PREC_DD)
        ctx.upload(ht)
        for _ in range(args.warmup):
            ctx.update_tangle(0.0)
        dt_ = []
        for _ in range(args.steps):
            ctx.flush_l2(256 << 20)
            ctx.timer_start()
            ctx.update_tangle(0.0)
            dt_.append(ctx.timer_stop())
        ctx.download(ht, abi.OV_F_VELS)
        dst = ctx.stats()
        per_node = np.linalg.norm(ht.vels - fp64_vels, axis=1) / np.linalg.norm(fp64_vels, axis=1)
        dd = {"value": world * n / (statistics.mean(dt_) * 1e-3), "unit": UNIT, "ms_per_step": statistics.mean(dt_),
              "rel_l2_vs_fp64_tree": rel_l2(ht.vels, fp64_vels), "max_node_rel_err_vs_fp64_tree": float(per_node.max()),
              "speedup_vs_fp64": mean_ms / statistics.mean(dt_),
              "same_decisions_as_fp64": bool(dst["accepts"] == acc and dst["visits"] == vis),
              "arithmetic": "FP32 walk and decisions (FP64 inside guard bands), each accepted interaction and "
                            "the sums in double-single (two floats)"}
        ctx.set_precision(abi.OV_PREC_FP64)
    except Exception as e:
        dd = {"unavailable": str(e)[:200]}

    # ---- RK4 steps/s: update_tangle (k1) + rk4_step (three stages + combine, one CUDA graph)
    rk4 = {}
    for name, prec in (("fp64", abi.OV_PREC_FP64), ("mixed", abi.OV_PREC_MIXED)):
        ctx.set_precision(prec)
        ctx.upload(ht)
        dt = 5e-5
        for w in range(2):
            ctx.update_tangle(w * dt)
            ctx.rk4_step(w * dt, dt)
        ts = []
        for k in range(max(2, args.steps // 2)):
            ctx.flush_l2(256 << 20)
            ctx.timer_start()
            ctx.update_tangle(k * dt)
            ctx.rk4_step(k * dt, dt)
            ts.append(ctx.timer_stop())
        rk4[name] = {"steps_per_s": 1e3 / statistics.mean(ts), "ms_per_step": statistics.mean(ts),
                     "node_evals_per_s": 4 * n / (statistics.mean(ts) * 1e-3)}
    ctx.set_precision(abi.OV_PREC_FP64)
    # ---- accuracy against FP64 direct sums on a 4,096-node subsample (after the
    # timed sections: the direct sums are O(N) per node)
    ctx.upload(ht)
    ctx.update_tangle(0.0)
    sub = direct_subsample(n, 4096, 1)
    direct_v, _ = ctx.direct_velocities(sub)
    fp64_vs_direct = rel_l2(fp64_vels[sub], direct_v)
    if isinstance(mixed, dict) and "value" in mixed:
        mixed["rel_l2_vs_direct_subsample"] = rel_l2(mixed_vels[sub], direct_v)

    ensemble = precision_form = large = next_rows = config_a = None
    if world == 1 and args.config_a:
        try:
            config_a = run_config_a(args, device)
        except Exception as e:
            config_a = {"error": str(e)[:300]}
    if world == 1 and args.ensemble_steps >= 0:
        try:
            ensemble = run_ensemble(args, device)
        except Exception as e:
            ensemble = {"error": str(e)[:300]}
    if world == 1 and args.precision_form:
        try:
            precision_form = run_precision_form(args, device)
        except Exception as e:
            precision_form = {"error": str(e)[:300]}
    if world == 1 and args.large_steps >= 0:
        try:
            large = run_large(args, device)
        except Exception as e:
            large = {"error": str(e)[:300]}
    if world == 1 and args.next_rows:
        try:
            next_rows = run_next_rows(args, device)
        except Exception as e:
            next_rows = {"error": str(e)[:300]}
    clk.__exit__(None, None, None)

    # ---- CPU baseline (rank 0 only, bounded sample)
    cpu = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        kind = cpu_kind()
        times = cpu_eval_time(kind, threads, 2, ht)
        cpu = cpu_line(n / min(times), threads, kind, "2 full update_tangle of the 65,536-node tangle (best of 2)")

    ctx.close()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox random-walk tangle)",
        "config": WORKLOAD,
        "l2": "flushed between timed steps (256 MiB write)",
        "parallelism": "replicas" if world > 1 else "single GPU",
        "phases_ms": {"tangents": phases[0], "tree_build": phases[1], "traversal": phases[2]},
        "roofline": {"bound": "fma", "pipe": "fp64", "achieved": achieved, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp64_peak, "traffic": K_VEL_FP64_DRAM_BYTES,
                     "traffic_note": "DRAM bytes per launch from ncu; the traversal is FP64-pipe bound",
                     "peak_source": "measured in this run (FP64 FMA chains, all SMs)",
                     "work": "42 flops per accepted interaction + 9 per visited cell (fixed convention); the split "
                             "walk runs the visits' tests in FP32 and the interactions in FP64",
                     "accepts": acc, "visits": vis, "fp32_fma_peak_tflops": fp32_peak,
                     "warp_efficiency": vis / max(1, 32 * st["warp_steps"])},
        "accuracy": {"fp64_tree_rel_l2_vs_direct_subsample": fp64_vs_direct,
                     "subsample": "4,096 nodes, FP64 direct sums (tree == NULL branch) on the GPU"},
        "cpu_baseline": cpu,
        "e2e": {"value": world * n / (e2e_mean * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "mixed": mixed,
        "double_single": dd,
        "fp64_walk": walk64,
        "rk4": rk4,
        "config_a": config_a,
        "ensemble": ensemble,
        "precision_form": precision_form,
        "large": large,
        "next_rows": next_rows,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "peaks_source": peak_src,
    }
    print(json.dumps(line))
    return 0


def run_build_profile(args):
    """The large tangle's tree build (keys, radix sort, cells, moments, FP32
    cell copy) repeated; one line with the phase times (CUDA events)."""
    from openvort_gb300 import abi, gpu, workloads as W
    E = LARGE
    ht = W.random_walk_tangle(E["n_loops"], E["per_loop"], D=E["D"], seed=E["seed"])
    ctx = gpu.Context(0, params=W.config_params("large", bh_resolution=E["theta"]), precision=abi.OV_PREC_MIXED)
    ctx.upload(ht)
    ctx.set_phase_timing(True)
    ph = []
    for _ in range(args.build_profile):
        ctx.flush_l2(256 << 20)
        ctx.update_tangle(0.0)
        ph.append(ctx.phase_times())
    ctx.close()
    ph = np.array(ph)
    print(json.dumps({"mode": "build_profile", "workload": E["workload"], "nodes": ht.n,
                      "tree_build_ms": float(np.median(ph[:, 1])), "tangents_ms": float(np.median(ph[:, 0])),
                      "traversal_ms": float(np.median(ph[:, 2])), "repeats": args.build_profile}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ensemble-steps", type=int, default=100,
                    help="full time steps of the 48-tangle ensemble (-1: skip the ensemble section)")
    ap.add_argument("--large-steps", type=int, default=50,
                    help="full time steps of the 1,048,576-node tangle (-1: skip that section)")
    ap.add_argument("--precision-form", type=int, default=1, help="262,144-node theta 0.3/0.5 section (0: skip)")
    ap.add_argument("--config-a", type=int, default=1,
                    help="the 8-ring configuration's 200 steps (and crossing rings), GPU and CPU (0: skip)")
    ap.add_argument("--next-rows", type=int, default=1,
                    help="walls, frames, injection and spherical-fork sections (0: skip)")
    ap.add_argument("--cpu-sections", type=int, default=1,
                    help="time the CPU baseline of the ensemble, precision-form and large sections too (0: skip)")
    ap.add_argument("--build-profile", type=int, default=0,
                    help="only rebuild the 1,048,576-node tangle's tree this many times and print the build "
                         "times (a workload for profiling the sort and build kernels)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.build_profile > 0:
        return run_build_profile(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
