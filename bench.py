"""Benchmark: voxel-message updates/s of plain BP on one GB300.

Workload (default): 13 keyframes 640x480 (fx=fy=525, cx=320, cy=240) of a
seeded 6x6x3 m room with 20 boxes and 3 spheres, 1 cm voxels, max range 5 m,
20 BP iterations, full-ray brick activation.  A step is one complete
perform_inference (20 Gauss-Seidel iterations over the 13 cameras) from the
prior; the unit of work is one incidence-iteration (one ray->voxel message
computed and consumed), so

    value = N_inc * iters * steps / time.

The incidence arrays (several GB) are far larger than L2, so no flush is
needed between steps.  ``e2e`` times the same work through the public C ABI
with host buffers: map creation, upload of the 13 depth images from pinned
host memory, brick activation, incidence build, 20 iterations and the
read-back of all beliefs.

``--impl reference`` times the reference's algorithm on the host cores.  The
reference (GVDB + Eigen + yaml-cpp + OpenCV) cannot be built here, so its
CPU restatement in ``oracle/`` (FP64 BP, OpenMP over rays) stands in on the
same workload: all 13 keyframes' incidence lists held, one Gauss-Seidel
camera update per step.

Multi-GPU: the path does not shard here -- ``--gpus N`` runs N independent
replicas (one per rank) and reports the whole-job rate.
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

METRIC = "voxel-msg updates/s (plain BP, 13x640x480, 1 cm, 20 iters)"
UNIT = "updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="full", choices=["full", "mid", "small", "mixed", "large", "batched"])
    ap.add_argument("--frames", type=int, default=2000, help="large workload: frames streamed")
    ap.add_argument("--window", type=int, default=8, help="large workload: live keyframes")
    ap.add_argument("--policy", default="fullray", choices=["fullray", "endpoint"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ray-variant", type=int, default=None,
                    help="use this ray-kernel variant instead of autotuning (profiling runs)")
    ap.add_argument("--warm-scenes", type=int, default=20,
                    help="held-out 10x320x240 2 cm scenes for the warm-start comparison (0: skip)")
    return ap.parse_args()


def workload(name):
    from mrfmap_gb300 import synthetic
    if name == "full":
        return synthetic.full_room(1)
    if name == "mid":  # profiling-sized cut of the full scene: 3 views at 320x240, same voxels
        return synthetic.full_room(1, n_frames=3, rows=240, cols=320)
    if name == "mixed":  # uneven batch: 24 views of 160x120 / 320x240 / 640x480, 2 cm
        return synthetic.mixed_room(2, n_frames=24)
    return synthetic.small_room(0)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("MRF_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def mem_available_gb():
    """Host memory available to this process (GB), from /proc/meminfo."""
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 1e6
    except Exception:
        pass
    return None


# host memory the FP64 oracle needs per 640x480 1 cm full-ray view of the
# bench workload: ~104 M incidences x 21 B (voxel, length, exit distance,
# run flag, FP64 potential) + 12 B per voxel of the map for its messages
ORACLE_GB_PER_VIEW = 3.2


def workload_config(w, policy, ws):
    """The workload both arms run (identical in the two bench lines)."""
    p = w.params
    return {"workload": w.name, "views": len(w.poses), "rows": p.rows, "cols": p.cols,
            "voxel_m": p.res, "dims_m": list(p.dims), "activation": policy, "iters": p.max_iters,
            "schedule": "gauss-seidel", "seed": w.seed,
            "l2": "inputs larger than L2 (no flush)",
            "parallelism": f"replicas{ws}" if ws > 1 else "single"}


class CpuPort:
    """The FP64 oracle (the reference's equations; OpenMP over rays) holding
    the whole workload: every keyframe's incidence lists built, then timed
    one Gauss-Seidel camera update at a time (the body of the reference's
    camera loop, src/GVDBInference.cpp:155-167) on the evolving state."""

    def __init__(self, w, policy, threads, max_views=None):
        from oracle import oracle as O
        self.threads = threads
        self.om = O.OracleMap(w.params, threads=threads)
        pol = O.ACT_FULL_RAY if policy == "fullray" else O.ACT_ENDPOINT
        n = len(w.poses) if max_views is None else min(max_views, len(w.poses))
        self.n_views = n
        for k in range(n):
            P, D = w.poses[k], w.depths[k]
            if w.cams:
                self.om.add_view_camera(P, D, D.shape[0], D.shape[1], *w.cams[k], pol)
            else:
                self.om.add_view(P, D, pol)
        t0 = time.perf_counter()
        self.om.build_all()  # incidence lists, outside every timed region
        self.build_s = time.perf_counter() - t0
        self.next = 0

    def step(self):
        """one camera update; returns (updates, seconds)"""
        c = self.next
        self.next = (self.next + 1) % self.n_views
        t0 = time.perf_counter()
        n = self.om.update_camera(c)
        return n, time.perf_counter() - t0

    def close(self):
        self.om.close()


def cpu_views_that_fit(w):
    """All keyframes when the host has the memory for the oracle's lists,
    else as many as fit (stated in the line)."""
    avail = mem_available_gb()
    if avail is None or w.params.res > 0.015:
        return len(w.poses)
    return max(1, min(len(w.poses), int((avail - 8.0) / ORACLE_GB_PER_VIEW)))


def cpu_insertion_rate(w, policy, n_views):
    """Classic log-odds ray insertion (OctoMap's update rule: miss along the
    ray, hit at the endpoint voxel, clamped) of the first n_views keyframes
    into the same active voxels, single-threaded on the host: voxel updates/s
    and rays/s.  A reported CPU baseline for insertion-style mapping, not
    OctoMap itself (absent here) and not MRFMap."""
    from oracle import oracle as O
    m = O.OracleMap(w.params, threads=1)
    pol = O.ACT_FULL_RAY if policy == "fullray" else O.ACT_ENDPOINT
    views = list(zip(w.poses, w.depths))[:n_views]
    for k, (P, D) in enumerate(views):
        if w.cams:
            m.add_view_camera(P, D, D.shape[0], D.shape[1], *w.cams[k], pol)
        else:
            m.add_view(P, D, pol)
    L = None
    upd, rays = 0, 0
    t0 = time.perf_counter()
    for k, (P, D) in enumerate(views):
        if w.cams:  # the oracle's insertion uses the map's camera
            continue
        n, L = m.insert_logodds(P, D, logodds=L)
        upd += n
        rays += int((D > 0).sum())
    dt = time.perf_counter() - t0
    m.close()
    return upd / max(dt, 1e-9), rays / max(dt, 1e-9), upd, dt


def cpu_baselines(w, policy, insertion_views=2):
    """The CPU baselines of the bench line: the FP64 oracle port holding the
    whole workload, timed over one full Gauss-Seidel sweep (every keyframe's
    camera update once, all host cores), and the classic log-odds insertion
    of a bounded sample (single-threaded)."""
    threads = os.cpu_count() or 1
    nv = cpu_views_that_fit(w)
    port = CpuPort(w, policy, threads, max_views=nv)
    upd, dt = 0, 0.0
    for _ in range(port.n_views):
        n, t = port.step()
        upd += n
        dt += t
    port.close()
    cpu = {"value": upd / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"FP64 oracle holding {nv} of {len(w.poses)} keyframes (incidence lists built in "
                     f"{port.build_s:.1f} s, untimed), one Gauss-Seidel sweep of {nv} camera updates "
                     f"({upd} updates in {dt:.1f} s)"}
    cpu_ins = None
    if not w.cams:
        try:
            ni = min(insertion_views, len(w.poses))
            ir, rr, iu, idt = cpu_insertion_rate(w, policy, ni)
            cpu_ins = {"value": ir, "unit": "voxel updates/s", "rays_per_s": rr, "cores": 1,
                       "kind": "classic log-odds ray insertion (OctoMap's update rule; OctoMap "
                               "itself is absent), single-threaded",
                       "sample": f"{ni} of {len(w.poses)} keyframes ({iu} voxel updates in {idt:.2f} s)"}
        except Exception as e:  # a reported extra: never fails the bench line
            cpu_ins = {"error": str(e)}
    return cpu, cpu_ins


def run_reference(args):
    """The reference's algorithm on the host cores (its GVDB build is not
    possible offline: the FP64 restatement in oracle/ stands in) on the same
    workload as the GPU arm: every keyframe's incidence lists held, each
    step one Gauss-Seidel camera update of the 20-iteration schedule (steps
    cycle through the keyframes, so 13 steps are one full iteration)."""
    rank, ws = dist_setup()
    if rank != 0:
        return
    w = workload(args.workload)
    threads = os.cpu_count() or 1
    nv = cpu_views_that_fit(w)
    port = CpuPort(w, args.policy, threads, max_views=nv)
    for _ in range(args.warmup):
        port.step()
    upd_tot, t_tot = 0, 0.0
    for _ in range(args.steps):
        n, dt = port.step()
        upd_tot += n
        t_tot += dt
    port.close()
    value = upd_tot / t_tot
    sample = (f"FP64 oracle holding {nv} of {len(w.poses)} keyframes (incidence lists built in "
              f"{port.build_s:.1f} s, untimed); one step = one Gauss-Seidel camera update "
              f"(steps cycle through the keyframes; {len(w.poses)} steps = one iteration)")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "impl": "reference",
        "config": workload_config(w, args.policy, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step": "one Gauss-Seidel camera update (the unit of the reference's camera loop); the GPU arm's "
                "step is 20 full iterations, the metric (updates/s) is a rate",
        "views_held": nv,
        "note": "reference (GVDB/Eigen/yaml-cpp/OpenCV) not buildable offline: its restatement "
                "in oracle/ (FP64, OpenMP over rays) is timed",
    }
    print(json.dumps(line))


# bumped whenever k_ray_bp's memory traffic changes (profiles/ray_bp_traffic.json)
RAY_KERNEL_VERSION = 7


HOME_SHARES = (60, 75, 90)  # per cent of an SM region's work on its home blocks, tried by the autotuner


def tune_jointly(m, flags):
    """The ray-kernel variant (and the pair-reduction variant) tuned at each
    home share of HOME_SHARES, keeping the fastest pair: the schedule's
    choices interact (an SM-region variant may win only at another share).
    Every choice moves work between threads, never a result.  Returns the
    chosen variant, its per-variant ms at the chosen share and the best ms
    per share."""
    best = None
    per_share = []
    for sh in HOME_SHARES:
        m.set_home_share(sh)
        v, ms = m.autotune(reps=2, flags=flags)
        per_share.append(float(np.min(ms)))
        if best is None or float(np.min(ms)) < best[0]:
            best = (float(np.min(ms)), sh, v, ms, m.tuning()[2])
    _, sh, v, ms, pv = best
    m.set_home_share(sh)
    m.set_ray_variant(v)
    m.set_pair_variant(pv)
    return v, ms, per_share


def ray_kernel_bytes(st, iters, half=False):
    """Algorithmic bytes of the ray-message work of one mrf_infer call of
    `iters` iterations, over the rays it runs over (those with a dynamic
    incidence); the call's stats say whether it took the fast path.  Gather width g and length width l: 4 B each with the
    default fp32 streams, 2 B each with 16-bit streams.
      the first two iterations (full path): per Pre incidence the pair id
        (4 B), length and ln q gather (l + g); per dynamic incidence +8 B
        (potential 4, message write 4); per ray 16 B of metadata;
      once per call, the quiet sums of the static prefixes [0, k4): per
        incidence pair id, fp32 length and gather (8 + g); per ray 16 B;
      every later iteration (fast path): per incidence from k4 on 4 + l + g;
        per loud prefix incidence pair id, fp32 length, position and gather
        (10 + g); per dynamic incidence +8 B; per ray 36 B (metadata 16,
        ray index 4, quiet sums 8, list bounds 8)."""
    g = 2 if half else 4
    ln = 2 if half else 4
    pre, k4, loud = st["n_inc_pre_bp"], st["n_inc_from_k4"], st["n_loud_prefix"]
    dyn, rays = st["n_inc_dyn"], st["n_rays_bp"]
    full = (4 + ln + g) * pre + 8 * dyn + 16 * rays
    if iters < 3 or not st.get("quiet_prefix_used"):
        return full * iters
    quiet = (8 + g) * (pre - k4) + 16 * rays
    fast = (4 + ln + g) * k4 + (10 + g) * loud + 8 * dyn + 36 * rays
    return 2 * full + quiet + (iters - 2) * fast


LONG_RAY = 512  # Pre incidences above which the ray kernel sums in FP64


def parity_cut(w, act, policy):
    """Beliefs of the CUDA path against the FP64 oracle on views 0 and V/2 of
    the workload (Gauss-Seidel, the workload's iteration count), over all
    voxels and over the voxels crossed by rays longer than LONG_RAY."""
    from mrfmap_gb300 import lib as L
    from oracle import oracle as O
    views = sorted({0, len(w.poses) // 2})
    gm = L.MRFMap(w.params, activation=act)
    om = O.OracleMap(w.params, threads=os.cpu_count() or 1)
    pol = O.ACT_FULL_RAY if policy == "fullray" else O.ACT_ENDPOINT
    for k in views:
        if w.cams:
            gm.add_view_camera(w.poses[k], w.depths[k], *w.cams[k])
            D = w.depths[k]
            om.add_view_camera(w.poses[k], D, D.shape[0], D.shape[1], *w.cams[k], pol)
        else:
            gm.add_view(w.poses[k], w.depths[k])
            om.add_view(w.poses[k], w.depths[k], pol)
    iters = w.params.max_iters
    gm.set_precision(L.PRECISION_HALF_STREAMS)
    gm.infer(iters=iters)
    g16 = gm.beliefs().astype(np.float64).ravel()
    gm.set_precision(L.PRECISION_FP32)
    gm.reset_state()
    gm.infer(iters=iters)
    t0 = time.perf_counter()
    om.infer(iters=iters)
    t_oracle = time.perf_counter() - t0
    gb, ob = gm.beliefs().astype(np.float64).ravel(), om.beliefs().ravel()
    om.close()
    err = np.abs(gb - ob)
    err16 = np.abs(g16 - ob)
    touched = (gb > 0) | (ob > 0)
    n_long, lv = 0, []
    for v in range(len(views)):
        meta, vox, _, _ = gm.view_incidences(v)
        n_pre = meta[:, 0].astype(np.int64)
        off = np.concatenate([[0], np.cumsum(n_pre)])
        long = np.flatnonzero(n_pre > LONG_RAY)
        n_long += len(long)
        for r in long[:: max(1, len(long) // 4000)]:
            lv.append(vox[off[r]:off[r + 1]])
        del meta, vox
    gm.close()
    lv = np.unique(np.concatenate(lv)) if lv else np.zeros(0, np.int64)
    out = {"workload": f"{w.name}, views {views}", "iters": iters, "schedule": "gauss-seidel",
           "max_abs_belief_err": float(err.max()),
           "class_agreement_at_0.5": float(((gb > 0.5) == (ob > 0.5))[touched].mean()),
           "rays_longer_than_512": int(n_long),
           "reference": "FP64 CPU oracle", "oracle_s": round(t_oracle, 1)}
    if len(lv):
        out["max_abs_belief_err_long_ray_voxels"] = float(err[lv].max())
        out["long_ray_voxels_checked"] = int(len(lv))
    out["half_streams"] = {"max_abs_belief_err": float(err16.max()),
                           "class_agreement_at_0.5": float(((g16 > 0.5) == (ob > 0.5))[touched].mean())}
    return out


def run_ours(args):
    import torch

    from mrfmap_gb300 import lib as L
    rank, ws = dist_setup()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    torch.cuda.init()
    w = workload(args.workload)
    iters = w.params.max_iters
    act = L.ACT_FULL_RAY if args.policy == "fullray" else L.ACT_ENDPOINT
    m = L.MRFMap(w.params, activation=act)
    # inputs resident in HBM before the timed region
    dev_depths = [torch.from_numpy(np.ascontiguousarray(d)).cuda() for d in w.depths]
    torch.cuda.synchronize()
    for k, (P, D) in enumerate(zip(w.poses, dev_depths)):
        if w.cams:  # views with their own cameras (host depth images)
            m.add_view_camera(P, w.depths[k], *w.cams[k])
        else:
            m.add_view_device(P, D.data_ptr())
    m.infer(iters=1)  # builds the incidence lists
    # ray-kernel variant chosen by the autotuner on this workload (before the
    # timed region; variants are numerically identical)
    share_ms = []
    if args.ray_variant is None:
        tuned, tune_ms, share_ms = tune_jointly(m, 0)
    else:
        m.set_ray_variant(args.ray_variant)
        tuned, tune_ms = args.ray_variant, []
    st = m.stats()
    n_upd_step = st["n_inc_post"] * iters
    stream = torch.cuda.ExternalStream(m.stream())
    for _ in range(args.warmup):
        m.reset_state()
        m.infer(iters=iters, flags=L.ASYNC)
    m.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        m.reset_state()
        m.infer(iters=iters, flags=L.ASYNC)
    e1.record(stream)
    m.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    # the same steps with 16-bit streams in the ray kernel (fp16 lengths and
    # ln q; reported beside the fp32 default with its error against the
    # FP64 oracle)
    m.set_precision(L.PRECISION_HALF_STREAMS)
    for _ in range(2):
        m.reset_state()
        m.infer(iters=iters, flags=L.ASYNC)
    m.synchronize()
    h0 = torch.cuda.Event(enable_timing=True)
    h1 = torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    for _ in range(args.steps):
        m.reset_state()
        m.infer(iters=iters, flags=L.ASYNC)
    h1.record(stream)
    m.synchronize()
    ms_half = h0.elapsed_time(h1)
    m.reset_state()
    m.infer(iters=iters, flags=L.PROFILE)
    prof_half = m.stats()
    m.set_precision(L.PRECISION_FP32)
    # the same steps reading every ray's whole Pre range in every iteration
    # (MRF_FULL_RAYS: no static prefixes from their quiet sums), profiled
    # once: the ray kernel's roofline on the full path
    m.reset_state()
    m.infer(iters=iters, flags=L.FULL_RAYS | L.PROFILE)
    prof_full = m.stats()
    ms_full = prof_full["infer_ms"]
    # per-kernel device times of one profiled step (events on the map stream)
    m.reset_state()
    m.infer(iters=iters, flags=L.PROFILE)
    prof = m.stats()
    clk = clocks.stop()
    ms = max_over_ranks(ms, ws)
    launches_step = prof["kernel_launches"] + 2  # + reset kernels
    value = sum_over_ranks(n_upd_step * args.steps, ws) / (ms / 1e3)

    # roofline of the dominant kernel (ray messages)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    k_ms = prof["kernel_ms"][1]
    k_n = max(prof["kernel_count"][1], 1)
    per_launch_bytes = ray_kernel_bytes(prof, iters) / k_n
    achieved = per_launch_bytes / (k_ms / k_n / 1e3) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "ray_bp_traffic.json")
    if os.path.exists(tfile):
        try:
            t = json.load(open(tfile))
            if t.get("kernel_version") == RAY_KERNEL_VERSION and t.get("activation") == args.policy:
                # DRAM bytes over algorithmic bytes from a capture of the same
                # kernel on a smaller case, applied to this launch's bytes
                traffic = t["dram_over_algorithmic"] * per_launch_bytes
        except Exception:
            pass
    kernel_share = {n: round(v / max(sum(prof["kernel_ms"]), 1e-9), 4)
                    for n, v in zip(("pair_prepare", "ray_bp", "pair_update", "voxel_apply"),
                                    prof["kernel_ms"])}
    # the same roofline with the survey's byte widths (16-bit lengths and
    # messages): the ray kernel's share is 12 B per incidence (voxel slot 4,
    # length 2, L gather 4, message 2); a whole iteration moves
    # B_iter = 16 N_inc + 12 N_cv + 8 N_vox
    survey_ray = 12 * st["n_inc_post"] * iters / k_n
    survey_ray_gbs = survey_ray / (k_ms / k_n / 1e3) / 1e9
    b_iter = 16 * st["n_inc_post"] + 12 * st["n_pairs"] + 8 * st["n_vox_touched"]
    step_gbs = b_iter * iters / (ms / args.steps / 1e3) / 1e9

    # e2e through the C ABI with host buffers (pinned), create -> read-back
    pinned = [torch.from_numpy(np.ascontiguousarray(d)).pin_memory() for d in w.depths]
    h2d = sum(p.numel() * 4 for p in pinned) + 16 * 4 * len(w.poses)
    e2e_times, d2h, phases = [], 0, []
    out = None  # pinned read-back buffers, allocated once from the warm-up pass's brick count
    for step in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        mm = L.MRFMap(w.params, activation=act)
        for k, (P, D) in enumerate(zip(w.poses, pinned)):
            if w.cams:
                mm.add_view_camera(P, D.numpy(), *w.cams[k])
            else:
                mm.add_view(P, D.numpy())
        t1 = time.perf_counter()
        mm.infer(iters=iters)
        t2 = time.perf_counter()
        if out is not None and out[1].shape[0] == mm.num_bricks:
            cen, bel = mm.read_bricks(out[0], out[1])
        else:
            cen, bel = mm.read_bricks()
        t3 = time.perf_counter()
        if out is None:
            nb = mm.num_bricks
            out_t = (torch.empty((nb, 3), dtype=torch.float32).pin_memory(),
                     torch.empty((nb, 512), dtype=torch.float32).pin_memory())
            out = (out_t[0].numpy(), out_t[1].numpy())
        est = mm.stats()
        mm.close()
        dt = time.perf_counter() - t0
        d2h = cen.nbytes + bel.nbytes
        if step > 0:  # first pass warms allocator and host paths
            e2e_times.append(dt)
            phases.append({"create_and_add_views_s": t1 - t0, "infer_s": t2 - t1,
                           "build_device_ms": est["build_ms"], "iterations_device_ms": est["infer_ms"],
                           "read_back_s": t3 - t2})
    if e2e_times:
        e2e_t = max_over_ranks(float(np.mean(e2e_times)), ws)
        e2e_val = sum_over_ranks(n_upd_step, ws) / e2e_t
    else:
        e2e_t, e2e_val = None, None

    # per-view likelihood of every keyframe under the final map (device buffers)
    like = None
    try:
        if w.cams:
            raise RuntimeError("per-view cameras: the device likelihood at a pose uses the params' camera")
        m.reset_state()
        m.infer(iters=iters)
        img = torch.empty(w.params.rows * w.params.cols, device="cuda")
        sums = torch.empty(len(w.poses), device="cuda")
        for k in range(2):  # warm-up
            m.likelihood_device(w.poses[k], dev_depths[k].data_ptr(), img.data_ptr(), sums[k:].data_ptr())
        m.synchronize()
        l0 = torch.cuda.Event(enable_timing=True)
        l1 = torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        for k in range(len(w.poses)):
            m.likelihood_device(w.poses[k], dev_depths[k].data_ptr(), img.data_ptr(), sums[k:].data_ptr())
        l1.record(stream)
        m.synchronize()
        lms = l0.elapsed_time(l1)
        like = {"frames_per_s": len(w.poses) / (lms / 1e3), "ms_per_frame": lms / len(w.poses),
                "rays_per_frame": w.params.rows * w.params.cols}
    except Exception as e:  # reported, not fatal
        like = {"error": str(e)}

    # time to a converged map: learned warm start vs plain BP (held-out
    # seeded scenes of the training distribution, weights trained by
    # python -m mrfmap_gb300.warmstart)
    warm = None
    if rank == 0 and args.warm_scenes > 0:
        try:
            from mrfmap_gb300 import warmstart as WS
            if not os.path.exists(WS.DEFAULT_WEIGHTS):
                raise FileNotFoundError("no trained warm-start weights")
            net = WS.WarmNet.load_file(WS.DEFAULT_WEIGHTS)
            rows = WS.evaluate(net, WS.scenes(range(9000, 9000 + args.warm_scenes)))
            warm = {"workload": "held-out full_room 10x320x240 2 cm, seeds 9000+",
                    "converged_map": "plain BP from the prior until the largest belief change < 1e-4 "
                                     "(at most 3000 iterations; scenes that never get there are not compared)",
                    "clock": "from the method's start until max |belief - converged| <= 1e-3 "
                             "(checked every iteration)",
                    **WS.summarize(rows),
                    "per_scene": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()}
                                  for r in rows]}
        except Exception as e:  # reported, not fatal
            warm = {"error": str(e)}

    # belief error against the FP64 oracle on a two-view cut of this
    # workload, same camera, voxels and iteration count
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            parity = parity_cut(w, act, args.policy)
        except Exception as e:
            parity = {"error": str(e)}

    cpu, cpu_ins = None, None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, cpu_ins = cpu_baselines(w, args.policy)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp64 sums on rays > 512)",
            "data": "synthetic (seeded room scenes; no public dataset)",
            "config": workload_config(w, args.policy, ws),
            "workload_stats": {"n_inc_per_iter": st["n_inc_post"],
                               "n_inc_pre_per_iter": st["n_inc_pre"], "n_inc_dyn_per_iter": st["n_inc_dyn"],
                               "n_pairs": st["n_pairs"], "n_pairs_dyn": st["n_pairs_dyn"],
                               "n_vox_touched": st["n_vox_touched"],
                               "n_rays": st["n_rays"], "n_rays_bp": st["n_rays_bp"],
                               "n_inc_pre_bp_per_iter": st["n_inc_pre_bp"], "n_bricks": st["n_bricks"],
                               "n_inc_from_k4": st["n_inc_from_k4"], "n_loud_prefix": prof["n_loud_prefix"],
                               "quiet_prefix_used": prof["quiet_prefix_used"],
                               "ray_variant": tuned, "ray_variant_ms": [round(x, 4) for x in tune_ms],
                               "pair_variant": m.tuning()[2],
                               "home_share": m.tuning()[1], "home_share_ms": dict(zip(HOME_SHARES[:len(share_ms)],
                                                                                     [round(float(x), 4) for x in share_ms])),
                               "static_messages": "exact constants (p = F_EPS before a ray's first "
                                                  "non-zero potential), summed once per build"},
            "dynamic_updates_per_s": st["n_inc_dyn"] * iters * args.steps / (ms / 1e3),
            "full_ray_path": {"ms_per_step_profiled": ms_full,
                              "ray_kernel_ms_per_launch": prof_full["kernel_ms"][1] / max(prof_full["kernel_count"][1], 1),
                              "ray_kernel_bytes_per_launch": ray_kernel_bytes(prof_full, iters)
                              / max(prof_full["kernel_count"][1], 1),
                              "ray_kernel_frac": ray_kernel_bytes(prof_full, iters) / (prof_full["kernel_ms"][1] / 1e3)
                              / 1e9 / peak,
                              "note": "one profiled step with MRF_FULL_RAYS (every iteration reads every ray's whole "
                                      "Pre range); the headline value uses the default choice"},
            "half_streams": {"value": n_upd_step * args.steps / (ms_half / 1e3), "ms_per_step": ms_half / args.steps,
                             "ray_kernel_ms_per_launch": prof_half["kernel_ms"][1] / max(prof_half["kernel_count"][1], 1),
                             "note": "the same steps with fp16 segment lengths and ln q gathers in the ray kernel "
                                     "(MRF_PRECISION_HALF_STREAMS); error against the FP64 oracle in "
                                     "parity_vs_fp64.half_streams"},
            "gpu_launches": launches_step * args.steps,
            "roofline": {"bound": "hbm", "kernel": "k_ray_bp", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback",
                         "bytes_per_launch": per_launch_bytes, "ms_per_launch": k_ms / k_n,
                         "survey_bytes": {
                             "ray_kernel_bytes_per_launch": survey_ray,
                             "ray_kernel_achieved": survey_ray_gbs,
                             "frac_survey_bytes": survey_ray_gbs / peak,
                             "step_bytes_per_iter": b_iter,
                             "step_achieved": step_gbs,
                             "step_frac_survey_bytes": step_gbs / peak,
                             "widths": "per incidence 12 B in the ray kernel (slot 4, length 2, L 4, "
                                       "message 2); per iteration 16 N_inc + 12 N_cv + 8 N_vox",
                             "note": "bytes of the schedule that reads every incidence every iteration; "
                                     "from the third iteration of a call on the ray kernel reads the static "
                                     "prefixes' loud incidences only (the quiet ones' sums are formed once "
                                     "per call), so these are effective rates, not DRAM bandwidths"}},
            "kernel_share": kernel_share,
            "clocks": clk,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "s_per_step": e2e_t,
                    "phases": {k: round(float(np.mean([p[k] for p in phases])), 4) for k in phases[0]}
                    if phases else None},
            "cpu_baseline": cpu,
            "cpu_insertion": cpu_ins,
            "likelihood": like,
            "parity_vs_fp64": parity, "warm_start": warm,
        }
        print(json.dumps(line))
    m.close()


LARGE_METRIC = "frames/s and voxel-msg updates/s (large incremental map, 640x480, 2 cm, 5 iters/frame)"
POOL_LIMIT = 180e9  # device bytes the map may hold (brick pool, window of incidence lists, scratch)


def run_large(args):
    """The large incremental map: frames of a seeded random walk through a
    20x20x4 m room of 150 boxes stream in from pinned host memory; each is
    added (upload, clean-up, activation), the keyframe leaving the window of
    `window` live views is retired (its messages stay in the log-odds), the
    window's incidence lists are built and 5 MRF_INCREMENTAL iterations run
    over it.  The map may hold at most 180 GB of device memory
    (mrf_set_memory_limit).  One step = one frame; the frames are rendered on
    the GPU before the timed region."""
    import torch

    from mrfmap_gb300 import lib as L
    from mrfmap_gb300 import synthetic
    rank, ws = dist_setup()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    walk = synthetic.walk_room(5, n_frames=args.frames)
    iters = walk.params.max_iters
    pinned = []
    for k0 in range(0, args.frames, 64):
        for d in synthetic.render_frames_torch(walk, range(k0, min(k0 + 64, args.frames))):
            pinned.append(d.cpu().pin_memory())
    torch.cuda.synchronize()
    lib = L.load()
    lib.mrf_set_memory_limit(int(POOL_LIMIT))
    m = L.MRFMap(walk.params, activation=L.ACT_FULL_RAY)
    W = args.window
    warm = min(args.warmup, args.frames)

    def frame(k):
        m.add_view(walk.poses[k], pinned[k].numpy())
        if k >= W:
            m.retire_view(k - W)
        m.infer(iters=iters, flags=L.INCREMENTAL)
        st = m.stats()
        return st

    for k in range(warm):
        frame(k)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    upd, peak, build_ms, infer_ms = 0, 0, 0.0, 0.0
    t0 = time.perf_counter()
    for k in range(warm, args.frames):
        st = frame(k)
        upd += st["n_inc_post"] * iters
        build_ms += st["build_ms"]
        infer_ms += st["infer_ms"]
        peak = max(peak, lib.mrf_memory_in_use())
    torch.cuda.synchronize()
    dt = max_over_ranks(time.perf_counter() - t0, ws)
    barrier(ws)
    clk = clocks.stop()
    st = m.stats()
    nb = st["n_bricks"]
    bel = m.beliefs()
    m.close()
    lib.mrf_set_memory_limit(0)
    n = args.frames - warm
    if rank == 0:
        print(json.dumps({
            "metric": LARGE_METRIC, "value": sum_over_ranks(n, ws) / dt, "unit": "frames/s", "n_gpus": ws,
            "steps": n, "warmup": warm, "ms_per_step": 1e3 * dt / max(n, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp64 sums on rays > 512)",
            "data": "synthetic (seeded random walk; no public dataset)",
            "config": {"workload": walk.name, "frames": args.frames, "window": W, "iters_per_frame": iters,
                       "voxel_m": walk.params.res, "dims_m": list(walk.params.dims), "boxes": 150,
                       "activation": "fullray", "seed": walk.seed, "pool_limit_bytes": POOL_LIMIT,
                       "parallelism": f"replicas{ws}" if ws > 1 else "single"},
            "updates_per_s": upd / dt, "updates": upd,
            "per_frame_ms": {"build": build_ms / max(n, 1), "bp": infer_ms / max(n, 1),
                             "other": 1e3 * dt / max(n, 1) - (build_ms + infer_ms) / max(n, 1)},
            "device_bytes_peak": peak, "n_bricks_final": nb,
            "list_builds": {"full": st["builds_full"], "appended": st["builds_appended"]},
            "quiet_prefix_used": st["quiet_prefix_used"],
            "occupied_voxels_final": int((bel > 0.5).sum()),
            "clocks": clk,
            "e2e": {"value": sum_over_ranks(n, ws) / dt, "unit": "frames/s",
                    "h2d_bytes_per_step": walk.params.rows * walk.params.cols * 4 + 64,
                    "d2h_bytes_per_step": 0},
        }))


BATCH_METRIC = "voxel-msg updates/s (batched BP: 8 scenes, 256 keyframes of mixed resolution, 2 cm, Jacobi)"


def batch_parity():
    """Beliefs of a reduced batch (3 scenes x 5 views, 4 cm) against the FP64
    oracle holding the same boxed views, 10 Jacobi iterations."""
    from mrfmap_gb300 import lib as L
    from mrfmap_gb300 import synthetic
    from oracle import oracle as O
    b = synthetic.batch_scenes(11, n_scenes=3, views_per_scene=5, sizes=((60, 80), (120, 160)),
                               size_cycle=(0, 1), res=0.04, n_boxes=6, room_range=(3.0, 6.0))
    gm = L.MRFMap(b.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(b.params, threads=os.cpu_count() or 1)
    for k in range(len(b.poses)):
        d = synthetic.render_batch_view(b, k)
        rows, cols, fx, fy, cx, cy = b.cams[k]
        lo, hi = b.boxes[b.scene_of[k]]
        gm.add_view_box(b.poses[k], d, fx, fy, cx, cy, lo, hi)
        om.add_view_box(b.poses[k], d, rows, cols, fx, fy, cx, cy, lo, hi, O.ACT_FULL_RAY)
    gm.infer(iters=10, flags=L.JACOBI)
    om.infer(iters=10, flags=O.JACOBI)
    gb, ob = gm.beliefs().astype(np.float64), om.beliefs()
    touched = (gb > 0) | (ob > 0)
    gm.close()
    om.close()
    return {"workload": b.name + " (3 scenes x 5 views, 4 cm)", "iters": 10, "schedule": "jacobi",
            "max_abs_belief_err": float(np.abs(gb - ob).max()),
            "class_agreement_at_0.5": float(((gb > 0.5) == (ob > 0.5))[touched].mean()),
            "reference": "FP64 CPU oracle"}


def run_batched(args):
    """The batched workload: 8 seeded box rooms in disjoint scene boxes of one
    map, 256 keyframes of mixed resolution (half 160x120, three eighths
    320x240, one eighth 640x480), 2 cm, full-ray activation, 20 Jacobi
    iterations per step: one persistent ray launch per iteration over every
    ray of every keyframe of every scene (longest first or SM regions, the
    autotuner's choice), each iteration replayed from a CUDA graph."""
    import torch

    from mrfmap_gb300 import lib as L
    from mrfmap_gb300 import synthetic
    rank, ws = dist_setup()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    b = synthetic.batch_scenes(3)
    iters = b.params.max_iters
    depths = [d.cpu().numpy() for d in synthetic.render_batch_torch(b, range(len(b.poses)))]
    m = L.MRFMap(b.params, activation=L.ACT_FULL_RAY)
    t0 = time.perf_counter()
    for k, d in enumerate(depths):
        rows, cols, fx, fy, cx, cy = b.cams[k]
        lo, hi = b.boxes[b.scene_of[k]]
        m.add_view_box(b.poses[k], d, fx, fy, cx, cy, lo, hi)
    m.infer(iters=1, flags=L.JACOBI)  # incidence lists, voxel CSR
    build_s = time.perf_counter() - t0
    tuned, tune_ms, share_ms = tune_jointly(m, L.JACOBI)
    st = m.stats()
    stream = torch.cuda.ExternalStream(m.stream())
    for _ in range(args.warmup):
        m.reset_state()
        m.infer(iters=iters, flags=L.JACOBI | L.ASYNC)
    m.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        m.reset_state()
        m.infer(iters=iters, flags=L.JACOBI | L.ASYNC)
    e1.record(stream)
    m.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    ms = max_over_ranks(e0.elapsed_time(e1), ws)
    clk = clocks.stop()
    m.reset_state()
    m.infer(iters=iters, flags=L.JACOBI | L.PROFILE)
    prof = m.stats()
    share_choice = m.tuning()[1]
    m.close()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    k_ms, k_n = prof["kernel_ms"][1], max(prof["kernel_count"][1], 1)
    per_launch = ray_kernel_bytes(prof, iters) / k_n
    achieved = per_launch / (k_ms / k_n / 1e3) / 1e9
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            parity = batch_parity()
        except Exception as e:
            parity = {"error": str(e)}
    n_upd = st["n_inc_post"] * iters * args.steps
    if rank == 0:
        sizes = {}
        for c in b.cams:
            sizes[f"{c[1]}x{c[0]}"] = sizes.get(f"{c[1]}x{c[0]}", 0) + 1
        print(json.dumps({
            "metric": BATCH_METRIC, "value": sum_over_ranks(n_upd, ws) / (ms / 1e3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp64 sums on rays > 512)",
            "data": "synthetic (seeded box rooms; no public dataset)",
            "config": {"workload": b.name, "scenes": len(b.boxes), "views": len(b.poses), "view_sizes": sizes,
                       "voxel_m": b.params.res, "max_range_m": b.max_range, "activation": "fullray",
                       "iters": iters, "schedule": "jacobi", "seed": b.seed,
                       "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas{ws}" if ws > 1 else "single"},
            "workload_stats": {"n_inc_per_iter": st["n_inc_post"], "n_inc_dyn_per_iter": st["n_inc_dyn"],
                               "n_pairs": st["n_pairs"], "n_rays": st["n_rays"], "n_bricks": st["n_bricks"],
                               "build_s": round(build_s, 3), "ray_variant": tuned,
                               "quiet_prefix_used": prof["quiet_prefix_used"],
                               "n_inc_from_k4": prof["n_inc_from_k4"], "n_loud_prefix": prof["n_loud_prefix"],
                               "ray_variant_ms": [round(x, 4) for x in tune_ms],
                               "home_share": share_choice,
                               "home_share_ms": dict(zip(HOME_SHARES, [round(float(x), 4) for x in share_ms]))},
            "ray_launches_per_iter": k_n / iters,
            "kernel_share": {n: round(v / max(sum(prof["kernel_ms"]), 1e-9), 4)
                             for n, v in zip(("pair_prepare", "ray_bp", "pair_update", "voxel_apply"),
                                             prof["kernel_ms"])},
            "roofline": {"bound": "hbm", "kernel": "k_ray_bp", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback",
                         "bytes_per_launch": per_launch, "ms_per_launch": k_ms / k_n},
            "clocks": clk, "parity_vs_fp64": parity,
            "gpu_launches": prof["kernel_launches"] * args.steps,
        }))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "large":
        run_large(args)
    elif args.workload == "batched":
        run_batched(args)
    else:
        run_ours(args)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
