"""Benchmark: aligned cloud pairs/s at <= 1 mm RMSE, learned proposal + ICP
against plain GPU ICP.

Default workload (config 4): 512 pairs of synthetic depth images of the
turntable object family (Kinect v1 640x480 uint16 mm and Kinect v2 512x424
float32 mm, at the super-resolution tools' upsampling factors 1, 2 and 4;
5k-500k points per view), resident in HBM.  One step = back-projection and
NormalEstimation (k = 30) of all 1024 views, dealt to 12 streams (the targets
keep their neighbour rows for ICP), then the proposal arm (learned pose
proposal, point-to-plane ICP 2 cm then 1 cm, plain ICP as the fallback, whose
pairs known after the 2 cm stage run on a second context beside the 1 cm
stage) and, beside it, the plain arm (centroid alignment, point-to-plane ICP
5 cm then 1 cm), each over all pairs in batched ICP calls.  A pair counts as
aligned when ICP converged and RMS |T_est p - T_gt p| over the source points
is <= 1 mm.  value = aligned pairs/s of preprocessing + the proposal arm;
e2e = the same from pinned host images (H2D inside the timed region).  L2 is
flushed (256 MB write) before every stage.  --impl reference times the
oracle's plain method (the reference path's CPU restatement, all host
threads), one pair per step.

--workload config1 keeps the single-pair pipeline (10-frame bursts, VoxelGrid
1 mm, SOR k=50, NormalEstimation k=30 from SOR's lists, point-to-plane ICP);
the other workloads are the turntable cycle, the point-sample proposal
evaluation, the SfM filters and the super-resolution front end.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "aligned cloud pairs/sec at ≤1 mm RMSE: proposal+ICP vs plain GPU ICP"
WORKLOAD = ("burst(10x640x480 u16) ZE-mean -> back-projection -> VoxelGrid 1mm -> SOR k=50 mul=1 -> NE k=30 "
            "-> point-to-plane ICP (20 deg + 3 cm, d_max 3 cm, <=100 it), 1 pair per step, plain GPU ICP "
            "(identity initial guess, no learned proposal)")
ICP = dict(max_correspondence_distance=0.03, max_iterations=100, transformation_epsilon=1e-8,
           euclidean_fitness_epsilon=1e-6, point_to_plane=True)
RMSE_LIMIT = 1e-3


class Clocks:
    """nvidia-smi sampling during the timed region (median SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.dev = device
        self.rows: list[list[str]] = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", "200"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._proc = None

    def _read(self):
        for line in self._proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self) -> dict:
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def make_inputs(seed: int = 1):
    from lowcost3dreconstruction_gb300 import synthetic as S
    pr = S.config1_pair(seed)
    return pr


def rmse_from_moments(T_est, T_gt, m1, m2, n) -> float:
    """RMS |(T_est - T_gt) p| from the source's first/second moments."""
    D = np.asarray(T_est, np.float64) - np.asarray(T_gt, np.float64)
    A, b = D[:3, :3], D[:3, 3]
    ms = np.trace(A @ m2 @ A.T) + 2.0 * b @ (A @ m1) + b @ b
    return float(np.sqrt(max(ms, 0.0)))


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops", 1900.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


# ---------------------------------------------------------------- GPU arm
def gpu_arm(args, rank: int, world: int, dist) -> dict | None:
    import torch

    from lowcost3dreconstruction_gb300 import _lib as L
    from lowcost3dreconstruction_gb300.core import Context, xyz_of

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    pr = make_inputs(1 + rank)
    # The two captures of a pair are independent: each runs on its own context
    # (CUDA stream) from its own host thread, so their kernels overlap; the
    # pair's ICP runs on the first context after an event wait on the second.
    ctxs = [Context(dev), Context(dev)]
    ctx = ctxs[0]
    streams = [torch.cuda.ExternalStream(c.stream, device=dev) for c in ctxs]
    params = ctx.depth_params(L.KINECT_V1, 640, 480, frames=10, scale=0.001, depth_max=4000.0, normals=False)
    icp_params = ctx.icp_params(**ICP)
    frames = [np.ascontiguousarray(pr.src_frames), np.ascontiguousarray(pr.tgt_frames)]
    d_frames = [torch.from_numpy(f.view(np.uint8).reshape(-1)).to(f"cuda:{dev}") for f in frames]
    h_frames = [torch.from_numpy(f.view(np.uint8).reshape(-1)).pin_memory() for f in frames]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    stage_ms = {}
    sor_n: list[int] = []  # SOR input sizes, one per k_sor_dist launch
    pool = ThreadPoolExecutor(max_workers=2)

    def capture(k: int, src_is_device: bool, timing: dict | None):
        c, st = ctxs[k], streams[k]
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)] if timing is not None else None
        with torch.cuda.stream(st):
            if ev: ev[0].record(st)
            cl = (c.backproject_device(d_frames[k].data_ptr(), params) if src_is_device
                  else c.backproject(h_frames[k].numpy().view(np.uint16), params))
            if ev: ev[1].record(st)
            v = c.voxel_grid(cl, 0.001)
            sor_n.append(len(v))
            if ev: ev[2].record(st)
            inl, _, _ = c.sor(v, 50, 1.0)
            if ev: ev[3].record(st)
            nrm = c.normals(inl, 30)
            if ev: ev[4].record(st)
        return nrm, ev

    def step(device_inputs: bool, timing: dict | None = None, start=None):
        if start is not None:
            streams[1].wait_event(start)  # the second stream starts with the timed region
        futs = [pool.submit(capture, k, device_inputs, timing) for k in (0, 1)]
        (src, ev0), (tgt, ev1) = [f.result() for f in futs]
        done1 = torch.cuda.Event()
        done1.record(streams[1])
        streams[0].wait_event(done1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(streams[0]):
            e0.record(streams[0])
            res = ctx.icp(src, tgt, icp_params)
            e1.record(streams[0])
        streams[0].synchronize()
        if timing is not None:
            streams[1].synchronize()
            for ev in (ev0, ev1):
                for name, a, b in (("backproject", 0, 1), ("voxel", 1, 2), ("sor", 2, 3), ("normals", 3, 4)):
                    timing[name] = timing.get(name, 0.0) + ev[a].elapsed_time(ev[b])
            timing["icp"] = timing.get("icp", 0.0) + e0.elapsed_time(e1)
            timing["icp_iters"] = timing.get("icp_iters", 0) + res.iterations
        return src, tgt, res

    # moments of the source cloud for the RMSE check (outside the timed region)
    src0, tgt0, res0 = step(True)
    # launch shapes for this cloud size and device (untimed; both contexts use them)
    v0 = ctx.voxel_grid(ctx.backproject_device(d_frames[0].data_ptr(), params), 0.001)
    tune = ctx.autotune(v0, tgt0)
    ctxs[1].tune_set(tune["sor_warps"], tune["normals_warps"], tune["icp_blocks_per_sm"])
    del v0
    xs = xyz_of(src0.download()).astype(np.float64)
    m1, m2, nsrc = xs.mean(0), (xs.T @ xs) / len(xs), len(xs)
    ntgt = len(tgt0)
    for _ in range(max(args.warmup, 3)):
        step(True)
        step(False)

    def timed(device_inputs: bool, timing: dict | None):
        aligned = 0
        total_ms = 0.0
        launches0 = sum(c.launches for c in ctxs)
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ea.record(streams[0])
            _, _, res = step(device_inputs, timing, start=ea)
            eb.record(streams[0])
            eb.synchronize()
            total_ms += ea.elapsed_time(eb)
            r = rmse_from_moments(res.transform64, pr.T_gt, m1, m2, nsrc)
            aligned += int(res.converged and r <= RMSE_LIMIT)
        return aligned, total_ms, sum(c.launches for c in ctxs) - launches0, r, res

    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    sor_n.clear()
    for c in ctxs:
        c.kernel_timing(True)
    # A step is ~4.5 ms: the K-step block is repeated until about 200 steps
    # have run, and the block at the median rate is reported (its stage times
    # and kernel timings are the whole run's averages).
    blocks = []
    for _ in range(max(1, -(-200 // args.steps))):
        blocks.append(timed(True, stage_ms))
    nblocks = len(blocks)
    blocks.sort(key=lambda b: b[0] / b[1])
    aligned, dev_ms, launches, last_rmse, last_res = blocks[len(blocks) // 2]
    kt = [c.kernel_time(L.KT_SOR_KNN) for c in ctxs]
    sor_ms, sor_launches = sum(t[0] for t in kt), sum(t[1] for t in kt)
    for c in ctxs:
        c.kernel_timing(False)
    sor_sizes = list(sor_n)
    clk = clocks.stop()
    torch.cuda.synchronize()
    e2e_aligned, e2e_ms, _, _, _ = timed(False, None)
    if dist is not None:
        # replicas: the slowest rank's clock, every rank's aligned pairs
        from lowcost3dreconstruction_gb300.replicas import combine
        dist.barrier()
        (dev_ms, e2e_ms), (aligned, e2e_aligned) = combine(dist, [dev_ms, e2e_ms], [aligned, e2e_aligned],
                                                           device=f"cuda:{dev}")
    if rank != 0:
        pool.shutdown()
        for c in ctxs:
            c.close()
        return None

    steps_total = args.steps * world
    value = aligned / (dev_ms / 1000.0)
    e2e_value = e2e_aligned / (e2e_ms / 1000.0)
    # Roofline of the dominant kernel, k_sor_dist (the unordered k-NN pass of
    # StatisticalOutlierRemoval, k = 51 including the point itself): its launches
    # are bracketed by CUDA events on the library's stream during the timed
    # region.  Algorithmic bytes per launch on n points in nleaf leaves of 32:
    # query points 16 n + reference points 16 n + the mean distance out 4 n +
    # the leaf boxes, 32 B per leaf.  The neighbour lists it also writes for the
    # inliers' normals (8 B per key) are a design choice, not algorithmic: they
    # show in the measured traffic.
    def sor_bytes(n: int) -> int:
        return 36 * n + 32 * ((n + 31) // 32)
    assert sor_launches == len(sor_sizes), (sor_launches, len(sor_sizes))
    bytes_per_launch = sum(sor_bytes(n) for n in sor_sizes) / max(1, len(sor_sizes))
    launch_ms = sor_ms / max(1, sor_launches)
    pk = peaks()
    achieved = bytes_per_launch / (launch_ms * 1e-3) / 1e9
    ncu_traffic, ncu_context = None, {}
    tfile = ROOT / "profiles" / "k_sor_dist_config1_traffic.json"
    if tfile.exists():
        tj = json.loads(tfile.read_text())
        ncu_traffic = tj.get("bytes_per_launch")
        ncu_context = {k: tj[k] for k in ("l2_hit_rate", "issue_active", "bound_note") if k in tj}
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points_src": nsrc, "points_tgt": ntgt, "l2": "flushed between steps "
                   "(256 MB write)", "icp": ICP, "rmse_limit_m": RMSE_LIMIT, "pairs_aligned": int(aligned),
                   "timed_blocks": {"blocks": nblocks, "steps_per_block": args.steps, "reported": "median block",
                                    "pairs_per_s_min_max": [round(blocks[0][0] / (blocks[0][1] / 1000.0), 3),
                                                            round(blocks[-1][0] / (blocks[-1][1] / 1000.0), 3)]},
                   "pairs_timed": steps_total, "last_rmse_m": last_rmse, "last_icp_iterations": last_res.iterations,
                   "parallelism": f"replicas x{world}; per pair the two captures run concurrently on two streams",
                   "stage_ms_per_step": {k: round(v / (args.steps * nblocks), 4) for k, v in stage_ms.items()
                                         if k != "icp_iters"},
                   "stage_ms_note": "summed over both captures, which overlap in time",
                   "icp_iterations_per_step": stage_ms.get("icp_iters", 0) / (args.steps * nblocks),
                   "launch_shapes": {k: tune[k] for k in ("sor_warps", "normals_warps", "icp_blocks_per_sm")},
                   "autotune_ms": {k: tune[k] for k in ("sor_ms", "normals_ms", "icp_ms")}},
        "roofline": {"kernel": "k_sor_dist (SOR k-NN pass, k=51)", "bound": "hbm",
                     "achieved": round(achieved, 2), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / pk["hbm_gbs"], 5), "peak_src": pk["src"],
                     "algorithmic_bytes_per_launch": int(bytes_per_launch), "avg_launch_ms": round(launch_ms, 5),
                     "launches": int(sor_launches), "traffic": ncu_traffic, **ncu_context},
        "e2e": {"value": round(e2e_value, 3), "unit": "pairs/s",
                "h2d_bytes_per_step": int(sum(f.nbytes for f in frames)), "d2h_bytes_per_step": 4 * 16 + 8 * 16},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(pr, sample_pairs=1)
    pool.shutdown()
    del src0, tgt0
    for c in ctxs:
        c.close()
    return out


# ------------------------------------------------- batched turntable cycle
def turntable_arm(args) -> dict:
    """Config 2: a 36-view turntable cycle of one object of the superquadric
    family (extents 0.1-0.4 m, a block and two balls attached, whose
    self-occlusion changes from view to view), rendered on the device with a
    Kinect v1 camera at the super-resolution tools' x2 resample factor
    (1280 x 960, ~0.8 mm pixel spacing), back-projected, VoxelGrid 1 mm and
    normals k=30 (untimed preprocessing).  One step: the 36 consecutive
    point-to-plane ICP pairs (2 cm, <= 100 iterations, from the nominal 10-deg
    step with a seeded 2 deg + 3 mm coarse error) in one lcr_icp_batch call --
    one CUDA-graph WHILE loop of batched rounds -- then accumulation of the
    cycle: every view moved into view 0's frame by the chained ICP transforms
    and merged in turn with accumulate_clouds' crop (1 mm) + SOR (k=50, 1.0)
    (accumulate_clouds.cpp:100-127).  The same pairs one lcr_icp call at a time
    are timed beside it, and so is the ICP round itself on tiny clouds (the
    launch cost of the round's kernels)."""
    import torch

    from lowcost3dreconstruction_gb300 import _lib as L
    from lowcost3dreconstruction_gb300 import synthetic as S
    from lowcost3dreconstruction_gb300.core import Context, points_from_xyz, xyz_of
    torch.cuda.set_device(0)
    views, step = 36, 10.0
    ctx = Context(0)
    cam = S.upsampled(S.KINECT_V1, 2)
    buf = torch.empty(views * cam["width"] * cam["height"], dtype=torch.int16, device="cuda:0")
    prm_bp = ctx.depth_params(L.KINECT_V1, cam["width"], cam["height"], fx=cam["fx"], fy=cam["fy"], cx=cam["cx"],
                              cy=cam["cy"], depth_min=300.0, depth_max=9000.0, scale=0.001, normals=False)
    pix = cam["width"] * cam["height"]

    def render(seed):
        torch.cuda.synchronize()
        P = ctx.synthetic_turntable(seed, views, step, L.KINECT_V1, cam["width"], cam["height"], cam["fx"],
                                    cam["fy"], cam["cx"], cam["cy"], buf.data_ptr(), distance=0.8)
        cl = [ctx.voxel_grid(ctx.backproject_device(buf.data_ptr() + 2 * pix * v, prm_bp), 0.001)
              for v in range(views)]
        return P.astype(np.float64), cl

    # the object: the largest of a few seeded draws (the family spans 40k-300k points per view at 1 mm)
    best = None
    for seed in range(8):
        P, cl = render(7000 + seed)
        m = max(len(c) for c in cl)
        if best is None or m > best[0]:
            best = (m, seed)
        for c in cl:
            c.free()
    P, vox = render(7000 + best[1])
    cl = [ctx.normals(c, 30, keep_neighbours=True) for c in vox]  # every view is a target
    for c in vox:
        c.free()
    src = [cl[(i + 1) % views] for i in range(views)]
    tgt = [cl[i] for i in range(views)]
    T_gt = [P[i] @ np.linalg.inv(P[(i + 1) % views]) for i in range(views)]
    xyz = [xyz_of(c.download()).astype(np.float64) for c in src]
    rng = np.random.default_rng(7)
    guesses = []
    for T in T_gt:
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        a = np.deg2rad(2.0)
        K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        E = np.eye(4)
        E[:3, :3] = np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * K @ K
        E[:3, 3] = rng.normal(size=3) * 0.003 / np.sqrt(3)
        guesses.append(E @ T)
    guesses = np.stack(guesses).astype(np.float32)
    prm = ctx.icp_params(max_correspondence_distance=0.02, max_iterations=100, transformation_epsilon=1e-10,
                         euclidean_fitness_epsilon=1e-8, point_to_plane=True)
    stream = torch.cuda.ExternalStream(ctx.stream, device=0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")

    def aligned(res):
        return sum(int(r.converged and S.rmse(r.transform64, T_gt[i], xyz[i]) <= RMSE_LIMIT) for i, r in enumerate(res))

    def accumulate(res):
        # view v in view 0's frame: T_0v = T_01 T_12 ... T_(v-1)v, T_(i)(i+1) the ICP result of pair i
        acc = ctx.transform(cl[0], np.eye(4, dtype=np.float32))
        Tc = np.eye(4)
        for v in range(1, views):
            Tc = Tc @ res[v - 1].transform64
            moved = ctx.transform(cl[v], Tc.astype(np.float32))
            out, rem = ctx.accumulate(moved, acc, radius=0.001, k=50, std_mul=1.0)
            acc.free()
            rem.free()
            moved.free()
            acc = out
        return acc

    def run(batch: bool, accum: bool = True):
        res = ctx.icp_batch(src, tgt, prm, guesses=guesses) if batch else \
            [ctx.icp(s_, t_, prm, guess=g) for s_, t_, g in zip(src, tgt, guesses)]
        acc = accumulate(res) if accum else None
        return res, acc

    def timed(fn, steps):
        total, last = 0.0, None
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ea.record(stream)
            last = fn()
            eb.record(stream)
            eb.synchronize()
            total += ea.elapsed_time(eb)
        return total, last

    for _ in range(max(args.warmup, 3)):
        _, acc = run(True)
        acc.free()
    clocks = Clocks(0)
    clocks.start()
    l0 = ctx.launches
    ms_all, (res, acc) = timed(lambda: run(True), args.steps)
    launches = (ctx.launches - l0) // args.steps
    clk = clocks.stop()
    n_acc = len(acc)
    acc.free()
    ms_icp, (res_icp, _) = timed(lambda: run(True, accum=False), args.steps)
    ms_seq, (res_seq, _) = timed(lambda: run(False, accum=False), max(1, min(args.steps, 3)))
    seq_steps = max(1, min(args.steps, 3))
    ok = aligned(res)
    rounds = max(r.iterations for r in res_icp)
    # the round's launch cost: the same batch call on 36 pairs of 64-point clouds
    tiny = [ctx.upload(points_from_xyz(xyz[i][o:: max(1, len(xyz[i]) // 64)][:64])) for i in range(views)
            for o in (0, 1)]
    tiny_n = [ctx.normals(c, 8) for c in tiny]
    tprm = ctx.icp_params(max_correspondence_distance=0.02, max_iterations=30, transformation_epsilon=0.0,
                          euclidean_fitness_epsilon=-1.0, point_to_plane=True, compute_fitness=False)
    ctx.icp_batch(tiny_n[0::2], tiny_n[1::2], tprm)
    ms_tiny, rt = timed(lambda: ctx.icp_batch(tiny_n[0::2], tiny_n[1::2], tprm), 3)
    tiny_rounds = max(r.iterations for r in rt)
    sizes = [len(c) for c in src]
    # CPU baseline: the oracle's point-to-plane ICP (own k-d tree, OpenMP over
    # the host cores) on the first pairs, about 10 s of them
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    t0 = time.perf_counter()
    cpu_ok = cpu_n = 0
    while cpu_n < views and time.perf_counter() - t0 < 10.0:
        i = cpu_n
        r = O.icp(src[i].download(), tgt[i].download(), max_corr_dist=0.02, max_iterations=100,
                  transformation_epsilon=1e-10, euclidean_fitness_epsilon=1e-8, point_to_plane=True,
                  guess=guesses[i].astype(np.float64))
        cpu_ok += int(r["converged"] and S.rmse(r["transform"], T_gt[i], xyz[i]) <= RMSE_LIMIT)
        cpu_n += 1
    cpu_dt = time.perf_counter() - t0
    for c in tiny + tiny_n + cl:
        c.free()
    ctx.close()
    K = args.steps
    v = ok * K / (ms_all / 1000.0)
    return {"metric": METRIC, "value": round(v, 3), "unit": "pairs/s", "n_gpus": 1, "steps": K,
            "warmup": args.warmup, "ms_per_step": round(ms_all / K, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "config 2: 36-view turntable cycle (10 deg steps) of one superquadric object with a "
                                   "block and two balls, Kinect v1 x2 (1280x960) depth images rendered on the device, "
                                   "VoxelGrid 1 mm, normals k=30 (untimed); per step the 36 consecutive point-to-plane "
                                   "ICP pairs (2 cm, <=100 it, nominal step + 2 deg / 3 mm coarse error) in one "
                                   "lcr_icp_batch call, then accumulation of the cycle (chained transforms, "
                                   "accumulate_clouds crop 1 mm + SOR k=50)",
                       "points_per_cloud": [min(sizes), int(np.median(sizes)), max(sizes)],
                       "pairs_aligned_per_step": ok, "pairs": views, "accumulated_points": n_acc,
                       "ms_per_step_by_stage": {"icp_batch": round(ms_icp / K, 3),
                                                "accumulation": round((ms_all - ms_icp) / K, 3)},
                       "icp_rounds": rounds,
                       "icp_round_ms": round(ms_icp / K / max(rounds, 1), 4),
                       "icp_round_launch_cost_ms": round(ms_tiny / 3 / max(tiny_rounds, 1), 4),
                       "icp_round_note": "round = one iteration of every live pair: 5 kernels in a CUDA-graph WHILE "
                                         "body; the launch cost is the same call on 36 pairs of 64-point clouds",
                       "sequential_lcr_icp_pairs_per_s": round(aligned(res_seq) * seq_steps / (ms_seq / 1000.0), 3),
                       "l2": "256 MB flush before every step"},
            "gpu_launches": launches, "clocks": clk,
            "cpu_baseline": {"value": round(cpu_ok / cpu_dt, 3), "unit": "pairs/s", "cores": cores, "kind": "port",
                             "sample": f"the oracle's point-to-plane ICP (own k-d tree, OpenMP) on the first {cpu_n} "
                                       f"pairs from the same guesses, {cpu_ok} aligned in {cpu_dt:.2f} s; no "
                                       f"accumulation"}}


# ------------------------------------------- learned proposal vs plain ICP
def proposal_arm(args) -> dict:
    """Config 3 evaluation: 2000 held-out pairs of the config-2 objects
    (superquadrics with a block and two balls, yaw uniform in +-180 deg, tilt
    +-20 deg, translation +-10 cm), captured as Kinect v1 640x480 depth images
    by lcr_synthetic_depth at ~20k pixels per view (seeds disjoint from the
    fine-tuning's), back-projected and given normals k=30 (untimed).  Both arms
    run per step over all pairs: plain GPU ICP from centroid alignment, and the
    trained proposal followed by ICP with plain ICP as the fallback; both refine
    with batched point-to-plane ICP (a first stage, then 1 cm).  value = aligned
    pairs/s of proposal+ICP; the plain arm, and the convergence rate of both,
    are reported beside it."""
    import torch

    from lowcost3dreconstruction_gb300 import _lib as L
    from lowcost3dreconstruction_gb300 import synthetic as S
    from lowcost3dreconstruction_gb300 import train_posenet as TP
    from lowcost3dreconstruction_gb300.core import Context
    from lowcost3dreconstruction_gb300.posenet import PoseNet, WEIGHTS
    torch.cuda.set_device(0)
    ctx = Context(0)
    net = PoseNet(ctx)
    net.load(WEIGHTS)
    npairs = args.pairs or 2000
    cam = S.KINECT_V1
    pix = cam["width"] * cam["height"]
    buf = torch.empty(2 * npairs * pix, dtype=torch.int16, device="cuda:0")
    torch.cuda.synchronize()
    T = ctx.synthetic_depth(987_654_321, npairs, L.KINECT_V1, cam["width"], cam["height"], cam["fx"], cam["fy"],
                            cam["cx"], cam["cy"], buf.data_ptr(),
                            points=np.full(npairs, TP.EVAL_POINTS, np.float32))
    bp = ctx.depth_params(L.KINECT_V1, cam["width"], cam["height"], fx=cam["fx"], fy=cam["fy"], cx=cam["cx"],
                          cy=cam["cy"], depth_min=300.0, depth_max=9000.0, scale=0.001, normals=False)
    clouds = []
    for v in range(2 * npairs):
        c = ctx.backproject_device(buf.data_ptr() + 2 * pix * v, bp)
        clouds.append(ctx.normals(c, 30, keep_neighbours=v % 2 == 1))
        c.free()
    del buf
    srcs, tgts = clouds[0::2], clouds[1::2]
    sizes = np.array([len(c) for c in srcs])
    stream = torch.cuda.ExternalStream(ctx.stream, device=0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")

    def plain():
        return TP.refine(ctx, srcs, tgts, TP.centroid_guesses(net, srcs, tgts))

    ctx2 = Context(0)  # runs the early fallback pairs beside the 1 cm stage
    stream2 = torch.cuda.ExternalStream(ctx2.stream, device=0)

    def proposal():
        return TP.propose_refine(ctx, net, srcs, tgts, ctx2)

    for _ in range(args.warmup):
        plain()
        proposal()
    steps = max(1, min(args.steps, 5))
    out = {}
    clocks = Clocks(0)
    clocks.start()
    for arm in ("plain", "proposal"):
        total, ok, fbs, conv = 0.0, 0, 0, 0
        l0 = ctx.launches + ctx2.launches
        if arm == "proposal":
            ctx.kernel_timing(True)
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ea.record(stream)
            stream2.wait_event(ea)
            if arm == "plain":
                res = plain()
            else:
                res, nfb = proposal()
                fbs += nfb
            eb.record(stream)
            eb.synchronize()
            total += ea.elapsed_time(eb)
            good, _ = TP.aligned(ctx, srcs, res, T)
            ok += int(good.sum())
            conv += sum(int(r.converged) for r in res)
        launches = ctx.launches + ctx2.launches - l0
        enc = ctx.kernel_time(L.KT_ENCODE) if arm == "proposal" else (0.0, 0)
        ctx.kernel_timing(False)
        out[arm] = dict(pairs_per_s=ok / (total / 1000.0), ms=total / steps, aligned=ok / steps,
                        converged=conv / steps, fallbacks=fbs / steps, launches=launches // steps, enc=enc)
    clk = clocks.stop()
    # CPU baseline: the plain method (centroid alignment, then the same two
    # point-to-plane ICP stages) through the oracle, OpenMP over the host
    # cores, on the first pairs up to 400k points in all
    from lowcost3dreconstruction_gb300.core import xyz_of
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    sample, pts_in = [], 0
    for i in range(npairs):
        if sample and pts_in + 2 * int(sizes[i]) > 400_000:
            break
        sample.append(i)
        pts_in += 2 * int(sizes[i])
    hs = [srcs[i].download() for i in sample]
    ht = [tgts[i].download() for i in sample]
    t0 = time.perf_counter()
    cpu_ok = 0
    for j, i in enumerate(sample):
        G = np.eye(4)
        G[:3, 3] = O.centroid(ht[j])[:3].astype(np.float64) - O.centroid(hs[j])[:3].astype(np.float64)
        r1 = O.icp(hs[j], ht[j], max_corr_dist=0.05, max_iterations=100, transformation_epsilon=1e-8,
                   euclidean_fitness_epsilon=1e-7, point_to_plane=True, guess=G)
        r2 = O.icp(hs[j], ht[j], max_corr_dist=0.01, max_iterations=50, transformation_epsilon=1e-9,
                   euclidean_fitness_epsilon=1e-8, point_to_plane=True, guess=r1["transform"])
        r = r2 if r2["state"] != 5 else r1
        cpu_ok += int(r["converged"] and S.rmse(r["transform"], T[i], xyz_of(hs[j])) <= RMSE_LIMIT)
    cpu_dt = time.perf_counter() - t0
    pr = peaks()
    enc_ms, enc_n = out["proposal"]["enc"]
    flops = 2 * npairs * 1024 * (2 * (64 * 128 + 128 * 1024))
    points = int(2 * sizes.sum())
    achieved = flops / (enc_ms / enc_n / 1000.0) / 1e12 if enc_n else None
    bf16_peak = pr.get("bf16_tflops", 1900.0)
    P = out["proposal"]
    ctx.close()
    return {"metric": METRIC, "value": round(P["pairs_per_s"], 3), "unit": "pairs/s", "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "ms_per_step": round(P["ms"], 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (proposal network) + f32/f64 (ICP)", "data": "synthetic",
            "config": {"workload": f"config 3 evaluation: {npairs} held-out pairs of the config-2 objects "
                                   "(superquadric + block + 2 balls, yaw +-180 deg, tilt +-20 deg, translation "
                                   "+-10 cm) as Kinect v1 640x480 depth images rendered on the device, "
                                   f"~{TP.EVAL_POINTS} pixels per view, back-projected with normals k=30 (untimed); "
                                   "proposal + point-to-plane ICP (2 cm then 1 cm) with plain ICP from centroid "
                                   "alignment as the fallback, all pairs batched per step",
                       "pairs": npairs, "points": points,
                       "points_per_view": [int(sizes.min()), int(np.median(sizes)), int(sizes.max())],
                       "points_per_s": round(points / (P["ms"] / 1000.0), 1),
                       "aligned_per_step": P["aligned"], "converged_per_step": P["converged"],
                       "fallbacks_per_step": P["fallbacks"],
                       "plain_gpu_icp": {"pairs_per_s": round(out["plain"]["pairs_per_s"], 3),
                                         "ms_per_step": round(out["plain"]["ms"], 3),
                                         "aligned_per_step": out["plain"]["aligned"],
                                         "converged_per_step": out["plain"]["converged"],
                                         "icp": "point-to-plane, 5 cm then 1 cm, from centroid alignment"},
                       "proposal_over_plain": round(P["pairs_per_s"] / max(out["plain"]["pairs_per_s"], 1e-9), 3),
                       "l2": "inputs (%.1f GB of clouds) larger than L2; 256 MB flush between steps" % (
                           points * 36 / 1e9)},
            "roofline": {"kernel": "k_encode (fused shared-MLP encoder + max-pool, tcgen05)", "bound": "tensor",
                         "achieved": round(achieved, 1) if achieved else None, "peak": bf16_peak,
                         "unit": "TFLOP/s", "frac": round(achieved / bf16_peak, 4) if achieved else None,
                         "peak_src": pr["src"], "algorithmic_flops_per_launch": flops,
                         "avg_launch_ms": round(enc_ms / enc_n, 5) if enc_n else None, "traffic": None},
            "e2e": None, "gpu_launches": P["launches"], "clocks": clk,
            "cpu_baseline": {"value": round(cpu_ok / cpu_dt, 3), "unit": "pairs/s", "cores": cores, "kind": "port",
                             "sample": f"the plain method (centroid alignment, then point-to-plane ICP 5 cm and 1 cm) "
                                       f"through the oracle on the first {len(sample)} pairs ({pts_in} points), "
                                       f"{cpu_ok} aligned in {cpu_dt:.2f} s"}}


# ------------------------------------------------------ SfM-side filters
def sfm_arm(args) -> dict:
    """The filters of sfm.sh:82-85 on a 1M-point synthetic dense model (a noisy
    2 x 2 m floor of 900k points, three blobs, scattered points): Euclidean
    clusters (tolerance 2 cm, clusters >= 10% of the points), the RANSAC plane
    of the clustered points (1 cm, 1024 hypotheses) and a CropBox; CUDA events
    per filter.  The CPU oracle runs the same filters on a 100k-point sample."""
    import torch

    from lowcost3dreconstruction_gb300.core import Context, points_from_xyz
    from oracle import sfm as OS
    torch.cuda.set_device(0)
    rng = np.random.default_rng(11)
    n_floor = 900_000
    floor = np.c_[rng.uniform(-1, 1, (n_floor, 2)), rng.normal(0, 0.003, n_floor)]
    blobs = [rng.normal(c, 0.04, (m, 3)) for c, m in (((0.3, 0.2, 0.4), 50_000), ((-0.4, -0.1, 0.5), 35_000),
                                                          ((0.0, 0.6, 0.3), 14_000))]
    xyz = np.concatenate([floor] + blobs + [rng.uniform(-1, 1, (1000, 3))]).astype(np.float32)
    xyz = xyz[rng.permutation(len(xyz))]
    n = len(xyz)
    ctx = Context(0)
    cloud = ctx.upload(points_from_xyz(xyz))
    stream = torch.cuda.ExternalStream(ctx.stream, device=0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    c0 = ctx.centroid(cloud)

    def step():
        labels, k, kept, rest = ctx.euclidean_clusters(cloud, 0.02, int(n * 0.1), n)
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record(stream)
        coef, m, plane, off = ctx.plane_segment(kept, 0.01, 1024, 0)
        e2 = torch.cuda.Event(enable_timing=True)
        e2.record(stream)
        inside, outside = ctx.crop_box(cloud, c0[:3] - 0.5, c0[:3] + 0.5)
        return k, len(kept), m, len(inside), e1, e2

    for _ in range(args.warmup):
        step()
    ms = {"clusters": 0.0, "plane": 0.0, "crop": 0.0}
    l0 = ctx.launches
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        k, nk, m, ni, e1, e2 = step()
        e3 = torch.cuda.Event(enable_timing=True)
        e3.record(stream)
        e3.synchronize()
        ms["clusters"] += e0.elapsed_time(e1)
        ms["plane"] += e1.elapsed_time(e2)
        ms["crop"] += e2.elapsed_time(e3)
    total = sum(ms.values()) / args.steps
    launches = (ctx.launches - l0) // args.steps
    # CPU oracle on a bounded sample
    sample = xyz[:100_000]
    t0 = time.perf_counter()
    OS.euclidean_clusters(sample, 0.02, 10_000, len(sample))
    t1 = time.perf_counter()
    OS.plane_segment(sample, 0.01, 64, 0)
    t2 = time.perf_counter()
    ctx.close()
    cpu_pps = len(sample) / ((t1 - t0) + (t2 - t1) * 1024 / 64)
    return {"metric": "points/s through the SfM filters (Euclidean clusters + RANSAC plane + CropBox)",
            "value": round(n / (total / 1000.0), 1), "unit": "points/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 plane refit)", "data": "synthetic",
            "config": {"workload": "1M-point dense model: clusters (2 cm, >= 10%), plane of the clustered points "
                                   "(1 cm, 1024 hypotheses), CropBox (0.5 m around the centroid)",
                       "points": n, "clusters": int(k), "clustered_points": int(nk), "plane_inliers": int(m),
                       "cropped_points": int(ni),
                       "ms_per_filter": {key: round(v / args.steps, 3) for key, v in ms.items()},
                       "l2": "256 MB flush between steps"},
            "roofline": None, "e2e": None, "gpu_launches": launches,
            "cpu_baseline": {"value": round(cpu_pps, 1), "unit": "points/s", "cores": 1, "kind": "port",
                             "sample": "the oracle (scipy cKDTree + connected components, numpy RANSAC scaled from "
                                       "64 to 1024 hypotheses) on the first 100k points"}}


def sr_arm(args) -> dict:
    """The super-resolution front end of capture/super_resolution (:236-314) on
    the reference's default capture: 18 views, each a burst of 16 Kinect v1
    frames of 640 x 480, fused at resample factor 4.  A frame is a smooth
    depth scene seen under a small random rigid motion (<= 0.4 deg, <= 0.8 px)
    with 0.3 mm noise.  One step is one view through lcr_super_resolve from
    host buffers (upload, ECC registration of 15 frames, warp, upsampling,
    ZE-mean, Lanczos-4, download); CUDA events on the library's stream.  The
    CPU baseline is the C restatement on two full views over all host cores."""
    import torch

    from lowcost3dreconstruction_gb300.core import Context
    torch.cuda.set_device(0)
    h, w, F, views = 480, 640, 16, 18
    rng = np.random.default_rng(21)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)

    def scene(X, Y):
        return (1000 + 120 * np.sin(X / 27.0) * np.cos(Y / 21.0) + 60 * np.exp(-((X - 320) ** 2 + (Y - 240) ** 2)
                                                                            / 1800.0) + 0.3 * X - 0.2 * Y)
    bursts = []
    for v in range(views):
        fr = []
        for f in range(F):
            a = 0.0 if f == 0 else np.deg2rad(rng.uniform(-0.4, 0.4))
            tx, ty = (0.0, 0.0) if f == 0 else rng.uniform(-0.8, 0.8, 2)
            X = np.cos(a) * x - np.sin(a) * y + tx + 7 * v
            Y = np.sin(a) * x + np.cos(a) * y + ty
            fr.append(np.clip(np.rint(scene(X, Y) + rng.normal(0, 0.3, x.shape)), 0, 65535).astype(np.uint16))
        bursts.append(np.stack(fr))
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=0)
    for i in range(args.warmup):
        ctx.super_resolve(bursts[i % views])
    l0 = ctx.launches
    iters = []
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        _, _, _, it = ctx.super_resolve(bursts[i % views])
        iters.append(int(it.sum()))
    e1 = torch.cuda.Event(enable_timing=True)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = (ctx.launches - l0) // args.steps
    ctx.close()
    # CPU baseline: the C restatement (oracle/sr_oracle.cpp) on two full views,
    # the frames registering in parallel over the host cores as the
    # reference's OpenMP loop does
    from oracle import oracle as OC
    cores = os.cpu_count() or 1
    OC.set_threads(cores)
    t0 = time.perf_counter()
    for v in range(2):
        OC.super_resolve(bursts[v], 4)
    dt = (time.perf_counter() - t0) / 2
    return {"metric": "depth views/s through the super-resolution front end (ECC + warp + ZE-mean + Lanczos-4)",
            "value": round(1000.0 / ms, 3), "unit": "views/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 ECC sums)", "data": "synthetic",
            "config": {"workload": "18 views x 16-frame 640x480 Kinect v1 bursts, resample factor 4, ECC <= 200 "
                                   "iterations, eps 1e-12", "mean_ecc_iterations_per_view": round(
                                       float(np.mean(iters)), 1),
                       "l2": "each view's burst (9.8 MB in, 4x upsampled 19.7 MB float) is uploaded per step"},
            "roofline": None,
            "e2e": {"value": round(1000.0 / ms, 3), "unit": "views/s", "h2d_bytes_per_step": F * h * w * 2,
                    "d2h_bytes_per_step": h * w * 2 + F * 24 + 8 + F * 4},
            "gpu_launches": launches,
            "cpu_baseline": {"value": round(1.0 / dt, 5), "unit": "views/s", "cores": cores, "kind": "port",
                             "sample": "the C restatement (oracle/sr_oracle.cpp, OpenMP over the frames) on the "
                                       f"first two views of the same workload, {2 * dt:.2f} s"}}


# ---------------------------------------- config 4: large uneven mixed batch
# Kinect v1 (uint16 mm) and Kinect v2 (float32 mm) cameras; an image at
# upsampling factor s is what the super-resolution tools' resample factor
# gives (super_resolution.cpp:274-314): s-times the pixels per axis with the
# intrinsics scaled to match.
C4_CAMERAS = {"kinect_v1": dict(model=0, width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5),
              "kinect_v2": dict(model=1, width=512, height=424, fx=365.0, fy=365.0, cx=255.5, cy=211.5)}
C4_SEED = 4
C4_DEPTH_RANGE_MM = (300.0, 9000.0)


def config4_layout(npairs: int = 512, seed: int = 4, area_typ: float = 0.15, z_min: float = 0.5):
    """Pair i: points wanted per view log-uniform in [5k, 500k], the camera
    alternating Kinect v1 / v2, and the smallest factor s in {1, 2, 4} that puts
    an object of typical surface area (0.15 m^2, projected area a quarter of
    that) at least z_min from the camera for that many pixels."""
    rng = np.random.default_rng(seed)
    want = np.exp(rng.uniform(np.log(5e3), np.log(5e5), npairs))
    cams = ["kinect_v1" if i % 2 == 0 else "kinect_v2" for i in range(npairs)]
    f = np.array([C4_CAMERAS[c]["fx"] for c in cams])
    need = z_min * np.sqrt(4.0 * want / area_typ) / f
    factor = np.clip(2 ** np.ceil(np.log2(np.maximum(need, 1.0))), 1, 4).astype(int)
    return want, cams, factor


def config4_camera(cam: str, s: int) -> dict:
    from lowcost3dreconstruction_gb300 import synthetic as S
    return S.upsampled(C4_CAMERAS[cam], s)


class Config4:
    """The 512 depth-image pairs of config 4, rendered on the device and kept
    resident: one buffer per (camera, factor) group, [2 m][h][w] (source and
    target view of each of the group's m pairs), plus pinned host copies for
    the end-to-end form.  Pair i is view 2 j and 2 j + 1 of group g[i]."""

    def __init__(self, ctx, device: int, npairs: int = 512, seed: int = 4, pinned: bool = True):
        import torch
        from lowcost3dreconstruction_gb300 import _lib as L
        self.want, self.cams, self.factor = config4_layout(npairs, seed)
        keys = sorted({(c, int(s)) for c, s in zip(self.cams, self.factor)})
        self.groups = []
        self.where = [None] * npairs
        self.T = np.zeros((npairs, 4, 4), np.float32)
        for gi, (cam, s) in enumerate(keys):
            idx = [i for i in range(npairs) if self.cams[i] == cam and self.factor[i] == s]
            c = config4_camera(cam, s)
            dt = torch.int16 if c["model"] == L.KINECT_V1 else torch.float32
            buf = torch.empty(2 * len(idx) * c["width"] * c["height"], dtype=dt, device=f"cuda:{device}")
            torch.cuda.synchronize()
            T = ctx.synthetic_depth(seed * 1000 + gi, len(idx), c["model"], c["width"], c["height"], c["fx"],
                                    c["fy"], c["cx"], c["cy"], buf.data_ptr(),
                                    points=self.want[idx].astype(np.float32))
            params = ctx.depth_params(c["model"], c["width"], c["height"], frames=1, fx=c["fx"], fy=c["fy"],
                                      cx=c["cx"], cy=c["cy"], depth_min=C4_DEPTH_RANGE_MM[0],
                                      depth_max=C4_DEPTH_RANGE_MM[1], scale=0.001 if c["model"] == L.KINECT_V1
                                      else 1.0, normals=False)
            host = buf.cpu().pin_memory() if pinned else None
            self.groups.append(dict(cam=cam, s=s, camera=c, buf=buf, host=host, params=params, pairs=idx,
                                    view_bytes=c["width"] * c["height"] * buf.element_size()))
            for j, i in enumerate(idx):
                self.where[i] = (gi, j)
                self.T[i] = T[j]

    @property
    def npairs(self) -> int:
        return len(self.where)

    def view(self, i: int, side: int):
        """(device pointer, host array or None, params) of view side (0 source, 1 target) of pair i."""
        gi, j = self.where[i]
        g = self.groups[gi]
        off = (2 * j + side) * g["view_bytes"]
        host = None
        if g["host"] is not None:
            n = g["view_bytes"] // g["buf"].element_size()
            host = g["host"][(2 * j + side) * n:(2 * j + side + 1) * n].numpy()
        return g["buf"].data_ptr() + off, host, g["params"]

    def image_bytes(self) -> int:
        return sum(g["buf"].numel() * g["buf"].element_size() for g in self.groups)

    def host_pair(self, i: int) -> dict:
        """Pair i on the host for the CPU arms: each view's image cropped to the
        box of its nonzero pixels, with the principal point moved to match (the
        back-projection gives the same points), and the exact transform."""
        gi, j = self.where[i]
        g = self.groups[gi]
        cam = g["camera"]
        n = cam["width"] * cam["height"]
        views = []
        for side in (0, 1):
            img = g["buf"][(2 * j + side) * n:(2 * j + side + 1) * n].cpu().numpy().reshape(cam["height"],
                                                                                         cam["width"])
            rows, cols = np.nonzero(img)
            r0, r1 = (rows.min(), rows.max() + 1) if len(rows) else (0, 1)
            c0, c1 = (cols.min(), cols.max() + 1) if len(cols) else (0, 1)
            views.append(dict(image=np.ascontiguousarray(img[r0:r1, c0:c1]), model=cam["model"], fx=cam["fx"],
                              fy=cam["fy"], cx=cam["cx"] - c0, cy=cam["cy"] - r0))
        return dict(views=views, T=self.T[i].astype(np.float64))


PRE_STREAMS = 12  # contexts (streams) the config-4 preprocessing deals its views to (throughput levels off near 12)


def config4_clouds(ctxs, c4: Config4, from_host: bool = False, k: int = 30):
    """Back-projection and NormalEstimation (k = 30) of every view, the views
    dealt round-robin to the contexts (one host thread and one stream each, so
    that several views' launches run on the device at once).  Returns
    (sources, targets) in pair order; every context's work is complete on
    return."""
    from concurrent.futures import ThreadPoolExecutor
    n = c4.npairs
    out = [None] * (2 * n)

    def work(t: int):
        c = ctxs[t]
        for v in range(t, 2 * n, len(ctxs)):
            ptr, host, params = c4.view(v // 2, v % 2)
            bp = c.backproject(host, params) if from_host else c.backproject_device(ptr, params)
            # targets keep their neighbour rows: ICP proves most correspondences from them
            out[v] = c.normals(bp, k, keep_neighbours=v % 2 == 1)
            bp.free()
        c.synchronize()

    with ThreadPoolExecutor(max_workers=len(ctxs)) as ex:
        list(ex.map(work, range(len(ctxs))))
    return out[0::2], out[1::2]


def config4_arm(args, rank: int, world: int, dist) -> dict | None:
    """Config 4: 512 pairs of depth images (the config-2 object family,
    Kinect v1 uint16 / Kinect v2 float32 at upsampling factors 1, 2 and 4,
    5k-500k points per view).  One step: back-projection and NormalEstimation
    (k = 30) of all 1024 views, then each alignment arm over all pairs,
    batched: proposal + point-to-plane ICP with plain ICP as the fallback (the
    headline), and plain GPU ICP from centroid alignment beside it.  value =
    aligned pairs/s of the proposal pipeline: pairs aligned (ICP converged,
    RMS |T_est p - T_gt p| <= 1 mm) over the time of preprocessing plus the
    arm.  L2 is flushed before every stage."""
    import torch

    from lowcost3dreconstruction_gb300 import _lib as L
    from lowcost3dreconstruction_gb300 import train_posenet as TP
    from lowcost3dreconstruction_gb300.core import Context
    from lowcost3dreconstruction_gb300.posenet import WEIGHTS, PoseNet

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    # preprocessing contexts: one host thread and one stream each, so that the
    # per-view launches of several views overlap on the device
    ctxs = [Context(dev) for _ in range(PRE_STREAMS)]
    ctx = ctxs[0]
    streams = [torch.cuda.ExternalStream(c.stream, device=dev) for c in ctxs]
    c4 = Config4(ctx, dev, npairs=args.pairs or 512, seed=4 + rank)
    net = PoseNet(ctx)
    net.load(WEIGHTS)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    T = c4.T

    def preprocess(from_host: bool):
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea.record(streams[0])
        for st in streams[1:]:
            st.wait_event(ea)
        srcs, tgts = config4_clouds(ctxs, c4, from_host=from_host)
        for st in streams[1:]:
            done = torch.cuda.Event()
            done.record(st)
            streams[0].wait_event(done)
        eb.record(streams[0])
        eb.synchronize()
        return srcs, tgts, ea.elapsed_time(eb)

    overlap = {"on": True}

    def proposal(srcs, tgts):
        # the early fallback pairs run on a second (preprocessing) context while
        # the 1 cm stage runs on the first: same results as the sequential order
        return TP.propose_refine(ctx, net, srcs, tgts, ctxs[1] if overlap["on"] else None)

    def plain(srcs, tgts):
        return TP.refine(ctx, srcs, tgts, TP.centroid_guesses(net, srcs, tgts)), 0

    def arm(fn, srcs, tgts):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea.record(streams[0])
        streams[1].wait_event(ea)  # the arm's second context starts inside the timed region
        res, nfb = fn(srcs, tgts)
        eb.record(streams[0])  # after both contexts' work: every ICP call returns synchronised
        eb.synchronize()
        ok, _ = TP.aligned(ctx, srcs, res, T)
        conv = np.array([r.converged for r in res])
        return dict(ms=ea.elapsed_time(eb), ok=int(ok.sum()), conv=int(conv.sum()), fb=nfb)

    def step(from_host: bool = False, both: bool = True):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        srcs, tgts, t_pre = preprocess(from_host)
        out = dict(pre=t_pre, prop=arm(proposal, srcs, tgts))
        if both:
            out["plain"] = arm(plain, srcs, tgts)
        out["sizes"] = np.array([len(c) for c in srcs + tgts])
        for c in srcs + tgts:
            c.free()
        return out

    for _ in range(max(args.warmup, 3)):
        step()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    for c in ctxs:
        c.kernel_timing(True)
    l0 = sum(c.launches for c in ctxs)
    pre = 0.0
    acc = {a: dict(ms=0.0, ok=0, conv=0, fb=0) for a in ("prop", "plain")}
    for _ in range(args.steps):
        o = step()
        pre += o["pre"]
        sizes = o["sizes"]
        for a in acc:
            for key in acc[a]:
                acc[a][key] += o[a][key]
    launches = sum(c.launches for c in ctxs) - l0
    kt = [c.kernel_time(L.KT_NORMALS_KNN) for c in ctxs]
    for c in ctxs:
        c.kernel_timing(False)
    clk = clocks.stop()
    # end to end: the depth images from pinned host memory (one H2D copy per
    # view inside the timed region) through the proposal pipeline, results read
    # back to the host
    e2e_steps = max(1, min(args.steps, 5))
    e2e_ok, e2e_ms = 0, 0.0
    for _ in range(e2e_steps):
        o = step(from_host=True, both=False)
        e2e_ms += o["pre"] + o["prop"]["ms"]
        e2e_ok += o["prop"]["ok"]
    # Roofline of the dominant kernel, k_icp_search (one ICP round's
    # correspondence search over every live pair; ~60% of the step's device
    # time in the launch list).  Inside the CUDA-graph loop no event can
    # bracket it, so one more step runs the rounds from the host loop with each
    # search launch bracketed by CUDA events on the library's stream.  Its
    # algorithmic bytes (the ICP-iteration figure: source points 16 B, target
    # points and normals 32 B, target leaf boxes 32 B per 32 points) are summed
    # over every pair and every round it was live, from the batch calls' own
    # results.
    os.environ["LCR_ICP_GRAPH"] = "0"
    icp_calls = []
    icp_batch = ctx.icp_batch

    def recording_icp_batch(s_, t_, prm_, guesses=None):
        res = icp_batch(s_, t_, prm_, guesses)
        icp_calls.append([(len(a), len(b), r.iterations) for a, b, r in zip(s_, t_, res)])
        return res

    ctx.icp_batch = recording_icp_batch
    ctx.kernel_timing(True)
    overlap["on"] = False  # every search launch on this context, alone on the device
    step()
    overlap["on"] = True
    search_ms, search_launches = ctx.kernel_time(L.KT_ICP_SEARCH)
    ctx.kernel_timing(False)
    ctx.icp_batch = icp_batch
    del os.environ["LCR_ICP_GRAPH"]
    search_bytes = sum(it * (16.0 * ns + 32.0 * nt + 32.0 * ((nt + 31) // 32)) for call in icp_calls
                       for ns, nt, it in call)
    K = args.steps
    t_prop, t_plain = pre + acc["prop"]["ms"], pre + acc["plain"]["ms"]
    ok_prop, ok_plain = acc["prop"]["ok"], acc["plain"]["ok"]
    if dist is not None:
        # replicas: the slowest rank's clock, every rank's aligned pairs
        from lowcost3dreconstruction_gb300.replicas import combine
        dist.barrier()
        (t_prop, t_plain, e2e_ms), (ok_prop, ok_plain, e2e_ok) = combine(
            dist, [t_prop, t_plain, e2e_ms], [ok_prop, ok_plain, e2e_ok], device=f"cuda:{dev}")
    if rank != 0:
        for c in ctxs:
            c.close()
        return None
    n = c4.npairs
    value = ok_prop / (t_prop / 1000.0)
    plain_value = ok_plain / (t_plain / 1000.0)
    # NormalEstimation's k-NN pass (k = 30), one cloud per launch, timed in the
    # timed region.  Algorithmic bytes of a cloud of m points in ceil(m/32)
    # leaves: query 16 m + reference 16 m + normal and curvature out 16 m +
    # the leaf boxes, 32 B per leaf.
    nk_ms, nk_launches = sum(t[0] for t in kt), sum(t[1] for t in kt)
    bytes_per_cloud = float(np.mean(48.0 * sizes + 32.0 * np.ceil(sizes / 32.0)))
    pk = peaks()
    avg_ms = nk_ms / max(1, nk_launches)
    normals_gbs = bytes_per_cloud / (avg_ms * 1e-3) / 1e9
    search_avg_ms = search_ms / max(1, search_launches)
    search_bytes_per_launch = search_bytes / max(1, search_launches)
    achieved = search_bytes / max(search_ms * 1e-3, 1e-12) / 1e9
    traffic, tctx = None, {}
    tfile = ROOT / "profiles" / "k_icp_search_config4_traffic.json"
    if tfile.exists():
        tj = json.loads(tfile.read_text())
        if tj.get("bytes_per_point_round"):
            # scaled from the capture by the source points the launch searched
            pts_per_launch = sum(it * ns for call in icp_calls for ns, _, it in call) / max(1, search_launches)
            traffic = int(tj["bytes_per_point_round"] * pts_per_launch)
        tctx = {k: tj[k] for k in ("l2_hit_rate", "issue_active", "bound_note") if k in tj}
    res_bytes = 224  # one lcr_icp_result read back per pair and ICP stage
    steps_total = K * world
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "pairs/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": round(t_prop / K, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (bf16 proposal network)", "data": "synthetic",
        "config": {
            "workload": CONFIG4_WORKLOAD, "pairs": n, "points_per_step": int(sizes.sum()),
            "points_per_view": [int(sizes.min()), int(np.median(sizes)), int(sizes.max())],
            "image_bytes": int(c4.image_bytes()),
            "points_per_s": round(float(sizes.sum()) * K / (t_prop / 1000.0), 1),
            "ms_per_step_by_stage": {"preprocess": round(pre / K, 3), "proposal_arm": round(acc["prop"]["ms"] / K, 3),
                                     "plain_arm": round(acc["plain"]["ms"] / K, 3)},
            "aligned_per_step": ok_prop / steps_total, "converged_per_step": acc["prop"]["conv"] / K,
            "fallbacks_per_step": acc["prop"]["fb"] / K,
            "plain_gpu_icp": {"pairs_per_s": round(plain_value, 3), "aligned_per_step": ok_plain / steps_total,
                              "converged_per_step": acc["plain"]["conv"] / K,
                              "icp": "point-to-plane 5 cm (<=100 it) then 1 cm (<=50 it) from centroid alignment"},
            "proposal_over_plain": round(value / max(plain_value, 1e-9), 3),
            "proposal_over_plain_alignment_only": round(
                (acc["prop"]["ok"] / acc["prop"]["ms"]) / max(acc["plain"]["ok"] / acc["plain"]["ms"], 1e-12), 3),
            "rmse_limit_m": RMSE_LIMIT,
            "l2": "inputs (%.1f GB of depth images) larger than L2; 256 MB flush before every stage" % (
                c4.image_bytes() / 1e9),
            "launch_shapes": ctx.tune_get(),
            "preprocess_streams": len(ctxs)},
        "roofline": {"kernel": "k_icp_search<1> (one ICP round's correspondence search over every live pair)",
                     "bound": "hbm", "achieved": round(achieved, 2), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / pk["hbm_gbs"], 5), "peak_src": pk["src"],
                     "algorithmic_bytes_per_launch": int(search_bytes_per_launch),
                     "avg_launch_ms": round(search_avg_ms, 5), "launches": int(search_launches),
                     "measured": "one extra step with the ICP rounds run from the host loop, CUDA events on the "
                                 "library's stream around every search launch",
                     "traffic": traffic, **tctx,
                     "normals_knn": {"kernel": "k_normals + k_normals_escaped (k=30, one cloud per launch, timed "
                                               "in the timed region)", "achieved_gbs": round(normals_gbs, 2),
                                     "avg_launch_ms": round(avg_ms, 5), "launches": int(nk_launches),
                                     "algorithmic_bytes_per_launch": int(bytes_per_cloud)}},
        "e2e": {"value": round(e2e_ok / (e2e_ms / 1000.0), 3), "unit": "pairs/s",
                "h2d_bytes_per_step": int(c4.image_bytes()), "d2h_bytes_per_step": int(2 * n * res_bytes + n * 64),
                "steps": e2e_steps},
        "gpu_launches": int(launches // max(1, K)),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = config4_cpu_baseline([c4.host_pair(i) for i in range(12)])
    for c in ctxs:
        c.close()
    return out


CONFIG4_WORKLOAD = ("config 4: 512 depth-image pairs (superquadric + block + 2 balls, yaw +-180 deg, tilt +-20 deg, "
                    "translation +-10 cm, Kinect noise), Kinect v1 640x480 uint16 / Kinect v2 512x424 float32 at "
                    "upsampling x1/x2/x4, 5k-500k points per view; per step: back-projection + NormalEstimation "
                    "k=30 of all 1024 views, then proposal + point-to-plane ICP (2 cm then 1 cm, plain ICP "
                    "fallback), all pairs batched")


def config4_cpu_pair(pair: dict, threads: int) -> bool:
    """The plain method on one pair through the oracle: back-projection,
    NormalEstimation k=30, centroid alignment, point-to-plane ICP 5 cm then
    1 cm; True when aligned."""
    from lowcost3dreconstruction_gb300 import synthetic as S
    from lowcost3dreconstruction_gb300.core import xyz_of
    from oracle import oracle as O
    O.set_threads(threads)
    clouds = []
    for v in pair["views"]:
        h, w = v["image"].shape
        prm = O.bp_params(w, h, fx=v["fx"], fy=v["fy"], cx=v["cx"], cy=v["cy"], depth_min=C4_DEPTH_RANGE_MM[0],
                          depth_max=C4_DEPTH_RANGE_MM[1], scale=0.001 if v["model"] == 0 else 1.0, normals=False)
        img = v["image"]
        c = O.backproject_v1(img.view(np.uint16), prm) if v["model"] == 0 else O.backproject_v2(img, prm)
        clouds.append(O.normals(c, 30))
    s, t = clouds
    G = np.eye(4)
    G[:3, 3] = O.centroid(t)[:3].astype(np.float64) - O.centroid(s)[:3].astype(np.float64)
    r1 = O.icp(s, t, max_corr_dist=0.05, max_iterations=100, transformation_epsilon=1e-8,
               euclidean_fitness_epsilon=1e-7, point_to_plane=True, guess=G)
    r2 = O.icp(s, t, max_corr_dist=0.01, max_iterations=50, transformation_epsilon=1e-9,
               euclidean_fitness_epsilon=1e-8, point_to_plane=True, guess=r1["transform"])
    r = r2 if r2["state"] != 5 else r1
    return bool(r["converged"] and S.rmse(r["transform"], pair["T"], xyz_of(s)) <= RMSE_LIMIT)


def config4_cpu_baseline(pairs: list[dict]) -> dict:
    """The oracle's plain method on the first pairs of the workload: all host
    threads (OpenMP) for about 10 s of pairs, then one thread on the first
    pairs for about 5 s; the value is the multi-threaded one."""
    threads = os.cpu_count() or 1

    def run(nthreads: int, budget_s: float):
        t0 = time.perf_counter()
        ok = done = 0
        while done < len(pairs) and time.perf_counter() - t0 < budget_s:
            ok += int(config4_cpu_pair(pairs[done], nthreads))
            done += 1
        return ok, done, time.perf_counter() - t0

    ok, done, dt = run(threads, 10.0)
    ok1, done1, dt1 = run(1, 5.0)
    return {"value": round(ok / dt, 4), "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"the oracle's plain method (back-projection, NormalEstimation k=30, centroid alignment, "
                      f"point-to-plane ICP 5 cm + 1 cm) on the first {done} pairs of the workload: {ok} aligned in "
                      f"{dt:.2f} s over {threads} threads",
            "pairs_processed_per_s": round(done / dt, 4),
            "single_thread": {"value": round(ok1 / dt1, 4), "unit": "pairs/s", "cores": 1,
                              "pairs_processed_per_s": round(done1 / dt1, 4),
                              "sample": f"the first {done1} pairs, {ok1} aligned in {dt1:.2f} s"}}


def config4_dump_inputs(path: str, count: int) -> None:
    """Renders the workload (as the GPU arm does) and writes its first `count`
    pairs, as host_pair gives them, to an .npz: the CPU reference arm runs in a
    process that never loads the GPU library."""
    import torch

    from lowcost3dreconstruction_gb300.core import Context
    torch.cuda.set_device(0)
    with Context(0) as ctx:
        c4 = Config4(ctx, 0, pinned=False)
        arrays = {}
        for i in range(count):
            p = c4.host_pair(i)
            arrays[f"T{i}"] = p["T"]
            for side, v in enumerate(p["views"]):
                arrays[f"img{i}_{side}"] = v["image"]
                arrays[f"cam{i}_{side}"] = np.array([v["model"], v["fx"], v["fy"], v["cx"], v["cy"]])
        np.savez(path, count=count, **arrays)


def config4_load_inputs(path: str) -> list[dict]:
    d = np.load(path)
    pairs = []
    for i in range(int(d["count"])):
        views = []
        for side in (0, 1):
            m, fx, fy, cx, cy = d[f"cam{i}_{side}"]
            views.append(dict(image=d[f"img{i}_{side}"], model=int(m), fx=fx, fy=fy, cx=cx, cy=cy))
        pairs.append(dict(views=views, T=d[f"T{i}"]))
    return pairs


def config4_reference_arm(args, rank: int) -> dict | None:
    """--impl reference on config 4: the oracle's plain method (the reference
    path's CPU restatement), all host threads, one pair of the workload per
    step in order.  The inputs are rendered by a child process (the GPU
    renderer, untimed) so that this process loads only the oracle."""
    if rank != 0:
        return None
    import tempfile
    count = max(1, min(args.steps + args.warmup, 64))
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "c4_inputs.npz")
        subprocess.run([sys.executable, str(Path(__file__).resolve()), "--dump-config4-inputs", path,
                        "--dump-count", str(count)], check=True)
        pairs = config4_load_inputs(path)
    threads = os.cpu_count() or 1
    for i in range(min(args.warmup, 1)):
        config4_cpu_pair(pairs[i], threads)
    t0 = time.perf_counter()
    ok = 0
    for k in range(args.steps):
        ok += int(config4_cpu_pair(pairs[(args.warmup + k) % len(pairs)], threads))
    dt = time.perf_counter() - t0
    v = ok / dt
    return {"impl": "reference", "metric": METRIC, "value": round(v, 5), "unit": "pairs/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * dt / args.steps, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": CONFIG4_WORKLOAD, "method": "plain: back-projection, NormalEstimation k=30, "
                       "centroid alignment, point-to-plane ICP 5 cm + 1 cm (the reference has no learned proposal)",
                       "pairs_timed": args.steps, "pairs_aligned": ok},
            "cpu_baseline": {"value": round(v, 5), "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} pairs of the workload in order (one per step), the oracle's "
                                       f"CPU restatement of the reference path, OpenMP over {threads} threads"},
            "e2e": {"value": round(v, 5), "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------------------------ CPU (oracle)
def cpu_pipeline(pr, threads: int):
    from lowcost3dreconstruction_gb300 import synthetic as S
    from oracle import oracle as O
    O.set_threads(threads)
    prm = O.bp_params(640, 480, scale=0.001, depth_max=4000.0, normals=False)
    clouds = []
    for fr in (pr.src_frames, pr.tgt_frames):
        c = O.backproject_v1(O.ze_mean_u16(fr), prm)
        v, _ = O.voxel_grid(c, 0.001)
        _, keep, _ = O.sor(v, 50, 1.0)
        clouds.append(O.normals(v[keep], 30))
    r = O.icp(clouds[0], clouds[1], max_corr_dist=ICP["max_correspondence_distance"],
              max_iterations=ICP["max_iterations"], transformation_epsilon=ICP["transformation_epsilon"],
              euclidean_fitness_epsilon=ICP["euclidean_fitness_epsilon"], point_to_plane=True)
    xs = np.c_[clouds[0]["x"], clouds[0]["y"], clouds[0]["z"]]
    ok = r["converged"] and S.rmse(r["transform"], pr.T_gt, xs) <= RMSE_LIMIT
    return ok, r


def cpu_baseline(pr, sample_pairs: int = 1) -> dict:
    """The CPU restatement on all host threads (the value), and on one thread
    as the pcl_tools run (they have no threading)."""
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    aligned = 0
    for _ in range(sample_pairs):
        ok, _ = cpu_pipeline(pr, threads)
        aligned += int(ok)
    dt = time.perf_counter() - t0
    t0 = time.perf_counter()
    ok1, _ = cpu_pipeline(pr, 1)
    dt1 = time.perf_counter() - t0
    return {"value": round(aligned / dt, 5), "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"{sample_pairs} full pair(s) of the same workload through the CPU restatement "
                      f"(own kd-tree, OpenMP over {threads} threads), {dt:.2f} s",
            "single_thread": {"value": round(int(ok1) / dt1, 5), "unit": "pairs/s", "cores": 1,
                              "sample": f"1 full pair on one thread, {dt1:.2f} s"}}


def reference_arm(args, rank: int) -> dict | None:
    if rank != 0:
        return None
    pr = make_inputs(1)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup if args.warmup < 2 else 1):
        cpu_pipeline(pr, threads)
    t0 = time.perf_counter()
    aligned = 0
    for _ in range(args.steps):
        ok, r = cpu_pipeline(pr, threads)
        aligned += int(ok)
    dt = time.perf_counter() - t0
    v = aligned / dt
    return {"impl": "reference", "metric": METRIC, "value": round(v, 5), "unit": "pairs/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * dt / args.steps, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "icp": ICP, "last_iterations": r["iterations"]},
            "cpu_baseline": {"value": round(v, 5), "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} pairs, each the full workload, CPU restatement of the "
                                       f"reference path (PCL semantics), OpenMP over {threads} threads"},
            "e2e": {"value": round(v, 5), "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="config4",
                    choices=["config4", "config1", "turntable36", "proposal", "sfm", "sr"],
                    help="config4 (the headline): 512 depth-image pairs, preprocessing + proposal + ICP vs plain "
                         "ICP; config1: the full per-capture pipeline on one 300k-point pair; turntable36: batched "
                         "ICP over a turntable cycle; proposal: learned pose proposal + ICP vs plain ICP on held-out "
                         "point-sample pairs; sfm: the SfM-side filters on a 1M-point model; sr: the "
                         "super-resolution front end on 16-frame 640x480 bursts")
    ap.add_argument("--pairs", type=int, default=None,
                    help="pairs of the config4 (default 512) and proposal (default 2000) workloads; a smaller "
                         "config4 (for profiling) keeps the size and camera draws of its first pairs")
    ap.add_argument("--dump-config4-inputs", help=argparse.SUPPRESS)
    ap.add_argument("--dump-count", type=int, default=16, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.dump_config4_inputs:
        from lowcost3dreconstruction_gb300 import build
        build.build_lib()
        config4_dump_inputs(args.dump_config4_inputs, args.dump_count)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "gpu" else args.warmup
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    from lowcost3dreconstruction_gb300 import build
    if args.impl == "reference":
        build.build_oracle()
        if args.workload == "config4":
            build.build_lib()  # the child process that renders the inputs loads it
            out = config4_reference_arm(args, rank)
        else:
            out = reference_arm(args, rank)
    elif args.workload == "turntable36":
        build.build_lib()
        build.build_oracle()
        out = turntable_arm(args) if rank == 0 else None
    elif args.workload == "sfm":
        build.build_lib()
        out = sfm_arm(args) if rank == 0 else None
    elif args.workload == "sr":
        build.build_lib()
        build.build_oracle()
        out = sr_arm(args) if rank == 0 else None
    elif args.workload == "proposal":
        build.build_lib()
        build.build_oracle()
        out = proposal_arm(args) if rank == 0 else None
    elif args.workload == "config4":
        build.build_lib()
        build.build_oracle()
        dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl")
        out = config4_arm(args, rank, world, dist)
        if dist is not None:
            dist.destroy_process_group()
    else:
        build.build_lib()
        build.build_oracle()
        dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl")
        out = gpu_arm(args, rank, world, dist)
        if dist is not None:
            dist.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
