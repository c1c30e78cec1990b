"""Training and evaluation of the learned pose proposal, all on the GPU.

Training pairs are generated on the device (lcr_synthetic_pairs: random
superquadric objects with a block and two balls attached, yaw uniform in
+-180 deg, tilt +-20 deg, translation +-10 cm, Kinect depth noise) and
labelled by converged plain point-to-plane ICP started from the generator's
exact transform (lcr_icp_batch); a pair whose ICP does not converge keeps the
exact transform.  Each step draws a fresh batch, so the step count times the
batch size is the number of training pairs.

Evaluation aligns held-out pairs two ways with the same point-to-plane ICP:
from centroid alignment (the plain method: identity rotation, centroids
matched, as centroid_align.cpp:102-130 does with zero angles) and from the
network's proposal, with the plain method as the fallback for pairs whose
refined alignment leaves too few inlier correspondences.  A pair counts as
aligned when ICP converged and the RMS over its source points of
|T_est p - T_gt p| is at most 1 mm.

    python -m lowcost3dreconstruction_gb300.train_posenet --steps 16000 --out posenet.npy
    python -m lowcost3dreconstruction_gb300.train_posenet --steps 0 --init posenet.npy \
        --depth-steps 4000 --out posenet.npy

The second form fine-tunes on depth-image pairs (depth_pairs: rendered by
lcr_synthetic_depth at Kinect v1 and v2 geometry and back-projected), the
input the depth pipeline hands the network.
"""
from __future__ import annotations

import argparse
import time
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .core import Context
from .posenet import PoseNet, adamw

TRAIN_POINTS = 4096
EVAL_POINTS = 20000
RMSE_LIMIT = 1e-3


def label_params() -> L.IcpParams:
    return Context.icp_params(max_correspondence_distance=0.01, max_iterations=15, transformation_epsilon=1e-8,
                              euclidean_fitness_epsilon=1e-7, point_to_plane=True, compute_fitness=False)


# Stop rules of the first ICP stages (lcr_icp_params.stop_iteration/stop_rms),
# measured on the 512-pair depth workload: every pair that aligned had its
# 5 cm stage below 15 mm RMS correspondence distance by iteration 12 (14
# iterations to converge on average), and its 2 cm proposal stage below 8 mm by
# iteration 8; stopping the rest there lost no aligned pair in either arm and
# cut the plain arm from 1297 to 959 ms and the proposal arm from 814 to
# 758 ms.  Pairs whose views share too little surface otherwise run to the
# iteration cap.
STOP_ITERATION, STOP_RMS = 12, 0.015
PROPOSAL_STOP_ITERATION, PROPOSAL_STOP_RMS = 8, 0.008


def eval_params() -> L.IcpParams:
    """Coarse refinement: a 5 cm correspondence threshold pulls guesses tens of degrees off into place; a pair
    still above STOP_RMS after STOP_ITERATION iterations stops there."""
    return Context.icp_params(max_correspondence_distance=0.05, max_iterations=100, transformation_epsilon=1e-8,
                              euclidean_fitness_epsilon=1e-7, point_to_plane=True, compute_fitness=False,
                              stop_iteration=STOP_ITERATION, stop_rms=STOP_RMS)


def fine_params() -> L.IcpParams:
    """Fine refinement from the coarse result: a 1 cm threshold keeps points that have no partner in the other
    view (partial overlap) from biasing the final transform."""
    return Context.icp_params(max_correspondence_distance=0.01, max_iterations=50, transformation_epsilon=1e-9,
                              euclidean_fitness_epsilon=1e-8, point_to_plane=True, compute_fitness=False)


def proposal_params() -> L.IcpParams:
    """First refinement of a proposal: its rotation error is a few degrees, so a 2 cm threshold holds it and
    admits fewer wrong partners than the 5 cm the centroid guess needs; a pair still above
    PROPOSAL_STOP_RMS after PROPOSAL_STOP_ITERATION iterations stops there (and goes to the fallback)."""
    return Context.icp_params(max_correspondence_distance=0.02, max_iterations=30, transformation_epsilon=1e-8,
                              euclidean_fitness_epsilon=1e-7, point_to_plane=True, compute_fitness=False,
                              stop_iteration=PROPOSAL_STOP_ITERATION, stop_rms=PROPOSAL_STOP_RMS)


def refine(ctx: Context, srcs, tgts, guesses: np.ndarray, first: L.IcpParams | None = None):
    """A first point-to-plane ICP (coarse by default) then the fine one, both batched; a pair the first stage
    stopped (or left without correspondences) keeps that result and skips the fine stage."""
    coarse = ctx.icp_batch(srcs, tgts, first or eval_params(), guesses)
    go = [i for i, r in enumerate(coarse)
          if r.state not in (L.ICP_STATE_STOPPED, L.ICP_STATE_NO_CORRESPONDENCES)]
    out = list(coarse)
    if go:
        start = np.stack([coarse[i].transform for i in go])
        fine = ctx.icp_batch([srcs[i] for i in go], [tgts[i] for i in go], fine_params(), start)
        for i, f in zip(go, fine):
            if f.state != L.ICP_STATE_NO_CORRESPONDENCES:
                out[i] = f
    return out


def icp_labels(ctx: Context, srcs, tgts, T_gt: np.ndarray, max_deg: float = 1.0,
               max_shift: float = 0.003) -> np.ndarray:
    """Converged point-to-plane ICP from the exact transform.  Where the views
    overlap too little for ICP to hold (it did not converge, or it slid more
    than max_deg / max_shift away from the exact transform), the exact
    transform is the label."""
    res = ctx.icp_batch(srcs, tgts, label_params(), T_gt)
    out = T_gt.copy()
    est = np.stack([r.transform for r in res])
    rot = rotation_error_deg(est, T_gt)
    shift = np.linalg.norm(est[:, :3, 3] - T_gt[:, :3, 3], axis=1)
    for i, r in enumerate(res):
        if r.converged and r.state != L.ICP_STATE_NO_CORRESPONDENCES and rot[i] <= max_deg and shift[i] <= max_shift:
            out[i] = r.transform
    return out


def train(ctx: Context, steps: int, batch: int = 256, lr: float = 1e-3, seed: int = 0, net: PoseNet | None = None,
          points: int = TRAIN_POINTS, label_with_icp: bool = True, log_every: int = 0,
          lr_final: float | None = None, yaw_deg: float = 180.0, warmup_frac: float = 0.0) -> tuple[PoseNet, list[float]]:
    """AdamW on fresh device-generated batches; cosine decay to lr_final
    (default lr/20).  warmup_frac > 0 widens the yaw range linearly from 30
    degrees to yaw_deg over that fraction of the steps (a curriculum)."""
    net = net or PoseNet(ctx, seed=seed)
    lr_final = lr / 20 if lr_final is None else lr_final
    losses = []
    for step in range(steps):
        yaw = yaw_deg
        if warmup_frac > 0:
            yaw = min(yaw_deg, 30.0 + (yaw_deg - 30.0) * step / max(1.0, warmup_frac * steps))
        srcs, tgts, T = ctx.synthetic_pairs(seed * 1_000_003 + step, batch, points, yaw_deg=yaw)
        labels = icp_labels(ctx, srcs, tgts, T) if label_with_icp else T
        a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * step / max(steps - 1, 1)))
        losses.append(net.train_step(srcs, tgts, labels, seed=step, opt=adamw(lr=float(a))))
        for c in srcs + tgts:
            c.free()
        if log_every and (step % log_every == 0 or step == steps - 1):
            print(f"step {step:5d}  loss {np.mean(losses[-log_every:]):.4f}  lr {a:.2e}", flush=True)
    return net, losses


def depth_pairs(ctx: Context, seed: int, batch: int, rng: np.random.Generator, yaw_deg: float = 180.0,
                max_points: float = 2e5):
    """Training pairs as the depth pipeline sees them: lcr_synthetic_depth
    renders `batch` pairs with one camera (Kinect v1 uint16 or Kinect v2
    float32, upsampling 1 or 2), each object at the distance that gives it
    5k-max_points pixels per view, and every view is back-projected in metres.
    Returns (sources, targets, exact transforms)."""
    import torch

    from . import synthetic as S
    v1 = bool(rng.random() < 0.5)
    cam = S.upsampled(S.KINECT_V1 if v1 else S.KINECT_V2, int(rng.choice([1, 2])))
    model = L.KINECT_V1 if v1 else L.KINECT_V2
    want = np.exp(rng.uniform(np.log(5e3), np.log(max_points), batch)).astype(np.float32)
    pix = cam["width"] * cam["height"]
    buf = torch.empty(2 * batch * pix, dtype=torch.int16 if v1 else torch.float32,
                      device=f"cuda:{torch.cuda.current_device()}")
    torch.cuda.synchronize()
    T = ctx.synthetic_depth(seed, batch, model, cam["width"], cam["height"], cam["fx"], cam["fy"], cam["cx"],
                            cam["cy"], buf.data_ptr(), points=want, yaw_deg=yaw_deg)
    params = ctx.depth_params(model, cam["width"], cam["height"], fx=cam["fx"], fy=cam["fy"], cx=cam["cx"],
                              cy=cam["cy"], depth_min=300.0, depth_max=9000.0, scale=0.001 if v1 else 1.0,
                              normals=False)
    es = buf.element_size()
    clouds = [ctx.backproject_device(buf.data_ptr() + v * pix * es, params) for v in range(2 * batch)]
    del buf
    return clouds[0::2], clouds[1::2], T


def train_depth(ctx: Context, net: PoseNet, steps: int, batch: int = 256, lr: float = 3e-4, lr_final: float = 1e-5,
                seed: int = 0, point_every: int = 2, log_every: int = 0) -> list[float]:
    """Fine-tuning on depth-image pairs (depth_pairs, exact transforms as
    labels), every point_every-th step on a batch of lcr_synthetic_pairs
    point samples so the network keeps both input forms; AdamW with cosine
    decay from lr to lr_final."""
    rng = np.random.default_rng(seed)
    losses = []
    for step in range(steps):
        if point_every and step % point_every == point_every - 1:
            srcs, tgts, T = ctx.synthetic_pairs(20_000_000 + seed * 100_003 + step, batch, TRAIN_POINTS)
        else:
            srcs, tgts, T = depth_pairs(ctx, 10_000_000 + seed * 100_003 + step, batch, rng)
        a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * step / max(steps - 1, 1)))
        losses.append(net.train_step(srcs, tgts, T, seed=step, opt=adamw(lr=float(a))))
        for c in srcs + tgts:
            c.free()
        if log_every and (step % log_every == 0 or step == steps - 1):
            print(f"depth step {step:5d}  loss {np.mean(losses[-log_every:]):.4f}  lr {a:.2e}", flush=True)
    return losses


@dataclass
class EvalResult:
    pairs: int
    aligned_plain: int
    aligned_proposal: int
    seconds_plain: float
    seconds_proposal: float
    fallbacks: int
    proposal_rot_err_deg: np.ndarray
    rmse_plain: np.ndarray
    rmse_proposal: np.ndarray

    @property
    def pairs_per_s_plain(self) -> float:
        return self.aligned_plain / self.seconds_plain

    @property
    def pairs_per_s_proposal(self) -> float:
        return self.aligned_proposal / self.seconds_proposal


def rotation_error_deg(Ta: np.ndarray, Tb: np.ndarray) -> np.ndarray:
    R = np.einsum("bij,bkj->bik", Ta[:, :3, :3].astype(np.float64), Tb[:, :3, :3].astype(np.float64))
    c = np.clip((np.trace(R, axis1=1, axis2=2) - 1) / 2, -1, 1)
    return np.degrees(np.arccos(c))


def centroid_guesses(net: PoseNet, srcs, tgts) -> np.ndarray:
    _, cen = net.sample(list(srcs) + list(tgts))
    n = len(srcs)
    G = np.tile(np.eye(4, dtype=np.float32), (n, 1, 1))
    G[:, :3, 3] = cen[n:] - cen[:n]
    return G


def aligned(ctx: Context, srcs, res, T_gt: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    est = np.stack([r.transform64 for r in res])
    rmse = ctx.rmse_batch(srcs, est, T_gt.astype(np.float64))
    conv = np.array([r.converged for r in res])
    return conv & (rmse <= RMSE_LIMIT), rmse


def settled(r, max_rms: float = 0.004) -> bool:
    """A refined alignment looks right: ICP converged and its inlier correspondences (within the fine
    threshold) are on average no farther apart than max_rms.  On 2000 held-out pairs with 20k points per
    view the aligned pairs' inlier RMS was 2.2 mm at the median and 2.6 mm at p90 (sensor noise plus
    sample spacing); 4 mm sent 1 of the 667 aligned pairs to the fallback."""
    return bool(r.converged) and r.state != L.ICP_STATE_NO_CORRESPONDENCES and r.mse <= max_rms * max_rms


def propose_refine(ctx: Context, net: PoseNet, srcs, tgts, ctx2: Context | None = None):
    """The proposal pipeline: the learned proposal, point-to-plane ICP at 2 cm
    then 1 cm (refine with proposal_params), and plain ICP from the centroid
    guess (refine with eval_params) as the fallback for every pair that did
    not settle; a fallback result replaces the pair's only if it settled.
    Returns (results, number of fallback pairs).

    A pair the 2 cm stage ended (stopped, or left without correspondences)
    skips the 1 cm stage, so its result is known once that stage returns.
    With a second context, the fallback of those pairs runs on it while the
    1 cm stage runs on ctx (two host threads).  Every pair's result is the one
    the sequential order gives: a batched ICP call gives each pair its
    single-pair result, and a centroid guess depends on its own pair only."""
    from concurrent.futures import ThreadPoolExecutor

    P = net.propose(srcs, tgts)
    coarse = ctx.icp_batch(srcs, tgts, proposal_params(), P)
    go = [i for i, r in enumerate(coarse) if r.state not in (L.ICP_STATE_STOPPED, L.ICP_STATE_NO_CORRESPONDENCES)]
    res = list(coarse)
    gos = set(go)
    early = [i for i in range(len(srcs)) if i not in gos and not settled(coarse[i])]
    late: list[int] = []

    def fallback(c: Context, idx: list[int], G: np.ndarray):
        return refine(c, [srcs[i] for i in idx], [tgts[i] for i in idx], G) if idx else []

    def fine_then_late():
        if go:
            start = np.stack([coarse[i].transform for i in go])
            fine = ctx.icp_batch([srcs[i] for i in go], [tgts[i] for i in go], fine_params(), start)
            for i, f in zip(go, fine):
                if f.state != L.ICP_STATE_NO_CORRESPONDENCES:
                    res[i] = f
        late.extend(i for i in go if not settled(res[i]))
        G = centroid_guesses(net, [srcs[i] for i in late], [tgts[i] for i in late]) if late else None
        return fallback(ctx, late, G)

    G_early = centroid_guesses(net, [srcs[i] for i in early], [tgts[i] for i in early]) if early else None
    if ctx2 is None:
        fb_early = fallback(ctx, early, G_early)
        fb_late = fine_then_late()
    else:
        with ThreadPoolExecutor(max_workers=2) as ex:
            f_early = ex.submit(fallback, ctx2, early, G_early)
            fb_late = fine_then_late()
            fb_early = f_early.result()
    for idx, fb in ((early, fb_early), (late, fb_late)):
        for j, i in enumerate(idx):
            if settled(fb[j]):
                res[i] = fb[j]
    return res, len(early) + len(late)


def evaluate(ctx: Context, net: PoseNet, npairs: int = 2000, seed: int = 987_654_321, points: int = EVAL_POINTS,
             chunk: int = 500, yaw_deg: float = 180.0) -> EvalResult:
    """Plain ICP from centroid alignment vs proposal + ICP on held-out pairs; plain ICP from the centroid
    guess is the fallback for pairs whose refined proposal did not settle."""
    n_plain = n_prop = n_fb = 0
    t_plain = t_prop = 0.0
    rot_err, r_plain, r_prop = [], [], []
    for c0 in range(0, npairs, chunk):
        m = min(chunk, npairs - c0)
        srcs, tgts, T = ctx.synthetic_pairs(seed + c0, m, points, yaw_deg=yaw_deg)
        ctx.synchronize()
        # plain: centroid guess + ICP
        t0 = time.perf_counter()
        G = centroid_guesses(net, srcs, tgts)
        res_plain = refine(ctx, srcs, tgts, G)
        t_plain += time.perf_counter() - t0
        # proposal + ICP, plain fallback where the refined proposal did not settle
        t0 = time.perf_counter()
        P = net.propose(srcs, tgts)
        res = refine(ctx, srcs, tgts, P, proposal_params())
        weak = [i for i, r in enumerate(res) if not settled(r)]
        if weak:
            Gw = centroid_guesses(net, [srcs[i] for i in weak], [tgts[i] for i in weak])
            fb = refine(ctx, [srcs[i] for i in weak], [tgts[i] for i in weak], Gw)
            for j, i in enumerate(weak):
                if settled(fb[j]):
                    res[i] = fb[j]
        t_prop += time.perf_counter() - t0
        n_fb += len(weak)
        ok_p, rp = aligned(ctx, srcs, res_plain, T)
        ok_n, rn = aligned(ctx, srcs, res, T)
        n_plain += int(ok_p.sum())
        n_prop += int(ok_n.sum())
        rot_err.append(rotation_error_deg(P, T))
        r_plain.append(rp)
        r_prop.append(rn)
        for c in srcs + tgts:
            c.free()
    return EvalResult(npairs, n_plain, n_prop, t_plain, t_prop, n_fb, np.concatenate(rot_err),
                      np.concatenate(r_plain), np.concatenate(r_prop))


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--steps", type=int, default=16000, help="training steps (fresh pairs each)")
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--init", help="start from these parameters (.npy)")
    ap.add_argument("--out", help="write the trained parameters here (.npy)")
    ap.add_argument("--eval-pairs", type=int, default=2000)
    ap.add_argument("--no-icp-labels", action="store_true", help="train on the exact transforms")
    ap.add_argument("--depth-steps", type=int, default=0,
                    help="then fine-tune this many steps on depth-image pairs (train_depth)")
    ap.add_argument("--depth-lr", type=float, default=3e-4)
    args = ap.parse_args()
    ctx = Context(0)
    net = PoseNet(ctx, seed=args.seed)
    if args.init:
        net.load(args.init)
    t0 = time.perf_counter()
    if args.steps:
        net, losses = train(ctx, args.steps, args.batch, args.lr, args.seed, net=net,
                            label_with_icp=not args.no_icp_labels, log_every=500, warmup_frac=0.3)
        print(f"trained {args.steps} steps x {args.batch} pairs in {time.perf_counter() - t0:.1f} s", flush=True)
    if args.depth_steps:
        t1 = time.perf_counter()
        train_depth(ctx, net, args.depth_steps, args.batch, lr=args.depth_lr, seed=args.seed, log_every=250)
        print(f"fine-tuned {args.depth_steps} steps x {args.batch} depth pairs in {time.perf_counter() - t1:.1f} s",
              flush=True)
    if args.out:
        net.save(args.out)
    for yaw in (180.0, 90.0, 30.0) if args.eval_pairs else ():
        r = evaluate(ctx, net, args.eval_pairs, yaw_deg=yaw)
        print(f"held-out pairs, yaw +-{yaw:.0f} deg: rotation error of the proposal median "
              f"{np.median(r.proposal_rot_err_deg):.1f} deg, p90 {np.percentile(r.proposal_rot_err_deg, 90):.1f} deg")
        print(f"  plain ICP (centroid guess): {r.aligned_plain}/{r.pairs} aligned in {r.seconds_plain:.2f} s "
              f"-> {r.pairs_per_s_plain:.1f} aligned pairs/s")
        print(f"  proposal + ICP:             {r.aligned_proposal}/{r.pairs} aligned in {r.seconds_proposal:.2f} s "
              f"({r.fallbacks} fallbacks) -> {r.pairs_per_s_proposal:.1f} aligned pairs/s", flush=True)


if __name__ == "__main__":
    main()
