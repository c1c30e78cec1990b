"""Seeded synthetic Kinect-shaped captures.

Analytic scenes (spheres, oriented boxes, superquadrics) are ray-cast into
depth images in the reference's camera convention (capture/depth_capture/
depth_capture.cpp:300-304: x = z(j-cx)/fx, y = -z(i-cy)/fy, z' = -z, i.e. the
camera looks down -z with y up).  Depth noise follows the Kinect model
sigma = 1.5 mm * (z / 1 m)^2; bursts add per-frame dropouts (zeros) that the
zero-eliminated mean removes.  A pair is the same scene captured before and
after a known rigid motion T_gt, so ICP accuracy is measured against ground
truth: RMSE = RMS over source points of |T_est p - T_gt p|.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

KINECT_V1 = dict(width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5)
KINECT_V2 = dict(width=512, height=424, fx=365.0, fy=365.0, cx=255.5, cy=211.5)


def upsampled(cam: dict, s: int) -> dict:
    """The camera of an image upsampled s times per axis, as the
    super-resolution tools' resample factor makes it (super_resolution.cpp:
    274-314): s x the pixels, focal lengths scaled, pixel centres kept."""
    c = dict(cam)
    c.update(width=cam["width"] * s, height=cam["height"] * s, fx=cam["fx"] * s, fy=cam["fy"] * s,
             cx=(cam["cx"] + 0.5) * s - 0.5, cy=(cam["cy"] + 0.5) * s - 0.5)
    return c


def rot_y(deg: float) -> np.ndarray:
    a = np.deg2rad(deg)
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def rot_x(deg: float) -> np.ndarray:
    a = np.deg2rad(deg)
    c, s = np.cos(a), np.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def rigid(R: np.ndarray, t) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def turntable(deg: float, axis_point, translation=(0.0, 0.0, 0.0), tilt_deg: float = 0.0) -> np.ndarray:
    """Rotation by `deg` about the vertical axis through axis_point (then an
    optional tilt about x), followed by a translation."""
    c = np.asarray(axis_point, dtype=np.float64)
    R = rot_x(tilt_deg) @ rot_y(deg)
    return rigid(np.eye(3), np.asarray(translation) + c) @ rigid(R, 0) @ rigid(np.eye(3), -c)


@dataclass
class Sphere:
    center: np.ndarray
    radius: float

    def moved(self, T):
        return Sphere(T[:3, :3] @ self.center + T[:3, 3], self.radius)

    def hit(self, d):  # d: (N,3) ray directions from the origin
        c = self.center
        dd = np.einsum("ij,ij->i", d, d)
        dc = d @ c
        disc = dc * dc - dd * (c @ c - self.radius ** 2)
        t = np.full(len(d), np.inf)
        ok = disc >= 0
        tt = (dc[ok] - np.sqrt(disc[ok])) / dd[ok]
        t[ok] = np.where(tt > 0, tt, np.inf)
        return t


@dataclass
class Box:
    center: np.ndarray
    half: np.ndarray
    R: np.ndarray = field(default_factory=lambda: np.eye(3))

    def moved(self, T):
        return Box(T[:3, :3] @ self.center + T[:3, 3], self.half, T[:3, :3] @ self.R)

    def hit(self, d):
        o = self.R.T @ (-self.center)
        dl = d @ self.R
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / dl
            t1 = (-self.half - o) * inv
            t2 = (self.half - o) * inv
        tn = np.nanmax(np.minimum(t1, t2), axis=1)
        tf = np.nanmin(np.maximum(t1, t2), axis=1)
        return np.where((tn <= tf) & (tn > 0), tn, np.inf)


@dataclass
class Superquadric:
    """|x/a|^(2/e2) + |y/b|^(2/e2))^(e2/e1) + |z/c|^(2/e1) = 1 in its own frame;
    ray-cast by bracketing the inside/outside sign change then bisection."""
    center: np.ndarray
    axes: np.ndarray
    e1: float
    e2: float
    R: np.ndarray = field(default_factory=lambda: np.eye(3))

    def moved(self, T):
        return Superquadric(T[:3, :3] @ self.center + T[:3, 3], self.axes, self.e1, self.e2, T[:3, :3] @ self.R)

    def _f(self, p):
        q = np.abs(p / self.axes) + 1e-12
        return (q[..., 0] ** (2 / self.e2) + q[..., 1] ** (2 / self.e2)) ** (self.e2 / self.e1) + q[..., 2] ** (2 / self.e1)

    def hit(self, d):
        o = self.R.T @ (-self.center)
        dl = d @ self.R
        # bounding sphere
        rad = float(np.linalg.norm(self.axes)) * 1.01
        dd = np.einsum("ij,ij->i", dl, dl)
        od = dl @ o
        disc = od * od - dd * (o @ o - rad * rad)
        t = np.full(len(d), np.inf)
        cand = np.nonzero(disc > 0)[0]
        if len(cand) == 0:
            return t
        sq = np.sqrt(disc[cand])
        t0 = np.maximum((-od[cand] - sq) / dd[cand], 1e-6)
        t1 = (-od[cand] + sq) / dd[cand]
        steps = 96
        ts = t0[:, None] + (t1 - t0)[:, None] * np.linspace(0, 1, steps)[None, :]
        pts = o[None, None, :] + ts[..., None] * dl[cand][:, None, :]
        inside = self._f(pts) <= 1.0
        first = np.argmax(inside, axis=1)
        has = inside[np.arange(len(cand)), first] & (first > 0)
        ci = cand[has]
        lo = ts[has, first[has] - 1]
        hi = ts[has, first[has]]
        dl_h = dl[ci]
        for _ in range(30):
            mid = 0.5 * (lo + hi)
            ins = self._f(o[None, :] + mid[:, None] * dl_h) <= 1.0
            hi = np.where(ins, mid, hi)
            lo = np.where(ins, lo, mid)
        t[ci] = hi
        return t


def ray_dirs(cam: dict) -> np.ndarray:
    j, i = np.meshgrid(np.arange(cam["width"]), np.arange(cam["height"]))
    return np.stack([(j - cam["cx"]) / cam["fx"], -(i - cam["cy"]) / cam["fy"], -np.ones_like(j, float)],
                    axis=-1).reshape(-1, 3)


def raycast(prims, cam: dict, T: np.ndarray | None = None) -> np.ndarray:
    """Depth in metres (inf where nothing is hit), shape (height, width)."""
    d = ray_dirs(cam)
    t = np.full(len(d), np.inf)
    for p in prims:
        q = p.moved(T) if T is not None else p
        t = np.minimum(t, q.hit(d))
    return t.reshape(cam["height"], cam["width"])


def kinect_frames(depth_m: np.ndarray, frames: int, rng: np.random.Generator, dropout: float = 0.0,
                  depth_max_mm: float = 4000.0, sigma_mm: float = 1.5, as_float: bool = False) -> np.ndarray:
    """A burst of noisy captures of one depth map (uint16 mm, or float32 mm)."""
    valid = np.isfinite(depth_m)
    z = np.where(valid, depth_m, 0.0) * 1000.0
    sig = sigma_mm * (z / 1000.0) ** 2
    out = []
    for _ in range(frames):
        zz = z + rng.standard_normal(z.shape) * sig
        keep = valid & (zz > 0) & (zz <= depth_max_mm)
        if dropout > 0:
            keep &= rng.random(z.shape) >= dropout
        if as_float:
            out.append(np.where(keep, zz, 0.0).astype(np.float32))
        else:
            out.append(np.where(keep, np.rint(zz), 0).astype(np.uint16))
    return np.stack(out)


# ----------------------------------------------------------------- scenes
def sphere_on_cube() -> list:
    """Sphere r=0.15 m, 1.0 m in front of the camera, resting on a 0.3 m cube."""
    return [Sphere(np.array([0.0, 0.0, -1.0]), 0.15),
            Box(np.array([0.0, -0.30, -1.0]), np.array([0.15, 0.15, 0.15]))]


def sphere_on_cube_room() -> list:
    """sphere_on_cube plus a floor and a back wall that fill the frame."""
    return sphere_on_cube() + [Box(np.array([0.0, -0.95, -1.5]), np.array([4.0, 0.5, 4.0])),
                               Box(np.array([0.0, 0.0, -2.1]), np.array([4.0, 4.0, 0.5]))]


def superquadric_object(rng: np.random.Generator) -> list:
    axes = rng.uniform(0.05, 0.2, size=3)
    e1, e2 = rng.uniform(0.3, 1.5, size=2)
    R = rot_y(rng.uniform(0, 360)) @ rot_x(rng.uniform(-20, 20))
    return [Superquadric(np.array([0.0, 0.0, -1.0]), axes, float(e1), float(e2), R)]


OBJECT_AXIS = np.array([0.0, 0.0, -1.0])


@dataclass
class Pair:
    src_frames: np.ndarray
    tgt_frames: np.ndarray
    T_gt: np.ndarray
    cam: dict


def make_pair(scene: list, deg: float, translation, frames: int, seed: int, cam: dict = KINECT_V1,
              dropout: float = 0.0, as_float: bool = False) -> Pair:
    rng = np.random.default_rng(seed)
    T = turntable(deg, OBJECT_AXIS, translation)
    d0 = raycast(scene, cam)
    d1 = raycast(scene, cam, T)
    return Pair(kinect_frames(d0, frames, rng, dropout, as_float=as_float),
                kinect_frames(d1, frames, rng, dropout, as_float=as_float), T, cam)


def config0_pair(seed: int = 0) -> Pair:
    """Sphere on cube, target rotated 15 deg about the object's vertical axis and
    moved by (2, 0, 1) cm; one frame per capture."""
    return make_pair(sphere_on_cube(), 15.0, (0.02, 0.0, 0.01), 1, seed)


def config1_pair(seed: int = 1) -> Pair:
    """Frame-filling room scene (~300k valid pixels), 10-frame bursts with 3%
    dropouts, target rotated 20 deg and moved 3 cm."""
    return make_pair(sphere_on_cube_room(), 20.0, (0.03, 0.0, 0.0), 10, seed, dropout=0.03)


def turntable_cycle(seed: int = 2, views: int = 36, step_deg: float = 10.0, frames: int = 1,
                    cam: dict = KINECT_V1) -> tuple[np.ndarray, list[np.ndarray]]:
    """A seeded superquadric object on a turntable, captured every `step_deg`
    degrees about its vertical axis: (frames-per-view depth bursts [views, F, H, W],
    ground-truth pose of each view relative to view 0).  Consecutive views
    overlap by 360/views degrees less than a full turn, so each pair sees part
    of the surface the other does not (self-occlusion)."""
    rng = np.random.default_rng(seed)
    # a seeded superquadric with a block and two balls attached around it: a
    # lone superquadric is often nearly symmetric about some axis, which leaves
    # ICP a sliding direction
    obj = superquadric_object(rng)
    sq = obj[0]
    a0 = rng.uniform(0, 360)
    r = sq.axes.max()
    for k, (dy, size) in enumerate(((-0.02, 0.03), (0.03, 0.025), (-0.05, 0.035))):
        side = rot_y(a0 + 120.0 * k)
        if k == 0:
            obj.append(Box(sq.center + side @ np.array([r + 0.03, dy, 0.0]), np.array([0.03, 0.05, 0.02]), side))
        else:
            obj.append(Sphere(sq.center + side @ np.array([r + 0.02, dy, 0.0]), size))
    caps, poses = [], []
    for v in range(views):
        T = turntable(step_deg * v, OBJECT_AXIS)
        d = raycast(obj, cam, T)
        caps.append(kinect_frames(d, frames, rng, 0.0))
        poses.append(T)
    return np.stack(caps), poses


def rmse(T_est: np.ndarray, T_gt: np.ndarray, xyz: np.ndarray) -> float:
    p = np.c_[np.asarray(xyz, np.float64), np.ones(len(xyz))]
    d = p @ (np.asarray(T_est, np.float64) - np.asarray(T_gt, np.float64)).T
    return float(np.sqrt(np.mean(np.sum(d[:, :3] ** 2, axis=1))))


def rotation_angle(T: np.ndarray) -> float:
    R = np.asarray(T, np.float64)[:3, :3]
    return float(np.arccos(np.clip((np.trace(R) - 1) / 2, -1.0, 1.0)))
