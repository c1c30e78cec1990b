"""Host side of the learned pose proposal (lcr_posenet_* in include/lcr.h).

``PoseNet`` owns the device network of one ``Context``: a shared-MLP point
encoder and a pair head that propose the source-to-target transform ICP
starts from, in place of centroid_align's guess
(pcl_tools/centroid_align.cpp:102-130).  Everything runs on the GPU; the
parameters cross to the host only through ``params``/``set_params`` (and the
``.npy`` files ``save``/``load`` write)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _lib as L
from .core import Cloud, Context

PARAMS = L.POSENET_PARAMS
# Trained parameters shipped with the package (train_posenet.py made them; fp32, LAYOUT order).
WEIGHTS = Path(__file__).resolve().parent / "weights" / "posenet.npy"
POINTS = L.POSENET_POINTS
# (name, shape) of each tensor in the flat parameter vector, in order
LAYOUT = [("W1", (64, 3)), ("b1", (64,)), ("W2", (128, 64)), ("b2", (128,)), ("W3", (1024, 128)), ("b3", (1024,)),
          ("H1", (512, 2048)), ("c1", (512,)), ("H2", (256, 512)), ("c2", (256,)), ("H3", (9, 256)), ("c3", (9,))]


def split(params: np.ndarray) -> dict[str, np.ndarray]:
    """Views of the flat parameter vector by tensor name."""
    out, o = {}, 0
    for name, shape in LAYOUT:
        n = int(np.prod(shape))
        out[name] = params[o:o + n].reshape(shape)
        o += n
    assert o == PARAMS
    return out


def adamw(lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
          weight_decay: float = 1e-4) -> L.AdamwParams:
    return L.AdamwParams(lr, beta1, beta2, eps, weight_decay)


class PoseNet:
    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        self.h = C.c_void_p()
        ctx._check(ctx.lib.lcr_posenet_create(ctx.h, seed, C.byref(self.h)))

    def free(self) -> None:
        if self.h and self.ctx.h:
            self.ctx.lib.lcr_posenet_free(self.ctx.h, self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # ---------------------------------------------------------- parameters
    def params(self) -> np.ndarray:
        p = np.zeros(PARAMS, dtype=np.float32)
        self.ctx._check(self.ctx.lib.lcr_posenet_get_params(self.ctx.h, self.h, L.ptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (PARAMS,)
        self.ctx._check(self.ctx.lib.lcr_posenet_set_params(self.ctx.h, self.h, L.ptr(p)))

    def save(self, path: os.PathLike | str) -> None:
        np.save(path, self.params())

    def load(self, path: os.PathLike | str) -> None:
        self.set_params(np.load(path))

    # ------------------------------------------------------------- compute
    def sample(self, clouds: list[Cloud], seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """Network input of each cloud: (pts [n][POINTS][4], centroids [n][3])."""
        n = len(clouds)
        pts = np.zeros((n, POINTS, 4), dtype=np.float32)
        cen = np.zeros((n, 3), dtype=np.float64)
        hs = (C.c_void_p * max(n, 1))(*[c.handle for c in clouds])
        self.ctx._check(self.ctx.lib.lcr_posenet_sample(self.ctx.h, hs, n, seed, L.ptr(pts), L.ptr(cen)))
        return pts, cen

    def forward(self, pts: np.ndarray, train: bool = False):
        """pts [2B][POINTS][4] (sources then targets) -> (features, argmax | None, out [B][9])."""
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        B = pts.shape[0] // 2
        feat = np.zeros((2 * B, 1024), dtype=np.float32)
        arg = np.zeros((2 * B, 1024), dtype=np.int32) if train else None
        out = np.zeros((B, 9), dtype=np.float32)
        self.ctx._check(self.ctx.lib.lcr_posenet_forward(self.ctx.h, self.h, L.ptr(pts), B, 1 if train else 0,
                                                         L.ptr(feat), L.ptr(arg) if train else None, L.ptr(out)))
        return feat, arg, out

    def gradients(self, pts: np.ndarray, labels: np.ndarray) -> tuple[float, np.ndarray]:
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        labels = np.ascontiguousarray(labels, dtype=np.float32)
        B = pts.shape[0] // 2
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(PARAMS, dtype=np.float32)
        self.ctx._check(self.ctx.lib.lcr_posenet_gradients(self.ctx.h, self.h, L.ptr(pts), L.ptr(labels), B,
                                                           L.ptr(loss), L.ptr(g)))
        return float(loss[0]), g

    def train_step(self, srcs: list[Cloud], tgts: list[Cloud], transforms: np.ndarray, seed: int = 0,
                   opt: L.AdamwParams | None = None) -> float:
        n = len(srcs)
        T = np.ascontiguousarray(transforms, dtype=np.float32).reshape(n * 16)
        hs = (C.c_void_p * n)(*[c.handle for c in srcs])
        ht = (C.c_void_p * n)(*[c.handle for c in tgts])
        loss = np.zeros(1, dtype=np.float32)
        self.ctx._check(self.ctx.lib.lcr_posenet_train_step(self.ctx.h, self.h, hs, ht, L.ptr(T), n, seed,
                                                            C.byref(opt or adamw()), L.ptr(loss)))
        return float(loss[0])

    def propose(self, srcs: list[Cloud], tgts: list[Cloud], seed: int = 0) -> np.ndarray:
        """Source-to-target guesses [n][4][4] (float32, row-major)."""
        n = len(srcs)
        out = np.zeros((max(n, 1), 16), dtype=np.float32)
        hs = (C.c_void_p * max(n, 1))(*[c.handle for c in srcs])
        ht = (C.c_void_p * max(n, 1))(*[c.handle for c in tgts])
        self.ctx._check(self.ctx.lib.lcr_posenet_propose(self.ctx.h, self.h, hs, ht, n, seed, L.ptr(out)))
        return out[:n].reshape(n, 4, 4)
