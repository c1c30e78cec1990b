"""CPU restatement of the super-resolution front end -- TEST INFRASTRUCTURE ONLY.

Used by tests/ to check lowcost3dreconstruction_gb300/csrc/sr.cu; never by the
library.  The reference (capture/super_resolution/super_resolution.cpp:
236-314) runs OpenCV, which is absent here, so this restates the published
methods the way the library does (parity unpinned):

* ECC affine registration (Evangelidis & Psarakis 2008), on images smoothed by
  a 5x5 Gaussian of sigma 1.1 with reflect-101 borders, central-difference
  gradients, bilinear sampling, every sum over the mask of pixels whose four
  bilinear taps lie inside the image (a half-outside sample of a depth image
  is a large outlier), zero-mean correlation, Gauss-Newton steps (lambda from
  the projections), stop when the correlation coefficient changes by less
  than eps;
* the inverse-map bilinear warp, nearest upsampling, the zero-eliminated mean
  (FP64 sum in frame order), separable Lanczos-4 resampling (taps clamped),
  rounding half to even and saturation to uint16.

The GPU evaluates the same expressions in FP32 with contracted multiply-adds,
so results agree within the tolerances of tests/test_sr.py, not bit for bit.
"""
from __future__ import annotations

import numpy as np


def _pad_reflect101(a: np.ndarray, k: int, axis: int) -> np.ndarray:
    pad = [(0, 0)] * a.ndim
    pad[axis] = (k, k)
    return np.pad(a, pad, mode="reflect")


def gauss5(img: np.ndarray) -> np.ndarray:
    s = 1.1
    g = np.array([1.0, np.exp(-1 / (2 * s * s)), np.exp(-4 / (2 * s * s))])
    g = (g / (g[0] + 2 * g[1] + 2 * g[2])).astype(np.float32)
    out = img.astype(np.float32)
    for axis in (-1, -2):
        p = _pad_reflect101(out, 2, axis)
        n = out.shape[axis]
        sl = lambda o: np.take(p, np.arange(2 + o, 2 + o + n), axis=axis)
        out = (g[0] * sl(0) + g[1] * (sl(-1) + sl(1)) + g[2] * (sl(-2) + sl(2))).astype(np.float32)
    return out


def grad(img: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    px = _pad_reflect101(img, 1, -1)
    py = _pad_reflect101(img, 1, -2)
    gx = (0.5 * (px[..., 2:] - px[..., :-2])).astype(np.float32)
    gy = (0.5 * (py[..., 2:, :] - py[..., :-2, :])).astype(np.float32)
    return gx, gy


def bilinear(img: np.ndarray, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    h, w = img.shape
    x0 = np.floor(u).astype(np.int64)
    y0 = np.floor(v).astype(np.int64)
    ax = (u - x0).astype(np.float32)
    ay = (v - y0).astype(np.float32)

    def at(x, y):
        ok = (x >= 0) & (y >= 0) & (x < w) & (y < h)
        out = np.zeros(x.shape, np.float32)
        out[ok] = img[y[ok], x[ok]]
        return out
    top = at(x0, y0) * (1 - ax) + at(x0 + 1, y0) * ax
    bot = at(x0, y0 + 1) * (1 - ax) + at(x0 + 1, y0 + 1) * ax
    return (top * (1 - ay) + bot * ay).astype(np.float32)


def ecc_affine(tmpl: np.ndarray, img: np.ndarray, gx: np.ndarray, gy: np.ndarray, iters: int, eps: float):
    """Warp (2x3 inverse map, float32) taking tmpl's grid into img, and the iterations run."""
    h, w = tmpl.shape
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    m = np.array([[1, 0, 0], [0, 1, 0]], np.float32)
    prev = -1.0
    it = 0
    T = tmpl.astype(np.float64)
    for it in range(1, iters + 1):
        u = (m[0, 0] * x + m[0, 1] * y + m[0, 2]).astype(np.float32)
        v = (m[1, 0] * x + m[1, 1] * y + m[1, 2]).astype(np.float32)
        I = bilinear(img, u, v).astype(np.float64)
        GX = bilinear(gx, u, v).astype(np.float64)
        GY = bilinear(gy, u, v).astype(np.float64)
        fu, fv = np.floor(u), np.floor(v)
        mk = ((fu >= 0) & (fv >= 0) & (fu + 1 < w) & (fv + 1 < h)).astype(np.float64)
        X, Y = x.astype(np.float64), y.astype(np.float64)
        J = (np.stack([X * GX, X * GY, Y * GX, Y * GY, GX, GY]) * mk).reshape(6, -1)
        n = mk.sum()
        if n <= 0:
            break
        mi, mt = (mk * I).sum() / n, (mk * T).sum() / n
        izm, tzm = (mk * (I - mi)).ravel(), (mk * (T - mt)).ravel()
        corr = izm @ tzm
        inorm, tnorm = np.sqrt(izm @ izm), np.sqrt(tzm @ tzm)
        r = corr / (inorm * tnorm) if inorm > 0 and tnorm > 0 else 0.0
        H = J @ J.T
        ip, tp = J @ izm, J @ tzm
        try:  # a singular (or indefinite) system stops the iteration, as on the GPU
            np.linalg.cholesky(H)
            hi, ht = np.linalg.solve(H, ip), np.linalg.solve(H, tp)
        except np.linalg.LinAlgError:
            break
        lam_n = izm @ izm - ip @ hi
        lam_d = corr - tp @ hi
        if not lam_d > 0:
            break
        dp = (lam_n / lam_d) * ht - hi
        m = m + np.array([[dp[0], dp[2], dp[4]], [dp[1], dp[3], dp[5]]], np.float32)
        if abs(r - prev) < eps:
            break
        prev = r
    return m, it


def lanczos4_weights(t: float) -> np.ndarray:
    if t < 1.1920929e-7:
        w = np.zeros(8)
        w[3] = 1
        return w.astype(np.float32)
    d = (np.arange(8) - 3) - t
    a = np.pi * d
    w = 4 * np.sin(a) * np.sin(a / 4) / (a * a)
    return (w / w.sum()).astype(np.float32)


def lanczos_down(img: np.ndarray, s: int) -> np.ndarray:
    out = img.astype(np.float32)
    for axis in (1, 0):
        n_in = out.shape[axis]
        n_out = n_in // s
        res = []
        for o in range(n_out):
            p = np.float32((o + 0.5) * s - 0.5)
            fl = np.floor(p)
            wgt = lanczos4_weights(float(p - fl))
            idx = np.clip(int(fl) - 3 + np.arange(8), 0, n_in - 1)
            taps = np.take(out, idx, axis=axis)
            res.append(np.tensordot(wgt, taps, axes=([0], [axis])) if axis == 0 else taps @ wgt)
        out = (np.stack(res, axis=axis)).astype(np.float32)
    return out


def super_resolve(frames: np.ndarray, factor: int = 4, iters: int = 200, eps: float = 1e-12):
    """(depth, warps [F][2][3], iterations [F]).  uint16 frames (Kinect v1,
    super_resolution.cpp): the fused image rounded half to even and saturated
    to uint16, a pixel no frame covers NaN before the resampling.  float32
    frames (Kinect v2, super_resolution_kv2.cpp:287-311): a pixel no frame
    covers is 0 and the float result is returned as is."""
    kv2 = np.asarray(frames).dtype == np.float32
    F, h, w = frames.shape
    img = frames.astype(np.float32)
    blur = gauss5(img)
    gx, gy = grad(blur)
    warps = np.tile(np.array([[1, 0, 0], [0, 1, 0]], np.float32), (F, 1, 1))
    its = np.zeros(F, np.int64)
    for f in range(1, F):
        warps[f], its[f] = ecc_affine(blur[0], blur[f], gx[f], gy[f], iters, eps)
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    warped = [img[0]]
    for f in range(1, F):
        m = warps[f]
        warped.append(bilinear(img[f], (m[0, 0] * x + m[0, 1] * y + m[0, 2]).astype(np.float32),
                               (m[1, 0] * x + m[1, 1] * y + m[1, 2]).astype(np.float32)))
    stack = np.stack(warped).astype(np.float64)
    pos = stack > 0
    with np.errstate(invalid="ignore", divide="ignore"):
        ze = (np.where(pos, stack, 0).sum(0) / pos.sum(0)).astype(np.float32)
    if kv2:
        ze[pos.sum(0) == 0] = 0
    hr = np.repeat(np.repeat(ze, factor, axis=0), factor, axis=1)
    lr = lanczos_down(hr, factor)
    if kv2:
        return lr.astype(np.float32), warps, its
    with np.errstate(invalid="ignore"):
        r = np.rint(lr)
        r = np.where(r > 0, r, 0)
        r = np.minimum(r, 65535)
    return r.astype(np.uint16), warps, its
