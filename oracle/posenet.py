"""CPU restatement of the learned pose proposal -- TEST INFRASTRUCTURE ONLY.

Used by tests/ to check the GPU network (lowcost3dreconstruction_gb300/csrc/
posenet.cu, posenet_train.cu); never by the library.  The reference has no
learned component (its coarse guess is centroid_align.cpp:102-130 followed by
Super4PCS, alignment.sh:106-113), so nothing here is pinned to reference
outputs: the network is checked against this restatement, and this
restatement's backward against finite differences of its own forward.

Arithmetic: the same bf16 roundings as the GPU (weights, layer inputs and
activations), products and sums in float64 (the GPU accumulates in fp32 in
an unspecified order inside the tensor core, hence the tolerances of the
tests).  ``exact=True`` drops every rounding (pure float64) for the
finite-difference check.
"""
from __future__ import annotations

import numpy as np

PTS = 1024
SCALE = 4.0
LAYOUT = [("W1", (64, 3)), ("b1", (64,)), ("W2", (128, 64)), ("b2", (128,)), ("W3", (1024, 128)), ("b3", (1024,)),
          ("H1", (512, 2048)), ("c1", (512,)), ("H2", (256, 512)), ("c2", (256,)), ("H3", (9, 256)), ("c3", (9,))]
PARAMS = sum(int(np.prod(s)) for _, s in LAYOUT)


def split(p: np.ndarray) -> dict[str, np.ndarray]:
    out, o = {}, 0
    for name, shape in LAYOUT:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def join(d: dict[str, np.ndarray]) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in LAYOUT])


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bf16 (round to nearest even), returned as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


# ------------------------------------------------------------------ sample
_M64 = (1 << 64) - 1


def splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def sample_indices(n: int, seed: int, cloud: int) -> np.ndarray:
    """Stratified sample i takes floor((i + u_i) n / PTS), u_i from splitmix64(seed ^ cloud<<32 ^ i)."""
    idx = np.zeros(PTS, np.int64)
    for i in range(PTS):
        h = splitmix64((seed ^ (cloud << 32) ^ i) & _M64)
        u = np.float32(h >> 40) * np.float32(1.0 / 16777216.0)
        j = int((float(i) + float(u)) * float(n) / PTS)
        idx[i] = min(j, n - 1)
    return idx


def sample(xyz: np.ndarray, seed: int, cloud: int) -> tuple[np.ndarray, np.ndarray]:
    """(pts [PTS][4], centroid [3]) as posenet.cu's k_sample builds them."""
    xyz = np.asarray(xyz, np.float32)
    fin = np.all(np.isfinite(xyz), axis=1)
    c = xyz[fin].astype(np.float64).mean(axis=0) if fin.any() else np.zeros(3)
    out = np.zeros((PTS, 4), np.float32)
    if len(xyz):
        idx = sample_indices(len(xyz), seed, cloud)
        p = xyz[idx].astype(np.float64)
        ok = np.all(np.isfinite(p), axis=1)
        v = bf16(((p - c) * SCALE).astype(np.float32))
        out[ok, :3] = v[ok]
    return out, c


# ------------------------------------------------------------------ forward
def forward(params: np.ndarray, pts: np.ndarray, argmax: np.ndarray | None = None, exact: bool = False):
    """pts [2B][PTS][4] (sources, then targets).  Returns (feat [2B][1024],
    argmax [2B][1024], y [B][9], cache).  ``argmax`` given: use those winners
    (the values are still this restatement's)."""
    r = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: bf16(a).astype(np.float64))
    f32 = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: np.asarray(a, np.float32).astype(np.float64))
    P = split(np.asarray(params, np.float64 if exact else np.float32))
    C2 = pts.shape[0]
    B = C2 // 2
    x = np.asarray(pts, np.float64)[:, :, :3]
    W1 = r(P["W1"])
    b1 = P["b1"].astype(np.float64)
    if exact:
        z1 = x @ W1.T + b1
    else:  # the GPU's fmaf chain b + w0 x + w1 y + w2 z, exact products, fp32 sums
        acc = np.broadcast_to(b1.astype(np.float32), x.shape[:2] + (64,)).copy()
        for i in range(3):
            acc = (acc + (W1[:, i][None, None, :] * x[:, :, i:i + 1]).astype(np.float32)).astype(np.float32)
        z1 = acc.astype(np.float64)
    h1 = r(np.maximum(z1, 0.0))
    z2 = f32(f32(h1 @ r(P["W2"]).T) + P["b2"].astype(np.float64))
    h2 = r(np.maximum(z2, 0.0))
    x3 = h2 @ r(P["W3"]).T                                  # [2B][PTS][1024]
    if argmax is None:
        argmax = np.argmax(x3, axis=1)                      # lowest index among equal maxima
    m = np.take_along_axis(x3, argmax[:, None, :], axis=1)[:, 0, :]
    feat = np.maximum(f32(f32(m) + P["b3"].astype(np.float64)), 0.0)
    X0 = r(np.concatenate([feat[:B], feat[B:]], axis=1))   # [B][2048]
    a1 = r(np.maximum(f32(X0 @ r(P["H1"]).T) + P["c1"], 0.0))
    a2 = r(np.maximum(f32(a1 @ r(P["H2"]).T) + P["c2"], 0.0))
    y = f32(a2 @ r(P["H3"]).T) + P["c3"].astype(np.float64)
    cache = dict(x=x, h1=h1, h2=h2, feat=feat, X0=X0, a1=a1, a2=a2, argmax=argmax, P=P, r=r)
    return feat, argmax, y, cache


def loss_and_grads(params: np.ndarray, pts: np.ndarray, labels: np.ndarray, argmax: np.ndarray | None = None,
                   exact: bool = False) -> tuple[float, np.ndarray, dict]:
    """Loss (mean over pairs of the summed squared error of the 9 outputs) and
    its gradient with respect to the parameter vector, by the chain rule of
    the forward above (the max-pool passes each channel's gradient to its
    winning point; ReLU masks are taken from the activations)."""
    feat, argmax, y, c = forward(params, pts, argmax, exact)
    r, P = c["r"], c["P"]
    B = y.shape[0]
    d = y - np.asarray(labels, np.float64)
    loss = float(np.sum(d * d) / B)
    dy = 2.0 * d / B
    g = {}
    g["H3"] = dy.T @ c["a2"]
    g["c3"] = dy.sum(0)
    dz2 = (dy @ r(P["H3"])) * (c["a2"] > 0)
    g["H2"] = dz2.T @ c["a1"]
    g["c2"] = dz2.sum(0)
    dz1 = (dz2 @ r(P["H2"])) * (c["a1"] > 0)
    g["H1"] = dz1.T @ c["X0"]
    g["c1"] = dz1.sum(0)
    dx0 = dz1 @ r(P["H1"])
    dg = np.concatenate([dx0[:, :1024], dx0[:, 1024:]], axis=0)        # [2B][1024]
    dm = dg * (feat > 0)
    h2, h1, x = c["h2"], c["h1"], c["x"]
    win = np.take_along_axis(h2, argmax[:, :, None], axis=1)           # [2B][1024][128]
    g["W3"] = np.einsum("lc,lck->ck", dm, win)
    g["b3"] = dm.sum(0)
    dh2 = np.zeros_like(h2)
    W3 = r(P["W3"])
    for cl in range(h2.shape[0]):
        np.add.at(dh2[cl], argmax[cl], dm[cl][:, None] * W3)
    dz2e = dh2 * (h2 > 0)
    g["W2"] = np.einsum("lpf,lpk->fk", dz2e, h1)
    g["b2"] = dz2e.sum((0, 1))
    dz1e = (dz2e @ r(P["W2"])) * (h1 > 0)
    g["W1"] = np.einsum("lpj,lpi->ji", dz1e, x)
    g["b1"] = dz1e.sum((0, 1))
    return loss, join(g), dict(y=y, feat=feat, argmax=argmax)


# ------------------------------------------------------------------- poses
def labels_from_transforms(T: np.ndarray, cen_src: np.ndarray, cen_tgt: np.ndarray) -> np.ndarray:
    """Targets [B][9]: first two columns of R, then (R c_src + t - c_tgt) * SCALE."""
    T = np.asarray(T, np.float64).reshape(-1, 4, 4)
    R, t = T[:, :3, :3], T[:, :3, 3]
    delta = np.einsum("bij,bj->bi", R, cen_src) + t - cen_tgt
    return np.concatenate([R[:, :, 0], R[:, :, 1], delta * SCALE], axis=1)


def transforms_from_outputs(y: np.ndarray, cen_src: np.ndarray, cen_tgt: np.ndarray) -> np.ndarray:
    """Gram-Schmidt of the two predicted columns, t = c_tgt + delta / SCALE - R c_src."""
    y = np.asarray(y, np.float64)
    a1, a2 = y[:, 0:3], y[:, 3:6]
    c0 = a1 / np.linalg.norm(a1, axis=1, keepdims=True)
    u = a2 - np.sum(c0 * a2, axis=1, keepdims=True) * c0
    c1 = u / np.linalg.norm(u, axis=1, keepdims=True)
    c2 = np.cross(c0, c1)
    R = np.stack([c0, c1, c2], axis=2)
    T = np.tile(np.eye(4), (len(y), 1, 1))
    T[:, :3, :3] = R
    T[:, :3, 3] = cen_tgt + y[:, 6:9] / SCALE - np.einsum("bij,bj->bi", R, cen_src)
    return T
