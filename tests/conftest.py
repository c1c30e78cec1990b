"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built
liblcr.so; everything else runs on the CPU (oracle, host logic, ABI surface)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblcr.so")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (and, where nvcc is present, the library) once per session."""
    from lowcost3dreconstruction_gb300 import build
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def ctx():
    from lowcost3dreconstruction_gb300 import build
    build.build_lib()
    from lowcost3dreconstruction_gb300.core import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def cfg0():
    """Config-0 pair: back-projected (metres) and voxel-downsampled at 2 mm by the oracle."""
    from lowcost3dreconstruction_gb300 import synthetic as S
    from oracle import oracle as O
    pr = S.config0_pair(0)
    prm = O.bp_params(640, 480, scale=0.001, depth_max=4000)
    src = O.backproject_v1(pr.src_frames[0], prm)
    tgt = O.backproject_v1(pr.tgt_frames[0], prm)
    vs, _ = O.voxel_grid(src, 0.002)
    vt, _ = O.voxel_grid(tgt, 0.002)
    return dict(pair=pr, src=src, tgt=tgt, vsrc=vs, vtgt=vt)


def random_cloud(n: int, seed: int, scale: float = 1.0, dup_frac: float = 0.0, lattice: float = 0.0) -> np.ndarray:
    from oracle.oracle import POINT_DTYPE
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(-scale, scale, size=(n, 3)).astype(np.float32)
    if lattice > 0:
        xyz = (np.round(xyz / lattice) * lattice).astype(np.float32)
    if dup_frac > 0 and n > 1:
        m = int(n * dup_frac)
        xyz[rng.integers(0, n, m)] = xyz[rng.integers(0, n, m)]
    out = np.zeros(n, dtype=POINT_DTYPE)
    out["x"], out["y"], out["z"] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    out["normal_x"], out["normal_y"], out["normal_z"] = nrm[:, 0], nrm[:, 1], nrm[:, 2]
    out["r"], out["g"], out["b"] = rng.integers(0, 256, (3, n), dtype=np.uint8)
    out["curvature"] = rng.uniform(0, 0.1, n).astype(np.float32)
    return out
