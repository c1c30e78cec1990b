"""Build recipe for the native parts of the package (no cmake, no setuptools).

* ``liblcr.so``   -- the CUDA kernels + C ABI, compiled for sm_103a only.
* ``bin/*``       -- the command-line tools (C++ host code over liblcr).
* ``oracle/liboracle.so`` -- the CPU oracle used by the tests and the CPU
  baseline (test infrastructure; the library never links it).

Translation units are compiled in parallel; everything lands in-tree and is
git-ignored.  ``python -m lowcost3dreconstruction_gb300.build`` runs it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "liblcr.so"
BIN = PKG / "bin"
ORACLE_SRC = ROOT / "oracle" / "oracle.cpp"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CU_SOURCES = ["api.cu", "context.cu", "sort.cu", "index.cu", "knn.cu", "icp.cu", "depth.cu", "voxel.cu",
              "filters.cu", "posenet.cu", "posenet_train.cu", "synth.cu", "tune.cu", "sfm.cu", "sr.cu"]
HOST_SOURCES = ["ply.cpp"]
TOOLS = ["fine_registration", "cloud_downsampling", "outlier_removal", "normal_estimation", "accumulate_clouds",
         "transform", "scale", "centroid_align", "depth_to_cloud", "rotate_align", "pose_proposal",
         "crop_cloud", "cluster_extraction", "planar_segmentation"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblcr")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_lib(jobs: int | None = None, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "lcr.h"]
    objs = []
    todo = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            todo.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    for src in HOST_SOURCES:
        s = CSRC / "host" / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s, ROOT / "include" / "lcr.h"]):
            todo.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo) or 1, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, todo))
    if todo or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart=static"])
    return LIB


# Tools with extra sources and libraries, built only where the library is present.
EXTRA_TOOLS = {"super_resolution": (["sr_tool.cpp", "png16.cpp"], ["-lz", "-pthread"], "zlib.h"),
               "super_resolution_kv2": (["sr_tool.cpp", "png16.cpp"], ["-lz", "-pthread"], "zlib.h")}


def _have_header(name: str) -> bool:
    res = subprocess.run(["g++", "-x", "c++", "-fsyntax-only", "-"], input=f"#include <{name}>\n", text=True,
                         capture_output=True)
    return res.returncode == 0


def build_tools() -> None:
    BIN.mkdir(exist_ok=True)
    common = [CSRC / "host" / "cli_common.cpp"]
    if not all(c.exists() for c in common):
        return
    deps = common + list((CSRC / "host").glob("*.h")) + [ROOT / "include" / "lcr.h", ROOT / "include" / "lcr_pcl.hpp", LIB]
    cmds = []
    for t in TOOLS + [t for t, (_, _, hdr) in EXTRA_TOOLS.items() if _have_header(hdr)]:
        src = CSRC / "host" / f"{t}.cpp"
        out = BIN / t
        if not src.exists():
            continue
        extra_src, extra_libs, _ = EXTRA_TOOLS.get(t, ([], [], ""))
        extra = [CSRC / "host" / e for e in extra_src]
        if _stale(out, [src] + extra + deps):
            cmds.append(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(CSRC / "host"), str(src),
                         *map(str, extra), *map(str, common), "-o", str(out), "-L", str(PKG), "-llcr", *extra_libs,
                         "-Wl,-rpath,$ORIGIN/.."])
    with cf.ThreadPoolExecutor(max_workers=min(len(cmds) or 1, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, cmds))


def build_oracle() -> Path:
    srcs = [ORACLE_SRC, ORACLE_SRC.parent / "sr_oracle.cpp"]
    if _stale(ORACLE_LIB, srcs + [ORACLE_SRC.with_suffix(".h")]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-o", str(ORACLE_LIB),
              *map(str, srcs)])
    return ORACLE_LIB


def build_all(with_oracle: bool = True) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fo = ex.submit(build_oracle) if with_oracle else None
        build_lib()
        if fo is not None:
            fo.result()
    build_tools()


if __name__ == "__main__":
    build_all()
    print(f"built {LIB}")
