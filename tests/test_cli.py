"""The command-line tools are drop-ins for pcl_tools: same flags and defaults,
`-h` exits 0, usage and load errors exit 255 (the reference's `return -1`)
with the reference's messages.  CPU tests stop before any GPU work; the
`gpu` tests run the tools end to end against the oracle."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import random_cloud

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "lowcost3dreconstruction_gb300" / "bin"

# tool -> flags its help must list (pcl_tools/<tool>.cpp option tables)
TOOLS = {
    "cloud_downsampling": ["--input", "--output", "--leaf_size"],
    "outlier_removal": ["--input", "--output", "--outliers_file", "--neighbors", "--dev_mult"],
    "normal_estimation": ["--input", "--output", "--neighbors", "--reverse_normals", "--centroid", "--origin"],
    "fine_registration": ["--input", "--target", "--output", "--accumulated", "--distance_threshold",
                          "--max_iterations", "--transformation_epsilon", "--euclidean_fitness_epsilon"],
    "accumulate_clouds": ["--input", "--target", "--output", "--radius", "--clean_neighbors", "--dev_mult",
                          "--negative", "--all"],
    "centroid_align": ["--input", "--target", "--output", "--roll", "--pitch", "--yaw", "--elevation"],
    "transform": ["--input", "--output", "--transform"],
    "scale": ["--input", "--output", "--scale"],
    "crop_cloud": ["--input", "--output", "--radius", "--negative"],
    "cluster_extraction": ["--input", "--output", "--outliers_file", "--cluster_percentage", "--tolerance"],
    "planar_segmentation": ["--input", "--output", "--threshold", "--negative"],
}


@pytest.fixture(scope="module", autouse=True)
def tools():
    from lowcost3dreconstruction_gb300 import build
    build.build_lib()
    build.build_tools()


def run(tool, *args, cwd=None):
    return subprocess.run([str(BIN / tool), *map(str, args)], capture_output=True, text=True, timeout=120, cwd=cwd)


@pytest.mark.parametrize("tool", sorted(TOOLS))
def test_help_lists_the_reference_flags(tool):
    r = run(tool, "-h")
    assert r.returncode == 0, r.stderr
    for f in TOOLS[tool]:
        assert f in r.stdout, (tool, f)


@pytest.mark.parametrize("tool", sorted(TOOLS))
def test_missing_arguments_exit_255_with_usage(tool):
    r = run(tool)
    assert r.returncode == 255
    assert "Correct mode of use" in (r.stdout + r.stderr)


@pytest.mark.parametrize("tool", ["outlier_removal", "fine_registration", "cloud_downsampling"])
def test_unknown_option_exits_255(tool):
    r = run(tool, "--bogus", "1")
    assert r.returncode == 255


def test_missing_input_file_message(tmp_path):
    r = run("outlier_removal", "-i", tmp_path / "nope.ply", "-o", tmp_path / "o.ply")
    assert r.returncode == 255
    assert "Couldn't load input point cloud" in (r.stdout + r.stderr)


def test_fine_registration_rejects_nonpositive_iterations(tmp_path):
    from lowcost3dreconstruction_gb300 import _lib as L
    pts = random_cloud(50, 1)
    L.write_ply(tmp_path / "a.ply", pts)
    r = run("fine_registration", "-i", tmp_path / "a.ply", "-t", tmp_path / "a.ply", "-o", tmp_path / "o.ply",
            "--max_iterations", "0")
    assert r.returncode == 255
    assert "max_iterations needs to be greater than zero" in (r.stdout + r.stderr)


# ------------------------------------------------------------ end to end
@pytest.mark.gpu
def test_tools_chain_matches_oracle(tmp_path, cfg0):
    from lowcost3dreconstruction_gb300 import _lib as L
    from oracle import oracle as O
    src, tgt = cfg0["src"], cfg0["tgt"]
    L.write_ply(tmp_path / "s.ply", src)
    L.write_ply(tmp_path / "t.ply", tgt)
    assert run("cloud_downsampling", "-i", tmp_path / "s.ply", "-o", tmp_path / "sv.ply", "-s", "0.002").returncode == 0
    assert run("cloud_downsampling", "-i", tmp_path / "t.ply", "-o", tmp_path / "tv.ply", "-s", "0.002").returncode == 0
    sv = L.read_ply(tmp_path / "sv.ply")
    np.testing.assert_array_equal(sv["x"].view(np.uint32), cfg0["vsrc"]["x"].view(np.uint32))
    r = run("outlier_removal", "-i", tmp_path / "sv.ply", "-o", tmp_path / "so.ply", "-n", "20", "-d", "2.0")
    assert r.returncode == 0, r.stderr
    _, keep, _ = O.sor(cfg0["vsrc"], 20, 2.0)
    assert len(L.read_ply(tmp_path / "so.ply")) == int(keep.sum())
    r = run("fine_registration", "-i", tmp_path / "sv.ply", "-t", tmp_path / "tv.ply", "-o", tmp_path / "reg.ply",
            "--distance_threshold", "0.05", "--max_iterations", "50", "--transformation_epsilon", "1e-8")
    assert r.returncode == 0, r.stderr
    assert "Has converged" in r.stdout and "Score" in r.stdout
    ref = O.icp(cfg0["vsrc"], cfg0["vtgt"], max_corr_dist=0.05, max_iterations=50, transformation_epsilon=1e-8)
    reg = L.read_ply(tmp_path / "reg.ply")
    want = O.transform(cfg0["vsrc"], ref["transform"].astype(np.float32))
    np.testing.assert_allclose(reg["x"], want["x"], atol=2e-5)


# ------------------------------------------------------------ rotate_align
def test_rotate_align_help_and_gui():
    r = run("rotate_align", "-h")
    assert r.returncode == 0
    for f in ("--gui", "--accumulated_file", "--capture_name", "--capture_step", "--num_captures", "--distance_x",
              "--distance_y", "--distance_z"):
        assert f in r.stdout, f
    r = run("rotate_align", "-g")
    assert r.returncode == 255 and "not available" in r.stderr


def test_rotate_align_missing_captures(tmp_path):
    """Unreadable views are reported and stay empty; the tool still writes every output."""
    r = run("rotate_align", "-n", "cap", "-s", "10", "-c", "2", cwd=tmp_path)
    assert r.returncode == 0
    assert "cap0.ply is not a valid file." in r.stdout and "cap10.ply is not a valid file." in r.stdout
    from lowcost3dreconstruction_gb300 import _lib as L
    for a in (0, 10):
        assert len(L.read_ply(tmp_path / f"cap{a}_rotated.ply")) == 0


@pytest.mark.gpu
def test_rotate_align_matches_oracle(tmp_path):
    from lowcost3dreconstruction_gb300 import _lib as L
    from oracle import oracle as O
    rng = np.random.default_rng(3)
    views = []
    for i in range(3):
        p = random_cloud(500 + 100 * i, 10 + i)
        p["x"][::50] = np.nan
        L.write_ply(tmp_path / f"v{20 * i}.ply", p)
        views.append(p)
    r = run("rotate_align", "-n", "v", "-s", "20", "-c", "3", "-a", "all.ply", "-x", "1.5", "-y", "-2", "-z", "30",
            cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("LOADED ALRIGHT!") == 3
    acc = []
    for i, p in enumerate(views):
        fin = p[np.isfinite(p["x"]) & np.isfinite(p["y"]) & np.isfinite(p["z"])]
        T = np.eye(4, dtype=np.float32)
        T[:3, 3] = [1.5, -2.0, 30.0]
        a = np.float32(-((20 * i + i * 1.17) * 0.017453293))
        c, s = np.float32(np.cos(a)), np.float32(np.sin(a))
        R = np.eye(4, dtype=np.float32)
        R[0, 0], R[2, 2], R[0, 2], R[2, 0] = c, c, s, -s
        want = O.transform(O.transform(fin, T), R)
        got = L.read_ply(tmp_path / f"v{20 * i}_rotated.ply")
        assert len(got) == len(want)
        for f in ("x", "y", "z", "normal_x", "normal_y", "normal_z"):
            np.testing.assert_allclose(got[f], want[f], rtol=1e-6, atol=1e-5, err_msg=f)
        acc.append(got)
    allp = L.read_ply(tmp_path / "all.ply")
    np.testing.assert_array_equal(allp["x"], np.concatenate([a["x"] for a in acc]))


# ------------------------------------------------------------ pose_proposal
def test_pose_proposal_usage():
    r = run("pose_proposal", "-h")
    assert r.returncode == 0
    for f in ("--input", "--matrix", "--registered", "--units", "--refine", "--weights"):
        assert f in r.stdout, f
    r = run("pose_proposal", "-i", "only_one.ply")
    assert r.returncode == 255 and "Correct mode of use" in (r.stdout + r.stderr)


@pytest.mark.gpu
@pytest.mark.parametrize("units", [1.0, 0.1])
def test_pose_proposal_drops_into_the_coarse_stage(tmp_path, ctx, units):
    """Super4PCS's place in alignment.sh: matrix file with two header lines
    (deleted by the script), then `transform -t` moves Q onto P."""
    from lowcost3dreconstruction_gb300 import _lib as L
    from lowcost3dreconstruction_gb300 import train_posenet as TP
    src, tgt, T = ctx.synthetic_pairs(424_242, 1, 20000, yaw_deg=60.0)
    q, p = src[0].download(), tgt[0].download()
    for c in (q, p):
        for f in ("x", "y", "z"):
            c[f] /= np.float32(units)
    L.write_ply(tmp_path / "P.ply", p)
    L.write_ply(tmp_path / "Q.ply", q)
    r = run("pose_proposal", "-i", tmp_path / "P.ply", tmp_path / "Q.ply", "-m", tmp_path / "m.txt", "-r",
            tmp_path / "reg.ply", "-t", "15", "-o", "0.6", "-d", "0.03", "-n", "700", "-u", str(units))
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "m.txt").read_text().splitlines()
    M = np.array([[float(v) for v in ln.split()] for ln in lines[2:6]])
    assert TP.rotation_error_deg(M[None], T)[0] < 2.0
    np.testing.assert_allclose(M[:3, 3] * units, T[0, :3, 3], atol=0.01)
    (tmp_path / "t.txt").write_text("\n".join(lines[2:]) + "\n")   # sed -i '1,2d'
    assert run("transform", "-i", tmp_path / "Q.ply", "-o", tmp_path / "q2.ply", "-t", tmp_path / "t.txt").returncode == 0
    np.testing.assert_allclose(L.read_ply(tmp_path / "q2.ply")["x"], L.read_ply(tmp_path / "reg.ply")["x"], atol=1e-4)


@pytest.mark.parametrize("form", [["--input={f}", "--output={o}"], ["-i{f}", "-o", "{o}"], ["-i", "{f}", "--output", "{o}"]])
def test_option_spellings(tmp_path, form):
    """boost::program_options spellings the scripts may use: --name=value,
    -xvalue and separate values all reach the same load step."""
    args = [a.format(f=tmp_path / "nope.ply", o=tmp_path / "o.ply") for a in form]
    r = run("outlier_removal", *args)
    assert r.returncode == 255
    assert f"Couldn't load input point cloud: {tmp_path / 'nope.ply'}" in (r.stdout + r.stderr)
