"""The drop-in gpu_water3D executable on the GPU: same files in and out as the reference program,
and the reference sample run's statistics (SOURCE/data.out) reproduced from its own inputs."""
import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
EXE = os.path.join(ROOT, "cvfbulkwater_gb300", "_build", "gpu_water3D")
pytestmark = pytest.mark.gpu


def write_input(path, **kw):
    vals = dict(Pressure=0.45, Temperature=0.815, Seed=44648604, Metropolis_Steps=1, Cluster_Steps=0,
                Equilibrium_Steps=100, Sampling_Steps=1000, Sampling_Interval=10, R_cutoff=6.0,
                Flag_config=0, Flag_distances=0, Flag_correlation=0, Flag_chessboard=1, Device_ID=0)
    L = kw.pop("L", None)
    vals.update(kw)
    text = "".join(f"{k:28s}{v}\n" for k, v in vals.items())
    if L:
        text += f"Lattice_Size {L}\n"
    open(os.path.join(path, "input_data"), "w").write(text)


def run(path):
    r = subprocess.run([EXE], cwd=path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def test_driver_outputs(engine_lib, tmp_path):
    write_input(tmp_path, L=16, Cluster_Steps=1, Equilibrium_Steps=50, Sampling_Steps=505)
    run(tmp_path)
    data = [l.split() for l in open(tmp_path / "data.out")]
    assert len(data) == 51 and [int(d[0]) for d in data] == list(range(0, 505, 10))
    assert all(len(d) == 7 for d in data)
    cl = [l.split() for l in open(tmp_path / "cluster.out")]
    assert len(cl) == 51 and all(len(c) == 7 for c in cl)
    assert all(int(c[1]) >= int(c[2]) for c in cl)
    cfg = np.loadtxt(tmp_path / "config.out", dtype=np.int64)
    assert cfg.shape == (4096, 12) and np.all(cfg[:, 6:].sum(1) == 4) and cfg[:, :6].max() <= 5
    log = open(tmp_path / "water3D.log").read()
    assert "16 x 16 x 16 lattice" in log and "Max_SW_scans = 1" in log and "** simulation done" in log
    assert open(tmp_path / "distances").readline().split() == ["16", "16", "16"]
    # resume from config.out with the distances file (Flag_config=1, Flag_distances=1)
    shutil.copy(tmp_path / "config.out", tmp_path / "input_config")
    write_input(tmp_path, L=16, Flag_config=1, Flag_distances=1, Equilibrium_Steps=0, Sampling_Steps=10)
    run(tmp_path)
    assert len(open(tmp_path / "data.out").readlines()) == 1


def test_driver_rejects_bad_input(engine_lib, tmp_path):
    open(tmp_path / "input_data", "w").write("Pressure 0.45\nTemperature\n")
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Error [Temperature]" in r.stderr
    write_input(tmp_path, L=16, Flag_chessboard=2)
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Flag_chessboard" in r.stderr


def test_driver_non_chessboard_mode(engine_lib, tmp_path):
    """Flag_chessboard = 0: every eta stays 1, data.out carries the capped bond count."""
    write_input(tmp_path, L=8, Flag_chessboard=0, Cluster_Steps=1, Equilibrium_Steps=20, Sampling_Steps=200)
    run(tmp_path)
    data = np.loadtxt(tmp_path / "data.out")
    assert data.shape == (20, 7)
    assert np.all(data[:, 4] <= 2 * 512)  # at most 4 counted bonds per cell
    cfg = np.loadtxt(tmp_path / "config.out", dtype=np.int64)
    assert cfg.shape == (512, 12) and np.all(cfg[:, 6:] == 1)


def test_driver_reproduces_reference_statistics(engine_lib, tmp_path):
    """The reference's own input_data and input_config, unchanged (L=32, T=0.815, P=0.45, 10,000
    equilibration and 100,000 sampling steps, a record every 10): the same run length as the
    reference's data.out, every column within 2 combined standard errors (20 blocks each)."""
    shutil.copy(os.path.join(GOLD, "input_data.txt"), tmp_path / "input_data")
    cfg = np.load(os.path.join(GOLD, "input_config_L32.npz"))["cells12"]
    np.savetxt(tmp_path / "input_config", cfg, fmt="%d")
    run(tmp_path)
    d = np.loadtxt(tmp_path / "data.out")
    assert len(d) == 10000
    stats = json.load(open(os.path.join(GOLD, "data_out_stats.json")))["columns"]
    for col, name in [(1, "e"), (2, "h"), (3, "v"), (4, "n_hb"), (5, "m"), (6, "r_cell")]:
        x = d[:, col]
        b = x.reshape(20, -1).mean(1)
        err = b.std(ddof=1) / math.sqrt(20)
        z = (x.mean() - stats[name]["mean"]) / math.hypot(err, stats[name]["block_err"])
        assert abs(z) < 2.0, (name, x.mean(), stats[name]["mean"], z)
    assert "Energy:" in open(tmp_path / "water3D.log").read()
