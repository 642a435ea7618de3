"""File formats of the gpu_water3D contract, through the C ABI, against the reference's own files
(input_data, input_config, distances, data.out and cluster.out lines). No GPU needed."""
import ctypes as C
import os

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def test_read_reference_input_data(engine_lib):
    inp = abi.Input()
    assert engine_lib.cvf_read_input_data(os.path.join(GOLD, "input_data.txt").encode(), C.byref(inp)) == 0
    assert inp.P == pytest.approx(0.45) and inp.T == pytest.approx(0.815)
    assert inp.seed == 44648604
    assert (inp.metropolis_steps, inp.cluster_steps, inp.equilibrium_steps, inp.sampling_steps,
            inp.sampling_interval) == (1, 0, 10000, 100000, 10)
    assert inp.R_cutoff == pytest.approx(6.0)
    assert (inp.flag_config, inp.flag_distances, inp.flag_correlation, inp.flag_chessboard,
            inp.device_id) == (1, 0, 0, 1, 0)
    assert inp.L == 32


def test_input_data_errors_and_lattice_size(engine_lib, tmp_path):
    lines = open(os.path.join(GOLD, "input_data.txt")).read().splitlines()
    bad = tmp_path / "bad"
    bad.write_text("\n".join(lines[:3]) + "\n")
    inp = abi.Input()
    assert engine_lib.cvf_read_input_data(str(bad).encode(), C.byref(inp)) == -1
    assert engine_lib.cvf_last_error_string() == b"Error[Metropolis_Steps]: Can't read input file"
    bad.write_text("Pressure # 0.45\n")
    assert engine_lib.cvf_read_input_data(str(bad).encode(), C.byref(inp)) == -1
    assert engine_lib.cvf_last_error_string() == b"Error [Pressure]: Can't read input file"
    good = tmp_path / "good"
    good.write_text("\n".join(lines) + "\nLattice_Size 16\n")
    assert engine_lib.cvf_read_input_data(str(good).encode(), C.byref(inp)) == 0
    assert inp.L == 16


def test_config_file_roundtrip(engine_lib, tmp_path):
    cfg = np.load(os.path.join(GOLD, "input_config_L32.npz"))["cells12"].astype(np.int32)
    path = tmp_path / "config.out"
    assert engine_lib.cvf_write_config_file(str(path).encode(), P(cfg), len(cfg)) == 0
    text = path.read_text().splitlines()
    assert text[0] == " ".join(str(v) for v in cfg[0])
    back = np.zeros_like(cfg)
    assert engine_lib.cvf_read_config_file(str(path).encode(), P(back), len(cfg)) == 0
    assert np.array_equal(back, cfg)
    # reference checks: out-of-range values and short files (GW:759-800)
    bad = cfg[:4].copy()
    bad[2, 3] = 6
    np.savetxt(tmp_path / "bad", bad, fmt="%d")
    out = np.zeros((4, 12), dtype=np.int32)
    assert engine_lib.cvf_read_config_file(str(tmp_path / "bad").encode(), P(out), 4) == -1
    assert b"Unexpected value for spin (6)" in engine_lib.cvf_last_error_string()
    assert engine_lib.cvf_read_config_file(str(tmp_path / "bad").encode(), P(np.zeros((5, 12), np.int32)), 5) == -1


def test_distances_file_matches_reference(engine_lib, oracle_mod, tmp_path):
    d, f = oracle_mod.distances(32, 6.0)
    path = tmp_path / "distances"
    assert engine_lib.cvf_write_distances_file(str(path).encode(), 32, P(d), P(f), len(d)) == 0
    assert path.read_text() == open(os.path.join(GOLD, "distances_L32_Rc6.txt")).read()
    dd = np.zeros(512, np.float32)
    ff = np.zeros(512, np.int32)
    n = C.c_int()
    assert engine_lib.cvf_read_distances_file(str(path).encode(), 32, P(dd), P(ff), 512, C.byref(n)) == 0
    # the file keeps six decimals (%f), so a table read back is the rounded one, as in the reference
    assert n.value == 30 and np.array_equal(ff[:30], f)
    assert np.array_equal(dd[:30], np.array(["%f" % x for x in d], dtype=np.float32))
    assert engine_lib.cvf_read_distances_file(str(path).encode(), 16, P(dd), P(ff), 512, C.byref(n)) == -1
    assert engine_lib.cvf_last_error_string() == b"Error: Distances file. X rank mismatch"


def test_data_and_cluster_line_formats(engine_lib):
    ref = open(os.path.join(GOLD, "data_out_head.txt")).readline()
    v = [float(x) for x in ref.split()]
    o = abi.Obs(0, 0, v[6], 0.0, 0.0, v[4], v[1], v[2], v[3], v[5])
    buf = C.create_string_buffer(256)
    n = engine_lib.cvf_format_data_line(buf, 256, int(v[0]), C.byref(o))
    assert buf.value.decode() == ref and n == len(ref)
    # the Cluster_Steps = 0 line of SOURCE/cluster.out: one cluster of 6N sites
    N6 = 6 * 32 ** 3
    c = abi.CStats(N6, 0, 1, 1, N6, N6 * N6, int(np.int32(np.uint32((N6 * N6) & 0xFFFFFFFF))), 0.0, 0.0,
                   np.float32(N6), np.float32(0.0) - np.float32(N6) * np.float32(N6))
    engine_lib.cvf_format_cluster_line(buf, 256, 0, C.byref(c))
    assert buf.value.decode() == open(os.path.join(GOLD, "cluster_out_head.txt")).readline()
