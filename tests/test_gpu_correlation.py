"""The multi-tau correlator on the GPU (Flag_correlation; GW:1245-1313, GW:2983-3128) against the
oracle (oracle/correlator.py, pinned on the reference's own correlator) on the same Markov chain:
after every step the oracle takes the most-populated sigma fraction of its lattice and adds it.
The evaluated (t, f) must agree bit for bit; so must correlation.dat of the drop-in driver."""
import os
import subprocess

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params
from oracle import correlator as K

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "cvfbulkwater_gb300", "_build", "gpu_water3D")


def oracle_run(oracle_mod, L, T, P, seed, replica, start, equil, steps, nmet=1):
    ora = oracle_mod.Oracle(L, T, P, seed, 6.0, replica, start)
    for _ in range(equil):
        ora.step(nmet, 0)
    m = K.MultiTau()
    for _ in range(steps):
        ora.step(nmet, 0)
        m.add(K.max_mass(ora.get_config()))
    return m.evaluate()


def test_device_correlator_matches_oracle(engine_lib, oracle_mod):
    specs = [(8, 0.70, 0.45), (6, 0.90, 0.10)]
    lat = Lattice([Params(L=L, T=T, P=P, seed=900 + i, start=0, replica=i) for i, (L, T, P) in enumerate(specs)])
    lat.run(20, 1, 0)
    lat.set_correlation(True)
    lat.run(37, 1, 0)            # a 32-step graph and a remainder
    lat.run_sampled(50, 1, 0, 7)  # recorded steps take the fused-measurement path
    lat.run(13, 1, 0)
    for r, (L, T, P) in enumerate(specs):
        t, f = lat.correlation(r)
        to, fo = oracle_run(oracle_mod, L, T, P, 900 + r, r, 0, 20, 100)
        assert len(t) == len(to) > 16
        assert np.array_equal(t, to) and np.array_equal(f, fo), r


def test_correlation_reset_and_stop(engine_lib, oracle_mod):
    lat = Lattice(Params(L=8, T=0.8, P=0.45, seed=4, start=0))
    lat.set_correlation(True)
    lat.run(30, 1, 0)
    lat.set_correlation(True)  # reset
    lat.run(40, 1, 0)
    lat.set_correlation(False)
    lat.run(25, 1, 0)  # not added
    t, f = lat.correlation()
    ora = oracle_mod.Oracle(8, 0.8, 0.45, 4, 6.0, 0, 0)
    for _ in range(30):
        ora.step(1, 0)
    m = K.MultiTau()
    for _ in range(40):
        ora.step(1, 0)
        m.add(K.max_mass(ora.get_config()))
    to, fo = m.evaluate()
    assert np.array_equal(t, to) and np.array_equal(f, fo)


def test_driver_writes_reference_correlation_file(engine_lib, oracle_mod, tmp_path):
    vals = dict(Pressure=0.45, Temperature=0.815, Seed=44648604, Metropolis_Steps=1, Cluster_Steps=0,
                Equilibrium_Steps=40, Sampling_Steps=300, Sampling_Interval=10, R_cutoff=6.0,
                Flag_config=0, Flag_distances=0, Flag_correlation=1, Flag_chessboard=1, Device_ID=0)
    text = "".join(f"{k:28s}{v}\n" for k, v in vals.items()) + "Lattice_Size 8\n"
    open(tmp_path / "input_data", "w").write(text)
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    t, f = oracle_run(oracle_mod, 8, np.float32(0.815), np.float32(0.45), 44648604, 0, 0, 40, 300)
    assert open(tmp_path / "correlation.dat").read() == K.correlation_text(t, f)
