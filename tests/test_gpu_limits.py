"""Device waits that run out of their bound end with an error status, not a hang.

The reference polls its Swendsen-Wang convergence flag from the host with no bound
(SOURCE/gpu_water3D.cu:1480-1555). The engine's waits are bounded on the device: a union that
keeps losing its atomicMin gives up after a number of attempts (error code 1), and a block of the
persistent step kernel waiting at a grid barrier gives up after a number of polls (error code 3);
either sets the replica's error word, the kernel returns, and the next cvf_synchronize reports
CVF_ELIMIT. cvf_set_wait_limits lowers the bounds to 0, so the error path runs on every launch
without a fault or a hang; a fresh handle afterwards still matches the oracle bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu

CVF_ELIMIT = -3


def _sync_rc(lat):
    return abi.lib().cvf_synchronize(lat._h)


def _fresh_matches_oracle(oracle_mod, nmet, ncl, launch_mode=0):
    eng = Lattice(Params(L=16, T=0.7, P=0.45, seed=404, start=0))
    eng.launch_mode = launch_mode
    ora = oracle_mod.Oracle(16, 0.7, 0.45, 404, 6.0, 0, 0)
    eng.run(4, nmet, ncl)
    for _ in range(4):
        ora.step(nmet, ncl)
    assert np.array_equal(eng.get_config(), ora.get_config())
    if ncl:
        assert np.array_equal(eng.labels(), ora.labels())
    eng.close()


def test_union_bound_reports_elimit(engine_lib, oracle_mod):
    lat = Lattice(Params(L=16, T=0.6, P=0.45, seed=404, start=0))
    assert engine_lib.cvf_set_wait_limits(lat._h, -1, 0) == 0
    lat.run(1, 0, 1)  # enqueues only; the error word is read at the next synchronisation
    assert _sync_rc(lat) == CVF_ELIMIT
    assert b"code 1" in engine_lib.cvf_last_error_string()
    lat.close()
    _fresh_matches_oracle(oracle_mod, 0, 1)


def test_grid_barrier_bound_reports_elimit(engine_lib, oracle_mod):
    lat = Lattice(Params(L=16, T=0.7, P=0.45, seed=404, start=0))
    lat.launch_mode = 1
    if lat.launch_mode != 1:
        pytest.skip("the persistent cooperative launch is not available on this device")
    assert engine_lib.cvf_set_wait_limits(lat._h, 0, -1) == 0
    lat.run(2, 1, 0)
    assert _sync_rc(lat) == CVF_ELIMIT
    assert b"code 3" in engine_lib.cvf_last_error_string()
    lat.close()
    _fresh_matches_oracle(oracle_mod, 1, 0, launch_mode=1)


def test_wolff_grid_barrier_bound_reports_elimit(engine_lib, oracle_mod):
    """The Wolff step's cooperative grid waits at the same bounded barrier (three per batch)."""
    lat = Lattice(Params(L=16, T=0.7, P=0.45, seed=404, start=0))
    lat.set_cluster_algorithm(True)
    assert engine_lib.cvf_set_wait_limits(lat._h, 0, -1) == 0
    lat.run(1, 0, 1)
    assert _sync_rc(lat) == CVF_ELIMIT
    assert b"code 3" in engine_lib.cvf_last_error_string()
    lat.close()
    eng = Lattice(Params(L=16, T=0.7, P=0.45, seed=404, start=0))
    eng.set_cluster_algorithm(True)
    ora = oracle_mod.Oracle(16, 0.7, 0.45, 404, 6.0, 0, 0)
    ora.set_wolff(True)
    eng.run(2, 1, 1)
    for _ in range(2):
        ora.step(1, 1)
    assert np.array_equal(eng.get_config(), ora.get_config())
    assert eng.wolff_stats() == ora.wolff_stats()
    eng.close()


def test_default_bounds_restored(engine_lib, oracle_mod):
    """Negative values restore the defaults: the same handle then runs as an untouched one."""
    eng = Lattice(Params(L=16, T=0.7, P=0.45, seed=404, start=0))
    assert engine_lib.cvf_set_wait_limits(eng._h, 0, 0) == 0
    assert engine_lib.cvf_set_wait_limits(eng._h, -1, -1) == 0
    ora = oracle_mod.Oracle(16, 0.7, 0.45, 404, 6.0, 0, 0)
    eng.run(4, 1, 1)
    for _ in range(4):
        ora.step(1, 1)
    assert _sync_rc(eng) == 0
    assert np.array_equal(eng.get_config(), ora.get_config())
    assert np.array_equal(eng.labels(), ora.labels())
