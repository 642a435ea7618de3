"""Multi-tau correlator oracle (oracle/correlator.py) pinned on the reference's own correlator:
initialize / add / evaluate of SOURCE/gpu_water3D.cu (GW:2983-3107). The golden fixture holds its
output for a seeded random walk of 20000 values (tests/golden/make_golden.py); where the
reference checkout exists, oracle/build_ref.py compiles those functions from the reference's
sources and the oracle is compared with them on more inputs. Bit for bit in both cases."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from oracle import correlator as K

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def run_oracle(w):
    m = K.MultiTau()
    for x in w:
        m.add(float(x))
    return m.evaluate()


def test_oracle_matches_reference_golden():
    g = json.load(open(os.path.join(GOLD, "correlator_ref.json")))
    rng = np.random.default_rng(20261203)
    w = 0.5 + 0.01 * np.cumsum(rng.standard_normal(20000))
    t, f = run_oracle(w)
    assert [float(x).hex() for x in t] == g["t"]
    assert [float(x).hex() for x in f] == g["f"]


@pytest.fixture(scope="module")
def ref_lib():
    from oracle import build_ref
    try:
        lib = build_ref.build()
    except Exception as e:  # no nvcc or a failed build: the golden test still pins the oracle
        pytest.skip(f"reference correlator not buildable here: {e}")
    if lib is None:
        pytest.skip("reference checkout not present")
    return C.CDLL(lib)


@pytest.mark.parametrize("n", [1, 2, 15, 16, 17, 33, 1000, 65537])
def test_oracle_matches_reference_code(ref_lib, n):
    rng = np.random.default_rng(n)
    w = np.ascontiguousarray(0.3 + 0.2 * rng.random(n))
    t, f = np.zeros(512), np.zeros(512)
    k = ref_lib.ref_corr_run(w.ctypes.data_as(C.c_void_p), n, t.ctypes.data_as(C.c_void_p),
                             f.ctypes.data_as(C.c_void_p), 512)
    to, fo = run_oracle(w)
    assert k == len(to)
    assert np.array_equal(t[:k], to) and np.array_equal(f[:k], fo)


def test_max_mass():
    cells = np.zeros((8, 12), dtype=np.int64)
    cells[:, :6] = np.array([0, 1, 1, 2, 5, 1])
    assert K.max_mass(cells) == 3 / 6
