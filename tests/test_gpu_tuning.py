"""The autotuner's choices change the thread mapping or the launch, never the chain.

cvf_autotune picks the sweep tile (cells per thread), the row order of the sweep (rows by y then
z, or patches of 2, 4 or 8 rows in y across z planes) and, for a batch, the launch mode; it saves
and restores the state it times on. Every row order must give the oracle's lattice bit for bit,
and a tuned batch must continue exactly as an untuned copy of it.
"""
import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L,tile", [(16, 4), (16, 8), (24, 4), (32, 2)])
@pytest.mark.parametrize("lg_rows", [-1, 1, 2, 3])
def test_row_orders_match_oracle(engine_lib, oracle_mod, L, tile, lg_rows):
    # L = 24 and lg_rows = 3: 8 divides 24, a patch of 8 rows; the SW step runs beside the sweeps
    eng = Lattice(Params(L=L, T=0.7, P=0.45, seed=300 + L, start=0))
    assert eng.set_sweep_tile(tile) == tile
    eng.set_row_tile(lg_rows)
    ora = oracle_mod.Oracle(L, 0.7, 0.45, 300 + L, 6.0, 0, 0)
    for step in range(4):
        eng.run(1, 2, 1 if step == 2 else 0)
        ora.step(2, 1 if step == 2 else 0)
    assert np.array_equal(eng.get_config(), ora.get_config())
    ob, oo = eng.observables(), ora.measure()
    assert (ob.n_hb2, ob.n_sigma) == (oo.n_hb2, oo.n_sigma)
    tile_now, lg_now, _ = eng.tuning()
    assert tile_now == tile and lg_now == (lg_rows if (lg_rows < 0 or (1 << lg_rows) < L) else -1)


def test_autotuned_batch_continues_the_same_chain(engine_lib):
    specs = [(16, 0.6, 0.0), (32, 0.9, 0.6), (24, 0.75, 0.3), (32, 0.55, 0.45)]

    def make():
        return Lattice([Params(L=L, T=T, P=P, seed=900 + i, start=0, replica=i) for i, (L, T, P) in enumerate(specs)])

    a, b = make(), make()
    a.run(3, 1, 0)
    b.run(3, 1, 0)
    tile = a.autotune()
    t, lg, mode = a.tuning()
    assert t == tile and tile in (1, 2, 4, 8) and lg in (-1, 1, 2, 3) and mode in (0, 1)
    a.run(7, 1, 0)
    b.run(7, 1, 0)
    for r in range(len(specs)):
        assert np.array_equal(a.get_config(r), b.get_config(r))
        assert a.state(r)[:2] == b.state(r)[:2]
        assert list(a.state(r)[3]) == list(b.state(r)[3])
