"""The tile union-find (lattice patches in shared memory, then the crossing vertices globally)
against the oracle and against the all-global union-find.

The patches only exist on lattices larger than one tile, so these cases are larger than the
small parity models: square, cubic (with a field, and with frozen graphs) and a long chain, at
every tile capacity.  The last test makes tiles whose segments exceed shared memory, which take
the fallback path (every vertex and segment handled globally), next to ordinary tiles in the
same arena.  Every comparison is bit for bit: spins, operator strings and the integer records.
"""
import numpy as np
import pytest

import oracle_lib as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


CASES = {
    "square40_b12": dict(dim=2, L=40, beta=12.0, jxy=1.0, jz=1.0, h=0.0),
    "cubic10_xxz_field": dict(dim=3, L=10, beta=3.0, jxy=1.0, jz=0.5, h=0.3),
    "cubic8_frozen_field": dict(dim=3, L=8, beta=2.0, jxy=1.0, jz=1.5, h=0.2),
    "chain3000_b8": dict(dim=1, L=3000, beta=8.0, jxy=1.0, jz=1.0, h=0.0),
}


def _params(lg, m, seed):
    return lg.make_params(LATTICE=m["dim"], L=m["L"], BETA=m["beta"], Jxy=m["jxy"], Jz=m["jz"],
                          h=m["h"], SEED=seed, SWEEPS=1000, THERMALIZATION=0,
                          INITIAL_SPINS="random")


def _oracle(m, seed):
    return orc.Oracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=seed)


def _assert_same_state(g, o):
    gs, gb, gt = g.state()
    os_, ob, ot = o.state()
    assert gs.tolist() == os_.tolist()
    assert gb.tolist() == ob.tolist()
    assert gt.view(np.uint64).tolist() == ot.view(np.uint64).tolist()


@pytest.mark.parametrize("cap", [2048, 4096, 8192])
@pytest.mark.parametrize("name", sorted(CASES))
def test_tiles_bit_exact_vs_oracle(lg, name, cap):
    m = CASES[name]
    seed = 4242 + len(name)
    g = lg.LoopWorker(_params(lg, m, seed))
    g.shape = dict(tile_cap=cap)
    g.keep_records(True)
    o = _oracle(m, seed)
    for _ in range(2):
        g.run(3)
        o.sweep(3)
        _assert_same_state(g, o)
    assert (g.fetch_records() == o.records()).all()
    o.close()
    g.close()


def test_tiles_equal_global_union_find_after_retiling(lg):
    # the tiling follows the last sweep's operator count after autotuning-style re-shaping
    m = CASES["square40_b12"]
    runs = []
    for caps in ([0, 0], [4096, 2048], [8192, 4096]):
        g = lg.LoopWorker(_params(lg, m, 99))
        g.keep_records(True)
        for cap in caps:
            g.shape = dict(tile_cap=cap)
            g.run(4)
        runs.append((g.state(), g.fetch_records()))
        g.close()
    for (st, rec) in runs[1:]:
        for x, y in zip(runs[0][0], st):
            assert np.array_equal(x, y)
        assert (rec == runs[0][1]).all()


def test_oversized_tiles_take_the_global_path(lg):
    # a long chain at very low temperature has thousands of segments per site: even a one-site
    # tile exceeds 2048 segments; the square and cubic chains beside it tile normally
    ms = [dict(dim=1, L=8, beta=2500.0, jxy=1.0, jz=1.0, h=0.0),
          dict(dim=2, L=24, beta=6.0, jxy=1.0, jz=1.0, h=0.0),
          dict(dim=3, L=6, beta=1.0, jxy=1.0, jz=0.5, h=0.2)]
    b = lg.Batch([_params(lg, m, 500 + i) for i, m in enumerate(ms)])
    b.shape = dict(tile_cap=2048)
    b.run(4)
    for i, m in enumerate(ms):
        o = _oracle(m, 500 + i)
        o.sweep(4)
        _assert_same_state(b.chain(i), o)
        o.close()
    b.close()
