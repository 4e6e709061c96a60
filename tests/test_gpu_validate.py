"""Structural invariants of the sweep, checked on the device between the kernels.

In place of a memory checker, which is not available for these runs, every index the kernels
dereference is traced back to a few structures, and those are checked after insertion, merge,
cluster sums and the end of each sweep (lg_validate_sweeps):
* bond vertex ranges lie in their regions and are time ordered;
* segment offsets agree with the incident vertex counts, and vertex <-> segment links agree;
* union-find pointers decrease, and every parent is a root after the cluster sums;
* the next sweep's off-diagonal lists are ordered, and even per spin-1/2 site.
The checks run for chain, square, cubic, frozen, spin-S and field models, a mixed arena under
narrow and wide launch shapes, and a chain whose buffers grow during the checked sweeps.  The
validated sweeps also give the same trajectory as ordinary ones.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


MODELS = [
    dict(LATTICE="square", L=16, BETA=4.0),
    dict(LATTICE="chain", L=100, BETA=16.0),
    dict(LATTICE="cubic", L=6, BETA=2.0, Jxy=1.0, Jz=0.5, h=0.3),
    dict(LATTICE="cubic", L=4, BETA=1.5, Jxy=1.0, Jz=1.5, h=0.2),   # frozen graphs
    dict(LATTICE="chain", L=12, BETA=3.0, local_S=1),
    dict(LATTICE="chain", L=8, BETA=0.3, local_S=1.5, h=0.1),
]


@pytest.mark.parametrize("i", range(len(MODELS)))
def test_validated_sweeps_pass_and_match_plain_sweeps(lg, i):
    p = lg.make_params(SEED=70 + i, INITIAL_SPINS="random", SWEEPS=1000, THERMALIZATION=0,
                       **MODELS[i])
    a = lg.LoopWorker(p)
    a.run(5)
    a.validate_sweeps(12)
    b = lg.LoopWorker(p)
    b.run(17)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_validated_mixed_arena_under_both_shapes(lg):
    ps = [lg.make_params(SEED=90 + i, INITIAL_SPINS="random", SWEEPS=1000, THERMALIZATION=0, **m)
          for i, m in enumerate(MODELS)]
    for shape in (dict(insert_k=0.0, narrow_k=0.0), dict(insert_k=1e300, narrow_k=1e300)):
        b = lg.Batch(ps)
        b.shape = shape
        b.validate_sweeps(10)
        b.close()


def test_validated_sweeps_through_buffer_growth(lg):
    w = lg.LoopWorker(lg.make_params(LATTICE="square", L=12, BETA=0.5, SEED=9,
                                     INITIAL_SPINS="random", SWEEPS=1000, THERMALIZATION=0))
    w.validate_sweeps(3)
    w.set_beta(16.0)          # many more operators: regions overflow and grow
    w.validate_sweeps(8)
    w.close()
