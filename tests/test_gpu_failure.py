"""Failure detection without a GPU fault.

Every device loop whose trip count depends on the data has a cap and reports LG_EITERCAP
instead of hanging.  These tests:
* lower the union-find cap through a test seam, so that the sweep gives up at once (on the
  chain-resident path and on the grid path with each way of making the unions);
* check that the error is reported, stays reported (the sweep had already overwritten the
  chain's operator lists), and is cleared by loading a checkpoint, after which the chain
  continues exactly like an undisturbed one;
* check that a request whose vertex capacity cannot be addressed is refused before allocation;
* check that the CUDA context stays usable throughout.
No test traps, faults or hangs the GPU.
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


def _params(lg):
    return lg.make_params(LATTICE="square", L=8, BETA=2.0, SEED=21, SWEEPS=1000,
                          THERMALIZATION=0, INITIAL_SPINS="random")


@pytest.mark.parametrize("shape", [None, dict(resident=0, union_mode=0),
                                   dict(resident=0, union_mode=1), dict(resident=0, union_mode=2)],
                         ids=["default", "grid-lanes", "grid-pairs", "grid-balanced"])
def test_union_find_cap_is_reported_and_recoverable(lg, shape):
    w = lg.LoopWorker(_params(lg))
    if shape is not None:
        w.shape = shape
    w.run(5)
    blob = w.save()
    w.set_iteration_cap(-1)          # no union may run: the next sweep stops
    with pytest.raises(lg.LoopError) as e:
        w.run(3)
    assert e.value.code == -5 and "iteration cap" in str(e.value)
    w.set_iteration_cap(0)           # default cap again, but the state is still lost
    with pytest.raises(lg.LoopError) as e:
        w.run(1)
    assert e.value.code == -5
    w.load(blob)                     # a checkpoint restores the chain
    w.run(3)
    ref = lg.LoopWorker(_params(lg))  # the same chain, undisturbed
    ref.run(8)
    for x, y in zip(w.state(), ref.state()):
        assert np.array_equal(x, y)
    w.close()
    ref.close()


def test_unaddressable_capacity_is_refused_before_allocation(lg):
    # about 1.6e11 expected operators: beyond the 2^30 vertex slots one arena addresses
    with pytest.raises(lg.LoopError) as e:
        lg.LoopWorker(lg.make_params(LATTICE="square", L=1024, BETA=1e5))
    assert e.value.code == -6


def test_context_usable_after_failures(lg):
    w = lg.LoopWorker(_params(lg))
    w.run(4)
    assert w.observables()["count"] == 4
    w.close()
