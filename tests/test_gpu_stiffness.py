"""Spin stiffness: the reference's default "Stiffness" observable (stiffness.h:41-160).

Its per-sweep inputs are exact integer winding sums and are compared bit for bit with the oracle
by the record parity tests.  Here the two estimators of the same model are checked against each
other.  The improved estimator averages the sum over clusters of the squared cluster winding;
the normal estimator averages the square of the total winding.  Both estimate
<sum_d (W_d/2)^2> / (beta dim), since the cluster flips make the cross terms average to zero.
"""
import math

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


@pytest.mark.parametrize("lattice,L,beta", [("chain", 16, 4.0), ("square", 6, 2.0), ("cubic", 4, 1.0)])
def test_improved_and_normal_stiffness_agree(lg, lattice, L, beta):
    vals = []
    for disable in (0, 1):
        w = lg.LoopWorker(lg.make_params(LATTICE=lattice, L=L, BETA=beta, SEED=21, SWEEPS=1 << 15,
                                         THERMALIZATION=1 << 10, INITIAL_SPINS="random",
                                         DISABLE_IMPROVED_ESTIMATOR=disable))
        w.run((1 << 15) + (1 << 10))
        vals.append(w.observables()["Stiffness"])
        w.close()
    (a, ea), (b, eb) = vals
    assert a > 0 and b > 0
    assert abs(a - b) <= 4.0 * math.hypot(ea, eb) + 1e-12, (a, ea, b, eb)
    assert ea < eb  # the improved estimator has the smaller error
