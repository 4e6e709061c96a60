"""Spin correlations and structure factor (looper's correlation.h) on the GPU.

* the exact integer sums behind the estimator equal the oracle's, sweep window and all, for
  all-pairs displacements on chain, square and cubic lattices, for one origin site, and for a
  chain inside a ragged batch                                                  (bit exact)
* "Spin Correlations", "Staggered Spin Correlations" and "Spin Structure Factor" of the S=1/2
  Heisenberg chain L=4 at T=0.5 (the reference's loop.op block with MEASURE[Correlations] and
  MEASURE[Structure Factor]) within 3.5 sigma of exact diagonalization
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


CASES = [
    dict(dim=1, L=16, beta=4.0, jxy=1.0, jz=1.0, h=0.0),
    dict(dim=2, L=6, beta=2.0, jxy=1.0, jz=0.5, h=0.0),
    dict(dim=3, L=4, beta=1.5, jxy=1.0, jz=1.5, h=0.2),
]


def _params(lg, m, seed, therm, **kw):
    return lg.make_params(LATTICE=m["dim"], L=m["L"], BETA=m["beta"], Jxy=m["jxy"], Jz=m["jz"],
                          h=m["h"], SEED=seed, SWEEPS=1000, THERMALIZATION=therm,
                          INITIAL_SPINS="random", **kw)


def _oracle_sums(m, seed, therm, sweeps, origin=-1):
    o = orc.Oracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=seed)
    tot = np.zeros(m["L"] ** m["dim"], dtype=np.int64)
    for k in range(sweeps):
        o.sweep(1)
        if k >= therm:
            spins = o.state()[0]
            tot += orc.correlation_sums(spins, m["dim"], m["L"], origin=origin)
    o.close()
    return tot


@pytest.mark.parametrize("i", range(len(CASES)))
def test_correlation_sums_bit_exact_vs_oracle(lg, i):
    m = CASES[i]
    seed, therm, sweeps = 900 + i, 3, 23
    g = lg.LoopWorker(_params(lg, m, seed, therm, MEASURE_CORRELATIONS=True,
                              MEASURE_STRUCTURE_FACTOR=True))
    g.run(10)
    g.run(sweeps - 10)  # two chunks: the host adds the sums chunk by chunk
    sums, n = g.correlation_sums(0)
    assert n == sweeps - therm
    ref = _oracle_sums(m, seed, therm, sweeps)
    assert sums.tolist() == ref.tolist()
    N = m["L"] ** m["dim"]
    assert sums[0] == n * N
    mean, err = g.correlations("Spin Correlations")
    assert np.allclose(mean, 0.25 * ref / n / N)
    sf, _ = g.correlations("Spin Structure Factor")
    assert np.allclose(sf, orc.structure_factor(0.25 * ref / n / N, m["dim"], m["L"]))
    g.close()


def test_origin_correlations_bit_exact_vs_oracle(lg):
    m = CASES[1]
    seed, therm, sweeps, origin = 77, 2, 15, 7
    g = lg.LoopWorker(_params(lg, m, seed, therm, MEASURE_CORRELATIONS=True, INITIAL_SITE=origin))
    g.run(sweeps)
    sums, n = g.correlation_sums(1)
    assert n == sweeps - therm
    assert sums.tolist() == _oracle_sums(m, seed, therm, sweeps, origin=origin).tolist()
    mean, _ = g.correlations("Spin Correlations")
    assert mean[origin] == pytest.approx(0.25)
    with pytest.raises(lg.LoopError):
        g.correlations("Spin Structure Factor")  # not requested
    with pytest.raises(lg.LoopError):
        g.correlation_sums(0)
    g.close()


def test_correlations_of_a_batch_member_equal_alone(lg):
    ps = [_params(lg, CASES[0], 31, 1, MEASURE_CORRELATIONS=True),
          _params(lg, CASES[2], 32, 0),
          _params(lg, CASES[1], 33, 2, MEASURE_STRUCTURE_FACTOR=True)]
    b = lg.Batch(ps)
    b.run(12)
    for i in (0, 2):
        alone = lg.LoopWorker(ps[i])
        alone.run(12)
        s_b, n_b = b.chain(i).correlation_sums(0)
        s_a, n_a = alone.correlation_sums(0)
        assert n_b == n_a and s_b.tolist() == s_a.tolist()
        alone.close()
    with pytest.raises(lg.LoopError):
        b.chain(1).correlations("Spin Correlations")
    b.close()


def test_correlations_vs_exact_diagonalization(lg):
    # the loop.op block: S=1/2 Heisenberg chain, L=4, T=0.5
    g = lg.LoopWorker(lg.make_params(LATTICE="chain", L=4, T=0.5, J=1.0, SEED=5,
                                     SWEEPS=1 << 16, THERMALIZATION=1 << 10,
                                     INITIAL_SPINS="random", MEASURE_CORRELATIONS=True,
                                     MEASURE_STRUCTURE_FACTOR=True))
    g.run((1 << 16) + (1 << 10))
    ref = orc.ed.thermal(1, 4, 0.5)
    for name in ("Spin Correlations", "Staggered Spin Correlations", "Spin Structure Factor"):
        mean, err = g.correlations(name)
        for r in range(4):
            if err[r] == 0:  # r = 0: exactly 1/4
                assert mean[r] == pytest.approx(ref[name][r], abs=1e-12)
            else:
                assert abs(mean[r] - ref[name][r]) <= 3.5 * err[r], (name, r, mean[r], err[r],
                                                                       ref[name][r])
    g.close()
