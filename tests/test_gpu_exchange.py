"""Exchange Monte Carlo (parallel tempering) over a temperature ladder in one arena.

The reference runs loop_worker under ALPS parapack's exchange worker with the hooks
weight_parameter() = operator count and log_weight(n, beta) = n log beta
(path_integral.C:98-109, 874-875).  Checks:
* the ladder is deterministic, stays a permutation of the chains, and accepts some swaps;
* a chain of the ladder follows exactly the trajectory of the same chain run alone with the same
  inverse temperature history (set_beta between blocks): a swap only changes beta;
* the observables accumulated per temperature agree with exact diagonalization.
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


def _params(lg, **kw):
    base = dict(LATTICE="chain", L=8, SEED=77, SWEEPS=1 << 12, THERMALIZATION=1 << 8,
                INITIAL_SPINS="random")
    base.update(kw)
    return lg.make_params(**base)


def test_ladder_is_deterministic_and_a_permutation(lg):
    betas = [1.0, 1.5, 2.25, 3.4]
    runs = []
    for _ in range(2):
        x = lg.Exchange(_params(lg), betas)
        x.run(1200, interval=2)
        cot, att, acc = x.state()
        obs = [x.observables(t)["Energy"] for t in range(len(betas))]
        runs.append((cot.copy(), att.copy(), acc.copy(), obs))
        x.close()
    (cot, att, acc, obs), (cot2, att2, acc2, obs2) = runs
    assert sorted(cot.tolist()) == list(range(len(betas)))
    np.testing.assert_array_equal(cot, cot2)
    np.testing.assert_array_equal(att, att2)
    np.testing.assert_array_equal(acc, acc2)
    assert obs == obs2
    assert att.sum() == 600 + 300 - 0  # 600 steps: pairs (0,1),(2,3) on even, (1,2) on odd steps
    assert (acc > 0).all() and (acc <= att).all()


def test_ladder_chain_equals_the_chain_alone_with_the_same_beta_history(lg):
    betas = [0.8, 1.2, 1.8]
    kw = dict(LATTICE="square", L=4, SWEEPS=1000, THERMALIZATION=0)
    x = lg.Exchange(_params(lg, **kw), betas)
    interval = 3
    history = []
    for _ in range(16):
        cot, _, _ = x.state()
        history.append(betas[int(np.where(cot == 0)[0][0])])
        x.run(interval, interval)
    assert len(set(history)) > 1  # chain 0 changed temperature at least once
    sx, bx, tx = x.chain(0).state()
    w = lg.LoopWorker(_params(lg, SEED=lg.chain_seed(77, 0), BETA=history[0], **kw))
    for b in history:
        w.set_beta(b)
        w.run(interval)
    sw, bw, tw = w.state()
    np.testing.assert_array_equal(sx, sw)
    np.testing.assert_array_equal(bx, bw)
    np.testing.assert_array_equal(tx.view(np.uint64), tw.view(np.uint64))
    w.close()
    x.close()


def test_observables_per_temperature_vs_exact_diagonalization(lg):
    betas = [1.0, 2.0, 4.0]
    L = 6
    x = lg.Exchange(_params(lg, L=L, SWEEPS=1 << 15, THERMALIZATION=1 << 10), betas)
    x.run((1 << 15) + (1 << 10), interval=1)
    _, att, acc = x.state()
    assert (acc > 0).all()
    for t, b in enumerate(betas):
        obs = x.observables(t)
        ref = orc.ed.thermal(1, L, 1.0 / b, jxy=1.0, jz=1.0, h=0.0)
        for k in ("Energy", "Susceptibility", "Staggered Magnetization^2"):
            mean, err = obs[k]
            assert abs(mean - ref[k]) <= 4.0 * err + 1e-9, (b, k, mean, err, ref[k])
    x.close()
