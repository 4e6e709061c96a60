"""Spin S > 1/2 on the GPU: 2S virtual spin-1/2 sites per site, every real bond as the (2S)^2
virtual bonds of looper's virtual graph, and the random boundary matching of the virtual sites at
tau = 0 (path_integral.C:590-613, permutation.h:91-111).

* whole trajectories (spins, operator strings, per-sweep records) equal the oracle's, bit for bit,
  for S = 1 and S = 3/2 chains with and without anisotropy and field, a spin-1 ferromagnet, and
  S = 1, 3/2 and 2 on square and simple-cubic lattices (up to 24 virtual bonds per virtual site)
* a spin-S chain inside a batch with spin-1/2 chains equals the chain alone
* observables of the S = 1 Heisenberg chain L = 4 at T = 0.5 (the reference's loop.op block),
  of an S = 3/2 XXZ chain in a field, and of S = 1 on the 2x2 square and S = 1 XXZ in a field on
  the 2x2x2 cube within 3.5 sigma of exact diagonalization
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


MODELS = {
    "s1_heisenberg": dict(L=8, beta=4.0, jxy=1.0, jz=1.0, h=0.0, spin2=2),
    "s1_xxz_field": dict(L=6, beta=2.0, jxy=1.0, jz=0.5, h=0.2, spin2=2),
    "s3half_heisenberg": dict(L=6, beta=2.0, jxy=1.0, jz=1.0, h=0.0, spin2=3),
    "s1_ferro_odd": dict(L=5, beta=1.5, jxy=-1.0, jz=-1.0, h=0.1, spin2=2),
    # few operators: many virtual sites have a single segment, which is both their bottom and
    # their top and so takes part in two boundary pairs
    "s3half_sparse": dict(L=6, beta=0.3, jxy=1.0, jz=1.0, h=0.1, spin2=3),
    # higher dimensions: 2 dim 2S virtual bonds at every virtual site (8, 12, 12, 18, 16)
    "square_s1": dict(dim=2, L=4, beta=2.0, jxy=1.0, jz=1.0, h=0.0, spin2=2),
    "square_s1_xxz_field": dict(dim=2, L=4, beta=1.5, jxy=1.0, jz=0.5, h=0.2, spin2=2),
    "cubic_s1": dict(dim=3, L=2, beta=1.0, jxy=1.0, jz=1.0, h=0.0, spin2=2),
    "cubic_s3half_field": dict(dim=3, L=2, beta=0.7, jxy=1.0, jz=0.8, h=0.1, spin2=3),
    "square_s2": dict(dim=2, L=4, beta=0.8, jxy=1.0, jz=1.0, h=0.0, spin2=4),
}


def _params(lg, m, seed, **kw):
    return lg.make_params(LATTICE=m.get("dim", 1), L=m["L"], BETA=m["beta"], Jxy=m["jxy"], Jz=m["jz"],
                          h=m["h"], local_S=m["spin2"] / 2, SEED=seed, SWEEPS=1000,
                          THERMALIZATION=0, INITIAL_SPINS="random", **kw)


def _assert_same_state(g, o):
    gs, gb, gt = g.state()
    os_, ob, ot = o.state()
    assert gs.tolist() == os_.tolist()
    assert gb.tolist() == ob.tolist()
    assert gt.view(np.uint64).tolist() == ot.view(np.uint64).tolist()


@pytest.mark.parametrize("name", sorted(MODELS))
def test_spin_s_trajectory_bit_exact_vs_oracle(lg, name):
    m = MODELS[name]
    seed = 300 + len(name)
    g = lg.LoopWorker(_params(lg, m, seed))
    g.keep_records(True)
    dim = m.get("dim", 1)
    o = orc.Oracle(dim, m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=seed, spin2=m["spin2"])
    assert g.num_sites() == o.N == m["L"] ** dim * m["spin2"]
    for _ in range(3):
        g.run(10)
        o.sweep(10)
        _assert_same_state(g, o)
    assert (g.fetch_records() == o.records()).all()
    o.close()
    g.close()


def test_spin_s_batch_member_equals_alone(lg):
    ps = [_params(lg, MODELS["s1_xxz_field"], 41),
          lg.make_params(LATTICE="square", L=6, BETA=2.0, SEED=42, SWEEPS=1000, THERMALIZATION=0,
                         INITIAL_SPINS="random"),
          _params(lg, MODELS["s3half_heisenberg"], 43)]
    b = lg.Batch(ps)
    b.run(25)
    for i in (0, 2):
        alone = lg.LoopWorker(ps[i])
        alone.run(25)
        for x, y in zip(b.chain(i).state(), alone.state()):
            assert np.array_equal(x, y)
        alone.close()
    total_sites, _ = b.stats()
    assert total_sites == 6 + 36 + 6  # real sites
    b.close()


def test_spin_s_unsupported_inputs(lg):
    with pytest.raises(lg.LoopError) as e:  # 30 virtual neighbours per virtual site
        lg.LoopWorker(lg.make_params(LATTICE="cubic", L=2, BETA=1.0, local_S=2.5))
    assert e.value.code == -4
    with pytest.raises(lg.LoopError) as e:
        lg.LoopWorker(_params(lg, MODELS["s1_heisenberg"], 1, MEASURE_CORRELATIONS=True))
    assert e.value.code == -4


@pytest.mark.parametrize("case", [(1, 4, 0.5, 1.0, 1.0, 0.0, 2), (1, 4, 1.0, 1.0, 0.5, 0.2, 3),
                                  (2, 2, 0.5, 1.0, 1.0, 0.0, 2), (3, 2, 1.0, 1.0, 0.5, 0.2, 2)])
def test_spin_s_observables_vs_exact_diagonalization(lg, case):
    dim, L, T, jxy, jz, h, spin2 = case
    g = lg.LoopWorker(lg.make_params(LATTICE=dim, L=L, T=T, Jxy=jxy, Jz=jz, h=h,
                                     local_S=spin2 / 2, SEED=17, SWEEPS=1 << 16,
                                     THERMALIZATION=1 << 10, INITIAL_SPINS="random"))
    g.run((1 << 16) + (1 << 10))
    obs = g.observables()
    ref = orc.ed.thermal(dim, L, T, jxy=jxy, jz=jz, h=h, spin2=spin2)
    keys = ["Energy", "Specific Heat", "Susceptibility", "Magnetization^2",
            "Staggered Magnetization^2"]
    if h == 0:
        keys.append("Staggered Susceptibility")
    for k in keys:
        mean, err = obs[k]
        assert abs(mean - ref[k]) <= 3.5 * err + 1e-9, (k, mean, err, ref[k])
