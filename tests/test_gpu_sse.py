"""The SSE form (ALGORITHM = "loop; sse", sse.C) on the GPU: one thread per chain (k_sse).

* whole trajectories (spins, the whole operator string, per-sweep integer records) equal the
  oracle's SSE restatement running the same Philox streams, for Heisenberg / XXZ / XY / Ising /
  ferromagnetic models on chain, square and cubic lattices, hot and cold          (bit exact)
* a chain inside a ragged batch equals the chain alone; a string that outgrows its capacity is
  replayed after the capacity grows without changing the trajectory; a checkpoint restores the
  trajectory exactly                                                                (bit exact)
* observables within 3.5 sigma of exact diagonalization and within 3 combined sigma of the
  reference's own "loop; sse" blocks of loop.op; exchange Monte Carlo over SSE chains vs ED
* the per-sweep values reproduce the accumulated means; unsupported inputs are refused
"""
import struct

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
    "chain16_heisenberg": dict(dim=1, L=16, beta=4.0, jxy=1.0, jz=1.0),
    "chain6_xxz": dict(dim=1, L=6, beta=3.0, jxy=1.0, jz=0.5),
    "chain6_xy": dict(dim=1, L=6, beta=2.0, jxy=1.0, jz=0.0),
    "chain6_ferro": dict(dim=1, L=6, beta=2.0, jxy=-1.0, jz=-0.5),
    "chain4_ising": dict(dim=1, L=4, beta=2.0, jxy=0.0, jz=1.0),
    "chain2_doubled": dict(dim=1, L=2, beta=3.0, jxy=1.0, jz=1.0),
    "chain16_hot": dict(dim=1, L=16, beta=0.02, jxy=1.0, jz=1.0),
    "square8": dict(dim=2, L=8, beta=2.0, jxy=1.0, jz=1.0),
    "square6_xxz_cold": dict(dim=2, L=6, beta=8.0, jxy=1.0, jz=0.7),
    "cubic4_xxz": dict(dim=3, L=4, beta=1.0, jxy=1.0, jz=0.5),
    # spin S on the virtual lattice, closed in imaginary time by the boundary matching
    "chain6_s1": dict(dim=1, L=6, beta=3.0, jxy=1.0, jz=1.0, spin2=2),
    "chain5_s3half_ferro": dict(dim=1, L=5, beta=1.5, jxy=-1.0, jz=-0.5, spin2=3),
    "square4_s1_xxz": dict(dim=2, L=4, beta=1.5, jxy=1.0, jz=0.5, spin2=2),
    "cubic2_s2": dict(dim=3, L=2, beta=0.7, jxy=1.0, jz=1.0, spin2=4),
}


def _params(lg, m, seed, **kw):
    base = dict(LATTICE=m["dim"], L=m["L"], BETA=m["beta"], Jxy=m["jxy"], Jz=m["jz"], SEED=seed,
                SWEEPS=1000, THERMALIZATION=0, INITIAL_SPINS="random", ALGORITHM="loop; sse",
                local_S=m.get("spin2", 1) / 2)
    base.update(kw)
    return lg.make_params(**base)


def sse_state(blob, nsites):
    """(sweeps done, spins, operator codes) of an SSE checkpoint (version 4)."""
    assert blob[:4] == b"LGCK"
    ver, _, _, mcs, n = struct.unpack_from("<IIIQQ", blob, 4)
    assert ver == 4
    spins = np.frombuffer(blob, dtype=np.uint8, count=nsites, offset=32).astype(np.int32)
    rows = np.frombuffer(blob, dtype=np.dtype([("op", "<i4"), ("t", "<f8")]), count=n,
                         offset=32 + nsites)
    return mcs, spins, rows["op"].astype(np.uint32)


def _assert_same_state(g, o, nsites):
    _, gs, gops = sse_state(g.save(), nsites)
    os_, oops = o.state()
    assert gs.tolist() == os_.tolist()
    assert gops.tolist() == oops.tolist()


@pytest.mark.parametrize("name", sorted(MODELS))
def test_sse_trajectory_bit_exact_vs_oracle(lg, name):
    m = MODELS[name]
    seed = 4321 + len(name)
    g = lg.LoopWorker(_params(lg, m, seed))
    g.keep_records(True)
    o = orc.SseOracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], seed=seed,
                      spin2=m.get("spin2", 1))
    n = m["L"] ** m["dim"] * m.get("spin2", 1)
    _assert_same_state(g, o, n)
    for k in (1, 9, 30, 64, 96):         # chunks of one launch and of several
        g.run(k)
        o.sweep(k)
        _assert_same_state(g, o, n)
    gr, orr = g.fetch_records(), o.records()
    assert gr.shape == orr.shape == (200, 32)
    assert (gr == orr).all()
    # the off-diagonal operators in state() are those of the string, in order
    spins, bonds, times = g.state()
    _, oops = o.state()
    assert bonds.tolist() == (oops[(oops & 1) == 1] >> 1).tolist()
    assert np.all(np.diff(times) > 0)
    o.close()
    g.close()


def test_sse_batch_member_equals_alone(lg):
    names = ["square8", "chain16_hot", "chain6_xxz", "cubic4_xxz", "chain2_doubled"]
    ps = [_params(lg, MODELS[k], 900 + i) for i, k in enumerate(names)]
    b = lg.Batch(ps)
    for i in range(len(ps)):
        b.chain(i).keep_values(True)
    for k in (3, 50, 11):
        b.run(k)
    for i, p in enumerate(ps):
        w = lg.LoopWorker(p)
        w.keep_values(True)
        w.run(64)
        got, ref = b.chain(i).fetch_values(), w.fetch_values()
        assert sorted(got) == sorted(ref)
        for k in ref:
            assert np.array_equal(got[k], ref[k]), (names[i], k)
        assert b.chain(i).save() == w.save()
        w.close()
    b.close()


def test_sse_capacity_growth_replays_exactly(lg):
    """A chain at beta = 0.5 is moved to beta = 16: its string grows about 30-fold, past the
    capacity sized for the old beta, so chunks overflow, the capacity grows and the chunk is
    replayed.  The trajectory equals the oracle's, which has no capacity."""
    m = dict(dim=2, L=8, beta=0.5, jxy=1.0, jz=1.0)
    g = lg.LoopWorker(_params(lg, m, 5150))
    o = orc.SseOracle(2, 8, 0.5, seed=5150)
    g.run(20)
    o.sweep(20)
    _assert_same_state(g, o, 64)
    g.set_beta(16.0)
    spins, ops = o.state()
    o2 = orc.SseOracle(2, 8, 16.0, seed=5150)
    o2.set_state(spins, ops, 20)
    g.keep_records(True)
    for k in (64, 64):
        g.run(k)
        o2.sweep(k)
        _assert_same_state(g, o2, 64)
    assert (g.fetch_records() == o2.records()).all()
    assert o2.records()[-1, 0] > 10 * o.records()[-1, 0]


def test_sse_checkpoint_round_trip(lg):
    m = MODELS["square6_xxz_cold"]
    a = lg.LoopWorker(_params(lg, m, 61))
    a.run(25)
    blob = a.save()
    mcs, spins, ops = sse_state(blob, 36)
    assert mcs == 25 and len(ops) > 0
    b = lg.LoopWorker(_params(lg, m, 61))
    b.load(blob)
    o = orc.SseOracle(2, 6, m["beta"], m["jxy"], m["jz"], seed=61)
    o.set_state(spins, ops, 25)
    for w in (a, b):
        w.keep_records(True)
        w.run(40)
    o.sweep(40)
    ra, rb = a.fetch_records(), b.fetch_records()
    assert (ra == rb).all() and (ra == o.records()).all()
    assert a.save() == b.save()
    # a string that is not periodic in imaginary time, or a path-integral checkpoint, is refused
    bad = bytearray(blob)
    j = 32 + 36
    code = struct.unpack_from("<i", bad, j)[0]
    struct.pack_into("<i", bad, j, code ^ 1)
    struct.pack_into("<Q", bad, len(bad) - 8, lg.checkpoint_checksum(bad))  # re-signed
    with pytest.raises(lg.LoopError) as e:
        b.load(bytes(bad))
    assert e.value.code == -1
    pi = lg.LoopWorker(lg.make_params(LATTICE=2, L=6, BETA=1.0, SEED=1))
    with pytest.raises(lg.LoopError) as e:
        pi.load(blob)
    assert e.value.code == -7
    for w in (a, b, pi):
        w.close()


ED_CASES = [(1, 8, 0.5, 1.0, 1.0, False, 1), (1, 6, 0.3, 1.0, 0.5, False, 1),
            (2, 2, 0.5, 1.0, 1.0, False, 1), (3, 2, 0.5, 1.0, 0.5, False, 1),
            (1, 6, 0.5, 1.0, 1.0, True, 1), (1, 4, 0.5, 1.0, 1.0, False, 2),
            (1, 4, 1.0, 1.0, 0.5, False, 3), (2, 2, 0.5, 1.0, 1.0, False, 2)]


@pytest.mark.parametrize("case", ED_CASES)
def test_sse_observables_vs_exact_diagonalization(lg, case):
    dim, L, T, jxy, jz, normal, spin2 = case
    kw = dict(DISABLE_IMPROVED_ESTIMATOR=True) if normal else {}
    g = lg.LoopWorker(lg.make_params(LATTICE=dim, L=L, T=T, Jxy=jxy, Jz=jz, SEED=17,
                                     SWEEPS=1 << 16, THERMALIZATION=1 << 10, local_S=spin2 / 2,
                                     INITIAL_SPINS="random", ALGORITHM="loop; sse", **kw))
    g.run((1 << 16) + (1 << 10))
    obs = g.observables()
    ref = orc.ed.thermal(dim, L, T, jxy=jxy, jz=jz, spin2=spin2)
    for k in ["Energy", "Specific Heat", "Susceptibility", "Magnetization^2",
              "Staggered Magnetization^2", "Staggered Susceptibility"]:
        mean, err = obs[k]
        assert abs(mean - ref[k]) <= 3.5 * err + 1e-9, (k, mean, err, ref[k])
    g.close()


def test_sse_agrees_with_reference_sse_blocks(lg, golden):
    """The "loop; sse" blocks of loop.op without single-ion anisotropy (L = 4 rings: S = 1/2
    Heisenberg and Ising, S = 1 Heisenberg; 4096 sweeps each): every printed value within 3
    combined standard errors, the number of clusters included."""
    n = 0
    for blk in golden("loop_op.json"):
        if blk["algorithm"] != "loop; sse":
            continue
        w = lg.LoopWorker(lg.make_params(LATTICE="chain", L=blk["L"], T=blk["T"], Jxy=blk["jxy"],
                                         Jz=blk["jz"], SEED=2718 + n, SWEEPS=1 << 16,
                                         THERMALIZATION=1 << 10, INITIAL_SPINS="random",
                                         local_S=blk.get("spin2", 1) / 2, ALGORITHM="loop; sse"))
        w.run((1 << 16) + (1 << 10))
        obs = w.observables()
        for k, (v, e) in blk["values"].items():
            mean, err = obs[k]
            tol = 3.0 * (float(e) ** 2 + err ** 2) ** 0.5
            assert abs(mean - v) <= tol + 1e-9, (blk["T"], k, mean, err, v, e)
            n += 1
        w.close()
    assert n == 21


def test_sse_exchange_vs_exact_diagonalization(lg):
    betas = [0.5, 1.0, 2.0, 4.0]
    x = lg.Exchange(lg.make_params(LATTICE="chain", L=6, SEED=99, SWEEPS=1 << 15,
                                   THERMALIZATION=1 << 9, INITIAL_SPINS="random",
                                   ALGORITHM="loop; sse; exchange"), betas)
    x.run((1 << 15) + (1 << 9))
    _, att, acc = x.state()
    assert (acc > 0).all()
    for t, b in enumerate(betas):
        obs = x.observables(t)
        ref = orc.ed.thermal(1, 6, 1.0 / b)
        for k in ("Energy", "Susceptibility", "Staggered Magnetization^2"):
            mean, err = obs[k]
            assert abs(mean - ref[k]) <= 3.5 * err + 1e-9, (b, k, mean, err, ref[k])
    x.close()


def test_sse_values_reproduce_observables(lg):
    p = lg.make_params(LATTICE="square", L=6, BETA=2.0, SEED=8, SWEEPS=300, THERMALIZATION=20,
                       INITIAL_SPINS="random", ALGORITHM="loop; sse")
    w = lg.LoopWorker(p)
    w.keep_values(True)
    rows = {}
    for k in (64, 64, 64, 64, 64):
        w.run(k)
        for name, col in w.fetch_values().items():
            rows.setdefault(name, []).append(col)
    rows = {k: np.concatenate(v) for k, v in rows.items()}
    obs = w.observables()
    for k in ("Energy", "Susceptibility", "Staggered Susceptibility", "Number of Clusters",
              "Generalized Susceptibility", "Stiffness"):
        assert len(rows[k]) == 300
        s = 0.0
        for x in rows[k]:
            s += float(x)
        assert s / 300 == pytest.approx(obs[k][0], rel=1e-12), k
    w.close()


def test_sse_unsupported_inputs(lg):
    m = MODELS["chain6_xxz"]
    for kw in (dict(h=0.1), dict(MEASURE_CORRELATIONS=True), dict(local_S=4.5)):
        with pytest.raises(lg.LoopError) as e:
            lg.LoopWorker(_params(lg, m, 1, **kw))
        assert e.value.code == -4, kw
    with pytest.raises(lg.LoopError) as e:
        lg.Batch([_params(lg, m, 1), _params(lg, m, 2, ALGORITHM="loop; path integral")])
    assert e.value.code == -1
    w = lg.LoopWorker(_params(lg, m, 3))
    with pytest.raises(lg.LoopError) as e:
        w.validate_sweeps(2)
    assert e.value.code == -4
    with pytest.raises(lg.LoopError) as e:
        w.set_state(np.zeros(6, dtype=np.int32), np.zeros(0, dtype=np.int32),
                    np.zeros(0), 0)
    assert e.value.code == -4
    w.close()
    s = lg.Server(budget_bytes=1 << 28, sweeps_per_tick=4)
    with pytest.raises(lg.LoopError) as e:
        s.submit(_params(lg, m, 4))
    assert e.value.code == -4
    s.close()
