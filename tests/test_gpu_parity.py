"""GPU parity: the CUDA sweep against the CPU oracle and the reference's golden data.

* cluster labels of dumped configurations == the reference union_find.h (deterministic unify),
  partitions == the default weighted unify, up to 1.2e6 vertices            (bit exact)
* whole trajectories (spins, operator strings, per-sweep integer records) == the oracle
  running the same random streams, for Heisenberg / XXZ / Ising / ferromagnet / field models
  on chain, square and cubic lattices                                      (bit exact)
* a chain gives the same trajectory alone and inside a ragged batch          (bit exact)
* buffer growth after a capacity overflow does not change the trajectory     (bit exact)
* full-size invariants (128x128, beta=64): conservation of the time-integrated magnetisation,
  determinism, one-sweep agreement with the oracle from the GPU's own state
* observables within 3 sigma of exact diagonalization
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


def _canon(labels):
    m = {}
    return [m.setdefault(int(x), len(m)) for x in labels]


@pytest.mark.parametrize("idx", range(7))
def test_uf_labels_bit_exact_vs_reference_union_find(lg, golden, idx):
    c = golden("uf_labels.json")[idx]
    lab, nc = lg.uf_label(c["dim"], c["L"], c["bonds"], c["graphs"])
    assert nc == c["nc"]
    assert lab.tolist() == c["labels_deterministic"]
    assert _canon(lab) == _canon(c["labels_weighted"])


@pytest.mark.parametrize("name", ["square32_b16", "square128_b64"])
def test_uf_labels_at_scale_bit_exact_vs_reference_union_find(lg, golden, name):
    """Configurations of 2e4 and 1.2e6 vertices (the latter the bench workload's size, where the
    lock-free unions really race), made again by the oracle from their seeds: the GPU labels equal
    those of the reference's own looper/union_find.h (deterministic unify), compiled in place in
    the build container (tests/golden/make_uf_scale.py)."""
    import hashlib
    import os
    meta = golden("uf_scale.json")[name]
    o = orc.Oracle(meta["dim"], meta["L"], meta["beta"], 1.0, 1.0, 0.0, seed=meta["seed"])
    o.sweep(meta["sweeps"])
    cfg = o.last_config()
    o.close()
    bonds = np.asarray(cfg["bonds"], dtype=np.int32)
    graphs = np.asarray(cfg["graphs"], dtype=np.int32)
    sha = hashlib.sha256(bonds.astype("<i4").tobytes() + graphs.astype("<i4").tobytes()).hexdigest()
    assert sha == meta["config_sha256"]          # the same configuration as in the build container
    lab, nc = lg.uf_label(meta["dim"], meta["L"], bonds, graphs)
    assert nc == meta["nc"] and len(lab) == meta["nfrag"]
    assert hashlib.sha256(np.asarray(lab, dtype="<i4").tobytes()).hexdigest() == meta["labels_sha256"]
    if name == "square32_b16":
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "uf_scale_32.npz"))
        assert np.array_equal(z["labels"], lab)


def test_uf_labels_random_configs_vs_oracle(lg):
    for seed, (dim, L, beta, jxy, jz) in enumerate([(1, 32, 8.0, 1.0, 1.0), (2, 10, 3.0, 1.0, 0.5),
                                                     (3, 4, 2.0, 1.0, 1.5), (2, 8, 2.0, -1.0, -0.5)]):
        o = orc.Oracle(dim, L, beta, jxy, jz, 0.0, seed=100 + seed)
        o.sweep(7)
        cfg = o.last_config()
        lab, nc = lg.uf_label(dim, L, cfg["bonds"], cfg["graphs"])
        ref, rnc = orc.uf_label(dim, L, cfg["bonds"], cfg["graphs"], deterministic=True)
        assert nc == rnc
        assert lab.tolist() == ref.tolist()
        o.close()


MODELS = {
    "chain16_heisenberg": dict(dim=1, L=16, beta=10.0, jxy=1.0, jz=1.0, h=0.0),
    "chain64_heisenberg_b10": dict(dim=1, L=64, beta=10.0, jxy=1.0, jz=1.0, h=0.0),
    "square8_heisenberg": dict(dim=2, L=8, beta=4.0, jxy=1.0, jz=1.0, h=0.0),
    "square6_xxz_easy_plane": dict(dim=2, L=6, beta=3.0, jxy=1.0, jz=0.5, h=0.0),
    "cubic4_xxz_field": dict(dim=3, L=4, beta=2.0, jxy=1.0, jz=0.5, h=0.3),
    "cubic4_ising_like_field": dict(dim=3, L=4, beta=1.5, jxy=1.0, jz=1.5, h=0.2),
    "chain12_ferro": dict(dim=1, L=12, beta=5.0, jxy=-1.0, jz=-1.0, h=0.0),
    "chain10_ising": dict(dim=1, L=10, beta=2.0, jxy=0.0, jz=1.0, h=0.0),
    "chain9_ferro_odd": dict(dim=1, L=9, beta=2.0, jxy=-1.0, jz=0.3, h=0.1),
    # edge cases: the smallest periodic lattices (both bonds of a pair join the same two sites),
    # a model with no operators at all (only the field acts on single-site clusters), and a
    # temperature so high that most sweeps have none
    "chain2_heisenberg": dict(dim=1, L=2, beta=3.0, jxy=1.0, jz=1.0, h=0.0),
    "square2_xxz": dict(dim=2, L=2, beta=2.0, jxy=1.0, jz=0.5, h=0.0),
    "cubic2_field": dict(dim=3, L=2, beta=1.0, jxy=1.0, jz=1.0, h=0.1),
    "chain8_free_spins_field": dict(dim=1, L=8, beta=2.0, jxy=0.0, jz=0.0, h=0.5),
    "chain16_hot": dict(dim=1, L=16, beta=0.01, jxy=1.0, jz=1.0, h=0.0),
}


def _gpu_chain(lg, m, seed, sweeps=1000, therm=0, random_spins=True):
    return lg.LoopWorker(lg.make_params(LATTICE=m["dim"], L=m["L"], BETA=m["beta"], Jxy=m["jxy"],
                                        Jz=m["jz"], h=m["h"], SEED=seed, SWEEPS=sweeps,
                                        THERMALIZATION=therm,
                                        INITIAL_SPINS="random" if random_spins else "up"))


def _assert_same_state(g, o):
    gs, gb, gt = g.state()
    os_, ob, ot = o.state()
    assert gs.tolist() == os_.tolist()
    assert gb.tolist() == ob.tolist()
    assert gt.view(np.uint64).tolist() == ot.view(np.uint64).tolist()


@pytest.mark.parametrize("path", ["grid", "resident"])
@pytest.mark.parametrize("name", sorted(MODELS))
def test_trajectory_bit_exact_vs_oracle(lg, name, path):
    """Both sweep paths: the grid path (one CUDA graph of grid-wide kernels per sweep) and the
    chain-resident path (one CTA per chain, whole chunks of sweeps in shared memory)."""
    m = MODELS[name]
    seed = 1234 + len(name)
    g = _gpu_chain(lg, m, seed)
    g.shape = dict(resident=1 if path == "resident" else 0)
    assert g.shape["resident"] == (path == "resident")
    g.keep_records(True)
    o = orc.Oracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=seed)
    for _ in range(4):
        g.run(10)
        o.sweep(10)
        _assert_same_state(g, o)
    gr = g.fetch_records()
    orr = o.records()
    assert gr.shape == orr.shape == (40, 32)
    assert (gr == orr).all()
    o.close()
    g.close()


def test_resident_equals_grid_over_a_long_run(lg):
    """The two sweep paths agree bit for bit over thousands of sweeps (chunks of 64 sweeps per
    resident launch), on the CPU-runnable chain workload's model."""
    def mk(res):
        w = lg.LoopWorker(lg.make_params(LATTICE="chain", L=16, T=0.1, J=1.0, SEED=1234,
                                         SWEEPS=1 << 14, THERMALIZATION=1 << 12,
                                         INITIAL_SPINS="random"))
        w.shape = dict(resident=res)
        w.keep_records(True)
        return w
    a, b = mk(1), mk(0)
    for _ in range(5):
        a.run(1000)
        b.run(1000)
        assert (a.fetch_records() == b.fetch_records()).all()
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_all_up_start_matches_oracle(lg):
    m = MODELS["square8_heisenberg"]
    g = _gpu_chain(lg, m, 5, random_spins=False)
    o = orc.Oracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=5,
                   random_spins=False)
    g.run(25)
    o.sweep(25)
    _assert_same_state(g, o)


@pytest.mark.parametrize("path", ["grid", "resident"])
def test_batch_member_equals_alone(lg, path):
    names = ["square8_heisenberg", "chain16_heisenberg", "cubic4_xxz_field", "chain10_ising"]
    params = []
    for i, n in enumerate(names):
        m = MODELS[n]
        params.append(lg.make_params(LATTICE=m["dim"], L=m["L"], BETA=m["beta"], Jxy=m["jxy"],
                                     Jz=m["jz"], h=m["h"], SEED=77 + i, SWEEPS=1000,
                                     THERMALIZATION=0, INITIAL_SPINS="random"))
    b = lg.Batch(params)
    b.shape = dict(resident=1 if path == "resident" else 0)
    b.chain(0).keep_records(True)
    b.run(30)
    for i, p in enumerate(params):
        alone = lg.LoopWorker(p)
        if i == 0:
            alone.keep_records(True)
        alone.run(30)
        bs = b.chain(i).state()
        al = alone.state()
        for x, y in zip(bs, al):
            assert np.array_equal(x, y)
        if i == 0:
            assert (b.chain(0).fetch_records() == alone.fetch_records()).all()
        alone.close()
    b.close()


def test_capacity_growth_keeps_trajectory(lg):
    # Start hot (few operators, small buffers), then cool down: the buffers must grow.
    m = dict(dim=2, L=12, beta=0.5, jxy=1.0, jz=1.0, h=0.0)
    g = _gpu_chain(lg, m, 9)
    o = orc.Oracle(2, 12, 0.5, 1.0, 1.0, 0.0, seed=9)
    g.run(5)
    o.sweep(5)
    _assert_same_state(g, o)
    spins, bonds, times = o.state()
    g.set_beta(16.0)
    o2 = orc.Oracle(2, 12, 16.0, 1.0, 1.0, 0.0, seed=9)
    o2.set_state(spins, bonds, times, 5)
    g.run(12)
    o2.sweep(12)
    _assert_same_state(g, o2)


def test_set_state_then_sweep_matches_oracle(lg):
    m = MODELS["cubic4_xxz_field"]
    o = orc.Oracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=31)
    o.sweep(15)
    spins, bonds, times = o.state()
    g = _gpu_chain(lg, m, 31)
    g.set_state(spins, bonds, times, 15)
    g.run(6)
    o.sweep(6)
    _assert_same_state(g, o)


def test_set_state_rejects_a_non_periodic_configuration(lg):
    m = MODELS["cubic4_xxz_field"]
    o = orc.Oracle(m["dim"], m["L"], m["beta"], m["jxy"], m["jz"], m["h"], seed=32)
    o.sweep(15)
    spins, bonds, times = o.state()
    assert len(bonds) > 0
    g = _gpu_chain(lg, m, 32)
    g.set_state(spins, bonds, times, 15)
    # one operator fewer: its two sites flip an odd number of times
    with pytest.raises(lg.LoopError) as e:
        g.set_state(spins, bonds[1:], times[1:], 15)
    assert e.value.code == -1 and "periodic" in str(e.value)
    g.run(6)  # the chain kept the valid state
    o.sweep(6)
    _assert_same_state(g, o)


def test_checkpoint_roundtrip_and_corruption(lg):
    m = MODELS["square6_xxz_easy_plane"]
    g = _gpu_chain(lg, m, 3)
    g.run(20)
    blob = g.save()
    g2 = _gpu_chain(lg, m, 3)
    g2.load(blob)
    g.run(10)
    g2.run(10)
    for x, y in zip(g.state(), g2.state()):
        assert np.array_equal(x, y)
    bad = bytearray(blob)
    bad[40] ^= 0x5A
    with pytest.raises(lg.LoopError) as e:
        g2.load(bytes(bad))
    assert e.value.code == -7
    with pytest.raises(lg.LoopError):
        g2.load(blob[:20])


def test_full_size_invariants_and_one_sweep_parity(lg):
    # the bench workload: 128x128 square Heisenberg AF, beta = 64, seed 7.
    p = lg.make_params(LATTICE="square", L=128, BETA=64.0, J=1.0, SEED=7, SWEEPS=8192,
                       THERMALIZATION=1024, INITIAL_SPINS="random")
    g = lg.LoopWorker(p)
    g.keep_records(True)
    g.run(40)
    r = g.fetch_records()
    assert r.shape == (40, 32)
    # total Sz is conserved along imaginary time: integral of M == M(0) exactly
    m0 = r[:, 2].view(np.int64)
    ma = r[:, 25].view(np.int64)
    assert (ma == m0 * (1 << 40)).all()
    nop = r[:, 0].astype(np.float64)
    N = 128 * 128
    e = (2 * N * 0.25 - nop / 64.0) / N
    assert -0.75 < e[-1] < -0.55
    assert (r[:, 1] > 0).all()
    # determinism: a second chain with the same seed reproduces the state
    g2 = lg.LoopWorker(p)
    g2.run(40)
    for x, y in zip(g.state(), g2.state()):
        assert np.array_equal(x, y)
    # one more sweep from the GPU's own state, on both sides
    spins, bonds, times = g.state()
    o = orc.Oracle(2, 128, 64.0, 1.0, 1.0, 0.0, seed=7)
    o.set_state(spins, bonds, times, 40)
    g.run(1)
    o.sweep(1)
    _assert_same_state(g, o)
    assert (g.fetch_records() == o.records()).all()


@pytest.mark.parametrize("case", [
    (1, 4, 0.25, 1.0, 1.0, 0.0), (1, 4, 0.5, 0.0, 1.0, 0.0), (1, 6, 0.5, 1.0, 0.5, 0.3),
    (2, 2, 0.5, 1.0, 1.0, 0.0)])
def test_observables_vs_exact_diagonalization(lg, case):
    dim, L, T, jxy, jz, h = case
    g = lg.LoopWorker(lg.make_params(LATTICE=dim, L=L, T=T, Jxy=jxy, Jz=jz, h=h, SEED=11,
                                     SWEEPS=1 << 16, THERMALIZATION=1 << 10,
                                     INITIAL_SPINS="random"))
    g.run((1 << 16) + (1 << 10))
    obs = g.observables()
    ref = orc.ed.thermal(dim, L, T, jxy=jxy, jz=jz, h=h)
    for k in ("Energy", "Specific Heat", "Susceptibility", "Staggered Susceptibility",
              "Magnetization^2", "Staggered Magnetization^2"):
        mean, err = obs[k]
        assert abs(mean - ref[k]) <= 3.5 * err + 1e-9, (k, mean, err, ref[k])


def test_chain16_vs_exact_diagonalization(lg, golden):
    # the CPU-runnable chain workload (Heisenberg AF chain, J=1, T=0.1, 2^12 + 2^14 sweeps,
    # seed 1234, random spins) at L=16, where its correctness point is exact diagonalization
    g = golden("ed_chain16.json")
    w = lg.LoopWorker(lg.make_params(LATTICE="chain", L=16, T=0.1, J=1.0, SEED=1234,
                                     SWEEPS=1 << 14, THERMALIZATION=1 << 12,
                                     INITIAL_SPINS="random"))
    w.run((1 << 14) + (1 << 12))
    obs = w.observables()
    for k in ("Energy", "Energy Density", "Susceptibility", "Staggered Magnetization^2",
              "Specific Heat"):
        mean, err = obs[k]
        assert abs(mean - g["values"][k]) <= 3.5 * err, (k, mean, err, g["values"][k])
    w.close()


def test_observables_vs_reference_path_integral_runs(lg, golden):
    # every "loop; path integral" block of the reference's loop.op (S=1/2 and S=1 chains, L=4):
    # the GPU's values within 3 combined standard errors of the reference's own binned results,
    # including the mean number of clusters, which depends on the cluster algorithm itself.
    # One printed value is itself an outlier: the Ising ring's cluster count (2.09204 +/- 0.0142)
    # lies 3.7 sigma from the exact 2.1449, so that entry is checked against the exact value.
    n = 0
    for blk in golden("loop_op.json"):
        if blk["algorithm"] != "loop; path integral":
            continue
        spin2 = blk.get("spin2", 1)
        w = lg.LoopWorker(lg.make_params(LATTICE="chain", L=blk["L"], T=blk["T"], Jxy=blk["jxy"],
                                         Jz=blk["jz"], local_S=spin2 / 2, SEED=2718 + n,
                                         SWEEPS=1 << 16, THERMALIZATION=1 << 10,
                                         INITIAL_SPINS="random"))
        w.run((1 << 16) + (1 << 10))
        obs = w.observables()
        for k, (v, e) in blk["values"].items():
            mean, err = obs[k]
            if k == "Number of Clusters" and blk["jxy"] == 0.0 and spin2 == 1:
                exact = orc.ising_ring_clusters(blk["L"], blk["T"], blk["jz"])
                assert abs(v - exact) > 3 * float(e)            # the reference's outlier
                assert abs(mean - exact) <= 3.0 * err, (k, mean, err, exact)
            else:
                tol = 3.0 * (float(e) ** 2 + err ** 2) ** 0.5
                assert abs(mean - v) <= tol + 1e-9, (blk["T"], spin2, k, mean, err, v, e)
            n += 1
        w.close()
    assert n >= 30
