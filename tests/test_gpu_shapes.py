"""Launch shapes and the autotuner change speed only, never a result.

A shape picks, per arena, the path (chain-resident: one CTA per chain, whole chunks of sweeps in
shared memory; or the grid path of grid-wide kernels) and, on the grid path, which chains run
insertion / merge / list compaction with a thread per bond or site ("narrow") instead of a warp
per site, and the CTA sizes of the union-find, cluster sum and cluster flip kernels.  Every shape must give the same trajectories and the same exact
per-sweep sums, so the arena below (chains of mixed lattices, temperatures, anisotropy and field,
all smaller than one k_cluster tile so that the per-chain reductions of tiles spanning chains are
exercised) is run under several shapes and compared bit for bit.
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
    dict(LATTICE="chain", L=32, BETA=3.0),
    dict(LATTICE="square", L=8, BETA=1.0),
    dict(LATTICE="square", L=12, BETA=8.0, h=0.2),
    dict(LATTICE="cubic", L=4, BETA=2.0, Jxy=1.0, Jz=0.5, h=0.3),
    dict(LATTICE="square", L=16, BETA=0.5),
    dict(LATTICE="chain", L=64, BETA=16.0, Jxy=1.0, Jz=1.5),
]

SHAPES = [
    dict(insert_k=0.0, narrow_k=0.0, resident=0),                 # every chain warp-per-site
    dict(insert_k=1e300, narrow_k=1e300, resident=0),             # every chain thread-per-site
    dict(insert_k=1e300, narrow_k=10.0, acc_tile=512, cl_tile=2048, union_warps=4, resident=0,
         union_mode=0),                                           # a lane per vertex
    dict(insert_k=10.0, narrow_k=32.0, acc_tile=2048, cl_tile=8192, union_warps=16, resident=0,
         union_mode=1),                                           # lower-leg pairs first
    dict(insert_k=0.0, narrow_k=1e300, acc_tile=1024, cl_tile=4096, resident=0,
         union_mode=2),                                           # pairs, then lane-balanced
    dict(resident=1),                                             # one CTA per chain
]


def _params(lg):
    return [lg.make_params(SEED=31 + i, INITIAL_SPINS="random", SWEEPS=4096, THERMALIZATION=0, **m)
            for i, m in enumerate(MODELS)]


def _snapshot(b):
    out = []
    for i in range(len(b)):
        spins, bonds, times = b.chain(i).state()
        out.append((spins, bonds, times, b.observables(i)))
    return out


def _assert_same(a, b):
    assert len(a) == len(b)
    for (s0, b0, t0, o0), (s1, b1, t1, o1) in zip(a, b):
        np.testing.assert_array_equal(s0, s1)
        np.testing.assert_array_equal(b0, b1)
        np.testing.assert_array_equal(t0.view(np.uint64), t1.view(np.uint64))
        for k, v in o0.items():
            v1 = o1[k]
            if isinstance(v, float) and np.isnan(v):
                assert np.isnan(v1), k
            else:
                assert v == v1, k


def test_every_shape_gives_the_same_trajectories(lg):
    ref = None
    for sh in SHAPES:
        b = lg.Batch(_params(lg))
        b.shape = sh
        got = b.shape
        for k, v in sh.items():
            assert got[k] == v
        b.run(40)
        snap = _snapshot(b)
        b.close()
        if ref is None:
            ref = snap
        else:
            _assert_same(ref, snap)


def test_bad_shape_is_rejected(lg):
    b = lg.Batch(_params(lg)[:2])
    with pytest.raises(lg.LoopError) as e:
        b.shape = dict(acc_tile=300)
    assert e.value.code == -1
    b.close()


def test_autotune_keeps_the_trajectory(lg):
    b1 = lg.Batch(_params(lg))
    shape, report = b1.autotune(trial_sweeps=2)
    assert "chosen:" in report
    assert shape["acc_tile"] in (512, 1024, 2048) and shape["cl_tile"] in (2048, 4096, 8192)
    assert shape["union_warps"] in (4, 8, 16)
    total_sites, site_sweeps = b1.stats()
    done = site_sweeps // total_sites
    assert done >= 2
    b1.run(10)
    b2 = lg.Batch(_params(lg))
    b2.run(done + 10)
    _assert_same(_snapshot(b1), _snapshot(b2))
    b1.close()
    b2.close()


def test_single_chain_autotune(lg):
    w = lg.LoopWorker(lg.make_params(LATTICE="square", L=16, BETA=4.0, SEED=5, SWEEPS=4096,
                                     THERMALIZATION=0))
    shape, report = w.autotune(trial_sweeps=1)
    assert report.count("ms") >= 2
    w.close()


def test_single_chain_shape_roundtrip(lg):
    w = lg.LoopWorker(lg.make_params(LATTICE="cubic", L=4, BETA=2.0, SEED=9, SWEEPS=4096,
                                     THERMALIZATION=0))
    w.shape = dict(insert_k=1e300, narrow_k=1e300, acc_tile=512, cl_tile=2048, union_warps=16,
                   resident=0)
    sh = w.shape
    assert sh["acc_tile"] == 512 and sh["cl_tile"] == 2048 and sh["union_warps"] == 16
    w.run(5)
    spins_a, bonds_a, times_a = w.state()
    w.close()
    v = lg.LoopWorker(lg.make_params(LATTICE="cubic", L=4, BETA=2.0, SEED=9, SWEEPS=4096,
                                     THERMALIZATION=0))
    v.run(5)
    spins_b, bonds_b, times_b = v.state()
    v.close()
    np.testing.assert_array_equal(spins_a, spins_b)
    np.testing.assert_array_equal(bonds_a, bonds_b)
    np.testing.assert_array_equal(times_a.view(np.uint64), times_b.view(np.uint64))


def test_paths_switch_mid_run_without_changing_the_trajectory(lg):
    """A batch moved between the chain-resident and the grid path every few sweeps (the state
    moves with it: spins, off-diagonal lists, sweep counters, accumulators) ends where the same
    batch run on one path ends."""
    ref = lg.Batch(_params(lg))
    ref.shape = dict(resident=0)
    ref.run(45)
    want = _snapshot(ref)
    ref.close()
    b = lg.Batch(_params(lg))
    for k, res in ((7, 1), (10, 0), (3, 1), (25, 0)):
        b.shape = dict(resident=res)
        assert b.shape["resident"] == res
        b.run(k)
    _assert_same(want, _snapshot(b))
    b.close()
