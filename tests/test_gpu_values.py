"""Per-sweep measurement values through the C ABI (lg_keep_values / lg_fetch_values).

These are what loop_worker::run pushes into its ObservableSet after every sweep
(path_integral.C:832-861), so a parapack plug-in over the engine reports measurements as the
reference worker does.  The tests drive the ABI the way the plug-in in INTEGRATION.md does: sweeps
in chunks, one row replayed per sweep, and check that plain accumulators over the fetched rows
reproduce the means lg_observables reports.
"""
import numpy as np
import pytest

import looper_gb300 as lg

pytestmark = pytest.mark.gpu

SAME = ["Energy", "Energy Density", "Energy^2", "Magnetization", "|Magnetization|",
        "Magnetization^2", "Magnetization^4", "Susceptibility", "Staggered Magnetization^2",
        "Staggered Magnetization^4", "Staggered Susceptibility", "Number of Clusters",
        "Stiffness", "Generalized Magnetization^2", "Generalized Susceptibility"]

MODELS = {
    "square_heisenberg": dict(LATTICE="square", L=8, BETA=2.0, J=1.0),
    "cubic_xxz_field": dict(LATTICE="cubic", L=4, BETA=1.5, Jxy=1.0, Jz=0.5, h=0.3),
    "chain_normal": dict(LATTICE="chain", L=16, BETA=4.0, J=1.0, DISABLE_IMPROVED_ESTIMATOR=True),
}


def _plugin_rows(w, total, chunk=64):
    """The plug-in's run(): sweeps in chunks, then one fetched row per measurement sweep."""
    rows = {}
    done = 0
    while done < total:
        k = min(chunk, total - done)
        w.run(k)
        done += k
        for name, col in w.fetch_values().items():
            rows.setdefault(name, []).append(col)
    return {k: np.concatenate(v) for k, v in rows.items()}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_fetched_values_reproduce_observables(name):
    therm, sweeps = 37, 300
    p = lg.make_params(SEED=11, SWEEPS=sweeps, THERMALIZATION=therm, INITIAL_SPINS="random",
                       **MODELS[name])
    w = lg.LoopWorker(p)
    w.keep_values(True)
    rows = _plugin_rows(w, therm + sweeps)
    obs = w.observables()
    assert sorted(rows) == sorted(w.value_names())
    for k, col in rows.items():
        assert len(col) == sweeps, k            # thermalization sweeps push nothing
        assert np.all(np.isfinite(col)), k
    improved = "Generalized Magnetization^2" in rows
    assert improved == (name == "square_heisenberg")
    for k in SAME:
        if k not in rows:
            continue
        s = 0.0
        for x in rows[k]:                        # plain accumulator, sweep order
            s += float(x)
        assert s / len(rows[k]) == pytest.approx(obs[k][0], rel=1e-12, abs=1e-300), k
    assert np.all(rows["Inverse Temperature"] == p.beta)
    assert np.all(rows["Volume"] == p.L ** p.lattice)
    w.close()


def test_values_identical_in_chunks_and_in_batches():
    """The rows do not depend on how the sweeps are chunked, nor on batching."""
    ps = [lg.make_params(LATTICE="square", L=L, BETA=b, SEED=5 + i, SWEEPS=150,
                         THERMALIZATION=10, INITIAL_SPINS="random")
          for i, (L, b) in enumerate([(6, 3.0), (10, 1.0)])]
    alone = []
    for p in ps:
        w = lg.LoopWorker(p)
        w.keep_values(True)
        w.run(160)
        alone.append(w.fetch_values())
        w.close()
    b = lg.Batch(ps)
    for i in range(len(ps)):
        b.chain(i).keep_values(True)
    got = [dict() for _ in ps]
    for k in (1, 7, 64, 88):
        b.run(k)
        for i in range(len(ps)):
            for name, col in b.chain(i).fetch_values().items():
                got[i].setdefault(name, []).append(col)
    for i in range(len(ps)):
        for name, col in alone[i].items():
            assert np.array_equal(np.concatenate(got[i][name]), col), (i, name)
    b.close()
