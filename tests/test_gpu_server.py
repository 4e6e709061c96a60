"""Continuous-batching server: every served result equals the same request run alone, with one
arena or with requests spread over size-class lanes that run side by side."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


REQS = [
    dict(LATTICE="chain", L=48, BETA=4.0, Jxy=1.0, Jz=0.8, h=0.2, SWEEPS=160, THERMALIZATION=20),
    dict(LATTICE="square", L=10, BETA=2.0, Jxy=1.0, Jz=1.2, h=0.0, SWEEPS=96, THERMALIZATION=12),
    dict(LATTICE="cubic", L=4, BETA=1.5, Jxy=1.0, Jz=1.0, h=0.3, SWEEPS=64, THERMALIZATION=8),
    dict(LATTICE="square", L=16, BETA=8.0, Jxy=1.0, Jz=1.0, h=0.0, SWEEPS=128, THERMALIZATION=16),
    dict(LATTICE="chain", L=200, BETA=1.0, Jxy=1.0, Jz=0.5, h=0.4, SWEEPS=48, THERMALIZATION=6),
    dict(LATTICE="cubic", L=6, BETA=0.7, Jxy=1.0, Jz=1.5, h=0.1, SWEEPS=80, THERMALIZATION=10),
    # about 3x10^4 operators per sweep: a different size class from the others
    dict(LATTICE="square", L=32, BETA=16.0, Jxy=1.0, Jz=1.0, h=0.0, SWEEPS=40, THERMALIZATION=8),
]


@pytest.mark.parametrize("lanes", [1, 3])
def test_served_results_equal_alone(lg, lanes):
    params = [lg.make_params(SEED=500 + i, INITIAL_SPINS="random", **r) for i, r in enumerate(REQS)]
    srv = lg.Server(sweeps_per_tick=8, rebuild_interval_s=0.0, lanes=lanes)
    import time
    ids = [srv.submit(params[0])]
    t_end = time.time() + 60
    while srv.stats()["rebuilds"] < 1 and time.time() < t_end:  # the first arena exists
        time.sleep(0.005)
    for p in params[1:]:      # staggered arrivals: admitted into a running arena
        ids.append(srv.submit(p))
        time.sleep(0.01)
    srv.wait(300)
    res = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(params) and st["rejected"] == 0
    assert st["rebuilds"] >= 2
    for i, p in zip(ids, params):
        r = res[i]
        assert r["status"] == 0 and r["t_finish"] >= r["t_start"] >= r["t_submit"]
        alone = lg.LoopWorker(p)
        alone.run(p.sweeps + p.thermalization)
        a = alone.observables()
        alone.close()
        assert r["obs"]["count"] == a["count"] == p.sweeps
        for k, v in a.items():
            if isinstance(v, tuple):
                assert np.array_equal(np.array(r["obs"][k]), np.array(v), equal_nan=True), k


def test_server_rejects_requests_beyond_budget(lg):
    srv = lg.Server(budget_bytes=5e6)
    small = srv.submit(lg.make_params(LATTICE="chain", L=16, T=1.0, SWEEPS=32, THERMALIZATION=4))
    huge = srv.submit(lg.make_params(LATTICE="square", L=128, BETA=64.0, SWEEPS=32))
    srv.wait(120)
    res = {r["id"]: r for r in srv.poll()}
    srv.close()
    assert res[small]["status"] == 0
    assert res[huge]["status"] == -6
