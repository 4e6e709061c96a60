"""Pins the CPU oracle against the reference's own golden outputs (no GPU needed).

* standalone mode == standalone/loop.op, digit for digit
* union-find replay == test/union_find.op (parents, roots, tree sizes)
* cluster labels == the reference union_find.h (both unify variants) on dumped configurations
* ED restatement == loop.op's diagonalization blocks
* philox mode: statistics within 3.5 sigma of exact diagonalization (chain, square and cubic
  lattices; S = 1/2, 1, 3/2; antiferromagnetic, ferromagnetic, Ising, XY, field)
"""
import math

import numpy as np
import pytest

import oracle_lib as orc


def _fmt(x):
    return "%g" % x


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10.
    assert [hex(x) for x in orc.philox_raw([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in orc.philox_raw([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in orc.philox_raw([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                                           [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_float_log_exp_accuracy():
    L = orc.lib()
    for u in np.linspace(1e-7, 1 - 1e-7, 2001).astype(np.float32):
        ref = math.log(float(u))
        assert abs(L.orc_log_spec(float(u)) - ref) <= 3e-7 * max(1.0, abs(ref))
    for x in np.linspace(-80, 80, 1601).astype(np.float32):
        ref = math.exp(float(x))
        assert abs(L.orc_exp_spec(float(x)) - ref) <= 4e-7 * ref


def test_exponential_gap_tail():
    """The exponential gaps (path_integral.C:71,412-420 draws them as double exponentials) come
    from -ln U with U a float uniform.  The lowest of its 2^23 bins (U < 2^-23) is refined by 23
    more random bits, so the largest gap is 32.6 mean gaps instead of -ln 2^-24 = 16.6: a draw
    reaches the end of the table with probability 2^-47.  The refinement keeps the bin's mean,
    and -ln U stays accurate down there."""
    import math
    L = orc.lib()
    u_last = L.orc_gap_uniform(0, 0)                       # x = 0, t = 0: U = 2^-47
    assert u_last == 2.0 ** -47
    g_max = -L.orc_log_spec(u_last)
    assert abs(g_max - 47 * math.log(2)) <= 1e-5 * g_max and g_max > 32.5
    # outside the lowest bin nothing changes: U = (2x+1) 2^-24
    for w in (1 << 9, 12345 << 9, 0xFFFFFFFF, 0x80000000):
        assert L.orc_gap_uniform(w, 0xDEADBEEF) == ((w >> 9) * 2 + 1) * 2.0 ** -24
    # inside it, U = (2t+1) 2^-47 for the top 23 bits t of the tail word: exact, and the bin's
    # mean over t is its old centre 2^-24
    ts = list(range(0, 1 << 23, 4099)) + [(1 << 23) - 1]
    for t in ts:
        u = L.orc_gap_uniform(0x1FF, t << 9)
        assert u == (2 * t + 1) * 2.0 ** -47
        assert abs(-L.orc_log_spec(u) + math.log(u)) <= 3e-7 * -math.log(u)
    n = 1 << 23                                            # sum_t (2t+1) = n^2
    assert n * n * 2.0 ** -47 / n == 2.0 ** -24


def test_standalone_matches_golden(golden):
    g = golden("standalone_loop_op.json")
    out, _ = orc.standalone(g["L"], g["T"], g["sweeps"], g["therm"])
    names = ["Number of Clusters        = ", "Energy Density            = ",
             "Uniform Susceptibility    = ", "Staggered Magnetization^2 = ",
             "Staggered Susceptibility  = "]
    lines = [n + _fmt(out[2 * i]) + " +- " + _fmt(out[2 * i + 1]) for i, n in enumerate(names)]
    assert lines == g["lines"][4:9]


def test_union_find_replay_matches_golden(golden):
    g = golden("union_find_op.json")
    n = g["n"]
    parent, root, weight = orc.uf_replay(n, g["pairs"])
    listing = []
    for i in range(n):
        if parent[i] < 0:
            listing.append("node %d is root and tree size is %d" % (i, weight[i]))
        else:
            listing.append("node %d's parent is %d and its root is %d" % (i, parent[i], root[i]))
    for i in range(n):
        if parent[i] < 0:
            listing.append("node %d is root" % i)
        else:
            listing.append("node %d's parent is %d and its root is %d" % (i, parent[i], root[i]))
    assert listing == g["listing"]


def _canon(labels):
    """Canonical partition: relabel clusters by first appearance."""
    m = {}
    return [m.setdefault(x, len(m)) for x in labels]


@pytest.mark.parametrize("idx", range(7))
def test_uf_labels_match_reference_union_find(golden, idx):
    c = golden("uf_labels.json")[idx]
    lab_d, nc_d = orc.uf_label(c["dim"], c["L"], c["bonds"], c["graphs"], deterministic=True)
    lab_w, nc_w = orc.uf_label(c["dim"], c["L"], c["bonds"], c["graphs"], deterministic=False)
    assert nc_d == c["nc"] and nc_w == c["nc"]
    assert lab_d.tolist() == c["labels_deterministic"]
    assert lab_w.tolist() == c["labels_weighted"]
    assert _canon(c["labels_deterministic"]) == _canon(c["labels_weighted"])


def test_ed_matches_golden(golden):
    for b in golden("loop_op.json"):
        if b["algorithm"] != "diagonalization":
            continue
        r = orc.ed.thermal(1, b["L"], b["T"], jxy=b["jxy"], jz=b["jz"], spin2=b.get("spin2", 1))
        for k, (v, _) in b["values"].items():
            assert r[k] == pytest.approx(v, rel=2e-5, abs=2e-6), k


def test_ed_agrees_with_reference_path_integral(golden):
    # every "loop; path integral" block of loop.op (S=1/2 and S=1 chains) within 3 sigma of ED
    n = 0
    for b in golden("loop_op.json"):
        if b["algorithm"] != "loop; path integral":
            continue
        r = orc.ed.thermal(1, b["L"], b["T"], jxy=b["jxy"], jz=b["jz"], spin2=b.get("spin2", 1))
        for k, (v, e) in b["values"].items():
            if k in r and k != "Specific Heat":
                assert abs(v - r[k]) <= 3 * float(e) + 1e-9, (b["T"], b.get("spin2", 1), k, v, e, r[k])
                n += 1
    assert n >= 20


def test_ed_correlations_agree_with_reference_path_integral(golden):
    # loop.op: "loop; path integral" with MEASURE[Correlations] / MEASURE[Structure Factor],
    # S=1/2 Heisenberg chain L=4, T=0.5, 4096 sweeps: the exact correlations must lie within
    # 3 sigma of the reference's binned Monte Carlo values
    blk = [b for b in golden("loop_op.json") if "vectors" in b and b.get("spin2", 1) == 1]
    assert len(blk) == 1
    b = blk[0]
    r = orc.ed.thermal(1, b["L"], b["T"], jxy=b["jxy"], jz=b["jz"])
    for name, entries in b["vectors"].items():
        assert len(entries) == 4
        for (label, mean, err), exact in zip(entries, r[name]):
            assert abs(mean - exact) <= 3 * err + 1e-6, (name, label, mean, err, exact)


def test_correlation_sums_restatement():
    # all up: every product is +1; a Neel state on an even chain: (-1)^r; the origin form
    up = np.zeros(16, dtype=np.int32)
    assert orc.correlation_sums(up, 2, 4).tolist() == [16] * 16
    neel = np.array([i % 2 for i in range(8)], dtype=np.int32)
    assert orc.correlation_sums(neel, 1, 8).tolist() == [8 * (-1) ** r for r in range(8)]
    assert orc.correlation_sums(neel, 1, 8, origin=3).tolist() == [-(-1) ** j for j in range(8)]
    rng = np.random.default_rng(3)
    s = rng.integers(0, 2, size=27)
    c = orc.correlation_sums(s, 3, 3)
    m = 1 - 2 * s
    assert c[0] == 27 and c[1 + 3 * 2] == sum(
        m[x + 3 * y + 9 * z] * m[(x + 1) % 3 + 3 * ((y + 2) % 3) + 9 * z]
        for x in range(3) for y in range(3) for z in range(3))
    # the structure factor at k = 0 is the sum of the correlations
    assert orc.structure_factor(c, 3, 3)[0] == pytest.approx(c.sum())


def _check_vs_ed(dim, L, T, jxy, jz, h, therm, sweeps, seed, keys, spin2=1):
    beta = 1.0 / T
    o = orc.Oracle(dim, L, beta, jxy, jz, h, seed=seed, spin2=spin2)
    o.sweep(therm)
    o.clear_records()
    o.sweep(sweeps)
    obs = orc.observables(o.records(), dim, L, beta, jxy, jz, h, spin2=spin2)
    ref = orc.ed.thermal(dim, L, T, jxy=jxy, jz=jz, h=h, spin2=spin2)
    N = L ** dim
    for k in keys:
        if k == "Specific Heat":
            m, e = orc.specific_heat(obs, beta, N)
        else:
            m, e = orc.binned(obs[k])
        assert abs(m - ref[k]) <= 3.5 * e + 1e-12, (k, m, e, ref[k])


def test_philox_heisenberg_chain_vs_ed():
    _check_vs_ed(1, 4, 0.25, 1.0, 1.0, 0.0, 1000, 40000, 7,
                 ["Energy", "Specific Heat", "Susceptibility", "Staggered Magnetization^2",
                  "Staggered Susceptibility"])


def test_philox_ising_chain_vs_ed():
    _check_vs_ed(1, 4, 0.5, 0.0, 1.0, 0.0, 1000, 40000, 8,
                 ["Energy", "Specific Heat", "Susceptibility", "Staggered Magnetization^2"])


def test_philox_xxz_field_chain_vs_ed():
    _check_vs_ed(1, 6, 0.5, 1.0, 0.5, 0.3, 1000, 40000, 9,
                 ["Energy", "Specific Heat", "Magnetization", "Susceptibility",
                  "Staggered Susceptibility"])


def test_philox_square_vs_ed():
    _check_vs_ed(2, 2, 0.5, 1.0, 1.0, 0.0, 1000, 20000, 10,
                 ["Energy", "Susceptibility", "Staggered Magnetization^2"])


def test_philox_spin1_chain_vs_ed():
    # S = 1 by two virtual spin-1/2 sites per site with the random boundary matching
    _check_vs_ed(1, 4, 0.5, 1.0, 1.0, 0.0, 1000, 40000, 12,
                 ["Energy", "Specific Heat", "Susceptibility", "Staggered Magnetization^2",
                  "Staggered Susceptibility"], spin2=2)


def test_philox_spin3half_xxz_field_chain_vs_ed():
    _check_vs_ed(1, 4, 1.0, 1.0, 0.5, 0.2, 1000, 30000, 13,
                 ["Energy", "Specific Heat", "Magnetization", "Susceptibility"], spin2=3)


def test_philox_square_spin1_vs_ed():
    # S = 1 on the 2x2 square lattice: 8 virtual spin-1/2 bonds meet at every virtual site
    _check_vs_ed(2, 2, 0.5, 1.0, 1.0, 0.0, 1000, 20000, 15,
                 ["Energy", "Specific Heat", "Susceptibility", "Staggered Magnetization^2"], spin2=2)


def test_philox_cubic_spin1_xxz_field_vs_ed():
    # S = 1 XXZ in a field on the 2x2x2 cube: 12 virtual bonds per virtual site
    _check_vs_ed(3, 2, 1.0, 1.0, 0.5, 0.2, 1000, 10000, 16,
                 ["Energy", "Magnetization", "Susceptibility"], spin2=2)


def test_philox_cubic_xxz_field_vs_ed():
    # simple cubic L = 2 (8 sites; the periodic wrap doubles every bond, in ED as in the engine)
    _check_vs_ed(3, 2, 0.5, 1.0, 0.5, 0.3, 1000, 30000, 14,
                 ["Energy", "Specific Heat", "Magnetization", "Susceptibility",
                  "Staggered Susceptibility"])


def test_philox_ferro_xxz_field_chain_vs_ed():
    # ferromagnetic couplings: the crossed graph (g = 1) and its frozen form
    _check_vs_ed(1, 6, 0.5, -1.0, -0.5, 0.1, 1000, 40000, 15,
                 ["Energy", "Specific Heat", "Magnetization", "Susceptibility",
                  "Staggered Susceptibility"])


def test_philox_xy_chain_vs_ed():
    # Jz = 0: both graphs at equal weight
    _check_vs_ed(1, 6, 0.4, 1.0, 0.0, 0.0, 1000, 40000, 16,
                 ["Energy", "Specific Heat", "Susceptibility", "Staggered Magnetization^2",
                  "Staggered Susceptibility"])


def _check_sse_vs_ed(dim, L, T, jxy, jz, therm, sweeps, seed, keys, normal=False, spin2=1):
    beta = 1.0 / T
    o = orc.SseOracle(dim, L, beta, jxy, jz, seed=seed, spin2=spin2)
    o.sweep(therm)
    o.clear_records()
    o.sweep(sweeps)
    obs = orc.sse_observables(o.records(), dim, L, beta, jxy, jz, normal=normal, spin2=spin2)
    ref = orc.ed.thermal(dim, L, T, jxy=jxy, jz=jz, spin2=spin2)
    for k in keys:
        if k == "Specific Heat":
            m, e = orc.specific_heat(obs, beta, L ** dim)
        else:
            m, e = orc.binned(obs[k])
        assert abs(m - ref[k]) <= 3.5 * e + 1e-12, (k, m, e, ref[k])


SSE_KEYS = ["Energy", "Specific Heat", "Magnetization^2", "Susceptibility",
            "Staggered Magnetization^2", "Staggered Susceptibility"]


def test_sse_oracle_agrees_with_reference_sse_blocks(golden):
    # every "loop; sse" block of loop.op without single-ion anisotropy (S = 1/2 Heisenberg ring
    # T = 0.25, Ising ring T = 0.5, S = 1 Heisenberg ring T = 0.25; L = 4, 4096 sweeps each)
    # within 3 combined sigma of the restatement, the number of clusters included (it depends on
    # the fragments the SSE string makes)
    n = 0
    for b in golden("loop_op.json"):
        if b["algorithm"] != "loop; sse":
            continue
        beta = 1.0 / b["T"]
        sp2 = b.get("spin2", 1)
        o = orc.SseOracle(1, b["L"], beta, b["jxy"], b["jz"], seed=31 + n, spin2=sp2)
        o.sweep(1000)
        o.clear_records()
        o.sweep(1 << 16)
        obs = orc.sse_observables(o.records(), 1, b["L"], beta, b["jxy"], b["jz"], spin2=sp2)
        for k, (v, e) in b["values"].items():
            if k == "Specific Heat":
                m, err = orc.specific_heat(obs, beta, b["L"])
            else:
                m, err = orc.binned(obs[k])
            assert abs(m - v) <= 3.0 * (err ** 2 + float(e) ** 2) ** 0.5, (b["T"], k, m, err, v, e)
            n += 1
    assert n == 21


@pytest.mark.parametrize("case", [
    (1, 8, 0.5, 1.0, 1.0),      # Heisenberg ring
    (1, 6, 0.3, 1.0, 0.5),      # XXZ
    (1, 6, 0.4, 1.0, 0.0),      # XY: graphs 0 and 1 at equal weight
    (1, 6, 0.5, -1.0, -0.5),    # ferromagnetic: the crossed graph and its frozen form
    (1, 4, 0.5, 0.0, 1.0),      # Ising: frozen graphs only
    (2, 2, 0.5, 1.0, 1.0),      # 2x2 square (doubled bonds)
    (3, 2, 0.5, 1.0, 0.5),      # 2x2x2 cube
])
def test_sse_oracle_vs_ed(case):
    dim, L, T, jxy, jz = case
    _check_sse_vs_ed(dim, L, T, jxy, jz, 1000, 40000, 40 + L + dim, SSE_KEYS)


def test_sse_oracle_normal_estimator_vs_ed():
    _check_sse_vs_ed(1, 6, 0.5, 1.0, 1.0, 1000, 60000, 77, SSE_KEYS, normal=True)


@pytest.mark.parametrize("case", [
    (1, 4, 0.5, 1.0, 1.0, 2),    # S = 1 ring
    (1, 4, 1.0, 1.0, 0.5, 3),    # S = 3/2 XXZ ring
    (1, 5, 0.7, -1.0, -0.5, 2),  # S = 1 ferromagnet on an odd ring
    (2, 2, 0.5, 1.0, 1.0, 2),    # S = 1 on the 2x2 square
])
def test_sse_oracle_spin_s_vs_ed(case):
    dim, L, T, jxy, jz, spin2 = case
    _check_sse_vs_ed(dim, L, T, jxy, jz, 1000, 40000, 90 + spin2 + L, SSE_KEYS, spin2=spin2)


def test_momentum_ed_matches_dense_ed():
    for (L, T, jxy, jz, h) in [(8, 0.3, 1.0, 0.5, 0.2), (8, 1.0, -1.0, 1.0, 0.0)]:
        a = orc.ed.thermal(1, L, T, jxy=jxy, jz=jz, h=h)
        b = orc.ed.chain_translation(L, T, jxy, jz, h)
        for k in ("Energy", "Specific Heat", "Magnetization^2", "Staggered Magnetization^2"):
            assert b[k] == pytest.approx(a[k], rel=1e-9, abs=1e-12), k
        assert np.allclose(b["Spin Correlations"], a["Spin Correlations"], atol=1e-12)


def test_philox_chain16_vs_exact_golden(golden):
    # the CPU-runnable chain workload's correctness point: Heisenberg chain L=16 at T=0.1
    g = golden("ed_chain16.json")
    o = orc.Oracle(1, 16, 10.0, 1.0, 1.0, 0.0, seed=1234)
    o.sweep(1 << 12)
    o.clear_records()
    o.sweep(1 << 14)
    obs = orc.observables(o.records(), 1, 16, 10.0)
    for k in ("Energy", "Susceptibility", "Staggered Magnetization^2"):
        m, e = orc.binned(obs[k])
        assert abs(m - g["values"][k]) <= 3.5 * e, (k, m, e, g["values"][k])
    m, e = orc.specific_heat(obs, 10.0, 16)
    assert abs(m - g["values"]["Specific Heat"]) <= 3.5 * e


def test_oracle_cluster_count_vs_exact_ising_ring():
    # the loop algorithm's mean cluster count on the classical Ising ring is known exactly
    o = orc.Oracle(1, 4, 2.0, 0.0, 1.0, 0.0, seed=44)
    o.sweep(1000)
    o.clear_records()
    o.sweep(40000)
    m, e = orc.binned(o.records()[:, 1].astype(np.float64))
    exact = orc.ising_ring_clusters(4, 0.5, 1.0)
    assert abs(m - exact) <= 3.5 * e, (m, e, exact)


def _scale_case(golden, name):
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
    return meta, bonds, graphs, sha


@pytest.mark.parametrize("name", ["square32_b16", "square128_b64"])
def test_uf_labels_at_scale_match_reference_union_find(golden, name):
    """Configurations of 2e4 and 1.2e6 vertices (the bench workload's size), made again by the
    oracle from their seeds, labelled by the oracle's union-find: the same labels as the
    reference's own looper/union_find.h (deterministic unify) gave in the build container."""
    import hashlib
    import os
    meta, bonds, graphs, sha = _scale_case(golden, name)
    assert len(bonds) == meta["nops"] and sha == meta["config_sha256"]
    lab, nc = orc.uf_label(meta["dim"], meta["L"], bonds, graphs, deterministic=True)
    assert nc == meta["nc"] and len(lab) == meta["nfrag"]
    assert hashlib.sha256(np.asarray(lab, dtype="<i4").tobytes()).hexdigest() == meta["labels_sha256"]
    if name == "square32_b16":
        z = np.load(os.path.join(os.path.dirname(__file__), "golden", "uf_scale_32.npz"))
        assert np.array_equal(z["bonds"], bonds) and np.array_equal(z["graphs"], graphs)
        assert np.array_equal(z["labels"], lab)
