"""ctypes access to the CPU oracle (oracle/looper_oracle.cpp) — test infrastructure only."""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
sys.path.insert(0, ORACLE_DIR)

import ed  # noqa: E402  (oracle/ed.py)

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_void_p]
        for f in ("orc_destroy", "orc_sweep", "orc_num_sites", "orc_num_ops", "orc_num_records",
                  "orc_get_records", "orc_clear_records", "orc_get_state", "orc_set_state",
                  "orc_last_config", "orc_last_labels", "orc_last_nc"):
            getattr(L, f).argtypes = None
        L.orc_log_spec.restype = ctypes.c_float
        L.orc_log_spec.argtypes = [ctypes.c_float]
        L.orc_gap_uniform.restype = ctypes.c_float
        L.orc_gap_uniform.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.orc_exp_spec.restype = ctypes.c_float
        L.orc_exp_spec.argtypes = [ctypes.c_float]
        L.orc_weights.restype = ctypes.c_double
        L.orc_weights.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_void_p]
        L.orc_standalone.argtypes = [ctypes.c_uint, ctypes.c_double, ctypes.c_uint, ctypes.c_uint,
                                     ctypes.c_void_p, ctypes.c_void_p]
        L.orc_philox.argtypes = [ctypes.c_uint64] + [ctypes.c_uint32] * 4 + [ctypes.c_void_p]
        _lib = L
    return _lib


class _P(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("L", ctypes.c_int), ("beta", ctypes.c_double),
                ("jxy", ctypes.c_double), ("jz", ctypes.c_double), ("h", ctypes.c_double),
                ("force_scatter", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("random_spins", ctypes.c_int), ("deterministic_uf", ctypes.c_int),
                ("spin2", ctypes.c_int)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


RECORD_WORDS = 32


class Oracle:
    """One Markov chain in philox mode (the GPU's random source)."""

    def __init__(self, dim, L, beta, jxy=1.0, jz=1.0, h=0.0, seed=1, random_spins=True,
                 force_scatter=0.0, deterministic_uf=False, spin2=1):
        self.dim, self.L, self.beta = dim, L, beta
        self.jxy, self.jz, self.h = jxy, jz, h
        self.spin2 = spin2
        p = _P(dim, L, beta, jxy, jz, h, force_scatter, seed, 1 if random_spins else 0,
               1 if deterministic_uf else 0, spin2)
        self._h = ctypes.c_void_p(lib().orc_create(ctypes.byref(p)))
        self.N = lib().orc_num_sites(self._h)

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sweep(self, n=1):
        lib().orc_sweep(self._h, ctypes.c_int(n))
        assert lib().orc_status(self._h) == 0, "boundary spin sectors differ"

    def bonds(self):
        N, bonds, _ = ed.lattice(self.dim, self.L)
        return [b[0] for b in bonds], [b[1] for b in bonds]

    def records(self):
        n = lib().orc_num_records(self._h)
        r = np.zeros(n * RECORD_WORDS, dtype=np.uint64)
        if n:
            lib().orc_get_records(self._h, _ptr(r))
        return r.reshape(n, RECORD_WORDS)

    def clear_records(self):
        lib().orc_clear_records(self._h)

    def state(self):
        cap = 1 << 22
        spins = np.zeros(self.N, dtype=np.int32)
        bonds = np.zeros(cap, dtype=np.int32)
        times = np.zeros(cap, dtype=np.float64)
        n = lib().orc_get_state(self._h, _ptr(spins), _ptr(bonds), _ptr(times), ctypes.c_int(cap))
        return spins, bonds[:n].copy(), times[:n].copy()

    def set_state(self, spins, bonds, times, sweep):
        spins = np.ascontiguousarray(spins, dtype=np.int32)
        bonds = np.ascontiguousarray(bonds, dtype=np.int32)
        times = np.ascontiguousarray(times, dtype=np.float64)
        lib().orc_set_state(self._h, _ptr(spins), _ptr(bonds), _ptr(times),
                            ctypes.c_int(len(bonds)), ctypes.c_uint32(sweep))

    def last_config(self):
        cap = 1 << 22
        spins = np.zeros(self.N, dtype=np.int32)
        b = np.zeros(cap, dtype=np.int32)
        t = np.zeros(cap, dtype=np.float64)
        g = np.zeros(cap, dtype=np.int32)
        o = np.zeros(cap, dtype=np.int32)
        n = lib().orc_last_config(self._h, _ptr(spins), _ptr(b), _ptr(t), _ptr(g), _ptr(o),
                                  ctypes.c_int(cap))
        return {"spins": spins.tolist(), "bonds": b[:n].tolist(), "times": t[:n].tolist(),
                "graphs": g[:n].tolist(), "offdiag": o[:n].tolist()}

    def last_labels(self):
        cap = 1 << 23
        lab = np.zeros(cap, dtype=np.int32)
        n = lib().orc_last_labels(self._h, _ptr(lab), ctypes.c_int(cap))
        return lab[:n].copy(), lib().orc_last_nc(self._h)


class SseOracle:
    """One SSE chain (sse.C) in philox mode: the random source of the GPU's SSE form."""

    def __init__(self, dim, L, beta, jxy=1.0, jz=1.0, seed=1, random_spins=True, spin2=1):
        self.dim, self.L, self.beta = dim, L, beta
        p = _P(dim, L, beta, jxy, jz, 0.0, 0.0, seed, 1 if random_spins else 0, 1, spin2)
        L_ = lib()
        L_.orc_sse_create.restype = ctypes.c_void_p
        L_.orc_sse_create.argtypes = [ctypes.c_void_p]
        self._h = ctypes.c_void_p(L_.orc_sse_create(ctypes.byref(p)))
        assert self._h.value
        self.N = L ** dim * spin2

    def close(self):
        if self._h:
            lib().orc_sse_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sweep(self, n=1):
        lib().orc_sse_sweep(self._h, ctypes.c_int(n))
        assert lib().orc_sse_status(self._h) == 0, "boundary spin sectors differ"

    def records(self):
        n = lib().orc_sse_num_records(self._h)
        r = np.zeros(n * RECORD_WORDS, dtype=np.uint64)
        if n:
            lib().orc_sse_get_records(self._h, _ptr(r))
        return r.reshape(n, RECORD_WORDS)

    def clear_records(self):
        lib().orc_sse_clear_records(self._h)

    def state(self):
        """(spins at the bottom, operator codes bond << 1 | off-diagonal in string order)"""
        cap = 1 << 22
        spins = np.zeros(self.N, dtype=np.int32)
        ops = np.zeros(cap, dtype=np.uint32)
        n = lib().orc_sse_get_state(self._h, _ptr(spins), _ptr(ops), ctypes.c_int(cap))
        return spins, ops[:n].copy()

    def set_state(self, spins, ops, sweep):
        spins = np.ascontiguousarray(spins, dtype=np.int32)
        ops = np.ascontiguousarray(ops, dtype=np.uint32)
        lib().orc_sse_set_state(self._h, _ptr(spins), _ptr(ops), ctypes.c_int(len(ops)),
                                ctypes.c_uint32(sweep))


def standalone(L, T, sweeps, therm):
    out = np.zeros(10)
    speed = ctypes.c_double()
    lib().orc_standalone(L, T, sweeps, therm, _ptr(out), ctypes.byref(speed))
    return out, speed.value


def uf_label(dim, L, bonds, graphs, deterministic=True):
    bonds = np.ascontiguousarray(bonds, dtype=np.int32)
    graphs = np.ascontiguousarray(graphs, dtype=np.int32)
    cap = L ** dim + len(bonds) + 8
    lab = np.zeros(cap, dtype=np.int32)
    nc = ctypes.c_int()
    n = lib().orc_uf_label(ctypes.c_int(dim), ctypes.c_int(L), ctypes.c_int(len(bonds)), _ptr(bonds),
                           _ptr(graphs), ctypes.c_int(1 if deterministic else 0), _ptr(lab),
                           ctypes.c_int(cap), ctypes.byref(nc))
    return lab[:n].copy(), nc.value


def uf_replay(n, pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1)
    parent = np.zeros(n, dtype=np.int32)
    root = np.zeros(n, dtype=np.int32)
    weight = np.zeros(n, dtype=np.int32)
    lib().orc_uf_replay(ctypes.c_int(n), ctypes.c_int(len(pairs) // 2), _ptr(pairs), _ptr(parent),
                        _ptr(root), _ptr(weight))
    return parent, root, weight


def philox(seed, c0, c1, c2, c3):
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox(seed, c0, c1, c2, c3, _ptr(out))
    return out


def philox_raw(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox_raw(_ptr(c), _ptr(k), _ptr(out))
    return out


def weights(jxy, jz, force_scatter=0.0):
    v = np.zeros(4)
    W = lib().orc_weights(jxy, jz, force_scatter, _ptr(v))
    return v, W


def u128(r, i):
    return r[:, i].astype(np.float64) + r[:, i + 1].astype(np.float64) * 2.0 ** 64


def observables(records, dim, L, beta, jxy=1.0, jz=1.0, h=0.0, spin2=1):
    """Per-sweep observables from oracle records (path_integral.C:827-862; energy.h:76-84;
    susceptibility.h:200-254 improved / :303-335 normal).  N is the number of real sites (the
    volume); a spin-S chain has spin2^2 virtual bonds per real bond."""
    r = records
    N = L ** dim
    NB = N * dim * spin2 * spin2
    v, W = weights(jxy, jz)
    offset = NB * W / 2
    nop = r[:, 0].astype(np.float64)
    s = lambda i: r[:, i].view(np.int64).astype(np.float64)  # noqa: E731
    ene = offset - nop / beta
    field = abs(h) > 1e-12
    if field:
        ene = ene + (-h) * s(24) * 2.0 ** -40 / 2
    out = {"Energy": ene, "Energy^2": ene ** 2 - nop / beta ** 2,
           "Number of Clusters": r[:, 1].astype(np.float64)}
    if not field:
        out["Magnetization^2"] = r[:, 4].astype(np.float64) / 4
        out["Susceptibility"] = beta * u128(r, 18) * 2.0 ** -80 / 4 / N
        out["Staggered Magnetization^2"] = r[:, 6].astype(np.float64) / 4
        out["Staggered Susceptibility"] = beta * u128(r, 22) * 2.0 ** -80 / 4 / N
    else:
        m = s(2) / 2
        ms = s(3) / 2
        ma = s(25) * 2.0 ** -40 / 2
        sma = s(26) * 2.0 ** -40 / 2
        out["Magnetization"] = m
        out["Magnetization^2"] = m ** 2
        out["Susceptibility"] = beta * ma ** 2 / N
        out["Staggered Magnetization^2"] = ms ** 2
        out["Staggered Susceptibility"] = beta * sma ** 2 / N
    return out


def sse_observables(records, dim, L, beta, jxy=1.0, jz=1.0, normal=False, spin2=1):
    """Per-sweep observables from SSE oracle records: energy as on the path-integral form
    (sse.C:383-384, energy.h:76-84) and the SSE susceptibilities of the improved estimator
    (susceptibility.h:224-225, 231-232): beta (dip(integral, n) + tau0) / (n + 1) / V, with the
    time-integrated sums in operator-index units."""
    r = records
    N = L ** dim
    NB = N * dim * spin2 * spin2
    v, W = weights(jxy, jz)
    nop = r[:, 0].astype(np.float64)
    ene = NB * W / 2 - nop / beta
    dip = lambda x: np.where(nop > 0, x / np.maximum(nop, 1), 0.0)  # noqa: E731
    if normal:  # susceptibility.h:303-335: M at the bottom, its operator-index integral MA
        s = lambda i: r[:, i].view(np.int64).astype(np.float64)  # noqa: E731
        m, sm, ma, sma = s(2) / 2, s(3) / 2, s(25) / 2, s(26) / 2
        return {"Energy": ene, "Energy^2": ene ** 2 - nop / beta ** 2,
                "Magnetization^2": m ** 2,
                "Susceptibility": beta * (dip(ma ** 2) + m ** 2) / (nop + 1) / N,
                "Staggered Magnetization^2": sm ** 2,
                "Staggered Susceptibility": beta * (dip(sma ** 2) + sm ** 2) / (nop + 1) / N}
    m2 = r[:, 4].astype(np.float64) / 4
    sm2 = r[:, 6].astype(np.float64) / 4
    return {"Energy": ene, "Energy^2": ene ** 2 - nop / beta ** 2,
            "Number of Clusters": r[:, 1].astype(np.float64),
            "Magnetization^2": m2,
            "Susceptibility": beta * (dip(u128(r, 18) / 4) + m2) / (nop + 1) / N,
            "Staggered Magnetization^2": sm2,
            "Staggered Susceptibility": beta * (dip(u128(r, 22) / 4) + sm2) / (nop + 1) / N}


def binned(x, nbins=64):
    """Mean and error from equal-size bins (a jackknife-free binning estimate)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x) // nbins * nbins
    b = x[:n].reshape(nbins, -1).mean(axis=1)
    return float(x.mean()), float(b.std(ddof=1) / np.sqrt(nbins))


def specific_heat(obs, beta, N, nbins=64):
    """C = beta^2 (<E^2> - <E>^2) / V (energy.h:89-101) with a jackknife error over bins."""
    e = np.asarray(obs["Energy"])
    e2 = np.asarray(obs["Energy^2"])
    n = len(e) // nbins * nbins
    eb = e[:n].reshape(nbins, -1).mean(axis=1)
    e2b = e2[:n].reshape(nbins, -1).mean(axis=1)
    tot_e, tot_e2 = eb.sum(), e2b.sum()
    jk = []
    for i in range(nbins):
        me = (tot_e - eb[i]) / (nbins - 1)
        me2 = (tot_e2 - e2b[i]) / (nbins - 1)
        jk.append(beta ** 2 * (me2 - me ** 2) / N)
    jk = np.array(jk)
    c = beta ** 2 * (e2b.mean() - eb.mean() ** 2) / N
    err = np.sqrt((nbins - 1) / nbins * ((jk - jk.mean()) ** 2).sum())
    return float(c), float(err)


def correlation_sums(spins, dim, L, origin=-1):
    """The exact integer behind looper's spin-correlation normal estimator for one tau = 0
    configuration (correlation.h:222-266, before the 1/4 and multiplicity factors): with m = 1 - 2s,
    entry r = x + L y + L^2 z is sum_i m_i m_{i+r} over all sites i (periodic displacement), or,
    for an origin o, m_o m_r."""
    m = 1 - 2 * np.asarray(spins, dtype=np.int64)
    if origin >= 0:
        return m[origin] * m
    g = m.reshape((L,) * dim)  # axes (z, y, x): site = x + L y + L^2 z
    out = np.zeros_like(g)
    for idx in np.ndindex(*g.shape):
        out[idx] = int((g * np.roll(g, tuple(-i for i in idx), axis=tuple(range(dim)))).sum())
    return out.reshape(-1)


def structure_factor(corr, dim, L):
    """sum_r e^{ik.r} C(r) over the periodic grid (site order), k = 2 pi (x, y, z) / L: the
    spin structure factor of correlation.h:268-281 from the displacement correlations."""
    c = np.asarray(corr, dtype=np.float64).reshape((L,) * dim)
    return np.real(np.fft.ifftn(c) * c.size).reshape(-1)


def ising_ring_clusters(L, T, jz):
    """Exact mean cluster count of the loop algorithm on the classical Ising ring (Jxy = 0): each
    antiparallel bond holds at least one frozen graph (weight Jz/2, graph_impl.h:255-328) with
    probability p = 1 - exp(-beta Jz / 2), independently; k connected bonds leave L - k clusters,
    or 1 when all L are connected."""
    import math
    from itertools import product
    beta = 1.0 / T
    p = 1.0 - math.exp(-beta * jz / 2)
    z = num = 0.0
    for spins in product((0, 1), repeat=L):
        na = sum(spins[i] != spins[(i + 1) % L] for i in range(L))
        w = math.exp(-beta * jz * (L - 2 * na) / 4)
        nc = sum(math.comb(na, k) * p ** k * (1 - p) ** (na - k) * (L - k if k < L else 1)
                 for k in range(na + 1))
        z += w
        num += w * nc
    return num / z
