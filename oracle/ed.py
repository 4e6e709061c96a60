"""Exact diagonalization oracle — test infrastructure only.

Restates the reference's diagonalization worker (diag.C:313-488) for spin-S XXZ models (S = 1/2
and, with spin2 = 2S > 1, higher spins: diag.C builds the local spin-S operators the same way)
with a uniform longitudinal field on periodic chain / square / cubic lattices:

    H = sum_<ij> [ Jz Sz_i Sz_j + Jxy/2 (S+_i S-_j + S-_i S+_j) ] - h sum_i Sz_i

H conserves total Sz, so instead of the full 2^N basis of diag.C:339-353 the matrix is built and
diagonalized one Sz sector at a time (numpy.linalg.eigh).  The thermal averages follow
diag.C:159-293:

  * Energy, Specific Heat = beta^2 (<E^2> - <E>^2) / V           (static_average2, :377-403)
  * Magnetization^2, ^4 of M = sum Sz                              (static_average4, :405-420)
  * Susceptibility = Kubo integral of M / Z / V                    (dynamic_average2, :421-424)
  * Staggered Magnetization^2 / Susceptibility with gauge (+1/-1)  (:433-462)
  * Spin Correlations <Sz_0 Sz_r> per displacement r (site order) and the Spin Structure Factor
    sum_r e^{ik.r} <Sz_0 Sz_r>, the exact values behind looper's correlation estimator
    (correlation.h:222-281)

The Kubo integral (dynamic_average2, diag.C:245-293) is evaluated within each sector, which is
exact because both M and the staggered magnetization are diagonal in the Sz basis.
"""
from __future__ import annotations

import itertools
import math

import numpy as np


def lattice(dim: int, L: int):
    """Periodic hypercubic lattice: site = x + L*y + L*L*z, bond (site, site+e_d)."""
    N = L ** dim
    bonds = []
    gauge = np.zeros(N)
    for s in range(N):
        x = [(s // L ** i) % L for i in range(dim)]
        gauge[s] = 1.0 if sum(x) % 2 == 0 else -1.0
        for d in range(dim):
            y = list(x)
            y[d] = (y[d] + 1) % L
            t = sum(y[i] * L ** i for i in range(dim))
            bonds.append((s, t))
    return N, bonds, gauge


def _sector_states_s(N: int, spin2: int, tot: int) -> np.ndarray:
    """Basis states of total (Sz + S) = tot / ... : digits d_i in [0, 2S], sum d_i = tot."""
    base = spin2 + 1
    out = []
    for digits in itertools.product(range(base), repeat=N):
        if sum(digits) == tot:
            out.append(sum(d * base ** i for i, d in enumerate(digits)))
    return np.array(out, dtype=np.int64)


def _sector_states(N: int, nup: int) -> np.ndarray:
    states = []
    for ups in itertools.combinations(range(N), nup):
        v = 0
        for u in ups:
            v |= 1 << u
        states.append(v)
    return np.array(states, dtype=np.int64)


def thermal(dim: int, L: int, T: float, jxy: float = 1.0, jz: float = 1.0, h: float = 0.0,
            spin2: int = 1):
    """Return a dict of the diag.C observables at temperature T (local spin S = spin2 / 2)."""
    beta = 1.0 / T
    N, bonds, gauge = lattice(dim, L)
    vol = float(N)
    sectors = []
    e_min = math.inf
    S = spin2 / 2.0
    base = spin2 + 1
    for nup in range(N * spin2 + 1):
        st = _sector_states(N, nup) if spin2 == 1 else _sector_states_s(N, spin2, nup)
        dimn = len(st)
        index = {int(v): i for i, v in enumerate(st)}
        H = np.zeros((dimn, dimn))
        sz = np.zeros((dimn, N))
        for i, v in enumerate(st):
            if spin2 == 1:
                bits = [(int(v) >> k) & 1 for k in range(N)]  # 1 = up
            else:
                bits = [(int(v) // base ** k) % base for k in range(N)]
            sz[i] = np.array(bits) - S
        for (a, b) in bonds:
            H[np.arange(dimn), np.arange(dimn)] += jz * sz[:, a] * sz[:, b]
            if jxy == 0.0:
                continue
            if spin2 == 1:
                for i, v in enumerate(st):
                    ba, bb = (int(v) >> a) & 1, (int(v) >> b) & 1
                    if ba != bb:
                        w = int(v) ^ (1 << a) ^ (1 << b)
                        H[index[w], i] += jxy / 2
            else:
                # Jxy/2 (S+_a S-_b + S-_a S+_b); S+|m> = sqrt(S(S+1) - m(m+1)) |m+1>
                for i, v in enumerate(st):
                    ma, mb = sz[i, a], sz[i, b]
                    if ma < S and mb > -S:
                        c = math.sqrt(S * (S + 1) - ma * (ma + 1)) * math.sqrt(S * (S + 1) - mb * (mb - 1))
                        w = int(v) + base ** a - base ** b
                        H[index[w], i] += jxy / 2 * c
                    if ma > -S and mb < S:
                        c = math.sqrt(S * (S + 1) - ma * (ma - 1)) * math.sqrt(S * (S + 1) - mb * (mb + 1))
                        w = int(v) - base ** a + base ** b
                        H[index[w], i] += jxy / 2 * c
        m = sz.sum(axis=1)
        H[np.arange(dimn), np.arange(dimn)] -= h * m
        ev, U = np.linalg.eigh(H)
        ms = sz @ gauge
        szz = sz[:, :1] * sz  # Sz_0 Sz_r per basis state
        sectors.append((ev, U, m, ms, szz))
        e_min = min(e_min, ev[0])

    Z = E1 = E2 = 0.0
    M2 = M4 = Ms2 = Ms4 = 0.0
    M1 = 0.0
    chi = chis = 0.0
    corr = np.zeros(N)
    for ev, U, m, ms, szz in sectors:
        w = np.exp(-beta * (ev - e_min))
        Z += w.sum()
        E1 += (ev * w).sum()
        E2 += (ev ** 2 * w).sum()
        # static averages of diagonal operators: <n|D|n> = sum_i U_in^2 D_i
        P = U ** 2
        M1 += (w * (P.T @ m)).sum()
        M2 += (w * (P.T @ m ** 2)).sum()
        M4 += (w * (P.T @ m ** 4)).sum()
        Ms2 += (w * (P.T @ ms ** 2)).sum()
        Ms4 += (w * (P.T @ ms ** 4)).sum()
        corr += (P.T @ szz).T @ w
        chi += _kubo(beta, ev, U, m, w, e_min)
        chis += _kubo(beta, ev, U, ms, w, e_min)
    E1 /= Z
    E2 /= Z
    corr /= Z
    sfac = np.real(np.fft.ifftn(corr.reshape((L,) * dim)) * N).reshape(-1)
    return {
        "Spin Correlations": corr,
        "Staggered Spin Correlations": corr * gauge * gauge[0],
        "Spin Structure Factor": sfac,
        "Energy": E1,
        "Energy Density": E1 / vol,
        "Specific Heat": beta ** 2 * (E2 - E1 ** 2) / vol,
        "Magnetization": M1 / Z,
        "Magnetization^2": M2 / Z,
        "Magnetization^4": M4 / Z,
        "Susceptibility": chi / Z / vol,
        "Staggered Magnetization^2": Ms2 / Z,
        "Staggered Magnetization^4": Ms4 / Z,
        "Staggered Susceptibility": chis / Z / vol,
    }


def _kubo(beta, ev, U, d, w, e_min):
    """dynamic_average2 (diag.C:245-293) within one sector for a diagonal operator d."""
    A = U.T @ (d[:, None] * U)
    A2 = A ** 2
    En = ev[:, None]
    Em = ev[None, :]
    wn = w[:, None]
    wm = w[None, :]
    diff = En - Em
    with np.errstate(divide="ignore", invalid="ignore"):
        wij = np.where(np.abs(diff) > 1e-12, -(wn - wm) / diff, beta * wn)
    return float((A2 * wij).sum())
