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


def chain_translation(L: int, T: float, jxy: float = 1.0, jz: float = 1.0, h: float = 0.0):
    """diag.C's thermal averages for the periodic S=1/2 XXZ chain, block-diagonal in total Sz
    and crystal momentum (the translation eigenbasis |a(k)> = N_a^-1/2 sum_r e^{-ikr} T^r |a> of
    representatives a), so that L = 16 needs blocks of ~800 states instead of 12870.  Returns the
    operators that commute with translations: Energy (Density), Specific Heat, Magnetization^2,
    Susceptibility (= beta <M^2> / V, M conserved), the Spin Correlations <Sz_0 Sz_r> and from them
    Staggered Magnetization^2 = L sum_r (-1)^r <Sz_0 Sz_r> (L even)."""
    beta = 1.0 / T
    full = (1 << L) - 1

    def rot(v):  # translation by one site: bit i -> bit i+1
        return ((v << 1) | (v >> (L - 1))) & full

    def szz_row(v):  # sum_i Sz_i Sz_{i+r} for every r (diagonal, translation invariant)
        s = np.array([((v >> i) & 1) - 0.5 for i in range(L)])
        return np.array([float((s * np.roll(s, -r)).sum()) for r in range(L)])

    levels = []   # (energies, weights over representatives per eigenvector, rep diag values)
    e_min = math.inf
    for nup in range(L + 1):
        reps, per = [], {}
        for st in _sector_states(L, nup):
            v = int(st)
            orbit, w, R = [v], v, 0
            for r in range(1, L + 1):
                w = rot(w)
                if w == v:
                    R = r
                    break
                orbit.append(w)
            if min(orbit) == v:
                reps.append(v)
                per[v] = R
        idx = {a: i for i, a in enumerate(reps)}
        # representative and shift of every state of the sector
        rep_of = {}
        for a in reps:
            w = a
            for l in range(per[a]):
                rep_of[w] = (a, l)   # T^l a = w, so T^{-l} w = a
                w = rot(w)
        diag = np.zeros(len(reps))
        offd = []   # (i_a, i_b, l): H_j |a> = Jxy/2 T^{-l}... stored as the shift from b to the state
        for i, a in enumerate(reps):
            bits = [(a >> k) & 1 for k in range(L)]
            e = 0.0
            for k in range(L):
                b1, b2 = bits[k], bits[(k + 1) % L]
                e += jz * (b1 - 0.5) * (b2 - 0.5)
                if b1 != b2 and jxy != 0.0:
                    w = a ^ (1 << k) ^ (1 << ((k + 1) % L))
                    b, l = rep_of[w]
                    offd.append((i, idx[b], l))
            e -= h * (nup - L / 2.0)
            diag[i] = e
        corr_rep = np.array([szz_row(a) for a in reps]) / L if reps else np.zeros((0, L))
        m2 = (nup - L / 2.0) ** 2
        for m in range(L):
            k = 2.0 * math.pi * m / L
            ok = [i for i, a in enumerate(reps) if (m * per[a]) % L == 0]
            if not ok:
                continue
            pos = {i: j for j, i in enumerate(ok)}
            H = np.zeros((len(ok), len(ok)), dtype=complex)
            for j, i in enumerate(ok):
                H[j, j] = diag[i]
            for (i, ib, l) in offd:
                if i in pos and ib in pos:
                    # H|a(k)> gets jxy/2 e^{-ik l'} sqrt(R_a / R_b) |b(k)>, where T^{l'} w = b, i.e.
                    # l' = -l (w = T^l b)
                    ra, rb = per[reps[i]], per[reps[ib]]
                    H[pos[ib], pos[i]] += jxy / 2 * np.exp(1j * k * l) * math.sqrt(ra / rb)
            ev, U = np.linalg.eigh(H)
            P = np.abs(U) ** 2
            levels.append((ev, P.T @ corr_rep[ok], m2))
            e_min = min(e_min, ev[0])
    Z = E1 = E2 = M2 = 0.0
    corr = np.zeros(L)
    for ev, cr, m2 in levels:
        w = np.exp(-beta * (ev - e_min))
        Z += w.sum()
        E1 += (w * ev).sum()
        E2 += (w * ev ** 2).sum()
        M2 += w.sum() * m2
        corr += w @ cr
    E1 /= Z
    E2 /= Z
    corr /= Z
    sign = np.array([(-1.0) ** r for r in range(L)])
    return {
        "Energy": E1,
        "Energy Density": E1 / L,
        "Specific Heat": beta ** 2 * (E2 - E1 ** 2) / L,
        "Magnetization^2": M2 / Z,
        "Susceptibility": beta * M2 / Z / L,
        "Spin Correlations": corr,
        "Staggered Magnetization^2": L * float((sign * corr).sum()),
    }
