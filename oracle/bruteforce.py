"""Brute-force second-quantised RDMs for tiny active spaces.

TEST INFRASTRUCTURE ONLY.  An independent check of the RDM generator: it
applies fermionic annihilators to an explicit determinant dictionary and
forms every spin-free element directly from its definition,

    Gamma_k(P;Q) = sum_sigma <Psi| a+_{P1 s1} .. a+_{Pk sk} a_{Qk sk} .. a_{Q1 s1} |Psi>,

the convention of the reference's arrays (dal(i,j) = <E_ij>, taa(i,j,k,l) =
sum <a+_i a+_j a_l a_k>, daaa and the packed ro4 likewise;
src/koopro4QD.F90:4881-5049 fix the pair ordering through bro3/bro2/bro1).
No code is shared with the generator.
"""
from __future__ import annotations

import itertools

import numpy as np


def _annihilate(state: dict, so: int) -> dict:
    out = {}
    for det, c in state.items():
        if not (det >> so) & 1:
            continue
        sign = -1.0 if bin(det & ((1 << so) - 1)).count("1") % 2 else 1.0
        nd = det & ~(1 << so)
        out[nd] = out.get(nd, 0.0) + sign * c
    return out


def _dot(a: dict, b: dict) -> float:
    if len(a) > len(b):
        a, b = b, a
    return sum(v * b.get(k, 0.0) for k, v in a.items())


def spinfree_rdm(n: int, amask, bmask, cbra, cket, k: int) -> np.ndarray:
    """Dense Gamma_k with shape (n,)*2k, axes (P1..Pk, Q1..Qk)."""
    def vec(c):
        st = {}
        for a, b, x in zip(amask, bmask, c):
            st[int(a) | (int(b) << n)] = st.get(int(a) | (int(b) << n), 0.0) + float(x)
        return st

    bra, ket = vec(cbra), vec(cket)
    cache_b, cache_k = {}, {}

    def phi(state, cache, orbs, spins):
        key = (orbs, spins)
        if key not in cache:
            st = state
            for o, s in zip(orbs, spins):  # a_{q1} acts first
                st = _annihilate(st, o + n * s)
                if not st:
                    break
            cache[key] = st
        return cache[key]

    out = np.zeros((n,) * (2 * k))
    for P in itertools.product(range(n), repeat=k):
        for Qt in itertools.product(range(n), repeat=k):
            tot = 0.0
            for spins in itertools.product((0, 1), repeat=k):
                pb = phi(bra, cache_b, P, spins)
                if not pb:
                    continue
                qk = phi(ket, cache_k, Qt, spins)
                if qk:
                    tot += _dot(pb, qk)
            out[P + Qt] = tot
    return out


def lindice(i1, i2, i3, i4):
    return (i1 - 1) * i1 * (i1 + 1) * (i1 + 2) // 24 + (i2 - 1) * i2 * (i2 + 1) // 6 + i3 * (i3 - 1) // 2 + i4


def normind(*q):
    s = sorted(q, reverse=True)
    return lindice(*s)


def _create(state: dict, so: int) -> dict:
    out = {}
    for det, c in state.items():
        if (det >> so) & 1:
            continue
        sign = -1.0 if bin(det & ((1 << so) - 1)).count("1") % 2 else 1.0
        nd = det | (1 << so)
        out[nd] = out.get(nd, 0.0) + sign * c
    return out


def _epq(state: dict, n: int, p: int, q: int) -> dict:
    """E_pq |state> = sum_sigma a+_{p sigma} a_{q sigma} |state>."""
    out = {}
    for s in (0, 1):
        t = _create(_annihilate(state, q + n * s), p + n * s)
        for k, v in t.items():
            out[k] = out.get(k, 0.0) + v
    return out


def casci(n: int, na: int, nb: int, h: np.ndarray, g: np.ndarray, nroots: int = 1):
    """Eigenstates of the active-space Hamiltonian
    H = sum_pq h_pq E_pq + 1/2 sum_pqrs g[p,q,r,s] (E_pq E_rs - delta_qr E_ps)
    in the full CAS determinant space.  Returns (amask, bmask, coef[ndet,nroots], energies)."""
    from itertools import combinations
    sa = [sum(1 << i for i in c) for c in combinations(range(n), na)]
    sb = [sum(1 << i for i in c) for c in combinations(range(n), nb)]
    sa.sort(); sb.sort()
    dets = [(a, b) for a in sa for b in sb]
    index = {a | (b << n): i for i, (a, b) in enumerate(dets)}
    H = np.zeros((len(dets), len(dets)))
    for j, (a, b) in enumerate(dets):
        ket = {a | (b << n): 1.0}
        ers = {(r, s): _epq(ket, n, r, s) for r in range(n) for s in range(n)}
        acc = {}
        for (r, s), st in ers.items():
            for p in range(n):
                for q in range(n):
                    coefs = 0.5 * g[p, q, r, s]
                    if coefs == 0.0 or not st:
                        continue
                    for k, v in _epq(st, n, p, q).items():
                        acc[k] = acc.get(k, 0.0) + coefs * v
            w = h[r, s] - 0.5 * sum(g[r, q, q, s] for q in range(n))
            for k, v in st.items():
                acc[k] = acc.get(k, 0.0) + w * v
        for k, v in acc.items():
            H[index[k], j] += v
    H = 0.5 * (H + H.T)
    w, V = np.linalg.eigh(H)
    amask = np.array([a for a, _ in dets], dtype=np.uint32)
    bmask = np.array([b for _, b in dets], dtype=np.uint32)
    return amask, bmask, np.asfortranarray(V[:, :nroots]), w[:nroots]


def expect_e_product(n: int, amask, bmask, coef, pairs) -> float:
    """<Psi| E_{p1 q1} E_{p2 q2} ... |Psi> for 0-based orbital pairs."""
    st = {}
    for a, b, x in zip(amask, bmask, coef):
        st[int(a) | (int(b) << n)] = float(x)
    ket = dict(st)
    for p, q in reversed(list(pairs)):
        ket = _epq(ket, n, p, q)
    return _dot(st, ket)
