"""Literal loop-by-loop restatement of the stage-2 class routines.

TEST INFRASTRUCTURE ONLY, for tiny active spaces: every routine below is a
line-for-line transliteration of the Fortran loop nests of src/qdnevpt.F
(1-based indices, the same loop order, the same accessor calls), kept
deliberately unvectorised so that it can be read side by side with the
reference.  It cross-checks the vectorised oracle (qdnevpt_oracle.py), whose
index permutations are the error-prone part.  Orbitals, transformed integrals
and the PC metric algebra are shared with the vectorised oracle.
"""
from __future__ import annotations

import numpy as np

from .qdnevpt_oracle import Stage2Result, _State, dense_B, pc_transform, unpack_tri


class _Acc:
    """The reference's accessor functions on one state's or pair's RDMs
    (src/qdnevpt.F:6448-6519; arrays indexed 1-based here)."""

    def __init__(self, d3, d2, d1):
        self.d3, self.d2, self.d1 = d3, d2, d1

    def D1(self, a, b):
        return self.d1[a - 1, b - 1]

    def D2(self, a, b, c, d):
        return self.d2[a - 1, b - 1, c - 1, d - 1]

    def D3(self, a, b, c, d, e, f):
        return self.d3[a - 1, b - 1, c - 1, d - 1, e - 1, f - 1]

    def ee2(self, a, b, c, d):
        v = self.D2(b, d, a, c)
        if b == c:
            v += self.D1(d, a)
        return v

    def eee2(self, a, b, c, d, e, f):
        v = self.D3(b, d, f, a, c, e)
        if e == d:
            v += self.D2(b, f, a, c)
        if e == b:
            v += self.D2(f, d, a, c)
        if b == c:
            v += self.D2(d, f, a, e)
        if b == c and e == d:
            v += self.D1(f, a)
        return v

    def eee2t(self, a, b, c, d, e, f):
        v = -self.eee2(a, b, d, c, e, f)
        if c == d:
            v += 2.0 * self.ee2(a, b, e, f)
        return v

    def ee2tr(self, a, b, c, d):
        v = -self.ee2(a, b, d, c)
        if c == d:
            v += 2.0 * self.D1(b, a)
        return v

    def ee2tl(self, a, b, c, d):
        v = -self.ee2(b, a, c, d)
        if a == b:
            v += 2.0 * self.D1(d, c)
        return v

    def ro2toff(self, ap, bp, a, b):
        v = self.D2(ap, bp, a, b)
        if ap == a:
            v -= 2.0 * self.D1(bp, b)
        if bp == b:
            v -= 2.0 * self.D1(ap, a)
        if ap == b:
            v += self.D1(bp, a)
        if bp == a:
            v += self.D1(ap, b)
        return v


def qdnevpt_loops(inp, classes=range(8)):
    M = inp.metat
    nc, na, nv, norb = inp.ncore, inp.nact, inp.nvirt, inp.norb
    B = dense_B(inp.chol, norb)
    h = unpack_tri(inp.oneint, norb)
    r = Stage2Result(e2mpp=np.zeros((8, M)), psimpp=np.zeros((8, M)), e2enp=np.zeros((8, M)),
                     psienep=np.zeros((8, M)), e2mp=np.zeros((M, M)), e2en=np.zeros((M, M)), psimp=np.zeros(M),
                     psien=np.zeros(M), nnew={}, epsnew=np.zeros((norb, M)))
    for s in range(M):
        st = _State(inp, s, B, h)
        L = _Loops(inp, st, s, r)
        for k, fn in ((0, L.v0), (1, L.v1k), (2, L.vm1k), (3, L.v2mod), (4, L.vm2mod), (7, L.v0pmod),
                      (6, L.vmupE), (5, L.vpupE)):
            if k in classes:
                fn()
    return r


class _Loops:
    def __init__(self, inp, st, s, r):
        self.inp, self.st, self.r = inp, st, r
        self.M = inp.metat
        self.i = s + 1          # istate, 1-based
        self.nc, self.na, self.nv = inp.ncore, inp.nact, inp.nvirt
        self.norb = inp.norb
        self.acc = _Acc(inp.daaa[s], inp.taa[s], inp.dal[s])
        self.thr = inp.thr_lindep

    # helpers -------------------------------------------------------------
    def eps(self, p):
        return self.st.eps[p - 1]

    def ct(self, p, q, r_, s_):
        """cholesky_traint(p,q,r,s) with 1-based orbital indices."""
        R = self.st.R
        return float(R[:, p - 1, q - 1] @ R[:, r_ - 1, s_ - 1])

    def hp(self, p, q):
        return self.st.h[p - 1, q - 1]

    def ijcou(self, j):
        i = self.i
        if j < i:
            return (i - 1) * (i - 2) // 2 + j
        return (j - 1) * (j - 2) // 2 + i

    def off(self, j):
        k = self.ijcou(j) - 1
        inp = self.inp
        d3 = inp.ro3off[k] if inp.ro3off else None
        d2 = inp.daaoff[k] if inp.daaoff else None
        return _Acc(d3, d2, inp.daoff[k])

    def others(self):
        return [j for j in range(1, self.M + 1) if j != self.i]

    def pc_finish(self, cls, e2, psi2):
        r, i = self.r, self.i - 1
        r.e2enp[cls, i] += e2[i, i]
        r.psienep[cls, i] += psi2
        r.psien[i] += r.psienep[cls, i]
        r.e2en[i, i] += e2[i, i]
        for j in self.others():
            r.e2en[j - 1, i] += e2[j - 1, i]

    def sc_add(self, cls, co, con):
        r, i = self.r, self.i - 1
        r.e2mp[i, i] += co
        r.psimp[i] += con
        r.e2mpp[cls, i] += co
        r.psimpp[cls, i] += con

    # class (0): v0 :1661 -------------------------------------------------
    def v0(self):
        nc, na, norb, i = self.nc, self.na, self.norb, self.i
        r = self.r
        for ii in range(1, nc + 1):
            for ij in range(ii, nc + 1):
                for ir in range(nc + na + 1, norb + 1):
                    for is_ in range(ir, norb + 1):
                        zrs, zij = ir == is_, ii == ij
                        ab2 = 0.0
                        ab1 = self.ct(ij, ir, is_, ii)
                        if not (zrs or zij):
                            ab2 = self.ct(ij, is_, ir, ii)
                        if zrs and zij:
                            dint = ab1
                        if zrs != zij:
                            dint = np.sqrt(2.0) * ab1
                        if not (zrs or zij):
                            dint = 2.0 * np.sqrt(ab1 ** 2 + ab2 ** 2 - ab1 * ab2)
                        co = -dint / (self.eps(ir) + self.eps(is_) - self.eps(ii) - self.eps(ij))
                        self.sc_add(0, dint * co, co * co)
        r.e2en[i - 1, i - 1] = r.e2mp[i - 1, i - 1]
        r.psien[i - 1] = r.psimp[i - 1]
        r.e2enp[0, i - 1] = r.e2mpp[0, i - 1]
        r.psienep[0, i - 1] = r.psimpp[0, i - 1]

    # class (+1): v1k :1775 and e2p1cont :3076 ----------------------------
    def v1k(self):
        nc, na, norb, i, M = self.nc, self.na, self.norb, self.i, self.M
        A = self.acc
        gk = self.inp.eako1[i - 1]
        for ii in range(1, nc + 1):
            for ij in range(ii, nc + 1):
                for is_ in range(nc + na + 1, norb + 1):
                    dnk = {j: 0.0 for j in range(1, M + 1)}
                    ek = 0.0
                    for ia in range(1, na + 1):
                        for iap in range(1, na + 1):
                            contj = self.ct(ia + nc, ii, is_, ij)
                            contjp = self.ct(iap + nc, ii, is_, ij)
                            if ij != ii:
                                contk = self.ct(ia + nc, ij, is_, ii)
                                contkp = self.ct(iap + nc, ij, is_, ii)
                                cint = contj * contjp + contk * contkp - 0.5 * contj * contkp - 0.5 * contk * contjp
                            else:
                                cint = 0.5 * contj * contjp
                            ro = 2.0 - A.D1(ia, iap) if ia == iap else -A.D1(ia, iap)
                            dnk[i] += 2.0 * ro * cint
                            ek += gk[ia - 1, iap - 1] * cint
                            for j in self.others():
                                O = self.off(j)
                                ro = -O.D1(iap, ia) if j < i else -O.D1(ia, iap)
                                dnk[j] += 2.0 * ro * cint
                    den = 0.0
                    if abs(dnk[i]) > 0.0:
                        ek = ek / dnk[i]
                        den = self.eps(ii) + self.eps(ij) - self.eps(is_) - ek
                        co = dnk[i] / den
                        self.sc_add(1, co, co / den)
                    for j in self.others():
                        if den != 0.0:
                            self.r.e2mp[j - 1, i - 1] += dnk[j] / den
        # PC
        S = np.zeros((na, na))
        for a in range(1, na + 1):
            for b in range(1, na + 1):
                S[a - 1, b - 1] = (2.0 if a == b else 0.0) - A.D1(a, b)
        C, w, nnew = pc_transform(S, 0.5 * gk, self.thr)
        s = np.zeros((na, na, M))  # s(a,mu,jstate)
        for a in range(1, na + 1):
            for mu in range(1, na + 1):
                for ap in range(1, na + 1):
                    ro = 2.0 - A.D1(ap, a) if ap == a else -A.D1(ap, a)
                    s[a - 1, mu - 1, i - 1] += ro * C[ap - 1, mu - 1]
                    for j in self.others():
                        O = self.off(j)
                        ro = -O.D1(a, ap) if j < i else -O.D1(ap, a)
                        s[a - 1, mu - 1, j - 1] += ro * C[ap - 1, mu - 1]
        e2 = np.zeros((M, M))
        psi2 = 0.0
        for ci in range(1, nc + 1):
            for cj in range(ci, nc + 1):
                for ir in range(nc + na + 1, norb + 1):
                    for mu in range(1, na + 1):
                        rj = np.zeros(M)
                        rp = np.zeros(M)
                        for a in range(1, na + 1):
                            contj = self.ct(a + nc, ci, ir, cj)
                            if ci != cj:
                                contk = self.ct(a + nc, cj, ir, ci)
                                rj += (contj + contk) * s[a - 1, mu - 1, :]
                                rp += (contj - contk) * s[a - 1, mu - 1, :]
                            else:
                                rj += contj * s[a - 1, mu - 1, :]
                        deno = w[mu - 1] + self.eps(ir) - self.eps(ci) - self.eps(cj)
                        if ci != cj:
                            contri = (0.5 * rj[i - 1] ** 2 + 1.5 * rp[i - 1] ** 2) / deno
                            e2[i - 1, i - 1] -= contri
                            psi2 += contri / deno
                            for j in self.others():
                                e2[j - 1, i - 1] -= (0.5 * rj[j - 1] * rj[i - 1] + 1.5 * rp[j - 1] * rp[i - 1]) / deno
                        else:
                            contri = rj[i - 1] ** 2 / deno
                            e2[i - 1, i - 1] -= contri
                            psi2 += contri / deno
                            for j in self.others():
                                e2[j - 1, i - 1] -= rj[j - 1] * rj[i - 1] / deno
        self.r.e2enp[1, i - 1] = e2[i - 1, i - 1]
        self.r.psienep[1, i - 1] = psi2
        self.r.psien[i - 1] += psi2
        self.r.e2en[i - 1, i - 1] += e2[i - 1, i - 1]
        for j in self.others():
            self.r.e2en[j - 1, i - 1] += e2[j - 1, i - 1]

    # class (-1): vm1k :2095 and e2m1cont :2400 ---------------------------
    def vm1k(self):
        nc, na, norb, i, M = self.nc, self.na, self.norb, self.i, self.M
        A = self.acc
        gk = self.inp.ipko1[i - 1]
        for ir in range(nc + na + 1, norb + 1):
            for is_ in range(ir, norb + 1):
                for ii in range(1, nc + 1):
                    dnk = {j: 0.0 for j in range(1, M + 1)}
                    ek = 0.0
                    for ia in range(1, na + 1):
                        contj = self.ct(ir, ii, is_, ia + nc)
                        contk = self.ct(is_, ii, ir, ia + nc) if ir != is_ else 0.0
                        for iap in range(1, na + 1):
                            contjp = self.ct(ir, ii, is_, iap + nc)
                            contkp = self.ct(is_, ii, ir, iap + nc) if ir != is_ else 0.0
                            if ir == is_:
                                cint = 0.5 * contj * contjp
                            else:
                                cint = contj * contjp + contk * contkp - 0.5 * contj * contkp - 0.5 * contk * contjp
                            dnk[i] += 2.0 * A.D1(ia, iap) * cint
                            ek += gk[ia - 1, iap - 1] * cint
                            for j in self.others():
                                O = self.off(j)
                                ro = O.D1(ia, iap) if j < i else O.D1(iap, ia)
                                dnk[j] += 2.0 * ro * cint
                    den = 0.0
                    if abs(dnk[i]) >= 1e-14:
                        ek = -ek / dnk[i]
                        den = ek + self.eps(ii) - self.eps(ir) - self.eps(is_)
                        co = dnk[i] / den
                        self.sc_add(2, co, co / den)
                    for j in self.others():
                        if den != 0.0:
                            self.r.e2mp[j - 1, i - 1] += dnk[j] / den
        S = np.array([[A.D1(a, b) for b in range(1, na + 1)] for a in range(1, na + 1)])
        C, w, nnew = pc_transform(S, 0.5 * gk, self.thr)
        s = np.zeros((na, na, M))
        for a in range(1, na + 1):
            for mu in range(1, na + 1):
                for ap in range(1, na + 1):
                    s[a - 1, mu - 1, i - 1] += A.D1(ap, a) * C[ap - 1, mu - 1]
                    for j in self.others():
                        O = self.off(j)
                        ro = O.D1(ap, a) if j < i else O.D1(a, ap)
                        s[a - 1, mu - 1, j - 1] += ro * C[ap - 1, mu - 1]
        e2 = np.zeros((M, M))
        psi2 = 0.0
        for ir in range(nc + na + 1, norb + 1):
            for is_ in range(ir, norb + 1):
                for ci in range(1, nc + 1):
                    for mu in range(1, na + 1):
                        rj = np.zeros(M)
                        rp = np.zeros(M)
                        for a in range(1, na + 1):
                            tj = self.ct(ir, ci, is_, a + nc)
                            if ir != is_:
                                tk = self.ct(is_, ci, ir, a + nc)
                                rj += (tj + tk) * s[a - 1, mu - 1, :]
                                rp += (tj - tk) * s[a - 1, mu - 1, :]
                            else:
                                rj += tj * s[a - 1, mu - 1, :]
                        deno = w[mu - 1] + self.eps(ir) + self.eps(is_) - self.eps(ci)
                        if ir != is_:
                            contri = (0.5 * rj[i - 1] ** 2 + 1.5 * rp[i - 1] ** 2) / deno
                            e2[i - 1, i - 1] -= contri
                            psi2 += contri / deno
                            for j in self.others():
                                e2[j - 1, i - 1] -= (0.5 * rj[j - 1] * rj[i - 1] + 1.5 * rp[j - 1] * rp[i - 1]) / deno
                        else:
                            contri = rj[i - 1] ** 2 / deno
                            e2[i - 1, i - 1] -= contri
                            psi2 += contri / deno
                            for j in self.others():
                                e2[j - 1, i - 1] -= rj[j - 1] * rj[i - 1] / deno
        self.r.e2enp[2, i - 1] = e2[i - 1, i - 1]
        self.r.psienep[2, i - 1] = psi2
        self.r.psien[i - 1] += psi2
        self.r.e2en[i - 1, i - 1] += e2[i - 1, i - 1]
        for j in self.others():
            self.r.e2en[j - 1, i - 1] += e2[j - 1, i - 1]

    # classes (+2)/(-2): v2mod :3256 / vm2mod :3685 -----------------------
    def _pc2(self, cls, dmat, kmat, offget, ints_pairs, ints_diag, deno_pair, deno_diag, rowfirst_off):
        """Shared PC part of (+2)/(-2): fillcm2 + e2?2cont, fillcm2p + e2?2contp."""
        na, M, i = self.na, self.M, self.i
        n2 = na * na
        S = np.zeros((n2, n2))
        K = np.zeros((n2, n2))
        ij = 0
        for a in range(1, na + 1):
            for b in range(1, na + 1):
                kl = 0
                for c in range(1, na + 1):
                    for d in range(1, na + 1):
                        S[ij, kl] = dmat[a - 1, b - 1, c - 1, d - 1]
                        K[ij, kl] = kmat[a - 1, b - 1, c - 1, d - 1]
                        kl += 1
                ij += 1
        C, w, nnew = pc_transform(S, K, self.thr)
        s = np.zeros((n2, n2, M))
        ab = 0
        for a in range(1, na + 1):
            for b in range(1, na + 1):
                for mu in range(n2):
                    abp = 0
                    for ap in range(1, na + 1):
                        for bp in range(1, na + 1):
                            coe = C[abp, mu]
                            s[ab, mu, i - 1] += dmat[ap - 1, bp - 1, a - 1, b - 1] * coe
                            for j in self.others():
                                ro = offget(j, (b, a, bp, ap) if (j < i) == rowfirst_off else (bp, ap, b, a))
                                s[ab, mu, j - 1] += ro * coe
                            abp += 1
                ab += 1
        e2 = np.zeros((M, M))
        psi2 = 0.0
        for (x, y), dint_fn, dfn in ints_pairs:
            for mu in range(n2):
                aij = np.zeros(M)
                ab = 0
                for a in range(1, na + 1):
                    for b in range(1, na + 1):
                        aij += dint_fn(a, b) * s[ab, mu, :]
                        ab += 1
                deno = w[mu] + dfn
                contri = aij[i - 1] ** 2 / deno
                e2[i - 1, i - 1] -= contri
                psi2 += contri / deno
                for j in self.others():
                    e2[j - 1, i - 1] -= aij[j - 1] * aij[i - 1] / deno
        n1 = na * (na + 1) // 2
        S = np.zeros((n1, n1))
        K = np.zeros((n1, n1))
        ij = 0
        for a in range(1, na + 1):
            for b in range(a, na + 1):
                kl = 0
                for c in range(1, na + 1):
                    for d in range(c, na + 1):
                        S[ij, kl] = dmat[a - 1, b - 1, c - 1, d - 1] + dmat[a - 1, b - 1, d - 1, c - 1]
                        K[ij, kl] = kmat[a - 1, b - 1, c - 1, d - 1] + kmat[a - 1, b - 1, d - 1, c - 1]
                        kl += 1
                ij += 1
        C, w, nnew2 = pc_transform(S, K, self.thr)
        s = np.zeros((n1, n1, M))
        ab = 0
        for a in range(1, na + 1):
            for b in range(a, na + 1):
                for mu in range(n1):
                    abp = 0
                    for ap in range(1, na + 1):
                        for bp in range(ap, na + 1):
                            coe = C[abp, mu]
                            s[ab, mu, i - 1] += 0.5 * (dmat[ap - 1, bp - 1, a - 1, b - 1] +
                                                        dmat[ap - 1, bp - 1, b - 1, a - 1]) * coe
                            for j in self.others():
                                if (j < i) == rowfirst_off:
                                    ro = 0.5 * (offget(j, (b, a, bp, ap)) + offget(j, (b, a, ap, bp)))
                                else:
                                    ro = 0.5 * (offget(j, (bp, ap, b, a)) + offget(j, (ap, bp, b, a)))
                                s[ab, mu, j - 1] += ro * coe
                            abp += 1
                ab += 1
        for x, dint_fn, dfn in ints_diag:
            for mu in range(n1):
                aij = np.zeros(M)
                ab = 0
                for a in range(1, na + 1):
                    for b in range(a, na + 1):
                        v = dint_fn(a, b)
                        if a != b:
                            v *= 2.0
                        aij += v * s[ab, mu, :]
                        ab += 1
                deno = w[mu] + dfn
                contri = aij[i - 1] ** 2 / deno
                e2[i - 1, i - 1] -= contri
                psi2 += contri / deno
                for j in self.others():
                    e2[j - 1, i - 1] -= aij[j - 1] * aij[i - 1] / deno
        self.pc_finish(cls, e2, psi2)

    def v2mod(self):
        nc, na, i, M = self.nc, self.na, self.i, self.M
        daat = self.inp.hrdm[i - 1]
        gk = self.inp.eako2[i - 1]
        for ir in range(1, nc + 1):
            for is_ in range(ir, nc + 1):
                dn = {j: 0.0 for j in range(1, M + 1)}
                dk = 0.0
                for ica in range(1, na + 1):
                    for ida in range(1, na + 1):
                        d2 = self.ct(ir, ica + nc, is_, ida + nc)
                        for icpa in range(1, na + 1):
                            for idpa in range(1, na + 1):
                                dum = daat[icpa - 1, idpa - 1, ica - 1, ida - 1]
                                dumk = gk[icpa - 1, idpa - 1, ica - 1, ida - 1]
                                d1 = self.ct(ir, icpa + nc, is_, idpa + nc)
                                cint = d1 * d2
                                if ir == is_:
                                    cint *= 0.25
                                    dum += daat[icpa - 1, idpa - 1, ida - 1, ica - 1]
                                    dumk += gk[idpa - 1, icpa - 1, ica - 1, ida - 1]
                                dn[i] += cint * dum
                                dk += cint * dumk
                                for j in self.others():
                                    O = self.off(j)
                                    if j < i:
                                        dum = O.ro2toff(icpa, idpa, ica, ida)
                                        if ir == is_:
                                            dum += O.ro2toff(idpa, icpa, ica, ida)
                                    else:
                                        dum = O.ro2toff(ica, ida, icpa, idpa)
                                        if ir == is_:
                                            dum += O.ro2toff(ica, ida, idpa, icpa)
                                    dn[j] += dum * cint
                den = 0.0
                if abs(dn[i]) >= 1e-14:
                    den = self.eps(ir) + self.eps(is_) - dk / dn[i]
                    co = dn[i] / den
                    self.sc_add(3, co, co / den)
                for j in self.others():
                    if den != 0.0:
                        self.r.e2mp[j - 1, i - 1] += dn[j] / den

        def offget(j, idx):
            return self.off(j).ro2toff(*idx)

        pairs = [((ci, cj), (lambda a, b, ci=ci, cj=cj: self.ct(ci, b + nc, cj, a + nc)),
                  -self.eps(ci) - self.eps(cj)) for ci in range(1, nc + 1) for cj in range(ci + 1, nc + 1)]
        diag = [(ci, (lambda a, b, ci=ci: self.ct(ci, b + nc, ci, a + nc)), -2.0 * self.eps(ci))
                for ci in range(1, nc + 1)]
        self._pc2(3, daat, gk, offget, pairs, diag, None, None, rowfirst_off=True)

    def vm2mod(self):
        nc, na, nv, norb, i, M = self.nc, self.na, self.nv, self.norb, self.i, self.M
        daa = self.inp.taa[i - 1]
        gk = self.inp.ipko2[i - 1]
        v0 = nc + na
        for ir in range(v0 + 1, norb + 1):
            for is_ in range(ir, norb + 1):
                dn = {j: 0.0 for j in range(1, M + 1)}
                dk = 0.0
                for ica in range(1, na + 1):
                    for ida in range(1, na + 1):
                        for icpa in range(1, na + 1):
                            for idpa in range(1, na + 1):
                                dum = daa[icpa - 1, idpa - 1, ica - 1, ida - 1]
                                dumk = gk[icpa - 1, idpa - 1, ica - 1, ida - 1]
                                cint = self.ct(is_, ica + nc, ir, ida + nc) * self.ct(is_, icpa + nc, ir, idpa + nc)
                                if ir == is_:
                                    cint *= 0.25
                                    dum += daa[icpa - 1, idpa - 1, ida - 1, ica - 1]
                                    dumk += gk[idpa - 1, icpa - 1, ica - 1, ida - 1]
                                dn[i] += dum * cint
                                dk += dumk * cint
                                for j in self.others():
                                    O = self.off(j)
                                    if j < i:
                                        dum = O.D2(ica, ida, icpa, idpa)
                                        if ir == is_:
                                            dum += O.D2(ica, ida, idpa, icpa)
                                    else:
                                        dum = O.D2(icpa, idpa, ica, ida)
                                        if ir == is_:
                                            dum += O.D2(idpa, icpa, ica, ida)
                                    dn[j] += dum * cint
                den = 0.0
                if abs(dn[i]) >= 1e-14:
                    den = -dk / dn[i] - self.eps(ir) - self.eps(is_)
                    co = dn[i] / den
                    self.sc_add(4, co, co / den)
                for j in self.others():
                    if den != 0.0:
                        self.r.e2mp[j - 1, i - 1] += dn[j] / den

        def offget(j, idx):
            return self.off(j).D2(*idx)

        pairs = [((rr, ss), (lambda a, b, rr=rr, ss=ss: self.ct(rr, b + nc, ss, a + nc)),
                  self.eps(rr) + self.eps(ss)) for rr in range(v0 + 1, norb + 1) for ss in range(rr + 1, norb + 1)]
        diag = [(rr, (lambda a, b, rr=rr: self.ct(rr, a + nc, rr, b + nc)), 2.0 * self.eps(rr))
                for rr in range(v0 + 1, norb + 1)]
        self._pc2(4, daa, gk, offget, pairs, diag, None, None, rowfirst_off=False)

    # class (0'): v0pmod :4326, fillc0p :4195, e20pcont :4771 --------------
    def v0pmod(self):
        nc, na, norb, i, M = self.nc, self.na, self.norb, self.i, self.M
        A = self.acc
        ga, gd, gf = self.inp.gk0pa[i - 1], self.inp.gk0pd[i - 1], self.inp.gk0pf[i - 1]
        v0 = nc + na

        def heffd(ik, ir):
            v = self.hp(ik, ir)
            for j in range(1, nc + 1):
                v += 2.0 * self.ct(j, j, ik, ir) - self.ct(j, ik, j, ir)
            return v

        for ii in range(1, nc + 1):
            for ir in range(v0 + 1, norb + 1):
                djm = lambda a, b: self.ct(ii, ir, a + nc, b + nc)
                dkm = lambda a, b: self.ct(ii, a + nc, ir, b + nc)
                dn = {j: 0.0 for j in range(1, M + 1)}
                dkoo = 0.0
                for a in range(1, na + 1):
                    for b in range(1, na + 1):
                        for ap in range(1, na + 1):
                            for bp in range(1, na + 1):
                                dj, djp, dk, dkp = djm(a, b), djm(ap, bp), dkm(a, b), dkm(ap, bp)
                                dint1 = 2.0 * djp * dj - djp * dk - dkp * dj
                                dint2 = dkp * dk
                                dint11 = djp * dj - 0.5 * djp * dk - 0.5 * dj * dkp
                                dum1 = A.ee2(bp, ap, a, b)
                                dum2 = A.ee2tr(bp, b, ap, a)
                                if a == b:
                                    dum2 += A.D1(bp, ap)
                                dn[i] += dint1 * dum1 + dint2 * dum2
                                dkoo += dint11 * ga[bp - 1, ap - 1, a - 1, b - 1] + dint2 * gd[bp - 1, ap - 1, a - 1, b - 1]
                                for j in self.others():
                                    O = self.off(j)
                                    d1o = O.ee2(bp, ap, a, b)
                                    d2o = O.ee2tr(bp, b, ap, a)
                                    if a == b:
                                        d2o += O.D1(ap, bp)
                                    dn[j] += dint1 * d1o + dint2 * d2o
                dummy = {j: 0.0 for j in range(1, M + 1)}
                dummyk = 0.0
                for a in range(1, na + 1):
                    for b in range(1, na + 1):
                        di1 = 2.0 * djm(a, b) - dkm(a, b)
                        dummy[i] += A.D1(b, a) * di1
                        for j in self.others():
                            O = self.off(j)
                            dummy[j] += (O.D1(b, a) + O.D1(a, b)) * di1
                        dummyk += gf[a - 1, b - 1] * di1 * 0.5
                hh = heffd(ii, ir)
                dn[i] += 2.0 * hh * dummy[i] + 2.0 * hh ** 2
                dkoo += hh * dummyk
                for j in self.others():
                    dn[j] += hh * dummy[j]
                den = 0.0
                if abs(dn[i]) > 1e-14:
                    den = self.eps(ii) - self.eps(ir) - dkoo / dn[i]
                    co = dn[i] / den
                    self.sc_add(7, co, co / den)
                for j in self.others():
                    if den != 0.0:
                        self.r.e2mp[j - 1, i - 1] += dn[j] / den
        nn = na * na
        n2 = 2 * nn
        S = np.zeros((n2, n2))
        K = np.zeros((n2, n2))
        ab = 0
        for a in range(1, na + 1):
            for b in range(1, na + 1):
                abp = 0
                for ap in range(1, na + 1):
                    for bp in range(1, na + 1):
                        K[ab, abp] = ga[b - 1, a - 1, ap - 1, bp - 1]
                        S[ab, abp] = 2.0 * A.ee2(bp, ap, a, b)
                        K[ab, abp + nn] = -0.5 * ga[b - 1, a - 1, ap - 1, bp - 1]
                        S[ab, abp + nn] = -A.ee2(bp, ap, a, b)
                        K[ab + nn, abp] = -0.5 * ga[b - 1, a - 1, ap - 1, bp - 1]
                        S[ab + nn, abp] = -A.ee2(bp, ap, a, b)
                        K[ab + nn, abp + nn] = gd[b - 1, a - 1, ap - 1, bp - 1]
                        S[ab + nn, abp + nn] = -A.D2(bp, a, b, ap) + (2.0 * A.D1(bp, b) if a == ap else 0.0)
                        abp += 1
                ab += 1
        C, w, nnew = pc_transform(S, K, self.thr)
        s = np.zeros((nn, n2, M))
        sp = np.zeros((nn, n2, M))
        spp = np.zeros((nn, n2, M))
        iab = 0
        for ia in range(1, na + 1):
            for ib in range(1, na + 1):
                iabp = 0
                for iap in range(1, na + 1):
                    for ibp in range(1, na + 1):
                        val = A.ee2(ibp, iap, ia, ib)
                        val2 = -A.D2(iap, ib, ia, ibp) + (2.0 * A.D1(ib, ibp) if iap == ia else 0.0)
                        s[iab, :, i - 1] += val * C[iabp, :]
                        sp[iab, :, i - 1] += val * C[iabp + nn, :]
                        spp[iab, :, i - 1] += val2 * C[iabp + nn, :]
                        for j in self.others():
                            O = self.off(j)
                            if j < i:
                                val = O.ee2(ib, ia, iap, ibp)
                                val2 = -O.D2(ia, ibp, iap, ib) + (2.0 * O.D1(ibp, ib) if iap == ia else 0.0)
                            else:
                                val = O.ee2(ibp, iap, ia, ib)
                                val2 = -O.D2(iap, ib, ia, ibp) + (2.0 * O.D1(ib, ibp) if iap == ia else 0.0)
                            s[iab, :, j - 1] += val * C[iabp, :]
                            sp[iab, :, j - 1] += val * C[iabp + nn, :]
                            spp[iab, :, j - 1] += val2 * C[iabp + nn, :]
                        iabp += 1
                iab += 1
        e2 = np.zeros((M, M))
        psi2 = 0.0
        for ci in range(1, nc + 1):
            for ir in range(v0 + 1, norb + 1):
                hir = heffd(ci, ir)
                for mu in range(n2):
                    rimu = np.zeros(M)
                    rimup = np.zeros(M)
                    iab = 0
                    for ia in range(1, na + 1):
                        for ib in range(1, na + 1):
                            raib = self.ct(ci, ir, ia + nc, ib + nc)
                            rabi = self.ct(ci, ia + nc, ir, ib + nc)
                            rimu[i - 1] += (2.0 * raib - rabi) * s[iab, mu, i - 1] + 2.0 * A.D1(ib, ia) * hir * C[iab, mu]
                            rimup[i - 1] += -raib * sp[iab, mu, i - 1] + rabi * spp[iab, mu, i - 1] - \
                                hir * A.D1(ib, ia) * C[iab + nn, mu]
                            for j in self.others():
                                O = self.off(j)
                                ro = O.D1(ib, ia) if j < i else O.D1(ia, ib)
                                rimu[j - 1] += (2.0 * raib - rabi) * s[iab, mu, j - 1] + 2.0 * ro * hir * C[iab, mu]
                                rimup[j - 1] += -raib * sp[iab, mu, j - 1] + rabi * spp[iab, mu, j - 1] - \
                                    hir * ro * C[iab + nn, mu]
                            iab += 1
                    deno = w[mu] + self.eps(ir) - self.eps(ci)
                    co = rimu[i - 1] + rimup[i - 1]
                    cirmu = co / deno
                    e2[i - 1, i - 1] -= co * cirmu
                    psi2 += cirmu ** 2
                    for j in self.others():
                        e2[j - 1, i - 1] -= (rimu[j - 1] + rimup[j - 1]) * (rimu[i - 1] + rimup[i - 1]) / deno
        self.r.e2enp[7, i - 1] = e2[i - 1, i - 1]
        self.r.psienep[7, i - 1] = psi2
        self.r.psien[i - 1] += psi2
        self.r.e2en[i - 1, i - 1] += e2[i - 1, i - 1]
        for j in self.others():
            self.r.e2en[j - 1, i - 1] += e2[j - 1, i - 1]

    # classes (-1') / (+1'): vmupE :5869 / vpupE :5437 ---------------------
    def _pupE(self, cls, minus):
        nc, na, norb, i, M = self.nc, self.na, self.norb, self.i, self.M
        A = self.acc
        inp = self.inp
        tag = "IP" if minus else "EA"
        am = getattr(inp, "amat" + tag)[i - 1]
        bm = getattr(inp, "bmat" + tag)[i - 1]
        cm = getattr(inp, "cmat" + tag)[i - 1]
        dm = getattr(inp, "dmat" + tag)[i - 1]
        v0 = nc + na
        if minus:
            ext = list(range(v0 + 1, norb + 1))

            def heffd(a):  # heffd(indice(a, r)) of vmupE
                def f(r_):
                    v = self.hp(a + nc, r_)
                    for j in range(1, nc + 1):
                        v += 2.0 * self.ct(a + nc, r_, j, j) - self.ct(a + nc, j, r_, j)
                    for b in range(1, na + 1):
                        v -= self.ct(a + nc, b + nc, b + nc, r_)
                    return v
                return f

            dint = lambda x, a, b, c: self.ct(a + nc, b + nc, c + nc, x)
            rho11 = lambda O, a, ap, lt: (O.D1(a, ap) if lt else O.D1(ap, a))
            W2 = lambda O, cp, ap, bp, a: O.ee2(cp, ap, bp, a)
            W2b = lambda O, a, bp, ap, cp: O.ee2(a, bp, ap, cp)
            W3 = lambda O, *x: O.eee2(*x)
            rho1 = lambda a, ap: A.D1(ap, a)
        else:
            ext = list(range(1, nc + 1))

            def heffd(a):  # heffd(indice(a, i)) of vpupE
                def f(ci):
                    v = self.hp(ci, a + nc)
                    for j in range(1, nc + 1):
                        v += 2.0 * self.ct(j, j, ci, a + nc) - self.ct(j, ci, j, a + nc)
                    return v
                return f

            dint = lambda x, a, b, c: self.ct(a + nc, b + nc, c + nc, x)
            rho11 = lambda O, a, ap, lt: -(O.D1(ap, a) if lt else O.D1(a, ap))
            W2 = lambda O, cp, ap, bp, a: O.ee2tr(cp, ap, bp, a)
            W2b = lambda O, a, bp, ap, cp: O.ee2tl(a, bp, ap, cp)
            W3 = lambda O, *x: O.eee2t(*x)
            rho1 = lambda a, ap: (2.0 if a == ap else 0.0) - A.D1(ap, a)
        hcache = {}
        for x in ext:
            hv = {a: heffd(a)(x) for a in range(1, na + 1)}
            hcache[x] = hv
            d = {(a, b, c): dint(x, a, b, c) for a in range(1, na + 1) for b in range(1, na + 1)
                 for c in range(1, na + 1)}
            dumm = {j: 0.0 for j in range(1, M + 1)}
            dumk = 0.0
            for ia in range(1, na + 1):
                for iap in range(1, na + 1):
                    dumm[i] += hv[iap] * rho1(ia, iap) * hv[ia]
                    dumk += hv[iap] * dm[iap - 1, ia - 1] * hv[ia]
                    for j in self.others():
                        dumm[j] += hv[iap] * rho11(self.off(j), ia, iap, j < i) * hv[ia]
                    for ibp in range(1, na + 1):
                        for icp in range(1, na + 1):
                            cint = d[(iap, icp, ibp)]
                            dumm[i] += 2.0 * cint * W2(A, icp, iap, ibp, ia) * hv[ia]
                            dumk += cint * (bm[iap - 1, ibp - 1, icp - 1, ia - 1] + cm[ia - 1, iap - 1, ibp - 1, icp - 1]) * hv[ia]
                            for j in self.others():
                                O = self.off(j)
                                dumm[j] += cint * (W2(O, icp, iap, ibp, ia) + W2b(O, ia, ibp, iap, icp)) * hv[ia]
                            for ib in range(1, na + 1):
                                for ic in range(1, na + 1):
                                    cint2 = d[(ia, ic, ib)]
                                    dumm[i] += cint * W3(A, icp, iap, ibp, ib, ia, ic) * cint2
                                    dumk += cint * am[iap - 1, ibp - 1, icp - 1, ia - 1, ib - 1, ic - 1] * cint2
                                    for j in self.others():
                                        O = self.off(j)
                                        if j < i:
                                            v = W3(O, icp, iap, ibp, ib, ia, ic)
                                        else:
                                            v = W3(O, ic, ia, ib, ibp, iap, icp)
                                        dumm[j] += cint * v * cint2
            den = 0.0
            if dumm[i] != 0.0:
                if minus:
                    den = -dumk / dumm[i] - self.eps(x)
                else:
                    den = self.eps(x) - dumk / dumm[i]
                co = dumm[i] / den
                self.sc_add(cls, co, co / den)
            for j in self.others():
                if den != 0.0:
                    self.r.e2mp[j - 1, i - 1] += dumm[j] / den
        # PC
        n3 = na ** 3
        S = np.zeros((n3, n3))
        K = np.zeros((n3, n3))
        abc = 0
        for a in range(1, na + 1):
            for b in range(1, na + 1):
                for c in range(1, na + 1):
                    abcp = 0
                    for ap in range(1, na + 1):
                        for bp in range(1, na + 1):
                            for cp in range(1, na + 1):
                                K[abc, abcp] = am[ap - 1, bp - 1, cp - 1, a - 1, b - 1, c - 1]
                                S[abc, abcp] = W3(A, cp, ap, bp, b, a, c)
                                abcp += 1
                    abc += 1
        C, w, nnew = pc_transform(S, K, self.thr)
        coefT = C.T
        s = np.zeros((n3, n3, M))   # s(mu, abc, j)
        sp = np.zeros((n3, na, M))  # sp(mu, a, j)
        for ia in range(1, na + 1):
            for ib in range(1, na + 1):
                for ic in range(1, na + 1):
                    for iap in range(1, na + 1):
                        for ibp in range(1, na + 1):
                            for icp in range(1, na + 1):
                                iabc = ic + na * ((ib - 1) + na * (ia - 1)) - 1
                                iabcp = icp + na * ((ibp - 1) + na * (iap - 1)) - 1
                                zc = ib == 1 and ic == 1
                                s[:, iabc, i - 1] += W3(A, icp, iap, ibp, ib, ia, ic) * coefT[:, iabcp]
                                if zc:
                                    sp[:, ia - 1, i - 1] += W2(A, icp, iap, ibp, ia) * coefT[:, iabcp]
                                for j in self.others():
                                    O = self.off(j)
                                    if j < i:
                                        s[:, iabc, j - 1] += W3(O, ic, ia, ib, ibp, iap, icp) * coefT[:, iabcp]
                                        if zc:
                                            sp[:, ia - 1, j - 1] += W2b(O, ia, ibp, iap, icp) * coefT[:, iabcp]
                                    else:
                                        s[:, iabc, j - 1] += W3(O, icp, iap, ibp, ib, ia, ic) * coefT[:, iabcp]
                                        if zc:
                                            sp[:, ia - 1, j - 1] += W2(O, icp, iap, ibp, ia) * coefT[:, iabcp]
        e2 = np.zeros((M, M))
        psi2 = 0.0
        for x in ext:
            hv = hcache[x]
            for mu in range(n3):
                rm = np.zeros(M)
                iabc = 0
                for ia in range(1, na + 1):
                    rm += hv[ia] * sp[mu, ia - 1, :]
                    for ib in range(1, na + 1):
                        for ic in range(1, na + 1):
                            rm += dint(x, ia, ic, ib) * s[mu, iabc, :]
                            iabc += 1
                deno = w[mu] + (self.eps(x) if minus else -self.eps(x))
                co = rm[i - 1] / deno
                e2[i - 1, i - 1] -= rm[i - 1] * co
                psi2 += co ** 2
                for j in self.others():
                    e2[j - 1, i - 1] -= rm[i - 1] * (rm[j - 1] / deno)
        self.r.e2enp[cls, i - 1] = e2[i - 1, i - 1]
        self.r.psienep[cls, i - 1] = psi2
        self.r.psien[i - 1] += psi2
        self.r.e2en[i - 1, i - 1] += e2[i - 1, i - 1]
        for j in self.others():
            self.r.e2en[j - 1, i - 1] += e2[j - 1, i - 1]

    def vmupE(self):
        self._pupE(6, True)

    def vpupE(self):
        self._pupE(5, False)
