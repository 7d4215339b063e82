"""Extended-precision evaluation of one PC class (test infrastructure only).

The (+2) partially contracted energy of state s (src/qdnevpt.F:2804-2935
e2p2cont, :2936-3010 e2p2contp) is, per inactive pair, a sum over the PC
basis: -sum_mu a_mu^2 / (w_mu - e_i - e_j), with w, C the eigenpairs of the
pencil (K, S) after the metric transformation and a = C^T y, y = D dint.
When every metric eigenvalue is above the threshold (the reference keeps all
of them), C (W - sigma)^-1 C^T = (K - sigma S)^-1, so the class energy is

    E = - sum_pairs y^T (K - sigma S)^-1 y

This module evaluates that sum by Gaussian elimination with partial pivoting
in numpy ``longdouble`` (64-bit significand on x86-64, 113-bit on aarch64),
on the same FP64 inputs the FP64 evaluations use.  It gives the value that
any FP64 evaluation of the class approximates, so the FP64 evaluations (the
oracle's eigenpair route under several LAPACK drivers, the GPU) can be
placed against it.

    python -m oracle.extended_pc --config cas16_qd4 [--states 0 1] [--gpu BENCH_JSON] [--inputs NPZ]

prints one JSON line per state.  Uses the oracle's stage 1 (the Koopmans
builders only; bamat is not needed for this class) and the oracle's
state preparation (canonical orbitals, transformed integrals).  With
--inputs (the file of ``bench.py --parity --parity-dump``) the class's
Koopmans matrices, the orbital energies and the compared GPU energies are
the GPU's own, so every evaluation sees the GPU's inputs (the transformed
integrals are the oracle's, equal to the GPU's up to rounding).
"""
import argparse
import json
import sys
import time

import numpy as np
import scipy.linalg as sla

from oracle import oracle as orc
from oracle import qdnevpt_oracle as q


def solve_batched(A, b):
    """x with A[k] x[k] = b[k] for a batch of dense systems, by Gaussian
    elimination with partial pivoting in the dtype of A (no LAPACK)."""
    A = np.array(A, copy=True)
    b = np.array(b, copy=True)
    nb, n, _ = A.shape
    ar = np.arange(nb)
    for k in range(n):
        p = k + np.argmax(np.abs(A[:, k:, k]), axis=1)
        rk, rp = A[ar, k, :].copy(), A[ar, p, :].copy()
        A[ar, k, :], A[ar, p, :] = rp, rk
        bk, bp = b[ar, k].copy(), b[ar, p].copy()
        b[ar, k], b[ar, p] = bp, bk
        if k + 1 < n:
            l = A[:, k + 1:, k] / A[:, k, k][:, None]
            A[:, k + 1:, k:] -= l[:, :, None] * A[:, None, k, k:]
            b[:, k + 1:] -= l * b[:, k][:, None]
    x = np.zeros_like(b)
    for k in range(n - 1, -1, -1):
        s = np.einsum("bj,bj->b", A[:, k, k + 1:], x[:, k + 1:]) if k + 1 < n else 0.0
        x[:, k] = (b[:, k] - s) / A[:, k, k]
    return x


def plus2_pc_energy(inp, st, s, dtype=np.longdouble, chunk=64, lapack=False):
    """-sum y^T (K - sigma S)^-1 y over the (+2) PC labels of state s in
    ``dtype``: part (a), inactive pairs i < j on the n^2 metric (fillcm2),
    and part (b), i = j on the n(n+1)/2 metric (fillcm2p); the same operands
    as q._v2mod.  Raises if a metric eigenvalue is below the threshold (the
    identity needs the full PC basis)."""
    na, nc = st.na, st.nc
    n2 = na * na
    daat = inp.hrdm[s]
    gk = inp.eako2[s]
    T = st.eri(st.core, st.act, st.core, st.act)
    eps = st.eps
    fro = np.zeros(nc, bool)
    for k in inp.frozen:
        if k < nc:
            fro[k] = True
    thr = inp.thr_lindep

    def part(S, K, D, labels):
        if np.linalg.eigvalsh(S).min() < thr:
            raise ValueError("a metric eigenvalue is below the threshold")
        Sx, Kx, Dx = S.astype(dtype), K.astype(dtype), D.astype(dtype)
        tot = dtype(0)
        for c0 in range(0, len(labels), chunk):
            lab = labels[c0:c0 + chunk]
            sig = np.array([x[0] for x in lab], dtype=dtype)
            dint = np.stack([x[1] for x in lab]).astype(dtype)
            y = dint @ Dx.T
            A = Kx[None, :, :] - sig[:, None, None] * Sx[None, :, :]
            x = (np.stack([sla.solve(A[k], y[k]) for k in range(len(lab))]) if lapack
                 else solve_batched(A, y))
            tot += np.sum(y * x)
        return -tot

    # (a) i < j
    S = q.upper_sym(daat.reshape(n2, n2))
    K = q.upper_sym(gk.reshape(n2, n2))
    la = [(np.longdouble(eps[i]) + np.longdouble(eps[j]), T[i, :, j, :].T.reshape(n2))
          for i in range(nc) if not fro[i] for j in range(i + 1, nc) if not fro[j]]
    ea = part(S, K, daat.reshape(n2, n2), la)
    # (b) i = j
    iu, ju = np.triu_indices(na)
    Sfull = daat + np.transpose(daat, (0, 1, 3, 2))
    Kfull = gk + np.transpose(gk, (0, 1, 3, 2))
    Sp = Sfull[iu, ju][:, iu, ju]
    Kp = Kfull[iu, ju][:, iu, ju]
    lb = []
    for i in range(nc):
        if fro[i]:
            continue
        tr = T[i, :, i, :]
        lb.append((2 * np.longdouble(eps[i]), np.where(iu == ju, tr[ju, iu], 2.0 * tr[ju, iu])))
    eb = part(q.upper_sym(Sp), q.upper_sym(Kp), 0.5 * Sp, lb)
    return ea + eb


def sensitivity(inp, st, s, draws=2, seed=1):
    """Largest change of the FP64 resolvent value of the (+2) class over
    ``draws`` random perturbations: one relative rounding (2^-52 xi, xi ~
    N(0,1)) of every orbital energy / 2-EA element / 2-HRDM element, and
    2^-52 max|2-EA| xi added to every 2-EA element."""
    rng = np.random.default_rng(seed)
    e0 = plus2_pc_energy(inp, st, s, np.float64, lapack=True)
    hr, ea, eps = inp.hrdm[s], inp.eako2[s], st.eps
    u = 2.0 ** -52
    cases = {
        "eps_one_rounding": lambda: (hr, ea, eps * (1 + u * rng.standard_normal(eps.shape))),
        "eako2_one_rounding": lambda: (hr, ea * (1 + u * rng.standard_normal(ea.shape)), eps),
        "hrdm_one_rounding": lambda: (hr * (1 + u * rng.standard_normal(hr.shape)), ea, eps),
        "eako2_one_rounding_of_max": lambda: (hr, ea + u * np.abs(ea).max() * rng.standard_normal(ea.shape), eps),
    }
    out = {}
    for name, make in cases.items():
        worst = 0.0
        for _ in range(draws):
            h2, e2, ep = make()
            inp.hrdm[s], inp.eako2[s], st.eps = h2, e2, ep
            worst = max(worst, abs(plus2_pc_energy(inp, st, s, np.float64, lapack=True) - e0))
        out[name] = worst
    inp.hrdm[s], inp.eako2[s], st.eps = hr, ea, eps
    return out


def stage2_inputs(p):
    """Stage-2 inputs from the oracle's stage 1 without bamat: the datasets
    the (+2) class reads (2-HRDM, 2-EAKO) are real, the others placeholders."""
    M, n, nc = p.metat, p.nact, p.ncore
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, n, nc, p.norb)
    f = np.zeros(p.norb * (p.norb + 1) // 2)
    o = orc.koop_matrices_ctl(M, n, nc, atwo, p.daaa, p.taa, p.dal, f, aj)
    names = {"ipko1": "1-IPKO", "eako1": "1-EAKO", "hrdm2": "2-HRDM", "ipko2": "2-IPKO", "eako2": "2-EAKO"}
    koop = {names.get(k, k): v for k, v in o.items()}
    for k in ("amatIP", "amatEA", "bmatIP", "bmatEA", "cmatIP", "cmatEA", "dmatIP", "dmatEA"):
        koop[k] = np.zeros((M, 1))
    # the class's QD couplings read the transition RDMs; the diagonal energy
    # evaluated here does not, so zero stand-ins keep the class routine whole
    npair = M * (M - 1) // 2
    tr = ([np.zeros((n, n))] * npair, [np.zeros((n, n, n, n))] * npair, [None] * npair)
    return q.inputs_from(p, koop, transition=tr if M > 1 else None)


def main(argv=None):
    from nevpt2_gb300 import synth

    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="cas16_qd4")
    ap.add_argument("--states", type=int, nargs="*")
    ap.add_argument("--gpu", help="a bench JSON line whose energies.per_class_pc holds the GPU's values")
    ap.add_argument("--inputs", help="npz from bench.py --parity --parity-dump: the GPU's inputs and energies")
    ap.add_argument("--sensitivity", action="store_true",
                    help="also the change of the FP64 resolvent value under one relative rounding of the orbital "
                         "energies, of the 2-EA / 2-HRDM elements, and one rounding of the largest 2-EA element")
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    p = synth.config_problem(a.config, with_ro4=False, with_trdm=False)
    inp = stage2_inputs(p)
    t_in = time.perf_counter() - t0
    gpu = None
    if a.gpu:
        for line in open(a.gpu):
            if line.startswith("{"):
                gpu = json.loads(line)["energies"]["per_class_pc"]
    dump = None
    if a.inputs:
        dump = np.load(a.inputs)
        inp.hrdm = [dump["hrdm"][s] for s in range(p.metat)]
        inp.eako2 = [dump["eako2"][s] for s in range(p.metat)]
        gpu = [list(dump["e2enp"][:, s]) for s in range(p.metat)]
    B = q.dense_B(inp.chol, inp.norb)
    h = q.unpack_tri(inp.oneint, inp.norb)
    states = a.states if a.states else range(p.metat)
    for s in states:
        st = q._State(inp, s, B, h)
        row = {"config": a.config, "state": s, "class": "(+2)", "inputs_s": round(t_in, 1),
               "inputs": "gpu" if dump is not None else "oracle stage 1"}
        if dump is not None:
            row["eps_gpu_minus_oracle_max"] = float(np.abs(dump["epsnew"][:, s] - st.eps).max())
            st.eps = np.array(dump["epsnew"][:, s])
        orig = q.dsyev_u
        for drv in ("evr", "evd", "ev"):
            q.dsyev_u = lambda A, d=drv: sla.eigh(q.upper_sym(A), lower=False, driver=d)
            r = q.Stage2Result(*(np.zeros((8, p.metat)) for _ in range(4)), np.zeros((p.metat, p.metat)),
                               np.zeros((p.metat, p.metat)), np.zeros(p.metat), np.zeros(p.metat), {},
                               np.zeros((p.norb, p.metat)))
            q._v2mod(inp, st, s, r, np.zeros(p.norb, bool), True)
            row[f"oracle_{drv}"] = float(r.e2enp[3, s])
        q.dsyev_u = orig
        t1 = time.perf_counter()
        row["resolvent_fp64"] = float(plus2_pc_energy(inp, st, s, np.float64))
        ext = plus2_pc_energy(inp, st, s, np.longdouble)
        row["extended"] = float(ext)
        row["extended_minus_fp64_resolvent"] = float(ext - np.longdouble(row["resolvent_fp64"]))
        for k in ("oracle_evr", "oracle_evd", "oracle_ev", "resolvent_fp64"):
            row[f"{k}_err"] = float(np.longdouble(row[k]) - ext)
        if gpu is not None:
            row["gpu"] = gpu[s][3]
            row["gpu_err"] = float(np.longdouble(gpu[s][3]) - ext)
        if a.sensitivity:
            row["sensitivity_eh"] = sensitivity(inp, st, s)
        row["longdouble_eps"] = float(np.finfo(np.longdouble).eps)
        row["extended_s"] = round(time.perf_counter() - t1, 1)
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    sys.exit(main())
