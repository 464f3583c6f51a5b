"""Independent brute-force model of the cip / cipsym perturber set (test only).

This enumerates, for every generator k of S, the single and double
excitations of k as plain occupation bitstrings and applies the rules that
the reference's loop nest (cip/pertu.f, igene.f, pert1.f, diexcit.f) realises,
written as set rules instead of list edits:

* generators: ygen(k) and not ysaut(k)  (pertu.f:111-116, diexcit.f:218-221);
* excitation classes by rank change D = rank(I) - rank(k):
    D = +2 come from diexcit (closed-shell doubles on top of k),
    D = +1 .. -2 from igene, skipped by the S-content flags
    yd (HF in S), ym (a single in S), yf (a double or single in S)
    exactly where igene.f:34-35, 89-90, 199-200, 296-298 return early;
* rank-1 perturbers (when ym) and HF (when not yd) come from pertu with no
  owner (pertu.f:62-108);
* owner rule: I is dropped at k if a ygen determinant j < k has degree <= 2
  with I (pert1.f:104-118, diexcit.f:246-259);
* I is dropped if it equals a determinant j >= k of S (pert1.f:139,
  diexcit.f:279); only j >= k enter <I|H|Psi> (pert1.f:129-144);
* diexcit on a generator without a spin-flip partner (yef false) only takes
  the "unflipped" spin patterns and doubles their weight
  (diexcit.f:183-194, 224, 304-316).

Matrix elements use canonical (alpha string then beta string) phases; the
coefficients read from unit 59 are converted with the excitation-list phase
of each S determinant, so <I|H|Psi>^2 is convention independent.
"""
from __future__ import annotations

import itertools
import os
import struct
from dataclasses import dataclass
from typing import Dict, List, Tuple

import numpy as np

from cipsi_gb300 import synth


@dataclass
class Inputs:
    norb: int
    nocc: int
    nsym: int
    itsym: np.ndarray      # 1-based orbital irreps, index 1..norb
    its: np.ndarray        # product table, 1-based
    F: np.ndarray          # packed lower triangle, 1-based index num(i)+j
    J: np.ndarray
    K: np.ndarray
    ij0: np.ndarray        # (norb+1, norb+1), ij0[i, j]
    ntttt: np.ndarray
    bijkl: np.ndarray      # float32, 1-based
    escf: float
    S: List[Tuple[Tuple[int, ...], Tuple[int, ...]]]
    ysaut: List[bool]
    nesp: List[int]
    yef: List[bool]
    C: np.ndarray          # (ncf, metat) reference phase
    E: np.ndarray          # relative to escf
    tau: float
    test: float
    ityper: int
    iselec: int


def read_inputs(workdir: str) -> Inputs:
    recs = synth.read_records(os.path.join(workdir, "ijkl"))
    hdr = recs[0]
    nsym, norb, noc, ntrans = struct.unpack_from("<4i", hdr, 0)
    itsym = np.zeros(norb + 1, dtype=np.int64)
    itsym[1:] = np.frombuffer(hdr, dtype="<i4", count=norb, offset=16)
    its = np.zeros((nsym + 1, nsym + 1), dtype=np.int64)
    its[1:, 1:] = np.frombuffer(recs[1], dtype="<i4").reshape(nsym, nsym).T
    nter = norb * (norb + 1) // 2
    J = np.concatenate([[0.0], np.frombuffer(recs[3], dtype="<f8")])
    K = np.concatenate([[0.0], np.frombuffer(recs[4], dtype="<f8")])
    F = np.concatenate([[0.0], np.frombuffer(recs[5], dtype="<f8")]).copy()
    F[1:][np.abs(F[1:]) < 1e-10] = 0.0
    ij0 = np.zeros((norb + 1, norb + 1), dtype=np.int64)
    ij0[1:, 1:] = np.frombuffer(recs[6], dtype="<i2").reshape(norb, norb).T
    ninte = struct.unpack_from("<i", recs[7], 0)[0]
    ntttt = np.zeros(nsym + 1, dtype=np.int64)
    ntttt[1:] = np.frombuffer(recs[7], dtype="<i4", offset=4, count=nsym)
    vals = np.concatenate([np.frombuffer(r, dtype="<f8") for r in recs[8:]])
    bijkl = np.concatenate([[np.float32(0)], vals.astype(np.float32)])
    er = synth.read_records(os.path.join(workdir, "ener"))
    escf = struct.unpack_from("<d", er[0], 44)[0]
    # S from unit 60 with the spin-flip closure of deter.f:478-567
    dets_by_rank: Dict[int, List] = {}
    hf = False
    for r in synth.read_records(os.path.join(workdir, "det")):
        m, n = struct.unpack_from("<ii", r, 0)
        idet = np.frombuffer(r, dtype="<i4", count=m, offset=8)
        nex = np.frombuffer(r, dtype="<i4", count=n, offset=8 + 4 * m)
        pos = 0
        for nec in nex:
            h = tuple(int(idet[pos + 2 * i]) for i in range(nec))
            p = tuple(int(idet[pos + 2 * i + 1]) for i in range(nec))
            pos += 2 * nec
            if nec == 0:
                hf = True
            else:
                dets_by_rank.setdefault(int(nec), []).append((h, p))
    S, ysaut, nesp, yef = [], [], [], []
    seen = set()
    if hf:
        S.append(((), ()))
        ysaut.append(False)
        nesp.append(0)
        yef.append(False)
        seen.add(((), ()))
    for nec in sorted(dets_by_rank):
        for h, p in dets_by_rank[nec]:
            key = (tuple(sorted(h)), tuple(sorted(p)))
            if key in seen:
                continue
            seen.add(key)
            S.append(key)
            ysaut.append(False)
            nesp.append(0)
            yef.append(False)
            fh, fp = synth.flip_lists(key[0], key[1], norb)
            fkey = (tuple(fh), tuple(fp))
            if fkey not in seen:
                seen.add(fkey)
                S.append(fkey)
                ysaut.append(True)
                nesp.append(0)
                yef.append(True)
                nesp[-2] = 1
                yef[-2] = True
    b = synth.read_records(os.path.join(workdir, "bdvec"))[0]
    ncf, metat = struct.unpack_from("<ii", b, 0)
    assert ncf == len(S), (ncf, len(S))
    C = np.frombuffer(b, dtype="<f8", count=ncf * metat, offset=8).reshape(metat, ncf).T.copy()
    E = np.frombuffer(b, dtype="<f8", count=metat, offset=8 + 8 * ncf * metat) - escf
    txt = open(os.path.join(workdir, "cip.in")).read().lower()

    def nl(key, default):
        import re
        mm = re.search(r"[\s,]" + key + r"\s*=\s*([^,\s]+)", txt)
        return mm.group(1) if mm else default

    tau = float(nl("tau", "1e-4").replace("d", "e"))
    test = float(nl("test", "0.5").replace("d", "e"))
    ityper = int(nl("ityper", "1"))
    iselec = int(nl("iselec", "1"))
    return Inputs(norb, noc, nsym, itsym, its, F, J, K, ij0, ntttt, bijkl, escf, S, ysaut, nesp,
                  yef, C, E, tau, test, ityper, iselec)


# ---------------------------------------------------------------- physics


class Model:
    def __init__(self, inp: Inputs):
        self.inp = inp
        n = inp.norb
        self.n = n
        self.hf = ((1 << inp.nocc) - 1) | (((1 << inp.nocc) - 1) << n)
        self.bits = [self.to_bits(h, p) for h, p in inp.S]
        self.index = {b: i for i, b in enumerate(self.bits)}
        self.sigma = np.array([synth.cip_phase(h, p, n, inp.nocc) for h, p in inp.S], dtype=float)
        self.Ccan = inp.C * self.sigma[:, None]
        self.ygen = [True] * len(inp.S)
        fd = np.zeros(2 * n + 1)
        for i in range(1, n + 1):
            fd[i] = fd[i + n] = inp.F[i * (i + 1) // 2]
        self.fdiag = fd

    def to_bits(self, holes, parts) -> int:
        x = self.hf
        for so in holes:
            x &= ~(1 << (so - 1))
        for so in parts:
            x |= 1 << (so - 1)
        return x

    def lists(self, x: int):
        holes = [so for so in range(1, 2 * self.n + 1) if (self.hf >> (so - 1) & 1) and not (x >> (so - 1) & 1)]
        parts = [so for so in range(1, 2 * self.n + 1) if not (self.hf >> (so - 1) & 1) and (x >> (so - 1) & 1)]
        return holes, parts

    def rank(self, x: int) -> int:
        return bin(self.hf & ~x).count("1")

    def ai(self, i, j, k, l):
        inp = self.inp
        ij0 = inp.ij0
        if j >= i:
            ij = ij0[i, j]
            isy = 1 if i == j else ij0[j, i]
        else:
            ij = ij0[j, i]
            isy = ij0[i, j]
        if l >= k:
            kl = ij0[k, l]
            jsy = 1 if k == l else ij0[l, k]
        else:
            kl = ij0[l, k]
            jsy = ij0[k, l]
        if isy != jsy:
            return 0.0
        lo, hi = (ij, kl) if ij <= kl else (kl, ij)
        return float(inp.bijkl[lo + (hi * hi - hi) // 2 + inp.ntttt[isy] - 1])

    def orb(self, so):
        return (so - 1) % self.n + 1

    def spin(self, so):
        return (so - 1) // self.n

    def phase(self, bits: int, p: int, q: int) -> int:
        lo, hi = (p, q) if p < q else (q, p)
        mask = ((1 << (hi - 1)) - 1) & ~((1 << lo) - 1)
        return -1 if bin(bits & mask).count("1") & 1 else 1

    def hmat(self, xi: int, xj: int) -> float:
        """<I|H|J> (canonical phases), spin orbitals 1-based; degree 1 or 2."""
        d = xi ^ xj
        rem = d & xj  # occupied in J only
        add = d & xi  # occupied in I only
        nrem = bin(rem).count("1")
        sos_r = [so for so in range(1, 2 * self.n + 1) if rem >> (so - 1) & 1]
        sos_a = [so for so in range(1, 2 * self.n + 1) if add >> (so - 1) & 1]
        if nrem == 1:
            p, q = sos_r[0], sos_a[0]
            sign = self.phase(xj, p, q)
            n1, n2 = self.orb(p), self.orb(q)
            s1 = self.spin(p)
            lo, hi = min(n1, n2), max(n1, n2)
            val = self.inp.F[hi * (hi - 1) // 2 + lo]
            holes, parts = self.lists(xi)
            for t in holes:
                nt = self.orb(t)
                val -= self.ai(n1, n2, nt, nt)
                if self.spin(t) == s1:
                    val += self.ai(n1, nt, n2, nt)
            for pp in parts:
                npp = self.orb(pp)
                val += self.ai(n1, n2, npp, npp)
                if self.spin(pp) == s1:
                    val -= self.ai(n1, npp, n2, npp)
            return sign * val
        if nrem == 2:
            p1, p2 = sos_r
            q1, q2 = sos_a
            s1 = self.phase(xj, p1, q1)
            mid = (xj & ~(1 << (p1 - 1))) | (1 << (q1 - 1))
            s2 = self.phase(mid, p2, q2)
            o = self.orb
            val = 0.0
            if self.spin(p1) == self.spin(q1):
                val += self.ai(o(p1), o(q1), o(p2), o(q2))
            if self.spin(p1) == self.spin(q2):
                val -= self.ai(o(p1), o(q2), o(p2), o(q1))
            return s1 * s2 * val
        raise ValueError("degree must be 1 or 2")

    def hmp_hdig(self, x: int):
        inp = self.inp
        holes, parts = self.lists(x)
        fm = self.fdiag  # faifoc with closed-shell tocom: fmpb = F_pp
        hmp = sum(fm[p] for p in parts) - sum(fm[h] for h in holes)
        num = lambda i: i * (i - 1) // 2  # noqa: E731

        def jk(a, b):
            oa, ob = self.orb(a), self.orb(b)
            lo, hi = min(oa, ob), max(oa, ob)
            idx = num(hi) + lo
            v = inp.J[idx]
            if self.spin(a) == self.spin(b):
                v -= inp.K[idx]
            return v
        e = sum(self.fdiag[p] for p in parts) - sum(self.fdiag[h] for h in holes)
        for a, b in itertools.combinations(holes, 2):
            e += jk(a, b)
        for a, b in itertools.combinations(parts, 2):
            e += jk(a, b)
        for a in holes:
            for b in parts:
                e -= jk(a, b)
        return hmp, e


def degree(x: int, y: int) -> int:
    return bin(x ^ y).count("1") // 2


def enumerate_semantic(inp: Inputs, model: Model):
    """List of (src, k(1-based, 0=pertu), bits, nmul, fmul, bcalc[metat])."""
    n = inp.norb
    ncf = len(inp.S)
    ranks = [len(h) for h, _ in inp.S]
    yd = 0 in ranks
    ym = 1 in ranks
    yf = (2 in ranks) or ym
    isym = 1
    hf = model.hf
    its = inp.its
    sym = lambda so: int(inp.itsym[model.orb(so)])  # noqa: E731
    out = []

    def process(src, kk, x, rule):
        # owner
        for j in range(1, kk):
            if model.ygen[j - 1] and degree(x, model.bits[j - 1]) <= 2:
                return
        start = max(kk, 1)
        inter = []
        for j in range(start, ncf + 1):
            d = degree(x, model.bits[j - 1])
            if d == 0:
                return
            if d <= 2:
                inter.append(j)
        if not inter:
            return
        hv = {j: model.hmat(x, model.bits[j - 1]) for j in inter}
        nespf = inp.nesp[kk - 1] if kk >= 1 else 0
        lesp = sum(1 for j in inter if kk < j <= kk + nespf) if kk >= 1 else 0
        if rule == "diexcit":
            inter = [j for j in inter if hv[j] != 0.0]
            if not inter:
                return
        if rule == "pert1":
            if nespf:
                fmul = (nespf + 1) / (lesp + 1) - 1.0
            else:
                fmul = 0.0
        else:
            ysyspi = rule_ysyspi[0]
            yefsk = inp.yef[kk - 1]
            if (yefsk or ysyspi) and not yefsk:
                nespf = 2 * nespf + 1
            fmul = (nespf + 1) / (lesp + 1) - 1.0
        bcalc = np.array([sum(hv[j] * model.Ccan[j - 1, m] for j in inter) for m in range(inp.C.shape[1])])
        out.append((src, kk, x, int(fmul), fmul, bcalc))

    rule_ysyspi = [False]
    # pertu kk = 0
    if yf and not yd and isym == 1:
        process(0, 0, hf, "pert1")
    if yf and ym:
        for s in range(2):
            for o in range(1, inp.nocc + 1):
                for v in range(inp.nocc + 1, n + 1):
                    if its[inp.itsym[o], inp.itsym[v]] != isym:
                        continue
                    so, sv = o + s * n, v + s * n
                    x = (hf & ~(1 << (so - 1))) | (1 << (sv - 1))
                    process(0, 0, x, "pert1")
    for k in range(1, ncf + 1):
        if not model.ygen[k - 1] or inp.ysaut[k - 1]:
            continue
        xk = model.bits[k - 1]
        nec = ranks[k - 1]
        allowed = set()
        if not ((nec == 0 and ym) or (nec == 1 and yd)):
            allowed.add(1)
            stop = nec < 1 or (ym and nec == 1) or (nec == 2 and yd)
            if not stop:
                allowed.add(0)
                if not ((nec == 3 and yd) or (nec == 2 and ym)):
                    allowed.add(-1)
                    if not ((nec == 2 and (yd or yf)) or (nec == 3 and ym) or (nec == 4 and yd)):
                        allowed.add(-2)
        occ = [so for so in range(1, 2 * n + 1) if xk >> (so - 1) & 1]
        vir = [so for so in range(1, 2 * n + 1) if not (xk >> (so - 1) & 1)]
        # singles
        for o in occ:
            for v in vir:
                if model.spin(o) != model.spin(v):
                    continue
                if its[sym(o), sym(v)] != 1:
                    continue
                x = (xk & ~(1 << (o - 1))) | (1 << (v - 1))
                D = model.rank(x) - nec
                if D in allowed:
                    process(1, k, x, "pert1")
        # doubles
        for o1, o2 in itertools.combinations(occ, 2):
            for v1, v2 in itertools.combinations(vir, 2):
                if model.spin(o1) + model.spin(o2) != model.spin(v1) + model.spin(v2):
                    continue
                g = its[its[sym(o1), sym(o2)], its[sym(v1), sym(v2)]]
                if g != 1:
                    continue
                x = (xk & ~(1 << (o1 - 1)) & ~(1 << (o2 - 1))) | (1 << (v1 - 1)) | (1 << (v2 - 1))
                D = model.rank(x) - nec
                if D == 2:
                    # diexcit pattern rules
                    ho = sorted([o1, o2])
                    pv = sorted([v1, v2])
                    spins_h = [model.spin(a) for a in ho]
                    spins_p = [model.spin(a) for a in pv]
                    oh = [model.orb(a) for a in ho]
                    op = [model.orb(a) for a in pv]
                    if spins_h[0] != spins_h[1]:
                        a_orb = oh[0] if spins_h[0] == 0 else oh[1]   # alpha hole orbital
                        b_orb = oh[1] if spins_h[0] == 0 else oh[0]
                        c_orb = op[0] if spins_p[0] == 0 else op[1]   # alpha particle orbital
                        d_orb = op[1] if spins_p[0] == 0 else op[0]
                        ysyspi = not (a_orb == b_orb and c_orb == d_orb)
                        unflipped = (a_orb < b_orb) or (a_orb == b_orb and c_orb <= d_orb)
                    else:
                        ysyspi = True
                        unflipped = spins_h[0] == 0
                    if not inp.yef[k - 1] and not unflipped:
                        continue
                    rule_ysyspi[0] = ysyspi
                    process(2, k, x, "diexcit")
                elif D in allowed:
                    process(1, k, x, "pert1")
    return out


def read_candlog(path: str, metat: int):
    rec = 4 * 4 + 32 * 4 + 16 + 8 * metat
    data = open(path, "rb").read()
    out = []
    for off in range(0, len(data), rec):
        src, kk, nec, nmul = struct.unpack_from("<4i", data, off)
        hp = struct.unpack_from("<32i", data, off + 16)
        xam, fmul = struct.unpack_from("<2d", data, off + 16 + 128)
        him = struct.unpack_from(f"<{metat}d", data, off + 16 + 128 + 16)
        holes = [x for x in hp[:nec]]
        parts = [x for x in hp[16:16 + nec]]
        out.append((src, kk, tuple(holes), tuple(parts), nmul, fmul, xam, np.array(him)))
    return out
