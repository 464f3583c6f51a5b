"""Seeded synthetic inputs for the CIPSI perturbation/selection step.

Writes a work directory in the reference's on-disk formats so that both the
GPU drop-in and the reference executable could run on it:

  ijkl   unit 40, the `fock` "new" layout (CIPSI_sources/fock/fock.f:25-146,
         CIPSI_sources/fock/wijkl_new.f:1-165): header, product table, bare h,
         J, K, closed-shell Fock F, ij0 pair map, ninte/ntttt, packed (pq|rs)
         in records of 8192 reals.
  ener   unit 33, "energie du determinant de reference" (fock/stkener.f).
  det    unit 60, the reference space S as cip's selection records
         (cip/pie.f record layout m,n,idet(m),nex(n),v(n)).
  bdvec  unit 59, ncf, metat, c(ncf*metat), e(metat) (cip/ic001.f:52).
  f04    unit 4, first record with ncf in 5th position (cip/ic001.f:47) and
         the identity iord60 record read by the non-symmetric variant.
  ocno   unit 21 (empty; opened by cip/openf.f).
  cip.in the &cipfil / &icinp namelists given on standard input.

Integrals follow the recipe: h = diag(eps) + symmetric N(0, 0.05), eps sorted
uniform[-2, 1]; (pq|rs) = sum_K L^K_pq L^K_rs with L^K symmetric
N(0, 0.3 * 0.85^K).  With nsym > 1 each orbital and each Cholesky vector carry
an irrep of an abelian group (product table = XOR), so integrals vanish by
symmetry exactly as the reference's packed layout assumes.

Determinants of S are closed under the Ms = 0 spin flip with partners stored
next to each other (so the reference's S build in cip/deter.f:478-567
reproduces the file order), and coefficients are equal on flip partners in the
canonical (alpha string, then beta string) phase convention, converted to the
reference's excitation-list phase before writing.
"""
from __future__ import annotations

import dataclasses
import os
import struct
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# --------------------------------------------------------------------------
# Fortran unformatted sequential records (4-byte markers)


def write_record(fh, payload: bytes) -> None:
    n = len(payload)
    fh.write(struct.pack("<i", n))
    fh.write(payload)
    fh.write(struct.pack("<i", n))


def read_records(path: str) -> List[bytes]:
    out = []
    with open(path, "rb") as fh:
        while True:
            hdr = fh.read(4)
            if len(hdr) < 4:
                break
            (n,) = struct.unpack("<i", hdr)
            body = fh.read(n)
            (n2,) = struct.unpack("<i", fh.read(4))
            if n2 != n:
                raise ValueError(f"bad record marker in {path}")
            out.append(body)
    return out


# --------------------------------------------------------------------------
# configurations


@dataclasses.dataclass
class SynthConfig:
    name: str
    norb: int
    nocc: int                # doubly occupied orbitals of the reference det
    ncholesky: int
    ncf: int                 # target size of S after spin-flip closure (may end one above)
    metat: int
    tau: float
    ityper: int = 2          # 1 = MP only, 2 = MP + EN
    seed: int = 0
    max_rank: int = 2        # excitation ranks drawn for S: 1..max_rank
    ranks: Tuple[int, ...] = (2,)
    coef_mode: str = "gauss005"  # "gauss005" (N(0,.05), HF=1) or "decay09"
    nsym: int = 1
    include_hf: bool = True
    iselec: int = 1
    variant: str = "cipsym"  # or "cip"
    extra_icinp: str = ""
    virt_shift: float = 0.0  # added to h_aa of virtual orbitals (0 = the plain recipe)
    coef_sigma: float = 0.05  # width of the non-HF coefficients in "gauss005" mode
    curve_R: Optional[float] = None  # potential-curve geometry R (bohr): integrals from
                                     # L(R) = L0 + exp(-R/3) L1, eps(R) = eps0 + 0.1 exp(-R/2) eps1
    energy: str = "rayleigh"  # root energies: "rayleigh" (<Psi|H|Psi>) or "diagonal"
                              # (sum_k c_k^2 H_kk: no O(ncf^2) pass, for many large geometries)
    # space = "cas": S is the complete active space of the cas_occ highest
    # occupied and cas_virt lowest virtual orbitals (every Ms = 0 placement
    # of their 2*cas_occ electrons, ncf is then C(cas_occ+cas_virt,
    # cas_occ)^2); core_shift lowers the other occupied orbitals and
    # virt_shift raises only the other virtuals, so every perturber (it has
    # an electron outside the active space) lies several Eh above every root
    # energy: E2 without small denominators, for any roots within S
    space: str = "random"
    cas_occ: int = 2
    cas_virt: int = 8
    core_shift: float = 0.0


CONFIGS: Dict[str, SynthConfig] = {
    # small: 20 MOs, 10 e-, HF + 49 doubles, 1 root, tau 0.02
    "small": SynthConfig("small", norb=20, nocc=5, ncholesky=40, ncf=50, metat=1,
                         tau=0.02, ranks=(2,), coef_mode="gauss005", seed=0),
    # medium: 60 MOs, 20 e-, S=2000 singles/doubles/triples, 3 roots, tau 0.01
    "medium": SynthConfig("medium", norb=60, nocc=10, ncholesky=120, ncf=2000, metat=3,
                          tau=0.01, ranks=(1, 2, 3), coef_mode="decay09", seed=1),
    # large: 120 MOs, 30 e-, S=20000 doubles, 2 roots, tau 0.005
    "large": SynthConfig("large", norb=120, nocc=15, ncholesky=240, ncf=20000, metat=2,
                         tau=0.005, ranks=(2,), coef_mode="gauss005", seed=2),
}


# --------------------------------------------------------------------------
# integrals


def make_integrals(cfg: SynthConfig, rng: np.random.Generator):
    n = cfg.norb
    nsym = cfg.nsym
    irrep = np.zeros(n, dtype=np.int64)  # 0-based irreps
    if nsym > 1:
        irrep = rng.integers(0, nsym, size=n)
        # keep the reference det totally symmetric-friendly: any assignment works
    eps = np.sort(rng.uniform(-2.0, 1.0, size=n))
    if cfg.curve_R is not None:
        eps = eps + 0.1 * np.exp(-cfg.curve_R / 2.0) * rng.normal(0.0, 1.0, size=n)
    h = np.diag(eps)
    off = rng.normal(0.0, 0.05, size=(n, n))
    off = np.triu(off, 1)
    off = off + off.T
    same = irrep[:, None] == irrep[None, :]
    h = h + off * same
    if cfg.virt_shift:
        # a gap between occupied and virtual orbital energies keeps every
        # perturbation denominator away from zero (well-conditioned E2)
        v0 = cfg.nocc + (cfg.cas_virt if cfg.space == "cas" else 0)
        h[np.arange(v0, n), np.arange(v0, n)] += cfg.virt_shift
    if cfg.core_shift:
        c1 = cfg.nocc - (cfg.cas_occ if cfg.space == "cas" else 0)
        h[np.arange(0, c1), np.arange(0, c1)] -= cfg.core_shift
    def cholesky_vectors():
        out = np.zeros((cfg.ncholesky, n, n))
        for K in range(cfg.ncholesky):
            a = rng.normal(0.0, 0.3 * 0.85 ** K, size=(n, n))
            a = np.triu(a)
            a = a + np.triu(a, 1).T
            if nsym > 1:
                gK = K % nsym
                mask = (irrep[:, None] ^ irrep[None, :]) == gK
                a = a * mask
            out[K] = a
        return out

    L = cholesky_vectors()
    if cfg.curve_R is not None:
        L = L + np.exp(-cfg.curve_R / 3.0) * cholesky_vectors()
    return h, L, irrep


def eri_full(L: np.ndarray) -> Optional[np.ndarray]:
    n = L.shape[1]
    if n > 72:
        return None
    return np.einsum("kpq,krs->pqrs", L, L, optimize=True)


class ERI:
    """(pq|rs) from the Cholesky factors, with an optional dense cache."""

    def __init__(self, L: np.ndarray):
        self.L = L
        self.full = eri_full(L)

    def __call__(self, p, q, r, s):
        if self.full is not None:
            return self.full[p, q, r, s]
        return np.einsum("k...,k...->...", self.L[:, p, q], self.L[:, r, s])


def pair_order(norb: int, nocc: int, irrep: np.ndarray, nsym: int):
    """Pair list per irrep in the order of fock/wijkl_new.f:21-101.

    Returns ipair[is] = list of (i, j) 1-based, nt/np per irrep.
    """
    its = lambda a, b: ((a - 1) ^ (b - 1)) + 1  # noqa: E731
    sym = irrep + 1
    occ_by = {s: [i + 1 for i in range(nocc) if sym[i] == s] for s in range(1, nsym + 1)}
    vir_by = {s: [i + 1 for i in range(nocc, norb) if sym[i] == s] for s in range(1, nsym + 1)}
    ipair = {}
    for is_ in range(1, nsym + 1):
        pairs = []
        for ks in range(1, nsym + 1):
            for ls in range(ks, nsym + 1):
                if its(ks, ls) != is_:
                    continue
                if not occ_by[ks] or not occ_by[ls]:
                    continue
                for ixx, i in enumerate(occ_by[ks]):
                    lim = ixx if ks == ls else 0
                    for j in occ_by[ls][lim:]:
                        pairs.append((i, j))
        for ks in range(1, nsym + 1):
            for ls in range(1, nsym + 1):
                if its(ks, ls) != is_:
                    continue
                if not occ_by[ks] or not vir_by[ls]:
                    continue
                for i in occ_by[ks]:
                    for j in vir_by[ls]:
                        pairs.append((i, j))
        for ks in range(1, nsym + 1):
            for ls in range(ks, nsym + 1):
                if its(ks, ls) != is_:
                    continue
                if not vir_by[ks] or not vir_by[ls]:
                    continue
                for ixx, i in enumerate(vir_by[ks]):
                    lim = ixx if ks == ls else 0
                    for j in vir_by[ls][lim:]:
                        pairs.append((i, j))
        ipair[is_] = pairs
    return ipair


def write_ijkl(path: str, cfg: SynthConfig, h, L, irrep, F, J, K) -> Tuple[np.ndarray, np.ndarray, int]:
    """Write unit 40 and return (ij0, ntttt, ninte)."""
    n = cfg.norb
    nsym = cfg.nsym
    sym = (irrep + 1).astype(np.int32)
    ipair = pair_order(n, cfg.nocc, irrep, nsym)
    ij0 = np.zeros((n + 1, n + 1), dtype=np.int16)  # 1-based, ij0[i, j]
    for is_ in range(1, nsym + 1):
        for idx, (i, j) in enumerate(ipair[is_], start=1):
            if i <= j:
                ij0[i, j] = idx
                if i != j:
                    ij0[j, i] = is_
            else:
                ij0[j, i] = idx
                ij0[i, j] = is_
    ntttt = np.zeros(nsym + 1, dtype=np.int64)
    nint = 1
    for is_ in range(1, nsym + 1):
        ntttt[is_] = nint
        npp = len(ipair[is_])
        nint += npp * (npp + 1) // 2
    ninte = nint - 1
    vals = np.empty(ninte, dtype=np.float64)
    pos = 0
    for is_ in range(1, nsym + 1):
        pr = np.array(ipair[is_], dtype=np.int64) - 1
        npp = len(pr)
        if npp == 0:
            continue
        # (pair ij | pair kl) for kl <= ij, row by row
        Lp = L[:, pr[:, 0], pr[:, 1]]  # (K, npp)
        for ij in range(npp):
            row = Lp[:, ij] @ Lp[:, : ij + 1]
            vals[pos: pos + ij + 1] = row
            pos += ij + 1
    assert pos == ninte
    with open(path, "wb") as fh:
        hdr = struct.pack("<4i", nsym, n, cfg.nocc, 0) + sym.astype("<i4").tobytes()
        hdr += struct.pack("<i", 0) + struct.pack("<B", 1) + struct.pack("<i", 0)  # noa, ydp, chstan
        write_record(fh, hdr)
        its = np.array([[((a - 1) ^ (b - 1)) + 1 for a in range(1, nsym + 1)] for b in range(1, nsym + 1)],
                       dtype="<i4")
        write_record(fh, its.tobytes())  # ((its(i,j),i=1,ns),j=1,ns): its symmetric
        tri = lambda M: np.concatenate([M[i, : i + 1] for i in range(n)])  # noqa: E731
        write_record(fh, tri(h).astype("<f8").tobytes())
        write_record(fh, tri(J).astype("<f8").tobytes())
        write_record(fh, tri(K).astype("<f8").tobytes())
        write_record(fh, tri(F).astype("<f8").tobytes())
        # ((ij0(i,j),i=1,norb),j=1,norb): column-major
        write_record(fh, ij0[1:, 1:].T.astype("<i2").tobytes())
        write_record(fh, struct.pack("<i", ninte) + ntttt[1:].astype("<i4").tobytes())
        lsize = 8192
        nbuf = ninte // lsize + 1
        buf = np.zeros(nbuf * lsize, dtype="<f8")
        buf[:ninte] = vals
        for b in range(nbuf):
            write_record(fh, buf[b * lsize: (b + 1) * lsize].tobytes())
    return ij0, ntttt, ninte


def fock_closed_shell(h, eri: ERI, L: np.ndarray, nocc: int):
    """Closed-shell F, J, K and the reference energy (fock/fock.f:80-128)."""
    n = h.shape[0]
    occ = np.arange(nocc)
    # J_pq = (pp|qq), K_pq = (pq|pq)
    Ld = np.einsum("kpp->kp", L)
    J = Ld.T @ Ld
    K = np.einsum("kpq,kpq->pq", L, L)
    # F_pq = h_pq + sum_j 2 (pq|jj) - (pj|qj)
    coul = np.einsum("kpq,k->pq", L, Ld[:, occ].sum(axis=1))
    exch = np.einsum("kpj,kqj->pq", L[:, :, occ], L[:, :, occ])
    F = h + 2.0 * coul - exch
    F = np.where(np.abs(F) < 1e-7, 0.0, F)
    val = 2.0 * np.trace(h[np.ix_(occ, occ)]) + 2.0 * J[np.ix_(occ, occ)].sum() - K[np.ix_(occ, occ)].sum()
    # exact J_pp == K_pp as in fock.f:112-113 (both read ai(i,i,i,i))
    np.fill_diagonal(K, np.diag(J))
    return F, J, K, float(val)


# --------------------------------------------------------------------------
# determinants: canonical bitstrings (python ints, bit p-1 = orbital p)


def popcount(x: int) -> int:
    return bin(x).count("1")


def single_phase(bits: int, p: int, q: int) -> int:
    """Phase of a_q^+ a_p on a canonical string (0-based orbitals)."""
    lo, hi = (p, q) if p < q else (q, p)
    mask = ((1 << hi) - 1) & ~((1 << (lo + 1)) - 1)
    return -1 if popcount(bits & mask) & 1 else 1


def det_from_lists(holes: Sequence[int], parts: Sequence[int], norb: int, nocc: int) -> Tuple[int, int]:
    """Spin-orbital lists (1-based, beta = norb+1..2norb) -> (alpha, beta) ints."""
    a = (1 << nocc) - 1
    b = (1 << nocc) - 1
    for so in holes:
        if so <= norb:
            a &= ~(1 << (so - 1))
        else:
            b &= ~(1 << (so - norb - 1))
    for so in parts:
        if so <= norb:
            a |= 1 << (so - 1)
        else:
            b |= 1 << (so - norb - 1)
    return a, b


def cip_phase(holes: Sequence[int], parts: Sequence[int], norb: int, nocc: int) -> int:
    """<canonical D | prod_i (a+_{p_i} a_{h_i}) | HF> for cip's pairing.

    The reference pairs hole i with particle i of its sorted lists
    (cip/hntd.f aligns lists position by position); each pair is an even
    operator so the product is order independent.
    """
    a = (1 << nocc) - 1
    b = (1 << nocc) - 1
    sign = 1
    full = a | (b << norb)
    for h_, p_ in zip(holes, parts):
        h0, p0 = h_ - 1, p_ - 1
        sign *= single_phase(full, h0, p0) if True else 1
        full &= ~(1 << h0)
        full |= 1 << p0
    return sign


def flip_lists(holes, parts, norb):
    f = lambda so: so + norb if so <= norb else so - norb  # noqa: E731
    return sorted(f(x) for x in holes), sorted(f(x) for x in parts)


def random_det(rng, rank: int, norb: int, nocc: int, irrep, isym: int):
    """Random Ms=0 excitation of given rank (sorted hole/particle lists)."""
    occ_a = list(range(1, nocc + 1))
    vir_a = list(range(nocc + 1, norb + 1))
    for _ in range(1000):
        na = int(rng.integers(0, rank + 1))
        nb = rank - na
        if na > len(occ_a) or nb > len(occ_a) or na > len(vir_a) or nb > len(vir_a):
            continue
        ha = rng.choice(occ_a, size=na, replace=False) if na else []
        pa = rng.choice(vir_a, size=na, replace=False) if na else []
        hb = rng.choice(occ_a, size=nb, replace=False) if nb else []
        pb = rng.choice(vir_a, size=nb, replace=False) if nb else []
        holes = sorted([int(x) for x in ha] + [int(x) + norb for x in hb])
        parts = sorted([int(x) for x in pa] + [int(x) + norb for x in pb])
        g = 0
        for so in holes + parts:
            g ^= int(irrep[(so - 1) % norb])
        if g + 1 != isym:
            continue
        return holes, parts
    raise RuntimeError("could not draw a determinant of the requested symmetry")


def build_cas_space(cfg: SynthConfig, irrep):
    """S = the complete active space (space = "cas"), as (holes, parts)
    lists closed under spin flip (partners adjacent) and orbit indices."""
    import itertools
    norb, nocc = cfg.norb, cfg.nocc
    act = list(range(nocc - cfg.cas_occ + 1, nocc + cfg.cas_virt + 1))
    occ_act = set(range(nocc - cfg.cas_occ + 1, nocc + 1))
    strings = []
    for sel in itertools.combinations(act, cfg.cas_occ):
        hs = sorted(occ_act - set(sel))
        ps = sorted(o for o in sel if o > nocc)
        g = 0
        for o in hs + ps:
            g ^= int(irrep[o - 1])
        strings.append((hs, ps, g))
    dets, rep_of = [], []
    nrep = 0
    for a, (ha, pa, ga) in enumerate(strings):
        for b in range(a, len(strings)):
            hb, pb, gb = strings[b]
            if ga ^ gb:
                continue
            key = (tuple(sorted(ha + [o + norb for o in hb])), tuple(sorted(pa + [o + norb for o in pb])))
            dets.append(key)
            rep_of.append(nrep)
            if a != b:
                fkey = (tuple(sorted(hb + [o + norb for o in ha])), tuple(sorted(pb + [o + norb for o in pa])))
                dets.append(fkey)
                rep_of.append(nrep)
            nrep += 1
    order = sorted(range(len(dets)), key=lambda i: (len(dets[i][0]), i))
    return [dets[i] for i in order], [rep_of[i] for i in order]


def build_space(cfg: SynthConfig, rng, irrep):
    """S as a list of (holes, parts, rep_index) closed under spin flip."""
    if cfg.space == "cas":
        return build_cas_space(cfg, irrep)
    norb, nocc = cfg.norb, cfg.nocc
    seen = set()
    dets: List[Tuple[Tuple[int, ...], Tuple[int, ...]]] = []
    rep_of: List[int] = []
    if cfg.include_hf:
        dets.append(((), ()))
        rep_of.append(0)
        seen.add(((), ()))
    ranks = list(cfg.ranks)
    nrep = 1 if cfg.include_hf else 0
    guard = 0
    while len(dets) < cfg.ncf:
        guard += 1
        if guard > 200 * cfg.ncf + 1000:
            raise RuntimeError("could not build S of the requested size")
        r = int(ranks[int(rng.integers(0, len(ranks)))])
        holes, parts = random_det(rng, r, norb, nocc, irrep, 1)
        key = (tuple(holes), tuple(parts))
        if key in seen:
            continue
        fh, fp = flip_lists(holes, parts, norb)
        fkey = (tuple(fh), tuple(fp))
        seen.add(key)
        dets.append(key)
        rep_of.append(nrep)
        if fkey != key:
            seen.add(fkey)
            dets.append(fkey)
            rep_of.append(nrep)
        nrep += 1
    # the reference groups S by excitation rank (cip/lec60.f, deter.f:478):
    # write rank-sorted so the file order is the reference's S order
    order = sorted(range(len(dets)), key=lambda i: (len(dets[i][0]), i))
    dets = [dets[i] for i in order]
    rep_of = [rep_of[i] for i in order]
    return dets, rep_of


# --------------------------------------------------------------------------
# Hamiltonian matrix elements over S (canonical phases) for the
# Rayleigh quotient E(m) = <Psi_m|H|Psi_m>


class SlaterCondon:
    def __init__(self, h, L, norb, nocc):
        self.h = h
        self.L = L
        self.eri = ERI(L)
        self.norb = norb
        self.nocc = nocc

    def diag(self, a: int, b: int) -> float:
        occ_a = [p for p in range(self.norb) if a >> p & 1]
        occ_b = [p for p in range(self.norb) if b >> p & 1]
        Ld = np.einsum("kpp->kp", self.L)
        e = sum(self.h[p, p] for p in occ_a) + sum(self.h[p, p] for p in occ_b)
        Ja = Ld[:, occ_a].sum(axis=1)
        Jb = Ld[:, occ_b].sum(axis=1)
        coul = 0.5 * float((Ja + Jb) @ (Ja + Jb))
        ex = 0.0
        for occ in (occ_a, occ_b):
            if occ:
                Lo = self.L[:, occ][:, :, occ]
                ex += 0.5 * float(np.einsum("kpq,kpq->", Lo, Lo))
        return float(e + coul - ex)

    def offdiag(self, a1, b1, a2, b2) -> float:
        """<D1|H|D2> for degree 1 or 2 (canonical phases)."""
        xa, xb = a1 ^ a2, b1 ^ b2
        da, db = popcount(xa) // 2, popcount(xb) // 2
        n = self.norb
        if da + db == 1:
            if da == 1:
                s_bits, o_bits = a2, b2
                x = xa
            else:
                s_bits, o_bits = b2, a2
                x = xb
            p = (x & a2 if da else x & b2).bit_length() - 1  # occupied in D2
            q = (x & a1 if da else x & b1).bit_length() - 1  # occupied in D1
            sign = single_phase(s_bits, p, q)
            occ_s = [r for r in range(n) if s_bits >> r & 1]
            occ_o = [r for r in range(n) if o_bits >> r & 1]
            val = self.h[p, q]
            allocc = occ_s + occ_o
            Lpq = self.L[:, p, q]
            Ld = np.einsum("kpp->kp", self.L)
            val += float(Lpq @ Ld[:, allocc].sum(axis=1))
            val -= float(np.einsum("kr,kr->", self.L[:, p, occ_s], self.L[:, q, occ_s]))
            return sign * float(val)
        if da + db == 2:
            if da == 1 and db == 1:
                p = (xa & a2).bit_length() - 1
                q = (xa & a1).bit_length() - 1
                r = (xb & b2).bit_length() - 1
                s = (xb & b1).bit_length() - 1
                sign = single_phase(a2, p, q) * single_phase(b2, r, s)
                return sign * float(self.eri(p, q, r, s))
            bits1, bits2 = (a1, a2) if da == 2 else (b1, b2)
            x = bits1 ^ bits2
            occ2 = x & bits2
            occ1 = x & bits1
            p1 = (occ2 & -occ2).bit_length() - 1
            p2 = occ2.bit_length() - 1
            q1 = (occ1 & -occ1).bit_length() - 1
            q2 = occ1.bit_length() - 1
            s1 = single_phase(bits2, p1, q1)
            mid = (bits2 & ~(1 << p1)) | (1 << q1)
            s2 = single_phase(mid, p2, q2)
            val = self.eri(p1, q1, p2, q2) - self.eri(p1, q2, p2, q1)
            return s1 * s2 * float(val)
        return 0.0


def diagonal_energy(F, J, K, dets, norb: int, C: np.ndarray) -> np.ndarray:
    """sum_k c_km^2 (H_kk - E_HF) for the columns of C, with H_kk - E_HF from
    the closed-shell F, J, K over the occupation changes dn of each
    determinant: sum_r dn_r F_rr + 1/2 sum_rs dn_r dn_s (J_rs - [same spin] K_rs)."""
    n = norb
    D = np.zeros((len(dets), 2 * n))
    for k, (hl, pt) in enumerate(dets):
        if hl:
            D[k, np.asarray(hl) - 1] -= 1.0
            D[k, np.asarray(pt) - 1] += 1.0
    Fso = np.concatenate([np.diag(F), np.diag(F)])
    orb = np.tile(np.arange(n), 2)
    spin = np.repeat([0, 1], n)
    X = J[np.ix_(orb, orb)] - (spin[:, None] == spin[None, :]) * K[np.ix_(orb, orb)]
    dg = D @ Fso + 0.5 * np.einsum("kr,rs,ks->k", D, X, D)
    return np.einsum("im,im,i->m", C, C, dg)


def curve_geometries(n: int = 256, seed: int = 100) -> List[SynthConfig]:
    """Potential-curve batch: n geometries with R uniform on [2, 12] bohr,
    norb uniform in {40..100}, |S| uniform in [500, 5000] (before spin-flip
    closure), 20 electrons, 1 root, S = reference + singles/doubles/triples
    with coefficients N(0,1) 0.9^rank, tau = 0.01, 2 norb Cholesky vectors."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        R = float(rng.uniform(2.0, 12.0))
        norb = int(rng.integers(40, 101))
        ncf = int(rng.integers(500, 5001))
        out.append(SynthConfig(f"geo{i:03d}", norb=norb, nocc=10, ncholesky=2 * norb, ncf=ncf, metat=1,
                               tau=0.01, ranks=(1, 2, 3), coef_mode="decay09", seed=seed * 1000 + i,
                               curve_R=R, energy="diagonal"))
    return out


def rayleigh(sc: SlaterCondon, bits: List[Tuple[int, int]], C: np.ndarray) -> np.ndarray:
    """<Psi_m|H - E_HF|Psi_m> for the columns of C (canonical phases)."""
    ncf = len(bits)
    hf_a = (1 << sc.nocc) - 1
    ehf = sc.diag(hf_a, hf_a)
    dg = np.array([sc.diag(a, b) - ehf for a, b in bits])
    E = np.einsum("im,im,i->m", C, C, dg)
    W = (sc.norb + 63) // 64
    A = np.zeros((ncf, W), dtype=np.uint64)
    B = np.zeros((ncf, W), dtype=np.uint64)
    mask64 = (1 << 64) - 1
    for i, (a, b) in enumerate(bits):
        for w in range(W):
            A[i, w] = (a >> (64 * w)) & mask64
            B[i, w] = (b >> (64 * w)) & mask64
    for i in range(ncf):
        d = np.zeros(ncf - i - 1, dtype=np.int64)
        for w in range(W):
            d += np.bitwise_count(A[i + 1:, w] ^ A[i, w]).astype(np.int64)
            d += np.bitwise_count(B[i + 1:, w] ^ B[i, w]).astype(np.int64)
        for jj in np.nonzero(d <= 4)[0]:
            j = i + 1 + int(jj)
            hij = sc.offdiag(bits[i][0], bits[i][1], bits[j][0], bits[j][1])
            E += 2.0 * C[i] * C[j] * hij
    return E


# --------------------------------------------------------------------------
# main entry


def generate(cfg: SynthConfig, workdir: str, verbose: bool = False) -> dict:
    os.makedirs(workdir, exist_ok=True)
    rng = np.random.default_rng(cfg.seed)
    h, L, irrep = make_integrals(cfg, rng)
    eri = ERI(L)
    F, J, K, ehf = fock_closed_shell(h, eri, L, cfg.nocc)
    ij0, ntttt, ninte = write_ijkl(os.path.join(workdir, "ijkl"), cfg, h, L, irrep, F, J, K)
    escf = ehf  # enuc = 0
    with open(os.path.join(workdir, "ener"), "wb") as fh:
        write_record(fh, b"energie du determinant de reference".ljust(40) + struct.pack("<i", 1)
                     + struct.pack("<d", escf))
    dets, rep_of = build_space(cfg, rng, irrep)
    ncf = len(dets)
    nrep = max(rep_of) + 1
    # coefficients on orbit representatives (canonical phase), equal on partners
    Crep = np.zeros((nrep, cfg.metat))
    ranks = np.zeros(nrep, dtype=np.int64)
    for i, (hl, _) in enumerate(dets):
        ranks[rep_of[i]] = len(hl)
    for m in range(cfg.metat):
        if cfg.coef_mode == "gauss005":
            v = rng.normal(0.0, cfg.coef_sigma, size=nrep)
            if cfg.include_hf:
                v[0] = 1.0 if m == 0 else v[0]
        else:
            v = rng.normal(0.0, 1.0, size=nrep) * 0.9 ** ranks
        Crep[:, m] = v
    C = Crep[np.array(rep_of)]
    # orthonormalise the full vectors (partners stay equal)
    Q, R = np.linalg.qr(C)
    C = Q * np.sign(np.diag(R))[None, :]
    bits = [det_from_lists(hl, pt, cfg.norb, cfg.nocc) for hl, pt in dets]
    sc = SlaterCondon(h, L, cfg.norb, cfg.nocc)
    if cfg.energy == "rayleigh":
        E = rayleigh(sc, bits, C) + escf
    else:
        E = diagonal_energy(F, J, K, dets, cfg.norb, C) + escf
    sigma = np.array([cip_phase(hl, pt, cfg.norb, cfg.nocc) for hl, pt in dets], dtype=np.float64)
    Ccip = C * sigma[:, None]
    # unit 60: S in cip/pie.f records (v = 1)
    with open(os.path.join(workdir, "det"), "wb") as fh:
        lungo = 1000
        for s in range(0, ncf, lungo):
            chunk = dets[s: s + lungo]
            idet: List[int] = []
            nex: List[int] = []
            for hl, pt in chunk:
                for t_, p_ in zip(hl, pt):
                    idet += [t_, p_]
                nex.append(len(hl))
            payload = struct.pack("<ii", len(idet), len(chunk))
            payload += np.array(idet, dtype="<i4").tobytes() + np.array(nex, dtype="<i4").tobytes()
            payload += np.ones(len(chunk), dtype="<f8").tobytes()
            if cfg.variant == "cipsym":
                payload += np.zeros(len(chunk) * cfg.metat, dtype="<f8").tobytes()
            write_record(fh, payload)
    with open(os.path.join(workdir, "bdvec"), "wb") as fh:
        write_record(fh, struct.pack("<ii", ncf, cfg.metat) + Ccip.T.astype("<f8").tobytes()
                     + E.astype("<f8").tobytes())
    with open(os.path.join(workdir, "f04"), "wb") as fh:
        write_record(fh, struct.pack("<5i", cfg.norb, cfg.nocc, cfg.nocc + cfg.norb, cfg.metat, ncf))
        write_record(fh, np.arange(1, ncf + 1, dtype="<i4").tobytes())
    open(os.path.join(workdir, "ocno"), "wb").close()
    with open(os.path.join(workdir, "cip.in"), "w") as fh:
        fh.write(" &cipfil\n &end\n")
        fh.write(f" &icinp\n  metat={cfg.metat}, ityper={cfg.ityper}, lecdet=5, tau={cfg.tau!r},"
                 f" test={cfg.tau!r}, iselec={cfg.iselec}, ymoyen=t, ybrd=f, ywvf=f,"
                 f" title='{cfg.name}'{(', ' + cfg.extra_icinp) if cfg.extra_icinp else ''}\n &end\n")
    info = dict(name=cfg.name, norb=cfg.norb, nocc=cfg.nocc, ncf=ncf, metat=cfg.metat,
                ninte=int(ninte), escf=escf, E=E.tolist(), variant=cfg.variant)
    if verbose:
        print(info)
    return info


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("config", choices=sorted(CONFIGS))
    ap.add_argument("workdir")
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--variant", choices=["cip", "cipsym"], default=None)
    a = ap.parse_args(argv)
    cfg = dataclasses.replace(CONFIGS[a.config])
    if a.seed is not None:
        cfg.seed = a.seed
    if a.variant:
        cfg.variant = a.variant
    generate(cfg, a.workdir, verbose=True)


if __name__ == "__main__":
    main()
