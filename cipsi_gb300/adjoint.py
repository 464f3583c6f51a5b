"""Adjoint form: dE2/dh_pq and dE2/d(pq|rs) in one backward pass.

`E2Function` is a torch.autograd.Function over the C ABI: its forward is
cipsi_run_pt2 (integrals kept in FP64 on the device), its backward
cipsi_run_pt2_adjoint.  Its inputs are the engine's own arrays (F, J, K,
packed (pq|rs), fmpb, e, eb, emp); its output the E2 sums
[e2mp, e2vp, e2b] x metat.

`System` builds those arrays from a one-electron matrix h and the unique
two-electron integrals with torch operations, so a backward pass reaches h
and (pq|rs):

  F_pq = h_pq + sum_i [2 (pq|ii) - (pi|qi)]         closed-shell Fock (fock)
  J_pq = (pp|qq), K_pq = (pq|pq)                      cip/ijkf.f:29-31
  E_HF = sum_i (h_ii + F_ii)                          the reference energy
  fmpb_p = F_pp (both spins)                          cip/faifoc.f, tocom = 0
  e_m = E_m(abs) - E_HF                               cip.f:99 (e relative)
  emp_m = sum_k c_km^2 hmp(k), eb_m = sum_k c_km^2 hdig(k)   cip.f:99-135

with i over the doubly occupied orbitals.  The S coefficients and the
absolute root energies (file 59) are held fixed, as a finite-field cip run
that reuses the bd vectors does.  A dipole-like property
sum_pq mu_pq dE2/dh_pq is then one pass of the one-electron adjoint
(`System.grad_h`: E2 and dE2/dh together, about the cost of one forward
run) instead of the cip runs at h +- F mu (two for a central difference,
three or more for the quadratic fit of Autocip_13/ffield.f90:66-127), and
gives every field direction at once.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import engine


def _tri(i, j):
    """Packed lower-triangle position of (i, j), 0-based (i >= j)."""
    hi = np.maximum(i, j)
    lo = np.minimum(i, j)
    return hi * (hi + 1) // 2 + lo


class Packing:
    """Packed (pq|rs) positions of cip/ai.f from the ij0 / ntttt tables."""

    def __init__(self, norb: int, ij0: np.ndarray, ntttt: np.ndarray):
        n = norb
        A = ij0.reshape(n, n).T  # A[i, j] = ij0(i+1, j+1) (column-major in the file)
        i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        lo, hi = np.minimum(i, j), np.maximum(i, j)
        self.pair = A[lo, hi].astype(np.int64)                  # pair index (1-based) of {i, j}
        self.irrep = np.where(lo == hi, 1, A[hi, lo]).astype(np.int64)
        self.ntttt = np.asarray(ntttt, np.int64)
        self.n = n

    def index(self, i, j, k, l):
        """0-based packed position of (ij|kl); -1 where the irreps differ."""
        p1, s1 = self.pair[i, j], self.irrep[i, j]
        p2, s2 = self.pair[k, l], self.irrep[k, l]
        lo, hi = np.minimum(p1, p2), np.maximum(p1, p2)
        idx = lo + hi * (hi - 1) // 2 + self.ntttt[s1 - 1] - 2
        return np.where(s1 == s2, idx, -1)

    def pack_from_cholesky(self, L: np.ndarray, ninte: int) -> np.ndarray:
        """(pq|rs) = sum_K L^K_pq L^K_rs in the packed order (FP64)."""
        n = self.n
        ti, tj = np.tril_indices(n)
        Lp = L[:, ti, tj]                          # K x npairs (lower triangle)
        V = Lp.T @ Lp                              # npairs x npairs
        tpos = np.full((n, n), -1, np.int64)
        tpos[ti, tj] = np.arange(len(ti))
        tpos[tj, ti] = np.arange(len(ti))
        out = np.zeros(ninte)
        # every (i >= j, k >= l) quadruple maps to one packed slot
        for a in range(len(ti)):
            i, j = ti[a], tj[a]
            idx = self.index(np.full(len(ti), i), np.full(len(ti), j), ti, tj)
            ok = idx >= 0
            out[idx[ok]] = V[a, tpos[ti[ok], tj[ok]]]
        return out


class System:
    """One cip input (work directory) whose integrals are driven from
    (h, packed (pq|rs)) through the closed-shell relations above."""

    def __init__(self, workdir: str, device: int = 0, variant: str = "cipsym"):
        self.inp = engine.Inputs(workdir, variant=variant)
        d = self.inp.dims
        self.dims, self.opts = d, engine.Opts.from_buffer_copy(self.inp.opts)
        n, nocc, ncf, mt = d.norb, d.noca, d.ncf, d.metat
        g = self.inp.array
        self.itsym, self.its, self.ij0, self.ntttt = g("itsym"), g("its"), g("ij0"), g("ntttt")
        self.c = g("c")                                  # metat x ncf (reference phase)
        self.teste, self.taum = g("teste"), g("taum")
        self.escf = float(g("escf")[0])
        self.e_abs = g("e") + self.escf
        self.ninte = self.inp.count("eri")
        self.pk = Packing(n, self.ij0, self.ntttt)
        ti, tj = np.tril_indices(n)
        tpos = _tri(ti, tj)
        order = np.argsort(tpos)
        ti, tj = ti[order], tj[order]                    # position t -> (i >= j)
        self.JI = torch.as_tensor(self.pk.index(ti, ti, tj, tj))
        self.KI = torch.as_tensor(self.pk.index(ti, tj, ti, tj))
        occ = np.arange(nocc)
        self.FD = torch.as_tensor(self.pk.index(ti[:, None], tj[:, None], occ[None, :], occ[None, :]))
        self.FX = torch.as_tensor(self.pk.index(ti[:, None], occ[None, :], tj[:, None], occ[None, :]))
        self.diag_t = torch.as_tensor(_tri(np.arange(n), np.arange(n)))
        # S: occupation changes relative to the reference (holes -1, particles +1)
        ne, nd, trou, part = g("ne"), g("nd"), g("trou"), g("part")
        D = np.zeros((ncf, 2 * n))
        for k in range(ncf):
            for q in range(ne[k]):
                D[k, trou[nd[k] + q] - 1] -= 1.0
                D[k, part[nd[k] + q] - 1] += 1.0
        self.D = torch.as_tensor(D)
        self.C2 = torch.as_tensor(self.c.reshape(mt, ncf).T ** 2)   # ncf x metat
        spin = np.repeat([0, 1], n)
        self.same_spin = torch.as_tensor((spin[:, None] == spin[None, :]).astype(np.float64))
        self.orb = torch.as_tensor(np.tile(np.arange(n), 2))
        self.device = device
        self._ctx = None

    @property
    def ctx(self) -> engine.Context:
        """The engine context (created, and the space uploaded, on first use)."""
        if self._ctx is None:
            self._ctx = engine.Context(self.dims, device=self.device)
            self._ctx.upload(self.inp)
        return self._ctx

    # ---- closed-shell relations (torch)
    def _gather(self, eri: torch.Tensor, idx: torch.Tensor) -> torch.Tensor:
        z = torch.zeros((), dtype=eri.dtype)
        return torch.where(idx >= 0, eri[idx.clamp(min=0)], z)

    def engine_inputs(self, h_tri: torch.Tensor, eri: torch.Tensor):
        """(F, J, K, fmpb, e, eb, emp) from h (packed lower triangle) and the
        packed (pq|rs)."""
        n = self.dims.norb
        J = self._gather(eri, self.JI)
        K = self._gather(eri, self.KI)
        F = h_tri + (2.0 * self._gather(eri, self.FD) - self._gather(eri, self.FX)).sum(dim=1)
        nocc = self.dims.noca
        hd = h_tri[self.diag_t]
        Fd = F[self.diag_t]
        ehf = (hd[:nocc] + Fd[:nocc]).sum()
        fmpb = torch.cat([Fd, Fd])
        # full spin-orbital matrix X_rs = J - [same spin] K over orbital pairs
        ii, jj = self.orb[:, None], self.orb[None, :]
        t = torch.maximum(ii, jj) * (torch.maximum(ii, jj) + 1) // 2 + torch.minimum(ii, jj)
        X = J[t] - self.same_spin * K[t]
        Fso = torch.cat([Fd, Fd])
        hdig = self.D @ Fso + 0.5 * torch.einsum("kr,rs,ks->k", self.D, X, self.D)
        hmp = self.D @ fmpb
        eb = self.C2.T @ hdig
        emp = self.C2.T @ hmp
        e = torch.as_tensor(self.e_abs) - ehf
        return F, J, K, fmpb, e, eb, emp

    def e2(self, h_tri: torch.Tensor, eri: torch.Tensor) -> torch.Tensor:
        """E2 sums [e2mp, e2vp, e2b] x metat; differentiable in h and eri."""
        F, J, K, fmpb, e, eb, emp = self.engine_inputs(h_tri, eri)
        return E2Function.apply(F, J, K, eri, fmpb, e, eb, emp, self)

    def load(self, F, J, K, eri, fmpb, e, eb, emp):
        """Put these engine inputs on the device (FP64 integrals)."""
        a = [x.detach().cpu().numpy() if torch.is_tensor(x) else np.asarray(x)
             for x in (F, J, K, eri, fmpb, e, eb, emp)]
        self.ctx.set_integrals_f64store(self.itsym, self.its, a[0], a[1], a[2], self.ij0, self.ntttt, a[3])
        self.ctx.set_roots(self.c, a[5], a[6], a[7], self.teste, self.taum, a[4])

    def run_engine(self, F, J, K, eri, fmpb, e, eb, emp) -> np.ndarray:
        self.load(F, J, K, eri, fmpb, e, eb, emp)
        r = self.ctx.run(self.opts)
        return np.array([r["e2mp"], r["e2vp"], r["e2b"]])

    def adjoint_at(self, F, J, K, eri, fmpb, e, eb, emp, seed) -> dict:
        """Gradients of sum(seed * E2) at these inputs (they are loaded
        first: the context may hold the inputs of a later forward run)."""
        self.load(F, J, K, eri, fmpb, e, eb, emp)
        return self.ctx.adjoint(self.opts, seed)

    def grad_h(self, h_tri, eri, seed) -> tuple:
        """E2 sums [3, metat] and dL/dh (packed lower triangle) with
        L = sum(seed * E2), from one one-electron adjoint pass
        (cipsi_run_pt2_adjoint_1e): the (pq|rs) are held fixed, so their
        gradient is not formed, and the pass costs about one forward run."""
        h = torch.tensor(np.asarray(h_tri, np.float64), requires_grad=True)
        eri_t = torch.as_tensor(eri, dtype=torch.float64)
        outs = self.engine_inputs(h, eri_t)  # F, J, K, fmpb, e, eb, emp
        self.load(outs[0], outs[1], outs[2], eri_t, *outs[3:])
        e2, g = self.ctx.adjoint_1e(self.opts, seed)
        grads = [torch.as_tensor(g[k], dtype=torch.float64) for k in ("F", "J", "K", "fmpb", "e", "eb", "emp")]
        # J and K come from (pq|rs) alone: they do not depend on h
        pairs = [(o, gr) for o, gr in zip(outs, grads) if o.requires_grad]
        torch.autograd.backward([o for o, _ in pairs], [gr for _, gr in pairs])
        return e2, h.grad.numpy().copy()

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
        self.inp.close()


class E2Function(torch.autograd.Function):
    """E2 of the engine as a function of its integral and zero-order arrays."""

    @staticmethod
    def forward(ctx, F, J, K, eri, fmpb, e, eb, emp, system: System):
        out = system.run_engine(F, J, K, eri, fmpb, e, eb, emp)
        ctx.system = system
        ctx.save_for_backward(F, J, K, eri, fmpb, e, eb, emp)
        return torch.as_tensor(out, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        s: System = ctx.system
        g = s.adjoint_at(*ctx.saved_tensors, grad_out.detach().cpu().numpy())
        t = lambda x: torch.as_tensor(x, dtype=torch.float64)  # noqa: E731
        return (t(g["F"]), t(g["J"]), t(g["K"]), t(g["eri"]), t(g["fmpb"]), t(g["e"]), t(g["eb"]),
                t(g["emp"]), None)


def dipole(system: System, h_tri: np.ndarray, eri: np.ndarray, mu: np.ndarray,
           seed: Optional[np.ndarray] = None, one_electron: bool = True) -> float:
    """sum_pq mu_pq dL/dh_pq with L = sum seed * [e2mp; e2vp; e2b] (default:
    e2vp of root 1); mu full symmetric.  one_electron: one pass of the
    one-electron adjoint (System.grad_h); otherwise a forward and a full
    backward pass through E2Function (which also forms dL/d(pq|rs))."""
    mt = system.dims.metat
    if seed is None:
        seed = np.zeros((3, mt))
        seed[1, 0] = 1.0
    if one_electron:
        _, gh = system.grad_h(h_tri, eri, seed)
    else:
        h = torch.tensor(h_tri, dtype=torch.float64, requires_grad=True)
        E = system.e2(h, torch.as_tensor(eri, dtype=torch.float64))
        (E * torch.as_tensor(seed)).sum().backward()
        gh = h.grad.numpy()
    n = system.dims.norb
    ti, tj = np.tril_indices(n)
    # the field h -> h + F mu moves the packed element of (i >= j) by F mu_ij
    return float((gh[_tri(ti, tj)] * mu[ti, tj]).sum())
