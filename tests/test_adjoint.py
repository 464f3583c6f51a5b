"""Adjoint form: gradients of the E2 sums from cipsi_run_pt2_adjoint (through
cipsi_gb300.adjoint.E2Function) against central finite differences of the
forward engine with FP64-stored integrals, and the finite-field dipole.

CPU tests check the torch restatement of the closed-shell relations against
the arrays the host reads from the work directory."""
import dataclasses

import numpy as np
import pytest
import torch

from cipsi_gb300 import adjoint, synth


def make_system(tmp_path, cfg):
    wd = str(tmp_path / cfg.name)
    synth.generate(cfg, wd)
    h, L, _ = synth.make_integrals(cfg, np.random.default_rng(cfg.seed))
    S = adjoint.System(wd)
    eri = S.pk.pack_from_cholesky(L, S.ninte)
    n = cfg.norb
    ti, tj = np.tril_indices(n)
    h_tri = np.zeros(n * (n + 1) // 2)
    h_tri[adjoint._tri(ti, tj)] = h[ti, tj]
    return S, h_tri, eri, h


SMALL_WELL = dataclasses.replace(synth.CONFIGS["small"], name="adj_well", virt_shift=3.0, metat=1)
MIX_SYM = synth.SynthConfig("adj_sym", norb=12, nocc=4, ncholesky=20, ncf=60, metat=2, tau=0.02,
                            ranks=(1, 2, 3), coef_mode="decay09", seed=4, nsym=2, virt_shift=3.0)


@pytest.mark.parametrize("cfg", [synth.CONFIGS["small"], MIX_SYM], ids=["small", "sym2"])
def test_closed_shell_relations_reproduce_the_inputs(tmp_path, engine_lib, cfg):
    S, h_tri, eri, _ = make_system(tmp_path, cfg)
    assert np.array_equal(eri.astype(np.float32), S.inp.array("eri"))
    vals = S.engine_inputs(torch.as_tensor(h_tri), torch.as_tensor(eri))
    for name, v in zip(("F", "J", "K", "fmpb", "e", "eb", "emp"), vals):
        ref = S.inp.array(name)
        np.testing.assert_allclose(v.numpy(), ref, rtol=0, atol=1e-12, err_msg=name)
    S.close()


def fd_check(S, args, seed, which, picks, step=1e-5, rtol=1e-6, atol=1e-8):
    """Adjoint gradient of <seed, E2> w.r.t. args[which] at `picks` against
    central differences at steps h and h/2 combined by Richardson
    extrapolation (error O(h^4): the EN denominators of excited roots can be
    small, which makes the O(h^2) error of one central difference visible)."""
    grads = S.adjoint_at(*args, seed)
    name = ("F", "J", "K", "eri", "fmpb", "e", "eb", "emp")[which]
    g_adj = grads[name]

    def central(i, h):
        vals = []
        for sgn in (1.0, -1.0):
            a = [x.copy() for x in args]
            a[which][i] += sgn * h
            vals.append((S.run_engine(*[torch.as_tensor(x) for x in a]) * seed).sum())
        return (vals[0] - vals[1]) / (2 * h)

    for i in picks:
        fd = (4.0 * central(i, step / 2) - central(i, step)) / 3.0
        assert abs(g_adj[i] - fd) <= atol + rtol * max(abs(fd), abs(g_adj[i])), (name, i, g_adj[i], fd)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [SMALL_WELL, MIX_SYM], ids=["small", "sym2"])
def test_adjoint_matches_finite_differences(tmp_path, engine_lib, cfg):
    S, h_tri, eri, _ = make_system(tmp_path, cfg)
    vals = [x.numpy().copy() for x in S.engine_inputs(torch.as_tensor(h_tri), torch.as_tensor(eri))]
    F, J, K, fmpb, e, eb, emp = vals
    args = [F, J, K, eri.copy(), fmpb, e, eb, emp]
    S.run_engine(*[torch.as_tensor(x) for x in args])
    mt = S.dims.metat
    rng = np.random.default_rng(7)
    seed = rng.normal(size=(3, mt))
    grads = S.adjoint_at(*args, seed)
    # 200 integrals among those the E2 sums depend on
    nz = np.nonzero(grads["eri"])[0]
    assert len(nz) > 200
    fd_check(S, args, seed, 3, rng.choice(nz, 200, replace=False))
    nt = len(F)
    for which, count in ((0, 20), (1, 10), (2, 10)):
        fd_check(S, args, seed, which, rng.choice(nt, count, replace=False))
    fd_check(S, args, seed, 4, rng.choice(len(fmpb), 10, replace=False))
    for which in (5, 6, 7):
        fd_check(S, args, seed, which, range(mt))
    S.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [SMALL_WELL, MIX_SYM], ids=["small", "sym2"])
def test_one_electron_adjoint_matches_full(tmp_path, engine_lib, cfg):
    """cipsi_run_pt2_adjoint_1e: its E2 sums are the forward run's and its
    F, J, K, fmpb and root-energy gradients the full adjoint's (FP64 atomics
    add in a run-dependent order: equal to rounding)."""
    S, h_tri, eri, _ = make_system(tmp_path, cfg)
    vals = [x.numpy().copy() for x in S.engine_inputs(torch.as_tensor(h_tri), torch.as_tensor(eri))]
    F, J, K, fmpb, e, eb, emp = vals
    args = [F, J, K, eri.copy(), fmpb, e, eb, emp]
    fwd = S.run_engine(*[torch.as_tensor(x) for x in args])
    mt = S.dims.metat
    seed = np.random.default_rng(5).normal(size=(3, mt))
    full = S.adjoint_at(*args, seed)
    S.load(*args)
    e2, one = S.ctx.adjoint_1e(S.opts, seed)
    np.testing.assert_allclose(e2, fwd, rtol=1e-12, atol=1e-16)
    for k in ("F", "J", "K", "fmpb", "e", "eb", "emp"):
        scale = max(np.abs(full[k]).max(), 1e-300)
        np.testing.assert_allclose(one[k], full[k], rtol=0, atol=1e-12 * scale, err_msg=k)
    S.close()


@pytest.mark.gpu
def test_dipole_matches_finite_field(tmp_path, engine_lib):
    """sum mu_pq dE2/dh_pq (one one-electron adjoint pass, and a forward plus
    a full backward pass) against cip-style runs at
    h +- F mu with F, J, K, E_HF and the zero-order sums regenerated."""
    S, h_tri, eri, _ = make_system(tmp_path, SMALL_WELL)
    n = S.dims.norb
    rng = np.random.default_rng(11)
    mu = rng.normal(0.0, 0.5, size=(n, n))
    mu = 0.5 * (mu + mu.T)
    seed = np.zeros((3, S.dims.metat))
    seed[1, 0] = 1.0  # e2vp of the first root
    d_adj = adjoint.dipole(S, h_tri, eri, mu, seed)  # one-electron adjoint pass
    d_full = adjoint.dipole(S, h_tri, eri, mu, seed, one_electron=False)
    assert abs(d_adj - d_full) <= 1e-11 * max(1.0, abs(d_full)), (d_adj, d_full)
    ti, tj = np.tril_indices(n)
    mu_tri = np.zeros_like(h_tri)
    mu_tri[adjoint._tri(ti, tj)] = mu[ti, tj]
    field = 1e-4
    e = []
    for sgn in (1.0, -1.0):
        with torch.no_grad():
            E = S.e2(torch.as_tensor(h_tri + sgn * field * mu_tri), torch.as_tensor(eri))
        e.append(float((E.numpy() * seed).sum()))
    d_ff = (e[0] - e[1]) / (2 * field)
    assert abs(d_adj - d_ff) <= 1e-6 * max(1.0, abs(d_ff)), (d_adj, d_ff)
    S.close()
