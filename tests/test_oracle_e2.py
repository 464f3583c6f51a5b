"""The oracle's E2 sums against E2 recomputed from the independent brute-force
model: the model's perturber set, spin-flip weights and couplings
b_m = <I|H|Psi_m>, its own diagonal energies (hmp, hdig from the closed-shell
F, J, K), and the textbook partitions of pert1.f:148-191 --

    E2_MP(m)  = sum_I (1 + fmul_I) b_m^2 / (emp_m - hmp(I))
    E2_ENvp(m) = sum_I (1 + fmul_I) b_m^2 / (e_m  - hdig(I))
    E2_ENb(m)  = sum_I (1 + fmul_I) b_m^2 / (eb_m - hdig(I))

with emp_m = sum_k c_km^2 hmp(k), eb_m = sum_k c_km^2 hdig(k) over S
(cip.f:99-120); and the selection of pert1.f:192-264: the unit-60 value
xam = max_m |b_m / (e_m - hdig(I))| taum_m of every perturber, the
near-degeneracy flag (|denominator| <= 0.05 with |term| >= 1e-6 selects it),
dpivot, and the set written to unit 60 (values within 1e-9 of tau exempt);
the norms psimp / psivp, ietat, and the histogram of isto.f.
Together with the set and coupling checks of
test_oracle_semantics this pins the oracle's arithmetic, not only its
enumeration.  Tolerance: 1e-10 Eh plus the oracle's first-order rounding
bound of each sum (cond_e2*), which is tiny on the well-conditioned systems
(virtual orbitals shifted up) and covers the near-zero denominators of the
plain recipe."""
import collections
import json
import os

import numpy as np
import pytest

import brute_force as bf
from cases import small_cases
from cipsi_gb300 import synth
from conftest import copy_dir
from oracle import build as ob
from test_autocip_chain import _all_records


def _gap(seed, ranks, nsym):
    return synth.SynthConfig("gap", norb=16, nocc=4, ncholesky=16, ncf=60, metat=2, tau=0.01, ranks=ranks,
                             coef_mode="gauss005", seed=seed, nsym=nsym, virt_shift=3.0)


CASES = [("gap31", _gap(31, (2,), 1)), ("gap32", _gap(32, (1, 2, 3), 1)), ("gap33", _gap(33, (1, 2), 2)),
         ("gap34_d2h", _gap(34, (1, 2, 3), 8)),
         ("gap35_6roots", synth.SynthConfig("gap", norb=14, nocc=4, ncholesky=14, ncf=60, metat=6, tau=0.01,
                                            ranks=(1, 2), coef_mode="decay09", seed=35, virt_shift=3.0))]
CASES += small_cases()


@pytest.mark.parametrize("name,cfg", CASES, ids=[c[0] for c in CASES])
def test_oracle_e2_matches_bruteforce_sums(tmp_path, oracle_exe, name, cfg):
    _check(tmp_path, cfg)


@pytest.mark.parametrize("ityper,iselec", [(1, 1), (2, 2), (2, 3), (1, 3)])
def test_oracle_options_match_bruteforce(tmp_path, oracle_exe, ityper, iselec):
    """MP only (ityper = 1: the MP coefficient sets the selection value, no EN
    sums), iselec = 2 (teste = test, taum = 1) and iselec = 3 (selection on
    the energy term |b^2/d| instead of |b/d|)."""
    import dataclasses
    for seed, ranks, nsym in ((32, (1, 2, 3), 1), (33, (1, 2), 2)):
        cfg = dataclasses.replace(_gap(seed, ranks, nsym), ityper=ityper, iselec=iselec)
        _check(tmp_path / f"s{seed}", cfg)


@pytest.mark.parametrize("coeff", [0.02, 0.1])
def test_oracle_cip_generators_by_coeff(tmp_path, oracle_exe, coeff):
    """cip (not cipsym) runs only the determinants with |c| >= coeff on some
    root as generators (cip/ic001.f); the owner rule then sees only those."""
    import dataclasses
    cfg = dataclasses.replace(_gap(32, (1, 2, 3), 1), variant="cip", extra_icinp=f"coeff={coeff}")
    _check(tmp_path, cfg, variant="cip", coeff=coeff)


def test_oracle_without_ywdeg(tmp_path, oracle_exe):
    """ywdeg = .false.: near-degenerate perturbers are not forced into the
    selection (pert1.f:195-198), on the plain recipe where many are."""
    import dataclasses
    cfg = dataclasses.replace(small_cases()[0][1], extra_icinp="ywdeg=f")
    _check(tmp_path, cfg, ywdeg=False)


def _check(tmp_path, cfg, variant="cipsym", coeff=None, ywdeg=True):
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    run = copy_dir(wd, str(tmp_path / "run"))
    jo = json.load(open(ob.run(run, variant=variant, candlog="cand.bin")))
    inp = bf.read_inputs(wd)
    model = bf.Model(inp)
    if coeff is not None:
        model.ygen = [bool(np.any(np.abs(inp.C[k]) >= coeff)) for k in range(len(inp.S))]
        assert 0 < sum(model.ygen) < len(inp.S)
    metat = inp.C.shape[1]
    diag = [model.hmp_hdig(x) for x in model.bits]
    hmp_s = np.array([d[0] for d in diag])
    hdig_s = np.array([d[1] for d in diag])
    emp = (inp.C ** 2 * hmp_s[:, None]).sum(axis=0)
    eb = (inp.C ** 2 * hdig_s[:, None]).sum(axis=0)
    np.testing.assert_allclose(jo["emp"], emp, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(jo["eb"], eb, rtol=1e-12, atol=1e-12)
    e = np.asarray(inp.E)
    # selection thresholds of cip.f:104-135: with iselec = 1, teste = t * test
    # and taum = 1 / t, t the largest |c| of the root; else test and 1
    yen, ysele = inp.ityper == 2, inp.iselec == 3
    t = np.abs(inp.C).max(axis=0)
    if inp.iselec == 1:
        teste, taum = t * inp.test, 1.0 / t
    else:
        teste, taum = np.full(metat, inp.test), np.ones(metat)
    e2 = {k: np.zeros(metat) for k in ("e2mp", "e2vp", "e2b")}
    n = 0
    dpivot = 0.0
    xam_of, selected, near = {}, [], set()
    psi = {"psimp": np.zeros(metat), "psivp": np.zeros(metat)}
    ietat = 0
    # isto.f: classes bounded by aval (deter.f:199-211 defaults), teseff = 0.05 tau
    aval = np.array([0.128e-6, 0.64e-6, 0.32e-5, 0.16e-4, 0.8e-4, 0.4e-3, 0.2e-2, 0.1e-1, 0.5e-1, 1.0])
    nclass, teseff = 10, 0.05 * inp.tau
    nom = np.zeros(nclass, dtype=np.int64)
    nam = np.zeros((metat, nclass), dtype=np.int64)
    tab = {"tabmp": np.zeros((metat, nclass)), "tabvp": np.zeros((metat, nclass))}

    def klass(v):
        below = np.nonzero(v < aval[:nclass - 1])[0]
        return int(below[0]) if len(below) else nclass - 1

    for src, k, x, nmul, fmul, b in bf.enumerate_semantic(inp, model):
        hmp, hdig = model.hmp_hdig(x)
        w = 1.0 + fmul
        b = np.asarray(b)
        b2 = b ** 2
        dmp, dvp = emp - hmp, e - hdig
        cmp_, cvp = b / dmp, b / dvp
        e2["e2mp"] += w * b2 / dmp
        if yen:
            e2["e2vp"] += w * b2 / dvp
            e2["e2b"] += w * b2 / (eb - hdig)
        n += 1
        # pert1.f:148-244: the last partition computed (EN eigenvalue with
        # yen, else MP) gives the selection value, its denominator and term
        deno, cim = (dvp, cvp) if yen else (dmp, cmp_)
        eim = b * cim
        xim = np.abs(eim) if ysele else np.abs(cim)
        ydeg = ywdeg and bool(np.any((np.abs(deno) <= 0.05) & (np.abs(eim) >= 1e-6)))
        below = xim < teste
        if np.any(below):
            dpivot = max(dpivot, float(xim[below].max()))
        xam = float((xim * taum).max())
        xam_of[(src, k, x)] = xam
        psi["psimp"] += w * cmp_ ** 2
        if yen:
            psi["psivp"] += w * cvp ** 2
        ietat += nmul + 1
        if xam >= teseff:
            vil = xim * taum
            c = klass(xam)
            nom[c] += 1 + nmul
            for m in range(metat):
                if vil[m] >= teseff:
                    tab["tabmp"][m, c] += b2[m] / dmp[m] * w
                    if yen:
                        tab["tabvp"][m, c] += b2[m] / dvp[m] * w
                    nam[m, klass(vil[m])] += 1 + nmul
        v = 1.0 if ydeg else xam
        if abs(v - inp.tau) <= 1e-9 * inp.tau:
            near.add(x)
        elif v > inp.tau:
            selected.append(x)
    assert n == jo["n_processed"]
    for key, val in e2.items():
        tol = 1e-10 + np.asarray(jo["cond_" + key]) + 1e-12 * np.abs(val)
        assert np.all(np.abs(np.asarray(jo[key]) - val) <= tol), (key, jo[key], val, tol)
    for key, val in psi.items():
        np.testing.assert_allclose(jo[key], val, rtol=1e-9, atol=1e-14, err_msg=key)
    assert jo["ietat"] == ietat
    # histogram (isto.f): counts exact, sums to the E2 tolerance
    assert list(jo["nom"]) == nom.tolist()
    assert [list(r) for r in jo["nam"]] == nam.tolist()
    for key, part in (("tabmp", "e2mp"), ("tabvp", "e2vp")):
        tol = 1e-10 + np.asarray(jo["cond_" + part])[:, None] + 1e-12 * np.abs(tab[key])
        assert np.all(np.abs(np.asarray(jo[key]) - tab[key]) <= tol), key
    # the unit-60 value of every perturber, dpivot, and the selected set
    ora = bf.read_candlog(os.path.join(run, "cand.bin"), metat)
    for r in ora:
        got = r[6]
        want = xam_of[(r[0], r[1], model.to_bits(r[2], r[3]))]
        assert abs(got - want) <= 1e-9 * abs(want) + 1e-300, (r[:4], got, want)
    assert jo["dpivot"] == pytest.approx(dpivot, rel=1e-9, abs=1e-15)
    recs = [d for d, _ in _all_records(synth.read_records(os.path.join(run, "det")), metat)]
    got_sel = collections.Counter(model.to_bits(h, p) for h, p in recs[jo["ncf"]:])
    want_sel = collections.Counter(selected)
    for x in near:
        got_sel.pop(x, None)
    assert got_sel == want_sel
