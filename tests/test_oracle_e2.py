"""The oracle's E2 sums against E2 recomputed from the independent brute-force
model: the model's perturber set, spin-flip weights and couplings
b_m = <I|H|Psi_m>, its own diagonal energies (hmp, hdig from the closed-shell
F, J, K), and the textbook partitions of pert1.f:148-191 --

    E2_MP(m)  = sum_I (1 + fmul_I) b_m^2 / (emp_m - hmp(I))
    E2_ENvp(m) = sum_I (1 + fmul_I) b_m^2 / (e_m  - hdig(I))
    E2_ENb(m)  = sum_I (1 + fmul_I) b_m^2 / (eb_m - hdig(I))

with emp_m = sum_k c_km^2 hmp(k), eb_m = sum_k c_km^2 hdig(k) over S
(cip.f:99-120).  Together with the set and coupling checks of
test_oracle_semantics this pins the oracle's arithmetic, not only its
enumeration.  Tolerance: 1e-10 Eh plus the oracle's first-order rounding
bound of each sum (cond_e2*), which is tiny on the well-conditioned systems
(virtual orbitals shifted up) and covers the near-zero denominators of the
plain recipe."""
import json

import numpy as np
import pytest

import brute_force as bf
from cases import small_cases
from cipsi_gb300 import synth
from conftest import copy_dir
from oracle import build as ob


def _gap(seed, ranks, nsym):
    return synth.SynthConfig("gap", norb=16, nocc=4, ncholesky=16, ncf=60, metat=2, tau=0.01, ranks=ranks,
                             coef_mode="gauss005", seed=seed, nsym=nsym, virt_shift=3.0)


CASES = [("gap31", _gap(31, (2,), 1)), ("gap32", _gap(32, (1, 2, 3), 1)), ("gap33", _gap(33, (1, 2), 2))]
CASES += small_cases()


@pytest.mark.parametrize("name,cfg", CASES, ids=[c[0] for c in CASES])
def test_oracle_e2_matches_bruteforce_sums(tmp_path, oracle_exe, name, cfg):
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    run = copy_dir(wd, str(tmp_path / "run"))
    jo = json.load(open(ob.run(run, variant="cipsym")))
    inp = bf.read_inputs(wd)
    model = bf.Model(inp)
    metat = inp.C.shape[1]
    diag = [model.hmp_hdig(x) for x in model.bits]
    hmp_s = np.array([d[0] for d in diag])
    hdig_s = np.array([d[1] for d in diag])
    emp = (inp.C ** 2 * hmp_s[:, None]).sum(axis=0)
    eb = (inp.C ** 2 * hdig_s[:, None]).sum(axis=0)
    np.testing.assert_allclose(jo["emp"], emp, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(jo["eb"], eb, rtol=1e-12, atol=1e-12)
    e = np.asarray(inp.E)
    e2 = {k: np.zeros(metat) for k in ("e2mp", "e2vp", "e2b")}
    n = 0
    for src, k, x, nmul, fmul, b in bf.enumerate_semantic(inp, model):
        hmp, hdig = model.hmp_hdig(x)
        w = 1.0 + fmul
        b2 = np.asarray(b) ** 2
        e2["e2mp"] += w * b2 / (emp - hmp)
        e2["e2vp"] += w * b2 / (e - hdig)
        e2["e2b"] += w * b2 / (eb - hdig)
        n += 1
    assert n == jo["n_processed"]
    for key, val in e2.items():
        tol = 1e-10 + np.asarray(jo["cond_" + key]) + 1e-12 * np.abs(val)
        assert np.all(np.abs(np.asarray(jo[key]) - val) <= tol), (key, jo[key], val, tol)
