"""A seeded sweep of small random systems against the oracle: sizes, point
groups, excitation ranks of S, root counts, thresholds, the partitions
(ityper), the selection rules (iselec), ywdeg, the reference determinant in
S or not, the cip and cipsym variants, cip's coeff-restricted generators,
and one- and two-word spin strings, drawn together so that combinations the targeted tests do not
pair up are run too.  Each case is checked as the other parity tests are:
integers, counts and the selected set exactly, E2 to 1e-10 Eh plus the
oracle's condition bound."""
import numpy as np
import pytest

from cipsi_gb300 import synth
from test_gpu_parity import check, run_both

pytestmark = pytest.mark.gpu


def sweep_cases(n=20, n_wide=4, seed=20261204):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        norb = int(rng.integers(10, 21))
        nocc = int(rng.integers(3, 6))
        nsym = int(rng.choice([1, 2, 4]))
        nr = int(rng.integers(1, 4))
        ranks = tuple(sorted(int(x) for x in rng.choice([1, 2, 3, 4], size=nr, replace=False)))
        metat = int(rng.integers(1, 5))
        ncf = int(rng.integers(20, 80))
        tau = float(rng.choice([0.005, 0.02, 0.05]))
        ityper = int(rng.choice([1, 2]))
        iselec = int(rng.choice([1, 2, 3]))
        coef = str(rng.choice(["decay09", "gauss005"]))
        hf = bool(rng.random() < 0.7)
        variant = str(rng.choice(["cipsym", "cip"]))
        extra = []
        if rng.random() < 0.3:
            extra.append("ywdeg=f")
        if variant == "cip" and rng.random() < 0.5:
            extra.append(f"coeff={float(rng.choice([0.02, 0.1]))}")
        shift = float(rng.choice([0.0, 3.0]))
        name = f"sweep{i:02d}"
        cfg = synth.SynthConfig(name, norb=norb, nocc=nocc, ncholesky=norb, ncf=ncf, metat=metat, tau=tau,
                                ityper=ityper, iselec=iselec, ranks=ranks, coef_mode=coef, seed=1000 + i,
                                nsym=nsym, include_hf=hf, variant=variant, extra_icinp=", ".join(extra),
                                virt_shift=shift)
        out.append((name, cfg, variant))
    # two 64-bit words per spin string (65-90 orbitals), S of singles and
    # doubles, either variant
    for i in range(n_wide):
        norb = int(rng.integers(65, 91))
        nocc = int(rng.integers(3, 6))
        variant = str(rng.choice(["cipsym", "cip"]))
        name = f"wide{i}"
        cfg = synth.SynthConfig(name, norb=norb, nocc=nocc, ncholesky=24, ncf=int(rng.integers(20, 60)),
                                metat=int(rng.integers(1, 4)), tau=float(rng.choice([0.005, 0.02])),
                                ityper=int(rng.choice([1, 2])), iselec=int(rng.choice([1, 2, 3])),
                                ranks=(1, 2), coef_mode=str(rng.choice(["decay09", "gauss005"])), seed=2000 + i,
                                nsym=int(rng.choice([1, 2])), variant=variant)
        out.append((name, cfg, variant))
    return out


@pytest.mark.parametrize("name,cfg,variant", sweep_cases(), ids=[c[0] for c in sweep_cases()])
def test_parity_sweep(tmp_path, oracle_exe, engine_lib, name, cfg, variant):
    jo, jg, wo, wg = run_both(tmp_path, cfg, variant=variant)
    check(jo, jg, wo, wg, variant)


def moy_sweep_cases(seed=20261205):
    """The one-word cipsym systems of the sweep (their unit 60 holds at most
    a few tens of thousands of records: moy's pair scan is O(n^2) in the
    oracle), each with a moy threshold and options drawn for it."""
    rng = np.random.default_rng(seed)
    out = []
    for name, cfg, variant in sweep_cases(n_wide=0):
        if variant != "cipsym":
            continue
        tau = float(rng.choice([0.0, 0.0, 0.01, 0.05]))
        extra = "y_secd=t" if rng.random() < 0.3 else ""
        out.append((name, cfg, tau, extra))
    return out


@pytest.mark.parametrize("name,cfg,tau,extra", moy_sweep_cases(), ids=[c[0] for c in moy_sweep_cases()])
def test_moy_sweep(tmp_path, oracle_exe, engine_lib, name, cfg, tau, extra):
    """moy_gpu against the oracle's moy on the unit 60 of the oracle's
    cipsym run of each sweep system: lists, unit 1 and morue's sums, as
    tests/test_gpu_moy.py compares them."""
    import shutil

    import cipsi_gb300 as cg
    import moy_files as mf
    from test_gpu_moy import _compare
    wo = str(tmp_path / "ora")
    mf.prepare(wo, cfg, moy_tau=tau, extra=extra)
    wg = str(tmp_path / "gpu")
    shutil.copytree(wo, wg)
    jo = mf.run_oracle_moy(wo)
    jg = cg.run_moy(wg)
    _compare(wo, wg, jo, jg)
