"""The moy drop-in (GPU pair scan and matrix elements, cipsi_moy_main) against
the oracle's restatement of moy on the same files.

Byte for byte: the determinant lists (units 64, 61), the MP diagonal (unit
63), the row and column of every unit-1 element and the record layout,
including what the last record keeps from the one before.  Floating point:
the unit-1 values to 1e-12 (relative, 1e-13 absolute; the one-difference
elements sum their integral terms in another order), morue's second-order
sums (unit 33 records and the fourth unit-4 record) to 1e-9 relative."""
import os
import shutil
import struct

import numpy as np
import pytest

import cipsi_gb300 as cg
import moy_files as mf
from cases import small_cases
from cipsi_gb300 import synth
from oracle import build as ob

pytestmark = pytest.mark.gpu

CASES = {name: cfg for name, cfg in small_cases()}


def _compare(wo, wg, jo, jg):
    for k in ("ncf", "ndims", "nhntd", "nhij", "unit1_records"):
        assert jo[k] == jg[k], k
    for f in ("det_spin", "det_cl", "enmp"):
        assert os.path.exists(os.path.join(wo, f)) == os.path.exists(os.path.join(wg, f)), f
        if os.path.exists(os.path.join(wo, f)):
            assert open(os.path.join(wo, f), "rb").read() == open(os.path.join(wg, f), "rb").read(), f
    ro, Io, Jo, Vo = mf.read_unit1(os.path.join(wo, "mat"))
    rg, Ig, Jg, Vg = mf.read_unit1(os.path.join(wg, "mat"))
    assert len(ro) == len(rg)
    for (a, b, c), (x, y, z) in zip(ro, rg):
        assert np.array_equal(a, x) and np.array_equal(b, y)
        np.testing.assert_allclose(z, c, rtol=1e-12, atol=1e-13)
    assert np.array_equal(Io, Ig) and np.array_equal(Jo, Jg)
    d = Io == Jo
    assert np.array_equal(Vo[d], Vg[d])  # diagonal: the same host arithmetic
    e33o = synth.read_records(os.path.join(wo, "ener"))
    e33g = synth.read_records(os.path.join(wg, "ener"))
    assert len(e33o) == len(e33g)
    for a, b in zip(e33o, e33g):  # the records cip wrote, then morue's (char*40, real*8 x metat)
        assert len(a) == len(b) and a[:40] == b[:40]
        if a[:6] == b"moyens":
            np.testing.assert_allclose(np.frombuffer(b[40:], "<f8"), np.frombuffer(a[40:], "<f8"), rtol=1e-9,
                                       atol=1e-12)
        else:
            assert a == b
    r4o = synth.read_records(os.path.join(wo, "f04"))
    r4g = synth.read_records(os.path.join(wg, "f04"))
    assert len(r4o) == len(r4g) == 4
    assert r4o[:3] == r4g[:3]
    mmm = 3 * jo["metat"] * (jo["metat"] + 1) // 2
    np.testing.assert_allclose(np.frombuffer(r4g[3], "<f8", count=mmm), np.frombuffer(r4o[3], "<f8", count=mmm),
                               rtol=1e-9, atol=1e-12)
    assert r4o[3][8 * mmm:] == r4g[3][8 * mmm:]


def _both(tmp_path, prep):
    wo = str(tmp_path / "ora")
    prep(wo)
    wg = str(tmp_path / "gpu")
    shutil.copytree(wo, wg)
    jo = mf.run_oracle_moy(wo)
    jg = cg.run_moy(wg)
    _compare(wo, wg, jo, jg)
    return jo, jg


@pytest.mark.parametrize("name,tau,extra", [("small", 0.0, ""), ("small", 0.05, ""), ("mix1", 0.0, ""),
                                            ("mix2", 0.0, ""), ("mix4", 0.0, ""), ("mix1", 0.0, "y_secd=t")])
def test_moy_matches_oracle(tmp_path, oracle_exe, engine_lib, name, tau, extra):
    """After a cipsym perturbation run: S + the selected perturbers
    (several thousand determinants, symmetry groups of order 1, 2, 4)."""
    jo, jg = _both(tmp_path, lambda wd: mf.prepare(wd, CASES[name], moy_tau=tau, extra=extra))
    assert jo["ncf"] > jo["ndims"]
    assert jg["pairs"] >= jg["nhntd"] - jg["ncf"]


def _two_word(wd, ncf_s, ncf_60, seed):
    """120 orbitals (two 64-bit words per spin string): unit 4 from the run
    that only writes S (S of ncf_s determinants), unit 60 replaced by the
    determinants of a larger S drawn from the same recipe, so that the list
    holds S and ncf_60 - ncf_s others; morue then has rows beyond S."""
    import dataclasses
    base = synth.SynthConfig("w2", norb=120, nocc=15, ncholesky=60, ncf=ncf_s, metat=2, tau=0.005,
                             ranks=(1, 2), coef_mode="gauss005", seed=seed, virt_shift=3.0)
    synth.generate(base, wd)
    txt = open(os.path.join(wd, "cip.in")).read().replace("ityper=2", "ityper=-1")
    open(os.path.join(wd, "cip.in"), "w").write(txt)
    ob.run(wd, variant="cipsym")
    big = str(wd) + "_big"
    synth.generate(dataclasses.replace(base, ncf=ncf_60), big)
    shutil.copy(os.path.join(big, "det"), os.path.join(wd, "det"))
    shutil.rmtree(big)
    with open(os.path.join(wd, "moy.in"), "w") as fh:
        fh.write(" &moyfil\n &end\n &moyen\n  tau=0d0, ystkmp=t, title='w2'\n &end\n")


def test_moy_two_word_strings(tmp_path, oracle_exe, engine_lib):
    """norb = 120: the W = 2 kernels over a list of 3000 determinants (many
    256-row blocks and 512-column tiles)."""
    jo, jg = _both(tmp_path, lambda wd: _two_word(wd, 400, 3000, 41))
    assert jo["ncf"] > 2500


def test_moy_s_only_list(tmp_path, oracle_exe, engine_lib):
    """Autocip's use: the S written by the run that only writes S (ndims =
    ncf: morue writes a zero fourth record to unit 4)."""
    def prep(wd):
        synth.generate(CASES["mix0"], wd)
        txt = open(os.path.join(wd, "cip.in")).read().replace("ityper=2", "ityper=-1")
        open(os.path.join(wd, "cip.in"), "w").write(txt)
        ob.run(wd, variant="cipsym")
        with open(os.path.join(wd, "moy.in"), "w") as fh:
            fh.write(" &moyfil\n &end\n &moyen\n  tau=0d0\n &end\n")
    jo, jg = _both(tmp_path, prep)
    assert jo["ncf"] == jo["ndims"]
