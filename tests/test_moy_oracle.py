"""The oracle's restatement of moy (the Hamiltonian over S + the selected
perturbers, moy/moy.f) against an independent model, and the drop-in's
determinant lists against the oracle's (CPU only).

Model: the determinant set is the unit-60 records with value >= tau and
their spin-flip partners; every element of unit 1 is sigma_i sigma_j <i|H|j>
from the brute-force Slater-Condon rules (canonical phases, sigma = the
phase of the excitation lists), every row holds exactly the columns j < i
within two excitations whose element is not below 1e-10, then its diagonal
hdig(i)/2 (closed-shell F, J, K, the Fock matrix as unit 40 holds it); and
morue's second-order sums are recomputed with numpy from the stored
elements and the S coefficients of unit 4."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import brute_force as bf
import moy_files as mf
from cases import small_cases
from cipsi_gb300 import synth

CASES = {name: cfg for name, cfg in small_cases()}


def _model(workdir_inputs):
    inp = bf.read_inputs(workdir_inputs)
    recs = synth.read_records(os.path.join(workdir_inputs, "ijkl"))
    inp.F = np.concatenate([[0.0], np.frombuffer(recs[5], dtype="<f8")])  # moy/ijkf.f: F as it stands
    return bf.Model(inp)


def _bits(model, dets):
    return [model.to_bits(h, p) for h, p in dets]


def _check(tmp_path, name, moy_tau, extra="", nsample=2500):
    cfg = CASES[name]
    src = str(tmp_path / "in")
    synth.generate(cfg, src)
    model = _model(src)
    wd = str(tmp_path / "run")
    mf.prepare(wd, cfg, moy_tau=moy_tau, extra=extra)
    jo = mf.run_oracle_moy(wd)
    n = model.n
    dets, raw = mf.read_unit64(os.path.join(wd, "det_spin"))
    assert jo["ncf"] == len(dets)
    # the set: unit-60 records >= tau and their partners, no repeats, by degree
    recs = mf.read_unit60_dets(os.path.join(wd, "det"), moy_tau)
    want = set(recs) | {tuple(map(tuple, synth.flip_lists(h, p, n))) for h, p in recs if h}
    assert set(dets) == want
    assert len(set(dets)) == len(dets)
    deg = [len(h) for h, _ in dets]
    assert deg == sorted(deg)
    assert np.all(raw["iorb"][:2 * n] == np.r_[np.arange(1, n + 1), np.arange(1, n + 1)])
    assert np.all(raw["ispin"][:2 * n] == np.r_[np.zeros(n, int), np.ones(n, int)])
    # unit 1
    bits = _bits(model, dets)
    ndims = jo["ndims"]
    y_secd = "y_secd=t" in extra
    _, I, J, V = mf.read_unit1(os.path.join(wd, "mat"))
    assert len(I) == jo["nhij"]
    # rows in order, each ending with its diagonal
    diag_pos = np.nonzero(I == J)[0]
    assert np.all(I[diag_pos] == np.arange(1, len(dets) + 1))
    assert np.all(np.diff(I) >= 0)
    starts = np.r_[0, diag_pos[:-1] + 1]
    alpha = np.array([b & ((1 << n) - 1) for b in bits], dtype=np.uint64)
    beta = np.array([b >> n for b in bits], dtype=np.uint64)
    sig = np.array([synth.cip_phase(h, p, n, model.inp.nocc) for h, p in dets], dtype=float)
    missing = []
    for i in range(len(dets)):
        cols = J[starts[i]:diag_pos[i]] - 1
        assert np.all(np.diff(cols) > 0)
        jl = min(i, ndims) if y_secd else i
        d = np.bitwise_count(alpha[:jl] ^ alpha[i]) + np.bitwise_count(beta[:jl] ^ beta[i])
        near = np.nonzero(d <= 4)[0]
        assert set(cols.tolist()) <= set(near.tolist())
        for j in set(near.tolist()) - set(cols.tolist()):
            missing.append((i, j))
    for i, j in missing:  # dropped elements are below 1e-10
        assert abs(model.hmat(bits[i], bits[j])) < 1e-10 + 1e-12
    rng = np.random.default_rng(5)
    off = np.nonzero(I != J)[0]
    for t in rng.choice(off, size=min(nsample, len(off)), replace=False):
        i, j = int(I[t]) - 1, int(J[t]) - 1
        h = sig[i] * sig[j] * model.hmat(bits[i], bits[j])
        assert V[t] == pytest.approx(h, rel=1e-11, abs=1e-12), (i, j)
    stefen = np.zeros(len(dets))
    for i in range(len(dets)):
        hmp_i, e_i = model.hmp_hdig(bits[i])
        assert V[diag_pos[i]] == pytest.approx(0.5 * e_i, rel=1e-12, abs=1e-12)
        stefen[i] = 2.0 * V[diag_pos[i]]
    # unit 63 (ystkmp): MP diagonal energies
    stefmp = np.frombuffer(synth.read_records(os.path.join(wd, "enmp"))[0], dtype="<f8")
    for i in range(0, len(dets), 7):
        assert stefmp[i] == pytest.approx(model.hmp_hdig(bits[i])[0], rel=1e-12, abs=1e-12)
    # unit 61: the lists one determinant at a time
    r61 = synth.read_records(os.path.join(wd, "det_cl"))
    q = 0
    for h, p in dets:
        assert struct.unpack("<i", r61[q])[0] == len(h)
        q += 1
        if h:
            assert r61[q] == struct.pack(f"<{2 * len(h)}i", *h, *p)
            q += 1
    assert q == len(r61)
    # morue: second order of the rows beyond S, from the stored elements
    _check_morue(wd, jo, I, J, V, stefen, stefmp)
    return jo


def _check_morue(wd, jo, I, J, V, stefen, stefmp):
    r4 = synth.read_records(os.path.join(wd, "f04"))
    assert len(r4) == 4
    b = r4[0]
    norb, noca, nocb, metat, ndims, isz = struct.unpack_from("<6i", b, 0)
    ii, jj = struct.unpack_from("<2i", b, 25)
    pos = 33 + 8 * ndims + 8 * ii
    c = np.frombuffer(b, dtype="<f8", count=jj, offset=pos).reshape(metat, ndims)
    pos += 8 * jj
    e, ebmp, eben = (np.frombuffer(b, dtype="<f8", count=metat, offset=pos + 8 * metat * q) for q in range(3))
    mmm = metat * (metat + 1) // 2
    hm, he, hb = np.zeros(mmm), np.zeros(mmm), np.zeros(mmm)
    if ndims != jo["ncf"]:
        rows = (I > ndims) & (I != J) & (J <= ndims) & (I != 1)
        cunt = np.zeros((jo["ncf"] + 1, metat))
        np.add.at(cunt, I[rows], V[rows, None] * c.T[J[rows] - 1])
        for k in range(ndims + 1, jo["ncf"] + 1):
            ii_ = 0
            for m in range(metat):
                for nn in range(m + 1):
                    hmn = 2.0 * cunt[k, m] * cunt[k, nn]
                    hm[ii_] += hmn / (ebmp[m] + ebmp[nn] - 2 * stefmp[k - 1])
                    he[ii_] += hmn / (e[m] + e[nn] - 2 * stefen[k - 1])
                    hb[ii_] += hmn / (eben[m] + eben[nn] - 2 * stefen[k - 1])
                    ii_ += 1
    for key, ref in (("hefmp", hm), ("hefen", he), ("hefenb", hb)):
        np.testing.assert_allclose(jo[key], ref, rtol=1e-9, atol=1e-12, err_msg=key)
    rec4 = np.frombuffer(r4[3], dtype="<f8", count=3 * mmm)
    np.testing.assert_array_equal(rec4, np.r_[jo["hefmp"], jo["hefen"], jo["hefenb"]])
    assert struct.unpack_from("<i", r4[3], 24 * mmm)[0] == 0


@pytest.mark.parametrize("name,tau", [("small", 0.05), ("mix1", 0.0), ("mix2", 0.0), ("mix4", 0.0)])
def test_moy_oracle_matches_model(tmp_path, oracle_exe, name, tau):
    """Determinant list, unit 1 (structure, every dropped element, a sample of
    stored elements, every diagonal), units 61, 63, 64, and morue's sums."""
    jo = _check(tmp_path, name, tau)
    assert jo["ncf"] > jo["ndims"]


def test_moy_oracle_y_secd(tmp_path, oracle_exe):
    """y_secd: columns limited to the first ndims determinants (moy.f:128)."""
    _check(tmp_path, "mix1", 0.0, extra="y_secd=t")


def test_moy_oracle_s_only_list(tmp_path, oracle_exe):
    """Autocip's use: unit 60 of the run that only writes S, so the list is S
    (ndims = ncf) and morue writes zeros."""
    cfg = CASES["mix0"]
    wd = str(tmp_path / "run")
    synth.generate(cfg, wd)
    txt = open(os.path.join(wd, "cip.in")).read().replace("ityper=2", "ityper=-1")
    open(os.path.join(wd, "cip.in"), "w").write(txt)
    from oracle import build as ob
    ob.run(wd, variant="cipsym")
    with open(os.path.join(wd, "moy.in"), "w") as fh:
        fh.write(" &moyfil\n &end\n &moyen\n  tau=0d0, ystkmp=t\n &end\n")
    jo = mf.run_oracle_moy(wd)
    assert jo["ncf"] == jo["ndims"]
    assert jo["hefmp"] == [0.0] * (jo["metat"] * (jo["metat"] + 1) // 2)


@pytest.mark.parametrize("name,tau", [("small", 0.05), ("mix2", 0.0)])
def test_moy_drop_in_lists_match_oracle(tmp_path, oracle_exe, engine_lib, name, tau):
    """The drop-in's determinant lists (units 64 and 61) byte for byte against
    the oracle's; yrcmp stops both before the matrix (moy.f:106-107), so this
    runs without a GPU."""
    cfg = CASES[name]
    wo = str(tmp_path / "ora")
    mf.prepare(wo, cfg, moy_tau=tau, extra="yrcmp=t")
    wg = str(tmp_path / "gpu")
    shutil.copytree(wo, wg)
    mf.run_oracle_moy(wo)
    from cipsi_gb300 import build
    exe = os.path.join(os.path.dirname(build.LIB), "moy_gpu")
    with open(os.path.join(wg, "moy.in")) as fin:
        r = subprocess.run([exe], cwd=wg, stdin=fin, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    for f in ("det_spin", "det_cl"):
        assert open(os.path.join(wo, f), "rb").read() == open(os.path.join(wg, f), "rb").read(), f
    assert not os.path.exists(os.path.join(wg, "mat"))
