"""The oracle's S-space CI (ic001.f:81-131: a perturbation run with lecdet !=
5 diagonalises H over S itself) against the brute-force model, and against
the lecdet = 5 path fed with the same vectors (CPU only).

The model builds H over S from its own Slater-Condon rules (canonical
phases times the excitation-list phases, hdig on the diagonal); the
oracle's root energies must be H's lowest eigenvalues and its vectors (read
back from the zero-order record of unit 4) eigenvectors of H.  A lecdet = 5
run whose unit 59 holds those vectors must then give the same E2, counts
and selection as the S-space CI run, bit for bit."""
import json
import os
import shutil
import struct

import numpy as np
import pytest

import brute_force as bf
from cipsi_gb300 import synth
from oracle import build as ob
from test_autocip_s_runs import _write_icinp

CAS = (" NUMAC=3,4,5,6,7,8,9,10,\n NUSYM=1,\n NOAC=8,\n NELAC=2,\n NEMAX=2,\n")


def _chain_cfg(seed=41, nsym=1):
    return synth.SynthConfig("sci", norb=12, nocc=3, ncholesky=12, ncf=40, metat=2, tau=0.02,
                             ranks=(1, 2), coef_mode="gauss005", seed=seed, virt_shift=3.0, nsym=nsym)


def _unit4_space_and_vectors(path):
    """S (holes, particles) and c[metat, ncf] from the zero-order record."""
    rec = synth.read_records(path)[0]
    norb, noca, nocb, metat, ncf = struct.unpack_from("<5i", rec, 0)
    ii, jj = struct.unpack_from("<ii", rec, 25)
    off = 33
    nend = np.frombuffer(rec, dtype="<i4", count=2 * ncf, offset=off).reshape(ncf, 2)
    off += 8 * ncf
    tp = np.frombuffer(rec, dtype="<i4", count=2 * ii, offset=off).reshape(ii, 2)
    off += 8 * ii
    c = np.frombuffer(rec, dtype="<f8", count=jj, offset=off).reshape(metat, ncf)
    dets = [(tuple(int(x) for x in tp[nd:nd + ne, 0]), tuple(int(x) for x in tp[nd:nd + ne, 1])) for ne, nd in nend]
    return dets, c


def _model_h(wd_inputs, dets):
    inp = bf.read_inputs(wd_inputs)
    m = bf.Model(inp)
    bits = [m.to_bits(h, p) for h, p in dets]
    sig = np.array([synth.cip_phase(h, p, m.n, inp.nocc) for h, p in dets], dtype=float)
    n = len(dets)
    H = np.zeros((n, n))
    for i in range(n):
        H[i, i] = m.hmp_hdig(bits[i])[1]
        for j in range(i):
            if bf.degree(bits[i], bits[j]) <= 2:
                H[i, j] = H[j, i] = sig[i] * sig[j] * m.hmat(bits[i], bits[j])
    return H


@pytest.mark.parametrize("lecdet", [4, 2])
def test_s_space_ci_matches_model_and_lecdet5(tmp_path, oracle_exe, lecdet):
    cfg = _chain_cfg()
    src = str(tmp_path / "src")
    synth.generate(cfg, src)  # unit 59 of the generated S lets the model read its inputs
    wd = str(tmp_path / "sci")
    shutil.copytree(src, wd)
    body = "metat=2, ityper=2, tau=0.01, test=0.01, iselec=1, ymoyen=t, ybrd=f, ywvf=f, twdet=0.5"
    if lecdet == 4:
        _write_icinp(wd, body + ", lecdet=4,\n" + CAS)
    else:
        _write_icinp(wd, body + ", lecdet=2, tdet=0.0")
    w5 = str(tmp_path / "l5")
    shutil.copytree(wd, w5)
    jo = json.load(open(ob.run(wd, variant="cipsym")))
    dets, c = _unit4_space_and_vectors(os.path.join(wd, "f04"))
    H = _model_h(src, dets)
    w, _ = np.linalg.eigh(H)
    np.testing.assert_allclose(jo["e"], w[:2], rtol=0, atol=1e-10)
    for m in range(2):
        assert np.linalg.norm(H @ c[m] - jo["e"][m] * c[m]) < 1e-9
        assert abs(np.linalg.norm(c[m]) - 1) < 1e-12
    # the same run through lecdet = 5 with these vectors on unit 59: S from
    # unit 60, so unit 60 must hold this S first (the S-only run writes it)
    escf = struct.unpack_from("<d", synth.read_records(os.path.join(src, "ener"))[0], 44)[0]
    with open(os.path.join(w5, "bdvec"), "wb") as fh:
        synth.write_record(fh, struct.pack("<ii", len(dets), 2) + c.astype("<f8").tobytes()
                           + (np.array(jo["e"]) + escf).astype("<f8").tobytes())
    with open(os.path.join(w5, "det"), "wb") as fh:  # S in the order of unit 4, v = 1
        idet, nex = [], []
        for h, p in dets:
            for t, q in zip(h, p):
                idet += [t, q]
            nex.append(len(h))
        synth.write_record(fh, struct.pack("<ii", len(idet), len(dets)) + np.array(idet, "<i4").tobytes()
                           + np.array(nex, "<i4").tobytes() + np.ones(len(dets), "<f8").tobytes()
                           + np.zeros(2 * len(dets), "<f8").tobytes())
    with open(os.path.join(w5, "f04"), "wb") as fh:  # lecdet = 5 reads ncf from unit 4
        synth.write_record(fh, struct.pack("<5i", cfg.norb, cfg.nocc, cfg.nocc + cfg.norb, 2, len(dets)))
    _write_icinp(w5, body + ", lecdet=5")
    j5 = json.load(open(ob.run(w5, variant="cipsym")))
    assert j5["ncf"] == jo["ncf"]
    for k in ("ietat", "n_processed", "ntot60", "nom", "nam"):
        assert j5[k] == jo[k], k
    for k in ("e2mp", "e2vp", "e2b", "psimp", "psivp"):
        np.testing.assert_allclose(j5[k], jo[k], rtol=1e-13, atol=1e-14, err_msg=k)
