"""Two iterations of the Autocip CIPSI loop (Autocip_13/calcul.f90:304-357)
through the drop-in's unit files:

  cipsym ITYPER=-1 LECDET=4   the CAS, ordered, written to units 60 and 4
  moy + bd                     here: exact diagonalisation of H over S
                               (numpy), vectors and energies to unit 59
  cipsym ITYPER=2  LECDET=5   E2 and the selection appended to unit 60
  cipsym ITYPER=-1 LECDET=5   S grown by the selection, ordered, written
  moy + bd, cipsym ITYPER=2   again on the larger S

The S-only runs are made by the drop-in (engine library, no GPU) and checked
byte for byte against the oracle; the perturbation runs are the oracle's (the
GPU's are compared with the oracle in the gpu-marked parity tests).  Checks:
the files of one step are accepted by the next, S grows by exactly the
selected determinants (closed under the spin flip), and the variational
energy of the lowest root does not rise."""
import json
import os
import shutil
import struct

import numpy as np

from cipsi_gb300 import synth

from test_autocip_s_runs import _unit60_dets, _write_icinp


def _space_in_deter_order(wd, metat):
    """S as the perturbation run builds it from unit 60 (deter.f:478-567):
    the zero-order record that an S-only run without ymoyen writes."""
    import cipsi_gb300
    d = wd + "_order"
    shutil.rmtree(d, ignore_errors=True)
    shutil.copytree(wd, d)
    _write_icinp(d, f"metat={metat}, ityper=-1, lecdet=5, ymoyen=f, iselec=1")
    cipsi_gb300.run_cip(d, variant="cipsym")
    rec = synth.read_records(os.path.join(d, "f04"))[0]
    ncf = struct.unpack_from("<5i", rec, 0)[4]
    off = 25
    ii, _ = struct.unpack_from("<ii", rec, off)
    off += 8
    nend = np.frombuffer(rec, dtype="<i4", count=2 * ncf, offset=off).reshape(ncf, 2)
    off += 8 * ncf
    tp = np.frombuffer(rec, dtype="<i4", count=2 * ii, offset=off).reshape(ii, 2)
    dets = []
    for ne, nd in nend:
        dets.append((tuple(int(x) for x in tp[nd:nd + ne, 0]), tuple(int(x) for x in tp[nd:nd + ne, 1])))
    return dets


def _moy_bd(wd, cfg, metat):
    """Lowest `metat` roots of H over S, in the reference phase, to unit 59."""
    dets = _space_in_deter_order(wd, metat)
    h, L, _ = synth.make_integrals(cfg, np.random.default_rng(cfg.seed))
    sc = synth.SlaterCondon(h, L, cfg.norb, cfg.nocc)
    bits = [synth.det_from_lists(hl, pt, cfg.norb, cfg.nocc) for hl, pt in dets]
    hf = (1 << cfg.nocc) - 1
    ehf = sc.diag(hf, hf)
    n = len(bits)
    H = np.zeros((n, n))
    for i in range(n):
        H[i, i] = sc.diag(*bits[i]) - ehf
        for j in range(i):
            dx = synth.popcount(bits[i][0] ^ bits[j][0]) + synth.popcount(bits[i][1] ^ bits[j][1])
            if dx <= 4:
                H[i, j] = H[j, i] = sc.offdiag(bits[i][0], bits[i][1], bits[j][0], bits[j][1])
    w, V = np.linalg.eigh(H)
    escf = struct.unpack_from("<d", synth.read_records(os.path.join(wd, "ener"))[0], 44)[0]
    sigma = np.array([synth.cip_phase(hl, pt, cfg.norb, cfg.nocc) for hl, pt in dets], dtype=np.float64)
    C = V[:, :metat] * sigma[:, None]
    E = w[:metat] + escf
    with open(os.path.join(wd, "bdvec"), "wb") as fh:
        synth.write_record(fh, struct.pack("<ii", n, metat) + C.T.astype("<f8").tobytes()
                           + E.astype("<f8").tobytes())
    return dets, w[:metat]


def _s_only_both(wd, body):
    """An S-only run by the oracle and by the drop-in; identical files."""
    import cipsi_gb300
    from oracle import build as ob
    wo = wd + "_s_oracle"
    shutil.rmtree(wo, ignore_errors=True)
    shutil.copytree(wd, wo)
    _write_icinp(wo, body)
    ob.run(wo, variant="cipsym")
    _write_icinp(wd, body)
    cipsi_gb300.run_cip(wd, variant="cipsym")
    for u in ("det", "f04"):
        assert open(os.path.join(wo, u), "rb").read() == open(os.path.join(wd, u), "rb").read(), u


def _e2_run(wd, metat, tau):
    from oracle import build as ob
    _write_icinp(wd, f"metat={metat}, ityper=2, lecdet=5, tau={tau}, test={tau}, iselec=1, "
                     f"ymoyen=t, ybrd=f, ywvf=f, twdet=0.5")
    return json.load(open(ob.run(wd, variant="cipsym")))


def _flip_closure(dets, norb):
    out = set(dets)
    for hl, pt in dets:
        fh, fp = synth.flip_lists(hl, pt, norb)
        out.add((tuple(fh), tuple(fp)))
    return out


def test_two_cipsi_iterations_through_the_drop_in(tmp_path, engine_lib, oracle_exe):
    cfg = synth.SynthConfig("chain", norb=12, nocc=3, ncholesky=12, ncf=10, metat=2, tau=0.02,
                            ranks=(1, 2), coef_mode="gauss005", seed=41, virt_shift=3.0)
    wd = str(tmp_path / "chain")
    synth.generate(cfg, wd)
    for u in ("det", "bdvec", "f04"):
        os.remove(os.path.join(wd, u))
    metat, tau = 2, 0.01
    # iteration 1: the CAS of 2 electrons in orbitals 3..10
    _s_only_both(wd, "NUMAC=3,4,5,6,7,8,9,10,\n twdet=0.5\n ISZ=0, NUSYM=1, NOAC=8, METAT=2, LECDET=4,\n"
                     " ITYPER=-1, YMOYEN=T, NELAC=2, YBRD=F, NEMAX=2, YION=F, ISELEC=  1,\n TEST=0d0, TAU=0d0,")
    S1 = _unit60_dets(os.path.join(wd, "det"), metat, True)
    assert len(S1) == 64  # C(8,1)^2, all of symmetry 1
    dets1, w1 = _moy_bd(wd, cfg, metat)
    assert set(dets1) == set(S1)
    r1 = _e2_run(wd, metat, tau)
    assert r1["ncf"] == len(S1) and r1["ntot60"] > r1["ncf"]
    recs = synth.read_records(os.path.join(wd, "det"))
    selected = [d for d in _all_records(recs, metat) if d[1] != 1.0]
    assert len(selected) == r1["ntot60"] - r1["ncf"] and all(v > tau for _, v in selected)
    # iteration 2: S grows by the selection (and its spin-flip partners)
    _s_only_both(wd, f"metat={metat}, ityper=-1, lecdet=5, ymoyen=t, iselec=1, twdet=0.5")
    S2 = _unit60_dets(os.path.join(wd, "det"), metat, True)
    assert len(S2) == len(set(S2))
    assert set(S2) == _flip_closure(list(S1) + [d for d, _ in selected], cfg.norb)
    dets2, w2 = _moy_bd(wd, cfg, metat)
    assert set(dets2) == set(S2)
    assert w2[0] <= w1[0] + 1e-12  # the variational energy does not rise
    r2 = _e2_run(wd, metat, tau)
    assert r2["ncf"] == len(S2) and all(np.isfinite(r2["e2vp"]))
    # the larger S leaves less to the perturbation (-2.65 -> -0.23 Eh here)
    assert abs(r2["e2vp"][0]) < 0.5 * abs(r1["e2vp"][0])


def _all_records(recs, metat):
    """(determinant, v) of every unit-60 record, in file order."""
    out = []
    for rec in recs:
        mw, nw = struct.unpack_from("<ii", rec, 0)
        idet = np.frombuffer(rec, dtype="<i4", count=mw, offset=8)
        nex = np.frombuffer(rec, dtype="<i4", count=nw, offset=8 + 4 * mw)
        v = np.frombuffer(rec, dtype="<f8", count=nw, offset=8 + 4 * mw + 4 * nw)
        my = 0
        for n, x in zip(nex, v):
            pairs = idet[my: my + 2 * n].reshape(-1, 2)
            my += 2 * n
            out.append(((tuple(sorted(int(t) for t in pairs[:, 0])), tuple(sorted(int(p) for p in pairs[:, 1]))),
                        float(x)))
    return out
