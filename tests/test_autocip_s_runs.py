"""The runs of cipsym that only write S (ityper < 0), as the Autocip driver
makes them before each perturbation run (Autocip_13/calcul.f90:318-321):
S read from unit 60 (lecdet = 5) or generated as a complete active space
(lecdet = 4, cip/cas.f), ordered by increasing diagonal energy (shell.f,
cip/cip.f:200-206), written to unit 60 and unit 4, and no perturbation.

These runs do no device work, so the drop-in (the engine library's
cipsi_cip_main) runs here on the CPU; its unit files are compared byte for
byte with the oracle's, and the determinant sets and their order with an
independent model (combinatorics of the active space, EN diagonal energies
from the closed-shell F, J, K)."""
import itertools
import os
import shutil
import struct

import numpy as np
import pytest

from cipsi_gb300 import synth

import cases


def _lib_or_skip():
    import cipsi_gb300
    try:
        cipsi_gb300.load_library()
    except cipsi_gb300.CipsiError as e:  # pragma: no cover - the build fixture makes it
        pytest.skip(str(e))


def _write_icinp(wd, body, cipfil=""):
    with open(os.path.join(wd, "cip.in"), "w") as fh:
        fh.write(f" &cipfil {cipfil}\n &end\n &icinp\n  {body}\n &end\n")


def _run_both(wd, variant):
    """Run the oracle and the drop-in on copies of `wd`; return both dirs."""
    from oracle import build as ob
    import cipsi_gb300
    wo, wg = wd + "_oracle", wd + "_engine"
    for d in (wo, wg):
        shutil.rmtree(d, ignore_errors=True)
        shutil.copytree(wd, d)
    ob.run(wo, variant=variant)
    cipsi_gb300.run_cip(wg, variant=variant)
    return wo, wg


def _same_file(a, b):
    with open(a, "rb") as fa, open(b, "rb") as fb:
        return fa.read() == fb.read()


def _unit60_dets(path, metat, sym):
    """Determinants of a unit-60 file (pie.f records), in file order."""
    out = []
    for rec in synth.read_records(path):
        mw, nw = struct.unpack_from("<ii", rec, 0)
        idet = np.frombuffer(rec, dtype="<i4", count=mw, offset=8)
        nex = np.frombuffer(rec, dtype="<i4", count=nw, offset=8 + 4 * mw)
        v = np.frombuffer(rec, dtype="<f8", count=nw, offset=8 + 4 * mw + 4 * nw)
        assert np.all(v == 1.0)
        if sym:
            assert len(rec) == 8 + 4 * mw + 4 * nw + 8 * nw + 8 * nw * metat
        my = 0
        for n in nex:
            pairs = idet[my: my + 2 * n].reshape(-1, 2)
            my += 2 * n
            out.append((tuple(sorted(int(x) for x in pairs[:, 0])), tuple(sorted(int(x) for x in pairs[:, 1]))))
    return out


def _fjk(wd):
    """Closed-shell F, J, K (full matrices) and orbital irreps of unit 40."""
    recs = synth.read_records(os.path.join(wd, "ijkl"))
    nsym, norb = struct.unpack_from("<ii", recs[0], 0)
    irrep = np.frombuffer(recs[0], dtype="<i4", count=norb, offset=16)
    its = np.frombuffer(recs[1], dtype="<i4", count=nsym * nsym).reshape(nsym, nsym).T

    def tri(rec):
        v = np.frombuffer(rec, dtype="<f8")
        M = np.zeros((norb, norb))
        t = 0
        for i in range(norb):
            for j in range(i + 1):
                M[i, j] = M[j, i] = v[t]
                t += 1
        return M
    return tri(recs[5]), tri(recs[3]), tri(recs[4]), irrep, its


def _en_diagonal(wd, dets):
    """EN diagonal energies relative to the reference determinant."""
    F, J, K, _, _ = _fjk(wd)
    n = F.shape[0]
    D = np.zeros((len(dets), 2 * n))
    for k, (hl, pt) in enumerate(dets):
        if hl:
            D[k, np.asarray(hl) - 1] -= 1.0
            D[k, np.asarray(pt) - 1] += 1.0
    Fso = np.concatenate([np.diag(F), np.diag(F)])
    orb = np.tile(np.arange(n), 2)
    spin = np.repeat([0, 1], n)
    X = J[np.ix_(orb, orb)] - (spin[:, None] == spin[None, :]) * K[np.ix_(orb, orb)]
    return D @ Fso + 0.5 * np.einsum("kr,rs,ks->k", D, X, D)


def _s_run_case(tmp_path, name, cfg):
    wd = str(tmp_path / name)
    synth.generate(cfg, wd)
    return wd


@pytest.mark.parametrize("variant", ["cipsym", "cip"])
@pytest.mark.parametrize("case", [c for c in cases.small_cases()][:4], ids=lambda c: c[0])
def test_sorted_space_run_matches_oracle(tmp_path, engine_lib, oracle_exe, case, variant):
    """ityper = -1, lecdet = 5: S from unit 60, sorted, written back."""
    _lib_or_skip()
    name, cfg = case
    wd = _s_run_case(tmp_path, name, cfg)
    S_in = _unit60_dets(os.path.join(wd, "det"), cfg.metat, sym=True)
    _write_icinp(wd, f"metat={cfg.metat}, ityper=-1, lecdet=5, tau=0.0, test=0.0, iselec=1, "
                     f"ymoyen=t, ybrd=f, title='{name}'")
    wo, wg = _run_both(wd, variant)
    for unit in ("det", "f04"):
        assert _same_file(os.path.join(wo, unit), os.path.join(wg, unit)), unit
    S_out = _unit60_dets(os.path.join(wg, "det"), cfg.metat, sym=variant == "cipsym")
    # the same determinants (the input is already closed under the spin flip)
    assert sorted(S_out) == sorted(S_in) and len(S_out) == len(S_in)
    # ordered by increasing EN diagonal energy
    dg = _en_diagonal(wd, S_out)
    assert np.all(np.diff(dg) >= -1e-9 * (1.0 + np.abs(dg[1:]))), np.diff(dg).min()
    # unit 4: the zero-order record then two effective-Hamiltonian records of
    # zeros (escf, ityper = -1 and the root signs in the first)
    r4 = synth.read_records(os.path.join(wg, "f04"))
    assert len(r4) == 3
    nbr = cfg.metat * (cfg.metat + 1) // 2
    hz = np.frombuffer(r4[1], dtype="<f8", count=nbr)
    assert np.all(hz == 0.0)
    ityper, ntrsy = struct.unpack_from("<ii", r4[1], 8 * nbr + 8)
    assert (ityper, ntrsy) == (-1, 1)
    assert np.all(np.frombuffer(r4[2], dtype="<f8") == 0.0) and len(r4[2]) == 24 * nbr
    mcf = struct.unpack_from("<5i", r4[0], 0)[4]
    assert mcf == len(S_out)


def _cas_model(norb, noca, act, nelac, nusym, nemax, irrep, its):
    """The CAS as a set: every alpha and beta string of (nelac+1)/2 electrons
    in the active orbitals, as holes / particles relative to the reference
    determinant (orbitals 1..noca doubly occupied)."""
    n = (nelac + 1) // 2
    strings = []
    for occ in itertools.combinations(act, n):
        holes = [o for o in act if o <= noca and o not in occ]
        parts = [o for o in occ if o > noca]
        strings.append((holes, parts))
    out = set()
    first_sym = None
    for ta, pa in strings:
        for tb, pb in strings:
            holes = ta + [x + norb for x in tb]
            parts = pa + [x + norb for x in pb]
            if len(holes) > nemax:
                continue
            s = 1
            for so in holes + parts:
                s = its[s - 1, irrep[(so - 1) % norb] - 1]
            if first_sym is None:
                first_sym = s
            want = nusym if nusym else first_sym
            if s != want:
                continue
            out.add((tuple(sorted(holes)), tuple(sorted(parts))))
    return out


CAS_CASES = [
    # (norb, nocc, nsym, numac, nelac, nusym, nemax, seed)
    (10, 3, 1, [2, 3, 4, 5, 6, 7], 4, 1, 8, 11),
    (12, 4, 2, [3, 4, 5, 6, 8, 10, 11], 4, 1, 8, 12),
    (12, 4, 4, [4, 5, 6, 7, 9], 2, 0, 8, 13),
    (14, 4, 2, [3, 4, 5, 6, 7, 8, 9], 4, 2, 3, 14),
    (12, 3, 4, [1, 2, 3, 4, 5, 6, 7, 8], 6, 1, 4, 15),
    (14, 4, 8, [3, 4, 5, 6, 7, 8, 9, 10, 11], 4, 0, 8, 16),
]


@pytest.mark.parametrize("spec", CAS_CASES, ids=lambda s: f"n{s[0]}_sym{s[2]}_act{len(s[3])}_e{s[4]}")
def test_cas_space_run_matches_oracle_and_model(tmp_path, engine_lib, oracle_exe, spec):
    """ityper = -1, lecdet = 4: the CAS generated, sorted and written."""
    _lib_or_skip()
    norb, nocc, nsym, numac, nelac, nusym, nemax, seed = spec
    cfg = synth.SynthConfig("cas", norb=norb, nocc=nocc, ncholesky=12, ncf=10, metat=2, tau=0.02,
                            ranks=(1, 2), coef_mode="decay09", seed=seed, nsym=nsym)
    wd = _s_run_case(tmp_path, "cas", cfg)
    os.remove(os.path.join(wd, "det"))  # lecdet = 4 does not read unit 60
    act = ",".join(str(x) for x in numac)
    _write_icinp(wd, f"numac={act}, isz=0, nusym={nusym}, noac={len(numac)}, metat=2, lecdet=4, "
                     f"ityper=-1, ymoyen=t, nelac={nelac}, ybrd=f, nemax={nemax}, yion=f, iselec=1, "
                     f"test=0d0, tau=0d0")
    wo, wg = _run_both(wd, "cipsym")
    for unit in ("det", "f04"):
        assert _same_file(os.path.join(wo, unit), os.path.join(wg, unit)), unit
    S = _unit60_dets(os.path.join(wg, "det"), 2, sym=True)
    _, _, _, irrep, its = _fjk(wd)
    model = _cas_model(norb, nocc, numac, nelac, nusym, nemax, irrep, its)
    # the CAS is closed under the spin flip, so S is exactly the model's set
    assert len(S) == len(set(S)) == len(model)
    assert set(S) == model
    if nsym == 1 and nemax >= nelac:
        n = (nelac + 1) // 2
        from math import comb
        assert len(S) == comb(len(numac), n) ** 2
    dg = _en_diagonal(wd, S)
    assert np.all(np.diff(dg) >= -1e-9 * (1.0 + np.abs(dg[1:])))


def test_s_run_without_ymoyen_leaves_unit60(tmp_path, engine_lib, oracle_exe):
    """Without ymoyen nothing is written to unit 60 (cip.f:222); unit 4 is."""
    _lib_or_skip()
    name, cfg = cases.small_cases()[1]
    wd = _s_run_case(tmp_path, name, cfg)
    _write_icinp(wd, f"metat={cfg.metat}, ityper=-1, lecdet=5, ymoyen=f, iselec=1")
    with open(os.path.join(wd, "det"), "rb") as fh:
        before = fh.read()
    wo, wg = _run_both(wd, "cipsym")
    for d in (wo, wg):
        with open(os.path.join(d, "det"), "rb") as fh:
            assert fh.read() == before
    assert _same_file(os.path.join(wo, "f04"), os.path.join(wg, "f04"))


def test_lecdet5_ignores_tdet(tmp_path, engine_lib, oracle_exe):
    """deter.f:224-226: lecdet = 5 reads all of unit 60 whatever tdet says."""
    _lib_or_skip()
    name, cfg = cases.small_cases()[2]
    wd = _s_run_case(tmp_path, name, cfg)
    _write_icinp(wd, f"metat={cfg.metat}, ityper=-1, lecdet=5, tdet=2.0, ymoyen=t, iselec=1")
    wo, wg = _run_both(wd, "cipsym")
    assert _same_file(os.path.join(wo, "det"), os.path.join(wg, "det"))
    assert len(_unit60_dets(os.path.join(wg, "det"), cfg.metat, True)) == len(
        _unit60_dets(os.path.join(wd, "det"), cfg.metat, True))


@pytest.mark.parametrize("body,msg", [
    ("metat=1, ityper=-1, lecdet=4, numac=2,3,4, noac=3, nelac=22, nusym=1", "20"),
    ("metat=1, ityper=-1, lecdet=4, numac=2,3,99, noac=3, nelac=2, nusym=1", "numac"),
    ("metat=1, ityper=-1, lecdet=4, numac=2, noac=1, nelac=4, nusym=1", "active"),
    ("metat=1, ityper=-1, lecdet=1", "lecdet"),
    ("metat=1, ityper=-1, lecdet=5, iord=2,1", "iord"),
])
def test_s_run_rejects_what_it_does_not_support(tmp_path, engine_lib, oracle_exe, body, msg):
    """Inputs outside the supported set fail with a message, in both."""
    _lib_or_skip()
    import subprocess
    import cipsi_gb300
    from oracle import build as ob
    name, cfg = cases.small_cases()[1]
    wd = _s_run_case(tmp_path, name, cfg)
    _write_icinp(wd, body)
    with pytest.raises(cipsi_gb300.CipsiError, match=msg):
        cipsi_gb300.run_cip(wd, variant="cipsym")
    with open(os.path.join(wd, "cip.in")) as fin:
        r = subprocess.run([ob.build(), "--sym"], cwd=wd, stdin=fin, capture_output=True, text=True)
    assert r.returncode != 0


def test_executable_takes_the_autocip_s_only_call(tmp_path, engine_lib, oracle_exe):
    """The process-level drop-in, as the Autocip driver calls it
    (`cip_gpu --sym < f_bd > listing`, Autocip_13/calcul.f90:320), on the
    first call of the loop: the CAS with ITYPER=-1, the namelist laid out as
    makedata_cip.f90:201-221 writes it."""
    import subprocess
    from cipsi_gb300 import EXE_PATH
    from oracle import build as ob
    cfg = synth.SynthConfig("exe", norb=12, nocc=4, ncholesky=12, ncf=10, metat=3, tau=0.02,
                            ranks=(1, 2), coef_mode="decay09", seed=51, nsym=2)
    wd = str(tmp_path / "exe")
    synth.generate(cfg, wd)
    for u in ("det", "bdvec", "f04"):
        os.remove(os.path.join(wd, u))
    text = ("&cipfil\nprefix='',\nf04='f04',\n bdvec='bdvec',\n&END\n\n"
            "&icinp\nNUMAC=3,4,5,6,7,8,9,\ntwdet=0.5\n ISZ=0,\n NUSYM=1,\n NOAC=7,\n METAT=3,\n"
            " LECDET=4,\n ITYPER=-1,\n YMOYEN=T,\n NELAC=4,\n YBRD=F,\n NEMAX=4,\n YION=F,\n"
            " ISELEC=  1,\n TEST=0d0,\n TAU=0d0,\n&END\n\n&MOYFIL\n&end\n")
    with open(os.path.join(wd, "cip.in"), "w") as fh:
        fh.write(text)
    wo = wd + "_oracle"
    shutil.copytree(wd, wo)
    with open(os.path.join(wd, "cip.in")) as fin:
        r = subprocess.run([EXE_PATH, "--sym"], cwd=wd, stdin=fin, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ob.run(wo, variant="cipsym")
    for unit in ("det", "f04"):
        assert _same_file(os.path.join(wo, unit), os.path.join(wd, unit)), unit
    assert len(_unit60_dets(os.path.join(wd, "det"), 3, True)) > 100


@pytest.mark.parametrize("body,keep", [
    ("lecdet=2, tdet=0.5", lambda v, i: v >= 0.5),          # lec60.f: v >= tdet
    ("lecdet=3, maxdet=37", lambda v, i: i < 37),            # the first maxdet read
    ("lecdet=2, tdet=0.0", lambda v, i: True),
])
def test_space_from_unit60_with_threshold_or_count(tmp_path, engine_lib, oracle_exe, body, keep):
    """lecdet 2 (records with v >= tdet) and 3 (the first maxdet records) on
    a unit 60 that holds S (v = 1) and earlier selected determinants with
    values below and above the threshold."""
    _lib_or_skip()
    name, cfg = cases.small_cases()[1]
    wd = _s_run_case(tmp_path, name, cfg)
    S = _unit60_dets(os.path.join(wd, "det"), cfg.metat, True)
    # rewrite unit 60: the first half of S with v = 1, the rest with values in (0, 1)
    rng = np.random.default_rng(3)
    vals = np.where(np.arange(len(S)) < len(S) // 2, 1.0, rng.uniform(0.01, 0.99, len(S)))
    with open(os.path.join(wd, "det"), "wb") as fh:
        for s0 in range(0, len(S), 25):
            chunk = list(range(s0, min(len(S), s0 + 25)))
            idet = [x for i in chunk for hp in zip(*S[i]) for x in hp]
            payload = struct.pack("<ii", len(idet), len(chunk)) + np.array(idet, "<i4").tobytes()
            payload += np.array([len(S[i][0]) for i in chunk], "<i4").tobytes()
            payload += vals[chunk].astype("<f8").tobytes() + np.zeros(len(chunk) * cfg.metat, "<f8").tobytes()
            synth.write_record(fh, payload)
    _write_icinp(wd, f"metat={cfg.metat}, ityper=-1, {body}, ymoyen=t, iselec=1")
    wo, wg = _run_both(wd, "cipsym")
    for unit in ("det", "f04"):
        assert _same_file(os.path.join(wo, unit), os.path.join(wg, unit)), unit
    kept = [S[i] for i in range(len(S)) if keep(vals[i], i)]
    out = set(_unit60_dets(os.path.join(wg, "det"), cfg.metat, True))
    # the kept determinants and their spin-flip partners
    want = set(kept) | {tuple(tuple(x) for x in synth.flip_lists(h, p, cfg.norb)) for h, p in kept}
    assert out == want


def test_zero_order_record_against_the_model(tmp_path, engine_lib, oracle_exe):
    """Unit 4's zero-order record (cip.f:144-150) as the drop-in writes it:
    the determinant lists are S in the order the brute-force model builds it,
    empdet is the model's MP diagonal hmp of each determinant, and fmpb the
    closed-shell orbital energies F_pp (faifoc.f with closed-shell tocom)."""
    _lib_or_skip()
    import cipsi_gb300
    import brute_force as bf
    name, cfg = cases.small_cases()[2]
    wd = _s_run_case(tmp_path, name, cfg)
    inp = bf.read_inputs(wd)
    model = bf.Model(inp)
    wg = wd + "_engine"
    shutil.copytree(wd, wg)
    _write_icinp(wg, f"metat={cfg.metat}, ityper=-1, lecdet=5, ymoyen=f, iselec=1")
    cipsi_gb300.run_cip(wg, variant="cipsym")
    rec = synth.read_records(os.path.join(wg, "f04"))[0]
    norb, noca, nocb, metat, ncf, isz = struct.unpack_from("<6i", rec, 0)
    assert (norb, noca, nocb, metat, ncf, isz) == (cfg.norb, cfg.nocc, cfg.nocc + cfg.norb, cfg.metat,
                                                    len(inp.S), 0)
    off = 25
    ii, jj = struct.unpack_from("<ii", rec, off)
    off += 8
    nend = np.frombuffer(rec, dtype="<i4", count=2 * ncf, offset=off).reshape(ncf, 2)
    off += 8 * ncf
    tp = np.frombuffer(rec, dtype="<i4", count=2 * ii, offset=off).reshape(ii, 2)
    off += 8 * ii
    dets = [(tuple(int(x) for x in tp[nd:nd + ne, 0]), tuple(int(x) for x in tp[nd:nd + ne, 1])) for ne, nd in nend]
    assert dets == [(tuple(h), tuple(p)) for h, p in inp.S]
    c = np.frombuffer(rec, dtype="<f8", count=jj, offset=off)
    assert jj == ncf * metat and np.all(c == 0.0)  # ityper < 0: ic001 not called
    off += 8 * jj + 3 * 8 * metat + 4 * metat  # e, emp, eb, numero
    empdet = np.frombuffer(rec, dtype="<f8", count=ncf, offset=off)
    off += 8 * ncf
    fmpb = np.frombuffer(rec, dtype="<f8", count=norb, offset=off)
    want = np.array([model.hmp_hdig(x)[0] for x in model.bits])
    np.testing.assert_allclose(empdet, want, rtol=0, atol=1e-12)
    np.testing.assert_allclose(fmpb, model.fdiag[1:norb + 1], rtol=0, atol=1e-13)


@pytest.mark.parametrize("fault", ["degree9", "marker"])
def test_corrupt_unit60_fails_cleanly(tmp_path, engine_lib, oracle_exe, fault):
    """A unit-60 record with an excitation degree above 8 (lec60.f:52-56
    stops) or a record whose trailing length marker disagrees: both the
    drop-in (an error code and message, no exit) and the oracle refuse it."""
    _lib_or_skip()
    import subprocess
    import cipsi_gb300
    from oracle import build as ob
    name, cfg = cases.small_cases()[1]
    wd = _s_run_case(tmp_path, name, cfg)
    path = os.path.join(wd, "det")
    if fault == "degree9":
        idet = list(range(1, 10)) + list(range(cfg.norb + 1, cfg.norb + 10))
        payload = struct.pack("<ii", 18, 1) + np.array(idet, "<i4").tobytes() + struct.pack("<i", 9)
        payload += struct.pack("<d", 1.0) + np.zeros(cfg.metat, "<f8").tobytes()
        with open(path, "ab") as fh:
            synth.write_record(fh, payload)
        msg = "degre"
    else:
        with open(path, "ab") as fh:
            fh.write(struct.pack("<i", 8) + b"\0" * 8 + struct.pack("<i", 9))
        msg = "marker"
    _write_icinp(wd, f"metat={cfg.metat}, ityper=-1, lecdet=5, ymoyen=t, iselec=1")
    with pytest.raises(cipsi_gb300.CipsiError, match=msg):
        cipsi_gb300.run_cip(wd, variant="cipsym")
    with open(os.path.join(wd, "cip.in")) as fin:
        r = subprocess.run([ob.build(), "--sym"], cwd=wd, stdin=fin, capture_output=True, text=True)
    assert r.returncode != 0
