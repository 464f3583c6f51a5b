"""Standard input read as the Fortran runtime reads the reference's namelists
(&cipfil, cip/openf.f:5-21; &icinp, cip/deter.f:52-58 and 222): repeat
counts, null values, subscripted names, comments, unknown names, and the
unit file names of nomfil.f / nomf.f.  Each form is checked against the same
input spelled out element by element, in the drop-in (engine library) and in
the oracle, through runs that need no GPU (ityper < 0) and through the host
inputs of a perturbation run."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cipsi_gb300 import synth

import cases


def _case(tmp_path, idx=1):
    name, cfg = cases.small_cases()[idx]
    wd = str(tmp_path / name)
    synth.generate(cfg, wd)
    return wd, cfg


def _write(wd, icinp, cipfil=""):
    with open(os.path.join(wd, "cip.in"), "w") as fh:
        fh.write(f" &cipfil {cipfil}\n &end\n &icinp\n{icinp}\n &end\n")


def _files_after(wd, icinp, tag, variant="cipsym"):
    """Units 4 and 60 written by the oracle and by the drop-in for `icinp`."""
    import cipsi_gb300
    from oracle import build as ob
    out = {}
    for who in ("oracle", "engine"):
        d = f"{wd}_{tag}_{who}"
        shutil.rmtree(d, ignore_errors=True)
        shutil.copytree(wd, d)
        _write(d, icinp)
        if who == "oracle":
            ob.run(d, variant=variant)
        else:
            cipsi_gb300.run_cip(d, variant=variant)
        out[who] = {u: open(os.path.join(d, u), "rb").read() for u in ("f04", "det")}
    assert out["oracle"] == out["engine"]
    return out["engine"]


def test_fortran_forms_read_like_the_spelled_out_input(tmp_path, engine_lib, oracle_exe):
    wd, cfg = _case(tmp_path)
    fancy = ("  METAT=2, ityper=-1, LecDet=5,  ! a comment, with = and , inside\n"
             "  numero(2)=7, tocom=2.0,,1.5 , ymoyen=.true.\n"
             "  iselec= 1, title='it''s', test=1*")
    plain = ("  metat=2, ityper=-1, lecdet=5, numero=1,7, tocom=2.0,2.0,1.5, ymoyen=t,\n"
             "  iselec=1, title='it''s'")
    a = _files_after(wd, fancy, "fancy")
    b = _files_after(wd, plain, "plain")
    assert a == b
    # and the assignments took effect: tocom changes the barycentric energies
    c = _files_after(wd, "  metat=2, ityper=-1, lecdet=5, ymoyen=t", "defaults")
    assert c["f04"] != a["f04"] and c["det"] == a["det"]


def test_repeat_counts_nulls_and_subscripts_in_the_host_inputs(tmp_path, engine_lib):
    from cipsi_gb300 import engine
    wd, cfg = _case(tmp_path)
    default = [0.128e-6, 0.64e-6, 0.32e-5, 0.16e-4, 0.8e-4, 0.4e-3, 0.2e-2, 0.1e-1, 0.5e-1, 1.0]
    _write(wd, f"  metat={cfg.metat}, ityper=2, lecdet=5, ymoyen=t, tau=1*,\n"
               "  aval=3*1d-3, 2*, 5.0D-2, aval(9)=0.25, nclass=9, teseff=0.5e-3")
    inp = engine.Inputs(wd)
    want = [1e-3, 1e-3, 1e-3, default[3], default[4], 5e-2, default[6], default[7], 0.25, 1.0]
    np.testing.assert_array_equal(np.array(inp.opts.aval[:10]), np.array(want))
    assert inp.opts.tau == 1.0e-4  # null: the default of deter.f:207
    assert inp.opts.nclass == 9 and inp.opts.teseff == 0.5e-3
    inp.close()


@pytest.mark.parametrize("icinp,variant,msg", [
    ("  metat=1, ityper=-1, lecdet=5, nosuchname=3", "cipsym", "nosuchname"),
    ("  metat=1, ityper=-1, lecdet=5, nemax=4", "cip", "nemax"),
    ("  metat=1,2, ityper=-1, lecdet=5", "cipsym", "metat"),
    ("  metat=1, ityper=-1, lecdet=5, aval(11)=1.0", "cipsym", "aval"),
    ("  metat=1, ityper=-1, lecdet=5, tau=0.1x", "cipsym", "0.1x"),
    ("  metat=1, ityper=-1, lecdet=5, ymoyen=yes", "cipsym", "yes"),
])
def test_input_errors_stop_both(tmp_path, engine_lib, oracle_exe, icinp, variant, msg):
    import cipsi_gb300
    from oracle import build as ob
    wd, _ = _case(tmp_path)
    _write(wd, icinp)
    with pytest.raises(cipsi_gb300.CipsiError, match=msg):
        cipsi_gb300.run_cip(wd, variant=variant)
    args = [ob.build()] + (["--sym"] if variant == "cipsym" else [])
    with open(os.path.join(wd, "cip.in")) as fin:
        r = subprocess.run(args, cwd=wd, stdin=fin, capture_output=True, text=True)
    assert r.returncode != 0 and msg in r.stderr


def test_unit_file_names_follow_nomf(tmp_path, engine_lib, oracle_exe):
    """prefix up to its first blank + root name up to its first blank (of 10
    characters); a root of 10 characters without a blank contributes nothing;
    det1 and friends replace the whole name."""
    import cipsi_gb300
    from oracle import build as ob
    wd, cfg = _case(tmp_path)
    for u in ("ijkl", "ener", "f04", "bdvec"):
        os.rename(os.path.join(wd, u), os.path.join(wd, "pre" + u))
    os.rename(os.path.join(wd, "det"), os.path.join(wd, "pre"))  # root 'detfile123': nothing
    cipfil = "prefix='pre  ignored', det='detfile123', ener1='preener'"
    icinp = f"  metat={cfg.metat}, ityper=-1, lecdet=5, ymoyen=t"
    outs = []
    for who in ("oracle", "engine"):
        d = f"{wd}_{who}"
        shutil.copytree(wd, d)
        _write(d, icinp, cipfil)
        if who == "oracle":
            with open(os.path.join(d, "cip.in")) as fin:
                r = subprocess.run([ob.build(), "--sym"], cwd=d, stdin=fin, capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
        else:
            cipsi_gb300.run_cip(d, variant="cipsym")
        outs.append({u: open(os.path.join(d, u), "rb").read() for u in ("pre", "pref04")})
    assert outs[0] == outs[1]


def test_cip_variant_cas_has_no_nemax_filter(tmp_path, engine_lib, oracle_exe):
    """cip/cas.f keeps every CAS determinant; cipsym/cas.f:227 drops those
    above nemax (default 8, so the same space here)."""
    cfg = synth.SynthConfig("cas", norb=10, nocc=3, ncholesky=10, ncf=10, metat=1, tau=0.02,
                            ranks=(1, 2), coef_mode="decay09", seed=21, nsym=2)
    wd = str(tmp_path / "cas")
    synth.generate(cfg, wd)
    body = "  numac=2,3,4,5,6,7, noac=6, nelac=4, nusym=1, metat=1, lecdet=4, ityper=-1, ymoyen=t"
    a = _files_after(wd, body, "cip", variant="cip")
    b = _files_after(wd, body, "sym", variant="cipsym")
    c = _files_after(wd, body + ", nemax=2", "sym2", variant="cipsym")
    # same determinants; the cipsym file carries the ENvp block, so compare sets
    from test_autocip_s_runs import _unit60_dets
    da = _unit60_dets(os.path.join(f"{wd}_cip_engine", "det"), 1, False)
    db = _unit60_dets(os.path.join(f"{wd}_sym_engine", "det"), 1, True)
    dc = _unit60_dets(os.path.join(f"{wd}_sym2_engine", "det"), 1, True)
    assert da == db and len(dc) < len(db) and all(len(h) <= 2 for h, _ in dc)
    assert a["f04"] == b["f04"]


def _fmpb_model(wd, tocom_in, noca):
    """faifoc.f from the closed-shell F, J, K of unit 40 and the occupations
    transformed as cip.f:75-85 does (numpy restatement)."""
    from test_autocip_s_runs import _fjk
    F, J, K, _, _ = _fjk(wd)
    n = F.shape[0]
    ta, tb = np.zeros(n), np.zeros(n)
    for i in range(n):
        if tocom_in[i] > 1.0:
            ta[i], tb[i] = 1.0, tocom_in[i] - 1.0
        else:
            ta[i], tb[i] = tocom_in[i], 0.0
    ta[:noca] -= 1.0
    tb[:noca] -= 1.0
    t = np.diag(F) + J @ (ta + tb)
    return 0.5 * ((t - K @ ta) + (t - K @ tb))


def test_ytocom_reads_the_occupations_of_unit21(tmp_path, engine_lib, oracle_exe):
    from cipsi_gb300 import engine
    wd, cfg = _case(tmp_path)
    occ = np.full(cfg.norb, 0.0)
    occ[:cfg.nocc] = 2.0
    occ[cfg.nocc - 1], occ[cfg.nocc] = 1.5, 0.5  # fractional frontier occupations
    with open(os.path.join(wd, "ocno"), "wb") as fh:
        synth.write_record(fh, occ.astype("<f8").tobytes())
    body = f"  metat={cfg.metat}, ityper=-1, lecdet=5, ymoyen=t, ytocom=t, tocom=3*1.0"
    a = _files_after(wd, body, "ocno")  # byte-equal with the oracle
    b = _files_after(wd, f"  metat={cfg.metat}, ityper=-1, lecdet=5, ymoyen=t", "plain")
    assert a["f04"] != b["f04"] and a["det"] == b["det"]
    # the file wins over the namelist's tocom (read after it, deter.f:229)
    _write(wd, body.replace("ityper=-1", "ityper=2"))
    inp = engine.Inputs(wd)
    fmpb = inp.array("fmpb")
    inp.close()
    want = _fmpb_model(wd, occ, cfg.nocc)
    np.testing.assert_allclose(fmpb[:cfg.norb], want, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(fmpb[:cfg.norb], fmpb[cfg.norb:])
