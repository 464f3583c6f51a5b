"""The in-process CIPSI loop of the Autocip driver (cipsi_gb300.autocip,
Autocip_13/calcul.f90:255-480) on the GPU drop-ins: a complete active space
as the first S, CIPSI iterations that grow S until it holds det_bounds[0]
determinants, then the final space chosen by the ENvp of the selected
records and its moy/bd.  Checks: the steps come in calcul_cip's order, each
S-only run writes S grown by the previous selection, the namelist edits are
sed's, E2 and the vectors feed the next step, and the final space is S plus
the records down to the chosen threshold."""
import os
import shutil
import struct

import numpy as np
import pytest

from cipsi_gb300 import autocip, synth

COMMON = (" &MOYFIL\n &end\n &moyen\n TAU=0d0,\n &end\n &bdfil\n &end\n &option\n QGIV =T,\n NCPER=800,\n"
          " test=0.3d-3,\n qws=t,\n qwb=t,\n qwvec=t,\n &end\n")


def _icinp(extra):
    return (" &cipfil\n &end\n &icinp\n twdet=0.5\n ISZ=0,\n METAT=2,\n YMOYEN=T,\n YBRD=F,\n YION=F,\n"
            " ISELEC=  1,\n TEST=0d0,\n TAU=0d0,\n ITYPER=-1,\n" + extra + " &end\n")


def _files(wd):
    f_bd = os.path.join(wd, "chain.bd")
    cas = " NUMAC=3,4,5,6,7,8,9,10,\n NUSYM=1,\n NOAC=8,\n NELAC=2,\n NEMAX=2,\n LECDET=4,\n"
    with open(f_bd, "w") as fh:
        fh.write(_icinp(cas) + COMMON)
    for suffix in ("_loop", "_end"):
        with open(f_bd + suffix, "w") as fh:
            fh.write(_icinp(" LECDET=5,\n") + COMMON)
    return f_bd


def test_sed_item_is_seds_substitution():
    t = " &icinp\n ITYPER=2, LECDET=5,\n TAU=0.01,\n XITYPER=3,\n &end"
    out = autocip.sed_item(t, "ITYPER", "-1")
    assert out.split("\n")[1] == " ITYPER=-1,"  # the rest of the line goes, as with sed
    assert out.split("\n")[3] == " XITYPER=3,"  # ' ITYPER=' with its blank only
    assert autocip.sed_item(t, "TAU", "0d0").split("\n")[2] == " TAU=0d0,"


@pytest.mark.gpu
def test_cipsi_loop_on_the_drop_ins(tmp_path, engine_lib):
    cfg = synth.SynthConfig("chain", norb=12, nocc=3, ncholesky=12, ncf=10, metat=2, tau=0.02,
                            ranks=(1, 2), coef_mode="gauss005", seed=41, virt_shift=3.0)
    wd = str(tmp_path / "geo")
    synth.generate(cfg, wd)
    for u in ("det", "bdvec", "f04"):
        os.remove(os.path.join(wd, u))
    f_bd = _files(wd)
    log = []
    out = autocip.calcul_cip(wd, f_bd, metat=2, netat_pertu=1, envp_max=1e-3, det_bounds=(400, 100000, 10, 10 ** 6),
                             imax_s=4, tau_init=0.05, tau_step=0.5, ncf=0, log=log)
    kinds = [s["step"] for s in log]
    # per iteration: cip (S), moy, bd, cip (E2); then the final moy, bd
    n_it = (len(kinds) - 2) // 4
    assert kinds == ["cip", "moy", "bd", "cip"] * n_it + ["moy", "bd"]
    assert 2 <= n_it <= 4
    s_sizes = [log[4 * i + 2]["result"]["ncf"] for i in range(n_it)]  # bd over S in iteration i
    assert s_sizes[0] == 64  # the CAS of 2 electrons in 8 orbitals
    assert all(b > a for a, b in zip(s_sizes, s_sizes[1:]))
    for i in range(n_it):
        pert = log[4 * i + 3]["result"]
        assert pert["ncf"] == s_sizes[i] and pert["ntot60"] >= pert["ncf"]
        if i + 1 < n_it:  # the next S is this S plus the selection (and partners)
            assert s_sizes[i + 1] >= pert["ntot60"]
    # the variational energy of the lowest root does not rise as S grows
    e0 = [log[4 * i + 2]["result"]["eigenvalues"][0] for i in range(n_it)]
    assert all(b <= a + 1e-10 for a, b in zip(e0, e0[1:]))
    # the final space: S and the records whose xam reaches the chosen tau
    last = log[4 * (n_it - 1) + 3]["result"]
    xam, _ = autocip._unit60_xam_envp(os.path.join(wd, "det"), last["metat"])
    # nbase: the size read back at the start of the last iteration, the
    # previous run's unit-60 record count (S + selection, before the
    # spin-flip closure that the S-only run then adds)
    assert out["nbase"] == log[4 * (n_it - 2) + 3]["result"]["ntot60"] <= s_sizes[-1] <= out["ncf"]
    assert out["ncf"] >= int(np.sum(xam >= out["tau"]))
    assert len(out["e_corr"]) == 2 and all(np.isfinite(out["e_corr"]))
    assert out["e_corr"][0] < abs(last["e2vp"][0]) + 1e-12


def _grid_point(base, k, seed, det_max=100000):
    cfg = synth.SynthConfig("chain", norb=12, nocc=3, ncholesky=12, ncf=10, metat=2, tau=0.02,
                            ranks=(1, 2), coef_mode="gauss005", seed=seed, virt_shift=3.0)
    wd = os.path.join(base, f"point{k}")
    synth.generate(cfg, wd)
    for u in ("det", "bdvec", "f04"):
        os.remove(os.path.join(wd, u))
    return dict(workdir=wd, f_bd=_files(wd), metat=2, netat_pertu=1, envp_max=1e-3,
                det_bounds=(400, det_max, 10, 10 ** 6), imax_s=4, tau_init=0.05, tau_step=0.5)


def test_grid_needs_one_directory_per_point(tmp_path):
    pt = dict(workdir=str(tmp_path), f_bd="x")
    with pytest.raises(ValueError):
        autocip.run_grid([pt, dict(pt)])


def test_grid_records_a_failed_point_and_goes_on(tmp_path):
    """A point whose chain stops (here S outgrows det_bounds[1] = 10 after
    its first S-only run; on a machine without a GPU, its first GPU step)
    gets an error entry; the driver returns one entry per point."""
    pts = [_grid_point(str(tmp_path), 0, 41, det_max=10), _grid_point(str(tmp_path), 1, 42, det_max=10)]
    logs = []
    out = autocip.run_grid(pts, workers=2, logs=logs)
    assert len(out) == 2 and all("error" in r for r in out)
    assert len(logs) == 2 and all(log and log[0]["step"] == "cip" for log in logs)


@pytest.mark.gpu
def test_grid_matches_points_run_one_by_one(tmp_path, engine_lib):
    """Three points on three threads (and one that stops) give the results
    of calcul_cip run on each point alone."""
    pts = [_grid_point(str(tmp_path / "grid"), k, 41 + k) for k in range(3)]
    pts.append(_grid_point(str(tmp_path / "grid"), 3, 44, det_max=10))
    alone = []
    for k, pt in enumerate(pts[:3]):
        wd = str(tmp_path / "alone" / f"point{k}")
        shutil.copytree(pt["workdir"], wd)
        kw = dict(pt, workdir=wd, f_bd=os.path.join(wd, os.path.basename(pt["f_bd"])))
        alone.append(autocip.calcul_cip(**kw))
    out = autocip.run_grid(pts, workers=3)
    assert "S size too big" in out[3]["error"]
    for a, g in zip(alone, out[:3]):
        assert "error" not in g
        assert a["e_corr"] == g["e_corr"] and a["ncf"] == g["ncf"] and a["nbase"] == g["nbase"]
        assert a["tau"] == g["tau"]


def test_grid_takes_points_on_its_threads_in_order(monkeypatch):
    """run_grid with a stand-in for calcul_cip: every point runs once, on at
    most `workers` threads at a time, the results come back in point order,
    and a point that raises CipsiError gets an error entry while the others
    finish."""
    import threading
    import time
    from cipsi_gb300 import CipsiError
    lock = threading.Lock()
    state = {"now": 0, "peak": 0, "seen": []}

    def fake(workdir, log=None, **kw):
        with lock:
            state["now"] += 1
            state["peak"] = max(state["peak"], state["now"])
            state["seen"].append(workdir)
        time.sleep(0.02)
        with lock:
            state["now"] -= 1
        log.append({"step": "cip", "result": {}})
        if workdir.endswith("bad"):
            raise CipsiError("S size too big for calculation")
        return {"e_corr": [float(len(workdir))], "device": kw["device"]}

    monkeypatch.setattr(autocip, "calcul_cip", fake)
    pts = [dict(workdir=f"/tmp/grid/p{k}" + ("bad" if k == 5 else ""), f_bd="x") for k in range(12)]
    logs = []
    out = autocip.run_grid(pts, workers=3, device=1, logs=logs)
    assert sorted(state["seen"]) == sorted(p["workdir"] for p in pts)
    assert 1 < state["peak"] <= 3
    assert "S size too big" in out[5]["error"]
    for k, r in enumerate(out):
        if k != 5:
            assert r == {"e_corr": [float(len(pts[k]["workdir"]))], "device": 1}
    assert all(len(log) == 1 for log in logs)
