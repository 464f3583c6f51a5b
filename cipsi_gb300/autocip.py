"""In-process CIPSI loop of the Autocip driver for one geometry and symmetry
(Autocip_13/calcul.f90:255-480, subroutine calcul_cip), with the GPU
drop-ins in place of the cipsym.exe, moy.exe and bd.exe processes.

The reference edits its namelist file with `sed` between steps and runs one
process per step through `system()`, reading the values it needs back from
the listings.  Here the same edits are made to the namelist text, each step
is a call into the engine library (cipsi_cip_main, cipsi_moy_main,
cipsi_bd_main) on the same unit files, and the values come from each
call's summary instead of the listing:

  'nombre de determinants sur la file 60'  -> the cip run's ntot60, metat
  ' energies CIPSI envp'                   -> the cip run's e2vp
  ' ncf,netat,ncper,iget'                  -> the bd run's ncf

Steps, as calcul.f90 orders them (imax_s > 0, the CIPSI method):
  for i = 1 .. imax_s:
    cipsym ITYPER=-1 (S from the CAS the first time, then from unit 60)
    moy TAU=0, bd                        (the vectors of S on unit 59)
    final S when i = imax_s or ncf >= max(metat, det_bounds[0]): tau = 0
    stop if ncf >= det_bounds[1]
    cipsym ITYPER=2 with TEST = TAU = tau (E2 and the selection)
    leave the loop at the final S, else tau *= tau_step
  then, from the last unit 60 (records by decreasing selection value
  xam): subtract each record's ENvp from E2 until the largest |E2| of the
  first netat_pertu roots is below envp_max (and at least det_bounds[2]
  records were taken; at most det_bounds[3]); tau = that record's xam;
  moy with TAU = tau and bd on the end namelist: the final S + M space.
With imax_s <= 0 (the FCI method): cipsym once on the first namelist, then
moy and bd on the end namelist.

run_grid runs calcul_cip over the points of a grid on a pool of threads, as
the reference's OpenMP loop over grid points does (autocip13.f90:525-640).
"""
from __future__ import annotations

import os
import re
import struct
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import CipsiError, run_bd, run_cip, run_moy


def sed_item(text: str, name: str, value: str) -> str:
    """What `sed -i "s# NAME=.*# NAME=value,#"` does to the namelist file
    (calcul.f90:318, 325, 347-351): on every line holding ' NAME=', that text
    and the rest of the line become ' NAME=value,'."""
    pat = re.compile(" " + re.escape(name) + "=.*")
    return "\n".join(pat.sub(lambda m: f" {name}={value},", line, count=1) for line in text.split("\n"))


def _tau_str(tau: float) -> str:
    """write(tau_str,'(f20.12)') tau (calcul.f90:346): fixed point, 12 decimals."""
    return f"{tau:20.12f}"


def _unit60_xam_envp(path: str, metat: int):
    """xam (the record value) and the per-root ENvp of every record of
    cipsym's unit 60, in file order (calcul.f90:381-388)."""
    from . import synth
    xam: List[float] = []
    envp: List[float] = []
    for r in synth.read_records(path):
        mw, nw = struct.unpack_from("<ii", r, 0)
        off = 8 + 4 * mw + 4 * nw
        xam.extend(struct.unpack_from(f"<{nw}d", r, off))
        envp.extend(struct.unpack_from(f"<{nw * metat}d", r, off + 8 * nw))
    return np.array(xam), np.array(envp).reshape(-1, metat) if xam else np.zeros((0, metat))


def calcul_cip(workdir: str, f_bd: str, metat: int, netat_pertu: int, envp_max: float,
               det_bounds: Sequence[int], imax_s: int, tau_init: float, tau_step: float, ncf: int = 0,
               device: int = 0, log: Optional[List[Dict]] = None) -> Dict:
    """One geometry's CIPSI loop in `workdir`.  f_bd is the namelist file of
    the first step; f_bd + '_loop' and f_bd + '_end' those of the later
    steps and of the final moy/bd (makedata_cip.f90 writes all three).
    Returns e_corr (|E2| per root), the final S size nbase and the size of
    the final space ncf; `log` (optional) receives one entry per step."""
    steps = log if log is not None else []
    stdin = os.path.join(workdir, "_autocip.in")

    def call(kind: str, text: str) -> Dict:
        with open(stdin, "w") as fh:
            fh.write(text)
        if kind == "cip":
            r = run_cip(workdir, variant="cipsym", stdin_path=stdin, device=device,
                        json_path=os.path.join(workdir, "_cip.json"))
        elif kind == "moy":
            r = run_moy(workdir, stdin_path=stdin, device=device, json_path=os.path.join(workdir, "_moy.json"))
        else:
            r = run_bd(workdir, stdin_path=stdin, device=device, json_path=os.path.join(workdir, "_bd.json"))
        steps.append({"step": kind, "result": r})
        return r

    def read(path: str) -> str:
        with open(path) as fh:
            return fh.read()

    text = read(f_bd)
    tau = tau_init
    nbase = 0
    energ2 = np.zeros(metat)
    if imax_s > 0:
        pert = None
        for i in range(1, imax_s + 1):
            if i > 1:
                ncf, metat2 = pert["ntot60"], pert["metat"]
            text = sed_item(text, "ITYPER", "-1")
            call("cip", text)
            text = read(f_bd + "_loop")
            text = sed_item(text, "TAU", "0d0")
            call("moy", text)
            call("bd", text)
            final = i == imax_s or (ncf >= metat and ncf >= det_bounds[0])
            if final:
                tau = 0.0
                nbase = ncf
            if ncf >= det_bounds[1]:
                raise CipsiError(f"S size too big for calculation (ncf = {ncf})")
            text = sed_item(text, "TEST", _tau_str(tau))
            text = sed_item(text, "TAU", _tau_str(tau))
            text = sed_item(text, "ITYPER", "2")
            pert = call("cip", text)
            if ncf >= metat and ncf >= det_bounds[0]:
                break
            tau = tau * tau_step
        ncf, metat2 = pert["ntot60"], pert["metat"]
        energ2 = np.array(pert["e2vp"][:metat2], dtype=float)
        xam, envp_lim = _unit60_xam_envp(os.path.join(workdir, "det"), metat2)
        order = np.argsort(xam, kind="stable")  # mrgrnk: ascending ranks, ties in file order
        counter = 0
        ind = order[-1] if len(order) else 0
        for i in range(len(order) - 1, -1, -1):
            counter += 1
            ind = order[i]
            energ2 = energ2 - envp_lim[ind]
            envp = float(np.max(np.abs(energ2[:netat_pertu]))) if netat_pertu > 0 else 0.0
            if envp < envp_max and counter >= det_bounds[2]:
                break
            if counter >= det_bounds[3]:
                raise CipsiError(f"too many determinants for calculation (precision reached {envp})")
        tau = float(xam[ind]) if len(xam) else 0.0
        text = read(f_bd + "_end")
        text = sed_item(text, "TAU", _tau_str(tau))
        call("moy", text)
        bd = call("bd", text)
    else:
        call("cip", text)
        text = read(f_bd + "_end")
        call("moy", text)
        bd = call("bd", text)
    return {"e_corr": [abs(float(x)) for x in energ2[:metat]] + [0.0] * max(0, metat - len(energ2)),
            "nbase": nbase, "ncf": bd["ncf"], "tau": tau, "steps": len(steps)}


def run_grid(points: Sequence[Dict], workers: int = 4, device: int = 0,
             logs: Optional[List] = None) -> List[Dict]:
    """The loop over the points of an Autocip grid for the CIPSI step
    (Autocip_13/autocip13.f90:525-640: an OpenMP loop with
    SCHEDULE(DYNAMIC), one work directory per thread, calcul_cip per point).

    points: one dict of calcul_cip keyword arguments per point (workdir,
    f_bd, metat, netat_pertu, envp_max, det_bounds, imax_s, tau_init,
    tau_step[, ncf, device]); each point needs its own work directory.
    `workers` threads take the points in order as they become free.  The
    engine library releases the interpreter lock during its calls, and each
    call's context runs on its own stream.  One point's host steps
    (namelists, unit files, the S build, moy's lists) therefore overlap
    other points' GPU work.

    Returns one result per point, in point order: calcul_cip's dict, or
    {"error": message} for a point whose chain stopped (the reference marks
    such a point as not accepted and carries on with the others).  `logs`,
    if given, is filled with each point's step log."""
    dirs = [os.path.abspath(pt["workdir"]) for pt in points]
    if len(set(dirs)) != len(dirs):
        raise ValueError("run_grid: every point needs its own work directory")
    results: List[Optional[Dict]] = [None] * len(points)
    if logs is not None:
        logs[:] = [None] * len(points)

    def one(i: int) -> None:
        kw = dict(points[i])
        kw.setdefault("device", device)
        log: List[Dict] = []
        try:
            results[i] = calcul_cip(log=log, **kw)
        except CipsiError as e:
            results[i] = {"error": str(e)}
        if logs is not None:
            logs[i] = log

    with ThreadPoolExecutor(max_workers=max(1, int(workers))) as ex:
        list(ex.map(one, range(len(points))))
    return results
