"""Readers of the files moy writes, and the set-up of a moy run (test only).

A moy run needs what a cipsym perturbation run leaves in its directory: unit
60 with S followed by the selected perturbers, and unit 4 with the zero-order
record of S.  `prepare` makes the synthetic inputs, runs the oracle's cipsym
on them, and writes moy's namelists (moy/openf.f &moyfil, moy/moy.f
&moyen)."""
from __future__ import annotations

import os
import struct

import numpy as np

from cipsi_gb300 import synth
from oracle import build as ob

LSIZE = 8192


def prepare(workdir: str, cfg, moy_tau: float = 0.0, extra: str = "", cip_tau=None) -> dict:
    """Inputs of `cfg` in `workdir`, the oracle's cipsym perturbation run
    (ymoyen: unit 60 = S + selected), then moy.in with &moyen tau and
    `extra` namelist items."""
    import dataclasses
    if cip_tau is not None:
        cfg = dataclasses.replace(cfg, tau=cip_tau)
    info = synth.generate(cfg, workdir)
    ob.run(workdir, variant="cipsym", json_name="cip_ref.json")
    with open(os.path.join(workdir, "moy.in"), "w") as fh:
        fh.write(" &moyfil\n &end\n &moyen\n")
        fh.write(f"  tau={moy_tau!r}, title='{cfg.name[:20]}', ystkmp=t{(', ' + extra) if extra else ''}\n")
        fh.write(" &end\n")
    return info


def run_oracle_moy(workdir: str) -> dict:
    import json
    import subprocess
    exe = ob.build()
    with open(os.path.join(workdir, "moy.in")) as fin:
        r = subprocess.run([exe, "--moy", "--json", "moy_ref.json"], cwd=workdir, stdin=fin,
                           stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle moy failed: " + r.stderr)
    with open(os.path.join(workdir, "moy_ref.json")) as fh:
        return json.load(fh)


def read_unit1(path: str):
    """Records (itab, jtab, vbuf) of unit 1 and the elements they hold in
    file order: every element of the full records, then jtab(lsize) of the
    last one (moy.f:150-184)."""
    recs = []
    for r in synth.read_records(path):
        assert len(r) == LSIZE * 16
        it = np.frombuffer(r, dtype="<i4", count=LSIZE, offset=0)
        jt = np.frombuffer(r, dtype="<i4", count=LSIZE, offset=4 * LSIZE)
        vb = np.frombuffer(r, dtype="<f8", count=LSIZE, offset=8 * LSIZE)
        recs.append((it, jt, vb))
    assert recs and recs[-1][0][LSIZE - 1] == -1
    for it, _, _ in recs[:-1]:
        assert it[LSIZE - 1] != -1
    last = int(recs[-1][1][LSIZE - 1])
    I = np.concatenate([r[0] for r in recs[:-1]] + [recs[-1][0][:last]]).astype(np.int64)
    J = np.concatenate([r[1] for r in recs[:-1]] + [recs[-1][1][:last]]).astype(np.int64)
    V = np.concatenate([r[2] for r in recs[:-1]] + [recs[-1][2][:last]])
    return recs, I, J, V


def read_unit64(path: str):
    """moy.f:79-82: ncf, ii, mnorb, yion, (ne, nd) per determinant, (trou,
    part) of the lists, iorb and ispin of the spin orbitals.  Returns the
    determinants as (holes, particles) tuples and the raw fields."""
    r = synth.read_records(path)
    assert len(r) == 1
    b = r[0]
    ncf, ii, mnorb = struct.unpack_from("<3i", b, 0)
    pos = 13
    nend = np.frombuffer(b, dtype="<i4", count=2 * ncf, offset=pos).reshape(ncf, 2)
    pos += 8 * ncf
    tp = np.frombuffer(b, dtype="<i4", count=2 * ii, offset=pos).reshape(ii, 2)
    pos += 8 * ii
    iorb = np.frombuffer(b, dtype="<i4", count=mnorb + 1, offset=pos)
    pos += 4 * (mnorb + 1)
    ispin = np.frombuffer(b, dtype="<i4", count=mnorb + 1, offset=pos)
    pos += 4 * (mnorb + 1)
    assert pos == len(b)
    dets = []
    for k in range(ncf):
        ne, nd = int(nend[k, 0]), int(nend[k, 1])
        dets.append((tuple(int(x) for x in tp[nd:nd + ne, 0]), tuple(int(x) for x in tp[nd:nd + ne, 1])))
    return dets, {"ncf": ncf, "ii": ii, "mnorb": mnorb, "nend": nend, "tp": tp, "iorb": iorb, "ispin": ispin,
                  "yion": b[12]}


def read_unit60_dets(path: str, tau: float):
    """The determinants of the records of unit 60 with value >= tau, in file
    order, as sorted (holes, particles)."""
    out = []
    for r in synth.read_records(path):
        m, n = struct.unpack_from("<ii", r, 0)
        idet = struct.unpack_from(f"<{m}i", r, 8)
        nex = struct.unpack_from(f"<{n}i", r, 8 + 4 * m)
        v = struct.unpack_from(f"<{n}d", r, 8 + 4 * m + 4 * n)
        pos = 0
        for q, nec in enumerate(nex):
            h = tuple(sorted(idet[pos + 2 * i] for i in range(nec)))
            p = tuple(sorted(idet[pos + 2 * i + 1] for i in range(nec)))
            pos += 2 * nec
            if v[q] >= tau:
                out.append((h, p))
    return out
