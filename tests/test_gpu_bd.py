"""The bd drop-in (cipsi_bd_main: block Davidson on the GPU) on the matrices
that moy writes, and the Autocip loop cip -> moy -> bd -> cip through the
drop-ins.

bd computes the lowest eigenpairs of H = L + L^T (L: moy's unit 1, the
diagonal stored as half its value, bd/getmat.f); its own iteration stops
at a loose tolerance (bd/bigdia.f:402-411), so the check is the definition
of the result: the eigenpairs of the same matrix from dense LAPACK (numpy,
test infrastructure) for lists of up to a few thousand determinants --
eigenvalues to 1e-9 Eh, vectors to |<x, y>| >= 1 - 1e-9 -- and, for a
list of 100,000 determinants, residual norms |H x - e x| recomputed on the
CPU (scipy.sparse) and the eigenvalues of scipy's Lanczos solver."""
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
BD_IN = " &bdfil\n &end\n &option\n  qwvec=t, qws=t, qwb=t, title='{t}'{x}\n &end\n"


def _matrix(wd):
    _, I, J, V = mf.read_unit1(os.path.join(wd, "mat"))
    return I - 1, J - 1, V


def _dense(I, J, V, n):
    H = np.zeros((n, n))
    np.add.at(H, (I, J), V)
    return H + H.T


def _read59(wd):
    b = synth.read_records(os.path.join(wd, "bdvec"))[0]
    ncf, netat = struct.unpack_from("<ii", b, 0)
    vec = np.frombuffer(b, "<f8", count=ncf * netat, offset=8).reshape(netat, ncf)
    e = np.frombuffer(b, "<f8", count=netat, offset=8 + 8 * ncf * netat)
    assert len(b) == 8 + 8 * ncf * netat + 8 * netat
    return ncf, netat, vec, e


def _escf(wd):
    r = synth.read_records(os.path.join(wd, "f04"))
    metat = struct.unpack_from("<i", r[0], 12)[0]
    nbr = metat * (metat + 1) // 2
    return struct.unpack_from("<d", r[1], 8 * nbr)[0], metat


def _moy_then_bd(wd, name, tau, extra=""):
    mf.prepare(wd, CASES[name], moy_tau=tau)
    cg.run_moy(wd)
    with open(os.path.join(wd, "bd.in"), "w") as fh:
        fh.write(BD_IN.format(t=name, x=extra))
    return cg.run_bd(wd)


@pytest.mark.parametrize("name,tau", [("small", 0.05), ("mix1", 0.02), ("mix2", 0.0), ("mix4", 0.0)])
def test_bd_matches_dense_eigenpairs(tmp_path, oracle_exe, engine_lib, name, tau):
    wd = str(tmp_path / "run")
    jg = _moy_then_bd(wd, name, tau)
    I, J, V = _matrix(wd)
    n = jg["ncf"]
    assert n == int(max(I.max(), J.max())) + 1
    w, U = np.linalg.eigh(_dense(I, J, V, n))
    ncf, netat, vec, e59 = _read59(wd)
    escf, metat = _escf(wd)
    assert (ncf, netat) == (n, metat)
    ev = np.array(jg["eigenvalues"])
    np.testing.assert_allclose(ev, w[:netat], rtol=0, atol=1e-9)
    np.testing.assert_allclose(e59, ev + escf, rtol=0, atol=0)
    assert max(jg["residuals"]) <= 1e-8
    for m in range(netat):
        gap = min(abs(w[m] - w[q]) for q in range(len(w)) if q != m)
        if gap > 1e-6:  # a non-degenerate root: the vector is defined up to sign
            assert abs(vec[m] @ U[:, m]) >= 1 - 1e-9
        assert abs(np.linalg.norm(vec[m]) - 1) < 1e-12
        assert vec[m][np.argmax(np.abs(vec[m]))] > 0
    # unit 33: the eigenvalues after what cip and moy appended
    last = synth.read_records(os.path.join(wd, "ener"))[-1]
    assert last[:40] == ("energies var." + name.ljust(20)).ljust(40).encode()
    np.testing.assert_array_equal(np.frombuffer(last[40:], "<f8"), ev)
    # unit 55 (qws): each vector's first ncper components
    r55 = synth.read_records(os.path.join(wd, "fort.55"))[0]
    ncper, net55 = struct.unpack_from("<ii", r55, 0)
    assert net55 == netat and ncper == min(jg["ncper"], n)
    width = n if ncper >= n - metat else ncper
    c55 = np.frombuffer(r55, "<f8", count=netat * width, offset=8).reshape(netat, width)
    np.testing.assert_array_equal(c55, vec[:, :width])


def test_bd_large_list_residuals(tmp_path, engine_lib):
    """100,000 determinants (the moy benchmark's list): residual norms on
    the CPU and scipy's Lanczos eigenvalues."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    import bench
    wd = bench._moy_workdir(str(tmp_path), 100000, 7)
    cg.run_cip(wd)
    cg.run_moy(wd)
    with open(os.path.join(wd, "bd.in"), "w") as fh:
        fh.write(" &bdfil\n &end\n &option\n  ncper=800, test=0.3d-3, qwvec=t\n &end\n")
    jg = cg.run_bd(wd)
    I, J, V = _matrix(wd)
    n = jg["ncf"]
    L = sp.csr_matrix((V, (I, J)), shape=(n, n))
    H = (L + L.T).tocsr()
    ncf, netat, vec, e59 = _read59(wd)
    ev = np.array(jg["eigenvalues"])
    for m in range(netat):
        r = H @ vec[m] - ev[m] * vec[m]
        assert np.linalg.norm(r) <= 1e-7
    wl = np.sort(spl.eigsh(H, k=netat, which="SA", tol=1e-12)[0])
    np.testing.assert_allclose(ev, wl, rtol=0, atol=1e-8)


def test_autocip_loop_on_the_drop_ins(tmp_path, oracle_exe, engine_lib):
    """One Autocip iteration through the drop-ins only: cip_gpu writes S
    (ityper = -1), moy_gpu builds H, bd_gpu writes unit 59, cip_gpu runs the
    perturbation on those vectors; the oracle's perturbation run on the
    same files gives the same E2 and selection."""
    wd = str(tmp_path / "run")
    cfg = CASES["mix1"]
    synth.generate(cfg, wd)
    txt = open(os.path.join(wd, "cip.in")).read()
    open(os.path.join(wd, "cip.in"), "w").write(txt.replace("ityper=2", "ityper=-1"))
    cg.run_cip(wd)
    with open(os.path.join(wd, "moy.in"), "w") as fh:
        fh.write(" &moyfil\n &end\n &moyen\n  tau=0d0\n &end\n")
    cg.run_moy(wd)
    with open(os.path.join(wd, "bd.in"), "w") as fh:
        fh.write(BD_IN.format(t="loop", x=""))
    jb = cg.run_bd(wd)
    open(os.path.join(wd, "cip.in"), "w").write(txt)  # ityper = 2, lecdet = 5: S from unit 60, vectors from 59
    wo = str(tmp_path / "ora")
    shutil.copytree(wd, wo)
    jg = cg.run_cip(wd)
    jo = ob.run(wo, variant="cipsym")
    import json
    jo = json.load(open(jo))
    assert jg["ncf"] == jo["ncf"] == jb["ncf"]
    assert jg["n_processed"] == jo["n_processed"] and jg["ietat"] == jo["ietat"]
    for k in ("e2mp", "e2vp", "e2b"):
        np.testing.assert_allclose(jg[k], jo["comp_" + k], rtol=0,
                                   atol=1e-10 + max(jo["cond_" + k]) + max(abs(np.array(jo[k]) - jo["comp_" + k])))
