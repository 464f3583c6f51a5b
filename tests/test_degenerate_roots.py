"""The vectors of S as ic001 leaves them after reading unit 59 (lecdet = 5).

Roots degenerate within 1e-6 Eh (degen, brdnee.f:299-365, called by
ic001 after unit 59 is read): a run of exactly two degenerate roots is
rotated so that the first spin-flip pair of unequal weights on the first
root gets equal weights; the last two roots are never paired by the scan,
and a run of three ending at the last root is treated as a pair.  The host
inputs of the drop-in (the vectors it uploads) are compared bit for bit with
the vectors the oracle writes to unit 4 before its perturbation loop.  cip's
reordering by unit 4's iord60 (cip/ic001.f:46-73) is checked the same way."""
import os
import struct

import numpy as np
import pytest

from cipsi_gb300 import synth


def _system(tmp_path, name):
    cfg = synth.SynthConfig(name, norb=10, nocc=3, ncholesky=12, ncf=40, metat=3, tau=0.02,
                            ranks=(1, 2), coef_mode="decay09", seed=31)
    wd = str(tmp_path / name)
    synth.generate(cfg, wd)
    return wd


def _read59(wd):
    rec = synth.read_records(os.path.join(wd, "bdvec"))[0]
    ncf, metat = struct.unpack_from("<ii", rec, 0)
    c = np.frombuffer(rec, dtype="<f8", count=ncf * metat, offset=8).reshape(metat, ncf).copy()
    e = np.frombuffer(rec, dtype="<f8", count=metat, offset=8 + 8 * ncf * metat).copy()
    return c, e


def _write59(wd, c, e):
    metat, ncf = c.shape
    with open(os.path.join(wd, "bdvec"), "wb") as fh:
        synth.write_record(fh, struct.pack("<ii", ncf, metat) + c.astype("<f8").tobytes()
                           + e.astype("<f8").tobytes())


def _oracle_vectors(wd, metat):
    """c as the oracle writes it in the zero-order record of unit 4."""
    from oracle import build as ob
    ob.run(wd, variant="cipsym")
    rec = synth.read_records(os.path.join(wd, "f04"))[0]
    ncf = struct.unpack_from("<5i", rec, 0)[4]
    off = 24 + 1
    ii, jj = struct.unpack_from("<ii", rec, off)
    off += 8 + 8 * ncf + 8 * ii
    return np.frombuffer(rec, dtype="<f8", count=jj, offset=off).reshape(metat, ncf)


def _mixed_vectors(wd):
    """Roots 1 and 2 mixed with a root whose spin-flip partners carry opposite
    weights, so that the pairs of the mixed roots have unequal weights."""
    from cipsi_gb300 import engine
    inp = engine.Inputs(wd)
    nesp, ysaut = inp.array("nesp"), inp.array("ysaut")
    inp.close()
    c, e = _read59(wd)
    anti = c[1].copy()
    for k in range(len(nesp)):
        if not ysaut[k] and nesp[k] == 1:
            anti[k + 1] = -anti[k]
    anti /= np.linalg.norm(anti)
    t = 0.3
    r1 = np.cos(t) * c[0] + np.sin(t) * anti
    r2 = -np.sin(t) * c[0] + np.cos(t) * anti
    return np.stack([r1, r2, c[2]]), e, nesp, ysaut


@pytest.mark.parametrize("pattern", ["first_pair", "last_pair", "all_three"])
def test_degenerate_roots_rotate_like_the_oracle(tmp_path, engine_lib, oracle_exe, pattern):
    from cipsi_gb300 import engine
    wd = _system(tmp_path, pattern)
    c, e, nesp, ysaut = _mixed_vectors(wd)
    e = e.copy()
    if pattern == "first_pair":
        e[1] = e[0] + 4e-7
        e[2] = e[0] + 0.3
    elif pattern == "last_pair":
        c = c[[2, 0, 1]]
        e[1] = e[0] + 0.3
        e[2] = e[1] + 4e-7
    else:
        e[1] = e[0] + 3e-7
        e[2] = e[0] + 6e-7
    _write59(wd, c, e)
    inp = engine.Inputs(wd)
    host_c = inp.array("c").reshape(3, -1)
    inp.close()
    oracle_c = _oracle_vectors(wd, 3)
    np.testing.assert_array_equal(host_c, oracle_c)
    if pattern == "last_pair":
        np.testing.assert_array_equal(host_c, c)  # never paired
        return
    # roots 1 and 2 rotated in their plane, root 3 untouched
    assert not np.array_equal(host_c[:2], c[:2])
    np.testing.assert_array_equal(host_c[2], c[2])
    rot = host_c[:2] @ np.linalg.pinv(c[:2])  # host_c[:2] = rot @ c[:2], rot orthogonal
    np.testing.assert_allclose(rot @ c[:2], host_c[:2], atol=1e-12)
    np.testing.assert_allclose(rot @ rot.T, np.eye(2), atol=1e-12)
    # the first pair of unequal weights now has equal weights on root 1
    for k in range(len(nesp)):
        if not ysaut[k] and nesp[k] == 1 and abs(abs(c[0, k]) - abs(c[0, k + 1])) >= 1e-5:
            assert abs(abs(host_c[0, k]) - abs(host_c[0, k + 1])) < 1e-4
            break


def test_cip_reorders_vectors_by_iord60(tmp_path, engine_lib, oracle_exe):
    """cip (not cipsym) reads a permutation iord60 as unit 4's second record
    and moves coefficient k of unit 59 to position iord60(k)
    (cip/ic001.f:46-73); the host's vectors equal the oracle's and the
    permutation applied to unit 59."""
    from cipsi_gb300 import engine
    cfg = synth.SynthConfig("perm", norb=10, nocc=3, ncholesky=12, ncf=40, metat=2, tau=0.02,
                            ranks=(1, 2), coef_mode="decay09", seed=61, variant="cip")
    wd = str(tmp_path / "perm")
    synth.generate(cfg, wd)
    c59, _ = _read59(wd)
    ncf = c59.shape[1]
    perm = np.random.default_rng(7).permutation(ncf) + 1
    recs = synth.read_records(os.path.join(wd, "f04"))
    with open(os.path.join(wd, "f04"), "wb") as fh:
        synth.write_record(fh, recs[0])
        synth.write_record(fh, perm.astype("<i4").tobytes())
    inp = engine.Inputs(wd, variant="cip")
    host_c = inp.array("c").reshape(2, -1)
    inp.close()
    want = np.empty_like(c59)
    want[:, perm - 1] = c59
    np.testing.assert_array_equal(host_c, want)
    from oracle import build as ob
    ob.run(wd, variant="cip")
    rec = synth.read_records(os.path.join(wd, "f04"))[0]
    ii, jj = struct.unpack_from("<ii", rec, 25)
    np.testing.assert_array_equal(np.frombuffer(rec, dtype="<f8", count=jj, offset=33 + 8 * ncf + 8 * ii),
                                  want.reshape(-1))
