"""Input/output formats: the synthetic generator writes the reference's
unit files; records, S order (spin-flip partners adjacent, rank-sorted) and
the Fortran record markers are checked here."""
import struct

import numpy as np

from cipsi_gb300 import synth
import brute_force as bf


def test_records_roundtrip(tmp_path):
    p = tmp_path / "f"
    with open(p, "wb") as fh:
        synth.write_record(fh, b"abc")
        synth.write_record(fh, b"")
        synth.write_record(fh, struct.pack("<3d", 1, 2, 3))
    r = synth.read_records(str(p))
    assert r[0] == b"abc" and r[1] == b"" and struct.unpack("<3d", r[2]) == (1.0, 2.0, 3.0)


def test_generated_space_is_flip_closed_and_rank_sorted(tmp_path):
    cfg = synth.SynthConfig("t", norb=12, nocc=4, ncholesky=10, ncf=60, metat=2, tau=0.02,
                            ranks=(1, 2, 3), coef_mode="decay09", seed=9)
    info = synth.generate(cfg, str(tmp_path))
    inp = bf.read_inputs(str(tmp_path))
    assert len(inp.S) == info["ncf"]
    ranks = [len(h) for h, _ in inp.S]
    assert ranks == sorted(ranks)
    keys = set(inp.S)
    for h, p in inp.S:
        fh, fp = synth.flip_lists(h, p, inp.norb)
        assert (tuple(fh), tuple(fp)) in keys
    # partners follow their representative and carry equal canonical coefficients
    m = bf.Model(inp)
    for i, ys in enumerate(inp.ysaut):
        if ys:
            assert inp.nesp[i - 1] == 1 and not inp.ysaut[i - 1]
            np.testing.assert_allclose(m.Ccan[i], m.Ccan[i - 1], atol=1e-15)
    # vectors are orthonormal
    np.testing.assert_allclose(inp.C.T @ inp.C, np.eye(inp.C.shape[1]), atol=1e-12)


def test_integral_file_layout(tmp_path):
    cfg = synth.SynthConfig("t", norb=8, nocc=3, ncholesky=6, ncf=10, metat=1, tau=0.02, seed=1, nsym=2)
    synth.generate(cfg, str(tmp_path))
    inp = bf.read_inputs(str(tmp_path))
    n = inp.norb
    # every pair has an index and irrep; ij0(i,i) pair index, irrep implicit 1
    for i in range(1, n + 1):
        for j in range(1, n + 1):
            lo, hi = min(i, j), max(i, j)
            assert inp.ij0[lo, hi] >= 1
            if lo != hi:
                assert 1 <= inp.ij0[hi, lo] <= inp.nsym
    # J_pp == K_pp exactly (fock.f:112-113 reads both from ai(i,i,i,i))
    for i in range(1, n + 1):
        t = i * (i + 1) // 2
        assert inp.J[t] == inp.K[t]
