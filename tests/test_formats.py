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


def test_curve_geometries_follow_the_batch_recipe():
    a = synth.curve_geometries(256, seed=100)
    b = synth.curve_geometries(256, seed=100)
    assert [(g.norb, g.ncf, g.curve_R, g.seed) for g in a] == [(g.norb, g.ncf, g.curve_R, g.seed) for g in b]
    assert all(40 <= g.norb <= 100 and 500 <= g.ncf <= 5000 and 2.0 <= g.curve_R <= 12.0 for g in a)
    assert len({g.seed for g in a}) == 256
    assert min(g.norb for g in a) <= 45 and max(g.norb for g in a) >= 95


def test_curve_integrals_move_with_R(tmp_path):
    import dataclasses
    import numpy as np
    base = synth.SynthConfig("c", norb=10, nocc=3, ncholesky=20, ncf=30, metat=1, tau=0.02,
                             ranks=(1, 2), coef_mode="decay09", seed=3, curve_R=2.0, energy="diagonal")
    h1, L1, _ = synth.make_integrals(base, np.random.default_rng(base.seed))
    h2, L2, _ = synth.make_integrals(dataclasses.replace(base, curve_R=12.0), np.random.default_rng(base.seed))
    assert not np.allclose(L1, L2) and not np.allclose(np.diag(h1), np.diag(h2))
    # the R-independent parts are shared: the difference is exp(-R/3) L1 scaled
    info = synth.generate(base, str(tmp_path / "g"))
    assert info["ncf"] >= 30
