"""The CPU oracle (a restatement of the reference's list-editing loop nest)
against an independent brute-force model of the same perturber set: same
(source, owner, perturber) multiset, same spin-flip weights, same
|<I|H|Psi>|.  This pins the oracle where the reference ships no test data."""
import collections
import os

import numpy as np
import pytest

import brute_force as bf
from cases import small_cases
from cipsi_gb300 import synth
from conftest import copy_dir
from oracle import build as ob


@pytest.mark.parametrize("name,cfg", small_cases(), ids=[c[0] for c in small_cases()])
def test_oracle_matches_bruteforce(tmp_path, oracle_exe, name, cfg):
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    run = copy_dir(wd, str(tmp_path / "run"))
    ob.run(run, variant="cipsym", candlog="cand.bin")
    inp = bf.read_inputs(wd)
    model = bf.Model(inp)
    sem = bf.enumerate_semantic(inp, model)
    ora = bf.read_candlog(os.path.join(run, "cand.bin"), inp.C.shape[1])
    ko = collections.Counter((r[0], r[1], model.to_bits(r[2], r[3])) for r in ora)
    ks = collections.Counter((r[0], r[1], r[2]) for r in sem)
    assert ko == ks
    assert all(v == 1 for v in ko.values()), "a perturber was processed twice"
    do = {(r[0], r[1], model.to_bits(r[2], r[3])): r for r in ora}
    for r in sem:
        o = do[(r[0], r[1], r[2])]
        assert o[4] == r[3]  # nmul
        assert abs(o[5] - r[4]) < 1e-14  # fmul
        np.testing.assert_allclose(np.abs(o[7]), np.abs(r[5]), rtol=0, atol=1e-13)
