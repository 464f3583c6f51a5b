"""Known-answer test: the oracle on the committed 20-orbital fixture
reproduces the committed expected values (E2, counts, histogram, the set of
selected determinants).  Regenerate with tests/golden/make_golden.py."""
import json
import os

import numpy as np

from conftest import copy_dir
from oracle import build as ob

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_oracle_reproduces_golden(tmp_path, oracle_exe):
    import sys
    sys.path.insert(0, GOLD)
    from make_golden import selection_digest
    exp = json.load(open(os.path.join(GOLD, "small_expected.json")))
    run = copy_dir(os.path.join(GOLD, "small"), str(tmp_path / "run"))
    got = json.load(open(ob.run(run, variant="cipsym")))
    for k in ("ncf", "ietat", "n_processed", "ntot60", "nom", "nam"):
        assert got[k] == exp[k], k
    for k in ("e2mp", "e2vp", "e2b", "psimp", "psivp", "dpivot", "e", "emp", "eb"):
        np.testing.assert_allclose(got[k], exp[k], rtol=1e-13, atol=1e-12, err_msg=k)
    n, dig = selection_digest(os.path.join(run, "det"), exp["metat"], True)
    assert n == exp["unit60_records"]
    assert dig == exp["unit60_sets_sha256"]
