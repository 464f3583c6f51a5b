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


def test_oracle_writes_unit4(tmp_path, oracle_exe):
    """The oracle writes the three unit-4 records of cip.f:144-150, 410-414."""
    import struct
    import numpy as np
    from cipsi_gb300 import synth
    from conftest import copy_dir
    from oracle import build as ob
    wd = copy_dir(os.path.join(os.path.dirname(__file__), "golden", "small"), str(tmp_path / "w"))
    j = json.load(open(ob.run(wd)))
    recs = synth.read_records(os.path.join(wd, "f04"))
    assert len(recs) == 3
    norb, noca, nocb, metat, ncf, isz = struct.unpack_from("<6i", recs[0], 0)
    assert (norb, noca, nocb, metat, ncf, isz) == (j["norb"], j["noca"], j["noca"] + j["norb"], j["metat"],
                                                    j["ncf"], 0)
    ii, jj = struct.unpack_from("<2i", recs[0], 25)
    assert jj == ncf * metat
    size = 33 + 8 * ncf + 8 * ii + 8 * jj + 24 * metat + 4 * metat + 8 * ncf + 16 * norb + 8 * 500000 \
        + 16 * norb + 2 * norb * ncf
    assert len(recs[0]) == size
    nbr = metat * (metat + 1) // 2
    assert len(recs[1]) == 8 * nbr + 8 + 4 + 4 + 4 * metat
    assert len(recs[2]) == 24 * nbr
    h = np.frombuffer(recs[2], dtype="<f8")
    escf = struct.unpack_from("<d", recs[1], 8 * nbr)[0]
    assert np.allclose(h[nbr - 1] - (j["e"][0] + escf), j["e2mp"][0])


def test_cas_space_run_known_answer(tmp_path, oracle_exe, engine_lib):
    """Autocip's first cipsym call (a CAS of 4 electrons in orbitals 4..11,
    ityper = -1) on the committed 20-orbital files: the oracle and the drop-in
    both write the committed unit 60 and unit 4, byte for byte (784
    determinants in the order of shell.f).  Regenerate with
    tests/golden/make_golden.py --cas."""
    import sys
    import cipsi_gb300
    sys.path.insert(0, GOLD)
    from make_golden import CAS_ICINP, cas_digests
    exp = json.load(open(os.path.join(GOLD, "cas_expected.json")))
    for who in ("oracle", "engine"):
        run = copy_dir(os.path.join(GOLD, "small"), str(tmp_path / who))
        os.remove(os.path.join(run, "det"))
        with open(os.path.join(run, "cip.in"), "w") as fh:
            fh.write(CAS_ICINP)
        if who == "oracle":
            got = json.load(open(ob.run(run, variant="cipsym")))
        else:
            got = cipsi_gb300.run_cip(run, variant="cipsym")
        assert (got["ncf"], got["ntot60"]) == (exp["ncf"], exp["ntot60"]), who
        assert cas_digests(run) == exp["sha256"], who
