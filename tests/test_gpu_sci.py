"""The drop-in's S-space CI (a perturbation run with lecdet != 5: H over S
from cipsi_hamiltonian_build, its lowest roots from cipsi_davidson) against
the oracle's (dense H, Jacobi), then the perturbation on those vectors.

Bit-exact: S, the processed-perturber counts, ietat, the histogram counts,
the selected set.  Floating point: the root energies to 1e-10 Eh, the
vectors written to unit 4 to 1e-9, E2 to 1e-10 Eh against the oracle's
error-free sums (these systems have every perturber several Eh above the
roots)."""
import collections
import json
import os
import shutil

import numpy as np
import pytest

import cipsi_gb300 as cg
from cipsi_gb300 import synth
from oracle import build as ob
from test_autocip_s_runs import _write_icinp
from test_gpu_parity import read60
from test_oracle_sci import CAS, _chain_cfg, _unit4_space_and_vectors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lecdet,seed,nsym", [(4, 41, 1), (2, 41, 1), (2, 43, 2)])
def test_s_space_ci_matches_oracle(tmp_path, oracle_exe, engine_lib, lecdet, seed, nsym):
    cfg = _chain_cfg(seed, nsym)
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    body = "metat=2, ityper=2, tau=0.01, test=0.01, iselec=1, ymoyen=t, ybrd=f, ywvf=f, twdet=0.5"
    _write_icinp(wd, body + (", lecdet=4,\n" + CAS if lecdet == 4 else ", lecdet=2, tdet=0.0"))
    wo, wg = str(tmp_path / "ora"), str(tmp_path / "gpu")
    shutil.copytree(wd, wo)
    shutil.copytree(wd, wg)
    jo = json.load(open(ob.run(wo, variant="cipsym")))
    jg = cg.run_cip(wg, variant="cipsym")
    for k in ("ncf", "ietat", "n_processed", "ntot60", "nom", "nam"):
        assert jo[k] == jg[k], k
    np.testing.assert_allclose(jg["e"], jo["e"], rtol=0, atol=1e-10)
    for k in ("e2mp", "e2vp", "e2b"):
        assert max(jo["cond_" + k]) < 1e-11
        np.testing.assert_allclose(jg[k], jo["comp_" + k], rtol=0, atol=1e-10, err_msg=k)
    do, co = _unit4_space_and_vectors(os.path.join(wo, "f04"))
    dg, cgv = _unit4_space_and_vectors(os.path.join(wg, "f04"))
    assert do == dg
    np.testing.assert_allclose(cgv, co, rtol=0, atol=1e-9)
    so = read60(os.path.join(wo, "det"), 2, True)
    sg = read60(os.path.join(wg, "det"), 2, True)
    assert collections.Counter(x[0] for x in so) == collections.Counter(x[0] for x in sg)
