"""The listing lines the Autocip driver reads from a perturbation run of
cipsym (Autocip_13/calcul.f90:360-378): after 'nombre de determinants sur
la file 60' the pair (ntot, metat), and after the first line holding
' energies CIPSI envp' -- printed by stkener.f when it stores the ENvp
energies on unit 33 -- metat values read list-directed.  A run with
ityper = 0 (no perturbation, deter.f:231) goes through the same output path
with no device work, so the drop-in's executable runs it here; its units
60, 4 and 33 are compared byte for byte with the oracle's."""
import json
import os
import shutil
import struct
import subprocess

import numpy as np

from cipsi_gb300 import synth

import cases


def autocip_reads(listing: str, name: str, count: int):
    """find_str(name) then read(*) `count` values, as calcul.f90 does:
    list-directed input continues over lines until `count` items are read."""
    lines = listing.splitlines()
    for i, line in enumerate(lines):
        if name in line:
            vals = []
            for nxt in lines[i + 1:]:
                vals += [float(t.replace("D", "E").replace("d", "e")) for t in nxt.replace(",", " ").split()]
                if len(vals) >= count:
                    return vals[:count]
            raise AssertionError("listing ends before %d values after %r" % (count, name))
    raise AssertionError("%r not in the listing" % name)


def test_listing_read_like_the_autocip_driver(tmp_path, engine_lib, oracle_exe):
    from cipsi_gb300 import EXE_PATH
    from oracle import build as ob
    name, cfg = cases.small_cases()[1]
    wd = str(tmp_path / name)
    synth.generate(cfg, wd)
    with open(os.path.join(wd, "cip.in")) as fh:
        txt = fh.read()
    with open(os.path.join(wd, "cip.in"), "w") as fh:
        fh.write(txt.replace(f"ityper={cfg.ityper}", "ityper=0"))
    wo = wd + "_oracle"
    shutil.copytree(wd, wo)
    with open(os.path.join(wd, "cip.in")) as fin:
        r = subprocess.run([EXE_PATH, "--sym", "--json", "run.json"], cwd=wd, stdin=fin, capture_output=True,
                           text=True)
    assert r.returncode == 0, r.stderr
    jo = json.load(open(ob.run(wo, variant="cipsym")))
    for unit in ("det", "f04", "ener"):
        with open(os.path.join(wo, unit), "rb") as a, open(os.path.join(wd, unit), "rb") as b:
            assert a.read() == b.read(), unit
    jg = json.load(open(os.path.join(wd, "run.json")))
    metat = cfg.metat
    ntot, metat2 = autocip_reads(r.stdout, "nombre de determinants sur la file 60", 2)
    assert (ntot, metat2) == (jg["ntot60"], metat) == (jo["ntot60"], metat)
    # no perturbation: zero E2, and the variational energies in 'var'
    assert autocip_reads(r.stdout, " energies CIPSI envp", metat) == [0.0] * metat
    escf = struct.unpack_from("<d", synth.read_records(os.path.join(wd, "ener"))[0], 44)[0]
    var = autocip_reads(r.stdout, " energies CIPSI var", metat)
    np.testing.assert_allclose(var, np.asarray(jg["e"]) + escf, rtol=1e-15)
    # unit 33: the four records appended after escf's, values as printed
    recs = synth.read_records(os.path.join(wd, "ener"))
    assert [rec[:19] for rec in recs[1:]] == [b"energies CIPSI var ", b"energies CIPSI mpb ",
                                             b"energies CIPSI envp", b"energies CIPSI enb "]
    np.testing.assert_array_equal(np.frombuffer(recs[1], dtype="<f8", offset=40), var)


def test_autocip_reader_on_the_reference_layout():
    """The reader itself, on text laid out as stkener.f's list-directed
    writes lay it out (values possibly spread over lines)."""
    text = (" *************************************\n"
            " energies CIPSI envp                      stockee sur la file 33\n"
            "  -1.234567890123457E-002  -2.500000000000000E-003\n"
            "  -7.0E-004\n"
            " *************************************\n")
    assert autocip_reads(text, " energies CIPSI envp", 3) == [-1.234567890123457e-2, -2.5e-3, -7.0e-4]
