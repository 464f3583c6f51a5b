"""Regenerate the committed known-answer fixtures (run from the repo root):

    python tests/golden/make_golden.py

Writes tests/golden/small/ (the seeded 20-orbital configuration in the
reference's file formats: ijkl, ener, det, bdvec, f04, cip.in) and
tests/golden/small_expected.json: the CPU oracle's E2 totals, counters,
histogram and a digest of the unit-60 selection for those exact files.

    python tests/golden/make_golden.py --cas

writes only tests/golden/cas_expected.json from the committed small/ files:
the S-only run of Autocip's first cipsym call (CAS_ICINP: a complete active
space of 4 electrons in orbitals 4..11, ordered and written with ityper = -1)
as the oracle makes it, by SHA-256 of the unit-60 file and of unit 4.
"""
import hashlib
import json
import os
import shutil
import struct
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cipsi_gb300 import synth  # noqa: E402
from oracle import build as ob  # noqa: E402


def selection_digest(det_path, metat, sym):
    """Order-independent digest of the unit-60 records after S: sorted
    (holes, particles, round(v, 12)) tuples."""
    items = []
    for r in synth.read_records(det_path):
        m, n = struct.unpack_from("<ii", r, 0)
        idet = struct.unpack_from(f"<{m}i", r, 8)
        nex = struct.unpack_from(f"<{n}i", r, 8 + 4 * m)
        v = struct.unpack_from(f"<{n}d", r, 8 + 4 * m + 4 * n)
        pos = 0
        for i, nec in enumerate(nex):
            h = sorted(idet[pos + 2 * q] for q in range(nec))
            p = sorted(idet[pos + 2 * q + 1] for q in range(nec))
            pos += 2 * nec
            items.append((tuple(h), tuple(p), round(v[i], 12)))
    items.sort()
    return len(items), hashlib.sha256(repr([(h, p) for h, p, _ in items]).encode()).hexdigest()


CAS_ICINP = (" &cipfil\n &end\n &icinp\n  numac=4,5,6,7,8,9,10,11, noac=8, nelac=4, nusym=1,"
             " metat=2, lecdet=4, ityper=-1, ymoyen=t, ybrd=f, yion=f, iselec=1, test=0d0,"
             " tau=0d0\n &end\n")


def cas_digests(run_dir):
    """SHA-256 of the unit-60 file and of unit 4 after the CAS S-only run."""
    return {u: hashlib.sha256(open(os.path.join(run_dir, u), "rb").read()).hexdigest() for u in ("det", "f04")}


def cas_main():
    with tempfile.TemporaryDirectory() as td:
        run = os.path.join(td, "run")
        shutil.copytree(os.path.join(HERE, "small"), run)
        os.remove(os.path.join(run, "det"))
        with open(os.path.join(run, "cip.in"), "w") as fh:
            fh.write(CAS_ICINP)
        j = json.load(open(ob.run(run, variant="cipsym")))
        out = dict(ncf=j["ncf"], ntot60=j["ntot60"], sha256=cas_digests(run))
    with open(os.path.join(HERE, "cas_expected.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print(json.dumps(out))


def main():
    out = os.path.join(HERE, "small")
    shutil.rmtree(out, ignore_errors=True)
    synth.generate(synth.CONFIGS["small"], out)
    with tempfile.TemporaryDirectory() as td:
        run = os.path.join(td, "run")
        shutil.copytree(out, run)
        j = json.load(open(ob.run(run, variant="cipsym")))
        nrec, dig = selection_digest(os.path.join(run, "det"), j["metat"], True)
    j.pop("t_pertu_s", None)
    j.pop("t_diexcit_s", None)
    j["unit60_records"] = nrec
    j["unit60_sets_sha256"] = dig
    with open(os.path.join(HERE, "small_expected.json"), "w") as fh:
        json.dump(j, fh, indent=1, sort_keys=True)
    print(json.dumps({k: j[k] for k in ("ncf", "ietat", "n_processed", "e2mp", "e2vp")}))


if __name__ == "__main__":
    cas_main() if "--cas" in sys.argv else main()
